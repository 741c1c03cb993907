// The reference's seven gtests (test/undirected_triangle_counting_test.cpp:6-13,
// test/n_clique_test.cpp:6-12, test/undirected_lollipop_counting_test.cpp:6-13,
// test/similar_nodes_test.cpp:6-13, test/symbiosity_test.cpp:6-20,
// test/n_path_test.cpp:6-12), restated without gtest: the same loader, Parser
// arguments, app classes, template layouts and expected values, run against
// the drop-in headers and the GPU library on the reference's own test graphs.
// Usage: dropin_gtests <dir holding facebook.bin and dfacebook.bin>
// Prints one line per test and exits 0 when all seven pass.
#define GOOGLE_TEST
#include "undirected_triangle_counting.cpp"
#include "n_clique.cpp"
#include "undirected_lollipop_counting.cpp"
#include "similar_nodes.cpp"
#include "symbiosity.cpp"
#include "n_path.cpp"

static std::string g_dir;
static std::string path(const char* name) { return g_dir + "/" + name; }

static int report(const char* test, unsigned long long got, unsigned long long want) {
  std::cout << (got == want ? "[       OK ] " : "[  FAILED  ] ") << test << " got " << got << " want " << want
            << std::endl;
  return got == want ? 0 : 1;
}

static int triangles() {
  MutableGraph* g = MutableGraph::undirectedFromBinary(path("facebook.bin"));
  Parser p(4, false, 0, 0, g, "hybrid");
  undirected_triangle_counting<hybrid, hybrid> app(p);
  app.run();
  return report("TEST1.FACEBOOK_TRIANGLES_HYBRID", app.num_triangles, 1612010ull);
}

static int cliques() {
  MutableGraph* g = MutableGraph::undirectedFromBinary(path("facebook.bin"));
  Parser p(4, false, 4, 0, g, "hybrid");
  n_clique<hybrid, hybrid> app(p);
  app.run();
  return report("CliqueTest.FacebookCliqueCounting", (unsigned long long)app.num_cliques, 30004668ull);
}

static int lollipops() {
  MutableGraph* g = MutableGraph::undirectedFromBinary(path("facebook.bin"));
  Parser p(4, false, 0, 0, g, "hybrid");
  undirected_lollipop_counting<hybrid, hybrid> app(p);
  app.run();
  return report("LollipopTest.FacebookLollipopCountingHybrid", app.num_lollipops, 713455740ull);
}

static int similar() {
  MutableGraph* g = MutableGraph::undirectedFromBinary(path("facebook.bin"));
  Parser p(4, false, 0, 0, g, "hybrid");
  similar_nodes<hybrid, hybrid> app(p);
  app.run();
  return report("SimilarNodesTest.SimilarNodesCountingFacebookHybrid", app.count, 904ull);
}

static int symbiosity_directed() {
  MutableGraph* g = MutableGraph::directedFromBinary(path("dfacebook.bin"));
  Parser p(4, false, 0, 0, g, "hybrid");
  symbiosity<hybrid, hybrid> app(p);
  app.run();
  return report("SymbiosityTest.FacebookSymbiosityCountingHybrid", app.count, 0ull);
}

static int symbiosity_undirected() {
  MutableGraph* g = MutableGraph::undirectedFromBinary(path("facebook.bin"));
  Parser p(4, false, 0, 0, g, "hybrid");
  symbiosity<hybrid, hybrid> app(p);
  app.run();
  return report("SymbiosityTest.FacebookSymbiosityCountingHybridUndirected", app.count, 4039ull);
}

static int bfs() {
  MutableGraph* g = MutableGraph::directedFromBinary(path("dfacebook.bin"));
  Parser p(4, false, 4, 0, g, "uint");
  n_path<uinteger, uinteger> app(p);
  app.run();
  return report("BFSTest.FacebookCliqueCounting", app.path_length, 4ull);
}

int main(int argc, char** argv) {
  if (argc != 2) {
    std::cerr << "usage: " << argv[0] << " <fixture dir>" << std::endl;
    return 2;
  }
  g_dir = argv[1];
  int bad = 0;
  try {
    bad += triangles();
    bad += cliques();
    bad += lollipops();
    bad += similar();
    bad += symbiosity_directed();
    bad += symbiosity_undirected();
    bad += bfs();
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    return 1;
  }
  std::cout << (7 - bad) << " of 7 passed" << std::endl;
  return bad ? 1 : 0;
}
