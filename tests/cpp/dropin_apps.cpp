// Drives the drop-in app classes the way the reference's gtests do
// (test/undirected_triangle_counting_test.cpp, test/n_clique_test.cpp,
// test/undirected_lollipop_counting_test.cpp, test/similar_nodes_test.cpp):
// load a binary graph, build a Parser, construct the app, run(), read the
// public count member.  Usage:
//   dropin_apps <graph.bin> <layout> <triangles> <cliques4> <lollipops> <similar_nodes>
// Exit status 0 when all four counts equal the expected values.
#define GOOGLE_TEST
#include "undirected_triangle_counting.cpp"
#include "n_clique.cpp"
#include "undirected_lollipop_counting.cpp"
#include "similar_nodes.cpp"

template <class L>
static int run_all(const char* path, const unsigned long long want[4]) {
  int bad = 0;
  {
    MutableGraph* g = MutableGraph::undirectedFromBinary(path);
    Parser p(4, false, 0, 0, g, "layout");
    undirected_triangle_counting<L, L> app(p);
    app.run();
    if (app.num_triangles != want[0]) {
      std::cerr << "triangles " << app.num_triangles << " != " << want[0] << std::endl;
      bad++;
    }
  }
  {
    MutableGraph* g = MutableGraph::undirectedFromBinary(path);
    Parser p(4, false, 4, 0, g, "layout");
    n_clique<L, L> app(p);
    app.run();
    if ((unsigned long long)app.num_cliques != want[1]) {
      std::cerr << "cliques " << app.num_cliques << " != " << want[1] << std::endl;
      bad++;
    }
  }
  {
    MutableGraph* g = MutableGraph::undirectedFromBinary(path);
    Parser p(4, false, 0, 0, g, "layout");
    undirected_lollipop_counting<L, L> app(p);
    app.run();
    if (app.num_lollipops != want[2]) {
      std::cerr << "lollipops " << app.num_lollipops << " != " << want[2] << std::endl;
      bad++;
    }
  }
  {
    MutableGraph* g = MutableGraph::undirectedFromBinary(path);
    Parser p(4, false, 0, 0, g, "layout");
    similar_nodes<L, L> app(p);
    app.run();
    if (app.count != want[3]) {
      std::cerr << "similar_nodes " << app.count << " != " << want[3] << std::endl;
      bad++;
    }
    // get_row: host view of a device row, walked with Set::foreach.
    Set<L> row = app.graph->get_row(0);
    size_t seen = 0;
    row.foreach([&](uint32_t) { seen++; });
    if (seen != row.cardinality) {
      std::cerr << "get_row(0) walked " << seen << " of " << row.cardinality << std::endl;
      bad++;
    }
  }
  return bad;
}

int main(int argc, char** argv) {
  if (argc != 7) {
    std::cerr << "usage: " << argv[0] << " graph.bin layout tri clq4 lolli similar" << std::endl;
    return 2;
  }
  const unsigned long long want[4] = {strtoull(argv[3], 0, 10), strtoull(argv[4], 0, 10),
                                      strtoull(argv[5], 0, 10), strtoull(argv[6], 0, 10)};
  const std::string layout = argv[2];
  int bad;
  try {
    if (layout == "uint") bad = run_all<uinteger>(argv[1], want);
    else if (layout == "bs") bad = run_all<bitset>(argv[1], want);
    else if (layout == "pshort") bad = run_all<pshort>(argv[1], want);
    else bad = run_all<hybrid>(argv[1], want);
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    return 1;
  }
  return bad ? 1 : 0;
}
