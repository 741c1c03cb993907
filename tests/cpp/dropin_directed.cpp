// Drives the drop-in symbiosity and n_path classes the way the reference's
// gtests do (test/symbiosity_test.cpp, test/n_path_test.cpp): load a graph,
// build a Parser, construct the app, run(), read the public result member.
// Usage:
//   dropin_directed <graph> <layout> <directed 0|1> <symbiosity> <n_path> <start> <depth> <n_path_from_start>
// <n_path> is the BFS from the largest row with no depth limit; the last value
// is the BFS from external id <start> limited to <depth>.  Exit status 0 when
// every result equals the expected value.
#define GOOGLE_TEST
#include "symbiosity.cpp"
#include "n_path.cpp"

static MutableGraph* load(const char* path, bool directed) {
  return directed ? MutableGraph::directedFromBinary(path) : MutableGraph::undirectedFromBinary(path);
}

template <class L>
static int run_all(const char* path, bool directed, const unsigned long long* want, long start, int depth) {
  int bad = 0;
  {
    MutableGraph* g = load(path, directed);
    Parser p(4, false, 0, 0, g, "layout");
    symbiosity<L, L> app(p);
    app.run();
    if (app.count != want[0]) {
      std::cerr << "symbiosity " << app.count << " != " << want[0] << std::endl;
      bad++;
    }
    // get_column: the in-neighbourhood (the row itself when undirected).
    for (uint32_t i = 0; i < 4 && i < g->num_nodes; i++) {
      Set<L> col = app.graph->get_column(i);
      size_t seen = 0;
      col.foreach([&](uint32_t) { seen++; });
      if (seen != g->in_neighborhoods->at(i)->size() || col.cardinality != seen) {
        std::cerr << "get_column(" << i << ") has " << seen << " entries, want "
                  << g->in_neighborhoods->at(i)->size() << std::endl;
        bad++;
      }
    }
    delete g;
  }
  {
    MutableGraph* g = load(path, directed);
    Parser p(4, false, 0xeffffff, (size_t)-1, g, "layout");
    n_path<L, L> app(p);
    app.run();
    if (app.path_length != want[1]) {
      std::cerr << "n_path " << app.path_length << " != " << want[1] << std::endl;
      bad++;
    }
    delete g;
  }
  {
    MutableGraph* g = load(path, directed);
    Parser p(4, false, depth, (size_t)start, g, "layout");
    n_path<L, L> app(p);
    app.run();
    if (app.path_length != want[2]) {
      std::cerr << "n_path from " << start << " " << app.path_length << " != " << want[2] << std::endl;
      bad++;
    }
    delete g;
  }
  return bad;
}

int main(int argc, char** argv) {
  if (argc != 9) {
    std::cerr << "usage: " << argv[0] << " graph layout directed symbiosity n_path start depth n_path_from_start"
              << std::endl;
    return 2;
  }
  const bool directed = atoi(argv[3]) != 0;
  const unsigned long long want[3] = {strtoull(argv[4], 0, 10), strtoull(argv[5], 0, 10), strtoull(argv[8], 0, 10)};
  const long start = atol(argv[6]);
  const int depth = atoi(argv[7]);
  const std::string layout = argv[2];
  int bad;
  try {
    if (layout == "uint") bad = run_all<uinteger>(argv[1], directed, want, start, depth);
    else if (layout == "bs") bad = run_all<bitset>(argv[1], directed, want, start, depth);
    else if (layout == "pshort") bad = run_all<pshort>(argv[1], directed, want, start, depth);
    else bad = run_all<hybrid>(argv[1], directed, want, start, depth);
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    return 1;
  }
  return bad ? 1 : 0;
}
