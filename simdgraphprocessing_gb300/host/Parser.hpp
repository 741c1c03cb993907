// Drop-in Parser and input_parser::parse (the reference's src/Parser.hpp:10-180):
// same constructor and command-line flags
//   --graph=<path> --input_type=<binary|text> --t=<threads> --layout=<uint|pshort|bs|hybrid>
//   [--n=<clique size, default 4 for n_clique; BFS depth for n_path>]
//   [--start_node=<external id>] [--asymmetric: load a directed graph]
// plus --device=<cuda device ordinal>.
#ifndef EH_DROPIN_PARSER_HPP
#define EH_DROPIN_PARSER_HPP

#include <getopt.h>

#include <cuda_runtime.h>

#include "MutableGraph.hpp"

class Parser {
 public:
  int num_threads;
  bool attributes;
  int n;
  long start_node;
  MutableGraph* input_graph;
  string layout;

  Parser(int num_threads_in, bool attributes_in, int n_in, size_t start_node_in, MutableGraph* in_graph,
         string layout_in)
      : num_threads(num_threads_in),
        attributes(attributes_in),
        n(n_in),
        start_node((long)start_node_in),
        input_graph(in_graph),
        layout(layout_in) {}
};

namespace input_parser {

inline void printUsage(const string& app) {
  cout << "USAGE: ./application <OPTIONS>" << endl;
  cout << "OPTIONS: " << endl;
  cout << "\tREQUIRED: --graph=<path to graph> --input_type=<'binary' or 'text'> --t=<# of threads>" << endl;
  cout << "\t\t--layout=<uint,pshort,bs,hybrid>" << endl;
  if (app == "n_clique") cout << "\tOPTIONAL: --n=<size of cliques to find, default is 4>" << endl;
  if (app == "n_path") {
    cout << "\tOPTIONAL: --start_node=<start node, default is highest degree> --n=<path length, default finds all "
            "paths> --asymmetric"
         << endl;
    cout << "*takes a directed graph as input*" << endl;
  }
  cout << "\tOPTIONAL: --device=<CUDA device ordinal, default 0>" << endl;
  exit(0);
}

inline Parser parse(int argc, char* argv[], string app) {
  const char* graph_path = nullptr;
  const char* input_type = nullptr;
  const char* layout = nullptr;
  int num_threads = 0, n = -1, device = 0;
  long start_node = -1;
  bool help = false, directed = false;
  static struct option opts[] = {{"help", no_argument, 0, 'h'},
                                 {"t", required_argument, 0, 't'},
                                 {"graph", required_argument, 0, 'g'},
                                 {"layout", required_argument, 0, 'l'},
                                 {"n", required_argument, 0, 'n'},
                                 {"start_node", required_argument, 0, 's'},
                                 {"input_type", required_argument, 0, 'f'},
                                 {"device", required_argument, 0, 'd'},
                                 {"asymmetric", no_argument, 0, 'm'},
                                 {0, 0, 0, 0}};
  int c, idx = 0;
  optind = 1;
  while ((c = getopt_long(argc, argv, "ht:g:l:n:s:f:d:m", opts, &idx)) != -1) {
    switch (c) {
      case 'h': help = true; break;
      case 't': num_threads = atoi(optarg); break;
      case 'g': graph_path = optarg; break;
      case 'l': layout = optarg; break;
      case 'n': n = atoi(optarg); break;
      case 's': start_node = atol(optarg); break;
      case 'f': input_type = optarg; break;
      case 'd': device = atoi(optarg); break;
      case 'm': directed = true; break;
      default: break;
    }
  }
  if (num_threads == 0 || !graph_path || !input_type || help || !layout) printUsage(app);
  if (n == -1 && app == "n_clique") n = 4;
  if (n == -1 && app == "n_path") n = 0xeffffff;
  if (cudaSetDevice(device) != cudaSuccess) {
    cerr << "cannot select CUDA device " << device << endl;
    exit(1);
  }
  MutableGraph* g;
  if (directed) {
    cout << "Loading a directed graph" << endl;
    g = string(input_type) == "text" ? MutableGraph::directedFromEdgeList(graph_path)
                                     : MutableGraph::directedFromBinary(graph_path);
  } else {
    cout << "Loading a undirected graph" << endl;
    g = string(input_type) == "text" ? MutableGraph::undirectedFromEdgeList(graph_path)
                                     : MutableGraph::undirectedFromBinary(graph_path);
  }
  return Parser(num_threads, false, n, (size_t)start_node, g, layout);
}

}  // namespace input_parser

#endif
