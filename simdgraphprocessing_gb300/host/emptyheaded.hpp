// Drop-in application base and command-line entry (the reference's
// src/emptyheaded.hpp:8-83).  An app .cpp defines its class template and
// init_app<T,R>; unless GOOGLE_TEST is defined, main() parses the flags and
// runs the app with the layout named by --layout.
#ifndef EH_DROPIN_EMPTYHEADED_HPP
#define EH_DROPIN_EMPTYHEADED_HPP

#include "MutableGraph.hpp"
#include "ParallelBuffer.hpp"
#include "Parser.hpp"
#include "SparseMatrix.hpp"
#include "Table.hpp"

template <class T, class R>
class application {
 public:
  SparseMatrix<T, R>* graph;
  MutableGraph* input_graph;
  size_t num_threads;
  string layout;
  size_t query_depth;
  long start_node;

  application(Parser input_data)
      : graph(nullptr),
        input_graph(input_data.input_graph),
        num_threads(input_data.num_threads),
        layout(input_data.layout),
        query_depth(input_data.n),
        start_node(input_data.start_node) {}
  virtual ~application() {}
  virtual void run() = 0;
};

template <class T, class R>
application<T, R>* init_app(Parser input_data);

#ifndef GOOGLE_TEST
int main(int argc, char* argv[]) {
  std::string s(argv[0]);
  const size_t slash = s.find_last_of('/');
  const std::string app = slash == std::string::npos ? s : s.substr(slash + 1);
  Parser input_data = input_parser::parse(argc, argv, app);
  try {
    if (input_data.layout == "uint") init_app<uinteger, uinteger>(input_data)->run();
    else if (input_data.layout == "bs") init_app<bitset, bitset>(input_data)->run();
    else if (input_data.layout == "pshort") init_app<pshort, pshort>(input_data)->run();
    else if (input_data.layout == "hybrid") init_app<hybrid, hybrid>(input_data)->run();
    else {
      cout << "No valid layout entered." << endl;
      exit(0);
    }
  } catch (const std::exception& e) {
    cerr << e.what() << endl;
    return 1;
  }
  return 0;
}
#endif

#endif
