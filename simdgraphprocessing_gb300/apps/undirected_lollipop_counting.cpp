// undirected_lollipop_counting<T,R> (the reference's
// apps/undirected_lollipop_counting.cpp): same class, members and output line;
// counted on the device over the full (unpruned) matrix.
#include "emptyheaded.hpp"

template <class T, class R>
class undirected_lollipop_counting : public application<T, R> {
 public:
  size_t num_lollipops;

  undirected_lollipop_counting(Parser input_data) : application<T, R>(input_data) { num_lollipops = 0; }

  SparseMatrix<T, R>* materialize_graph() {
    auto node_selection = [](uint32_t node, uint32_t attribute) -> bool {
      (void)attribute;
      (void)node;
      return true;
    };
    auto edge_selection = [](uint32_t node, uint32_t nbr, uint32_t attribute) -> bool {
      (void)attribute;
      (void)node;
      (void)nbr;
      return true;
    };
    return SparseMatrix<T, R>::build(this->input_graph, node_selection, edge_selection, this->num_threads);
  }

  void run() {
    this->graph = materialize_graph();
    const double start_time = common::startClock();
    num_lollipops = this->graph->count_lollipops();
    common::stopClock("lollipop", start_time);
    cout << "Count: " << num_lollipops << endl;
  }
};

#ifndef GOOGLE_TEST  // the entry point needs one init_app; test drivers may include several apps
template <class T, class R>
application<T, R>* init_app(Parser input_data) {
  return new undirected_lollipop_counting<T, R>(input_data);
}
#endif
