// symbiosity<T,R> (the reference's apps/symbiosity.cpp): same class, members
// and output line; rows whose out- and in-neighbourhoods have Jaccard ratio
// above N, counted on the device.
#include "emptyheaded.hpp"

template <class T, class R>
class symbiosity : public application<T, R> {
 public:
  size_t count;
  double N;  // threshold

  symbiosity(Parser input_data) : application<T, R>(input_data) {
    count = 0;
    N = 0.5;
  }

  SparseMatrix<T, R>* materialize_graph() {
    auto node_selection = [](uint32_t node, uint32_t attribute) -> bool {
      (void)node;
      (void)attribute;
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
    count = this->graph->count_symbiosity(N);
    common::stopClock("symbiosity", start_time);
    cout << "Count: " << count << endl << endl;
  }
};

#ifndef GOOGLE_TEST  // the entry point needs one init_app; test drivers may include several apps
template <class T, class R>
application<T, R>* init_app(Parser input_data) {
  return new symbiosity<T, R>(input_data);
}
#endif
