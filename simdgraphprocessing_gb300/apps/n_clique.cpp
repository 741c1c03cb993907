// n_clique<T,R> (the reference's apps/n_clique.cpp): same class, members and
// output line; counts cliques of size query_depth (default 4) on the device.
#include "emptyheaded.hpp"

template <class T, class R>
class n_clique : public application<T, R> {
 public:
  long num_cliques;
  size_t query_depth;

  n_clique(Parser input_data) : application<T, R>(input_data) {
    num_cliques = 0;
    query_depth = input_data.n;
  }

  SparseMatrix<T, R>* materialize_graph() {
    auto node_selection = [](uint32_t node, uint32_t attribute) -> bool {
      (void)node;
      (void)attribute;
      return true;
    };
    auto edge_selection = [](uint32_t node, uint32_t nbr, uint32_t attribute) -> bool {
      (void)attribute;
      return nbr < node;
    };
    return SparseMatrix<T, R>::build(this->input_graph, node_selection, edge_selection, this->num_threads);
  }

  void run() {
    this->graph = materialize_graph();
    const double start_time = common::startClock();
    num_cliques = (long)this->graph->count_cliques((uint32_t)query_depth);
    common::stopClock("n_cliques", start_time);
    cout << "Number of cliques: " << num_cliques << endl;
  }
};

#ifndef GOOGLE_TEST  // the entry point needs one init_app; test drivers may include several apps
template <class T, class R>
application<T, R>* init_app(Parser input_data) {
  return new n_clique<T, R>(input_data);
}
#endif
