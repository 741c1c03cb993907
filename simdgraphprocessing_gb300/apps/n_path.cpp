// n_path<T,R> (the reference's apps/n_path.cpp): same class, members and
// output lines; breadth-first search along the rows from the start node (the
// largest row unless --start_node names one), on the device.
#include "emptyheaded.hpp"

template <class T, class R>
class n_path : public application<T, R> {
 public:
  size_t path_length;

  n_path(Parser input_data) : application<T, R>(input_data) { path_length = 0; }

  SparseMatrix<T, R>* materialize_graph() {
    auto node_selection = [](uint32_t node, uint32_t attribute) -> bool {
      (void)node;
      (void)attribute;
      return true;
    };
    auto edge_selection = [](uint32_t node, uint32_t nbr, uint32_t attribute) -> bool {
      (void)node;
      (void)nbr;
      (void)attribute;
      return true;
    };
    return SparseMatrix<T, R>::build(this->input_graph, node_selection, edge_selection, this->num_threads);
  }

  void run() {
    this->graph = materialize_graph();
    SparseMatrix<T, R>* graph = this->graph;
    uint32_t internal_start;
    if (this->start_node == -1)
      internal_start = graph->get_max_row_id();
    else
      internal_start = graph->get_internal_id(this->start_node);
    cout << "Start node - External: " << graph->id_map[internal_start] << " Internal: " << internal_start << endl;
    const double pure_bfs_time = common::startClock();
    path_length = graph->bfs_path_length(internal_start, this->query_depth);
    common::stopClock("pure bfs time", pure_bfs_time);
    cout << "path length: " << path_length << endl;
  }
};

#ifndef GOOGLE_TEST  // the entry point needs one init_app; test drivers may include several apps
template <class T, class R>
application<T, R>* init_app(Parser input_data) {
  return new n_path<T, R>(input_data);
}
#endif
