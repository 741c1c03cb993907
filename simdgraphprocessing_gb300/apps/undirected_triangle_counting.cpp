// undirected_triangle_counting<T,R> (the reference's
// apps/undirected_triangle_counting.cpp): same class, members and output line;
// the count is one device launch over the pruned (nbr < node) matrix.
#include "emptyheaded.hpp"

template <class T, class R>
class undirected_triangle_counting : public application<T, R> {
 public:
  size_t num_triangles;

  undirected_triangle_counting(Parser input_data) : application<T, R>(input_data) { num_triangles = 0; }

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
    num_triangles = this->graph->count_triangles();
    common::stopClock("UNDIRECTED TRIANGLE COUNTING", start_time);
    cout << "Number of triangles: " << num_triangles << endl;
  }
};

#ifndef GOOGLE_TEST  // the entry point needs one init_app; test drivers may include several apps
template <class T, class R>
application<T, R>* init_app(Parser input_data) {
  return new undirected_triangle_counting<T, R>(input_data);
}
#endif
