// Drop-in SparseMatrix<T,R> (the reference's src/SparseMatrix.hpp): same build
// signature and public fields.  The rows live in device memory: build() turns
// the selection lambdas into an edge mask on the host, then the engine uploads
// the adjacency and selects, optimizes and encodes on the device.  get_row()
// returns host copies of rows in the reference's flattened byte format (made
// on first use; the pattern counts never need them).  A directed graph also
// gets a column matrix built from its in-neighbourhoods (get_column).
#ifndef EH_DROPIN_SPARSEMATRIX_HPP
#define EH_DROPIN_SPARSEMATRIX_HPP

#include "MutableGraph.hpp"
#include "set/Set.hpp"

template <class T, class R>
class SparseMatrix {
 public:
  size_t matrix_size;
  size_t cardinality;
  size_t row_total_bytes_used;
  size_t col_total_bytes_used;
  size_t max_nbrhood_size;
  bool symmetric;
  uint32_t* row_lengths;
  uint8_t** row_arrays;
  uint32_t* row_ranges;
  uint32_t* column_lengths;
  uint8_t** column_arrays;
  uint64_t* id_map;
  eh_matrix_t handle;
  eh_matrix_t column_handle;  // == handle for an undirected graph
  eh_selection selection;

  SparseMatrix(eh_matrix_t h, eh_selection sel, uint64_t* ids, eh_matrix_t cols = nullptr)
      : col_total_bytes_used(0), symmetric(cols == nullptr), row_lengths(nullptr), row_arrays(nullptr),
        row_ranges(nullptr), column_lengths(nullptr), column_arrays(nullptr), id_map(ids), handle(h),
        column_handle(cols ? cols : h), selection(sel) {
    eh_matrix_info info;
    common::check(eh_matrix_get_info(h, &info));
    matrix_size = info.matrix_size;
    cardinality = info.cardinality;
    row_total_bytes_used = info.row_total_bytes_used;
    max_nbrhood_size = info.max_nbrhood_size;
    if (cols) {
      common::check(eh_matrix_get_info(cols, &info));
      cardinality += info.cardinality;
      col_total_bytes_used = info.row_total_bytes_used;
    }
  }
  ~SparseMatrix() {
    if (column_handle != handle) {
      eh_matrix_free(column_handle);
      delete[] column_lengths;
      delete[] column_arrays;
      delete[] host_cols_;
    }
    eh_matrix_free(handle);
    delete[] row_lengths;
    delete[] row_arrays;
    delete[] host_rows_;
  }

  // SparseMatrix<T,R>::build (src/SparseMatrix.hpp:268-290,406-494): keeps edge
  // (i, nbr) when node_selection(nbr, 0) && edge_selection(i, nbr, 0), as
  // pack_data (:249-266) does.  A directed graph (from_asymmetric_graph,
  // :648-760) gets its columns from the in-neighbourhoods the same way.
  static SparseMatrix* build(MutableGraph* g, const std::function<bool(uint32_t, uint32_t)> node_selection,
                             const std::function<bool(uint32_t, uint32_t, uint32_t)> edge_selection,
                             const size_t num_threads) {
    vector<uint64_t> off;
    vector<uint32_t> nbr;
    g->to_csr(off, nbr);
    eh_selection sel;
    eh_matrix_t h = encode(g->num_nodes, off, nbr, node_selection, edge_selection, num_threads, &sel);
    eh_matrix_t cols = nullptr;
    if (!g->symmetric) {
      g->to_in_csr(off, nbr);
      eh_selection csel;
      try {
        cols = encode(g->num_nodes, off, nbr, node_selection, edge_selection, num_threads, &csel);
      } catch (...) {
        eh_matrix_free(h);
        throw;
      }
    }
    return new SparseMatrix(h, sel, g->id_map->data(), cols);
  }

  // SparseMatrix::get_max_row_id (src/SparseMatrix.hpp:133-145).
  uint32_t get_max_row_id() {
    uint32_t r = 0;
    common::check(eh_matrix_get_max_row_id(handle, &r));
    std::cout << "MAXIMUM NODE: " << id_map[r] << " INTERNAL ID: " << r << std::endl;
    return r;
  }
  uint32_t get_internal_id(uint64_t external_id) {
    for (size_t i = 0; i < matrix_size; i++)
      if (id_map[i] == external_id) return (uint32_t)i;
    return 0;
  }
  Set<T> get_row(uint32_t row) {
    materialize_host_rows();
    return Set<T>::from_flattened(row_arrays[row], row_lengths[row]);
  }
  Set<R> get_decoded_row(uint32_t row, uint32_t*) {
    materialize_host_rows();
    return Set<R>::from_flattened(row_arrays[row], row_lengths[row]);
  }
  // SparseMatrix::get_column (src/SparseMatrix.hpp:161-165).
  Set<T> get_column(uint32_t column) {
    if (column_handle == handle) return get_row(column);
    if (!column_arrays) materialize(column_handle, column_lengths, column_arrays, host_cols_);
    return Set<T>::from_flattened(column_arrays[column], column_lengths[column]);
  }

  // Pattern counts on the device (one launch each).
  uint64_t count_triangles() {
    uint64_t c = 0;
    common::check(eh_count_triangles(handle, &c, nullptr));
    return c;
  }
  uint64_t count_cliques(uint32_t k) {
    uint64_t c = 0;
    common::check(eh_count_cliques(handle, k, &c, nullptr));
    return c;
  }
  uint64_t count_lollipops() {
    uint64_t c = 0;
    common::check(eh_count_lollipops(handle, &c, nullptr));
    return c;
  }
  uint64_t count_similar_nodes(uint32_t threshold) {
    uint64_t c = 0;
    common::check(eh_similar_nodes(handle, threshold, &c, nullptr));
    return c;
  }
  // Rows whose get_row / get_column Jaccard ratio is above N (apps/symbiosity.cpp:46-58).
  uint64_t count_symbiosity(double N) {
    uint64_t c = 0;
    common::check(eh_symbiosity(handle, column_handle, N, &c, nullptr));
    return c;
  }
  // The n_path BFS along the rows from `start` (apps/n_path.cpp:58-83).
  size_t bfs_path_length(uint32_t start, uint64_t max_depth) {
    uint64_t p = 0;
    common::check(eh_bfs_path_length(handle, start, max_depth, &p, nullptr, nullptr));
    return (size_t)p;
  }

 private:
  uint8_t* host_rows_ = nullptr;
  uint8_t* host_cols_ = nullptr;

  static eh_matrix_t encode(size_t n, const vector<uint64_t>& off, const vector<uint32_t>& nbr,
                            const std::function<bool(uint32_t, uint32_t)>& node_selection,
                            const std::function<bool(uint32_t, uint32_t, uint32_t)>& edge_selection,
                            size_t num_threads, eh_selection* sel_out) {
    vector<uint8_t> mask(nbr.size());
    bool all = true, lower = true;
#pragma omp parallel for schedule(dynamic, 256) num_threads(num_threads > 0 ? (int)num_threads : 1) \
    reduction(&& : all, lower)
    for (int64_t i = 0; i < (int64_t)n; i++) {
      for (uint64_t e = off[i]; e < off[i + 1]; e++) {
        const bool keep = node_selection(nbr[e], 0) && edge_selection((uint32_t)i, nbr[e], 0);
        mask[e] = keep;
        all = all && keep;
        lower = lower && (keep == (nbr[e] < (uint32_t)i));
      }
    }
    const eh_selection sel = all ? EH_SELECT_ALL : lower ? EH_SELECT_LOWER : EH_SELECT_MASK;
    eh_matrix_t h = nullptr;
    common::check(eh_matrix_build(n, off.data(), nbr.data(), sel == EH_SELECT_MASK ? mask.data() : nullptr, sel,
                                  T::engine_layout(), nullptr, &h));
    *sel_out = sel;
    return h;
  }

  void materialize(eh_matrix_t h, uint32_t*& lengths, uint8_t**& arrays, uint8_t*& bytes) {
    vector<uint8_t> types(matrix_size);
    vector<uint64_t> nbytes(matrix_size);
    lengths = new uint32_t[matrix_size];
    common::check(eh_matrix_row_meta(h, types.data(), lengths, nbytes.data()));
    uint64_t total = 0;
    common::check(eh_matrix_export_flattened(h, nullptr, 0, &total));
    bytes = new uint8_t[total + 8];
    common::check(eh_matrix_export_flattened(h, bytes, total, &total));
    arrays = new uint8_t*[matrix_size];
    uint64_t pos = 0;
    for (size_t i = 0; i < matrix_size; i++) {
      arrays[i] = bytes + pos;
      pos += nbytes[i];
    }
  }
  void materialize_host_rows() {
    if (!row_arrays) materialize(handle, row_lengths, row_arrays, host_rows_);
  }
};

#endif
