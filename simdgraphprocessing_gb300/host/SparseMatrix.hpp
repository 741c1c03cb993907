// Drop-in SparseMatrix<T,R> (the reference's src/SparseMatrix.hpp): same build
// signature and public fields.  The rows live in device memory: build() turns
// the selection lambdas into an edge mask on the host, then the engine uploads
// the adjacency and selects, optimizes and encodes on the device.  get_row()
// returns host copies of rows in the reference's flattened byte format (made
// on first use; the pattern counts never need them).
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
  uint64_t* id_map;
  eh_matrix_t handle;
  eh_selection selection;

  SparseMatrix(eh_matrix_t h, eh_selection sel, uint64_t* ids)
      : col_total_bytes_used(0), symmetric(true), row_lengths(nullptr), row_arrays(nullptr),
        row_ranges(nullptr), id_map(ids), handle(h), selection(sel) {
    eh_matrix_info info;
    common::check(eh_matrix_get_info(h, &info));
    matrix_size = info.matrix_size;
    cardinality = info.cardinality;
    row_total_bytes_used = info.row_total_bytes_used;
    max_nbrhood_size = info.max_nbrhood_size;
  }
  ~SparseMatrix() {
    eh_matrix_free(handle);
    delete[] row_lengths;
    delete[] row_arrays;
    delete[] host_rows_;
  }

  // SparseMatrix<T,R>::build (src/SparseMatrix.hpp:268-290,406-494): keeps edge
  // (i, nbr) when node_selection(nbr, 0) && edge_selection(i, nbr, 0), as
  // pack_data (:249-266) does.
  static SparseMatrix* build(MutableGraph* g, const std::function<bool(uint32_t, uint32_t)> node_selection,
                             const std::function<bool(uint32_t, uint32_t, uint32_t)> edge_selection,
                             const size_t num_threads) {
    vector<uint64_t> off;
    vector<uint32_t> nbr;
    g->to_csr(off, nbr);
    const size_t n = g->num_nodes;
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
    return new SparseMatrix(h, sel, g->id_map->data());
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

 private:
  uint8_t* host_rows_ = nullptr;

  void materialize_host_rows() {
    if (row_arrays) return;
    vector<uint8_t> types(matrix_size);
    vector<uint64_t> nbytes(matrix_size);
    row_lengths = new uint32_t[matrix_size];
    common::check(eh_matrix_row_meta(handle, types.data(), row_lengths, nbytes.data()));
    uint64_t total = 0;
    common::check(eh_matrix_export_flattened(handle, nullptr, 0, &total));
    host_rows_ = new uint8_t[total + 8];
    common::check(eh_matrix_export_flattened(handle, host_rows_, total, &total));
    row_arrays = new uint8_t*[matrix_size];
    uint64_t pos = 0;
    for (size_t i = 0; i < matrix_size; i++) {
      row_arrays[i] = host_rows_ + pos;
      pos += nbytes[i];
    }
  }
};

#endif
