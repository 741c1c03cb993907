/*
 * eh_gb300.h — C ABI of the GB300 set-intersection pattern engine.
 *
 * Plain pointers and sizes only; no C++ or torch types cross this boundary.
 * Every function returns an eh_status; on failure a message is available from
 * eh_last_error() (thread-local).  Handles are opaque; the library owns the
 * device memory behind them.  A handle may be used from one host thread at a
 * time.  `stream` arguments are cudaStream_t values passed as void* (NULL = the
 * legacy default stream).
 *
 * Each entry point names the reference interface it replaces
 * (chrisaberger/SIMDGraphProcessing, paths relative to that project).
 */
#ifndef EH_GB300_H
#define EH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum eh_status {
  EH_OK = 0,
  EH_ERR_INVALID_ARGUMENT = 1, /* bad handle, size, layout, unsorted row, ... */
  EH_ERR_CUDA = 2,             /* a CUDA runtime call failed */
  EH_ERR_OUT_OF_MEMORY = 3,    /* device or host allocation failed */
  EH_ERR_UNSUPPORTED = 4,      /* layout / pattern combination not provided */
  EH_ERR_IO = 5,               /* file could not be opened / was truncated */
  EH_ERR_DEVICE_CHECK = 6,     /* a device-side bounds or consistency check fired */
  EH_ERR_TIMEOUT = 7,          /* a bounded wait ran out */
  EH_ERR_ADMISSION = 8         /* request rejected by the memory admission rule */
} eh_status;

/* Set layouts.  The numeric values of the first three equal the reference's
 * common::type tags (src/common.hpp:171-181): BITSET=0, PSHORT=1, UINTEGER=2,
 * HYBRID=5.  EH_LAYOUT_HYBRID3 is the optional three-tier optimizer
 * (hybrid::compute_type, src/set/layouts/hybrid.hpp:55-63); EH_LAYOUT_HYBRID is
 * the rule the reference actually runs (hybrid::get_type, hybrid.hpp:73-100). */
typedef enum eh_layout {
  EH_LAYOUT_BITSET = 0,
  EH_LAYOUT_PSHORT = 1,
  EH_LAYOUT_UINTEGER = 2,
  EH_LAYOUT_HYBRID = 5,
  EH_LAYOUT_HYBRID3 = 16
} eh_layout;

/* Edge selections the apps pass to SparseMatrix::build.  LOWER keeps nbr < node
 * (apps/undirected_triangle_counting.cpp:20-23, apps/n_clique.cpp:23-26); ALL
 * keeps every edge (apps/undirected_lollipop_counting.cpp:20-23,
 * apps/similar_nodes.cpp:24-27).  MASK uses a caller-evaluated per-edge mask. */
typedef enum eh_selection {
  EH_SELECT_ALL = 0,
  EH_SELECT_LOWER = 1,
  EH_SELECT_MASK = 2
} eh_selection;

const char* eh_last_error(void);
const char* eh_status_string(eh_status s);
const char* eh_version(void);

/* ------------------------------------------------------------------------- */
/* Host graph: the reference's MutableGraph (src/MutableGraph.hpp:49-93).     */
/* Symmetric adjacency in CSR form: offsets[n+1] (u64), nbrs[offsets[n]] (u32)
 * sorted ascending per row, ext_ids[n] (u64) the external id of each row.     */
/* ------------------------------------------------------------------------- */
typedef struct eh_hgraph* eh_hgraph_t;

/* Copy a CSR adjacency into a new host graph (ext_ids may be NULL: identity). */
eh_status eh_hgraph_from_csr(uint64_t n, const uint64_t* offsets, const uint32_t* nbrs,
                             const uint64_t* ext_ids, eh_hgraph_t* out);
/* MutableGraph::undirectedFromBinary (src/MutableGraph.hpp:316-360). */
eh_status eh_hgraph_read_binary(const char* path, eh_hgraph_t* out);
/* MutableGraph::writeUndirectedToBinary (src/MutableGraph.hpp:298-314). */
eh_status eh_hgraph_write_binary(eh_hgraph_t g, const char* path);
/* MutableGraph::undirectedFromEdgeList (src/MutableGraph.hpp:517-599): text
 * "src dst" pairs; both directions inserted, rows sorted and deduplicated,
 * self-loops kept (as the reference does). */
eh_status eh_hgraph_read_edge_list(const char* path, eh_hgraph_t* out);
/* MutableGraph::reorder_by_degree (src/MutableGraph.hpp:268-272) with the
 * OrderNeighborhoodByDegree order (:20-32) and reassign_ids (:100-123). */
eh_status eh_hgraph_reorder_by_degree(eh_hgraph_t g);
/* Borrowed views of the arrays (valid until the graph is freed or reordered).
 * num_edges = offsets[n] (directed entries, the reference's num_edges). */
eh_status eh_hgraph_view(eh_hgraph_t g, uint64_t* n, uint64_t* num_edges,
                         const uint64_t** offsets, const uint32_t** nbrs,
                         const uint64_t** ext_ids, uint64_t* max_nbrhood_size);
void eh_hgraph_free(eh_hgraph_t g);

/* Directed host graphs (MutableGraph with symmetric == false): the CSR above
 * holds the out-neighbourhoods, a second CSR the in-neighbourhoods.
 * MutableGraph::directedFromBinary (src/MutableGraph.hpp:656-714): per node
 * u64 ext id, size_t out_len, u32 out[out_len], size_t in_len, u32 in[in_len]. */
eh_status eh_hgraph_read_directed_binary(const char* path, eh_hgraph_t* out);
/* MutableGraph::writeDirectedToBinary (src/MutableGraph.hpp:634-654).  An
 * undirected graph is written with in = out. */
eh_status eh_hgraph_write_directed_binary(eh_hgraph_t g, const char* path);
/* MutableGraph::directedFromEdgeList (src/MutableGraph.hpp:893-986): text
 * "src dst" pairs, ids interned in order of first appearance, out and in rows
 * sorted and deduplicated, self-loops kept. */
eh_status eh_hgraph_read_directed_edge_list(const char* path, eh_hgraph_t* out);
/* A directed graph from its out-CSR (rows sorted ascending, no duplicates);
 * the in-CSR is built as its transpose.  ext_ids may be NULL (identity). */
eh_status eh_hgraph_directed_from_csr(uint64_t n, const uint64_t* out_offsets, const uint32_t* out_nbrs,
                                      const uint64_t* ext_ids, eh_hgraph_t* out);
/* In-neighbourhood CSR (the reference's SparseMatrix::get_column source).
 * *directed = 0 for an undirected graph, whose in-CSR is its CSR. */
eh_status eh_hgraph_in_view(eh_hgraph_t g, int* directed, uint64_t* num_edges,
                            const uint64_t** in_offsets, const uint32_t** in_nbrs);

/* Seeded generators (no reference counterpart; the reference has none).
 * All draw from a counter-based SplitMix64 stream so that the same call gives
 * the same graph on any host.  Output: symmetric, deduplicated, self-loops
 * removed, vertex ids as generated (call eh_hgraph_reorder_by_degree next).
 * R-MAT keeps the first `num_edges` distinct undirected edges in draw order.
 * ER is G(n, M): `num_edges` distinct uniform pairs.  BA attaches each new
 * vertex to m distinct earlier vertices by degree-proportional choice.  The
 * planted graph is an ER background plus `num_cliques` cliques whose sizes are
 * log-uniform integers in [min_size, max_size] over random vertex subsets. */
eh_status eh_generate_rmat(uint32_t scale, uint64_t num_edges, double a, double b, double c,
                           uint64_t seed, eh_hgraph_t* out);
eh_status eh_generate_er(uint64_t n, uint64_t num_edges, uint64_t seed, eh_hgraph_t* out);
eh_status eh_generate_ba(uint64_t n, uint32_t m, uint64_t seed, eh_hgraph_t* out);
eh_status eh_generate_planted_cliques(uint64_t n, uint64_t background_edges, uint32_t num_cliques,
                                      uint32_t min_size, uint32_t max_size, uint64_t seed,
                                      eh_hgraph_t* out);
/* Directed R-MAT: the first `num_edges` distinct ordered pairs (u, v), u != v,
 * in draw order, as a directed graph (out- and in-CSR). */
eh_status eh_generate_directed_rmat(uint32_t scale, uint64_t num_edges, double a, double b, double c,
                                    uint64_t seed, eh_hgraph_t* out);

/* Device ingestion: the work of MutableGraph::undirectedFromEdgeList
 * (src/MutableGraph.hpp:517-599) and reorder_by_degree (:268-272) on the GPU.
 * num_edges pairs (d_src[e], d_dst[e]) of vertex ids < n in device memory become
 * a symmetric CSR with sorted, deduplicated rows; self-loops are kept as the
 * reference's loader keeps them unless drop_self_loops.  degree_order relabels
 * by descending degree, ties by ascending id, and d_new2old (from eh_dcsr_view)
 * then maps new ids to input ids.  The CSR feeds eh_matrix_build_device. */
typedef struct eh_dcsr* eh_dcsr_t;
eh_status eh_dcsr_from_edges(uint64_t n, uint64_t num_edges, const uint32_t* d_src, const uint32_t* d_dst,
                             int drop_self_loops, int degree_order, void* stream, eh_dcsr_t* out);
eh_status eh_dcsr_view(eh_dcsr_t g, uint64_t* n, uint64_t* num_entries, const uint64_t** d_offsets,
                       const uint32_t** d_nbrs, const uint32_t** d_new2old);
void eh_dcsr_free(eh_dcsr_t g);

/* ------------------------------------------------------------------------- */
/* Device matrix: the reference's SparseMatrix<T,R> (src/SparseMatrix.hpp).  */
/* ------------------------------------------------------------------------- */
typedef struct eh_matrix* eh_matrix_t;

typedef struct eh_matrix_info {
  uint64_t matrix_size;          /* rows (SparseMatrix::matrix_size)                  */
  uint64_t cardinality;          /* selected edges (SparseMatrix::cardinality)       */
  uint64_t row_total_bytes_used; /* bytes of all rows in the reference's flattened
                                    format (SparseMatrix::row_total_bytes_used)       */
  uint64_t max_nbrhood_size;     /* max full-graph row length (as the reference)    */
  uint64_t max_row_cardinality;  /* max selected row length                          */
  uint64_t num_uint_rows;        /* rows encoded per layout (common::num_uint etc.) */
  uint64_t num_pshort_rows;
  uint64_t num_bitset_rows;
  uint64_t device_bytes;         /* device memory held by the matrix                 */
  int32_t layout;                /* eh_layout                                        */
  int32_t selection;             /* eh_selection                                     */
} eh_matrix_info;

/* SparseMatrix<T,R>::build -> from_symmetric_noattribute_graph
 * (src/SparseMatrix.hpp:268-290,406-494) and pack_data (:249-266).
 * Host pointers; the adjacency is copied to the device in chunks of rows on an
 * internal upload stream, and selected, layout-optimized and encoded there,
 * each chunk's first pass starting on `stream` as soon as it has landed (the
 * copy overlaps the build when the host buffers are pinned).  `edge_mask` (u8
 * per entry of nbrs) is read only for EH_SELECT_MASK and may be NULL
 * otherwise. */
eh_status eh_matrix_build(uint64_t n, const uint64_t* offsets, const uint32_t* nbrs,
                          const uint8_t* edge_mask, eh_selection sel, eh_layout layout,
                          void* stream, eh_matrix_t* out);
/* Same, with offsets / nbrs / edge_mask already in device memory. */
eh_status eh_matrix_build_device(uint64_t n, const uint64_t* d_offsets, const uint32_t* d_nbrs,
                                 const uint8_t* d_edge_mask, eh_selection sel, eh_layout layout,
                                 void* stream, eh_matrix_t* out);
eh_status eh_matrix_get_info(eh_matrix_t m, eh_matrix_info* info);
/* Per-row layout tag (common::type), cardinality (row_lengths) and flattened
 * byte count, copied to host arrays of matrix_size entries (any may be NULL). */
eh_status eh_matrix_row_meta(eh_matrix_t m, uint8_t* types, uint32_t* cards, uint64_t* nbytes);
/* Row `row` in the reference's flattened byte format, exactly as
 * T::build_flattened writes it (hybrid.hpp:132-166, bitset.hpp:99-109,
 * pshort.hpp:81-91, uinteger.hpp:56-59).  *nbytes receives the size; nothing is
 * written if cap is too small (EH_ERR_INVALID_ARGUMENT). */
eh_status eh_matrix_export_row(eh_matrix_t m, uint32_t row, uint8_t* buf, uint64_t cap,
                               uint64_t* nbytes);
/* Every row's flattened bytes back to back in row order (the contents of the
 * reference's row_arrays, src/SparseMatrix.hpp:406-494).  Call with buf=NULL to
 * get the size in *nbytes; EH_ERR_INVALID_ARGUMENT if cap is too small. */
eh_status eh_matrix_export_flattened(eh_matrix_t m, uint8_t* buf, uint64_t cap, uint64_t* nbytes);
/* SparseMatrix::get_max_row_id (src/SparseMatrix.hpp:133-145). */
eh_status eh_matrix_get_max_row_id(eh_matrix_t m, uint32_t* row);
/* Algorithmic bytes of one triangle-count pass:
 * sum_i [8 + bytes(A_i)] + sum_{(i,j) selected} bytes(B_j), bytes = layout payload. */
eh_status eh_matrix_triangle_bytes(eh_matrix_t m, uint64_t* bytes);
/* Returns the matrix's memory to the library's pools (each keeps up to 16 GiB
 * of freed memory mapped per device), stream-ordered: once every launch the
 * library made on the matrix, on any stream, has finished; the host and
 * unrelated streams do not wait. */
void eh_matrix_free(eh_matrix_t m);

/* ------------------------------------------------------------------------- */
/* Pattern counts.  The synchronous forms write the count to host memory; the  */
/* _async forms write it to device memory on `stream` without synchronizing.   */
/* ------------------------------------------------------------------------- */
/* undirected_triangle_counting<T,R>::run (apps/undirected_triangle_counting.cpp:27-65):
 * sum_i sum_{j in row(i)} |row(i) ∩ row(j)|.  Matrix built with EH_SELECT_LOWER. */
eh_status eh_count_triangles(eh_matrix_t m, uint64_t* count, void* stream);
eh_status eh_count_triangles_async(eh_matrix_t m, uint64_t* d_count, void* stream);
/* n_clique<T,R>::run / apply_function (apps/n_clique.cpp:30-101), k >= 3. */
eh_status eh_count_cliques(eh_matrix_t m, uint32_t k, uint64_t* count, void* stream);
eh_status eh_count_cliques_async(eh_matrix_t m, uint32_t k, uint64_t* d_count, void* stream);
/* No counterpart in the reference.  The same count as eh_count_cliques_async,
 * for callers that may not allocate device memory when they count: a serving
 * loop that reserves its whole device-memory budget at start-up and must not
 * grow its footprint or meet an allocation failure mid-request, or a host
 * framework that owns every device allocation (cudaFree also synchronizes the
 * device).  Nothing is allocated: the largest pivots' scratch slots and the
 * work counters come from one fixed 16 MiB array in device memory, held by
 * every GPU that loads the library until exit; a pivot needing a larger slot is
 * rejected with EH_ERR_UNSUPPORTED.  The matrix must already have its work plan
 * (made by its first eh_count_* call), else EH_ERR_INVALID_ARGUMENT.  The first
 * call on a device looks up the array's address (cudaGetSymbolAddress) and
 * should come before any stream capture; the address is kept for the life of
 * the process, so the device must not be reset (cudaDeviceReset) after that
 * first call.  All calls share the array: calls whose kernels overlap on the
 * GPU race.  It runs the shared-memory tier as one launch sized for its
 * largest pivot (eh_count_cliques splits it into size bands), so on skewed
 * graphs it can be slower than eh_count_cliques.  eh_matrix_free does not wait
 * for these launches: synchronize their stream before freeing the matrix. */
eh_status eh_count_cliques_noalloc(eh_matrix_t m, uint32_t k, uint64_t* d_count, void* stream);
/* undirected_lollipop_counting<T,R>::run (apps/undirected_lollipop_counting.cpp:27-77).
 * Matrix built with EH_SELECT_ALL. */
eh_status eh_count_lollipops(eh_matrix_t m, uint64_t* count, void* stream);
eh_status eh_count_lollipops_async(eh_matrix_t m, uint64_t* d_count, void* stream);
/* similar_nodes<T,R>::run (apps/similar_nodes.cpp:29-68): rows i with
 * |row(v*) ∩ row(i)| > threshold, v* = get_max_row_id().  EH_SELECT_ALL. */
eh_status eh_similar_nodes(eh_matrix_t m, uint32_t threshold, uint64_t* count, void* stream);
eh_status eh_similar_nodes_async(eh_matrix_t m, uint32_t threshold, uint64_t* d_count,
                                 void* stream);
/* Triangle tuples, as undirected_triangle_counting would emit them with tuple
 * output (Table<T>::write_table, src/Table.hpp:30-43): every (i, j, k) with
 * i > j > k, j in row(i), k in row(i) ∩ row(j), written as three u32 row ids
 * to d_out[3t .. 3t+2] for t < capacity, in no particular order; *d_total (device)
 * receives the number of triangles (tuples past capacity are counted, not
 * written).  Map rows to external ids with the graph's id map.  Matrix built
 * with EH_SELECT_LOWER. */
eh_status eh_list_triangles(eh_matrix_t m, uint32_t* d_out, uint64_t capacity, uint64_t* d_total,
                            void* stream);
/* Clique tuples, as n_clique<T,R> writes them with WRITE_TABLE
 * (apps/n_clique.cpp:30-50: at the last level Table<T>::write_table appends one
 * tuple per element of C, src/Table.hpp:30-43): every k-clique (x_1, ..., x_k)
 * with x_1 > x_2 > ... > x_k, x_1 the pivot row and the others entries of
 * row(x_1) in descending order, written as k u32 row ids to
 * d_out[k*t .. k*t+k-1] for t < capacity, in no particular order; *d_total
 * (device) receives the number of cliques, which equals eh_count_cliques(m, k)
 * (tuples past capacity are counted, not written).  k = 3 or 4
 * (EH_ERR_UNSUPPORTED otherwise).  Matrix built with EH_SELECT_LOWER. */
eh_status eh_list_cliques(eh_matrix_t m, uint32_t k, uint32_t* d_out, uint64_t capacity, uint64_t* d_total,
                          void* stream);
/* ops::set_intersect on rows (src/set/ops/intersection.hpp, dispatcher :2067-2117):
 * d_counts[p] = |row(d_a[p]) ∩ row(d_b[p])| for p < npairs (device arrays);
 * a pair that names a row >= matrix_size gets 0xffffffff. */
eh_status eh_intersect_rows(eh_matrix_t m, const uint32_t* d_a, const uint32_t* d_b,
                            uint64_t npairs, uint32_t* d_counts, void* stream);
/* symbiosity<T,R>::run (apps/symbiosity.cpp:39-58): rows i with
 * |out(i) ∩ in(i)| / (|out(i)| + |in(i)| - |out(i) ∩ in(i)|) > threshold, the
 * ratio in double precision (0/0 counts as not above).  `rows` holds the
 * out-neighbourhoods (SparseMatrix::get_row), `cols` the in-neighbourhoods
 * (get_column; pass `rows` again for an undirected graph).  Both EH_SELECT_ALL,
 * same matrix_size and device; the reference's threshold is 0.5. */
eh_status eh_symbiosity(eh_matrix_t rows, eh_matrix_t cols, double threshold, uint64_t* count,
                        void* stream);
eh_status eh_symbiosity_async(eh_matrix_t rows, eh_matrix_t cols, double threshold,
                              uint64_t* d_count, void* stream);
/* n_path<T,R>::run (apps/n_path.cpp:30-88): breadth-first search along rows
 * from `start`; each level ORs the rows of the frontier into the visited
 * bitset (ops::set_union, src/set/ops/union.hpp) and the next frontier is the
 * newly set bits (ops::set_difference, src/set/ops/difference.hpp:5-84).
 * *path_length = the number of levels that found new vertices, stopping once
 * it reaches max_depth (the reference's --n; 0xeffffff when not given).
 * *reached (may be NULL) = vertices visited, start included.  EH_SELECT_ALL. */
eh_status eh_bfs_path_length(eh_matrix_t m, uint32_t start, uint64_t max_depth, uint64_t* path_length,
                             uint64_t* reached, void* stream);

/* ------------------------------------------------------------------------- */
/* Work-shape autotuning (no reference counterpart).                           */
/* ------------------------------------------------------------------------- */
typedef struct eh_tuning {
  uint32_t light_max;     /* pivots with at most this many entries (2..160) run one
                             per warp                                               */
  uint32_t unit_span;     /* pivot positions per CTA work unit for larger pivots    */
  uint32_t ctas_per_sm;   /* resident CTAs per SM of the persistent count kernel     */
  uint32_t core_rows;     /* highest-degree rows kept as a dense bitmap (0 = none)   */
  float ms;               /* median triangle-count time with the chosen shape        */
  uint32_t configs_tried;
  uint32_t core_hot_words; /* light-pivot probes of the first words of each dense-core
                              row keep their L2 lines, the rest are evicted first
                              (0 = no cache hints)                                  */
  uint32_t core_filter_words; /* words of the per-row hashed filter checked before a
                              light-pivot probe reads a dense-core word: 0 (none),
                              16, 32 or 64                                          */
} eh_tuning;
/* Times the triangle count (EH_SELECT_LOWER) or the lollipop count
 * (EH_SELECT_ALL) on this matrix for a small set of work shapes, coordinate by
 * coordinate, keeps the fastest for later counts, and caches it per (GPU,
 * layout, selection, size bucket) in the process (and in the file named by
 * EH_TUNE_CACHE, if set). */
eh_status eh_matrix_tune(eh_matrix_t m, void* stream, eh_tuning* result);
/* As eh_matrix_tune, for matrices that are built, counted counts_per_build
 * times and freed: each shape is ranked by its count time plus the one-shot
 * cost of its own plan parts (heavy work units, dense core, row filters; host
 * time, median of 3 builds) divided by counts_per_build, so a large core that
 * saves less per count than it costs to build loses.  0 ranks by count time
 * alone (eh_matrix_tune).  The choice is cached per counts_per_build beside
 * eh_matrix_tune's and is not applied to other matrices by itself: pass it to
 * eh_matrix_set_shape after each build.  result->ms is the count time.  (No
 * reference counterpart.) */
eh_status eh_matrix_tune_for(eh_matrix_t m, uint32_t counts_per_build, void* stream, eh_tuning* result);
/* Uses the given work shape (light_max, unit_span, ctas_per_sm, core_rows,
 * core_hot_words, core_filter_words of `shape`; ms and configs_tried are
 * ignored) for this matrix's later counts, rebuilding its plan as needed; a
 * cached tuned shape no longer applies to this matrix.  Counts do not depend
 * on the shape.  EH_ERR_INVALID_ARGUMENT for a value outside the tuner's
 * ranges (light_max 2..160, unit_span 1..65536, ctas_per_sm 1..the kernel's
 * occupancy, core_rows <= 262,144, core_filter_words 0/16/32/64).  (No
 * reference counterpart.) */
eh_status eh_matrix_set_shape(eh_matrix_t m, const eh_tuning* shape, void* stream);

/* ------------------------------------------------------------------------- */
/* Batches: many graphs counted in one launch (no reference counterpart; each   */
/* graph's count is what the reference's apps compute for it alone).           */
/* ------------------------------------------------------------------------- */
typedef struct eh_batch* eh_batch_t;
/* Graph g owns rows [graph_rows[g], graph_rows[g+1]) of one symmetric CSR over
 * all n rows (host arrays); its neighbour ids are global row ids inside that
 * range (an edge leaving its block is EH_ERR_INVALID_ARGUMENT). */
eh_status eh_batch_build(uint32_t num_graphs, const uint64_t* graph_rows, uint64_t n,
                         const uint64_t* offsets, const uint32_t* nbrs, eh_layout layout,
                         void* stream, eh_batch_t* out);
/* d_counts[g] (device, num_graphs entries) = k-clique count of graph g; k = 3
 * runs the triangle kernel. */
eh_status eh_batch_count(eh_batch_t b, uint32_t k, uint64_t* d_counts, void* stream);
/* Triangles and 4-cliques of every graph.  use_graph != 0: the launches are
 * captured into a CUDA graph on first use (for these output pointers) and
 * replayed afterwards; needs a non-default stream. */
eh_status eh_batch_run(eh_batch_t b, uint64_t* d_triangles, uint64_t* d_cliques4, int use_graph,
                       void* stream);
eh_status eh_batch_tune(eh_batch_t b, void* stream, eh_tuning* result);
/* Borrowed handle of the batch's union matrix (owned by the batch). */
eh_status eh_batch_matrix(eh_batch_t b, eh_matrix_t* m);
void eh_batch_free(eh_batch_t b);

/* ------------------------------------------------------------------------- */
/* Serving loop (no reference counterpart).  Graphs stay resident on the       */
/* device; queries run with continuous batching: each is launched as soon as a */
/* slot (stream + scratch) is free and its scratch fits under the HBM cap, so  */
/* queries arriving while others run overlap with them on the device.          */
/* ------------------------------------------------------------------------- */
typedef struct eh_server* eh_server_t;
typedef struct eh_server_config {
  uint32_t slots;          /* concurrent queries on the device (1..64)            */
  uint64_t hbm_cap_bytes;  /* resident matrices + query scratch never exceed this
                            * (the library's two pools may each keep up to
                            * 16 GiB of freed memory mapped on top of it)        */
} eh_server_config;
typedef enum eh_query_kind {
  EH_QUERY_TRIANGLES = 0,     /* param unused                                    */
  EH_QUERY_CLIQUES = 1,       /* param = clique size k                           */
  EH_QUERY_SIMILAR_NODES = 2  /* param = threshold N (apps/similar_nodes.cpp:14) */
} eh_query_kind;
typedef struct eh_query_result {
  uint64_t count;
  int32_t status;          /* eh_status of the query                              */
  int32_t slot;            /* slot that ran it                                    */
  int64_t submit_ns, start_ns, done_ns;  /* steady-clock times: latency = done - submit */
} eh_query_result;
typedef struct eh_server_stats {
  uint32_t graphs, slots;
  uint64_t queued, completed, launched, max_inflight;
  uint64_t resident_bytes, scratch_bytes, hbm_cap_bytes;
} eh_server_counters;
/* Starts the dispatcher thread on the current device. */
eh_status eh_server_create(const eh_server_config* cfg, eh_server_t* out);
/* Uploads a symmetric CSR (host arrays) and keeps both matrices the queries
 * need resident (nbr < node rows and full rows).  EH_ERR_ADMISSION when they
 * do not fit under the cap. */
eh_status eh_server_add_graph(eh_server_t s, uint64_t n, const uint64_t* offsets, const uint32_t* nbrs,
                              eh_layout layout, uint32_t* graph_id);
eh_status eh_server_submit(eh_server_t s, uint32_t graph_id, eh_query_kind kind, uint32_t param,
                           uint64_t* ticket);
/* Waits at most timeout_ms (EH_ERR_TIMEOUT otherwise) and releases the ticket. */
eh_status eh_server_wait(eh_server_t s, uint64_t ticket, uint32_t timeout_ms, eh_query_result* out);
/* The same query run by itself on the default stream (for one-at-a-time
 * baselines and alone-vs-mix checks); call while no submitted work is pending. */
eh_status eh_server_run_alone(eh_server_t s, uint32_t graph_id, eh_query_kind kind, uint32_t param,
                              uint64_t* count);
eh_status eh_server_stats(eh_server_t s, eh_server_counters* out);
/* Finishes queued and running queries, stops the dispatcher, frees everything. */
void eh_server_free(eh_server_t s);

/* ------------------------------------------------------------------------- */
/* Diagnostics (no reference counterpart).                                     */
/* ------------------------------------------------------------------------- */
/* Runs one kernel that waits on an mbarrier nothing arrives on, with the
 * bounded wait the bulk-copy staging uses, limited to `tries` polls
 * (1..65536); *timed_out = 1 when the wait gave up and the kernel reported it
 * (the expected outcome).  Shows that a stuck device-side wait ends with a
 * status instead of a hang. */
eh_status eh_selftest_bounded_wait(uint32_t tries, uint32_t* timed_out);

#ifdef __cplusplus
}
#endif

#endif /* EH_GB300_H */
