// Kernel declarations shared between the build / count translation units and
// the C-ABI layer.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "eh_device.cuh"

namespace eh {

// Device error flag bits (set by kernels, read by the host after a launch).
enum : uint32_t {
  ERRF_UNSORTED = 1u,      // a row is not strictly ascending
  ERRF_RANGE = 2u,         // a neighbour id >= n
  ERRF_ROW_TOO_LONG = 4u,  // a row exceeds the 2^30 element limit of RowDesc
  ERRF_PSHORT_PART = 8u,   // a pshort partition would exceed 65536 elements
  ERRF_OFFSETS = 16u,      // offsets fall, or run past the neighbour array
};

// Per-row measurements produced by the build's first pass.
struct RowMeasure {
  uint32_t card;   // selected elements
  uint32_t aux;    // bitset: first word; pshort: partitions
  uint32_t lt;     // type | length (RowDesc::lt)
  uint32_t units;  // payload size in 16-byte units
};

struct BuildTotals {  // accumulated with atomics by the measure pass
  unsigned long long cardinality;
  unsigned long long ref_bytes;  // reference flattened bytes of all rows
  unsigned long long num_uint, num_pshort, num_bitset;
  unsigned long long max_full_degree;
  unsigned long long max_card;
  unsigned long long payload_units;
};

// eh_build.cu
// Pass 1 over rows [r_begin, r_end) of an n-row matrix (a launch per uploaded
// chunk of rows, or one for all): rows up to 4,096 entries are measured by a
// warp each; longer rows are appended to big / n_big (at most
// big_row_capacity(n, total) of them).  launch_measure_big measures the list
// entries [*big_begin, *big_end) by whole CTAs (device words, read when the
// kernel runs: the rows a range appended, or all of them).
cudaError_t launch_measure_rows(uint64_t n, uint64_t total, uint64_t r_begin, uint64_t r_end, const uint64_t* off,
                                const uint32_t* nbr, const uint8_t* mask, int sel, int layout, RowMeasure* meas,
                                BuildTotals* totals, uint32_t* err, uint32_t* big, uint32_t* n_big, cudaStream_t st);
cudaError_t launch_measure_big(uint64_t n, const uint64_t* off, const uint32_t* nbr, const uint8_t* mask, int sel,
                               int layout, RowMeasure* meas, BuildTotals* totals, uint32_t* err, const uint32_t* big,
                               const uint32_t* big_begin, const uint32_t* big_end, cudaStream_t st);
uint64_t big_row_capacity(uint64_t n, uint64_t total);
cudaError_t launch_scan_units(uint64_t n, const RowMeasure* meas, uint32_t* off16, uint32_t* block_tmp,
                              uint64_t n_block_tmp, cudaStream_t st);
uint64_t scan_tmp_words(uint64_t n);
cudaError_t launch_encode(uint64_t n, const uint64_t* off, const uint32_t* nbr, const uint8_t* mask,
                          int sel, const RowMeasure* meas, const uint32_t* off16, RowDesc* desc,
                          uint4* arena, const uint32_t* big, const uint32_t* n_big, cudaStream_t st);
// Work plan: rows with card >= min_card sorted by descending card.
// hist: 65536 + scan_tmp_words(65536) words; after the call hist[0..65536) holds
// the bin starts and cursor[0..65536) the bin ends (bin b = card 65535 - b).
cudaError_t launch_plan(uint64_t n, const RowDesc* desc, uint32_t min_card, uint32_t* hist,
                        uint32_t* order, uint32_t* cursor, cudaStream_t st);
cudaError_t exclusive_scan_u32(const uint32_t* in, uint64_t n, uint32_t* out, uint32_t* tmp,
                               cudaStream_t st);
cudaError_t launch_gather_desc(const RowDesc* desc, const uint32_t* rows, uint32_t nrows, RowDesc* out,
                               cudaStream_t st);
cudaError_t launch_decode_rows(const RowDesc* desc, const uint4* arena, const uint32_t* rows,
                               const unsigned long long* dst_off, uint32_t nrows, uint32_t* dst,
                               cudaStream_t st);
cudaError_t launch_triangle_bytes(uint64_t n, const RowDesc* desc, const uint4* arena,
                                  unsigned long long* out, cudaStream_t st);

// eh_count.cu
struct PivotArgs {
  const RowDesc* desc;
  const uint4* arena;
  const uint32_t* order;   // rows sorted by descending card
  uint32_t n_order;        // rows in the plan
  uint32_t n_heavy;        // order[0, n_heavy) are processed CTA-wide
  uint32_t n_giant;        // order[0, n_giant) have decoded lists in giant_lists
  const uint32_t* giant_lists;
  const unsigned long long* giant_off;
  uint32_t* counters;      // [0] next heavy unit, [1] next light chunk, [15] device error flags
  unsigned long long* out; // result; in batch mode out[num_graphs]
  uint32_t unit_span;      // pivot positions e per heavy unit
  const uint32_t* graph_rows;  // batch mode: graph g owns rows [graph_rows[g], graph_rows[g+1]); else null
  uint32_t num_graphs;
  const unsigned long long* core;  // dense core bitmap of rows j < core_k (see core_row_offset), or null
  uint32_t core_k;
  uint32_t core_hot_words;  // light-pivot core probes of words below this keep their L2 lines (0: no hints)
  const unsigned long long* filter;  // row filters of rows [kFilterLo, filter_k), or null (see filter_bit)
  uint32_t filter_words;             // words per row filter (16, 32 or 64)
  uint32_t filter_k;
};
constexpr uint32_t kCtaThreads = 256;
constexpr uint32_t kLightMax = 160;    // largest light_max: warp-wide pivots fit a slice of this size
constexpr uint32_t kDefaultLightMax = 96;
constexpr uint32_t kDefaultUnitSpan = 128;
constexpr uint32_t kCtaListCap = 2048; // CTA-staged list capacity (elements)
constexpr uint32_t kCtaWordCap = 1024; // CTA-staged bitset words capacity
cudaError_t launch_pivot_units(const RowDesc* desc, const uint32_t* order, uint32_t n_heavy,
                               uint32_t unit_span, uint32_t* cnt, cudaStream_t st);
cudaError_t launch_pivot_unit_fill(const uint32_t* cnt, const uint32_t* start, uint32_t n_heavy,
                                   uint2* units, cudaStream_t st);
cudaError_t launch_triangles(const PivotArgs& a, const uint2* units, uint32_t n_units, int grid,
                             cudaStream_t st);
cudaError_t launch_lollipops(const PivotArgs& a, const uint2* units, uint32_t n_units, int grid,
                             cudaStream_t st);
int pivot_grid(int device);  // persistent grid: SMs x resident CTAs of the pivot kernel

// Dense core: for every row j < core_k, the bits of row(j) ∩ [0, j) packed in
// ceil(j/64) words starting at word core_row_offset(j) (a lower-triangular
// bitmap of the highest-degree rows, which degree ordering puts first).
constexpr uint32_t kCoreMaxK = 262144;     // 4.3 GB of bits, the largest core a shape may ask for
constexpr uint32_t kCoreDefaultK = 65536;  // 268 MB: the core of a matrix the tuner has not seen
// Heavy pivots keep their elements below min(core_k, kCoreAndMax) as bits in
// shared memory, to AND with core rows in that range.
constexpr uint32_t kCoreAndMax = 65536;
__host__ __device__ inline uint64_t core_row_offset(uint32_t j) {
  if (j == 0) return 0;
  const uint64_t a = (uint64_t)(j - 1) >> 6, b = (uint64_t)(j - 1) & 63;
  return 32 * a * (a + 1) + b * (a + 1);  // sum over x < j of ceil(x / 64)
}
cudaError_t launch_core_build(const RowDesc* desc, const uint4* arena, uint32_t core_k, unsigned long long* core,
                              cudaStream_t st);

// Core row filters: for every core row j in [kFilterLo, filter_k = core_k), a
// bitmap of filter_words * 64 bits with bit filter_bit(x) set for each x in
// row(j) ∩ [0, j) (Fibonacci hashing: the top bits of x * 2^32 / phi).  A light
// pivot's probe (j, x) reads the filter word first and the core word only when
// the bit is set, so a probe that misses (about 91% of them at R-MAT scale 22)
// costs one word of the small filter, loaded with the L2 keep hint, instead of
// a DRAM sector of the core; that makes a larger core pay (at scale 22 the
// tuner picks 262,144 rows with filters, 8.35 ms per count, against 98,304
// rows without, 8.86 ms).  A set bit is only a hint: the core word decides, so
// counts are exact.  Rows below kFilterLo form a core block small enough to
// stay in L2 and have no filter.  (Filters on rows past the core, falling back
// to the row's binary search, measured no faster.)
constexpr uint32_t kFilterLo = 4096;
__host__ __device__ inline uint32_t filter_bit(uint32_t x, uint32_t filter_words) {
  const uint32_t log2_bits = filter_words == 16 ? 10u : filter_words == 32 ? 11u : 12u;
  return (x * 2654435769u) >> (32 - log2_bits);
}
cudaError_t launch_filter_build(const RowDesc* desc, const uint4* arena, uint32_t filter_k, uint32_t filter_words,
                                unsigned long long* filter, cudaStream_t st);
cudaError_t launch_similar(uint64_t n, const RowDesc* desc, const uint4* arena, uint32_t vstar,
                           uint32_t threshold, unsigned long long* out, cudaStream_t st);
cudaError_t launch_intersect_rows(uint64_t n, const RowDesc* desc, const uint4* arena, const uint32_t* a,
                                  const uint32_t* b, uint64_t np, uint32_t* counts, cudaStream_t st);
cudaError_t launch_max_row(uint64_t n, const RowDesc* desc, unsigned long long* out, cudaStream_t st);

// eh_clique.cu
struct CliqueArgs {
  const RowDesc* desc;
  const uint4* arena;
  const uint32_t* order;   // rows sorted by descending card
  uint32_t k;              // clique size, 3 <= k <= kCliqueMaxK
  unsigned long long* out; // result; in batch mode out[num_graphs]
  const uint32_t* graph_rows;  // batch mode: graph g owns rows [graph_rows[g], graph_rows[g+1]); else null
  uint32_t num_graphs;
  const unsigned long long* core;  // dense core bitmap (rows j < core_k), or null
  uint32_t core_k;
  // Tuple output (the list kernels, k = 3 or 4): clique j of the count goes to
  // tuples[k*j .. k*j+k-1] when j < capacity; out[0] is the count and the
  // cursor that hands out j.
  uint32_t* tuples;
  uint64_t capacity;
};
constexpr uint32_t kCliqueMaxK = 16;
// Largest pivot row a clique count accepts: a pivot's packed masks are indexed
// with 32-bit word offsets, which stay exact below 2^18 entries (a degree-
// ordered graph reaches that only past 2^35 edges).
constexpr uint32_t kCliqueMaxPivot = 1u << 18;
constexpr uint32_t kCliqueSmemMax = 2048;  // no pivot above this size keeps its masks in shared memory
// Words of one pivot's working set (list, masks, per-warp DFS stacks).
uint64_t clique_slot_words(uint32_t cmax, uint32_t k);
cudaError_t launch_clique_light(const CliqueArgs& a, uint32_t pos_begin, uint32_t pos_end, uint32_t* counter,
                                int grid, cudaStream_t st, bool list = false);
// Largest pivot (<= kCliqueSmemMax) whose k-clique working set fits one CTA's
// opt-in shared memory on `device`; larger pivots use global scratch slots.
uint32_t clique_smem_cap(uint32_t k, int device);
// gscratch == nullptr: masks in dynamic shared memory (grid <= 0: as many CTAs
// as fit on the GPU, at most one per pivot); else grid slots of
// clique_slot_words(cmax, k) words each in global memory.
cudaError_t launch_clique_cta(const CliqueArgs& a, uint32_t pos_begin, uint32_t pos_end, uint32_t* counter,
                              uint32_t cmax, uint32_t* gscratch, int grid, cudaStream_t st, bool list = false);

}  // namespace eh
