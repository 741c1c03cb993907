// Internal: the device matrix behind eh_matrix_t and its lazily built work plan.
#pragma once

#include <cstdint>
#include <mutex>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/eh_gb300.h"
#include "eh_kernels.cuh"

namespace eh {

struct Plan {
  bool ready = false;
  uint32_t* order = nullptr;  // rows with card >= 2, descending card
  uint32_t n_order = 0, n_giant = 0;
  uint32_t* giant_lists = nullptr;
  unsigned long long* giant_off = nullptr;
  std::vector<uint32_t> starts;  // bin starts: rows with card > x are order[0, starts[65535 - x])
  // Heavy units for the current (light_max, unit_span).
  uint32_t light_max = 0, unit_span = 0;
  uint32_t n_heavy = 0;           // order[0, n_heavy) have card > light_max
  uint2* units = nullptr;         // (order position, part)
  uint32_t n_units = 0;
  uint64_t units_cap = 0;
  unsigned long long* core = nullptr;  // dense core bitmap (rows j < core_k)
  uint32_t core_k = 0;
  unsigned long long* filter = nullptr;  // row filters (rows [kFilterLo, filter_k))
  uint32_t filter_words = 0, filter_k = 0;
  // rows in the plan with card > x (x < 65535)
  uint32_t above(uint32_t x) const { return starts.empty() ? 0 : starts[65535 - x]; }
  // largest card <= x present in the plan (0 if none)
  uint32_t largest_at_most(uint32_t x) const {
    if (starts.empty()) return 0;
    for (uint32_t b = 65535 - x; b < 65535; b++)
      if (starts[b + 1] > starts[b]) return 65535 - b;
    return 0;
  }
};

// Per-launch scratch: work-queue counters and the clique kernel's global slots.
// A matrix has its own; concurrent launches on one matrix (the serving loop)
// each bring theirs.
struct Workspace {
  uint32_t* counters = nullptr;        // >= 16 words
  uint32_t* clique_scratch = nullptr;
  uint64_t clique_scratch_words = 0;
};

struct Matrix {
  int device = 0;
  uint64_t n = 0;
  int layout = 0, selection = 0;
  RowDesc* desc = nullptr;
  uint4* arena = nullptr;
  uint64_t arena_units = 0;
  BuildTotals tot{};
  Plan plan;
  uint32_t* counters = nullptr;  // 16 work-queue counters, then `result`
  unsigned long long* result = nullptr;
  int grid = 0;
  int64_t vstar = -1;
  uint64_t device_bytes = 0;
  uint32_t* clique_scratch = nullptr;  // global slots for the largest clique pivots
  uint64_t clique_scratch_words = 0;
  // Work-shape parameters of the pivot kernel (set by the autotuner).
  uint32_t light_max = kDefaultLightMax;
  uint32_t unit_span = kDefaultUnitSpan;
  uint32_t core_limit = kCoreDefaultK;  // rows in the dense core at most (0 = no core)
  uint32_t core_hot_words = 0;          // see PivotArgs::core_hot_words
  uint32_t core_filter_words = 0;       // words per core row filter (0: no filters)
  bool is_batch = false;            // the union matrix of an eh_batch_t
  bool shape_set = false;           // a shape was given (eh_matrix_set_shape, the tuner): no cached shape
  // Where the matrix's buffers are read: one event per stream, recorded after
  // every launch that reads them (not while that stream is being captured).
  // Freeing or replacing a buffer makes the freeing stream wait for these
  // events, not for the whole device.
  std::mutex uses_mu;
  std::vector<std::pair<cudaStream_t, cudaEvent_t>> uses;
};

// eh_capi.cu
// Stream-ordered allocation (cudaMallocAsync semantics) from the library's own
// pools on the current device, for scratch and for a matrix's buffers, all freed
// with cudaFreeAsync: scratch on the stream that used it, a matrix's buffers on
// a stream made to wait for the matrix's recorded uses (note_use / wait_uses).
// Each pool keeps up to kPoolKeep bytes of freed memory mapped between calls:
// the device's default pool releases it at every synchronisation, and mapping
// 400 MB again costs about 1 ms on GB300.  16 GiB holds a rebuilt scale-22
// matrix with its largest tuned core (4.3 GB) and its build scratch.
constexpr uint64_t kPoolKeep = 16ull << 30;
// Which pool: the dense cores and row filters of work plans (large, and kept
// for the matrix's life) come from a pool of their own.  In the same pool as
// the other buffers, a resident 4.3 GB core made every later build and plan
// of another matrix 0.6 + 0.6 ms slower at scale 22; in their own pool (or
// from cudaMalloc) it costs nothing.
enum PoolKind { kPoolMain = 0, kPoolCore = 1 };
cudaError_t pool_alloc(void** p, size_t bytes, cudaStream_t st, PoolKind kind = kPoolMain);
// A non-blocking stream of the current device for host uploads that overlap
// the build (one per device, created on first use).
cudaError_t upload_stream(cudaStream_t* out);

// A host upload in flight: rows [rows[c], rows[c + 1]) of the adjacency have
// landed on the device once ready[c] has completed.
struct UploadChunks {
  std::vector<uint64_t> rows;
  std::vector<cudaEvent_t> ready;
};

// total = offsets[n] (the neighbour array's length), or kTotalUnknown to read it
// from the device.  With `up`, the first pass measures each chunk of rows as
// soon as its upload has landed (the offsets must be in place before chunk 0's
// event); without, the whole input is already on the device.
constexpr uint64_t kTotalUnknown = ~0ull;
eh_status build_device(uint64_t n, const uint64_t* d_off, const uint32_t* d_nbr, const uint8_t* d_mask, int sel,
                       int layout, cudaStream_t st, Matrix** out, uint64_t total, const UploadChunks* up = nullptr);
eh_status ensure_plan(Matrix* m, cudaStream_t st);
eh_status ensure_units(Matrix* m, uint32_t light_max, uint32_t unit_span, cudaStream_t st);
eh_status ensure_core(Matrix* m, cudaStream_t st);
// Frees the parts of the plan that depend on the work shape (heavy units, dense
// core, row filters), so that the next ensure_plan builds them from nothing.
eh_status drop_shape_parts(Matrix* m, cudaStream_t st);
// Records that launches reading m's buffers were just queued on st.
void note_use(Matrix* m, cudaStream_t st);
// Makes st wait for every launch note_use has recorded on m, on any stream.
cudaError_t wait_uses(Matrix* m, cudaStream_t st);
// eh_batch.cu: tuned work shape of this matrix's size class, if the tuner has one.
void apply_cached_shape(Matrix* m);
PivotArgs pivot_args(Matrix* m, unsigned long long* out);
// Count launches; graph_rows / num_graphs != null selects per-graph outputs
// out[num_graphs].  ws == null uses the matrix's own workspace.  The plan must
// already exist when ws != null (launches with a workspace never allocate it).
eh_status launch_triangle_count(Matrix* m, unsigned long long* out, const uint32_t* graph_rows, uint32_t num_graphs,
                                cudaStream_t st, Workspace* ws = nullptr);
eh_status launch_lollipop_count(Matrix* m, unsigned long long* out, cudaStream_t st);
// tuples != null or list: write the k = 3 or 4 cliques as tuples (CliqueArgs::tuples).
eh_status launch_cliques(Matrix* m, uint32_t k, unsigned long long* out, const uint32_t* graph_rows,
                         uint32_t num_graphs, cudaStream_t st, Workspace* ws = nullptr, bool list = false,
                         uint32_t* tuples = nullptr, uint64_t capacity = 0);

}  // namespace eh
