// Apps over directed graphs: symbiosity (apps/symbiosity.cpp) and the n_path
// breadth-first search (apps/n_path.cpp).
//
// symbiosity: one warp per row i intersects out(i) (the row matrix) with in(i)
// (the column matrix) and tests the Jaccard ratio in double precision, as
// symbiosity.cpp:46-58 does.  Rows too long for a warp (hubs) are listed and
// taken one per CTA, with the probed row staged in shared memory when it is a
// uint row that fits.
//
// n_path: level-synchronous BFS on a visited bitset of (n + 64) / 64 words,
// the reference's bs_size (n_path.cpp:45-53).  A level is two launches:
//   expand  ORs into `next` every element of the frontier's rows whose visited
//           bit is clear (set_union of the rows into the visited set,
//           union.hpp:6-127, minus what was already visited); a bitset row is
//           ORed word by word;
//   collect takes next AND NOT visited as the new frontier (set_difference,
//           difference.hpp:5-84), merges it into visited and clears next.
// Frontier rows longer than kBfsHeavy entries are split over every warp of
// the grid; shorter ones are taken one per warp.  Levels are launched
// kBfsChunk at a time: each kernel reads its frontier size from device memory
// and does nothing once a frontier is empty, so the host checks the sizes
// once per chunk instead of once per level.
#include <algorithm>
#include <cstdint>
#include <vector>

#include "eh_internal.h"
#include "eh_kernels.cuh"
#include "eh_matrix.cuh"

namespace eh {
namespace {

constexpr uint32_t kBfsHeavy = 4096;
constexpr uint32_t kBfsChunk = 8;
constexpr int kBfsThreads = 256;

// A row pair whose intersection is too long for one warp: streamed side (the
// smaller row) above kSymLight entries, or two bitsets sharing more than
// 8 * kSymLight words.  Such rows go to a list that whole CTAs work through.
constexpr uint32_t kSymLight = 256;
// Probed uint rows of up to kSymStage entries are staged in shared memory.
constexpr uint32_t kSymStage = 12288;

__device__ __forceinline__ bool sym_heavy(const RowView& A, const RowView& B) {
  if (!A.card || !B.card) return false;
  if (A.type == TY_BITSET && B.type == TY_BITSET) {
    const int64_t lo = max(A.aux, B.aux), hi = min((int64_t)A.aux + A.len, (int64_t)B.aux + B.len);
    return hi - lo > 8 * (int64_t)kSymLight;
  }
  return min(A.card, B.card) > kSymLight;
}

constexpr uint32_t kSymChunk = 32;  // rows a warp takes per grab (one per lane)
constexpr uint32_t kSymTiny = 64;   // uint rows a single lane intersects by merging

__device__ __forceinline__ bool sym_above(uint32_t both, const RowView& A, const RowView& B, double threshold) {
  // 0 / 0 is NaN, which is not above any threshold (as in the reference).
  return (double)both / (double)((uint64_t)A.card + B.card - both) > threshold;
}

// |A ∩ B| of two sorted uint rows by one thread (a merge).
__device__ __forceinline__ uint32_t merge_count(const uint32_t* a, uint32_t na, const uint32_t* b, uint32_t nb) {
  uint32_t i = 0, j = 0, c = 0;
  while (i < na && j < nb) {
    const uint32_t x = a[i], y = b[j];
    c += x == y;
    i += x <= y;
    j += y <= x;
  }
  return c;
}

// Rows are taken kSymChunk at a time from a shared cursor, one row per lane.
// A lane finishes its row alone when both sides are uint rows of at most
// kSymTiny entries (most rows of a sparse graph) or one side is empty; rows
// above that go to the whole warp, and rows too long for a warp to the list
// of k_symbiosity_heavy.
__global__ void __launch_bounds__(256, 5) k_symbiosity(uint32_t n, const RowDesc* __restrict__ dr,
                                                    const uint4* __restrict__ ar, const RowDesc* __restrict__ dc,
                                                    const uint4* __restrict__ ac, double threshold,
                                                    unsigned long long* out, uint32_t* heavy, uint32_t* n_heavy,
                                                    uint32_t* cursor) {
  __shared__ PshortHdr s_hdr[8];
  const uint32_t lane = threadIdx.x & 31;
  unsigned long long acc = 0;
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(cursor, kSymChunk);
    base = __shfl_sync(FULL, base, 0);
    if (base >= n) break;
    const uint32_t r = base + lane;
    bool warp_row = false;
    if (r < n) {
      const RowView A = load_view(dr, ar, r);
      const RowView B = load_view(dc, ac, r);
      if (!A.card || !B.card) {  // ratio 0, or 0/0 (NaN, never above)
        acc += sym_above(0, A, B, threshold);
      } else if (A.type == TY_UINT && B.type == TY_UINT && max(A.card, B.card) <= kSymTiny) {
        const uint32_t both = merge_count(static_cast<const uint32_t*>(A.p), A.card,
                                          static_cast<const uint32_t*>(B.p), B.card);
        acc += sym_above(both, A, B, threshold);
      } else if (sym_heavy(A, B)) {
        heavy[atomicAdd(n_heavy, 1u)] = r;
      } else {
        warp_row = true;
      }
    }
    for (uint32_t wm = __ballot_sync(FULL, warp_row); wm; wm &= wm - 1) {
      const uint32_t r2 = base + (__ffs(wm) - 1);
      const RowView A = load_view(dr, ar, r2);
      const RowView B = load_view(dc, ac, r2);
      const uint32_t both = warp_intersect_size(A, B, lane, &s_hdr[threadIdx.x >> 5]);  // header table: pshort rows
      if (lane == 0) acc += sym_above(both, A, B, threshold);
    }
  }
  acc = warp_sum_u64(acc);
  if (lane == 0 && acc) atomicAdd(out, acc);
}

// f(x) for every element of V, spread over the CTA (pshort: warps take
// partitions round-robin, lanes the entries of a partition).
template <class F>
__device__ __forceinline__ void cta_for_each(const RowView& V, F&& f) {
  const uint32_t tid = threadIdx.x, nt = blockDim.x;
  if (V.type == TY_UINT) {
    const uint32_t* a = static_cast<const uint32_t*>(V.p);
    for (uint32_t k = tid; k < V.card; k += nt) f(a[k]);
  } else if (V.type == TY_BITSET) {
    const unsigned long long* w = static_cast<const unsigned long long*>(V.p);
    for (uint32_t k = tid; k < V.len; k += nt)
      for (unsigned long long x = w[k]; x; x &= x - 1ull)
        f(64u * (V.aux + k) + (uint32_t)(__ffsll((long long)x) - 1));
  } else {
    const uint16_t* s = static_cast<const uint16_t*>(V.p);
    const uint32_t lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
    uint32_t i = 0, p = 0;
    while (i < V.len) {
      const uint32_t hb = (uint32_t)s[i] << 16, cnt = (uint32_t)s[i + 1] + 1;
      if (p % nwarps == warp)
        for (uint32_t k = lane; k < cnt; k += 32) f(hb | s[i + 2 + k]);
      i += cnt + 2;
      p++;
    }
  }
}

// The heavy rows of k_symbiosity, one CTA per row taken from a shared cursor.
__global__ void __launch_bounds__(256) k_symbiosity_heavy(const RowDesc* __restrict__ dr, const uint4* __restrict__ ar,
                                                          const RowDesc* __restrict__ dc, const uint4* __restrict__ ac,
                                                          double threshold, unsigned long long* out,
                                                          const uint32_t* __restrict__ heavy,
                                                          const uint32_t* n_heavy, uint32_t* cursor) {
  __shared__ uint32_t stage[kSymStage];
  __shared__ uint32_t s_sum[8];
  __shared__ uint32_t s_idx;
  const uint32_t tid = threadIdx.x, lane = tid & 31;
  const uint32_t nh = *n_heavy;
  unsigned long long acc = 0;
  for (;;) {
    __syncthreads();  // the previous row is finished with stage / s_sum / s_idx
    if (tid == 0) s_idx = atomicAdd(cursor, 1u);
    __syncthreads();
    const uint32_t idx = s_idx;
    if (idx >= nh) break;
    const uint32_t r = heavy[idx];
    RowView A = load_view(dr, ar, r);
    RowView B = load_view(dc, ac, r);
    const RowView A0 = A, B0 = B;
    uint32_t c = 0;
    if (A.type == TY_BITSET && B.type == TY_BITSET) {
      const unsigned long long* a = static_cast<const unsigned long long*>(A.p);
      const unsigned long long* b = static_cast<const unsigned long long*>(B.p);
      const uint32_t lo = max(A.aux, B.aux), hi = min(A.aux + A.len, B.aux + B.len);
      for (uint32_t w = lo + tid; w < hi; w += blockDim.x) c += __popcll(a[w - A.aux] & b[w - B.aux]);
    } else {
      if (A.card > B.card) {
        const RowView T = A;
        A = B;
        B = T;
      }
      if (B.type == TY_UINT && B.card <= kSymStage) {
        const uint32_t* b = static_cast<const uint32_t*>(B.p);
        for (uint32_t k = tid; k < B.card; k += blockDim.x) stage[k] = b[k];
        __syncthreads();
        cta_for_each(A, [&](uint32_t y) {
          const uint32_t pos = lower_bound_u32(stage, 0, B.card, y);
          c += pos < B.card && stage[pos] == y;
        });
      } else {
        cta_for_each(A, [&](uint32_t y) { c += row_contains(B, y); });
      }
    }
    c = warp_sum_u32(c);
    if (lane == 0) s_sum[tid >> 5] = c;
    __syncthreads();
    if (tid == 0) {
      uint32_t both = 0;
      for (uint32_t w = 0; w < (blockDim.x >> 5); w++) both += s_sum[w];
      both -= (uint32_t)pshort_pair_drop(A0, B0, ~0ull);
      if (sym_above(both, A0, B0, threshold)) acc++;
    }
  }
  if (tid == 0 && acc) atomicAdd(out, acc);
}

struct LevelCount {
  uint32_t light, heavy;
};

struct BfsArgs {
  const RowDesc* desc;
  const uint4* arena;
  uint32_t n;
  uint64_t words;
  unsigned long long* vis;
  unsigned long long* next;
  uint32_t* lists;     // two frontier lists of n entries: light rows from the front, heavy from the back
  LevelCount* counts;  // counts[j]: frontier sizes of the j-th level of the current chunk
  unsigned long long* reached;
};

__device__ __forceinline__ void visit(const unsigned long long* vis, unsigned long long* next, uint32_t x) {
  const uint32_t wi = x >> 6;
  const unsigned long long bit = 1ull << (x & 63);
  if (!((vis[wi] | __ldcg(next + wi)) & bit)) atomicOr(next + wi, bit);
}

// Marks in `next` the unvisited elements of slice `part` (of `nparts`) of row V;
// the warp's lanes share the slice.
__device__ __forceinline__ void expand_slice(const unsigned long long* vis, unsigned long long* next,
                                             const RowView& V, uint32_t part, uint32_t nparts, uint32_t lane) {
  if (V.type == TY_UINT) {
    const uint32_t* e = static_cast<const uint32_t*>(V.p);
    for (uint32_t k = part * 32 + lane; k < V.card; k += nparts * 32) visit(vis, next, e[k]);
  } else if (V.type == TY_BITSET) {
    const unsigned long long* w = static_cast<const unsigned long long*>(V.p);
    for (uint32_t k = part * 32 + lane; k < V.len; k += nparts * 32) {
      const uint32_t wi = V.aux + k;
      const unsigned long long x = w[k] & ~vis[wi];
      if (x & ~__ldcg(next + wi)) atomicOr(next + wi, x);
    }
  } else {
    const uint16_t* s = static_cast<const uint16_t*>(V.p);
    uint32_t i = 0, p = 0;
    while (i < V.len) {
      const uint32_t hb = (uint32_t)s[i] << 16, cnt = (uint32_t)s[i + 1] + 1;
      if (p % nparts == part)
        for (uint32_t k = lane; k < cnt; k += 32) visit(vis, next, hb | s[i + 2 + k]);
      i += cnt + 2;
      p++;
    }
  }
}

__global__ void k_bfs_init(BfsArgs a, uint32_t start) {
  a.vis[start >> 6] = 1ull << (start & 63);
  if (a.desc[start].card > kBfsHeavy) {
    a.lists[a.n - 1] = start;
    a.counts[0] = LevelCount{0, 1};
  } else {
    a.lists[0] = start;
    a.counts[0] = LevelCount{1, 0};
  }
  *a.reached = 1;
}

// Level j of the chunk: frontier F (sizes counts[j]) -> next.
__global__ void __launch_bounds__(kBfsThreads) k_bfs_expand(BfsArgs a, uint32_t j, const uint32_t* __restrict__ F) {
  const LevelCount c = a.counts[j];
  if (c.light + c.heavy == 0) return;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nw = gridDim.x * (blockDim.x / 32);
  const uint32_t gw = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (c.heavy) {
    // Warps form min(heavy, nw) groups; group g takes heavy rows g, g + groups, ...
    // and its gsz warps split each of them.
    const uint32_t groups = min(c.heavy, nw), gsz = nw / groups, g = gw / gsz;
    if (g < groups)
      for (uint32_t h = g; h < c.heavy; h += groups)
        expand_slice(a.vis, a.next, load_view(a.desc, a.arena, F[a.n - 1 - h]), gw % gsz, gsz, lane);
  }
  for (uint32_t f = gw; f < c.light; f += nw) expand_slice(a.vis, a.next, load_view(a.desc, a.arena, F[f]), 0, 1, lane);
}

// Level j of the chunk: next AND NOT visited -> frontier F (sizes counts[j + 1]).
__global__ void __launch_bounds__(kBfsThreads) k_bfs_collect(BfsArgs a, uint32_t j, uint32_t* __restrict__ F) {
  const LevelCount c = a.counts[j];
  if (c.light + c.heavy == 0) return;
  LevelCount* out = a.counts + j + 1;
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t nw = (uint64_t)gridDim.x * (blockDim.x / 32);
  unsigned long long found = 0;
  // Whole warps step together (the appends below use warp collectives).
  for (uint64_t w0 = ((uint64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5)) * 32; w0 < a.words;
       w0 += nw * 32) {
    const uint64_t w = w0 + lane;
    unsigned long long x = 0, heavy = 0;
    if (w < a.words) {
      const unsigned long long nx = a.next[w];
      if (nx) {
        x = nx & ~a.vis[w];
        a.next[w] = 0;
        a.vis[w] |= x;
      }
    }
    for (unsigned long long y = x; y; y &= y - 1) {
      const uint32_t v = (uint32_t)(64 * w) + (uint32_t)(__ffsll((long long)y) - 1);
      if (a.desc[v].card > kBfsHeavy) heavy |= y & (~y + 1);
    }
    found += __popcll(x);
    const uint32_t nh = __popcll(heavy), nl = __popcll(x) - nh;
    // Warp-exclusive prefix of nl and nh, one atomic per list and warp.
    uint32_t il = nl, ih = nh;
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t tl = __shfl_up_sync(FULL, il, d), th = __shfl_up_sync(FULL, ih, d);
      if (lane >= (uint32_t)d) {
        il += tl;
        ih += th;
      }
    }
    const uint32_t tot_l = __shfl_sync(FULL, il, 31), tot_h = __shfl_sync(FULL, ih, 31);
    uint32_t base_l = 0, base_h = 0;
    if (lane == 0) {
      if (tot_l) base_l = atomicAdd(&out->light, tot_l);
      if (tot_h) base_h = atomicAdd(&out->heavy, tot_h);
    }
    uint32_t pl = __shfl_sync(FULL, base_l, 0) + il - nl, ph = __shfl_sync(FULL, base_h, 0) + ih - nh;
    for (unsigned long long y = x; y; y &= y - 1) {
      const unsigned long long b = y & (~y + 1);
      const uint32_t v = (uint32_t)(64 * w) + (uint32_t)(__ffsll((long long)y) - 1);
      if (heavy & b) F[a.n - 1 - ph++] = v;
      else F[pl++] = v;
    }
  }
  found = warp_sum_u64(found);
  if (lane == 0 && found) atomicAdd(a.reached, found);
}

}  // namespace
}  // namespace eh

using eh::Matrix;

static eh_status cuda_err(cudaError_t e, const char* what) {
  return eh::set_error(EH_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

extern "C" eh_status eh_symbiosity_async(eh_matrix_t rh, eh_matrix_t ch, double threshold, uint64_t* d_count,
                                         void* stream) {
  using namespace eh;
  if (!rh || !ch) return set_error(EH_ERR_INVALID_ARGUMENT, "matrix is NULL");
  EH_CHECK_ARG(d_count, "d_count is NULL");
  Matrix* r = reinterpret_cast<Matrix*>(rh);
  Matrix* c = reinterpret_cast<Matrix*>(ch);
  if (r->n != c->n)
    return set_error(EH_ERR_INVALID_ARGUMENT, "row and column matrices differ in size (%llu vs %llu)",
                     (unsigned long long)r->n, (unsigned long long)c->n);
  if (r->device != c->device) return set_error(EH_ERR_INVALID_ARGUMENT, "row and column matrices are on different GPUs");
  cudaSetDevice(r->device);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(d_count, 0, sizeof(uint64_t), st);
  if (e != cudaSuccess) return cuda_err(e, "memset");
  if (r->n == 0) return EH_OK;
  // Heavy-row list: n entries, then its length, the CTAs' cursor and the warps' cursor.
  uint32_t* scratch = nullptr;
  e = pool_alloc((void**)&scratch, (r->n + 3) * sizeof(uint32_t), st);
  if (e != cudaSuccess) return set_error(EH_ERR_OUT_OF_MEMORY, "symbiosity scratch: %s", cudaGetErrorString(e));
  uint32_t* counts = scratch + r->n;
  e = cudaMemsetAsync(counts, 0, 3 * sizeof(uint32_t), st);
  int sms = 0, per = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, r->device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_symbiosity_heavy, 256, 0);
  if (e == cudaSuccess) {
    const uint64_t g = std::min<uint64_t>((r->n + 8 * kSymChunk - 1) / (8 * kSymChunk), (uint64_t)sms * 8);
    unsigned long long* out = reinterpret_cast<unsigned long long*>(d_count);
    k_symbiosity<<<(unsigned)std::max<uint64_t>(g, 1), 256, 0, st>>>((uint32_t)r->n, r->desc, r->arena, c->desc,
                                                                     c->arena, threshold, out, scratch, counts,
                                                                     counts + 2);
    k_symbiosity_heavy<<<(unsigned)(sms * std::max(per, 1)), 256, 0, st>>>(r->desc, r->arena, c->desc, c->arena,
                                                                           threshold, out, scratch, counts,
                                                                           counts + 1);
    e = cudaGetLastError();
  }
  const cudaError_t ef = cudaFreeAsync(scratch, st);
  if (e == cudaSuccess) e = ef;
  note_use(r, st);
  note_use(c, st);
  return e == cudaSuccess ? EH_OK : cuda_err(e, "symbiosity kernels");
}

extern "C" eh_status eh_symbiosity(eh_matrix_t rh, eh_matrix_t ch, double threshold, uint64_t* count,
                                   void* stream) {
  using namespace eh;
  EH_CHECK_ARG(count, "count is NULL");
  if (!rh) return set_error(EH_ERR_INVALID_ARGUMENT, "matrix is NULL");
  Matrix* r = reinterpret_cast<Matrix*>(rh);
  eh_status s = eh_symbiosity_async(rh, ch, threshold, reinterpret_cast<uint64_t*>(r->result), stream);
  if (s != EH_OK) return s;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemcpyAsync(count, r->result, sizeof(uint64_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? EH_OK : cuda_err(e, "symbiosity");
}

extern "C" eh_status eh_bfs_path_length(eh_matrix_t mh, uint32_t start, uint64_t max_depth, uint64_t* path_length,
                                        uint64_t* reached, void* stream) {
  using namespace eh;
  if (!mh) return set_error(EH_ERR_INVALID_ARGUMENT, "matrix is NULL");
  EH_CHECK_ARG(path_length, "path_length is NULL");
  Matrix* m = reinterpret_cast<Matrix*>(mh);
  EH_CHECK_ARG(start < m->n, "start row %u >= matrix size %llu", start, (unsigned long long)m->n);
  cudaSetDevice(m->device);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const uint64_t n = m->n;
  // No BFS has more than n levels, so a deeper limit never binds.
  const uint64_t depth = std::min<uint64_t>(max_depth, n);
  const uint64_t words = (n + 64) / 64;
  const size_t bytes = 2 * words * 8 + 2 * n * 4 + (kBfsChunk + 1) * sizeof(LevelCount) + 8;
  char* base = nullptr;
  cudaError_t e = pool_alloc((void**)&base, bytes, st);
  if (e != cudaSuccess) return set_error(EH_ERR_OUT_OF_MEMORY, "BFS scratch (%zu bytes): %s", bytes, cudaGetErrorString(e));
  BfsArgs a;
  a.desc = m->desc;
  a.arena = m->arena;
  a.n = (uint32_t)n;
  a.words = words;
  a.vis = reinterpret_cast<unsigned long long*>(base);
  a.next = a.vis + words;
  a.lists = reinterpret_cast<uint32_t*>(a.next + words);
  a.reached = reinterpret_cast<unsigned long long*>(a.lists + 2 * n);
  a.counts = reinterpret_cast<LevelCount*>(a.reached + 1);
  auto done = [&](eh_status s) {
    cudaFreeAsync(base, st);
    return s;
  };
  if ((e = cudaMemsetAsync(a.vis, 0, 2 * words * 8, st)) != cudaSuccess ||
      (e = cudaMemsetAsync(a.counts, 0, (kBfsChunk + 1) * sizeof(LevelCount), st)) != cudaSuccess)
    return done(cuda_err(e, "memset"));
  k_bfs_init<<<1, 1, 0, st>>>(a, start);
  int sms = 0, per = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, m->device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_bfs_expand, kBfsThreads, 0);
  const unsigned grid = (unsigned)std::max(1, sms * std::max(per, 1));
  const unsigned cgrid = (unsigned)std::min<uint64_t>((words + kBfsThreads - 1) / kBfsThreads, grid);
  LevelCount hc[kBfsChunk + 1];
  uint64_t level = 0, path = 0;
  for (;;) {
    // Expansions level .. level + k - 1; expansion L produces the frontier of level L + 1.
    const uint32_t k = (uint32_t)std::min<uint64_t>(kBfsChunk, depth + 1 - level);
    for (uint32_t j = 0; j < k; j++) {
      uint32_t* cur = a.lists + ((level + j) & 1) * n;
      uint32_t* nxt = a.lists + ((level + j + 1) & 1) * n;
      k_bfs_expand<<<grid, kBfsThreads, 0, st>>>(a, j, cur);
      k_bfs_collect<<<cgrid, kBfsThreads, 0, st>>>(a, j, nxt);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return done(cuda_err(e, "BFS kernels"));
    if ((e = cudaMemcpyAsync(hc, a.counts, (k + 1) * sizeof(LevelCount), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
      return done(cuda_err(e, "BFS level sizes"));
    bool stop = false;
    for (uint32_t j = 0; j < k && !stop; j++)
      if (hc[j + 1].light + hc[j + 1].heavy == 0) {
        path = level + j;
        stop = true;
      }
    if (!stop && level + k - 1 >= depth) {
      path = depth;
      stop = true;
    }
    if (stop) break;
    level += k;
    // The last frontier size of this chunk becomes the first of the next.
    if ((e = cudaMemcpyAsync(a.counts, a.counts + k, sizeof(LevelCount), cudaMemcpyDeviceToDevice, st)) != cudaSuccess ||
        (e = cudaMemsetAsync(a.counts + 1, 0, kBfsChunk * sizeof(LevelCount), st)) != cudaSuccess)
      return done(cuda_err(e, "BFS level sizes"));
  }
  uint64_t r = 0;
  if ((e = cudaMemcpyAsync(&r, a.reached, 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return done(cuda_err(e, "BFS result"));
  *path_length = path;
  if (reached) *reached = r;
  return done(EH_OK);
}

// ---- diagnostics: the bounded mbarrier wait used by the bulk-copy staging ----
namespace eh {
namespace {
// Waits on an mbarrier that nothing arrives on; the wait must give up after
// `tries` polls and the kernel report it instead of hanging.
__global__ void k_selftest_bounded_wait(uint32_t tries, uint32_t* status) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) mbar_init(&bar);
  __syncthreads();
  const bool done = mbar_wait(&bar, 0, tries);
  if (threadIdx.x == 0) *status = done ? 1u : 2u;
}
}  // namespace
}  // namespace eh

extern "C" eh_status eh_selftest_bounded_wait(uint32_t tries, uint32_t* timed_out) {
  using namespace eh;
  EH_CHECK_ARG(timed_out, "timed_out is NULL");
  EH_CHECK_ARG(tries > 0 && tries <= (1u << 16), "tries must be in [1, 65536]");
  uint32_t* d = nullptr;
  cudaError_t e = cudaMalloc((void**)&d, sizeof(uint32_t));
  if (e != cudaSuccess) return cuda_err(e, "selftest allocation");
  uint32_t h = 0;
  e = cudaMemset(d, 0, sizeof(uint32_t));
  if (e == cudaSuccess) {
    k_selftest_bounded_wait<<<1, 32>>>(tries, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(uint32_t), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_err(e, "selftest");
  *timed_out = h == 2u;
  return h ? EH_OK : set_error(EH_ERR_DEVICE_CHECK, "self-test kernel did not report");
}
