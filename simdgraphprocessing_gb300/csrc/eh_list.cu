// Triangle tuples: what undirected_triangle_counting would emit with tuple
// output on (Table<T>::write_table, src/Table.hpp:30-43, which n_clique calls
// under WRITE_TABLE, apps/n_clique.cpp:42-44): for every pivot i, j in row(i)
// and k in row(i) ∩ row(j), the tuple (i, j, k) with i > j > k.
//
// Every (e, t < e) pair of a pivot's decoded row L is probed once (k = L[t] in
// row(L[e]), through the dense core when L[e] < core_k); hits take output
// positions from one global cursor, one atomic per warp and ballot.  Pivots of
// up to 64 entries run one per warp, larger ones one per CTA.  Tuples past
// `capacity` are counted but not written; the order is unspecified.
#include <algorithm>
#include <cstdint>

#include "eh_internal.h"
#include "eh_kernels.cuh"
#include "eh_matrix.cuh"

namespace eh {
namespace {

constexpr uint32_t kListWarpMax = 64;
constexpr int NW = kCtaThreads / 32;

struct ListArgs {
  const RowDesc* desc;
  const uint4* arena;
  const uint32_t* order;
  uint32_t n_giant;
  const uint32_t* giant_lists;
  const unsigned long long* giant_off;
  const unsigned long long* core;
  uint32_t core_k;
  uint32_t* out;
  uint64_t capacity;
  unsigned long long* cursor;
  uint32_t* counters;  // [0] warp-tier positions, [1] CTA-tier positions
};

__device__ __forceinline__ bool pair_hit(const ListArgs& a, const RowView& A, uint32_t j, uint32_t x) {
  if (j < a.core_k && !(A.type == TY_PSHORT && A.card >= 65536u))
    return (__ldg(a.core + core_row_offset(j) + (x >> 6)) >> (x & 63)) & 1ull;
  const RowView B = load_view(a.desc, a.arena, j);
  if (!row_contains(B, x)) return false;
  // The reference's pshort ∩ pshort drops a fully shared 2^16 block (u16 count).
  if (A.type == TY_PSHORT && B.type == TY_PSHORT && A.card >= 65536u && B.card >= 65536u &&
      pshort_full_block(A, x >> 16) && pshort_full_block(B, x >> 16))
    return false;
  return true;
}

// Warp-aggregated output: lanes with hit write (i, j, x) at consecutive positions.
__device__ __forceinline__ void emit(const ListArgs& a, bool hit, uint32_t i, uint32_t j, uint32_t x, uint32_t lane) {
  const uint32_t bal = __ballot_sync(FULL, hit);
  if (!bal) return;
  unsigned long long base = 0;
  const uint32_t leader = __ffs(bal) - 1;
  if (lane == leader) base = atomicAdd(a.cursor, (unsigned long long)__popc(bal));
  base = __shfl_sync(FULL, base, leader);
  if (hit) {
    const unsigned long long pos = base + __popc(bal & ((1u << lane) - 1u));
    if (pos < a.capacity) {
      a.out[3 * pos] = i;
      a.out[3 * pos + 1] = j;
      a.out[3 * pos + 2] = x;
    }
  }
}

// Pairs (e, t < e) of pivot list L (c entries), q = first + stride * r.
__device__ __forceinline__ void walk_pairs(const ListArgs& a, const RowView& A, uint32_t i, const uint32_t* L,
                                           uint32_t c, uint32_t first, uint32_t stride, uint32_t lane) {
  const uint64_t pairs = (uint64_t)c * (c - 1) / 2;
  uint32_t e = 1;
  uint64_t t = first;
  while (t >= e && e < c) { t -= e; e++; }
  // All lanes of a warp run the same number of rounds (emit uses warp collectives).
  const uint64_t rounds = (pairs + stride - 1) / stride;
  for (uint64_t r = 0; r < rounds; r++) {
    const uint64_t q = first + r * stride;
    bool hit = false;
    uint32_t j = 0, x = 0;
    if (q < pairs) {
      j = L[e];
      x = L[t];
      hit = pair_hit(a, A, j, x);
    }
    emit(a, hit, i, j, x, lane);
    t += stride;
    while (t >= e && e < c) { t -= e; e++; }
  }
}

__global__ void __launch_bounds__(kCtaThreads) k_list_warp(ListArgs a, uint32_t pos_begin, uint32_t pos_end) {
  __shared__ uint32_t s_list[NW][kListWarpMax];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (;;) {
    uint32_t p = 0;
    if (lane == 0) p = atomicAdd(&a.counters[0], 1u);
    p = __shfl_sync(FULL, p, 0) + pos_begin;
    if (p >= pos_end) break;
    const uint32_t i = a.order[p];
    const RowView A = load_view(a.desc, a.arena, i);
    warp_decode(A, s_list[warp], lane);
    walk_pairs(a, A, i, s_list[warp], A.card, lane, 32, lane);
    __syncwarp();
  }
}

__global__ void __launch_bounds__(kCtaThreads) k_list_cta(ListArgs a, uint32_t pos_begin, uint32_t pos_end) {
  __shared__ uint32_t s_list[kCtaListCap];
  __shared__ uint32_t s_scan[kCtaThreads];
  __shared__ uint32_t s_unit;
  const uint32_t lane = threadIdx.x & 31;
  for (;;) {
    if (threadIdx.x == 0) s_unit = atomicAdd(&a.counters[1], 1u) + pos_begin;
    __syncthreads();
    const uint32_t p = s_unit;
    if (p >= pos_end) break;
    const uint32_t i = a.order[p];
    const RowView A = load_view(a.desc, a.arena, i);
    const uint32_t* L;
    if (p < a.n_giant) {
      L = (A.type == TY_UINT) ? static_cast<const uint32_t*>(A.p) : a.giant_lists + a.giant_off[p];
    } else {
      cta_decode<kCtaThreads>(A, s_list, s_scan);
      L = s_list;
    }
    __syncthreads();
    walk_pairs(a, A, i, L, A.card, threadIdx.x, kCtaThreads, lane);
    __syncthreads();
  }
}

}  // namespace
}  // namespace eh

extern "C" eh_status eh_list_triangles(eh_matrix_t mh, uint32_t* d_out, uint64_t capacity, uint64_t* d_total,
                                       void* stream) {
  using namespace eh;
  if (!mh) return set_error(EH_ERR_INVALID_ARGUMENT, "matrix is NULL");
  Matrix* m = reinterpret_cast<Matrix*>(mh);
  cudaSetDevice(m->device);
  EH_CHECK_ARG(d_total, "d_total is NULL");
  EH_CHECK_ARG(capacity == 0 || d_out, "d_out is NULL");
  if (m->selection != EH_SELECT_LOWER)
    return set_error(EH_ERR_UNSUPPORTED, "triangle listing needs a matrix built with EH_SELECT_LOWER");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  eh_status s = ensure_plan(m, st);
  if (s != EH_OK) return s;
  const Plan& p = m->plan;
  ListArgs a{m->desc, m->arena, p.order, p.n_giant, p.giant_lists, p.giant_off, p.core, p.core_k,
             d_out, capacity, reinterpret_cast<unsigned long long*>(d_total), m->counters + 4};
  cudaError_t e = cudaMemsetAsync(d_total, 0, sizeof(uint64_t), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->counters + 4, 0, 2 * sizeof(uint32_t), st);
  if (e != cudaSuccess) return set_error(EH_ERR_CUDA, "memset: %s", cudaGetErrorString(e));
  const uint32_t n_large = p.above(kListWarpMax);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, m->device);
  if (n_large) k_list_cta<<<(unsigned)std::min<uint64_t>(n_large, 4ull * sms), kCtaThreads, 0, st>>>(a, 0, n_large);
  if (p.n_order > n_large)
    k_list_warp<<<(unsigned)std::min<uint64_t>((p.n_order - n_large + 7) / 8, 8ull * sms), kCtaThreads, 0, st>>>(
        a, n_large, p.n_order);
  e = cudaGetLastError();
  note_use(m, st);
  return e == cudaSuccess ? EH_OK : set_error(EH_ERR_CUDA, "listing kernels: %s", cudaGetErrorString(e));
}
