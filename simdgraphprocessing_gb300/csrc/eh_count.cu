// Pattern-count kernels over an encoded matrix.
//
// Triangles (apps/undirected_triangle_counting.cpp:27-65) sum, over every pivot
// row i and every j in A_i = row(i), the intersection |A_i ∩ row(j)|.  Rows are
// pruned (nbr < node), so row(j) only holds ids below j and the count for the
// pair equals |{a in A_i : a < j} ∩ row(j)|; with A_i sorted and j = A_i[e]
// those are exactly A_i[0..e).  Lollipops (apps/undirected_lollipop_counting.cpp:
// 27-77) run on the full rows and count, for y = A_x[e], the z in A_x ∩ row(y)
// with z < y -- the same bounded intersection -- each weighted by |A_x|.
//
// One persistent kernel does both.  Work comes in two tiers, both handed out
// dynamically with an atomic counter (the GPU form of par_for_range's block
// stealing, src/common.hpp:214-276):
//  * heavy pivots (|A_i| > light_max) are split into units of unit_span values
//    of e; a CTA stages the pivot's decoded list (and, for bitset rows, its
//    words) in shared memory and its warps take one j each.  Per pair the warp
//    picks the cheapest of: AND of overlapping bitset words + popc (bitset ∩
//    bitset, intersection.hpp:880-955); probing each A_i[t], t < e, into row(j)
//    (uint ∩ bitset probe, :1023-1058, or the galloping search of :393-584);
//    streaming row(j) and looking each element up in the staged pivot (merge,
//    :696-771).
//  * light pivots run one per warp: the pivot is decoded into the warp's slice
//    of shared memory and all (e, t) pairs with t < e are probed at once, one
//    pair per lane, so short rows keep every lane busy.
// Per-lane counts stay in registers; one u64 atomic per CTA at the end replaces
// the reference's per-thread padded t_count array.
#include <algorithm>
#include <atomic>
#include <cstdint>

#include "eh_kernels.cuh"

namespace eh {

namespace {

constexpr int NWARPS = kCtaThreads / 32;
constexpr uint32_t kLightChunk = 16;  // light pivots per atomic grab
constexpr uint32_t kTinyPairs = 28;   // chunks of pivots with at most this many pairs (8 entries) share steps
constexpr uint32_t kStreamMinE = 256;  // core rows: consider streaming row(j) only past this many probes

struct __align__(16) HeavySmem {
  unsigned long long words[kCtaWordCap];
  unsigned long long abits[kCoreAndMax / 64];  // pivot ∩ [0, min(core_k, kCoreAndMax)) as bits
  uint32_t list[kCtaListCap];
  uint32_t scan[kCtaThreads];
  uint64_t bar;  // completion of the unit's bulk copy
  uint32_t unit;
};
// Device error flag (PivotArgs::counters[kErrWord]): a bulk copy's wait ran out.
constexpr uint32_t kErrWord = 15, kErrBulkWait = 1u;

// Warp, CTA, then one u64 atomic per CTA into the single count.
__device__ __forceinline__ void cta_add(unsigned long long acc, const PivotArgs& a) {
  __shared__ unsigned long long s_red[NWARPS];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  acc = warp_sum_u64(acc);
  if (lane == 0) s_red[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long tot = 0;
    for (int w = 0; w < NWARPS; w++) tot += s_red[w];
    if (tot && !a.graph_rows) atomicAdd(a.out, tot);
  }
}

__device__ __forceinline__ uint32_t ilog2p1(uint32_t x) { return 32u - __clz(x | 1u); }

// |{t < e : L[t] in B}| with j = L[e]; warp-uniform result.  A is the pivot row
// (shared or global payload), L its sorted elements.
__device__ uint32_t pair_count_warp(const uint32_t* L, uint32_t e, const RowView& A, const RowView& B,
                                    uint32_t j, uint32_t lane) {
  if (B.card == 0 || e == 0) return 0;
  uint32_t c = 0;
  if (A.type == TY_BITSET && B.type == TY_BITSET) {
    const uint32_t lo = max(A.aux, B.aux);
    const uint32_t hi = min(min(A.aux + A.len, B.aux + B.len), (j >> 6) + 1);
    if (hi <= lo) return 0;
    if (hi - lo <= 2 * e) {  // 128-bit AND + popcount over the overlapping words below j
      c = bitset_and_lane(A.p, A.aux, B.p, B.aux, B.len, lo, hi, j >> 6, (1ull << (j & 63)) - 1ull, lane);
      return warp_sum_u32(c);
    }
  }
  // Probe cost: e lookups into B.  Stream cost: |B| lookups into the pivot.
  // Merge cost (uint rows): e + |B| steps of a merge path.
  bool stream = false;
  if (B.type == TY_UINT) {
    const uint32_t look = (A.type == TY_BITSET) ? 1u : ilog2p1(e);
    const uint64_t probe_cost = (uint64_t)e * ilog2p1(B.card) * 4u, stream_cost = (uint64_t)B.card * look;
    if (A.type != TY_BITSET && e >= 64 && (uint64_t)e + B.card < min(probe_cost, stream_cost)) {
      const uint32_t* b = static_cast<const uint32_t*>(B.p);
      const uint32_t nb = lower_bound_u32(b, 0, B.card, j);  // full rows hold elements >= j too
      return warp_sum_u32(merge_path_lane(L, e, b, nb, lane));
    }
    stream = stream_cost < probe_cost;
  } else if (B.type == TY_PSHORT) {
    stream = (uint64_t)B.card * ilog2p1(e) < (uint64_t)e * (B.aux + ilog2p1(B.card)) * 4u;
  }
  if (!stream) {
    for (uint32_t t = lane; t < e; t += 32) c += row_contains(B, L[t]);
  } else if (A.type == TY_BITSET) {
    warp_for_each(B, j, lane, [&](uint32_t y) { c += row_contains(A, y); });
  } else {
    warp_for_each(B, j, lane, [&](uint32_t y) {
      const uint32_t p = lower_bound_u32(L, 0, e, y);
      c += (p < e && L[p] == y);
    });
  }
  return warp_sum_u32(c);
}

// Per-lane part of |{t < e : L[t] in B}| by streaming B's elements below j and
// looking each up in the pivot (a bit test for a bitset pivot, else a binary
// search of L[0, e)); the caller sums over the warp.
__device__ __forceinline__ uint32_t pair_count_stream(const uint32_t* L, uint32_t e, const RowView& A,
                                                      const RowView& B, uint32_t j, uint32_t lane) {
  uint32_t c = 0;
  if (A.type == TY_BITSET) {
    warp_for_each(B, j, lane, [&](uint32_t y) { c += row_contains(A, y); });
  } else {
    warp_for_each(B, j, lane, [&](uint32_t y) {
      const uint32_t p = lower_bound_u32(L, 0, e, y);
      c += (p < e && L[p] == y);
    });
  }
  return c;
}

// Heavy pivots: 6 resident CTAs per SM, 40 registers per thread (the per-pair
// choice keeps many values live, and at 32 registers it spilled).
template <bool LOLLI>
__global__ void __launch_bounds__(kCtaThreads, 6) k_pivots_heavy(PivotArgs a, const uint2* __restrict__ units,
                                                              uint32_t n_units) {
  __shared__ HeavySmem s;
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long acc = 0;
  uint32_t phase = 0;
  if (threadIdx.x == 0) mbar_init(&s.bar);

  // ---- heavy pivots: CTA-wide units ----
  for (;;) {
    if (threadIdx.x == 0) s.unit = atomicAdd(&a.counters[0], 1u);
    __syncthreads();  // also: every thread is done with the previous unit's staging
    const uint32_t unit = s.unit;
    if (unit >= n_units) break;
    const uint2 uu = units[unit];
    const uint32_t i = a.order[uu.x];
    RowView A = load_view(a.desc, a.arena, i);
    const uint32_t* L;
    // uint pivots and bitset words are staged by one bulk (TMA) copy: row
    // payloads start on 16-byte boundaries and are padded to 16 bytes.
    const bool bulk_list = uu.x >= a.n_giant && A.type == TY_UINT;
    const bool bulk_words = A.type == TY_BITSET && A.len <= kCtaWordCap;
    if (bulk_list || bulk_words) {
      if (threadIdx.x == 0) {
        if (bulk_list) bulk_copy_g2s(s.list, A.p, (4 * A.card + 15) & ~15u, &s.bar);
        else bulk_copy_g2s(s.words, A.p, (8 * A.len + 15) & ~15u, &s.bar);
      }
      if (!mbar_wait(&s.bar, phase)) {
        // Record the failure, then give the copy in flight a second bounded
        // wait before the buffer is used or the CTA exits.
        if (threadIdx.x == 0) atomicOr(&a.counters[kErrWord], kErrBulkWait);
        mbar_wait(&s.bar, phase);
      }
      phase ^= 1u;
    }
    if (uu.x < a.n_giant) {
      L = (A.type == TY_UINT) ? static_cast<const uint32_t*>(A.p) : a.giant_lists + a.giant_off[uu.x];
    } else if (bulk_list) {
      L = s.list;
    } else {
      cta_decode<kCtaThreads>(A, s.list, s.scan);
      L = s.list;
    }
    if (bulk_words) A.p = s.words;
    // The core path is skipped for pshort pivots of >= 65,536 entries, where the
    // reference's u16 partition count can drop a block (see pshort_pair_drop).
    const bool use_core = a.core_k && !(A.type == TY_PSHORT && A.card >= 65536u);
    const uint32_t and_k = min(a.core_k, kCoreAndMax);
    if (use_core) {
      for (uint32_t k = threadIdx.x; k < (and_k >> 6); k += kCtaThreads) s.abits[k] = 0ull;
      __syncthreads();
      for (uint32_t k = threadIdx.x; k < A.card; k += kCtaThreads) {
        const uint32_t x = L[k];
        if (x < and_k) atomicOr(&s.abits[x >> 6], 1ull << (x & 63));
      }
    }
    __syncthreads();
    const uint32_t c = A.card;
    const uint32_t e0 = 1 + uu.y * a.unit_span;
    const uint32_t e1 = min(c, e0 + a.unit_span);
    unsigned long long uacc = 0;
    for (uint32_t e = e0 + warp; e < e1; e += NWARPS) {
      const uint32_t j = L[e];
      uint32_t cnt;
      if (use_core && j < a.core_k) {
        // Core row j holds row(j) ∩ [0, j).  Cheapest of: AND it with the pivot's
        // bits (j within the staged bits; wj words), probe it at the e pivot
        // elements below j (e words), or stream row(j) itself and look each
        // element up in the pivot (|row(j)| lookups; rows past the highest-degree
        // ones are short while e grows with the pivot).
        const unsigned long long* row = a.core + core_row_offset(j);
        const uint32_t wj = (j + 63) >> 6;
        cnt = 0;
        if (j <= and_k && wj <= e) {
          // 8-byte words: padding the core rows to 16-byte pairs for 128-bit
          // loads here measured 0.15 ms slower per count at scale 22.
          for (uint32_t w = lane; w < wj; w += 32) cnt += __popcll(s.abits[w] & __ldg(row + w));
        } else {
          bool stream = false;
          RowView B;
          if (e > kStreamMinE) {
            B = load_view(a.desc, a.arena, j);
            stream = (uint64_t)B.card * (A.type == TY_BITSET ? 1u : ilog2p1(e)) < e;
          }
          if (stream) {
            cnt = pair_count_stream(L, e, A, B, j, lane);
          } else {
            for (uint32_t t = lane; t < e; t += 32) {
              const uint32_t x = L[t];
              cnt += (uint32_t)((__ldg(row + (x >> 6)) >> (x & 63)) & 1ull);
            }
          }
        }
        cnt = warp_sum_u32(cnt);
      } else {
        const RowView B = load_view(a.desc, a.arena, j);
        cnt = pair_count_warp(L, e, A, B, j, lane);
      }
      if (lane == 0) uacc += LOLLI ? (unsigned long long)cnt * c : (unsigned long long)cnt;
    }
    if (a.graph_rows) {  // batch: this unit's count goes to its graph
      if (lane == 0 && uacc) atomicAdd(&a.out[graph_of(a.graph_rows, a.num_graphs, i)], uacc);
    } else {
      acc += uacc;
    }
    __syncthreads();
  }

  cta_add(acc, a);
}

// Word x / 64 of core row j.  With core_hot_words set, words near the start of
// each core row (the highest-degree columns, where most probes land) keep
// their L2 lines and the others are evicted first.
template <bool HOT>
__device__ __forceinline__ unsigned long long core_word(const PivotArgs& a, uint32_t j, uint32_t x) {
  const unsigned long long* p = a.core + core_row_offset(j) + (x >> 6);
  if (!HOT) return __ldg(p);
  return (x >> 6) < a.core_hot_words ? ld_keep(p) : ld_stream(p);
}

// Two light-pivot probes at once, x0 in row(j0) and (if two) x1 in row(j1):
// the row's filter word first (if the row has a filter; a clear bit means x is
// not in row(j)), then one word of the core row j when j < core_k, else the
// row itself.  Both probes' loads are issued before either result is used.
// Returns the hits as bits 0 and 1.
template <bool HOT>
__device__ __forceinline__ uint32_t probe2(const PivotArgs& a, uint32_t j0, uint32_t x0, uint32_t j1, uint32_t x1,
                                           bool two) {
  const uint32_t b0 = filter_bit(x0, a.filter_words), b1 = filter_bit(x1, a.filter_words);
  const unsigned long long f0 = (j0 >= kFilterLo && j0 < a.filter_k)
                                    ? ld_keep(a.filter + (uint64_t)(j0 - kFilterLo) * a.filter_words + (b0 >> 6))
                                    : ~0ull;
  const unsigned long long f1 = (two && j1 >= kFilterLo && j1 < a.filter_k)
                                    ? ld_keep(a.filter + (uint64_t)(j1 - kFilterLo) * a.filter_words + (b1 >> 6))
                                    : ~0ull;
  const bool m0 = (f0 >> (b0 & 63)) & 1ull, m1 = two && ((f1 >> (b1 & 63)) & 1ull);
  const bool c0 = m0 && j0 < a.core_k, c1 = m1 && j1 < a.core_k;
  const unsigned long long v0 = c0 ? core_word<HOT>(a, j0, x0) : 0ull;
  const unsigned long long v1 = c1 ? core_word<HOT>(a, j1, x1) : 0ull;
  uint32_t h0 = (uint32_t)((v0 >> (x0 & 63)) & 1ull), h1 = (uint32_t)((v1 >> (x1 & 63)) & 1ull);
  if (m0 && !c0) h0 = row_contains(load_view(a.desc, a.arena, j0), x0);
  if (m1 && !c1) h1 = row_contains(load_view(a.desc, a.arena, j1), x1);
  return h0 | (h1 << 1);
}

// A chunk of light pivots whose first (largest) pivot has at most kTinyPairs
// pairs, as one pair space: the pivots' descriptors and rows are loaded by one
// lane each, and lane q of a step takes pair q of the whole chunk, so a pivot
// of a few pairs does not hold the warp for a step of its own.  Out of line:
// its registers do not weigh on the main loop.  Returns the chunk's count
// (each hit weighted by its pivot's card for lollipops).
template <bool LOLLI, bool HOT>
__device__ __noinline__ unsigned long long light_tiny_chunk(const PivotArgs& a, uint32_t base, uint32_t end,
                                                            uint32_t* list, uint32_t* pstart, uint32_t* poff,
                                                            uint32_t* pcard, uint32_t lane) {
  const uint32_t g = end - base;  // <= kLightChunk <= 32
  RowView V;
  uint32_t cl = 0;
  if (lane < g) {
    V = load_view(a.desc, a.arena, a.order[a.n_heavy + base + lane]);
    cl = V.card;  // <= the first pivot's card: rows in descending card order
  }
  const uint32_t pl = cl * (cl - 1) / 2;
  const uint32_t off = warp_exclusive_scan(cl, lane), pex = warp_exclusive_scan(pl, lane);
  const uint32_t total = __shfl_sync(FULL, pex + pl, 31);
  if (lane < g) {
    pstart[lane] = pex;
    poff[lane] = off;
    pcard[lane] = cl;
  }
  if (lane == 0) pstart[g] = total;
  if (lane < g && V.type == TY_UINT)
    for (uint32_t u = 0; u < cl; u++) list[off + u] = static_cast<const uint32_t*>(V.p)[u];
  __syncwarp();
  for (uint32_t rest = __ballot_sync(FULL, lane < g && V.type != TY_UINT); rest; rest &= rest - 1) {
    const uint32_t p = __ffs(rest) - 1;
    warp_decode(load_view(a.desc, a.arena, a.order[a.n_heavy + base + p]), list + poff[p], lane);
  }
  unsigned long long tcnt = 0;
  for (uint32_t q = lane; q < total; q += 64) {
    const bool two = q + 32 < total;
    uint32_t jj[2], xx[2], ww[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const uint32_t qh = (h == 0 || two) ? q + 32u * h : q;
      uint32_t p = 0;
      while (pstart[p + 1] <= qh) p++;
      uint32_t e = 1, t = qh - pstart[p];
      while (t >= e) { t -= e; e++; }
      jj[h] = list[poff[p] + e];
      xx[h] = list[poff[p] + t];
      ww[h] = LOLLI ? pcard[p] : 1u;
    }
    const uint32_t h = probe2<HOT>(a, jj[0], xx[0], jj[1], xx[1], two);
    tcnt += (unsigned long long)(h & 1u) * ww[0] + (unsigned long long)(h >> 1) * ww[1];
  }
  __syncwarp();  // the slice and tables are reused by the next chunk
  return tcnt;
}

// Light pivots: 8 resident CTAs per SM (64 warps, 32 registers per thread):
// bound by the latency of scattered probes, so occupancy and two probes in
// flight per lane pay.
template <bool LOLLI, bool HOT>  // HOT: core_hot_words != 0
__global__ void __launch_bounds__(kCtaThreads, 8) k_pivots_light(PivotArgs a) {
  __shared__ uint32_t wlist[NWARPS][kLightMax];
  __shared__ uint32_t wtiny[NWARPS][3][kLightChunk + 1];  // tiny chunks: pair starts, list offsets, cards
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long acc = 0;

  // ---- light pivots: one warp each, all (e, t) pairs probed in parallel ----
  const uint32_t n_light = a.n_order - a.n_heavy;
  uint32_t* list = wlist[warp];
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(&a.counters[1], kLightChunk);
    base = __shfl_sync(FULL, base, 0);
    if (base >= n_light) break;
    const uint32_t end = min(n_light, base + kLightChunk);
    // A chunk whose first (largest) pivot has at most kTinyPairs pairs runs as
    // one pair space: its pivots' descriptors and rows are loaded by one lane
    // each, and lane q of a step takes pair q of the whole chunk, so a pivot
    // of a few pairs does not hold the warp for a step of its own.
    const RowView F = load_view(a.desc, a.arena, a.order[a.n_heavy + base]);
    if (!a.graph_rows && F.card * (F.card - 1) / 2 <= kTinyPairs) {
      acc += light_tiny_chunk<LOLLI, HOT>(a, base, end, list, wtiny[warp][0], wtiny[warp][1], wtiny[warp][2], lane);
      continue;
    }
    for (uint32_t k = base; k < end; k++) {
      const uint32_t i = a.order[a.n_heavy + k];
      const RowView A = load_view(a.desc, a.arena, i);
      const uint32_t c = A.card;
      warp_decode(A, list, lane);
      const uint32_t pairs = c * (c - 1) / 2;
      // Lane q starts at pair q = e(e-1)/2 + t and advances by 32 pairs a step.
      uint32_t e = 1, t = lane;
      while (t >= e) { t -= e; e++; }
      uint32_t cnt = 0;
      // Two pairs per lane and step (q and q + 32), each probed the same way:
      // the row's filter word first (if the row has a filter; a clear bit means
      // x is not in row(j)), then one word of the core row j when j < core_k,
      // else the row itself.  Both pairs' loads are issued before either
      // result is used, so two probe chains are in flight per lane.
      for (uint32_t q = lane; q < pairs; q += 64) {
        const uint32_t j0 = list[e], x0 = list[t];
        t += 32;
        while (t >= e && e < c) { t -= e; e++; }
        const bool two = q + 32 < pairs;
        const uint32_t j1 = two ? list[e] : 0u, x1 = two ? list[t] : 0u;
        t += 32;
        while (t >= e && e < c) { t -= e; e++; }
        cnt += __popc(probe2<HOT>(a, j0, x0, j1, x1, two));
      }
      unsigned long long pc = LOLLI ? (unsigned long long)cnt * c : (unsigned long long)cnt;
      if (a.graph_rows) {  // batch: one atomic per pivot into its graph's count
        pc = warp_sum_u64(pc);
        if (lane == 0 && pc) atomicAdd(&a.out[graph_of(a.graph_rows, a.num_graphs, i)], pc);
      } else {
        acc += pc;
      }
      __syncwarp();
    }
  }

  cta_add(acc, a);
}

// Dense core build: one warp per row j < core_k writes row(j) ∩ [0, j) as bits.
__global__ void __launch_bounds__(256) k_core_build(const RowDesc* __restrict__ desc, const uint4* __restrict__ arena,
                                                    uint32_t core_k, unsigned long long* __restrict__ core) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nw = gridDim.x * (blockDim.x / 32);
  for (uint32_t j = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); j < core_k; j += nw) {
    unsigned long long* row = core + core_row_offset(j);
    const uint32_t wj = (j + 63) >> 6;
    for (uint32_t w = lane; w < wj; w += 32) row[w] = 0ull;
    __syncwarp();
    const RowView B = load_view(desc, arena, j);
    if (B.type == TY_BITSET) {
      const unsigned long long* bw = static_cast<const unsigned long long*>(B.p);
      for (uint32_t w = lane; w < B.len; w += 32) {
        const uint32_t gw = B.aux + w;
        if (gw >= wj) break;
        unsigned long long x = bw[w];
        if (gw == wj - 1 && (j & 63)) x &= (1ull << (j & 63)) - 1ull;
        row[gw] = x;
      }
    } else {
      warp_for_each(B, j, lane, [&](uint32_t x) { atomicOr(&row[x >> 6], 1ull << (x & 63)); });
    }
    __syncwarp();
  }
}

// Row filters: one warp per row j in [kFilterLo, filter_k) sets
// filter_bit(x) for each x in row(j) ∩ [0, j).
__global__ void __launch_bounds__(256) k_filter_build(const RowDesc* __restrict__ desc,
                                                      const uint4* __restrict__ arena, uint32_t filter_k,
                                                      uint32_t filter_words, unsigned long long* __restrict__ filter) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nw = gridDim.x * (blockDim.x / 32);
  for (uint32_t j = kFilterLo + blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); j < filter_k; j += nw) {
    unsigned long long* row = filter + (uint64_t)(j - kFilterLo) * filter_words;
    for (uint32_t w = lane; w < filter_words; w += 32) row[w] = 0ull;
    __syncwarp();
    const RowView B = load_view(desc, arena, j);
    warp_for_each(B, j, lane, [&](uint32_t x) {
      const uint32_t b = filter_bit(x, filter_words);
      atomicOr(&row[b >> 6], 1ull << (b & 63));
    });
    __syncwarp();
  }
}

// Heavy units: for order position u < n_heavy, ceil((card-1)/span) units (u, part).
__global__ void k_unit_counts(const RowDesc* __restrict__ desc, const uint32_t* __restrict__ order,
                              uint32_t n_heavy, uint32_t span, uint32_t* __restrict__ cnt) {
  const uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u < n_heavy) {
    const uint32_t c = desc[order[u]].card;
    cnt[u] = (c - 1 + span - 1) / span;
  }
}
__global__ void k_unit_fill(const uint32_t* __restrict__ cnt, const uint32_t* __restrict__ start,
                            uint32_t n_heavy, uint2* __restrict__ units) {
  const uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u < n_heavy)
    for (uint32_t p = 0; p < cnt[u]; p++) units[start[u] + p] = make_uint2(u, p);
}

// similar_nodes: rows i with |row(v*) ∩ row(i)| > threshold; one warp per row.
__global__ void __launch_bounds__(256) k_similar(uint64_t n, const RowDesc* __restrict__ desc,
                                                 const uint4* __restrict__ arena, uint32_t vstar,
                                                 uint32_t threshold, unsigned long long* out) {
  __shared__ PshortHdr s_hdr[8];
  const uint32_t lane = threadIdx.x & 31;
  const RowView A = load_view(desc, arena, vstar);
  unsigned long long acc = 0;
  const uint64_t nw = (uint64_t)gridDim.x * (blockDim.x / 32);
  for (uint64_t r = (uint64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); r < n; r += nw) {
    const RowView B = load_view(desc, arena, (uint32_t)r);
    const uint32_t c = warp_intersect_size(A, B, lane, &s_hdr[threadIdx.x >> 5]);
    if (lane == 0 && c > threshold) acc++;
  }
  if (lane == 0 && acc) atomicAdd(out, acc);
}

// counts[p] = |row(a[p]) ∩ row(b[p])|, one warp per pair.  A pair naming a
// row >= n gets 0xffffffff.
__global__ void __launch_bounds__(256) k_intersect_rows(uint64_t n, const RowDesc* __restrict__ desc,
                                                        const uint4* __restrict__ arena,
                                                        const uint32_t* __restrict__ ra,
                                                        const uint32_t* __restrict__ rb, uint64_t np,
                                                        uint32_t* __restrict__ counts) {
  __shared__ PshortHdr s_hdr[8];
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t nw = (uint64_t)gridDim.x * (blockDim.x / 32);
  for (uint64_t p = (uint64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); p < np; p += nw) {
    if (ra[p] >= n || rb[p] >= n) {
      if (lane == 0) counts[p] = 0xffffffffu;
      continue;
    }
    const uint32_t c = warp_intersect_size(load_view(desc, arena, ra[p]), load_view(desc, arena, rb[p]), lane,
                                           &s_hdr[threadIdx.x >> 5]);
    if (lane == 0) counts[p] = c;
  }
}

}  // namespace

// Persistent grid sizes per device: SMs x resident CTAs of the light kernel
// (the tunable grid) and of the heavy kernel (its cap), looked up once.
static int grid_of(int device, bool heavy) {
  static std::atomic<int> cache[64][2];
  if (device < 0 || device >= 64) return 152;
  int g = cache[device][heavy].load();
  if (g > 0) return g;
  int sms = 0, per = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (heavy) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pivots_heavy<false>, kCtaThreads, 0);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pivots_light<false, false>, kCtaThreads, 0);
  g = std::max(1, sms) * std::max(1, per);
  cache[device][heavy].store(g);
  return g;
}

int pivot_grid(int device) { return grid_of(device, false); }

template <bool LOLLI>
static cudaError_t launch_pivots(const PivotArgs& a, const uint2* units, uint32_t n_units, int grid,
                                 cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(a.counters, 0, 2 * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(a.out, 0, sizeof(unsigned long long) * (a.graph_rows ? a.num_graphs : 1), st);
  if (e != cudaSuccess) return e;
  int device = 0;
  if ((e = cudaGetDevice(&device)) != cudaSuccess) return e;
  if (n_units) {
    const int gh = std::min(grid, grid_of(device, true));
    k_pivots_heavy<LOLLI><<<std::max(gh, 1), kCtaThreads, 0, st>>>(a, units, n_units);
  }
  if (a.n_order > a.n_heavy) {
    if (a.core_hot_words) k_pivots_light<LOLLI, true><<<std::max(grid, 1), kCtaThreads, 0, st>>>(a);
    else k_pivots_light<LOLLI, false><<<std::max(grid, 1), kCtaThreads, 0, st>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t launch_pivot_units(const RowDesc* desc, const uint32_t* order, uint32_t n_heavy,
                               uint32_t unit_span, uint32_t* cnt, cudaStream_t st) {
  if (n_heavy == 0) return cudaSuccess;
  k_unit_counts<<<(n_heavy + 255) / 256, 256, 0, st>>>(desc, order, n_heavy, unit_span, cnt);
  return cudaGetLastError();
}
cudaError_t launch_pivot_unit_fill(const uint32_t* cnt, const uint32_t* start, uint32_t n_heavy,
                                   uint2* units, cudaStream_t st) {
  if (n_heavy == 0) return cudaSuccess;
  k_unit_fill<<<(n_heavy + 255) / 256, 256, 0, st>>>(cnt, start, n_heavy, units);
  return cudaGetLastError();
}

cudaError_t launch_triangles(const PivotArgs& a, const uint2* units, uint32_t n_units, int grid,
                             cudaStream_t st) {
  return launch_pivots<false>(a, units, n_units, grid, st);
}
cudaError_t launch_lollipops(const PivotArgs& a, const uint2* units, uint32_t n_units, int grid,
                             cudaStream_t st) {
  return launch_pivots<true>(a, units, n_units, grid, st);
}

cudaError_t launch_core_build(const RowDesc* desc, const uint4* arena, uint32_t core_k, unsigned long long* core,
                              cudaStream_t st) {
  if (core_k == 0) return cudaSuccess;
  const uint32_t blocks = std::min<uint32_t>((core_k + 7) / 8, 152u * 16u);
  k_core_build<<<blocks, 256, 0, st>>>(desc, arena, core_k, core);
  return cudaGetLastError();
}

cudaError_t launch_filter_build(const RowDesc* desc, const uint4* arena, uint32_t filter_k, uint32_t filter_words,
                                unsigned long long* filter, cudaStream_t st) {
  if (filter_k <= kFilterLo || filter_words == 0) return cudaSuccess;
  const uint32_t blocks = std::min<uint32_t>((filter_k - kFilterLo + 7) / 8, 152u * 16u);
  k_filter_build<<<blocks, 256, 0, st>>>(desc, arena, filter_k, filter_words, filter);
  return cudaGetLastError();
}

cudaError_t launch_similar(uint64_t n, const RowDesc* desc, const uint4* arena, uint32_t vstar,
                           uint32_t threshold, unsigned long long* out, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess || n == 0) return e;
  uint64_t g = (n + 7) / 8;
  if (g > 152 * 32) g = 152 * 32;
  k_similar<<<(unsigned)g, 256, 0, st>>>(n, desc, arena, vstar, threshold, out);
  return cudaGetLastError();
}

cudaError_t launch_intersect_rows(uint64_t n, const RowDesc* desc, const uint4* arena, const uint32_t* a,
                                  const uint32_t* b, uint64_t np, uint32_t* counts, cudaStream_t st) {
  if (np == 0) return cudaSuccess;
  uint64_t g = (np + 7) / 8;
  if (g > 152 * 32) g = 152 * 32;
  k_intersect_rows<<<(unsigned)g, 256, 0, st>>>(n, desc, arena, a, b, np, counts);
  return cudaGetLastError();
}

}  // namespace eh
