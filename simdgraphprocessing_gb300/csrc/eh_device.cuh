// Device-side data layout and warp-level set-intersection primitives.
//
// HBM layout of an encoded matrix (the reference's SparseMatrix rows,
// src/SparseMatrix.hpp:11-131):
//   desc[n]  : one 16-byte RowDesc per row (a single vector load per lookup);
//   arena    : every row's payload in its layout, each starting on a 16-byte
//              boundary so that rows can be staged with bulk copies and read
//              with 128-bit loads.  The payloads hold the reference's logical
//              bytes (uinteger.hpp, bitset.hpp, pshort.hpp); only the small
//              headers (the bitset's first-word index, the u32 byte counts
//              and the hybrid u64 type tag) move into RowDesc.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace eh {

// Layout tags: the reference's common::type values (src/common.hpp:171-181).
enum : uint32_t { TY_BITSET = 0, TY_PSHORT = 1, TY_UINT = 2 };

struct __align__(16) RowDesc {
  uint32_t off16;  // payload start, in 16-byte units from the arena base
  uint32_t card;   // cardinality (SparseMatrix::row_lengths)
  uint32_t aux;    // bitset: first word index (element / 64); pshort: #partitions; uint: 0
  uint32_t lt;     // bits 0..29: payload length in layout units (uint: elements,
                   // bitset: 64-bit words, pshort: 16-bit shorts); bits 30..31: type
};

__host__ __device__ inline uint32_t desc_type(const RowDesc& d) { return d.lt >> 30; }
__host__ __device__ inline uint32_t desc_len(const RowDesc& d) { return d.lt & 0x3fffffffu; }
__host__ __device__ inline uint32_t make_lt(uint32_t type, uint32_t len) { return (type << 30) | len; }

// A row as the kernels see it: generic pointer (global or shared) + metadata.
struct RowView {
  const void* p;
  uint32_t type, card, aux, len;
};

__device__ __forceinline__ RowView load_view(const RowDesc* __restrict__ desc,
                                             const uint4* __restrict__ arena, uint32_t r) {
  uint4 d = __ldg(reinterpret_cast<const uint4*>(desc) + r);
  RowView v;
  v.p = arena + d.x;
  v.card = d.y;
  v.aux = d.z;
  v.type = d.w >> 30;
  v.len = d.w & 0x3fffffffu;
  return v;
}

constexpr uint32_t FULL = 0xffffffffu;

// ---- Bulk (TMA) copies from global to shared memory, completing on an mbarrier ----
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// One thread: initialise a CTA-local mbarrier expecting one arrival per phase.
__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One thread: order this CTA's earlier shared-memory accesses (made visible to
// it by a __syncthreads) before the async proxy's writes, arm `bar` for `bytes`
// and start the copy.  dst and src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

// Every thread: wait for phase `parity` of `bar` to complete.  The wait is
// bounded; false means it ran out (the caller records an error and moves on).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t max_tries = 1u << 22) {
  for (uint32_t i = 0; i < max_tries; i++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ uint32_t warp_sum_u32(uint32_t x) { return __reduce_add_sync(FULL, x); }
__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long x) {
  for (int d = 16; d; d >>= 1) x += __shfl_xor_sync(FULL, x, d);
  return x;
}

// First position in a[lo, hi) with a[pos] >= x (a sorted ascending).
__device__ __forceinline__ uint32_t lower_bound_u32(const uint32_t* a, uint32_t lo, uint32_t hi, uint32_t x) {
  while (lo < hi) {
    uint32_t mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1; else hi = mid;
  }
  return lo;
}
__device__ __forceinline__ uint32_t lower_bound_u16(const uint16_t* a, uint32_t lo, uint32_t hi, uint32_t x) {
  while (lo < hi) {
    uint32_t mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Membership of one element in a row, by the row's layout.
//  bitset: one word load (the reference's bitset::is_set, bitset.hpp:124-127,
//          with the range test of intersection.hpp:1039);
//  uint  : binary search (the per-element step of set_intersect_galloping,
//          intersection.hpp:393-584);
//  pshort: walk partition prefixes, then binary search the low shorts
//          (the partition match of intersection.hpp:829-878).
__device__ __forceinline__ bool row_contains(const RowView& B, uint32_t x) {
  if (B.type == TY_BITSET) {
    uint32_t w = x >> 6;
    if (w < B.aux || w - B.aux >= B.len) return false;
    const unsigned long long* words = static_cast<const unsigned long long*>(B.p);
    return (words[w - B.aux] >> (x & 63)) & 1ull;
  }
  if (B.type == TY_UINT) {
    const uint32_t* a = static_cast<const uint32_t*>(B.p);
    uint32_t pos = lower_bound_u32(a, 0, B.card, x);
    return pos < B.card && a[pos] == x;
  }
  const uint16_t* s = static_cast<const uint16_t*>(B.p);
  uint32_t hi = x >> 16, lo = x & 0xffffu, i = 0;
  while (i < B.len) {
    uint32_t h = s[i], cnt = (uint32_t)s[i + 1] + 1;
    if (h == hi) {
      uint32_t pos = lower_bound_u16(s + i + 2, 0, cnt, lo);
      return pos < cnt && s[i + 2 + pos] == lo;
    }
    if (h > hi) return false;
    i += cnt + 2;
  }
  return false;
}

// Calls f(x) once for every element x < lim of V, the elements spread over the
// warp's lanes in layout order (the per-layout foreach: uinteger.hpp:67-80,
// bitset.hpp:148-173, pshort.hpp:134-158).  f must not use warp collectives.
template <class F>
__device__ __forceinline__ void warp_for_each(const RowView& V, uint32_t lim, uint32_t lane, F&& f) {
  if (V.type == TY_UINT) {
    const uint32_t* a = static_cast<const uint32_t*>(V.p);
    for (uint32_t k = lane; k < V.card; k += 32) {
      uint32_t x = a[k];
      if (x >= lim) break;
      f(x);
    }
  } else if (V.type == TY_BITSET) {
    const unsigned long long* w = static_cast<const unsigned long long*>(V.p);
    for (uint32_t k = lane; k < V.len; k += 32) {
      uint64_t base = 64ull * (V.aux + k);
      if (base >= lim) break;
      unsigned long long x = w[k];
      if (base + 64 > lim) x &= (1ull << (lim - base)) - 1ull;
      while (x) {
        f((uint32_t)(base + (uint32_t)(__ffsll((long long)x) - 1)));
        x &= x - 1ull;
      }
    }
  } else {
    const uint16_t* s = static_cast<const uint16_t*>(V.p);
    uint32_t i = 0;
    while (i < V.len) {
      uint32_t hb = (uint32_t)s[i] << 16, cnt = (uint32_t)s[i + 1] + 1;
      if (hb >= lim) break;
      for (uint32_t k = lane; k < cnt; k += 32) {
        uint32_t x = hb | s[i + 2 + k];
        if (x >= lim) break;
        f(x);
      }
      i += cnt + 2;
    }
  }
}

// The reference's pshort ∩ pshort kernel keeps each partition's intersection
// size in a uint16_t (intersection.hpp:857-865), so a partition pair whose
// 65,536 values are all common adds 0 and none of those values reach its
// output.  That needs a full 2^16 block in both rows, hence >= 65,536 entries
// in each; pshort_pair_drop() returns how many of the dropped values lie
// below `lim` (0 in every other case).  Run by one lane.
__device__ inline bool pshort_full_block(const RowView& V, uint32_t h) {
  const uint16_t* s = static_cast<const uint16_t*>(V.p);
  uint32_t i = 0;
  while (i < V.len) {
    const uint32_t hh = s[i], cnt = (uint32_t)s[i + 1] + 1;
    if (hh == h) return cnt == 65536u;
    if (hh > h) return false;
    i += cnt + 2;
  }
  return false;
}
__device__ inline uint64_t pshort_pair_drop(const RowView& A, const RowView& B, uint64_t lim) {
  if (A.type != TY_PSHORT || B.type != TY_PSHORT || A.card < 65536u || B.card < 65536u) return 0;
  const uint16_t* s = static_cast<const uint16_t*>(B.p);
  uint64_t drop = 0;
  uint32_t i = 0;
  while (i < B.len) {
    const uint32_t h = s[i], cnt = (uint32_t)s[i + 1] + 1;
    const uint64_t lo = (uint64_t)h << 16;
    if (lo >= lim) break;
    if (cnt == 65536u && pshort_full_block(A, h)) drop += min((uint64_t)65536, lim - lo);
    i += cnt + 2;
  }
  return drop;
}

// |A ∩ B| as the reference's set_intersect reports it, the pshort ∩ pshort
// u16 quirk included, computed by one warp; every lane returns the result.
// Two bitsets are ANDed word by word over their common word range; otherwise
// the smaller row is streamed and each element probed into the larger one.
__device__ inline uint32_t warp_intersect_size(RowView A, RowView B, uint32_t lane) {
  if (!A.card || !B.card) return 0;
  uint32_t c = 0;
  if (A.type == TY_BITSET && B.type == TY_BITSET) {
    const unsigned long long* a = static_cast<const unsigned long long*>(A.p);
    const unsigned long long* b = static_cast<const unsigned long long*>(B.p);
    const uint32_t lo = max(A.aux, B.aux), hi = min(A.aux + A.len, B.aux + B.len);
    for (uint32_t w = lo + lane; w < hi; w += 32) c += __popcll(a[w - A.aux] & b[w - B.aux]);
  } else {
    if (A.card > B.card) {
      const RowView T = A;
      A = B;
      B = T;
    }
    warp_for_each(A, 0xffffffffu, lane, [&](uint32_t y) { c += row_contains(B, y); });
  }
  c = warp_sum_u32(c);
  return c - (uint32_t)pshort_pair_drop(A, B, ~0ull);
}

// Batch mode: index g of the graph whose rows [graph_rows[g], graph_rows[g+1])
// hold `row` (graph_rows has num_graphs + 1 ascending entries).
__device__ __forceinline__ uint32_t graph_of(const uint32_t* graph_rows, uint32_t num_graphs, uint32_t row) {
  uint32_t lo = 0, hi = num_graphs;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (graph_rows[mid] <= row) lo = mid; else hi = mid;
  }
  return lo;
}

// Layout payload bytes of a row as the algorithmic-bytes formula counts them:
// uint 4|S|, bitset 8 (words + 1), pshort 2 (|S| + 2 partitions).
__device__ __forceinline__ uint64_t payload_bytes(const RowView& V) {
  if (V.type == TY_UINT) return 4ull * V.card;
  if (V.type == TY_BITSET) return V.card ? 8ull * (V.len + 1) : 0ull;
  return 2ull * V.len;
}

// CTA-cooperative decode of a row into a sorted u32 list in shared memory.
template <uint32_t kThreads>
__device__ inline void cta_decode(const RowView& A, uint32_t* list, uint32_t* scan) {
  const uint32_t tid = threadIdx.x;
  if (A.type == TY_UINT) {
    const uint32_t* a = static_cast<const uint32_t*>(A.p);
    for (uint32_t k = tid; k < A.card; k += kThreads) list[k] = a[k];
    return;
  }
  if (A.type == TY_BITSET) {
    // Thread t owns words [t*W/T, (t+1)*W/T); exclusive scan of their popcounts
    // gives each thread its output position.
    const unsigned long long* w = static_cast<const unsigned long long*>(A.p);
    const uint32_t W = A.len;
    const uint32_t w0 = (uint32_t)(((uint64_t)W * tid) / kThreads);
    const uint32_t w1 = (uint32_t)(((uint64_t)W * (tid + 1)) / kThreads);
    uint32_t c = 0;
    for (uint32_t k = w0; k < w1; k++) c += __popcll(w[k]);
    scan[tid] = c;
    __syncthreads();
    // Hillis-Steele inclusive scan over kThreads values.
    for (uint32_t d = 1; d < kThreads; d <<= 1) {
      const uint32_t v = tid >= d ? scan[tid - d] : 0u;
      __syncthreads();
      scan[tid] += v;
      __syncthreads();
    }
    uint32_t pos = scan[tid] - c;
    for (uint32_t k = w0; k < w1; k++) {
      unsigned long long x = w[k];
      while (x) {
        list[pos++] = 64u * (A.aux + k) + (uint32_t)(__ffsll((long long)x) - 1);
        x &= x - 1ull;
      }
    }
    return;
  }
  if (tid < 32) {  // pshort: walk the partitions with one warp
    const uint16_t* s = static_cast<const uint16_t*>(A.p);
    uint32_t i = 0, pos = 0;
    while (i < A.len) {
      const uint32_t hb = (uint32_t)s[i] << 16, cnt = (uint32_t)s[i + 1] + 1;
      for (uint32_t k = tid; k < cnt; k += 32) list[pos + k] = hb | s[i + 2 + k];
      pos += cnt;
      i += cnt + 2;
    }
  }
}

// Warp-cooperative decode into the warp's slice (card <= kLightMax).
__device__ __forceinline__ void warp_decode(const RowView& A, uint32_t* list, uint32_t lane) {
  if (A.type == TY_UINT) {
    const uint32_t* a = static_cast<const uint32_t*>(A.p);
    for (uint32_t k = lane; k < A.card; k += 32) list[k] = a[k];
  } else if (A.type == TY_BITSET) {
    const unsigned long long* w = static_cast<const unsigned long long*>(A.p);
    uint32_t pos = 0;
    for (uint32_t base = 0; base < A.len; base += 32) {
      const uint32_t k = base + lane;
      unsigned long long x = k < A.len ? w[k] : 0ull;
      const uint32_t c = __popcll(x);
      uint32_t inc = c;
      for (int d = 1; d < 32; d <<= 1) {
        const uint32_t t = __shfl_up_sync(FULL, inc, d);
        if (lane >= (uint32_t)d) inc += t;
      }
      uint32_t p = pos + inc - c;
      while (x) {
        list[p++] = 64u * (A.aux + k) + (uint32_t)(__ffsll((long long)x) - 1);
        x &= x - 1ull;
      }
      pos += __shfl_sync(FULL, inc, 31);
    }
  } else {
    const uint16_t* s = static_cast<const uint16_t*>(A.p);
    uint32_t i = 0, pos = 0;
    while (i < A.len) {
      const uint32_t hb = (uint32_t)s[i] << 16, cnt = (uint32_t)s[i + 1] + 1;
      for (uint32_t k = lane; k < cnt; k += 32) list[pos + k] = hb | s[i + 2 + k];
      pos += cnt;
      i += cnt + 2;
    }
  }
  __syncwarp();
}

}  // namespace eh
