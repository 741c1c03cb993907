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

// Layout payload bytes of a row as the algorithmic-bytes formula counts them:
// uint 4|S|, bitset 8 (words + 1), pshort 2 (|S| + 2 partitions).
__device__ __forceinline__ uint64_t payload_bytes(const RowView& V) {
  if (V.type == TY_UINT) return 4ull * V.card;
  if (V.type == TY_BITSET) return V.card ? 8ull * (V.len + 1) : 0ull;
  return 2ull * V.len;
}

}  // namespace eh
