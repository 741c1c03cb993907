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

// ---- L2 eviction priority of single loads (createpolicy + L2::cache_hint) ----
// ld_keep marks the line to be evicted last, ld_stream to be evicted first:
// probes into a small, hot region keep it in L2 while scattered one-off probes
// do not displace it.  Read-only data (the non-coherent path).
__device__ __forceinline__ unsigned long long ld_keep(const unsigned long long* p) {
  unsigned long long v;
  asm("{\n .reg .b64 pol;\n createpolicy.fractional.L2::evict_last.b64 pol, 1.0;\n"
      " ld.global.nc.L2::cache_hint.u64 %0, [%1], pol;\n}"
      : "=l"(v)
      : "l"(p));
  return v;
}
__device__ __forceinline__ unsigned long long ld_stream(const unsigned long long* p) {
  unsigned long long v;
  asm("{\n .reg .b64 pol;\n createpolicy.fractional.L2::evict_first.b64 pol, 1.0;\n"
      " ld.global.nc.L2::cache_hint.u64 %0, [%1], pol;\n}"
      : "=l"(v)
      : "l"(p));
  return v;
}

__device__ __forceinline__ uint32_t warp_sum_u32(uint32_t x) { return __reduce_add_sync(FULL, x); }
__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long x) {
  for (int d = 16; d; d >>= 1) x += __shfl_xor_sync(FULL, x, d);
  return x;
}

// ---- Bitset words as 16-byte pairs ----
// Every payload starts on a 16-byte boundary and is zero-padded to a multiple
// of 16 bytes (in the arena and in shared-memory copies of it), so words
// (2q, 2q+1) of a bitset row are one aligned 128-bit load for every pair
// q < ceil(len / 2): the GPU form of the reference's 256-bit AVX loads
// (intersection.hpp:880-955).
__device__ __forceinline__ unsigned long long lo64(uint4 v) { return ((unsigned long long)v.y << 32) | v.x; }
__device__ __forceinline__ unsigned long long hi64(uint4 v) { return ((unsigned long long)v.w << 32) | v.z; }
// Pair q of a row with np pairs (generic address: global or shared), zero outside [0, np).
__device__ __forceinline__ uint4 ld_pair(const void* w, int32_t q, int32_t np) {
  if (q < 0 || q >= np) return make_uint4(0u, 0u, 0u, 0u);
  return reinterpret_cast<const uint4*>(w)[q];
}

// Per-lane part of sum over words w in [lo, hi) of popc(A_w & B_w), where A_w
// is word w - a0 of A's payload (a0 = its first word index) and likewise for
// B (blen words); word mw (if in range) is ANDed with mmask.  Requires
// a0 <= lo, b0 <= lo and hi <= b0 + blen, hi <= a0 + A's length.  A is walked
// in aligned pairs, all inside its payload.  B's pairs line up when b0 - a0 is
// even (then they are inside its payload too); when it is odd each A pair
// takes the high word of one B pair and the low word of the next, and the two
// pair indices are clamped to B's payload: a clamped word lies outside
// [lo, hi) and is masked off.  Word indices are below 2^26, so 32-bit
// arithmetic is exact.
__device__ __forceinline__ uint32_t bitset_and_lane(const void* pa, uint32_t a0, const void* pb, uint32_t b0,
                                                    uint32_t blen, uint32_t lo, uint32_t hi, uint32_t mw,
                                                    unsigned long long mmask, uint32_t lane) {
  const uint4* a4 = reinterpret_cast<const uint4*>(pa);
  const uint4* b4 = reinterpret_cast<const uint4*>(pb);
  const int32_t d = (int32_t)b0 - (int32_t)a0;
  const int32_t q1 = (int32_t)(hi - a0 + 1) >> 1;
  uint32_t c = 0;
  for (int32_t q = (int32_t)((lo - a0) >> 1) + (int32_t)lane; q < q1; q += 32) {
    const uint4 va = a4[q];
    const int32_t wb = 2 * q - d;  // B-relative index of A's word 2q
    unsigned long long b_lo, b_hi;
    if ((d & 1) == 0) {
      const uint4 vb = b4[wb >> 1];
      b_lo = lo64(vb);
      b_hi = hi64(vb);
    } else {
      const int32_t last = (int32_t)((blen + 1) >> 1) - 1;
      b_lo = hi64(b4[max((wb - 1) >> 1, 0)]);
      b_hi = lo64(b4[min((wb + 1) >> 1, last)]);
    }
    const uint32_t w0 = a0 + 2 * (uint32_t)q;
    unsigned long long x0 = lo64(va) & b_lo, x1 = hi64(va) & b_hi;
    if (w0 < lo) x0 = 0ull;
    if (w0 == mw) x0 &= mmask;
    if (w0 + 1 >= hi) x1 = 0ull;
    if (w0 + 1 == mw) x1 &= mmask;
    c += __popcll(x0) + __popcll(x1);
  }
  return c;
}

// Exclusive prefix sum of x over the warp's lanes (all lanes active).
__device__ __forceinline__ uint32_t warp_exclusive_scan(uint32_t x, uint32_t lane) {
  uint32_t inc = x;
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= (uint32_t)d) inc += t;
  }
  return inc - x;
}

// Writes the elements of word pair (lo, hi) -- absolute word index w0 for lo --
// to list[pos...] in ascending order.
__device__ __forceinline__ void emit_pair_bits(unsigned long long lo, unsigned long long hi, uint32_t w0,
                                               uint32_t* list, uint32_t pos) {
  while (lo) {
    list[pos++] = 64u * w0 + (uint32_t)(__ffsll((long long)lo) - 1);
    lo &= lo - 1ull;
  }
  while (hi) {
    list[pos++] = 64u * (w0 + 1) + (uint32_t)(__ffsll((long long)hi) - 1);
    hi &= hi - 1ull;
  }
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

// ---- uint ∩ uint: warp merge path ----
// Per-lane count of the elements common to sorted A[0, na) and B[0, nb): the
// merge of the two lists (ties: A first) is cut into 32 runs of equal length;
// each lane finds where its run starts by a binary search along its cross
// diagonal (Green, McColl, Bader, "GPU merge path", ICS 2012), then merges the
// run sequentially and counts A[i] == B[j] when it takes A[i], so each match
// is counted by exactly one lane.  The GPU form of the reference's block merge
// set_intersect_standard (intersection.hpp:696-771), which it uses for pairs
// whose sizes differ by at most 32x (:1325-1336).
__device__ __forceinline__ uint32_t merge_path_lane(const uint32_t* A, uint32_t na, const uint32_t* B, uint32_t nb,
                                                    uint32_t lane) {
  const uint32_t total = na + nb, per = (total + 31) >> 5;
  uint32_t d = min(total, lane * per);
  const uint32_t dend = min(total, d + per);
  uint32_t lo = d > nb ? d - nb : 0u, hi = min(d, na);
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (A[mid] <= B[d - mid - 1]) lo = mid + 1;
    else hi = mid;
  }
  uint32_t i = lo, j = d - lo, c = 0;
  for (; d < dend; d++) {
    if (j >= nb || (i < na && A[i] <= B[j])) {
      c += (j < nb && A[i] == B[j]);
      i++;
    } else {
      j++;
    }
  }
  return c;
}

// ---- pshort: partition headers staged in shared memory ----
// A warp probing many elements into one pshort row first copies that row's
// partition headers (the 16-bit high half and the header's position, at most
// kPshortHdrCap partitions) into a per-warp table; each probe is then a
// binary search of the highs in the table and of the low shorts inside the
// matched partition, instead of a walk over the row's headers per element
// (the partition match of intersection.hpp:829-878).
constexpr uint32_t kPshortHdrCap = 64;
struct PshortHdr {
  uint32_t hi[kPshortHdrCap];
  uint32_t pos[kPshortHdrCap];
};
// Lane 0 walks the headers of V (V.aux partitions, <= kPshortHdrCap) into t.
__device__ __forceinline__ void pshort_stage(const RowView& V, PshortHdr* t, uint32_t lane) {
  if (lane == 0) {
    const uint16_t* s = static_cast<const uint16_t*>(V.p);
    uint32_t i = 0;
    for (uint32_t k = 0; k < V.aux; k++) {
      t->hi[k] = s[i];
      t->pos[k] = i;
      i += (uint32_t)s[i + 1] + 3;
    }
  }
  __syncwarp();
}
// Index in t of the partition with high half h, or -1.
__device__ __forceinline__ int pshort_find(const PshortHdr* t, uint32_t parts, uint32_t h) {
  uint32_t lo = 0, hi = parts;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (t->hi[mid] < h) lo = mid + 1;
    else hi = mid;
  }
  return (lo < parts && t->hi[lo] == h) ? (int)lo : -1;
}
__device__ __forceinline__ bool pshort_contains_staged(const RowView& V, const PshortHdr* t, uint32_t x) {
  const int k = pshort_find(t, V.aux, x >> 16);
  if (k < 0) return false;
  const uint16_t* s = static_cast<const uint16_t*>(V.p) + t->pos[k];
  const uint32_t cnt = (uint32_t)s[1] + 1, lo = x & 0xffffu;
  const uint32_t pos = lower_bound_u16(s + 2, 0, cnt, lo);
  return pos < cnt && s[2 + pos] == lo;
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
    const int32_t np = (int32_t)((V.len + 1) >> 1);  // 16-byte word pairs
    for (int32_t q = (int32_t)lane; q < np; q += 32) {
      const uint64_t base = 64ull * (V.aux + 2 * (uint64_t)q);
      if (base >= lim) break;
      const uint4 v = ld_pair(V.p, q, np);
      unsigned long long x = lo64(v), y = hi64(v);
      if (base + 64 > lim) {
        x &= (1ull << (lim - base)) - 1ull;
        y = 0ull;
      } else if (base + 128 > lim) {
        y &= (1ull << (lim - base - 64)) - 1ull;
      }
      while (x) {
        f((uint32_t)(base + (uint32_t)(__ffsll((long long)x) - 1)));
        x &= x - 1ull;
      }
      while (y) {
        f((uint32_t)(base + 64 + (uint32_t)(__ffsll((long long)y) - 1)));
        y &= y - 1ull;
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
//  * two bitsets: 128-bit AND + popcount over their common word range;
//  * two uint rows of sizes within 32x of each other: warp merge path;
//  * otherwise the smaller row is streamed and each element probed into the
//    larger one (a binary search for uint, a bit test for a bitset); a pshort
//    larger row with 4..kPshortHdrCap partitions is probed through its headers
//    staged in `hdr` (per-warp shared memory, may be null), and a streamed
//    pshort row meets it partition by partition: the high halves are matched
//    once per partition, then the lanes search the low shorts.
// Per-lane part of |A ∩ B| for A no larger than B (not both bitsets).
__device__ __forceinline__ uint32_t warp_intersect_small_large(const RowView& A, const RowView& B, uint32_t lane,
                                                               PshortHdr* hdr) {
  uint32_t c = 0;
  if (A.type == TY_UINT && B.type == TY_UINT && B.card <= 32u * A.card) {
    c = merge_path_lane(static_cast<const uint32_t*>(A.p), A.card, static_cast<const uint32_t*>(B.p), B.card, lane);
  } else if (B.type == TY_PSHORT && hdr && B.aux >= 4 && B.aux <= kPshortHdrCap) {
    pshort_stage(B, hdr, lane);
    if (A.type == TY_PSHORT) {
      const uint16_t* sa = static_cast<const uint16_t*>(A.p);
      const uint16_t* sb = static_cast<const uint16_t*>(B.p);
      for (uint32_t i = 0; i < A.len;) {
        const uint32_t h = sa[i], cnt = (uint32_t)sa[i + 1] + 1;
        const int k = pshort_find(hdr, B.aux, h);
        if (k >= 0) {
          const uint16_t* pb = sb + hdr->pos[k];
          const uint32_t cb = (uint32_t)pb[1] + 1;
          for (uint32_t t = lane; t < cnt; t += 32) {
            const uint32_t lo = sa[i + 2 + t];
            const uint32_t pos = lower_bound_u16(pb + 2, 0, cb, lo);
            c += (pos < cb && pb[2 + pos] == lo);
          }
        }
        i += cnt + 2;
      }
    } else {
      warp_for_each(A, 0xffffffffu, lane, [&](uint32_t y) { c += pshort_contains_staged(B, hdr, y); });
    }
    __syncwarp();  // the table is reused by the warp's next pair
  } else {
    warp_for_each(A, 0xffffffffu, lane, [&](uint32_t y) { c += row_contains(B, y); });
  }
  return c;
}

__device__ __forceinline__ uint32_t warp_intersect_size(const RowView& A, const RowView& B, uint32_t lane,
                                                        PshortHdr* hdr = nullptr) {
  if (!A.card || !B.card) return 0;
  uint32_t c;
  if (A.type == TY_BITSET && B.type == TY_BITSET) {
    const uint32_t lo = max(A.aux, B.aux), hi = min(A.aux + A.len, B.aux + B.len);
    c = lo < hi ? bitset_and_lane(A.p, A.aux, B.p, B.aux, B.len, lo, hi, 0xffffffffu, 0ull, lane) : 0u;
  } else {
    c = A.card > B.card ? warp_intersect_small_large(B, A, lane, hdr) : warp_intersect_small_large(A, B, lane, hdr);
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
    // Coalesced 16-byte loads, kThreads word pairs per round; a round whose
    // pairs are all zero is skipped after one barrier, otherwise a CTA-wide
    // scan of the per-thread popcounts gives each thread its output position.
    const uint32_t lane = tid & 31, warp = tid >> 5, nw = kThreads / 32;
    const int32_t np = (int32_t)((A.len + 1) >> 1);
    uint32_t base_pos = 0;
    for (int32_t base = 0; base < np; base += (int32_t)kThreads) {
      const int32_t q = base + (int32_t)tid;
      const uint4 v = ld_pair(A.p, q, np);
      const unsigned long long x0 = lo64(v), x1 = hi64(v);
      const uint32_t c = __popcll(x0) + __popcll(x1);
      if (!__syncthreads_or(c)) continue;
      const uint32_t ex = warp_exclusive_scan(c, lane);
      if (lane == 31) scan[warp] = ex + c;
      __syncthreads();
      uint32_t woff = 0, total = 0;
      for (uint32_t w = 0; w < nw; w++) {
        const uint32_t t = scan[w];
        woff += w < warp ? t : 0u;
        total += t;
      }
      if (c) emit_pair_bits(x0, x1, A.aux + 2u * (uint32_t)q, list, base_pos + woff + ex);
      base_pos += total;
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
    // 16-byte loads (32 word pairs = 512 bytes per warp round); rounds whose
    // words are all zero cost one vote.
    const int32_t np = (int32_t)((A.len + 1) >> 1);
    uint32_t pos = 0;
    for (int32_t base = 0; base < np; base += 32) {
      const int32_t q = base + (int32_t)lane;
      const uint4 v = ld_pair(A.p, q, np);
      const uint32_t c = __popcll(lo64(v)) + __popcll(hi64(v));
      if (!__any_sync(FULL, c != 0)) continue;
      const uint32_t ex = warp_exclusive_scan(c, lane);
      if (c) emit_pair_bits(lo64(v), hi64(v), A.aux + 2u * (uint32_t)q, list, pos + ex);
      pos += __shfl_sync(FULL, ex + c, 31);
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
