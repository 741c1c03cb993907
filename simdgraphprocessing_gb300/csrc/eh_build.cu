// Device build of the encoded matrix: the reference's SparseMatrix::build ->
// from_symmetric_noattribute_graph (src/SparseMatrix.hpp:268-290,406-494),
// pack_data (:249-266), the layout optimizer hybrid::get_type
// (src/set/layouts/hybrid.hpp:73-100) and the encoders T::build_flattened.
//
// Pass 1 (k_measure: one lane per row of up to 8 entries, one warp per longer
// row, one CTA per row over 4,096 entries in k_measure_big): validate the row
// (offsets rising within the neighbour array, strictly ascending, ids < n),
// apply the edge selection, and measure what the layout needs (count, first,
// last, 16-bit partitions).  Choose the layout and payload size.
// Pass 2: exclusive scan of payload sizes (16-byte units) -> row offsets.
// Pass 3 (k_encode / k_encode_big, the same split): write RowDesc and the
// payload.
#include <algorithm>
#include <cstdint>

#include "eh_kernels.cuh"

namespace eh {

namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ bool is_selected(int sel, uint32_t x, uint64_t row, const uint8_t* mask, uint64_t k) {
  if (sel == 0) return true;
  if (sel == 1) return x < row;
  return mask[k] != 0;
}

// Rows longer than this are measured and encoded by a whole CTA (k_*_big): a
// hub row of a degree-ordered graph would otherwise keep one warp busy long
// after the rest of the grid has finished.
constexpr uint64_t kBigRow = 4096;
constexpr int kBigBlock = 1024;
// Rows up to this many entries are measured and encoded by one lane each (most
// rows of a power-law graph: at R-MAT scale 22, 77% of the rows and 3% of the
// entries), so that a warp does not spend a round of shuffles and ballots on
// each of them.
constexpr uint64_t kLaneRow = 8;

struct SegMeasure {
  uint32_t cnt, parts, first, last, first_hi, last_hi, flags;
};

// One warp measures elements [s0, s1) of `row`: selected count, 16-bit
// partitions (the segment's first selected element counts as a new one),
// first / last selected, and validation flags.  `before` is the element at
// s0 - 1 when s0 > row_begin (for the strictly-ascending check).
__device__ __forceinline__ SegMeasure measure_segment(uint64_t n, uint64_t row, uint64_t row_begin, uint64_t s0,
                                                      uint64_t s1, uint32_t before,
                                                      const uint32_t* __restrict__ nbr,
                                                      const uint8_t* __restrict__ mask, int sel, uint32_t lane) {
  SegMeasure r{0, 0, 0xffffffffu, 0, 0, 0, 0};
  uint32_t carry = 0, last_sel = 0;
  bool have_carry = false;
  for (uint64_t base = s0; base < s1; base += 32) {
    const uint64_t k = base + lane;
    const bool valid = k < s1;
    const uint32_t x = valid ? nbr[k] : 0u;
    // The element before x: from the lane below, or the previous round's last.
    const uint32_t up = __shfl_up_sync(FULL, x, 1);
    const uint32_t prev_raw = lane ? up : before;
    before = __shfl_sync(FULL, x, 31);
    if (valid) {
      if (x >= n) r.flags |= ERRF_RANGE;
      if (k > row_begin && prev_raw >= x) r.flags |= ERRF_UNSORTED;
    }
    const bool s = valid && is_selected(sel, x, row, mask, k);
    const uint32_t bal = __ballot_sync(FULL, s);
    if (s) {
      r.first = min(r.first, x);
      r.last = max(r.last, x);
    }
    // Previous selected element (for counting distinct 16-bit prefixes).
    const uint32_t lower = bal & ((1u << lane) - 1u);
    const int src = lower ? 31 - __clz(lower) : (int)lane;
    const uint32_t px = __shfl_sync(FULL, x, src);
    const bool has_prev = lower != 0 || have_carry;
    const uint32_t prev = lower ? px : carry;
    const bool new_part = s && (!has_prev || (prev >> 16) != (x >> 16));
    r.parts += __popc(__ballot_sync(FULL, new_part));
    if (bal) {
      carry = __shfl_sync(FULL, x, 31 - __clz(bal));
      have_carry = true;
      last_sel = carry;
    }
    r.cnt += __popc(bal);
  }
  r.first = __reduce_min_sync(FULL, r.first);
  r.last = __reduce_max_sync(FULL, r.last);
  r.first_hi = r.first >> 16;
  r.last_hi = last_sel >> 16;
  r.flags = __reduce_or_sync(FULL, r.flags);
  return r;
}

struct RowResult {
  RowMeasure m;
  uint64_t ref;
  uint32_t type;
};

// Layout choice and payload size of one row from its measure (hybrid::get_type,
// src/set/layouts/hybrid.hpp:73-100; the three-tier rule for layout 16).
__device__ __forceinline__ RowResult finish_row(uint32_t cnt, uint32_t parts, uint32_t first, uint32_t last,
                                                int layout) {
  uint32_t type;
  if (layout == TY_UINT) type = TY_UINT;
  else if (layout == TY_BITSET) type = TY_BITSET;
  else if (layout == TY_PSHORT) type = TY_PSHORT;
  else {
    type = TY_UINT;
    if (cnt > 1 && last > first) {
      // The reference tests the double quotient cnt / range against 1/256 (and
      // 1/32).  With integers below 2^53 that equals the integer test
      // 256 * cnt > range: if 256 * cnt > range the quotient exceeds 2^-8 by at
      // least 1 / (256 * range) > 2^-61, more than half an ulp of 2^-8, so the
      // rounded quotient is still above it; otherwise it is at most 2^-8.
      const uint64_t range = (uint64_t)(last - first);
      if (layout == 16) {  // three-tier rule (hybrid::compute_type)
        if (32ull * cnt > range) type = TY_BITSET;
        else if (256ull * cnt > range) type = TY_PSHORT;
      } else if (256ull * cnt > range) {  // hybrid::get_type
        type = TY_BITSET;
      }
    }
  }
  uint32_t len = 0, aux = 0;
  uint64_t bytes = 0, ref = 0;
  if (type == TY_UINT) {
    len = cnt;
    bytes = 4ull * cnt;
    ref = bytes;
  } else if (type == TY_BITSET) {
    if (cnt) {
      aux = first >> 6;
      len = (last >> 6) - aux + 1;
      ref = 4 + 8 + 8ull * len;
    }
    bytes = 8ull * len;
  } else {
    if (cnt) {
      aux = parts;
      len = cnt + 2 * parts;
      ref = 4 + 2ull * len;
    }
    bytes = 2ull * len;
  }
  const bool hybrid = (layout != TY_UINT && layout != TY_BITSET && layout != TY_PSHORT);
  if (hybrid) ref += 8;
  const uint32_t units = (uint32_t)((bytes + 15) / 16);
  return RowResult{RowMeasure{cnt, aux, make_lt(type, len), units}, ref, type};
}

struct Totals {
  unsigned long long card = 0, ref = 0, units = 0, max_full = 0, max_card = 0;
  uint32_t n_uint = 0, n_pshort = 0, n_bitset = 0;
  __device__ __forceinline__ void add(const RowResult& r, uint64_t full) {
    card += r.m.card;
    ref += r.ref;
    units += r.m.units;
    n_uint += r.type == TY_UINT;
    n_pshort += r.m.card && r.type == TY_PSHORT;
    n_bitset += r.m.card && r.type == TY_BITSET;
    max_full = max(max_full, (unsigned long long)full);
    max_card = max(max_card, (unsigned long long)r.m.card);
  }
  // Sums / maxima over the warp, left in every lane.
  __device__ __forceinline__ void warp_reduce() {
    card = warp_sum_u64(card);
    ref = warp_sum_u64(ref);
    units = warp_sum_u64(units);
    for (int d = 16; d; d >>= 1) {
      max_full = max(max_full, __shfl_xor_sync(FULL, max_full, d));
      max_card = max(max_card, __shfl_xor_sync(FULL, max_card, d));
    }
    n_uint = __reduce_add_sync(FULL, n_uint);
    n_pshort = __reduce_add_sync(FULL, n_pshort);
    n_bitset = __reduce_add_sync(FULL, n_bitset);
  }
  __device__ __forceinline__ void flush(BuildTotals* tot) const {
    if (card) atomicAdd(&tot->cardinality, card);
    if (ref) atomicAdd(&tot->ref_bytes, ref);
    if (n_uint) atomicAdd(&tot->num_uint, (unsigned long long)n_uint);
    if (n_pshort) atomicAdd(&tot->num_pshort, (unsigned long long)n_pshort);
    if (n_bitset) atomicAdd(&tot->num_bitset, (unsigned long long)n_bitset);
    if (units) atomicAdd(&tot->payload_units, units);
    if (max_full) atomicMax(&tot->max_full_degree, max_full);
    if (max_card) atomicMax(&tot->max_card, max_card);
  }
};

__global__ void __launch_bounds__(kBlock) k_measure(uint64_t n, uint64_t total, uint64_t r_begin, uint64_t r_end,
                                                    const uint64_t* __restrict__ off,
                                                    const uint32_t* __restrict__ nbr,
                                                    const uint8_t* __restrict__ mask, int sel,
                                                    int layout, RowMeasure* __restrict__ meas,
                                                    BuildTotals* __restrict__ tot,
                                                    uint32_t* __restrict__ err, uint32_t* __restrict__ big,
                                                    uint32_t* __restrict__ n_big) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t nw = (uint64_t)gridDim.x * (kBlock / 32);
  uint32_t flags = 0;
  Totals t;  // this lane's running totals (summed over the warp, one atomic each at the end)
  // Rows [r_begin, r_end) are dealt to warps round-robin (row = r_begin + warp
  // + i * warps, so that the degree-ordered hubs at the front spread over the
  // grid); a warp loads the offsets of its next 32 rows at once (lane q: its
  // q-th row).  Each lane measures its own row if it has at most kLaneRow
  // entries; the warp then measures the longer ones one by one.
  for (uint64_t row0 = r_begin + (uint64_t)blockIdx.x * (kBlock / 32) + (threadIdx.x >> 5); row0 < r_end;
       row0 += nw * 32) {
    const uint64_t my = row0 + lane * nw;
    uint64_t my_b = my < r_end ? off[my] : 0, my_e = my < r_end ? off[my + 1] : 0;
    if (my_e < my_b || my_e > total) {  // offsets must rise monotonically within the nbr array
      flags |= ERRF_OFFSETS;
      my_b = my_e = 0;
    }
    const bool lane_row = my < r_end && my_e - my_b <= kLaneRow;
    if (lane_row) {
      uint32_t cnt = 0, parts = 0, first = 0xffffffffu, last = 0, prev = 0, prev_hi = 0;
      for (uint64_t k = my_b; k < my_e; k++) {
        const uint32_t x = nbr[k];
        if (x >= n) flags |= ERRF_RANGE;
        if (k > my_b && prev >= x) flags |= ERRF_UNSORTED;
        prev = x;
        if (is_selected(sel, x, my, mask, k)) {
          if (cnt == 0 || (x >> 16) != prev_hi) parts++;  // a new 16-bit partition
          prev_hi = x >> 16;
          first = min(first, x);
          last = max(last, x);
          cnt++;
        }
      }
      const RowResult r = finish_row(cnt, parts, first, last, layout);
      meas[my] = r.m;
      t.add(r, my_e - my_b);
    }
    for (uint32_t rest = __ballot_sync(FULL, my < r_end && !lane_row); rest; rest &= rest - 1) {
      const uint32_t q = __ffs(rest) - 1;
      const uint64_t row = row0 + q * nw;
      const uint64_t b = __shfl_sync(FULL, my_b, q), e = __shfl_sync(FULL, my_e, q);
      if (e - b > kBigRow) {
        if (lane == 0) big[atomicAdd(n_big, 1u)] = (uint32_t)row;
        continue;
      }
      const SegMeasure sm = measure_segment(n, row, b, b, e, 0u, nbr, mask, sel, lane);
      flags |= sm.flags;
      if (lane == 0) {
        const RowResult r = finish_row(sm.cnt, sm.parts, sm.first, sm.last, layout);
        if (sm.cnt >= (1u << 28)) flags |= ERRF_ROW_TOO_LONG;
        meas[row] = r.m;
        t.add(r, e - b);
      }
    }
  }
  t.warp_reduce();
  flags = __reduce_or_sync(FULL, flags);
  if (lane == 0) {
    t.flush(tot);
    if (flags) atomicOr(err, flags);
  }
}

// Rows longer than kBigRow, one CTA of kBigBlock threads each: warp w measures
// the w-th slice of the row; thread 0 merges the slices in order (a slice whose
// first 16-bit partition continues the previous non-empty slice's last one does
// not start a new partition).
__global__ void __launch_bounds__(kBigBlock) k_measure_big(uint64_t n, const uint64_t* __restrict__ off,
                                                           const uint32_t* __restrict__ nbr,
                                                           const uint8_t* __restrict__ mask, int sel, int layout,
                                                           RowMeasure* __restrict__ meas,
                                                           BuildTotals* __restrict__ tot, uint32_t* __restrict__ err,
                                                           const uint32_t* __restrict__ big,
                                                           const uint32_t* __restrict__ big_begin,
                                                           const uint32_t* __restrict__ big_end) {
  constexpr int NWB = kBigBlock / 32;
  __shared__ SegMeasure s_seg[NWB];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t nb = *big_end;
  Totals t;
  uint32_t flags = 0;
  for (uint32_t i = *big_begin + blockIdx.x; i < nb; i += gridDim.x) {
    const uint64_t row = big[i];
    const uint64_t b = off[row], e = off[row + 1];
    const uint64_t slice = ((e - b + NWB - 1) / NWB + 31) & ~31ull;
    const uint64_t s0 = min(e, b + warp * slice), s1 = min(e, s0 + slice);
    const uint32_t before = s0 > b ? nbr[s0 - 1] : 0u;
    const SegMeasure sm = measure_segment(n, row, b, s0, s1, before, nbr, mask, sel, lane);
    if (lane == 0) s_seg[warp] = sm;
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t cnt = 0, parts = 0, first = 0xffffffffu, last = 0, prev_hi = 0;
      bool any = false;
      for (int w = 0; w < NWB; w++) {
        const SegMeasure& g = s_seg[w];
        flags |= g.flags;
        if (!g.cnt) continue;
        cnt += g.cnt;
        parts += g.parts - (any && prev_hi == g.first_hi ? 1u : 0u);
        first = min(first, g.first);
        last = max(last, g.last);
        prev_hi = g.last_hi;
        any = true;
      }
      const RowResult r = finish_row(cnt, parts, first, last, layout);
      if (cnt >= (1u << 28)) flags |= ERRF_ROW_TOO_LONG;
      meas[row] = r.m;
      t.add(r, e - b);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    t.flush(tot);
    if (flags) atomicOr(err, flags);
  }
}

// ---- exclusive scan of u32 values (three passes: tiles, tile sums, add) ----
constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr uint64_t kScanTile = (uint64_t)kScanThreads * kScanItems;

struct UnitsOf {
  const RowMeasure* m;
  __device__ uint32_t operator()(uint64_t i) const { return m[i].units; }
};
struct Plain {
  const uint32_t* a;
  __device__ uint32_t operator()(uint64_t i) const { return a[i]; }
};

// Block-wide exclusive scan of one value per thread; returns the block total.
__device__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* excl) {
  constexpr int NW = kScanThreads / 32;
  __shared__ uint32_t s_warp[NW];
  __shared__ uint32_t s_total;
  const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t inc = v;
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t t = __shfl_up_sync(FULL, inc, d);
    if (lane >= (uint32_t)d) inc += t;
  }
  if (lane == 31) s_warp[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    const uint32_t w = lane < NW ? s_warp[lane] : 0u;
    uint32_t wi = w;
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t t = __shfl_up_sync(FULL, wi, d);
      if (lane >= (uint32_t)d) wi += t;
    }
    if (lane < NW) s_warp[lane] = wi - w;
    if (lane == 31) s_total = wi;
  }
  __syncthreads();
  *excl = inc - v + s_warp[wid];
  const uint32_t total = s_total;
  __syncthreads();  // s_warp / s_total are reused by the next call
  return total;
}

template <class In>
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(In in, uint64_t n, uint32_t* out, uint32_t* tile_sums) {
  const uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    v[k] = (base + k < n) ? in(base + k) : 0u;
    s += v[k];
  }
  uint32_t excl;
  uint32_t total = block_exclusive_scan(s, &excl);
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    if (base + k < n) out[base + k] = excl;
    excl += v[k];
  }
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

// One block scans all tile sums (looping with a carry), exclusive, in place.
__global__ void __launch_bounds__(kScanThreads) k_scan_sums(uint32_t* sums, uint64_t m) {
  __shared__ uint32_t s_carry;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (uint64_t base = 0; base < m; base += kScanThreads) {
    const uint64_t i = base + threadIdx.x;
    const uint32_t v = i < m ? sums[i] : 0u;
    uint32_t excl;
    const uint32_t total = block_exclusive_scan(v, &excl);
    const uint32_t carry = s_carry;
    if (i < m) sums[i] = excl + carry;
    __syncthreads();
    if (threadIdx.x == 0) s_carry = carry + total;
    __syncthreads();
  }
}

__global__ void k_scan_add(uint32_t* out, uint64_t n, const uint32_t* tile_sums) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += tile_sums[i / kScanTile];
}

template <class In>
cudaError_t exclusive_scan(In in, uint64_t n, uint32_t* out, uint32_t* tmp, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const uint64_t tiles = (n + kScanTile - 1) / kScanTile;
  k_scan_tiles<In><<<(unsigned)tiles, kScanThreads, 0, st>>>(in, n, out, tmp);
  k_scan_sums<<<1, kScanThreads, 0, st>>>(tmp, tiles);
  k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, n, tmp);
  return cudaGetLastError();
}

// Sequential partition writer (pshort::build, pshort.hpp:46-78): [hi][count-1][lo...].
__device__ void write_pshort(uint16_t* s, uint64_t row, uint64_t b, uint64_t e, const uint32_t* __restrict__ nbr,
                             const uint8_t* __restrict__ mask, int sel) {
  uint32_t w = 0, size_pos = 1, plen = 0, high = 0;
  bool started = false;
  for (uint64_t k = b; k < e; k++) {
    const uint32_t x = nbr[k];
    if (!is_selected(sel, x, row, mask, k)) continue;
    const uint32_t hi = x >> 16, lo = x & 0xffffu;
    if (started && hi == high) {
      plen++;
      s[w++] = (uint16_t)lo;
    } else {
      if (started) s[size_pos] = (uint16_t)plen;
      s[w] = (uint16_t)hi;
      s[w + 1] = 0;
      s[w + 2] = (uint16_t)lo;
      size_pos = w + 1;
      w += 3;
      plen = 0;
      high = hi;
      started = true;
    }
  }
  s[size_pos] = (uint16_t)plen;
}

// Warp-parallel form of write_pshort over a slice nbr[s0, s1) of a row.  In
// the payload, the selected element of rank s (0-based among the row's
// selected elements) in partition P (0-based) sits at u16 position
// s + 2 (P + 1), and partition P's header [hi][count - 1] at f_P + 2 P, where
// f_P is the rank of its first element.  So each element finds its slot from
// two warp prefix counts (selected elements and partition starts before it); a
// partition's first element writes its header's hi and the size of the
// partition before it (its own rank minus that partition's first rank, minus
// one).  `c` carries the row's state into the slice (rank of its first
// selected element, index of the open partition or -1, that partition's first
// rank and high half); the returned carry continues after the slice.  The
// size of the row's last partition is left to the caller.
struct PshortCarry {
  uint64_t s;           // rank of the next selected element
  int32_t part;         // partition of the last selected element so far (-1: none)
  uint64_t open_first;  // rank of that partition's first element
  uint32_t hi;          // its high half
};
__device__ PshortCarry warp_write_pshort(uint16_t* out, uint64_t row, uint64_t s0, uint64_t s1,
                                         const uint32_t* __restrict__ nbr, const uint8_t* __restrict__ mask,
                                         int sel, uint32_t lane, PshortCarry c) {
  const uint32_t lt = (1u << lane) - 1u;
  for (uint64_t base = s0; base < s1; base += 32) {
    const uint64_t k = base + lane;
    const bool valid = k < s1;
    const uint32_t x = valid ? nbr[k] : 0u;
    const bool take = valid && is_selected(sel, x, row, mask, k);
    const uint32_t bal = __ballot_sync(FULL, take);
    if (!bal) continue;
    const uint32_t hi = x >> 16;
    const uint32_t below = bal & lt;
    const uint32_t ph = __shfl_sync(FULL, hi, below ? 31 - __clz(below) : lane);
    const bool first = take && (below ? ph != hi : (c.part < 0 || c.hi != hi));
    const uint32_t fbal = __ballot_sync(FULL, first);
    const uint64_t rank = c.s + __popc(below);
    const int32_t part = c.part + (int32_t)__popc(fbal & (lt | (1u << lane)));
    const uint32_t fbelow = fbal & lt;
    const uint64_t fr = __shfl_sync(FULL, rank, fbelow ? 31 - __clz(fbelow) : lane);
    if (take) out[rank + 2 * (uint64_t)(part + 1)] = (uint16_t)(x & 0xffffu);
    if (first) {
      out[rank + 2 * (uint64_t)part] = (uint16_t)hi;
      if (part > 0) {
        const uint64_t pf = fbelow ? fr : c.open_first;  // first rank of partition part - 1
        out[pf + 2 * (uint64_t)(part - 1) + 1] = (uint16_t)(rank - pf - 1);
      }
    }
    const uint32_t top = 31 - __clz(bal);
    c.hi = __shfl_sync(FULL, hi, top);
    if (fbal) c.open_first = __shfl_sync(FULL, rank, 31 - __clz(fbal));
    c.s += __popc(bal);
    c.part += (int32_t)__popc(fbal);
  }
  return c;
}

// Per-slice summary for the CTA form: selected elements, partition starts
// counted as if the slice began a row, the first and last high halves, and the
// slice-local rank of its last such start.
struct PshortSlice {
  uint32_t cnt, starts, first_hi, last_hi, last_start;
};
__device__ PshortSlice warp_scan_pshort(uint64_t row, uint64_t s0, uint64_t s1, const uint32_t* __restrict__ nbr,
                                        const uint8_t* __restrict__ mask, int sel, uint32_t lane) {
  PshortSlice r{0, 0, 0, 0, 0};
  const uint32_t lt = (1u << lane) - 1u;
  for (uint64_t base = s0; base < s1; base += 32) {
    const uint64_t k = base + lane;
    const bool valid = k < s1;
    const uint32_t x = valid ? nbr[k] : 0u;
    const bool take = valid && is_selected(sel, x, row, mask, k);
    const uint32_t bal = __ballot_sync(FULL, take);
    if (!bal) continue;
    const uint32_t hi = x >> 16;
    const uint32_t below = bal & lt;
    const uint32_t ph = __shfl_sync(FULL, hi, below ? 31 - __clz(below) : lane);
    const bool first = take && (below ? ph != hi : (r.cnt == 0 || r.last_hi != hi));
    const uint32_t fbal = __ballot_sync(FULL, first);
    if (r.cnt == 0) r.first_hi = __shfl_sync(FULL, hi, __ffs(bal) - 1);
    if (fbal) r.last_start = r.cnt + __popc(bal & ((1u << (31 - __clz(fbal))) - 1u));
    r.last_hi = __shfl_sync(FULL, hi, 31 - __clz(bal));
    r.cnt += __popc(bal);
    r.starts += __popc(fbal);
  }
  return r;
}

__global__ void __launch_bounds__(kBlock, 6) k_encode(uint64_t n, const uint64_t* __restrict__ off,
                                                   const uint32_t* __restrict__ nbr,
                                                   const uint8_t* __restrict__ mask, int sel,
                                                   const RowMeasure* __restrict__ meas,
                                                   const uint32_t* __restrict__ off16,
                                                   RowDesc* __restrict__ desc, uint4* __restrict__ arena) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t nw = (uint64_t)gridDim.x * (kBlock / 32);
  // Rows are dealt to warps round-robin as in k_measure; lane q loads the measure,
  // offsets and payload start of the warp's q-th next row and writes its
  // RowDesc and, for rows of at most kLaneRow entries, its payload; the warp
  // then writes the longer rows' payloads one row after another (rows longer
  // than kBigRow are left to k_encode_big).
  for (uint64_t row0 = (uint64_t)blockIdx.x * (kBlock / 32) + (threadIdx.x >> 5); row0 < n; row0 += nw * 32) {
    const uint64_t my = row0 + lane * nw;
    RowMeasure mm{0, 0, 0, 0};
    uint64_t my_b = 0, my_e = 0;
    uint32_t my_o = 0;
    if (my < n) {
      mm = meas[my];
      my_o = off16[my];
      my_b = off[my];
      my_e = off[my + 1];
      desc[my] = RowDesc{my_o, mm.card, mm.aux, mm.lt};
    }
    const bool lane_row = my < n && my_e - my_b <= kLaneRow;
    if (lane_row && mm.card) {  // the lane owns the row's payload units
      uint4* dst = arena + my_o;
      const uint32_t type = mm.lt >> 30;
      if (type == TY_PSHORT) {
        write_pshort(reinterpret_cast<uint16_t*>(dst), my, my_b, my_e, nbr, mask, sel);
      } else if (type == TY_UINT) {
        uint32_t* a = reinterpret_cast<uint32_t*>(dst);
        for (uint64_t k = my_b; k < my_e; k++) {
          const uint32_t x = nbr[k];
          if (is_selected(sel, x, my, mask, k)) *a++ = x;
        }
      } else {
        unsigned long long* words = reinterpret_cast<unsigned long long*>(dst);
        for (uint64_t k = my_b; k < my_e; k++) {
          const uint32_t x = nbr[k];
          if (is_selected(sel, x, my, mask, k)) words[(x >> 6) - mm.aux] |= 1ull << (x & 63);
        }
      }
    }
    for (uint32_t rest = __ballot_sync(FULL, my < n && !lane_row && mm.card != 0); rest; rest &= rest - 1) {
      const uint32_t q = __ffs(rest) - 1;
      const uint64_t row = row0 + q * nw;
      const uint32_t aux = __shfl_sync(FULL, mm.aux, q);
      const uint32_t type = __shfl_sync(FULL, mm.lt, q) >> 30;
      const uint64_t b = __shfl_sync(FULL, my_b, q), e = __shfl_sync(FULL, my_e, q);
      if (e - b > kBigRow) continue;
      uint4* dst = arena + __shfl_sync(FULL, my_o, q);
      if (type == TY_PSHORT) {
        uint16_t* out = reinterpret_cast<uint16_t*>(dst);
        const PshortCarry c = warp_write_pshort(out, row, b, e, nbr, mask, sel, lane, PshortCarry{0, -1, 0, 0});
        if (lane == 0 && c.part >= 0) out[c.open_first + 2 * (uint64_t)c.part + 1] = (uint16_t)(c.s - c.open_first - 1);
        continue;
      }
      uint32_t k_sel = 0;
      for (uint64_t base = b; base < e; base += 32) {
        const uint64_t k = base + lane;
        const bool valid = k < e;
        const uint32_t x = valid ? nbr[k] : 0u;
        const bool s = valid && is_selected(sel, x, row, mask, k);
        const uint32_t bal = __ballot_sync(FULL, s);
        if (s) {
          if (type == TY_UINT) {
            reinterpret_cast<uint32_t*>(dst)[k_sel + __popc(bal & ((1u << lane) - 1u))] = x;
          } else {
            unsigned long long* words = reinterpret_cast<unsigned long long*>(dst);
            atomicOr(&words[(x >> 6) - aux], 1ull << (x & 63));
          }
        }
        k_sel += __popc(bal);
      }
    }
  }
}

// Payloads of the rows longer than kBigRow, one CTA each: warp w writes the
// w-th slice of the row (uint rows: at the slice's output position, from a
// count pass over the slices; bitset rows: one atomic OR per element; pshort
// rows keep the sequential writer).
__global__ void __launch_bounds__(kBigBlock) k_encode_big(const uint64_t* __restrict__ off,
                                                          const uint32_t* __restrict__ nbr,
                                                          const uint8_t* __restrict__ mask, int sel,
                                                          const RowMeasure* __restrict__ meas,
                                                          const uint32_t* __restrict__ off16,
                                                          uint4* __restrict__ arena, const uint32_t* __restrict__ big,
                                                          const uint32_t* __restrict__ n_big) {
  constexpr int NWB = kBigBlock / 32;
  __shared__ uint32_t s_cnt[NWB];
  __shared__ PshortSlice s_ps[NWB];
  __shared__ PshortCarry s_carry[NWB];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t nb = *n_big;
  for (uint32_t i = blockIdx.x; i < nb; i += gridDim.x) {
    const uint64_t row = big[i];
    const RowMeasure m = meas[row];
    const uint32_t type = m.lt >> 30;
    if (m.card == 0) continue;
    const uint64_t b = off[row], e = off[row + 1];
    uint4* dst = arena + off16[row];
    const uint64_t slice = ((e - b + NWB - 1) / NWB + 31) & ~31ull;
    const uint64_t s0 = min(e, b + warp * slice), s1 = min(e, s0 + slice);
    if (type == TY_PSHORT) {
      // Each warp summarises its slice, one thread chains the summaries into
      // each slice's carry-in, then every warp writes its slice.
      uint16_t* out = reinterpret_cast<uint16_t*>(dst);
      const PshortSlice ps = warp_scan_pshort(row, s0, s1, nbr, mask, sel, lane);
      if (lane == 0) s_ps[warp] = ps;
      __syncthreads();
      if (threadIdx.x == 0) {
        PshortCarry c{0, -1, 0, 0};
        for (int w = 0; w < NWB; w++) {
          s_carry[w] = c;
          const PshortSlice& q = s_ps[w];
          if (q.cnt == 0) continue;
          const uint32_t joins = (c.part >= 0 && c.hi == q.first_hi) ? 1u : 0u;  // slice continues the open partition
          if (q.starts > joins) c.open_first = c.s + q.last_start;
          c.part += (int32_t)(q.starts - joins);
          c.s += q.cnt;
          c.hi = q.last_hi;
        }
        if (c.part >= 0) out[c.open_first + 2 * (uint64_t)c.part + 1] = (uint16_t)(c.s - c.open_first - 1);
      }
      __syncthreads();
      warp_write_pshort(out, row, s0, s1, nbr, mask, sel, lane, s_carry[warp]);
      __syncthreads();  // s_ps / s_carry are rewritten for the next row
      continue;
    }
    if (type == TY_BITSET) {
      unsigned long long* words = reinterpret_cast<unsigned long long*>(dst);
      for (uint64_t k = s0 + lane; k < s1; k += 32) {
        const uint32_t x = nbr[k];
        if (is_selected(sel, x, row, mask, k)) atomicOr(&words[(x >> 6) - m.aux], 1ull << (x & 63));
      }
      continue;
    }
    uint32_t c = 0;
    for (uint64_t base = s0; base < s1; base += 32) {
      const uint64_t k = base + lane;
      c += __popc(__ballot_sync(FULL, k < s1 && is_selected(sel, nbr[k < s1 ? k : s0], row, mask, k)));
    }
    if (lane == 0) s_cnt[warp] = c;
    __syncthreads();
    uint32_t k_sel = 0;
    for (uint32_t w = 0; w < warp; w++) k_sel += s_cnt[w];
    for (uint64_t base = s0; base < s1; base += 32) {
      const uint64_t k = base + lane;
      const bool valid = k < s1;
      const uint32_t x = valid ? nbr[k] : 0u;
      const bool s = valid && is_selected(sel, x, row, mask, k);
      const uint32_t bal = __ballot_sync(FULL, s);
      if (s) reinterpret_cast<uint32_t*>(dst)[k_sel + __popc(bal & ((1u << lane) - 1u))] = x;
      k_sel += __popc(bal);
    }
    __syncthreads();  // s_cnt is rewritten for the next row
  }
}

// Row order by descending card: a histogram over 65,536 card buckets, a scan,
// then a scatter.  Most rows share a few small cards, so lanes of a warp with
// the same bucket combine their atomics (one per bucket and warp).
__global__ void k_plan_hist(uint64_t n, const RowDesc* __restrict__ desc, uint32_t min_card,
                            uint32_t* __restrict__ hist) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t r0 = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); r0 < n; r0 += step) {
    const uint64_t r = r0 + lane;
    const uint32_t c = r < n ? desc[r].card : 0u;
    const bool take = r < n && c >= min_card;
    const uint32_t bucket = take ? 65535u - min(c, 65535u) : 0xffffffffu;
    const uint32_t peers = __match_any_sync(FULL, bucket);
    if (take && lane == (uint32_t)(__ffs(peers) - 1)) atomicAdd(&hist[bucket], (uint32_t)__popc(peers));
  }
}
__global__ void k_plan_scatter(uint64_t n, const RowDesc* __restrict__ desc, uint32_t min_card,
                               uint32_t* __restrict__ cursor, uint32_t* __restrict__ order) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t r0 = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); r0 < n; r0 += step) {
    const uint64_t r = r0 + lane;
    const uint32_t c = r < n ? desc[r].card : 0u;
    const bool take = r < n && c >= min_card;
    const uint32_t bucket = take ? 65535u - min(c, 65535u) : 0xffffffffu;
    const uint32_t peers = __match_any_sync(FULL, bucket);
    const uint32_t leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (take && lane == leader) base = atomicAdd(&cursor[bucket], (uint32_t)__popc(peers));
    base = __shfl_sync(FULL, base, leader);
    if (take) order[base + __popc(peers & ((1u << lane) - 1u))] = (uint32_t)r;
  }
}

// Decodes whole rows into plain sorted u32 lists (one block per row).
// out[u] = desc[rows[u]]: the descriptors of a list of rows, for one copy to the host.
__global__ void k_gather_desc(const RowDesc* __restrict__ desc, const uint32_t* __restrict__ rows, uint32_t nrows,
                              RowDesc* __restrict__ out) {
  const uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u < nrows) out[u] = desc[rows[u]];
}

__global__ void k_decode_rows(const RowDesc* __restrict__ desc, const uint4* __restrict__ arena,
                              const uint32_t* __restrict__ rows,
                              const unsigned long long* __restrict__ dst_off, uint32_t* __restrict__ dst) {
  const RowView V = load_view(desc, arena, rows[blockIdx.x]);
  uint32_t* out = dst + dst_off[blockIdx.x];
  if (V.type == TY_UINT) {
    const uint32_t* a = static_cast<const uint32_t*>(V.p);
    for (uint32_t k = threadIdx.x; k < V.card; k += blockDim.x) out[k] = a[k];
    return;
  }
  if (threadIdx.x >= 32) return;  // one warp walks bitset words / pshort partitions in order
  const uint32_t lane = threadIdx.x;
  uint32_t pos = 0;
  if (V.type == TY_BITSET) {
    const unsigned long long* w = static_cast<const unsigned long long*>(V.p);
    for (uint32_t base = 0; base < V.len; base += 32) {
      const uint32_t k = base + lane;
      unsigned long long x = k < V.len ? w[k] : 0ull;
      const uint32_t c = __popcll(x);
      uint32_t inc = c;
      for (int d = 1; d < 32; d <<= 1) {
        uint32_t t = __shfl_up_sync(FULL, inc, d);
        if (lane >= (uint32_t)d) inc += t;
      }
      uint32_t p = pos + inc - c;
      while (x) {
        out[p++] = 64u * (V.aux + k) + (uint32_t)(__ffsll((long long)x) - 1);
        x &= x - 1ull;
      }
      pos += __shfl_sync(FULL, inc, 31);
    }
  } else {
    const uint16_t* s = static_cast<const uint16_t*>(V.p);
    uint32_t i = 0;
    while (i < V.len) {
      const uint32_t hb = (uint32_t)s[i] << 16, cnt = (uint32_t)s[i + 1] + 1;
      for (uint32_t k = lane; k < cnt; k += 32) out[pos + k] = hb | s[i + 2 + k];
      pos += cnt;
      i += cnt + 2;
    }
  }
}

// Algorithmic bytes of one triangle pass: sum_i [8 + bytes(A_i)] + sum_{j in A_i} bytes(B_j).
__global__ void __launch_bounds__(kBlock) k_triangle_bytes(uint64_t n, const RowDesc* __restrict__ desc,
                                                           const uint4* __restrict__ arena,
                                                           unsigned long long* __restrict__ out) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t nw = (uint64_t)gridDim.x * (kBlock / 32);
  unsigned long long acc = 0;
  for (uint64_t row = (uint64_t)blockIdx.x * (kBlock / 32) + (threadIdx.x >> 5); row < n; row += nw) {
    const RowView A = load_view(desc, arena, (uint32_t)row);
    if (lane == 0) acc += 8 + payload_bytes(A);
    warp_for_each(A, 0xffffffffu, lane, [&](uint32_t j) { acc += payload_bytes(load_view(desc, arena, j)); });
  }
  acc = warp_sum_u64(acc);
  if (lane == 0) atomicAdd(out, acc);
}

__global__ void k_max_row(uint64_t n, const RowDesc* __restrict__ desc, unsigned long long* out) {
  unsigned long long best = 0;
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (uint64_t)gridDim.x * blockDim.x) {
    // Largest card wins; among equals the smallest row id (SparseMatrix::get_max_row_id
    // keeps the first strict maximum).
    const unsigned long long key = ((unsigned long long)desc[r].card << 32) | (0xffffffffu - (uint32_t)r);
    best = key > best ? key : best;
  }
  for (int d = 16; d; d >>= 1) {
    unsigned long long o = __shfl_xor_sync(FULL, best, d);
    best = o > best ? o : best;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(out, best);
}

}  // namespace

static int grid_for(uint64_t items, int per_block) {
  uint64_t g = (items + per_block - 1) / per_block;
  if (g < 1) g = 1;
  if (g > 152ull * 64) g = 152ull * 64;
  return (int)g;
}

cudaError_t launch_measure_rows(uint64_t n, uint64_t total, uint64_t r_begin, uint64_t r_end, const uint64_t* off,
                                const uint32_t* nbr, const uint8_t* mask, int sel, int layout, RowMeasure* meas,
                                BuildTotals* totals, uint32_t* err, uint32_t* big, uint32_t* n_big, cudaStream_t st) {
  if (r_end <= r_begin) return cudaSuccess;
  k_measure<<<grid_for(r_end - r_begin, kBlock / 32), kBlock, 0, st>>>(n, total, r_begin, r_end, off, nbr, mask, sel,
                                                                        layout, meas, totals, err, big, n_big);
  return cudaGetLastError();
}

cudaError_t launch_measure_big(uint64_t n, const uint64_t* off, const uint32_t* nbr, const uint8_t* mask, int sel,
                               int layout, RowMeasure* meas, BuildTotals* totals, uint32_t* err, const uint32_t* big,
                               const uint32_t* big_begin, const uint32_t* big_end, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_measure_big<<<2 * 152, kBigBlock, 0, st>>>(n, off, nbr, mask, sel, layout, meas, totals, err, big, big_begin,
                                               big_end);
  return cudaGetLastError();
}

uint64_t big_row_capacity(uint64_t n, uint64_t total) { return std::min<uint64_t>(n, total / kBigRow + 1); }

uint64_t scan_tmp_words(uint64_t n) { return (n + kScanTile - 1) / kScanTile + 1; }

cudaError_t launch_scan_units(uint64_t n, const RowMeasure* meas, uint32_t* off16, uint32_t* tmp,
                              uint64_t n_tmp, cudaStream_t st) {
  (void)n_tmp;
  return exclusive_scan(UnitsOf{meas}, n, off16, tmp, st);
}

cudaError_t launch_encode(uint64_t n, const uint64_t* off, const uint32_t* nbr, const uint8_t* mask,
                          int sel, const RowMeasure* meas, const uint32_t* off16, RowDesc* desc,
                          uint4* arena, const uint32_t* big, const uint32_t* n_big, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_encode<<<grid_for(n, kBlock / 32), kBlock, 0, st>>>(n, off, nbr, mask, sel, meas, off16, desc, arena);
  k_encode_big<<<2 * 152, kBigBlock, 0, st>>>(off, nbr, mask, sel, meas, off16, arena, big, n_big);
  return cudaGetLastError();
}

// hist: 65536 + scan tmp words; counts[0] = rows in plan (host reads order count
// from the scanned histogram).
cudaError_t launch_plan(uint64_t n, const RowDesc* desc, uint32_t min_card, uint32_t* hist,
                        uint32_t* order, uint32_t* cursor, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(hist, 0, 65536 * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  if (n == 0) return cudaSuccess;
  k_plan_hist<<<grid_for(n, 256), 256, 0, st>>>(n, desc, min_card, hist);
  e = exclusive_scan(Plain{hist}, 65536, cursor, hist + 65536, st);
  if (e != cudaSuccess) return e;
  // Keep the scanned starts (cursor is advanced by the scatter): copy them after the
  // histogram so that the host can read bin starts.
  e = cudaMemcpyAsync(hist, cursor, 65536 * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return e;
  k_plan_scatter<<<grid_for(n, 256), 256, 0, st>>>(n, desc, min_card, cursor, order);
  return cudaGetLastError();
}

cudaError_t exclusive_scan_u32(const uint32_t* in, uint64_t n, uint32_t* out, uint32_t* tmp,
                               cudaStream_t st) {
  return exclusive_scan(Plain{in}, n, out, tmp, st);
}

cudaError_t launch_gather_desc(const RowDesc* desc, const uint32_t* rows, uint32_t nrows, RowDesc* out,
                               cudaStream_t st) {
  if (nrows == 0) return cudaSuccess;
  k_gather_desc<<<(nrows + 255) / 256, 256, 0, st>>>(desc, rows, nrows, out);
  return cudaGetLastError();
}

cudaError_t launch_decode_rows(const RowDesc* desc, const uint4* arena, const uint32_t* rows,
                               const unsigned long long* dst_off, uint32_t nrows, uint32_t* dst,
                               cudaStream_t st) {
  if (nrows == 0) return cudaSuccess;
  k_decode_rows<<<nrows, 256, 0, st>>>(desc, arena, rows, dst_off, dst);
  return cudaGetLastError();
}

cudaError_t launch_triangle_bytes(uint64_t n, const RowDesc* desc, const uint4* arena,
                                  unsigned long long* out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_triangle_bytes<<<grid_for(n, kBlock / 32), kBlock, 0, st>>>(n, desc, arena, out);
  return cudaGetLastError();
}

cudaError_t launch_max_row(uint64_t n, const RowDesc* desc, unsigned long long* out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_max_row<<<grid_for(n, 256), 256, 0, st>>>(n, desc, out);
  return cudaGetLastError();
}

}  // namespace eh
