// k-clique counting: the reference's n_clique<T,R>::run / apply_function
// (apps/n_clique.cpp:30-101).
//
// The reference walks, for every pivot i and j in A_i = row(i) (rows pruned to
// nbr < node), the materialized intersection C = A_i ∩ row(j), then for each
// k in C the intersection C ∩ row(k), and so on to depth n, returning |C| at
// the last level.  Every set on that path is a subset of A_i, so here each is a
// bitmask over the positions of A_i: M[e] = {t < e : A_i[t] in row(A_i[e])} is
// A_i ∩ row(A_i[e]) (row(j) only holds ids below j), and the reference's
// C ∩ row(k) for k = A_i[t] is M[e] & M[t].  The masks are built with the same
// layout-aware choice as the triangle kernel (probe each A_i[t] into row(j), or
// stream row(j) and look each element up in A_i); the counting is popcounts of
// ANDs:
//   k = 3: sum_e popc(M[e])
//   k = 4: sum_e sum_{t in M[e]} popc(M[e] & M[t])
//   k > 4: depth-first over the same masks.
// Tiers by |A_i| (rows sorted by descending size): one warp per pivot with
// one-word masks (|A_i| <= 32); one CTA per pivot with masks in shared memory
// (up to clique_smem_cap(k), about 1,650-1,850 entries), launched in size bands
// so that each launch's shared memory (and so its CTAs per SM) fits its own
// largest pivot; one CTA per pivot with masks in a global scratch slot (larger
// pivots).  The masks are stored as a packed lower-triangular bit matrix.
#include <algorithm>
#include <atomic>
#include <map>
#include <mutex>
#include <cstdint>

#include "eh_kernels.cuh"

namespace eh {

namespace {

constexpr int NW = kCtaThreads / 32;
constexpr uint32_t kCliqueWideMin = 1024;  // k <= 4 pivots above this run 1,024-thread CTAs

__device__ __forceinline__ uint32_t ilog2p1_c(uint32_t x) { return 32u - __clz(x | 1u); }

// Packed lower-triangular masks: row e holds bits < e in mask_len(e) words
// (ceil(e/32), made odd so that lanes reading rows e, e+1, ... at the same word
// index fall in different shared-memory banks); mask_off(e) = sum of the
// lengths of rows 0 .. e-1.  A c-entry pivot needs mask_off(c) words, about
// half of a c x c bit matrix.
__host__ __device__ __forceinline__ uint32_t mask_len(uint32_t e) { return ((e + 31) >> 5) | 1u; }
// 32-bit arithmetic: exact below kCliqueMaxPivot = 2^18 entries, the largest
// pivot a clique count accepts (mask_off(2^18 - 1) = 1,073,987,583 < 2^32).
__host__ __device__ __forceinline__ uint32_t mask_off(uint32_t e) {
  if (e == 0) return 0;
  const uint32_t A = (e - 1) >> 5, r = (e - 1) & 31;
  // row 0: 1 word; rows 32a+1 .. 32a+32: (a+1)|1 words each.
  return 1 + 32 * (A * (A + 1) / 2 + A / 2) + r * ((A + 1) | 1);
}

// Tuple output: the k ids of one clique (pivot row, then pivot entries in
// descending order) at the position the cursor a.out[0] hands out, if it is
// below the capacity.
__device__ __forceinline__ void put_tuple(const CliqueArgs& a, unsigned long long pos, uint32_t row, uint32_t x1,
                                          uint32_t x2, uint32_t x3) {
  if (pos >= a.capacity) return;
  uint32_t* o = a.tuples + pos * a.k;
  o[0] = row;
  o[1] = x1;
  o[2] = x2;
  if (a.k == 4) o[3] = x3;
}

// ---- light tier: |A_i| <= 32, one warp per pivot, one-word masks ----
// LIST: write the k = 3 or 4 cliques as tuples instead of counting them.
template <bool LIST>
__global__ void __launch_bounds__(kCtaThreads) k_clique_light(CliqueArgs a, uint32_t pos_begin,
                                                              uint32_t pos_end, uint32_t* counter) {
  __shared__ uint32_t s_list[NW][32];
  __shared__ uint32_t s_mask[NW][32];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t* list = s_list[warp];
  uint32_t* mask = s_mask[warp];
  const int top = (int)a.k - 3;  // DFS depth at which a popcount finishes the count
  unsigned long long acc = 0;
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(counter, 8u);
    base = __shfl_sync(FULL, base, 0) + pos_begin;
    if (base >= pos_end) break;
    const uint32_t end = min(pos_end, base + 8u);
    for (uint32_t p = base; p < end; p++) {
      const uint32_t row = a.order[p];
      const RowView A = load_view(a.desc, a.arena, row);
      const uint32_t c = A.card;
      const unsigned long long acc_before = acc;
      warp_decode(A, list, lane);
      mask[lane] = 0;
      __syncwarp();
      // phase 1: every (e, t < e) pair, one per lane
      const uint32_t pairs = c * (c - 1) / 2;
      uint32_t e = 1, t = lane;
      while (t >= e) { t -= e; e++; }
      for (uint32_t q = lane; q < pairs; q += 32) {
        const uint32_t j = list[e], x = list[t];
        bool hit;
        if (j < a.core_k) {
          hit = (__ldg(a.core + core_row_offset(j) + (x >> 6)) >> (x & 63)) & 1ull;
        } else {
          const RowView B = load_view(a.desc, a.arena, j);
          hit = row_contains(B, x);
        }
        if (hit) atomicOr(&mask[e], 1u << t);
        t += 32;
        while (t >= e && e < c) { t -= e; e++; }
      }
      __syncwarp();
      if (LIST) {
        // Lane e lists the cliques whose two largest members are i and A_i[e]:
        // (i, A_i[e], A_i[t]) for t in M[e], or (i, A_i[e], A_i[t], A_i[u]) for
        // u in M[e] & M[t]; one cursor atomic per warp and pivot.
        const uint32_t m0 = lane < c ? mask[lane] : 0u;
        uint32_t n = 0;
        if (top == 0) {
          n = __popc(m0);
        } else {
          for (uint32_t m = m0; m; m &= m - 1) n += __popc(m0 & mask[__ffs(m) - 1]);
        }
        const uint32_t ex = warp_exclusive_scan(n, lane);
        unsigned long long base = 0;
        if (lane == 31 && ex + n) base = atomicAdd(a.out, (unsigned long long)(ex + n));
        base = __shfl_sync(FULL, base, 31) + ex;
        for (uint32_t m = base < a.capacity ? m0 : 0u; m; m &= m - 1) {  // past the capacity: counted only
          const uint32_t tt = __ffs(m) - 1;
          if (top == 0) {
            put_tuple(a, base++, row, list[lane], list[tt], 0u);
          } else {
            for (uint32_t r = m0 & mask[tt]; r; r &= r - 1) put_tuple(a, base++, row, list[lane], list[tt], list[__ffs(r) - 1]);
          }
        }
        __syncwarp();
        continue;
      }
      // phase 2: lane e counts the cliques whose two largest members are i and A_i[e]
      if (lane < c) {
        const uint32_t m0 = mask[lane];
        if (top == 0) {
          acc += __popc(m0);
        } else if (top == 1) {
          uint32_t m = m0;
          while (m) {
            const uint32_t tt = __ffs(m) - 1;
            m &= m - 1;
            acc += __popc(m0 & mask[tt]);
          }
        } else {
          uint32_t S[kCliqueMaxK], R[kCliqueMaxK];
          S[0] = R[0] = m0;
          int d = 0;
          while (d >= 0) {
            if (d == top) {
              acc += __popc(S[d]);
              d--;
              continue;
            }
            if (!R[d]) {
              d--;
              continue;
            }
            const uint32_t tt = __ffs(R[d]) - 1;
            R[d] &= R[d] - 1;
            const uint32_t nx = S[d] & mask[tt];
            if ((uint32_t)__popc(nx) >= (uint32_t)(top - d)) {  // enough candidates left
              S[d + 1] = R[d + 1] = nx;
              d++;
            }
          }
        }
      }
      if (a.graph_rows) {  // batch: this pivot's cliques go to its graph
        const unsigned long long pc = warp_sum_u64(acc - acc_before);
        acc = acc_before;
        if (lane == 0 && pc) atomicAdd(&a.out[graph_of(a.graph_rows, a.num_graphs, row)], pc);
      }
      __syncwarp();
    }
  }
  acc = warp_sum_u64(acc);
  if (!LIST && lane == 0 && acc) atomicAdd(a.out, acc);
}

// ---- CTA tiers: one pivot per CTA; masks in shared memory or a global slot ----
// Per CTA working set (words): list[cmax] | masks[mask_off(cmax)] | stacks[NW][2 * (k-2) * W]
// (stacks only for k >= 5); W = mask_len(cmax) is the DFS stack row length.
// NT threads per CTA: 256, or 1,024 for the largest pivots at k <= 4, whose
// masks leave room for one CTA per SM (more warps to hide latency).
template <bool GLOBAL, int NT, bool LIST>
__global__ void __launch_bounds__(NT, NT == 1024 ? 1 : (GLOBAL ? 2 : 8)) k_clique_cta(CliqueArgs a, uint32_t pos_begin, uint32_t pos_end,
                                                            uint32_t* counter, uint32_t cmax, uint32_t W,
                                                            uint32_t* gscratch, uint64_t slot_words) {
  extern __shared__ __align__(16) uint32_t dyn[];
  __shared__ uint32_t s_unit;
  constexpr int NW = NT / 32;
  __shared__ uint32_t s_scan[NT];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t* base = GLOBAL ? gscratch + (uint64_t)blockIdx.x * slot_words : dyn;
  uint32_t* list = base;
  uint32_t* masks = base + cmax;
  const uint32_t stack_words = 2u * (a.k - 2) * W;
  uint32_t* stack = masks + mask_off(cmax) + (uint64_t)warp * stack_words;
  const int top = (int)a.k - 3;
  unsigned long long acc = 0;
  for (;;) {
    if (threadIdx.x == 0) s_unit = atomicAdd(counter, 1u) + pos_begin;
    __syncthreads();
    const uint32_t unit = s_unit;
    if (unit >= pos_end) break;
    const uint32_t row = a.order[unit];
    const RowView A = load_view(a.desc, a.arena, row);
    const uint32_t c = A.card;
    const unsigned long long acc_before = acc;
    cta_decode<NT>(A, list, s_scan);
    for (uint64_t x = threadIdx.x; x < mask_off(c); x += NT) masks[x] = 0;
    __syncthreads();
    // phase 1: warp per e builds M[e]
    for (uint32_t e = 1 + warp; e < c; e += NW) {
      const uint32_t j = list[e];
      uint32_t* Me = masks + mask_off(e);
      if (j < a.core_k) {  // core row j = row(j) ∩ [0, j): one word per probe, L2-resident
        const unsigned long long* row = a.core + core_row_offset(j);
        for (uint32_t b = 0; b < e; b += 32) {
          const uint32_t t = b + lane;
          const bool hit = t < e && ((__ldg(row + (list[t] >> 6)) >> (list[t] & 63)) & 1ull);
          const uint32_t word = __ballot_sync(FULL, hit);
          if (lane == 0) Me[b >> 5] = word;
        }
        continue;
      }
      const RowView B = load_view(a.desc, a.arena, j);
      if (B.card == 0) continue;
      bool stream = false;
      if (B.type == TY_UINT) stream = (uint64_t)B.card * ilog2p1_c(e) < (uint64_t)e * ilog2p1_c(B.card) * 4u;
      else if (B.type == TY_PSHORT) stream = (uint64_t)B.card * ilog2p1_c(e) < (uint64_t)e * (B.aux + ilog2p1_c(B.card)) * 4u;
      if (!stream) {
        for (uint32_t b = 0; b < e; b += 32) {
          const uint32_t t = b + lane;
          const bool hit = t < e && row_contains(B, list[t]);
          const uint32_t word = __ballot_sync(FULL, hit);
          if (lane == 0) Me[b >> 5] = word;
        }
      } else {
        warp_for_each(B, j, lane, [&](uint32_t y) {
          const uint32_t t = lower_bound_u32(list, 0, e, y);
          if (t < e && list[t] == y) atomicOr(&Me[t >> 5], 1u << (t & 31));
        });
      }
    }
    __syncthreads();
    // phase 2: warp per e
    for (uint32_t e = 1 + warp; e < c; e += NW) {
      const uint32_t* Me = masks + mask_off(e);
      const uint32_t we = (e + 31) >> 5;  // words that can hold bits < e
      if (LIST) {
        // Lane t of each word of M[e] lists (i, A_i[e], A_i[t]) or, for k = 4,
        // (i, A_i[e], A_i[t], A_i[u]) for u in M[e] & M[t], one cursor atomic per word of M[e].
        // Tuples past the capacity are counted, not enumerated.
        const uint32_t je = list[e];
        for (uint32_t w = 0; w < we; w++) {
          const uint32_t bits = Me[w];
          if (top == 0) {  // one cursor atomic per word of M[e]
            if (!bits) continue;
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(a.out, (unsigned long long)__popc(bits));
            base = __shfl_sync(FULL, base, 0);
            if ((bits >> lane) & 1u)
              put_tuple(a, base + __popc(bits & ((1u << lane) - 1u)), row, je, list[32 * w + lane], 0u);
            continue;
          }
          if (!bits) continue;  // k = 4: lane t of the word counts M[e] & M[t], one cursor atomic per word
          const bool has = (bits >> lane) & 1u;
          const uint32_t t = 32 * w + lane;
          const uint32_t* Mt = masks + mask_off(t);
          const uint32_t lt = (t + 31) >> 5;
          uint32_t n = 0;
          if (has)
            for (uint32_t x = 0; x < lt; x++) n += __popc(Me[x] & Mt[x]);
          const uint32_t ex = warp_exclusive_scan(n, lane);
          const uint32_t sum = __shfl_sync(FULL, ex + n, 31);
          unsigned long long pos = 0;
          if (lane == 0 && sum) pos = atomicAdd(a.out, (unsigned long long)sum);
          pos = __shfl_sync(FULL, pos, 0) + ex;
          if (has)
            for (uint32_t x = 0; x < lt && pos < a.capacity; x++)
              for (uint32_t r = Me[x] & Mt[x]; r; r &= r - 1) put_tuple(a, pos++, row, je, list[t], list[32 * x + __ffs(r) - 1]);
        }
        continue;
      }
      if (top == 0) {
        for (uint32_t w = lane; w < we; w += 32) acc += __popc(Me[w]);
      } else if (top == 1) {
        // k = 4: sum over t in M[e] of popc(M[e] & M[t]); M[t] has bits below t only,
        // in its ceil(t/32) words.
        if (GLOBAL && we > 8) {
          // Long rows in global memory: the warp walks the set bits t together and
          // lanes take consecutive words of the two rows (coalesced reads).
          for (uint32_t w0 = 0; w0 < we; w0++) {
            uint32_t bits = Me[w0];
            while (bits) {
              const uint32_t t = 32 * w0 + (__ffs(bits) - 1);
              bits &= bits - 1;
              const uint32_t* Mt = masks + mask_off(t);
              for (uint32_t x = lane; x < ((t + 31) >> 5); x += 32) acc += __popc(Me[x] & Mt[x]);
            }
          }
        } else {
          // Each lane takes one t of a word of M[e]; odd row lengths keep the
          // lanes' rows in different shared-memory banks.
          for (uint32_t w = 0; w < we; w++) {
            const uint32_t bits = Me[w];
            if (!((bits >> lane) & 1u)) continue;
            const uint32_t t = 32 * w + lane;
            // mask_off(t) from the word's first row: rows 32w+1 .. 32w+31 are (w+1)|1
            // words long, row 32w is w|1 words long.
            const uint32_t first = mask_off(32 * w + 1);
            const uint32_t* Mt = masks + (lane ? first + (lane - 1) * ((w + 1) | 1u) : first - (w | 1u));
            for (uint32_t x = 0; x < ((t + 31) >> 5); x++) acc += __popc(Me[x] & Mt[x]);
          }
        }
      } else {
        // Warp-cooperative depth-first search; S[d], R[d] live in the warp's stack.
        uint32_t* S = stack;
        uint32_t* R = stack + (a.k - 2) * W;
        for (uint32_t w = lane; w < W; w += 32) S[w] = R[w] = (w < we) ? Me[w] : 0u;
        __syncwarp();
        int d = 0;
        while (d >= 0) {
          uint32_t* Sd = S + (uint64_t)d * W;
          uint32_t* Rd = R + (uint64_t)d * W;
          if (d == top) {
            for (uint32_t w = lane; w < W; w += 32) acc += __popc(Sd[w]);  // summed over lanes at the end
            d--;
            continue;
          }
          // lowest remaining candidate t in Rd
          uint32_t t = 0xffffffffu;
          for (uint32_t w0 = 0; w0 < W && t == 0xffffffffu; w0 += 32) {
            const uint32_t w = w0 + lane;
            const uint32_t v = w < W ? Rd[w] : 0u;
            const uint32_t nz = __ballot_sync(FULL, v != 0);
            if (nz) {
              const uint32_t src = __ffs(nz) - 1;
              const uint32_t vw = __shfl_sync(FULL, v, src);
              t = 32 * (w0 + src) + (__ffs(vw) - 1);
            }
          }
          if (t == 0xffffffffu) {
            d--;
            continue;
          }
          __syncwarp();
          if (lane == 0) Rd[t >> 5] &= ~(1u << (t & 31));
          const uint32_t* Mt = masks + mask_off(t);
          const uint32_t lt = (t + 31) >> 5;  // words of M[t]; the rest are 0
          uint32_t* Sn = S + (uint64_t)(d + 1) * W;
          uint32_t* Rn = R + (uint64_t)(d + 1) * W;
          uint32_t cnt = 0;
          for (uint32_t w = lane; w < W; w += 32) {
            const uint32_t v = w < lt ? Sd[w] & Mt[w] : 0u;
            Sn[w] = v;
            Rn[w] = v;
            cnt += __popc(v);
          }
          cnt = warp_sum_u32(cnt);
          __syncwarp();
          if (cnt >= (uint32_t)(top - d)) d++;
        }
      }
    }
    if (a.graph_rows) {  // batch: each warp's share of this pivot goes to its graph
      const unsigned long long pc = warp_sum_u64(acc - acc_before);
      acc = acc_before;
      if (lane == 0 && pc) atomicAdd(&a.out[graph_of(a.graph_rows, a.num_graphs, row)], pc);
    }
    __syncthreads();
  }
  acc = warp_sum_u64(acc);
  if (!LIST && lane == 0 && acc) atomicAdd(a.out, acc);
}

}  // namespace

uint64_t clique_slot_words(uint32_t cmax, uint32_t k) {
  const uint64_t W = mask_len(cmax);
  // DFS stacks (k >= 5) are sized for the 256-thread CTAs that run those k.
  return (uint64_t)cmax + (uint64_t)mask_off(cmax) + (k >= 5 ? (uint64_t)NW * 2 * (k - 2) * W : 0);
}

uint32_t clique_smem_cap(uint32_t k, int device) {
  static std::atomic<int> optin[64];
  int o = (device >= 0 && device < 64) ? optin[device].load() : 0;
  if (o <= 0) {
    cudaDeviceGetAttribute(&o, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    if (device >= 0 && device < 64) optin[device].store(o);
  }
  // Leave room for the kernel's static shared memory (s_unit, s_scan: 4,112 bytes
  // in the 1,024-thread variant).
  const uint64_t budget = o > 4608 ? (uint64_t)o - 4608 : 0;
  uint32_t lo = 32, hi = kCliqueSmemMax;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) / 2;
    if (clique_slot_words(mid, k) * 4 <= budget) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// SMs x resident CTAs of the shared-memory clique kernel with `bytes` of
// dynamic shared memory; looked up once per (device, size), so that launches
// captured into a CUDA graph after a direct run make no occupancy query.
template <int NT, bool LIST>
static int resident_ctas(int dev, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, size_t>, int> cache;
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find({dev, bytes});
  if (it != cache.end()) return it->second;
  int sms = 0, per = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_clique_cta<false, NT, LIST>, NT, bytes);
  const int g = std::max(sms, 1) * std::max(per, 1);
  cache[{dev, bytes}] = g;
  return g;
}

// Shared-memory launch with NT threads per CTA.
template <int NT, bool LIST>
static cudaError_t launch_shared(const CliqueArgs& a, uint32_t pos_begin, uint32_t pos_end, uint32_t* counter,
                                 uint32_t cmax, uint32_t W, uint64_t slot, int grid, cudaStream_t st) {
  const size_t bytes = slot * 4;
  // Raise the kernel's dynamic shared-memory limit only when a launch needs more
  // than any before it (so replays of captured launches never call this).
  static std::atomic<int> set_bytes[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if ((int)bytes > set_bytes[dev].load()) {
    cudaError_t e = cudaFuncSetAttribute(k_clique_cta<false, NT, LIST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)bytes);
    if (e != cudaSuccess) return e;
    int prev = set_bytes[dev].load();
    while ((int)bytes > prev && !set_bytes[dev].compare_exchange_weak(prev, (int)bytes)) {
    }
  }
  if (grid <= 0)  // fill the GPU: SMs x resident CTAs at this shared-memory size, at most one per pivot
    grid = (int)std::min<uint64_t>(pos_end - pos_begin, (uint64_t)resident_ctas<NT, LIST>(dev, bytes));
  k_clique_cta<false, NT, LIST><<<grid, NT, bytes, st>>>(a, pos_begin, pos_end, counter, cmax, W, nullptr, slot);
  return cudaGetLastError();
}

cudaError_t launch_clique_light(const CliqueArgs& a, uint32_t pos_begin, uint32_t pos_end, uint32_t* counter,
                                int grid, cudaStream_t st, bool list) {
  if (pos_end <= pos_begin) return cudaSuccess;
  if (list) k_clique_light<true><<<grid, kCtaThreads, 0, st>>>(a, pos_begin, pos_end, counter);
  else k_clique_light<false><<<grid, kCtaThreads, 0, st>>>(a, pos_begin, pos_end, counter);
  return cudaGetLastError();
}

template <bool LIST>
static cudaError_t launch_cta(const CliqueArgs& a, uint32_t pos_begin, uint32_t pos_end, uint32_t* counter,
                              uint32_t cmax, uint32_t* gscratch, int grid, cudaStream_t st) {
  const uint32_t W = mask_len(cmax);
  const uint64_t slot = clique_slot_words(cmax, a.k);
  const bool wide = a.k <= 4 && cmax > kCliqueWideMin;
  if (gscratch) {
    if (wide) {
      // One 1,024-thread CTA per SM in place of two 256-thread ones.
      int sms = 0, dev = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      grid = std::max(1, std::min(grid, sms));
      k_clique_cta<true, 1024, LIST><<<grid, 1024, 0, st>>>(a, pos_begin, pos_end, counter, cmax, W, gscratch,
                                                            slot);
    } else {
      k_clique_cta<true, kCtaThreads, LIST><<<grid, kCtaThreads, 0, st>>>(a, pos_begin, pos_end, counter, cmax, W,
                                                                          gscratch, slot);
    }
    return cudaGetLastError();
  }
  return wide ? launch_shared<1024, LIST>(a, pos_begin, pos_end, counter, cmax, W, slot, grid, st)
              : launch_shared<kCtaThreads, LIST>(a, pos_begin, pos_end, counter, cmax, W, slot, grid, st);
}

cudaError_t launch_clique_cta(const CliqueArgs& a, uint32_t pos_begin, uint32_t pos_end, uint32_t* counter,
                              uint32_t cmax, uint32_t* gscratch, int grid, cudaStream_t st, bool list) {
  if (pos_end <= pos_begin) return cudaSuccess;
  return list ? launch_cta<true>(a, pos_begin, pos_end, counter, cmax, gscratch, grid, st)
              : launch_cta<false>(a, pos_begin, pos_end, counter, cmax, gscratch, grid, st);
}

}  // namespace eh
