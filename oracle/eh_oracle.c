/*
 * eh_oracle.c — CPU restatement of EmptyHeaded's set-intersection pattern
 * engine (chrisaberger/SIMDGraphProcessing), used as the parity oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference leg of bench.py load this library, and only as the
 * checker or the timed CPU baseline.  The product (libeh_gb300.so) never calls
 * it.
 *
 * Parity is pinned: tests compare these functions with the reference's own
 * golden counts on test/data/facebook.bin (the test/ gtests) when the reference tree
 * is present, and with committed fixtures produced by the reference binaries
 * compiled from unmodified sources (oracle/build_ref.sh, tests/golden/).
 *
 * Every function cites the reference code it restates (paths relative to the
 * reference project).  Plain C99 + OpenMP, scalar only, so that it builds and
 * gives the same results on x86-64 and aarch64 hosts.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

enum { T_BITSET = 0, T_PSHORT = 1, T_UINTEGER = 2, L_HYBRID = 5, L_HYBRID3 = 16 };
enum { SEL_ALL = 0, SEL_LOWER = 1 };

/* Set<T> view: src/set/Set.hpp:14-21 (data, cardinality, number_of_bytes, type). */
typedef struct {
  const uint8_t* data;
  uint64_t card;
  uint64_t nbytes;
  int type;
} oset;

/* SparseMatrix<T,R> (src/SparseMatrix.hpp:11-131), restricted to what the apps read. */
typedef struct {
  uint64_t n;
  int layout;
  uint64_t cardinality;       /* selected edges */
  uint64_t total_bytes;       /* row_total_bytes_used */
  uint32_t* row_lengths;      /* row_lengths[n] */
  uint64_t* row_offsets;      /* byte offset of each flattened row; [n+1] */
  uint8_t* row_data;          /* all flattened rows back to back */
  uint64_t num_uint, num_pshort, num_bitset;
} omatrix;

/* The reference's flattened rows put u32 elements at any byte offset (the
 * hybrid tag and byte-count headers shift them, hybrid.hpp:132-201): uint rows
 * are read and written through this type, whose loads are defined at any
 * alignment. */
typedef uint32_t u32u __attribute__((aligned(1), may_alias));

static inline uint64_t rd64(const uint8_t* p) { uint64_t v; memcpy(&v, p, 8); return v; }
static inline uint32_t rd32(const uint8_t* p) { uint32_t v; memcpy(&v, p, 4); return v; }
static inline uint16_t rd16(const uint8_t* p) { uint16_t v; memcpy(&v, p, 2); return v; }
static inline void wr64(uint8_t* p, uint64_t v) { memcpy(p, &v, 8); }
static inline void wr32(uint8_t* p, uint32_t v) { memcpy(p, &v, 4); }
static inline void wr16(uint8_t* p, uint16_t v) { memcpy(p, &v, 2); }
static inline int popc64(uint64_t x) { return __builtin_popcountll(x); }

/* ------------------------------------------------------------------------ */
/* Layout encoders: exactly the bytes T::build_flattened writes.            */
/* ------------------------------------------------------------------------ */

/* uinteger::build / build_flattened (src/set/layouts/uinteger.hpp:49-59). */
static uint64_t enc_uint(uint8_t* r, const uint32_t* a, uint64_t n) {
  if (r) memcpy(r, a, n * 4);
  return n * 4;
}

/* bitset::build (src/set/layouts/bitset.hpp:65-96): [u64 first/64][words first/64..last/64]. */
static uint64_t enc_bitset_body(uint8_t* r, const uint32_t* a, uint64_t n) {
  if (n == 0) return 0;
  uint64_t off = a[0] >> 6, words = (a[n - 1] >> 6) - off + 1;
  if (r) {
    wr64(r, off);
    memset(r + 8, 0, words * 8);
    for (uint64_t i = 0; i < n; i++) {
      uint8_t* w = r + 8 + ((a[i] >> 6) - off) * 8;
      wr64(w, rd64(w) | (1ULL << (a[i] & 63)));
    }
  }
  return words * 8 + 8;
}
/* bitset::build_flattened (bitset.hpp:99-109): leading u32 byte count, nothing if empty. */
static uint64_t enc_bitset(uint8_t* r, const uint32_t* a, uint64_t n) {
  if (n == 0) return 0;
  uint64_t b = enc_bitset_body(r ? r + 4 : 0, a, n);
  if (r) wr32(r, (uint32_t)b);
  return b + 4;
}

/* pshort::build (src/set/layouts/pshort.hpp:46-78): partitions [hi][count-1][lo...]. */
static uint64_t enc_pshort_body(uint8_t* r, const uint32_t* a, uint64_t n) {
  if (n == 0) return 0;
  uint64_t cnt = 0, size_pos = 1, plen = 0;
  uint16_t high = 0;
  for (uint64_t p = 0; p < n; p++) {
    uint16_t hi = (uint16_t)(a[p] >> 16), lo = (uint16_t)(a[p] & 0xFFFF);
    if (hi == high && p != 0) {
      plen++;
      if (r) wr16(r + 2 * cnt, lo);
      cnt++;
    } else {
      if (r) {
        wr16(r + 2 * cnt, hi);
        wr16(r + 2 * (cnt + 1), 0);
        wr16(r + 2 * (cnt + 2), lo);
        wr16(r + 2 * size_pos, (uint16_t)plen);
      }
      cnt += 3;
      plen = 0;
      size_pos = cnt - 2;
      high = hi;
    }
  }
  if (r) wr16(r + 2 * size_pos, (uint16_t)plen);
  return cnt * 2;
}
/* pshort::build_flattened (pshort.hpp:81-91). */
static uint64_t enc_pshort(uint8_t* r, const uint32_t* a, uint64_t n) {
  if (n == 0) return 0;
  uint64_t b = enc_pshort_body(r ? r + 4 : 0, a, n);
  if (r) wr32(r, (uint32_t)b);
  return b + 4;
}

/* hybrid::get_type (src/set/layouts/hybrid.hpp:73-100) with bitset_req = 1/256 and
 * bitset_length = 0 (src/common.hpp:71-73): the optimizer the reference runs. */
static int hybrid_type(const uint32_t* a, uint64_t n) {
  if (n > 1) {
    uint32_t range = a[n - 1] - a[0];
    if (range > 0) {
      double density = (double)n / range;
      if (density > (1.0 / 256.0) && n > 0) return T_BITSET;
      return T_UINTEGER;
    }
  }
  return T_UINTEGER;
}
/* Optional three-tier rule: hybrid::compute_type (hybrid.hpp:55-63) applied to the
 * density get_type computes (len / (last - first)). */
static int hybrid3_type(const uint32_t* a, uint64_t n) {
  if (n > 1) {
    uint32_t range = a[n - 1] - a[0];
    if (range > 0) {
      double density = (double)n / range;
      if (density > 1.0 / 32.0) return T_BITSET;
      if (density > 1.0 / 256.0) return T_PSHORT;
    }
  }
  return T_UINTEGER;
}

/* hybrid::build_flattened (hybrid.hpp:132-166): u64 type tag then the inner layout. */
static uint64_t enc_row(uint8_t* r, const uint32_t* a, uint64_t n, int layout, int* type_out) {
  int t;
  switch (layout) {
    case T_UINTEGER: *type_out = T_UINTEGER; return enc_uint(r, a, n);
    case T_BITSET: *type_out = T_BITSET; return enc_bitset(r, a, n);
    case T_PSHORT: *type_out = T_PSHORT; return enc_pshort(r, a, n);
    default:
      t = (layout == L_HYBRID3) ? hybrid3_type(a, n) : hybrid_type(a, n);
      *type_out = t;
      if (r) wr64(r, (uint64_t)t);
      if (t == T_BITSET) return 8 + enc_bitset(r ? r + 8 : 0, a, n);
      if (t == T_PSHORT) return 8 + enc_pshort(r ? r + 8 : 0, a, n);
      return 8 + enc_uint(r ? r + 8 : 0, a, n);
  }
}

/* Set<T>::from_flattened (Set.hpp:172-176) via T::get_flattened_data
 * (uinteger.hpp:61-64, bitset.hpp:111-118, pshort.hpp:93-100, hybrid.hpp:168-201). */
static oset view_inner(const uint8_t* p, uint64_t card, int t) {
  oset s;
  s.card = card;
  s.type = t;
  if (t == T_UINTEGER) {
    s.data = p;
    s.nbytes = card * 4;
  } else if (card > 0) {
    s.data = p + 4;
    s.nbytes = rd32(p);
  } else {
    s.data = p;
    s.nbytes = 0;
  }
  return s;
}
static oset get_row(const omatrix* m, uint64_t i) {
  const uint8_t* p = m->row_data + m->row_offsets[i];
  uint64_t card = m->row_lengths[i];
  if (m->layout == L_HYBRID || m->layout == L_HYBRID3) {
    int t = (int)rd64(p);
    return view_inner(p + 8, card, t);
  }
  return view_inner(p, card, m->layout);
}

/* ------------------------------------------------------------------------ */
/* Intersections (src/set/ops/intersection.hpp).  Each returns |A ∩ B| and,  */
/* when out != NULL (WRITE_VECTOR == 1), writes C in its result layout.      */
/* ------------------------------------------------------------------------ */

/* Merge of two sorted u32 arrays: ops::scalar (intersection.hpp:46-79); also the
 * result of set_intersect_standard's 4x4 block compare (:696-771). */
static uint64_t merge_u32(const u32u* a, uint64_t la, const u32u* b, uint64_t lb, u32u* out) {
  uint64_t i = 0, j = 0, c = 0;
  while (i < la && j < lb) {
    if (a[i] < b[j]) i++;
    else if (a[i] > b[j]) j++;
    else {
      if (out) out[c] = a[i];
      c++; i++; j++;
    }
  }
  return c;
}
/* set_intersect_galloping (intersection.hpp:393-584): each rare element is located
 * in freq by an exponential then binary search from the previous position. */
static uint64_t gallop_u32(const u32u* rare, uint64_t lr, const u32u* freq, uint64_t lf, u32u* out) {
  uint64_t lo = 0, c = 0;
  for (uint64_t i = 0; i < lr && lo < lf; i++) {
    uint32_t x = rare[i];
    uint64_t step = 1, hi = lo;
    while (hi < lf && freq[hi] < x) { lo = hi + 1; hi = lo + step; step <<= 1; }
    if (hi > lf) hi = lf;
    while (lo < hi) {  /* first position >= x in [lo, hi) */
      uint64_t mid = lo + (hi - lo) / 2;
      if (freq[mid] < x) lo = mid + 1; else hi = mid;
    }
    if (lo < lf && freq[lo] == x) {
      if (out) out[c] = x;
      c++;
      lo++;
    }
  }
  return c;
}
/* set_intersect(uint, uint) (intersection.hpp:1325-1336): galloping when the size
 * ratio exceeds 32, else the standard merge; rare = the smaller set. */
static uint64_t ix_uu(oset A, oset B, uint8_t* out) {
  const oset* rare = (A.card > B.card) ? &B : &A;
  const oset* freq = (A.card > B.card) ? &A : &B;
  uint64_t mn = rare->card ? rare->card : 1;
  if (freq->card / mn > 32)
    return gallop_u32((const u32u*)rare->data, rare->card, (const u32u*)freq->data, freq->card, (u32u*)out);
  return merge_u32((const u32u*)rare->data, rare->card, (const u32u*)freq->data, freq->card, (u32u*)out);
}
/* set_intersect(uint, bitset) (intersection.hpp:1023-1058): probe each uint element,
 * stop at the first element past the bitset's last word. */
static uint64_t ix_ub(oset A, oset B, uint8_t* out) {
  uint64_t sb = B.nbytes > 0 ? (B.nbytes - 8) / 8 : 0;
  uint64_t start = B.nbytes > 0 ? rd64(B.data) : 0;
  const u32u* a = (const u32u*)A.data;
  u32u* o = (u32u*)out;
  uint64_t c = 0;
  for (uint64_t i = 0; i < A.card; i++) {
    uint64_t w = a[i] >> 6;
    if (w < sb + start && w >= start && ((rd64(B.data + 8 + (w - start) * 8) >> (a[i] & 63)) & 1)) {
      if (o) o[c] = a[i];
      c++;
    } else if (w >= sb + start) {
      break;
    }
  }
  return c;
}
/* set_intersect(bitset, bitset) (intersection.hpp:880-955): AND over the overlap of
 * the two word ranges; C = [u64 start word][overlap words]. */
static uint64_t ix_bb(oset A, oset B, uint8_t* out, uint64_t* out_nbytes) {
  uint64_t c = 0;
  if (out_nbytes) *out_nbytes = 0;
  if (A.nbytes > 0 && B.nbytes > 0) {
    uint64_t ai = rd64(A.data), bi = rd64(B.data);
    uint64_t sa = (A.nbytes - 8) / 8, sb = (B.nbytes - 8) / 8;
    uint64_t start = ai > bi ? ai : bi;
    uint64_t end = (ai + sa > bi + sb) ? bi + sb : ai + sa;
    uint64_t total = start > end ? 0 : end - start;
    if (out) wr64(out, start);
    for (uint64_t k = 0; k < total; k++) {
      uint64_t r = rd64(A.data + 8 + (start - ai + k) * 8) & rd64(B.data + 8 + (start - bi + k) * 8);
      if (out) wr64(out + 8 + k * 8, r);
      c += popc64(r);
    }
    if (out_nbytes) *out_nbytes = total * 8 + 8;
  }
  return c;
}
/* simd_intersect_vector16 (intersection.hpp:773-828): |A ∩ B| of two sorted u16 arrays. */
static uint64_t merge_u16(const uint8_t* a, uint64_t la, const uint8_t* b, uint64_t lb, uint8_t* out) {
  uint64_t i = 0, j = 0, c = 0;
  while (i < la && j < lb) {
    uint16_t x = rd16(a + 2 * i), y = rd16(b + 2 * j);
    if (x < y) i++;
    else if (x > y) j++;
    else {
      if (out) wr16(out + 2 * c, x);
      c++; i++; j++;
    }
  }
  return c;
}
/* set_intersect(pshort, pshort) (intersection.hpp:829-878): merge on partition
 * prefixes, u16 intersection inside equal partitions.  The per-partition count is
 * held in a uint16_t there (partition_size), so it is taken modulo 65536 here too. */
static uint64_t ix_pp(oset A, oset B, uint8_t* out, uint64_t* out_nbytes) {
  uint64_t sa = A.nbytes / 2, sb = B.nbytes / 2, ia = 0, ib = 0, counter = 0, count = 0;
  while (ia < sa && ib < sb) {
    uint16_t ha = rd16(A.data + 2 * ia), hb = rd16(B.data + 2 * ib);
    if (ha < hb) ia += (uint64_t)rd16(A.data + 2 * (ia + 1)) + 3;
    else if (hb < ha) ib += (uint64_t)rd16(B.data + 2 * (ib + 1)) + 3;
    else {
      uint64_t na = (uint64_t)rd16(A.data + 2 * (ia + 1)) + 1, nb = (uint64_t)rd16(B.data + 2 * (ib + 1)) + 1;
      uint16_t psize = (uint16_t)merge_u16(A.data + 2 * (ia + 2), na, B.data + 2 * (ib + 2), nb,
                                           out ? out + 2 * (counter + 2) : 0);
      if (psize > 0) {
        if (out) {
          wr16(out + 2 * counter, ha);
          wr16(out + 2 * (counter + 1), (uint16_t)(psize - 1));
        }
        counter += 2 + psize;
      }
      count += psize;
      ia += na + 2;
      ib += nb + 2;
    }
  }
  if (out_nbytes) *out_nbytes = counter * 2;
  return count;
}
/* set_intersect(pshort, bitset) (intersection.hpp:956-1017): probe each pshort element
 * of partitions that overlap the bitset's word range.  Result layout pshort. */
static uint64_t ix_pb(oset A, oset B, uint8_t* out, uint64_t* out_nbytes) {
  uint64_t start = B.nbytes > 0 ? rd64(B.data) : 0;
  uint64_t sb = B.nbytes > 0 ? (B.nbytes - 8) / 8 : 0;
  uint64_t sa = A.nbytes / 2, count = 0, wpos = 0;
  for (uint64_t i = 0; i < sa;) {
    uint32_t prefix = (uint32_t)rd16(A.data + 2 * i) << 16;
    uint64_t size = rd16(A.data + 2 * (i + 1));
    i += 2;
    uint64_t part_end = i + size, pidx = prefix >> 6, pc = 0, hdr = wpos;
    if (pidx < sb + start && pidx + 1024 >= start) {
      wpos += 2;
      for (; i <= part_end; i++) {
        uint32_t cur = prefix | rd16(A.data + 2 * i);
        uint64_t w = cur >> 6;
        if (w < sb + start && w >= start && ((rd64(B.data + 8 + (w - start) * 8) >> (cur & 63)) & 1)) {
          if (out) wr16(out + 2 * wpos, (uint16_t)(cur & 0xFFFF));
          wpos++;
          pc++;
          count++;
        }
      }
      if (pc == 0) wpos -= 2;
      else if (out) {
        wr16(out + 2 * hdr, (uint16_t)(prefix >> 16));
        wr16(out + 2 * (hdr + 1), (uint16_t)(pc - 1));
      }
    } else if (pidx >= sb + start) {
      break;
    }
    i = part_end + 1;
  }
  if (out_nbytes) *out_nbytes = wpos * 2;
  return count;
}
/* set_intersect(uint, pshort) (intersection.hpp:1062-1173): partition-aware merge.
 * Result layout uint. */
static uint64_t ix_up(oset A, oset B, uint8_t* out) {
  const u32u* a = (const u32u*)A.data;
  u32u* o = (u32u*)out;
  uint64_t sb = B.nbytes / 2, ai = 0, bi = 0, c = 0;
  while (ai < A.card && bi < sb) {
    uint32_t prefix = (uint32_t)rd16(B.data + 2 * bi) << 16;
    uint64_t nb = (uint64_t)rd16(B.data + 2 * (bi + 1)) + 1;
    uint32_t x = a[ai];
    if (prefix < (x & 0xFFFF0000u)) bi += nb + 2;
    else if (prefix > x) ai++;
    else {
      const uint8_t* lows = B.data + 2 * (bi + 2);
      uint64_t k = 0;
      while (ai < A.card && k < nb && (a[ai] & 0xFFFF0000u) == prefix) {
        uint32_t y = prefix | rd16(lows + 2 * k);
        if (y < a[ai]) k++;
        else if (y > a[ai]) ai++;
        else {
          if (o) o[c] = a[ai];
          c++; ai++; k++;
        }
      }
      while (ai < A.card && (a[ai] & 0xFFFF0000u) == prefix) ai++;
      bi += nb + 2;
    }
  }
  return c;
}

/* set_intersect(hybrid, hybrid) (intersection.hpp:2067-2117) plus the fixed-layout
 * overloads: dispatch on the type pair; C's layout follows the kernel chosen. */
static uint64_t set_intersect(oset A, oset B, uint8_t* out, oset* C) {
  uint64_t c = 0, nb = 0;
  int t = T_UINTEGER;
  if (A.card == 0 || B.card == 0) {
    c = 0; t = A.type; nb = 0;
  } else if (A.type == T_UINTEGER && B.type == T_UINTEGER) {
    c = ix_uu(A, B, out); t = T_UINTEGER; nb = c * 4;
  } else if (A.type == T_UINTEGER && B.type == T_BITSET) {
    c = ix_ub(A, B, out); t = T_UINTEGER; nb = c * 4;
  } else if (A.type == T_BITSET && B.type == T_UINTEGER) {
    c = ix_ub(B, A, out); t = T_UINTEGER; nb = c * 4;
  } else if (A.type == T_BITSET && B.type == T_BITSET) {
    c = ix_bb(A, B, out, &nb); t = T_BITSET;
  } else if (A.type == T_PSHORT && B.type == T_PSHORT) {
    c = ix_pp(A, B, out, &nb); t = T_PSHORT;
  } else if (A.type == T_PSHORT && B.type == T_BITSET) {
    c = ix_pb(A, B, out, &nb); t = T_PSHORT;
  } else if (A.type == T_BITSET && B.type == T_PSHORT) {
    c = ix_pb(B, A, out, &nb); t = T_PSHORT;
  } else if (A.type == T_UINTEGER && B.type == T_PSHORT) {
    c = ix_up(A, B, out); t = T_UINTEGER; nb = c * 4;
  } else if (A.type == T_PSHORT && B.type == T_UINTEGER) {
    c = ix_up(B, A, out); t = T_UINTEGER; nb = c * 4;
  }
  if (C) {
    C->data = out;
    C->card = c;
    C->nbytes = nb;
    C->type = t;
  }
  return c;
}

/* Set<T>::foreach (Set.hpp:100-106) for each layout: uinteger.hpp:67-80,
 * bitset.hpp:148-173, pshort.hpp:134-158.  Fills `dst` with the elements. */
static uint64_t decode(oset S, uint32_t* dst) {
  uint64_t k = 0;
  if (S.type == T_UINTEGER) {
    memcpy(dst, S.data, S.card * 4);
    return S.card;
  }
  if (S.type == T_BITSET) {
    if (S.nbytes == 0) return 0;
    uint64_t words = (S.nbytes - 8) / 8, off = rd64(S.data);
    for (uint64_t w = 0; w < words; w++) {
      uint64_t x = rd64(S.data + 8 + w * 8);
      while (x) {
        dst[k++] = (uint32_t)(64 * (w + off) + __builtin_ctzll(x));
        x &= x - 1;
      }
    }
    return k;
  }
  uint64_t i = 0;
  while (k < S.card) {
    uint32_t prefix = (uint32_t)rd16(S.data + 2 * i) << 16;
    uint64_t size = rd16(S.data + 2 * (i + 1));
    i += 2;
    for (uint64_t e = i; e <= i + size; e++) dst[k++] = prefix | rd16(S.data + 2 * e);
    i += size + 1;
  }
  return k;
}

/* ------------------------------------------------------------------------ */
/* SparseMatrix::build -> from_symmetric_noattribute_graph                  */
/* (src/SparseMatrix.hpp:268-290,406-494) with pack_data (:249-266).        */
/* ------------------------------------------------------------------------ */
void* oracle_build(uint64_t n, const uint64_t* off, const uint32_t* nbr, const uint8_t* mask,
                   int sel, int layout, int nthreads) {
  omatrix* m = (omatrix*)calloc(1, sizeof(omatrix));
  m->n = n;
  m->layout = layout;
  m->row_lengths = (uint32_t*)malloc((n + 1) * 4);
  m->row_offsets = (uint64_t*)malloc((n + 1) * 8);
  uint64_t maxdeg = 0;
  for (uint64_t i = 0; i < n; i++) if (off[i + 1] - off[i] > maxdeg) maxdeg = off[i + 1] - off[i];
  uint64_t* bytes = (uint64_t*)malloc((n + 1) * 8);
  int* types = (int*)malloc((n + 1) * sizeof(int));
  if (nthreads > 0) omp_set_num_threads(nthreads);
  /* pass 1: select and size */
#pragma omp parallel
  {
    uint32_t* sel_buf = (uint32_t*)malloc((maxdeg + 1) * 4);
#pragma omp for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)n; i++) {
      uint64_t k = 0;
      for (uint64_t e = off[i]; e < off[i + 1]; e++) {
        int keep = (sel == SEL_ALL) ? 1 : (sel == SEL_LOWER) ? (nbr[e] < (uint32_t)i) : (mask[e] != 0);
        if (keep) sel_buf[k++] = nbr[e];
      }
      m->row_lengths[i] = (uint32_t)k;
      bytes[i] = enc_row(0, sel_buf, k, layout, &types[i]);
    }
    free(sel_buf);
  }
  m->row_offsets[0] = 0;
  for (uint64_t i = 0; i < n; i++) {
    m->row_offsets[i + 1] = m->row_offsets[i] + bytes[i];
    m->cardinality += m->row_lengths[i];
    if (m->row_lengths[i] > 0 || layout == L_HYBRID || layout == L_HYBRID3 || layout == T_UINTEGER) {
      if (types[i] == T_BITSET) m->num_bitset++;
      else if (types[i] == T_PSHORT) m->num_pshort++;
      else m->num_uint++;
    }
  }
  m->total_bytes = m->row_offsets[n];
  m->row_data = (uint8_t*)malloc(m->total_bytes + 16);
  /* pass 2: encode */
#pragma omp parallel
  {
    uint32_t* sel_buf = (uint32_t*)malloc((maxdeg + 1) * 4);
#pragma omp for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)n; i++) {
      uint64_t k = 0;
      for (uint64_t e = off[i]; e < off[i + 1]; e++) {
        int keep = (sel == SEL_ALL) ? 1 : (sel == SEL_LOWER) ? (nbr[e] < (uint32_t)i) : (mask[e] != 0);
        if (keep) sel_buf[k++] = nbr[e];
      }
      int t;
      enc_row(m->row_data + m->row_offsets[i], sel_buf, k, layout, &t);
    }
    free(sel_buf);
  }
  free(bytes);
  free(types);
  return m;
}

void oracle_free(void* mp) {
  omatrix* m = (omatrix*)mp;
  if (!m) return;
  free(m->row_lengths);
  free(m->row_offsets);
  free(m->row_data);
  free(m);
}

/* Matrix facts and per-row flattened bytes, for byte-format parity. */
void oracle_info(void* mp, uint64_t* out6) {
  omatrix* m = (omatrix*)mp;
  out6[0] = m->n;
  out6[1] = m->cardinality;
  out6[2] = m->total_bytes;
  out6[3] = m->num_uint;
  out6[4] = m->num_pshort;
  out6[5] = m->num_bitset;
}
void oracle_row_meta(void* mp, uint8_t* types, uint32_t* cards, uint64_t* nbytes) {
  omatrix* m = (omatrix*)mp;
  for (uint64_t i = 0; i < m->n; i++) {
    oset s = get_row(m, i);
    if (types) types[i] = (uint8_t)s.type;
    if (cards) cards[i] = m->row_lengths[i];
    if (nbytes) nbytes[i] = m->row_offsets[i + 1] - m->row_offsets[i];
  }
}
const uint8_t* oracle_row_bytes(void* mp, uint64_t i, uint64_t* nbytes) {
  omatrix* m = (omatrix*)mp;
  *nbytes = m->row_offsets[i + 1] - m->row_offsets[i];
  return m->row_data + m->row_offsets[i];
}

/* SparseMatrix::get_max_row_id (SparseMatrix.hpp:133-145): first row of maximum length. */
uint32_t oracle_max_row_id(void* mp) {
  omatrix* m = (omatrix*)mp;
  uint64_t mx = 0;
  uint32_t id = 0;
  for (uint64_t i = 0; i < m->n; i++)
    if (m->row_lengths[i] > mx) { mx = m->row_lengths[i]; id = (uint32_t)i; }
  return id;
}

/* ------------------------------------------------------------------------ */
/* Apps.  par_for_range (src/common.hpp:214-309) hands out 100-row blocks    */
/* dynamically; restated as an OpenMP dynamic schedule.                      */
/* ------------------------------------------------------------------------ */

/* undirected_triangle_counting<T,R>::run (apps/undirected_triangle_counting.cpp:27-65). */
uint64_t oracle_triangles(void* mp, int nthreads) {
  omatrix* m = (omatrix*)mp;
  uint64_t total = 0;
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel reduction(+ : total)
  {
    uint32_t* elems = (uint32_t*)malloc(((uint64_t)1 << 16) * 4);
    uint64_t cap = (uint64_t)1 << 16;
#pragma omp for schedule(dynamic, 100)
    for (int64_t i = 0; i < (int64_t)m->n; i++) {
      oset A = get_row(m, i);
      if (A.card > cap) { cap = A.card; elems = (uint32_t*)realloc(elems, cap * 4); }
      uint64_t k = decode(A, elems);
      for (uint64_t e = 0; e < k; e++) total += set_intersect(A, get_row(m, elems[e]), 0, 0);
    }
    free(elems);
  }
  return total;
}

/* n_clique<T,R>::apply_function (apps/n_clique.cpp:30-50): intersect the running set
 * with row(node); at the last level return the cardinality, else recurse over C. */
typedef struct {
  uint8_t** bufs;     /* per depth output buffers */
  uint32_t** elems;   /* per depth decoded elements */
  uint64_t cap;
} clique_scratch;
static uint64_t apply_function(const omatrix* m, uint64_t node, uint64_t depth, uint64_t k,
                               oset* sets, clique_scratch* s) {
  oset C;
  set_intersect(sets[depth - 1], get_row(m, node), s->bufs[depth], &C);
  sets[depth] = C;
  if (++depth == k) return C.card;
  uint64_t cnt = 0, ne = decode(C, s->elems[depth]);
  for (uint64_t e = 0; e < ne; e++) cnt += apply_function(m, s->elems[depth][e], depth, k, sets, s);
  return cnt;
}
/* n_clique<T,R>::run (apps/n_clique.cpp:52-101), k >= 3. */
uint64_t oracle_cliques(void* mp, int k, int nthreads) {
  omatrix* m = (omatrix*)mp;
  uint64_t total = 0;
  uint64_t maxc = 1;
  for (uint64_t i = 0; i < m->n; i++) if (m->row_lengths[i] > maxc) maxc = m->row_lengths[i];
  uint64_t maxb = 16;
  for (uint64_t i = 0; i < m->n; i++) {
    uint64_t b = m->row_offsets[i + 1] - m->row_offsets[i];
    if (b > maxb) maxb = b;
  }
  uint64_t bufsz = (maxb > maxc * 4 ? maxb : maxc * 4) + 64;
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel reduction(+ : total)
  {
    clique_scratch s;
    s.bufs = (uint8_t**)malloc((k + 1) * sizeof(uint8_t*));
    s.elems = (uint32_t**)malloc((k + 1) * sizeof(uint32_t*));
    for (int d = 0; d <= k; d++) {
      s.bufs[d] = (uint8_t*)malloc(bufsz);
      s.elems[d] = (uint32_t*)malloc((maxc + 16) * 4);  /* C is a subset of the pivot row */
    }
    oset* sets = (oset*)malloc((k + 1) * sizeof(oset));
#pragma omp for schedule(dynamic, 100)
    for (int64_t i = 0; i < (int64_t)m->n; i++) {
      oset A = get_row(m, i);
      sets[1] = A;
      uint64_t ne = decode(A, s.elems[1]);
      for (uint64_t e = 0; e < ne; e++) total += apply_function(m, s.elems[1][e], 2, (uint64_t)k, sets, &s);
    }
    for (int d = 0; d <= k; d++) { free(s.bufs[d]); free(s.elems[d]); }
    free(s.bufs); free(s.elems); free(sets);
  }
  return total;
}

/* undirected_lollipop_counting<T,R>::run (apps/undirected_lollipop_counting.cpp:27-77):
 * for x, y in N(x): rs = N(x) ∩ N(y); each z in rs with z < y adds |N(x)|. */
uint64_t oracle_lollipops(void* mp, int nthreads) {
  omatrix* m = (omatrix*)mp;
  uint64_t total = 0;
  uint64_t maxc = 1;
  for (uint64_t i = 0; i < m->n; i++) if (m->row_lengths[i] > maxc) maxc = m->row_lengths[i];
  uint64_t maxb = 16;
  for (uint64_t i = 0; i < m->n; i++) {
    uint64_t b = m->row_offsets[i + 1] - m->row_offsets[i];
    if (b > maxb) maxb = b;
  }
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel reduction(+ : total)
  {
    uint32_t* ys = (uint32_t*)malloc(maxc * 4 + 64);
    uint32_t* zs = (uint32_t*)malloc((maxc + 16) * 4);
    uint8_t* rbuf = (uint8_t*)malloc((maxb > maxc * 4 ? maxb : maxc * 4) + 64);
#pragma omp for schedule(dynamic, 20)
    for (int64_t x = 0; x < (int64_t)m->n; x++) {
      oset Y = get_row(m, x);
      uint64_t ny = decode(Y, ys), t = 0;
      for (uint64_t a = 0; a < ny; a++) {
        oset R;
        set_intersect(Y, get_row(m, ys[a]), rbuf, &R);
        uint64_t nz = decode(R, zs);
        for (uint64_t b = 0; b < nz; b++) if (zs[b] < ys[a]) t += Y.card;
      }
      total += t;
    }
    free(ys); free(zs); free(rbuf);
  }
  return total;
}

/* similar_nodes<T,R>::run (apps/similar_nodes.cpp:29-68). */
uint64_t oracle_similar_nodes(void* mp, uint32_t threshold, int nthreads) {
  omatrix* m = (omatrix*)mp;
  oset A = get_row(m, oracle_max_row_id(mp));
  uint64_t total = 0;
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 100) reduction(+ : total)
  for (int64_t i = 0; i < (int64_t)m->n; i++)
    if (set_intersect(A, get_row(m, i), 0, 0) > threshold) total++;
  return total;
}

/* symbiosity<T,R>::run (apps/symbiosity.cpp:39-58): rows i whose out-row
 * (get_row, matrix `rp`) and in-row (get_column, matrix `cp`; the same matrix
 * for an undirected graph) have Jaccard ratio above `threshold`; the ratio is
 * a double division of the intersection size by |A| + |B| - |A ∩ B|. */
uint64_t oracle_symbiosity(void* rp, void* cp, double threshold, int nthreads) {
  omatrix* r = (omatrix*)rp;
  omatrix* c = (omatrix*)cp;
  uint64_t total = 0;
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 100) reduction(+ : total)
  for (int64_t i = 0; i < (int64_t)r->n; i++) {
    oset A = get_row(r, i), B = get_row(c, i);
    uint64_t both = set_intersect(A, B, 0, 0);
    double ratio = (double)both / (double)(A.card + B.card - both);
    if (ratio > threshold) total++;
  }
  return total;
}

/* n_path<T,R>::run (apps/n_path.cpp:30-88).  visited / old_visited are bitsets
 * over every row; each level ORs the frontier's rows into visited
 * (ops::set_union(bitset, T), src/set/ops/union.hpp:6-127: every element of
 * the row sets its bit), and the next frontier is visited AND NOT old_visited
 * in ascending order (ops::set_difference, src/set/ops/difference.hpp:5-84).
 * The loop stops when that frontier is empty or path_length has reached
 * `depth`; otherwise path_length grows by one.  *reached = set bits. */
uint64_t oracle_n_path(void* mp, uint32_t start, uint64_t depth, uint64_t* reached) {
  omatrix* m = (omatrix*)mp;
  const uint64_t words = (m->n + 64) / 64;
  uint64_t* vis = (uint64_t*)calloc(words, 8);
  uint64_t* old = (uint64_t*)calloc(words, 8);
  uint32_t* frontier = (uint32_t*)malloc((m->n + 1) * 4);
  uint32_t* row = (uint32_t*)malloc((m->n + 1) * 4);
  uint64_t nf = 1, path = 0;
  frontier[0] = start;
  vis[start >> 6] |= 1ull << (start & 63);
  for (;;) {
    memcpy(old, vis, words * 8);
    for (uint64_t f = 0; f < nf; f++) {
      uint64_t k = decode(get_row(m, frontier[f]), row);
      for (uint64_t e = 0; e < k; e++) vis[row[e] >> 6] |= 1ull << (row[e] & 63);
    }
    nf = 0;
    for (uint64_t w = 0; w < words; w++) {
      uint64_t x = vis[w] & ~old[w];
      while (x) {
        frontier[nf++] = (uint32_t)(64 * w + __builtin_ctzll(x));
        x &= x - 1;
      }
    }
    if (nf == 0 || path >= depth) break;
    path++;
  }
  if (reached) {
    uint64_t t = 0;
    for (uint64_t w = 0; w < words; w++) t += popc64(vis[w]);
    *reached = t;
  }
  free(vis); free(old); free(frontier); free(row);
  return path;
}

/* ops::set_intersect on pairs of rows. */
void oracle_intersect_rows(void* mp, const uint32_t* a, const uint32_t* b, uint64_t np,
                           uint32_t* counts, int nthreads) {
  omatrix* m = (omatrix*)mp;
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t p = 0; p < (int64_t)np; p++)
    counts[p] = (uint32_t)set_intersect(get_row(m, a[p]), get_row(m, b[p]), 0, 0);
}

/* Triangle count over the vertex range [lo, hi) only: a bounded sample of the
 * same per-vertex work, for CPU timing. */
uint64_t oracle_triangles_range(void* mp, uint64_t lo, uint64_t hi, int nthreads) {
  omatrix* m = (omatrix*)mp;
  uint64_t total = 0;
  if (hi > m->n) hi = m->n;
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel reduction(+ : total)
  {
    uint64_t cap = (uint64_t)1 << 16;
    uint32_t* elems = (uint32_t*)malloc(cap * 4);
#pragma omp for schedule(dynamic, 100)
    for (int64_t i = (int64_t)lo; i < (int64_t)hi; i++) {
      oset A = get_row(m, i);
      if (A.card > cap) { cap = A.card; elems = (uint32_t*)realloc(elems, cap * 4); }
      uint64_t k = decode(A, elems);
      for (uint64_t e = 0; e < k; e++) total += set_intersect(A, get_row(m, elems[e]), 0, 0);
    }
    free(elems);
  }
  return total;
}

int oracle_max_threads(void) { return omp_get_max_threads(); }

/* All rows in the row-dump format of oracle/ref_rowdump.cpp: per row u8 type,
 * u32 cardinality, u64 flattened bytes, then those bytes.  Returns the size;
 * writes only when buf != NULL. */
uint64_t oracle_dump(void* mp, uint8_t* buf) {
  omatrix* m = (omatrix*)mp;
  uint64_t pos = 0;
  for (uint64_t i = 0; i < m->n; i++) {
    oset s = get_row(m, i);
    uint64_t nb = m->row_offsets[i + 1] - m->row_offsets[i];
    if (buf) {
      buf[pos] = (uint8_t)s.type;
      wr32(buf + pos + 1, m->row_lengths[i]);
      wr64(buf + pos + 5, nb);
      memcpy(buf + pos + 13, m->row_data + m->row_offsets[i], nb);
    }
    pos += 13 + nb;
  }
  return pos;
}

/* n_clique<T,R>::apply_function with WRITE_TABLE (apps/n_clique.cpp:30-50):
 * the tuple holds the pivot and one element per level; at the last level
 * Table<T>::write_table (src/Table.hpp:30-43) appends one tuple per element
 * of C.  Writes up to cap tuples of k u32 in the reference's loop order. */
static void list_function(const omatrix* m, uint64_t node, uint64_t depth, uint64_t k, oset* sets,
                          clique_scratch* s, uint32_t* tuple, uint32_t* out, uint64_t cap, uint64_t* total) {
  oset C;
  set_intersect(sets[depth - 1], get_row(m, node), s->bufs[depth], &C);
  sets[depth] = C;
  tuple[depth - 1] = (uint32_t)node;
  ++depth;
  uint64_t ne = decode(C, s->elems[depth]);
  for (uint64_t e = 0; e < ne; e++) {
    if (depth == k) {
      if (*total < cap) {
        for (uint64_t d = 0; d + 1 < k; d++) out[k * *total + d] = tuple[d];
        out[k * *total + k - 1] = s->elems[depth][e];
      }
      (*total)++;
    } else {
      list_function(m, s->elems[depth][e], depth, k, sets, s, tuple, out, cap, total);
    }
  }
}
/* n_clique<T,R>::run with WRITE_TABLE (apps/n_clique.cpp:52-101), one thread,
 * 3 <= k <= 16; returns the number of cliques. */
uint64_t oracle_list_cliques(void* mp, int k, uint32_t* out, uint64_t cap) {
  omatrix* m = (omatrix*)mp;
  if (k < 3 || k > 16) return 0;
  uint64_t maxc = 1, maxb = 16, total = 0;
  for (uint64_t i = 0; i < m->n; i++) {
    if (m->row_lengths[i] > maxc) maxc = m->row_lengths[i];
    if (m->row_offsets[i + 1] - m->row_offsets[i] > maxb) maxb = m->row_offsets[i + 1] - m->row_offsets[i];
  }
  uint64_t bufsz = (maxb > maxc * 4 ? maxb : maxc * 4) + 64;
  clique_scratch s;
  s.bufs = (uint8_t**)malloc((k + 1) * sizeof(uint8_t*));
  s.elems = (uint32_t**)malloc((k + 1) * sizeof(uint32_t*));
  for (int d = 0; d <= k; d++) {
    s.bufs[d] = (uint8_t*)malloc(bufsz);
    s.elems[d] = (uint32_t*)malloc((maxc + 16) * 4);
  }
  oset* sets = (oset*)malloc((k + 1) * sizeof(oset));
  uint32_t tuple[16];
  for (uint64_t i = 0; i < m->n; i++) {
    oset A = get_row(m, i);
    sets[1] = A;
    tuple[0] = (uint32_t)i;
    uint64_t ne = decode(A, s.elems[1]);
    for (uint64_t e = 0; e < ne; e++) list_function(m, s.elems[1][e], 2, (uint64_t)k, sets, &s, tuple, out, cap, &total);
  }
  for (int d = 0; d <= k; d++) { free(s.bufs[d]); free(s.elems[d]); }
  free(s.bufs); free(s.elems); free(sets);
  return total;
}

/* Triangle tuples as undirected_triangle_counting would emit them with tuple
 * output on (Table<T>::write_table, src/Table.hpp:30-43): for every pivot i and
 * j in row(i), each k in row(i) ∩ row(j) gives (i, j, k).  Writes up to cap
 * tuples (3 u32 each) in pivot order and returns the total. */
uint64_t oracle_list_triangles(void* mp, uint32_t* out, uint64_t cap) {
  omatrix* m = (omatrix*)mp;
  uint64_t total = 0, maxc = 1, maxb = 16;
  for (uint64_t i = 0; i < m->n; i++) {
    if (m->row_lengths[i] > maxc) maxc = m->row_lengths[i];
    if (m->row_offsets[i + 1] - m->row_offsets[i] > maxb) maxb = m->row_offsets[i + 1] - m->row_offsets[i];
  }
  uint32_t* as = (uint32_t*)malloc((maxc + 16) * 4);
  uint32_t* cs = (uint32_t*)malloc((maxc + 16) * 4);
  uint8_t* cbuf = (uint8_t*)malloc((maxb > maxc * 4 ? maxb : maxc * 4) + 64);
  for (uint64_t i = 0; i < m->n; i++) {
    oset A = get_row(m, i);
    uint64_t na = decode(A, as);
    for (uint64_t e = 0; e < na; e++) {
      oset Cs;
      set_intersect(A, get_row(m, as[e]), cbuf, &Cs);
      uint64_t nc = decode(Cs, cs);
      for (uint64_t t = 0; t < nc; t++) {
        if (total < cap) {
          out[3 * total] = (uint32_t)i;
          out[3 * total + 1] = as[e];
          out[3 * total + 2] = cs[t];
        }
        total++;
      }
    }
  }
  free(as);
  free(cs);
  free(cbuf);
  return total;
}
