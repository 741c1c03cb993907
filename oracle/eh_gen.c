/*
 * eh_gen.c — CPU regeneration of the seeded R-MAT benchmark graphs, for the
 * CPU baseline arm of bench.py (the reference's algorithm timed on the host
 * cores), so that arm builds its input without loading the GPU library.
 *
 * TEST INFRASTRUCTURE ONLY, like eh_oracle.c: loaded by tests/ and bench.py's
 * CPU legs, never by the product.
 *
 * It restates the library's own generator (eh_generate_rmat and
 * eh_hgraph_reorder_by_degree in simdgraphprocessing_gb300/csrc/eh_host.cpp;
 * the reference has no generator) and must produce the identical CSR, which
 * tests/test_oracle_gen.py checks by SHA-256:
 *  - draw k of R-MAT(a, b, c) picks one quadrant per level l < scale from the
 *    top 53 bits of value(k * scale + l) of a SplitMix64 counter stream (Steele,
 *    Lea, Flood, OOPSLA 2014) keyed by (seed, "RMAT");
 *  - the graph is the first `edges` distinct undirected pairs in draw order,
 *    self-loops dropped;
 *  - rows are sorted; the degree order relabels vertices by descending degree,
 *    ties by ascending id (src/MutableGraph.hpp:20-32, 268-272, 100-123 in the
 *    reference), and re-sorts every row.
 * The draws are deduplicated in parallel: pairs are bucketed by a hash of the
 * key (order of draws kept inside a bucket), each bucket marks the first draw
 * of each of its keys, and the cutoff is the draw index of the edges-th first
 * draw overall.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

static inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

#define SELF_LOOP (~0ULL)

typedef struct {
  uint64_t key, idx;
} kidx;

static void rmat_draws(uint32_t scale, uint64_t t1, uint64_t t2, uint64_t t3, uint64_t skey, uint64_t lo,
                       uint64_t hi, uint64_t* out) {
#pragma omp parallel for schedule(static)
  for (int64_t k = (int64_t)lo; k < (int64_t)hi; k++) {
    uint64_t u = 0, v = 0;
    for (uint32_t l = 0; l < scale; l++) {
      const uint64_t ctr = (uint64_t)k * scale + l;
      const uint64_t r = mix64(skey + (ctr + 1) * 0x9E3779B97F4A7C15ULL) >> 11;
      const uint64_t bu = r >= t2, bv = (r >= t1 && r < t2) || r >= t3;
      u = (u << 1) | bu;
      v = (v << 1) | bv;
    }
    out[k - lo] = (u == v) ? SELF_LOOP : (u < v ? (u << 32) | v : (v << 32) | u);
  }
}

/* First `target` distinct keys (self-loops excluded) of draws[0, D); returns
 * how many were found (< target when D draws are not enough) and writes them,
 * unordered, to result (capacity target). */
static uint64_t first_distinct(const uint64_t* draws, uint64_t D, uint64_t target, uint64_t* result) {
  const int B = 4096;
  const int nt = omp_get_max_threads();
  uint64_t* cnt = calloc((size_t)nt * B + 1, sizeof(uint64_t));
  kidx* part = malloc(D * sizeof(kidx));
  uint64_t* first = calloc((D + 63) / 64, sizeof(uint64_t));
  uint64_t* bstart = calloc(B + 1, sizeof(uint64_t));
  uint64_t found = 0;
#pragma omp parallel num_threads(nt)
  {
    const int t = omp_get_thread_num(), nth = omp_get_num_threads();  /* the team actually started */
    const uint64_t lo = D * t / nth, hi = D * (t + 1) / nth;
    for (uint64_t k = lo; k < hi; k++)
      if (draws[k] != SELF_LOOP) cnt[(uint64_t)t * B + (mix64(draws[k]) >> 52)]++;
#pragma omp barrier
#pragma omp single
    {
      uint64_t acc = 0;  /* bucket-major, thread-minor: draw order kept inside a bucket */
      for (int b = 0; b < B; b++) {
        bstart[b] = acc;
        for (int s = 0; s < nth; s++) {
          const uint64_t c = cnt[(uint64_t)s * B + b];
          cnt[(uint64_t)s * B + b] = acc;
          acc += c;
        }
      }
      bstart[B] = acc;
    }
    for (uint64_t k = lo; k < hi; k++)
      if (draws[k] != SELF_LOOP) {
        const uint64_t b = mix64(draws[k]) >> 52;
        part[cnt[(uint64_t)t * B + b]++] = (kidx){draws[k], k};
      }
#pragma omp barrier
    /* Per bucket: an open-addressing table of its keys; the first draw of each
     * key sets its bit in `first`. */
    uint64_t cap = 0;
    uint64_t* table = NULL;
#pragma omp for schedule(dynamic, 8) reduction(+ : found)
    for (int b = 0; b < B; b++) {
      const uint64_t n = bstart[b + 1] - bstart[b];
      uint64_t need = 16;
      while (need < 2 * n) need <<= 1;
      if (need > cap) {
        free(table);
        cap = need;
        table = malloc(cap * sizeof(uint64_t));
      }
      memset(table, 0xff, need * sizeof(uint64_t));
      for (uint64_t p = bstart[b]; p < bstart[b + 1]; p++) {
        const uint64_t key = part[p].key;
        uint64_t h = (mix64(key ^ 0x5bd1e995ULL) & (need - 1));
        for (;;) {
          if (table[h] == SELF_LOOP) {
            table[h] = key;
            __atomic_fetch_or(&first[part[p].idx >> 6], 1ULL << (part[p].idx & 63), __ATOMIC_RELAXED);
            found++;
            break;
          }
          if (table[h] == key) break;
          h = (h + 1) & (need - 1);
        }
      }
    }
    free(table);
  }
  uint64_t kept = 0;
  if (found >= target && target > 0) {
    /* cutoff = draw index of the target-th first draw */
    uint64_t seen = 0, w = 0;
    while (seen + (uint64_t)__builtin_popcountll(first[w]) < target) seen += __builtin_popcountll(first[w++]);
    uint64_t x = first[w];
    for (uint64_t r = target - seen; r > 1; r--) x &= x - 1;
    const uint64_t cutoff = 64 * w + (uint64_t)__builtin_ctzll(x);
    for (uint64_t k = 0; k <= cutoff; k++)
      if ((first[k >> 6] >> (k & 63)) & 1) result[kept++] = draws[k];
  }
  free(cnt);
  free(part);
  free(first);
  free(bstart);
  return found >= target ? kept : found;
}

static int cmp_u32(const void* a, const void* b) {
  const uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
  return x < y ? -1 : x > y;
}

/* Symmetric CSR of undirected keys (lo << 32 | hi), rows sorted. */
static void csr_from_keys(uint64_t n, const uint64_t* keys, uint64_t m, uint64_t** off_out, uint32_t** nbr_out) {
  uint64_t* off = calloc(n + 1, sizeof(uint64_t));
  uint32_t* nbr = malloc((2 * m + 1) * sizeof(uint32_t));
  uint64_t* cur = malloc((n + 1) * sizeof(uint64_t));
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < (int64_t)m; k++) {
    __atomic_fetch_add(&off[(keys[k] >> 32) + 1], 1, __ATOMIC_RELAXED);
    __atomic_fetch_add(&off[(keys[k] & 0xffffffffu) + 1], 1, __ATOMIC_RELAXED);
  }
  for (uint64_t i = 0; i < n; i++) off[i + 1] += off[i];
  memcpy(cur, off, n * sizeof(uint64_t));
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < (int64_t)m; k++) {
    const uint32_t lo = (uint32_t)(keys[k] >> 32), hi = (uint32_t)(keys[k] & 0xffffffffu);
    nbr[__atomic_fetch_add(&cur[lo], 1, __ATOMIC_RELAXED)] = hi;
    nbr[__atomic_fetch_add(&cur[hi], 1, __ATOMIC_RELAXED)] = lo;
  }
  free(cur);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t i = 0; i < (int64_t)n; i++) qsort(nbr + off[i], off[i + 1] - off[i], sizeof(uint32_t), cmp_u32);
  *off_out = off;
  *nbr_out = nbr;
}

/* Degree order: new id = rank by (degree descending, old id ascending). */
static void reorder_by_degree(uint64_t n, const uint64_t* off, const uint32_t* nbr, uint64_t** off_out,
                              uint32_t** nbr_out) {
  uint64_t maxd = 0;
  for (uint64_t i = 0; i < n; i++)
    if (off[i + 1] - off[i] > maxd) maxd = off[i + 1] - off[i];
  uint64_t* pos = calloc(maxd + 2, sizeof(uint64_t));
  for (uint64_t i = 0; i < n; i++) pos[maxd - (off[i + 1] - off[i]) + 1]++;
  for (uint64_t d = 0; d <= maxd; d++) pos[d + 1] += pos[d];
  uint32_t* new2old = malloc((n + 1) * sizeof(uint32_t));
  uint32_t* old2new = malloc((n + 1) * sizeof(uint32_t));
  for (uint64_t i = 0; i < n; i++) {
    const uint64_t r = pos[maxd - (off[i + 1] - off[i])]++;
    new2old[r] = (uint32_t)i;
    old2new[i] = (uint32_t)r;
  }
  free(pos);
  uint64_t* noff = malloc((n + 1) * sizeof(uint64_t));
  noff[0] = 0;
  for (uint64_t i = 0; i < n; i++) noff[i + 1] = noff[i] + (off[new2old[i] + 1] - off[new2old[i]]);
  uint32_t* nnbr = malloc((noff[n] + 1) * sizeof(uint32_t));
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t i = 0; i < (int64_t)n; i++) {
    const uint32_t o = new2old[i];
    uint64_t d = noff[i];
    for (uint64_t e = off[o]; e < off[o + 1]; e++) nnbr[d++] = old2new[nbr[e]];
    qsort(nnbr + noff[i], noff[i + 1] - noff[i], sizeof(uint32_t), cmp_u32);
  }
  free(new2old);
  free(old2new);
  *off_out = noff;
  *nbr_out = nnbr;
}

/* Degree-ordered R-MAT graph as a symmetric CSR (buffers freed with
 * oracle_gen_free).  Returns the vertex count 2^scale, or 0 when `edges`
 * distinct pairs were not reached. */
uint64_t oracle_rmat(uint32_t scale, uint64_t edges, double a, double b, double c, uint64_t seed,
                     uint64_t** off_out, uint32_t** nbr_out) {
  const uint64_t n = 1ULL << scale;
  const double two53 = 9007199254740992.0;
  const uint64_t t1 = (uint64_t)(a * two53), t2 = (uint64_t)((a + b) * two53), t3 = (uint64_t)((a + b + c) * two53);
  const uint64_t skey = mix64(seed * 0xD1B54A32D192ED03ULL + 0x524D4154ULL /* "RMAT" */);
  uint64_t D = edges + edges / 2;
  if (D < 1024) D = 1024;
  uint64_t* keys = malloc((edges + 1) * sizeof(uint64_t));
  uint64_t got = 0;
  for (int round = 0; round < 16; round++) {
    uint64_t* draws = malloc(D * sizeof(uint64_t));
    rmat_draws(scale, t1, t2, t3, skey, 0, D, draws);
    got = first_distinct(draws, D, edges, keys);
    free(draws);
    if (got >= edges) break;
    D = D + D / 2 + 1024;
  }
  if (got < edges) {
    free(keys);
    return 0;
  }
  uint64_t* off;
  uint32_t* nbr;
  csr_from_keys(n, keys, edges, &off, &nbr);
  free(keys);
  reorder_by_degree(n, off, nbr, off_out, nbr_out);
  free(off);
  free(nbr);
  return n;
}

void oracle_gen_free(void* p) { free(p); }
