/* Drives the C oracle (oracle/eh_oracle.c) under AddressSanitizer and
 * UndefinedBehaviorSanitizer on seeded graphs with hubs, dense blocks and
 * empty rows, in every layout.  Counts must agree across layouts (the
 * reference's own cross-layout invariant).  Prints "ok". */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

void* oracle_build(uint64_t n, const uint64_t* off, const uint32_t* nbr, const uint8_t* mask, int sel, int layout,
                   int nthreads);
void oracle_free(void* m);
uint64_t oracle_triangles(void* m, int nthreads);
uint64_t oracle_cliques(void* m, int k, int nthreads);
uint64_t oracle_lollipops(void* m, int nthreads);
uint64_t oracle_similar_nodes(void* m, uint32_t threshold, int nthreads);
uint64_t oracle_symbiosity(void* rows, void* cols, double threshold, int nthreads);
uint64_t oracle_n_path(void* m, uint32_t start, uint64_t depth, uint64_t* reached);
uint64_t oracle_list_triangles(void* m, uint32_t* out, uint64_t cap);
uint32_t oracle_max_row_id(void* m);

static uint64_t rng_state = 0x9e3779b97f4a7c15ull;
static uint64_t next_rand(void) {
  uint64_t z = (rng_state += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

static int cmp_u64(const void* a, const void* b) {
  const uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
  return x < y ? -1 : x > y;
}

/* Symmetric CSR from random edges: a hub (vertex 0 joined to most vertices), a
 * dense block over ids [70000, 70400) (pshort / bitset rows across a 2^16
 * boundary), random edges, and trailing isolated vertices. */
static void make_graph(uint64_t n, uint64_t m_rand, uint64_t** off_out, uint32_t** nbr_out) {
  uint64_t cap = 2 * (m_rand + n + 400 * 40) + 16, ne = 0;
  uint64_t* keys = (uint64_t*)malloc(cap * sizeof(uint64_t));
  const uint64_t active = n - 50;  /* the last 50 vertices stay isolated */
#define ADD(u, v) do { if ((u) != (v)) { keys[ne++] = ((uint64_t)(u) << 32) | (v); keys[ne++] = ((uint64_t)(v) << 32) | (u); } } while (0)
  for (uint64_t v = 1; v < active; v += 2) ADD(0, v);
  for (uint64_t i = 0; i < 400; i++)
    for (uint64_t j = 0; j < 40; j++) ADD(70000 + i, 70000 + (i + 1 + j * 7) % 400);
  for (uint64_t k = 0; k < m_rand; k++) ADD(next_rand() % active, next_rand() % active);
#undef ADD
  qsort(keys, ne, sizeof(uint64_t), cmp_u64);
  uint64_t u = 0;
  for (uint64_t k = 0; k < ne; k++)
    if (k == 0 || keys[k] != keys[k - 1]) keys[u++] = keys[k];
  uint64_t* off = (uint64_t*)calloc(n + 1, sizeof(uint64_t));
  uint32_t* nbr = (uint32_t*)malloc((u ? u : 1) * sizeof(uint32_t));
  for (uint64_t k = 0; k < u; k++) {
    off[(keys[k] >> 32) + 1]++;
    nbr[k] = (uint32_t)keys[k];
  }
  for (uint64_t i = 0; i < n; i++) off[i + 1] += off[i];
  free(keys);
  *off_out = off;
  *nbr_out = nbr;
}

int main(void) {
  const uint64_t n = 80000;
  uint64_t* off;
  uint32_t* nbr;
  make_graph(n, 120000, &off, &nbr);
  const int layouts[] = {2, 1, 0, 5, 16};  /* uint, pshort, bitset, hybrid, three-tier hybrid */
  uint64_t tri0 = 0, c40 = 0, lol0 = 0, sim0 = 0, sym0 = 0, path0 = 0, reach0 = 0;
  for (int li = 0; li < 5; li++) {
    void* low = oracle_build(n, off, nbr, NULL, 1, layouts[li], 2);
    void* all = oracle_build(n, off, nbr, NULL, 0, layouts[li], 2);
    if (!low || !all) { printf("build failed\n"); return 1; }
    const uint64_t tri = oracle_triangles(low, 2), c4 = oracle_cliques(low, 4, 2);
    const uint64_t lol = oracle_lollipops(all, 2), sim = oracle_similar_nodes(all, 3, 2);
    const uint64_t sym = oracle_symbiosity(all, all, 0.5, 2);
    uint64_t reach = 0;
    const uint64_t path = oracle_n_path(all, oracle_max_row_id(all), 0xeffffff, &reach);
    uint32_t* tuples = (uint32_t*)malloc((3 * tri + 3) * sizeof(uint32_t));
    const uint64_t listed = oracle_list_triangles(low, tuples, tri);
    free(tuples);
    if (li == 0) {
      tri0 = tri; c40 = c4; lol0 = lol; sim0 = sim; sym0 = sym; path0 = path; reach0 = reach;
    } else if (tri != tri0 || c4 != c40 || lol != lol0 || sim != sim0 || sym != sym0 || path != path0 ||
               reach != reach0) {
      printf("layout %d disagrees\n", layouts[li]);
      return 1;
    }
    if (listed != tri || tri == 0 || c4 == 0) { printf("unexpected counts\n"); return 1; }
    oracle_free(low);
    oracle_free(all);
  }
  free(off);
  free(nbr);
  printf("ok %llu %llu\n", (unsigned long long)tri0, (unsigned long long)c40);
  return 0;
}
