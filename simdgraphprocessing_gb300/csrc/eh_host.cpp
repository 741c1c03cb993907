// Host side of the engine: error reporting, the host graph (the reference's
// MutableGraph, src/MutableGraph.hpp), its binary / edge-list formats, degree
// ordering, and the seeded graph generators.
//
// Compiled with -ffp-contract=off so that the few double-precision steps in the
// generators round identically on x86-64 and aarch64 hosts.

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <numeric>
#include <parallel/algorithm>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include <omp.h>

#include "eh_internal.h"

namespace eh {

static thread_local std::string g_last_error;

eh_status set_error(eh_status s, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return s;
}

void clear_error() { g_last_error.clear(); }

void csr_from_undirected_keys(uint64_t n, std::vector<uint64_t>& keys, HostGraph& g) {
  g.n = n;
  g.offsets.assign(n + 1, 0);
  const int64_t m = (int64_t)keys.size();
  const uint64_t* kp = keys.data();
  {
    std::vector<uint64_t> deg(n, 0);
    uint64_t* dp = deg.data();
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < m; k++) {
      __atomic_fetch_add(&dp[kp[k] >> 32], 1, __ATOMIC_RELAXED);
      __atomic_fetch_add(&dp[kp[k] & 0xffffffffu], 1, __ATOMIC_RELAXED);
    }
    for (uint64_t i = 0; i < n; i++) g.offsets[i + 1] = g.offsets[i] + deg[i];
  }
  // Both directions of every edge, placed by atomic row cursors; each row is
  // sorted below, so the result does not depend on the order of placement.
  g.nbrs.resize(g.offsets[n]);
  std::vector<uint64_t> cur(g.offsets.begin(), g.offsets.end() - 1);
  uint64_t* cp = cur.data();
  uint32_t* np = g.nbrs.data();
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < m; k++) {
    const uint32_t lo = (uint32_t)(kp[k] >> 32), hi = (uint32_t)(kp[k] & 0xffffffffu);
    np[__atomic_fetch_add(&cp[lo], 1, __ATOMIC_RELAXED)] = hi;
    np[__atomic_fetch_add(&cp[hi], 1, __ATOMIC_RELAXED)] = lo;
  }
  std::vector<uint64_t>().swap(keys);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t i = 0; i < (int64_t)n; i++)
    std::sort(g.nbrs.begin() + g.offsets[i], g.nbrs.begin() + g.offsets[i + 1]);
  uint64_t mx = 0;
  for (uint64_t i = 0; i < n; i++) mx = std::max(mx, g.offsets[i + 1] - g.offsets[i]);
  g.max_nbrhood_size = mx;
  g.ext_ids.resize(n);
  std::iota(g.ext_ids.begin(), g.ext_ids.end(), 0);
}

void plan_upload_chunks(uint64_t n, const uint64_t* offsets, uint64_t m, uint64_t chunks,
                        std::vector<uint64_t>& rows, std::vector<uint64_t>& upto) {
  if (chunks < 1) chunks = 1;
  rows.assign(1, 0);
  for (uint64_t c = 1; c < chunks; c++) {
    const uint64_t target = m / chunks * c;
    uint64_t lo = 0, hi = n;  // first row whose offset reaches target
    while (lo < hi) {
      const uint64_t mid = lo + (hi - lo) / 2;
      if (offsets[mid] < target) lo = mid + 1;
      else hi = mid;
    }
    rows.push_back(std::max(lo, rows.back()));
  }
  rows.push_back(n);
  upto.assign(chunks, 0);
  uint64_t copied = 0;
  for (uint64_t c = 0; c < chunks; c++) {
    copied = c + 1 == chunks ? m : std::min(m, std::max(copied, offsets[rows[c + 1]]));
    upto[c] = copied;
  }
}

// ---------------------------------------------------------------------------
// Counter-based random stream: value(k) = SplitMix64 finalizer applied to
// key + (k+1) * golden-gamma (Steele, Lea, Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014).  Identical on every host.
// ---------------------------------------------------------------------------
static inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
struct Stream {
  uint64_t key;
  Stream(uint64_t seed, uint64_t tag) : key(mix64(seed * 0xD1B54A32D192ED03ULL + tag)) {}
  inline uint64_t at(uint64_t ctr) const { return mix64(key + (ctr + 1) * 0x9E3779B97F4A7C15ULL); }
};
// Uniform integer in [0, bound) by 64x64->128 multiply-high.
static inline uint64_t bounded(uint64_t r, uint64_t bound) {
  return (uint64_t)(((unsigned __int128)r * bound) >> 64);
}
static inline uint64_t ukey(uint64_t u, uint64_t v) {
  return u < v ? (u << 32) | v : (v << 32) | u;
}
static const uint64_t kSelfLoop = ~0ULL;

// Order-preserving parallel compaction: out receives, in order, the elements
// e of in[0, n) with keep(k) true for their index k; returns how many.
template <class T, class Keep>
static uint64_t compact(const T* in, uint64_t n, Keep keep, T* out) {
  std::vector<uint64_t> start(omp_get_max_threads() + 1, 0);
  uint64_t kept = 0;
#pragma omp parallel
  {
    const uint64_t t = omp_get_thread_num(), nt = omp_get_num_threads();  // the team actually started
    const uint64_t lo = n * t / nt, hi = n * (t + 1) / nt;
    uint64_t c = 0;
    for (uint64_t k = lo; k < hi; k++) c += keep(k) ? 1 : 0;
    start[t + 1] = c;
#pragma omp barrier
#pragma omp single
    {
      for (uint64_t i = 0; i < nt; i++) start[i + 1] += start[i];
      kept = start[nt];
    }
    uint64_t pos = start[t];
    for (uint64_t k = lo; k < hi; k++)
      if (keep(k)) out[pos++] = in[k];
  }
  return kept;
}

// Keeps the first `target` distinct keys in draw order.  `draw(lo, hi, out)`
// fills out[k - lo] for draws k in [lo, hi) (kSelfLoop for draws to discard).
template <class Draw>
static bool first_distinct(uint64_t target, uint64_t first_batch, Draw draw,
                           std::vector<uint64_t>& result) {
  struct KI {
    uint64_t key;
    uint64_t idx;
  };
  std::vector<uint64_t> draws;
  uint64_t total = 0, batch = std::max<uint64_t>(first_batch, 1024);
  for (int round = 0; round < 64; round++) {
    draws.resize(total + batch);
    draw(total, total + batch, draws.data() + total);
    total += batch;
    std::vector<KI> v(total);
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < (int64_t)total; k++) v[k] = KI{draws[k], (uint64_t)k};
    __gnu_parallel::sort(v.begin(), v.end(), [](const KI& a, const KI& b) {
      return a.key < b.key || (a.key == b.key && a.idx < b.idx);
    });
    // The first draw of every distinct key (self-loops, which sort last, dropped).
    std::vector<KI> heads(total);
    const KI* vp = v.data();
    const uint64_t nh = compact(vp, total, [vp](uint64_t k) {
      return vp[k].key != kSelfLoop && (k == 0 || vp[k].key != vp[k - 1].key);
    }, heads.data());
    heads.resize(nh);
    std::vector<KI>().swap(v);
    if (nh >= target) {
      // cutoff = the target-th smallest first-draw index: mark the heads' indices
      // in a bitmap of all draws and walk its popcounts.
      uint64_t cutoff = ~0ULL;
      if (target > 0) {
        const uint64_t nw = (total + 63) / 64;
        std::vector<uint64_t> bits(nw, 0);
#pragma omp parallel for schedule(static)
        for (int64_t h = 0; h < (int64_t)nh; h++)
          __atomic_fetch_or(&bits[heads[h].idx >> 6], 1ULL << (heads[h].idx & 63), __ATOMIC_RELAXED);
        uint64_t seen = 0, w = 0;
        while (seen + (uint64_t)__builtin_popcountll(bits[w]) < target) seen += __builtin_popcountll(bits[w++]);
        uint64_t x = bits[w];
        for (uint64_t r = target - seen; r > 1; r--) x &= x - 1;  // drop the lowest r - 1 set bits
        cutoff = 64 * w + (uint64_t)__builtin_ctzll(x);
      }
      result.resize(nh);
      const KI* hp = heads.data();
      std::vector<uint64_t> keys(nh);
#pragma omp parallel for schedule(static)
      for (int64_t h = 0; h < (int64_t)nh; h++) keys[h] = hp[h].key;
      const uint64_t kept = compact(keys.data(), nh, [hp, cutoff](uint64_t h) { return hp[h].idx <= cutoff; },
                                    result.data());
      result.resize(kept);
      return true;  // result is sorted by key
    }
    // Grow the draw count in proportion to the shortfall.
    double yield = (double)nh / (double)total;
    uint64_t need = (uint64_t)((double)(target - nh) / std::max(yield, 1e-3) * 1.2) + 1024;
    batch = need;
  }
  return false;
}

// in-CSR of a directed graph as the transpose of its out-CSR; sources are
// visited in ascending order, so every in-row comes out sorted.
static void build_in_csr(HostGraph& g) {
  const uint64_t n = g.n;
  g.in_offsets.assign(n + 1, 0);
  for (uint32_t v : g.nbrs) g.in_offsets[v + 1]++;
  for (uint64_t i = 0; i < n; i++) g.in_offsets[i + 1] += g.in_offsets[i];
  g.in_nbrs.resize(g.nbrs.size());
  std::vector<uint64_t> at(g.in_offsets.begin(), g.in_offsets.end() - 1);
  for (uint64_t u = 0; u < n; u++)
    for (uint64_t e = g.offsets[u]; e < g.offsets[u + 1]; e++) g.in_nbrs[at[g.nbrs[e]]++] = (uint32_t)u;
}

static uint64_t max_row(const std::vector<uint64_t>& off) {
  uint64_t mx = 0;
  for (size_t i = 0; i + 1 < off.size(); i++) mx = std::max(mx, off[i + 1] - off[i]);
  return mx;
}

// Whole file into buf: 0 on success, -1 if it cannot be opened, 1 if it cannot
// be read to the end.
static int read_whole_file(const char* path, std::vector<uint8_t>& buf) {
  FILE* f = fopen(path, "rb");
  if (!f) return -1;
  bool ok = fseeko(f, 0, SEEK_END) == 0;
  const off_t size = ok ? ftello(f) : -1;
  ok = ok && size >= 0 && fseeko(f, 0, SEEK_SET) == 0;
  if (ok) {
    buf.resize((size_t)size);
    ok = size == 0 || fread(buf.data(), 1, (size_t)size, f) == (size_t)size;
  }
  fclose(f);
  return ok ? 0 : 1;
}

// Bounds-checked little-endian reads from a byte buffer.
struct ByteCursor {
  const uint8_t* p;
  uint64_t size, pos;
  uint64_t left() const { return size - pos; }
  bool take64(uint64_t& v) {
    if (left() < 8) return false;
    memcpy(&v, p + pos, 8);
    pos += 8;
    return true;
  }
};

static eh_status finish_graph(uint64_t n, std::vector<uint64_t>& keys, eh_hgraph_t* out) {
  HostGraph* g = new (std::nothrow) HostGraph();
  if (!g) return set_error(EH_ERR_OUT_OF_MEMORY, "host graph allocation failed");
  csr_from_undirected_keys(n, keys, *g);
  *out = reinterpret_cast<eh_hgraph_t>(g);
  return EH_OK;
}

}  // namespace eh

using eh::HostGraph;
using eh::set_error;

static HostGraph* HG(eh_hgraph_t g) { return reinterpret_cast<HostGraph*>(g); }

extern "C" {

const char* eh_last_error(void) { return eh::g_last_error.c_str(); }

const char* eh_status_string(eh_status s) {
  switch (s) {
    case EH_OK: return "EH_OK";
    case EH_ERR_INVALID_ARGUMENT: return "EH_ERR_INVALID_ARGUMENT";
    case EH_ERR_CUDA: return "EH_ERR_CUDA";
    case EH_ERR_OUT_OF_MEMORY: return "EH_ERR_OUT_OF_MEMORY";
    case EH_ERR_UNSUPPORTED: return "EH_ERR_UNSUPPORTED";
    case EH_ERR_IO: return "EH_ERR_IO";
    case EH_ERR_DEVICE_CHECK: return "EH_ERR_DEVICE_CHECK";
    case EH_ERR_TIMEOUT: return "EH_ERR_TIMEOUT";
    case EH_ERR_ADMISSION: return "EH_ERR_ADMISSION";
  }
  return "EH_ERR_UNKNOWN";
}

const char* eh_version(void) { return "eh-gb300 0.1 (sm_103a)"; }

eh_status eh_hgraph_from_csr(uint64_t n, const uint64_t* offsets, const uint32_t* nbrs,
                             const uint64_t* ext_ids, eh_hgraph_t* out) {
  EH_CHECK_ARG(out != nullptr, "out is NULL");
  EH_CHECK_ARG(offsets != nullptr, "offsets is NULL");
  EH_CHECK_ARG(n < (1ULL << 32), "n=%llu exceeds the u32 vertex id space", (unsigned long long)n);
  EH_CHECK_ARG(offsets[0] == 0, "offsets[0] must be 0");
  for (uint64_t i = 0; i < n; i++)
    EH_CHECK_ARG(offsets[i + 1] >= offsets[i], "offsets not monotone at row %llu",
                 (unsigned long long)i);
  EH_CHECK_ARG(offsets[n] == 0 || nbrs != nullptr, "nbrs is NULL");
  HostGraph* g = new (std::nothrow) HostGraph();
  if (!g) return set_error(EH_ERR_OUT_OF_MEMORY, "host graph allocation failed");
  g->n = n;
  g->offsets.assign(offsets, offsets + n + 1);
  g->nbrs.assign(nbrs, nbrs + offsets[n]);
  g->ext_ids.resize(n);
  uint64_t mx = 0;
  for (uint64_t i = 0; i < n; i++) {
    g->ext_ids[i] = ext_ids ? ext_ids[i] : i;
    mx = std::max(mx, offsets[i + 1] - offsets[i]);
  }
  g->max_nbrhood_size = mx;
  *out = reinterpret_cast<eh_hgraph_t>(g);
  return EH_OK;
}

eh_status eh_hgraph_read_binary(const char* path, eh_hgraph_t* out) {
  EH_CHECK_ARG(path && out, "path/out is NULL");
  std::vector<uint8_t> buf;
  const int rf = eh::read_whole_file(path, buf);
  if (rf < 0) return set_error(EH_ERR_IO, "cannot open %s", path);
  HostGraph* g = new (std::nothrow) HostGraph();
  if (!g) return set_error(EH_ERR_OUT_OF_MEMORY, "host graph allocation failed");
  // Records: [u64 ext_id][u64 len][u32 x len].  One pass finds every row's
  // neighbours in the file, then the rows are copied in parallel.
  eh::ByteCursor in{buf.data(), rf == 0 ? buf.size() : 0, 0};
  uint64_t n = 0;
  bool ok = in.take64(n) && n < (1ULL << 32) && n <= in.left() / 16;
  std::vector<uint64_t> at;
  if (ok) {
    g->n = n;
    g->offsets.assign(n + 1, 0);
    g->ext_ids.resize(n);
    at.resize(n);
    for (uint64_t i = 0; i < n && ok; i++) {
      uint64_t len = 0;
      ok = in.take64(g->ext_ids[i]) && in.take64(len) && len <= in.left() / 4;
      if (!ok) break;
      at[i] = in.pos;
      in.pos += 4 * len;
      g->offsets[i + 1] = g->offsets[i] + len;
      g->max_nbrhood_size = std::max(g->max_nbrhood_size, len);
    }
  }
  if (!ok) {
    delete g;
    return set_error(EH_ERR_IO, "truncated or malformed binary graph %s", path);
  }
  g->nbrs.resize(g->offsets[n]);
#pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t i = 0; i < (int64_t)n; i++)
    memcpy(g->nbrs.data() + g->offsets[i], buf.data() + at[i], 4 * (g->offsets[i + 1] - g->offsets[i]));
  *out = reinterpret_cast<eh_hgraph_t>(g);
  return EH_OK;
}

eh_status eh_hgraph_write_binary(eh_hgraph_t gh, const char* path) {
  EH_CHECK_ARG(gh && path, "graph/path is NULL");
  HostGraph* g = HG(gh);
  FILE* f = fopen(path, "wb");
  if (!f) return set_error(EH_ERR_IO, "cannot open %s for writing", path);
  bool ok = fwrite(&g->n, sizeof(uint64_t), 1, f) == 1;
  for (uint64_t i = 0; i < g->n && ok; i++) {
    uint64_t hdr[2] = {g->ext_ids[i], g->offsets[i + 1] - g->offsets[i]};
    ok = fwrite(hdr, sizeof(uint64_t), 2, f) == 2;
    if (ok && hdr[1])
      ok = fwrite(g->nbrs.data() + g->offsets[i], sizeof(uint32_t), hdr[1], f) == hdr[1];
  }
  ok = (fclose(f) == 0) && ok;
  return ok ? EH_OK : set_error(EH_ERR_IO, "write to %s failed", path);
}

eh_status eh_hgraph_read_edge_list(const char* path, eh_hgraph_t* out) {
  EH_CHECK_ARG(path && out, "path/out is NULL");
  std::ifstream in(path, std::ios::binary);
  if (!in) return set_error(EH_ERR_IO, "cannot open %s", path);
  std::string text((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
  // Tokens are separated by ' ', '\t', '\n' or 'A', as the reference's strtok call.
  std::vector<uint64_t> tok;
  size_t p = 0, L = text.size();
  auto is_sep = [](char c) { return c == ' ' || c == '\t' || c == '\n' || c == 'A'; };
  while (p < L) {
    while (p < L && is_sep(text[p])) p++;
    if (p >= L) break;
    size_t q = p;
    while (q < L && !is_sep(text[q])) q++;
    tok.push_back(strtoull(text.c_str() + p, nullptr, 10));
    p = q;
  }
  if (tok.size() % 2) return set_error(EH_ERR_IO, "%s: odd number of ids", path);
  std::unordered_map<uint64_t, uint32_t> ids;
  std::vector<uint64_t> id_map;
  std::vector<std::vector<uint32_t>> rows;
  auto intern = [&](uint64_t x) -> uint32_t {
    auto it = ids.find(x);
    if (it != ids.end()) return it->second;
    uint32_t id = (uint32_t)id_map.size();
    ids.emplace(x, id);
    id_map.push_back(x);
    rows.emplace_back();
    return id;
  };
  for (size_t t = 0; t < tok.size(); t += 2) {
    uint32_t s = intern(tok[t]);
    uint32_t d = intern(tok[t + 1]);
    rows[s].push_back(d);
    rows[d].push_back(s);
  }
  HostGraph* g = new (std::nothrow) HostGraph();
  if (!g) return set_error(EH_ERR_OUT_OF_MEMORY, "host graph allocation failed");
  g->n = rows.size();
  g->offsets.assign(g->n + 1, 0);
  for (uint64_t i = 0; i < g->n; i++) {
    auto& r = rows[i];
    std::sort(r.begin(), r.end());
    // The reference takes the maximum row size before removing duplicates.
    g->max_nbrhood_size = std::max<uint64_t>(g->max_nbrhood_size, r.size());
    r.erase(std::unique(r.begin(), r.end()), r.end());
    g->offsets[i + 1] = g->offsets[i] + r.size();
  }
  g->nbrs.reserve(g->offsets[g->n]);
  for (auto& r : rows) g->nbrs.insert(g->nbrs.end(), r.begin(), r.end());
  g->ext_ids = id_map;
  *out = reinterpret_cast<eh_hgraph_t>(g);
  return EH_OK;
}

eh_status eh_hgraph_reorder_by_degree(eh_hgraph_t gh) {
  EH_CHECK_ARG(gh, "graph is NULL");
  HostGraph* g = HG(gh);
  // reassign_ids (src/MutableGraph.hpp:96-123) only handles undirected graphs.
  if (g->directed) return set_error(EH_ERR_UNSUPPORTED, "degree reordering needs an undirected graph");
  const uint64_t n = g->n;
  std::vector<uint32_t> new2old(n);
  std::iota(new2old.begin(), new2old.end(), 0);
  const uint64_t* off = g->offsets.data();
  // Descending degree, ties by ascending old id: a strict total order, so any
  // correct sort gives the same permutation as the reference's std::sort.
  __gnu_parallel::sort(new2old.begin(), new2old.end(), [off](uint32_t a, uint32_t b) {
    uint64_t da = off[a + 1] - off[a], db = off[b + 1] - off[b];
    return da != db ? da > db : a < b;
  });
  std::vector<uint32_t> old2new(n);
  for (uint64_t i = 0; i < n; i++) old2new[new2old[i]] = (uint32_t)i;
  std::vector<uint64_t> noff(n + 1, 0);
  for (uint64_t i = 0; i < n; i++) noff[i + 1] = noff[i] + (off[new2old[i] + 1] - off[new2old[i]]);
  std::vector<uint32_t> nnbr(g->nbrs.size());
  std::vector<uint64_t> next(n);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t i = 0; i < (int64_t)n; i++) {
    uint32_t o = new2old[i];
    uint64_t dst = noff[i];
    for (uint64_t e = off[o]; e < off[o + 1]; e++) nnbr[dst++] = old2new[g->nbrs[e]];
    std::sort(nnbr.begin() + noff[i], nnbr.begin() + noff[i + 1]);
    next[i] = g->ext_ids[o];
  }
  g->offsets.swap(noff);
  g->nbrs.swap(nnbr);
  g->ext_ids.swap(next);
  return EH_OK;
}

eh_status eh_hgraph_view(eh_hgraph_t gh, uint64_t* n, uint64_t* num_edges, const uint64_t** offsets,
                         const uint32_t** nbrs, const uint64_t** ext_ids,
                         uint64_t* max_nbrhood_size) {
  EH_CHECK_ARG(gh, "graph is NULL");
  HostGraph* g = HG(gh);
  if (n) *n = g->n;
  if (num_edges) *num_edges = g->offsets[g->n];
  if (offsets) *offsets = g->offsets.data();
  if (nbrs) *nbrs = g->nbrs.data();
  if (ext_ids) *ext_ids = g->ext_ids.data();
  if (max_nbrhood_size) *max_nbrhood_size = g->max_nbrhood_size;
  return EH_OK;
}

void eh_hgraph_free(eh_hgraph_t g) { delete HG(g); }

eh_status eh_hgraph_read_directed_binary(const char* path, eh_hgraph_t* out) {
  EH_CHECK_ARG(path && out, "path/out is NULL");
  std::vector<uint8_t> buf;
  const int rf = eh::read_whole_file(path, buf);
  if (rf < 0) return set_error(EH_ERR_IO, "cannot open %s", path);
  HostGraph* g = new (std::nothrow) HostGraph();
  if (!g) return set_error(EH_ERR_OUT_OF_MEMORY, "host graph allocation failed");
  g->directed = true;
  // Records: [u64 ext_id][u64 out_len][u32 x out_len][u64 in_len][u32 x in_len].
  eh::ByteCursor in{buf.data(), rf == 0 ? buf.size() : 0, 0};
  uint64_t n = 0;
  bool ok = in.take64(n) && n < (1ULL << 32) && n <= in.left() / 24;
  std::vector<uint64_t> at_out, at_in;
  if (ok) {
    g->n = n;
    g->offsets.assign(n + 1, 0);
    g->in_offsets.assign(n + 1, 0);
    g->ext_ids.resize(n);
    at_out.resize(n);
    at_in.resize(n);
    for (uint64_t i = 0; i < n && ok; i++) {
      uint64_t len = 0, in_len = 0;
      ok = in.take64(g->ext_ids[i]) && in.take64(len) && len <= in.left() / 4;
      if (!ok) break;
      at_out[i] = in.pos;
      in.pos += 4 * len;
      ok = in.take64(in_len) && in_len <= in.left() / 4;
      if (!ok) break;
      at_in[i] = in.pos;
      in.pos += 4 * in_len;
      g->offsets[i + 1] = g->offsets[i] + len;
      g->in_offsets[i + 1] = g->in_offsets[i] + in_len;
      g->max_nbrhood_size = std::max(g->max_nbrhood_size, std::max(len, in_len));
    }
  }
  if (ok) {
    g->nbrs.resize(g->offsets[n]);
    g->in_nbrs.resize(g->in_offsets[n]);
    int bad = 0;
#pragma omp parallel for schedule(dynamic, 4096) reduction(| : bad)
    for (int64_t i = 0; i < (int64_t)n; i++) {
      uint32_t* o = g->nbrs.data() + g->offsets[i];
      uint32_t* r = g->in_nbrs.data() + g->in_offsets[i];
      const uint64_t lo = g->offsets[i + 1] - g->offsets[i], li = g->in_offsets[i + 1] - g->in_offsets[i];
      memcpy(o, buf.data() + at_out[i], 4 * lo);
      memcpy(r, buf.data() + at_in[i], 4 * li);
      for (uint64_t k = 0; k < lo; k++) bad |= o[k] >= n;
      for (uint64_t k = 0; k < li; k++) bad |= r[k] >= n;
    }
    ok = !bad;
  }
  if (!ok) {
    delete g;
    return set_error(EH_ERR_IO, "truncated or malformed directed binary graph %s", path);
  }
  *out = reinterpret_cast<eh_hgraph_t>(g);
  return EH_OK;
}

eh_status eh_hgraph_write_directed_binary(eh_hgraph_t gh, const char* path) {
  EH_CHECK_ARG(gh && path, "graph/path is NULL");
  HostGraph* g = HG(gh);
  const std::vector<uint64_t>& io = g->directed ? g->in_offsets : g->offsets;
  const std::vector<uint32_t>& in = g->directed ? g->in_nbrs : g->nbrs;
  FILE* f = fopen(path, "wb");
  if (!f) return set_error(EH_ERR_IO, "cannot open %s for writing", path);
  bool ok = fwrite(&g->n, sizeof(uint64_t), 1, f) == 1;
  for (uint64_t i = 0; i < g->n && ok; i++) {
    uint64_t hdr[2] = {g->ext_ids[i], g->offsets[i + 1] - g->offsets[i]};
    ok = fwrite(hdr, sizeof(uint64_t), 2, f) == 2;
    if (ok && hdr[1]) ok = fwrite(g->nbrs.data() + g->offsets[i], sizeof(uint32_t), hdr[1], f) == hdr[1];
    const uint64_t len = io[i + 1] - io[i];
    ok = ok && fwrite(&len, sizeof(uint64_t), 1, f) == 1;
    if (ok && len) ok = fwrite(in.data() + io[i], sizeof(uint32_t), len, f) == len;
  }
  ok = (fclose(f) == 0) && ok;
  return ok ? EH_OK : set_error(EH_ERR_IO, "write to %s failed", path);
}

eh_status eh_hgraph_read_directed_edge_list(const char* path, eh_hgraph_t* out) {
  EH_CHECK_ARG(path && out, "path/out is NULL");
  std::ifstream in(path, std::ios::binary);
  if (!in) return set_error(EH_ERR_IO, "cannot open %s", path);
  std::string text((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
  std::vector<uint64_t> tok;
  size_t p = 0, L = text.size();
  auto is_sep = [](char c) { return c == ' ' || c == '\t' || c == '\n' || c == 'A'; };
  while (p < L) {
    while (p < L && is_sep(text[p])) p++;
    if (p >= L) break;
    size_t q = p;
    while (q < L && !is_sep(text[q])) q++;
    tok.push_back(strtoull(text.c_str() + p, nullptr, 10));
    p = q;
  }
  if (tok.size() % 2) return set_error(EH_ERR_IO, "%s: odd number of ids", path);
  std::unordered_map<uint64_t, uint32_t> ids;
  std::vector<uint64_t> id_map;
  std::vector<std::vector<uint32_t>> outs, ins;
  auto intern = [&](uint64_t x) -> uint32_t {
    auto it = ids.find(x);
    if (it != ids.end()) return it->second;
    uint32_t id = (uint32_t)id_map.size();
    ids.emplace(x, id);
    id_map.push_back(x);
    outs.emplace_back();
    ins.emplace_back();
    return id;
  };
  for (size_t t = 0; t < tok.size(); t += 2) {
    uint32_t s = intern(tok[t]);
    uint32_t d = intern(tok[t + 1]);
    outs[s].push_back(d);
    ins[d].push_back(s);
  }
  HostGraph* g = new (std::nothrow) HostGraph();
  if (!g) return set_error(EH_ERR_OUT_OF_MEMORY, "host graph allocation failed");
  g->directed = true;
  g->n = outs.size();
  auto pack = [g](std::vector<std::vector<uint32_t>>& rows, std::vector<uint64_t>& off,
                  std::vector<uint32_t>& nbr) {
    off.assign(g->n + 1, 0);
    for (uint64_t i = 0; i < g->n; i++) {
      auto& r = rows[i];
      std::sort(r.begin(), r.end());
      // The reference takes the maximum row size before removing duplicates.
      g->max_nbrhood_size = std::max<uint64_t>(g->max_nbrhood_size, r.size());
      r.erase(std::unique(r.begin(), r.end()), r.end());
      off[i + 1] = off[i] + r.size();
    }
    nbr.reserve(off[g->n]);
    for (auto& r : rows) nbr.insert(nbr.end(), r.begin(), r.end());
  };
  pack(ins, g->in_offsets, g->in_nbrs);
  pack(outs, g->offsets, g->nbrs);
  g->ext_ids = id_map;
  *out = reinterpret_cast<eh_hgraph_t>(g);
  return EH_OK;
}

eh_status eh_hgraph_directed_from_csr(uint64_t n, const uint64_t* offsets, const uint32_t* nbrs,
                                      const uint64_t* ext_ids, eh_hgraph_t* out) {
  EH_CHECK_ARG(out != nullptr, "out is NULL");
  EH_CHECK_ARG(offsets != nullptr, "offsets is NULL");
  EH_CHECK_ARG(n < (1ULL << 32), "n=%llu exceeds the u32 vertex id space", (unsigned long long)n);
  EH_CHECK_ARG(offsets[0] == 0, "offsets[0] must be 0");
  for (uint64_t i = 0; i < n; i++) {
    EH_CHECK_ARG(offsets[i + 1] >= offsets[i], "offsets not monotone at row %llu", (unsigned long long)i);
    for (uint64_t e = offsets[i]; e < offsets[i + 1]; e++) {
      EH_CHECK_ARG(nbrs[e] < n, "row %llu names vertex %u >= n", (unsigned long long)i, nbrs[e]);
      EH_CHECK_ARG(e == offsets[i] || nbrs[e] > nbrs[e - 1], "row %llu is not strictly ascending",
                   (unsigned long long)i);
    }
  }
  HostGraph* g = new (std::nothrow) HostGraph();
  if (!g) return set_error(EH_ERR_OUT_OF_MEMORY, "host graph allocation failed");
  g->directed = true;
  g->n = n;
  g->offsets.assign(offsets, offsets + n + 1);
  g->nbrs.assign(nbrs, nbrs + offsets[n]);
  g->ext_ids.resize(n);
  for (uint64_t i = 0; i < n; i++) g->ext_ids[i] = ext_ids ? ext_ids[i] : i;
  eh::build_in_csr(*g);
  g->max_nbrhood_size = std::max(eh::max_row(g->offsets), eh::max_row(g->in_offsets));
  *out = reinterpret_cast<eh_hgraph_t>(g);
  return EH_OK;
}

eh_status eh_hgraph_in_view(eh_hgraph_t gh, int* directed, uint64_t* num_edges, const uint64_t** in_offsets,
                            const uint32_t** in_nbrs) {
  EH_CHECK_ARG(gh, "graph is NULL");
  HostGraph* g = HG(gh);
  if (directed) *directed = g->directed ? 1 : 0;
  const std::vector<uint64_t>& io = g->directed ? g->in_offsets : g->offsets;
  const std::vector<uint32_t>& in = g->directed ? g->in_nbrs : g->nbrs;
  if (num_edges) *num_edges = io[g->n];
  if (in_offsets) *in_offsets = io.data();
  if (in_nbrs) *in_nbrs = in.data();
  return EH_OK;
}

eh_status eh_generate_rmat(uint32_t scale, uint64_t num_edges, double a, double b, double c,
                           uint64_t seed, eh_hgraph_t* out) {
  EH_CHECK_ARG(out, "out is NULL");
  EH_CHECK_ARG(scale >= 1 && scale <= 31, "scale %u out of range [1,31]", scale);
  EH_CHECK_ARG(a >= 0 && b >= 0 && c >= 0 && a + b + c <= 1.0, "bad R-MAT probabilities");
  const uint64_t n = 1ULL << scale;
  EH_CHECK_ARG(num_edges <= n * (n - 1) / 2, "more edges than vertex pairs");
  // Quadrant thresholds on the top 53 bits of each draw.
  const double two53 = 9007199254740992.0;
  const uint64_t t1 = (uint64_t)(a * two53), t2 = (uint64_t)((a + b) * two53),
                 t3 = (uint64_t)((a + b + c) * two53);
  eh::Stream st(seed, 0x524D4154ULL /* "RMAT" */);
  auto draw = [&](uint64_t lo, uint64_t hi, uint64_t* dst) {
#pragma omp parallel for schedule(static)
    for (int64_t k = (int64_t)lo; k < (int64_t)hi; k++) {
      uint64_t u = 0, v = 0;
      for (uint32_t l = 0; l < scale; l++) {
        uint64_t r = st.at((uint64_t)k * scale + l) >> 11;
        uint64_t bu = r >= t2, bv = (r >= t1 && r < t2) || r >= t3;
        u = (u << 1) | bu;
        v = (v << 1) | bv;
      }
      dst[k - lo] = (u == v) ? eh::kSelfLoop : eh::ukey(u, v);
    }
  };
  std::vector<uint64_t> keys;
  if (!eh::first_distinct(num_edges, num_edges + num_edges / 2, draw, keys))
    return set_error(EH_ERR_INVALID_ARGUMENT, "R-MAT could not reach %llu distinct edges",
                     (unsigned long long)num_edges);
  return eh::finish_graph(n, keys, out);
}

eh_status eh_generate_er(uint64_t n, uint64_t num_edges, uint64_t seed, eh_hgraph_t* out) {
  EH_CHECK_ARG(out, "out is NULL");
  EH_CHECK_ARG(n >= 2 && n < (1ULL << 32), "n out of range");
  EH_CHECK_ARG(num_edges <= n * (n - 1) / 2, "more edges than vertex pairs");
  eh::Stream st(seed, 0x4552ULL /* "ER" */);
  auto draw = [&](uint64_t lo, uint64_t hi, uint64_t* dst) {
#pragma omp parallel for schedule(static)
    for (int64_t k = (int64_t)lo; k < (int64_t)hi; k++) {
      uint64_t u = eh::bounded(st.at(2 * (uint64_t)k), n);
      uint64_t v = eh::bounded(st.at(2 * (uint64_t)k + 1), n);
      dst[k - lo] = (u == v) ? eh::kSelfLoop : eh::ukey(u, v);
    }
  };
  std::vector<uint64_t> keys;
  if (!eh::first_distinct(num_edges, num_edges + num_edges / 8 + 64, draw, keys))
    return set_error(EH_ERR_INVALID_ARGUMENT, "ER could not reach %llu distinct edges",
                     (unsigned long long)num_edges);
  return eh::finish_graph(n, keys, out);
}

eh_status eh_generate_ba(uint64_t n, uint32_t m, uint64_t seed, eh_hgraph_t* out) {
  EH_CHECK_ARG(out, "out is NULL");
  EH_CHECK_ARG(m >= 1 && n > (uint64_t)m + 1 && n < (1ULL << 32), "need n > m+1 >= 2");
  eh::Stream st(seed, 0x4241ULL /* "BA" */);
  std::vector<uint64_t> keys;
  std::vector<uint32_t> ends;  // every edge contributes both endpoints
  // Seed clique on vertices 0..m.
  for (uint32_t u = 0; u <= m; u++)
    for (uint32_t v = u + 1; v <= m; v++) {
      keys.push_back(eh::ukey(u, v));
      ends.push_back(u);
      ends.push_back(v);
    }
  uint64_t ctr = 0;
  std::vector<uint32_t> picked;
  for (uint64_t v = m + 1; v < n; v++) {
    picked.clear();
    while (picked.size() < m) {
      uint32_t t = ends[eh::bounded(st.at(ctr++), ends.size())];
      if (std::find(picked.begin(), picked.end(), t) == picked.end()) picked.push_back(t);
    }
    for (uint32_t t : picked) {
      keys.push_back(eh::ukey(t, v));
      ends.push_back(t);
      ends.push_back((uint32_t)v);
    }
  }
  std::sort(keys.begin(), keys.end());
  return eh::finish_graph(n, keys, out);
}

eh_status eh_generate_planted_cliques(uint64_t n, uint64_t background_edges, uint32_t num_cliques,
                                      uint32_t min_size, uint32_t max_size, uint64_t seed,
                                      eh_hgraph_t* out) {
  EH_CHECK_ARG(out, "out is NULL");
  EH_CHECK_ARG(min_size >= 2 && min_size <= max_size && max_size <= n, "bad clique sizes");
  eh_hgraph_t bg = nullptr;
  eh_status s = eh_generate_er(n, background_edges, seed, &bg);
  if (s != EH_OK) return s;
  HostGraph* g = HG(bg);
  std::vector<uint64_t> keys;
  keys.reserve(g->nbrs.size() / 2);
  for (uint64_t u = 0; u < n; u++)
    for (uint64_t e = g->offsets[u]; e < g->offsets[u + 1]; e++)
      if (g->nbrs[e] > u) keys.push_back((u << 32) | g->nbrs[e]);
  eh_hgraph_free(bg);
  // Discrete log-uniform sizes: P(s) proportional to 1/s on [min_size, max_size].
  std::vector<double> cdf(max_size - min_size + 1);
  double acc = 0.0;
  for (uint32_t s2 = min_size; s2 <= max_size; s2++) {
    acc += 1.0 / (double)s2;
    cdf[s2 - min_size] = acc;
  }
  eh::Stream st(seed, 0x434C51ULL /* "CLQ" */);
  uint64_t ctr = 0;
  std::vector<uint32_t> members;
  std::unordered_set<uint32_t> seen;
  for (uint32_t q = 0; q < num_cliques; q++) {
    double u = (double)(st.at(ctr++) >> 11) * (1.0 / 9007199254740992.0) * acc;
    uint32_t size = min_size + (uint32_t)(std::lower_bound(cdf.begin(), cdf.end(), u) - cdf.begin());
    if (size > max_size) size = max_size;
    members.clear();
    seen.clear();
    while (members.size() < size) {
      uint32_t v = (uint32_t)eh::bounded(st.at(ctr++), n);
      if (seen.insert(v).second) members.push_back(v);
    }
    for (size_t x = 0; x < members.size(); x++)
      for (size_t y = x + 1; y < members.size(); y++) keys.push_back(eh::ukey(members[x], members[y]));
  }
  __gnu_parallel::sort(keys.begin(), keys.end());
  keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
  return eh::finish_graph(n, keys, out);
}

eh_status eh_generate_directed_rmat(uint32_t scale, uint64_t num_edges, double a, double b, double c,
                                    uint64_t seed, eh_hgraph_t* out) {
  EH_CHECK_ARG(out, "out is NULL");
  EH_CHECK_ARG(scale >= 1 && scale <= 31, "scale %u out of range [1,31]", scale);
  EH_CHECK_ARG(a >= 0 && b >= 0 && c >= 0 && a + b + c <= 1.0, "bad R-MAT probabilities");
  const uint64_t n = 1ULL << scale;
  EH_CHECK_ARG(num_edges <= n * (n - 1), "more edges than ordered vertex pairs");
  const double two53 = 9007199254740992.0;
  const uint64_t t1 = (uint64_t)(a * two53), t2 = (uint64_t)((a + b) * two53),
                 t3 = (uint64_t)((a + b + c) * two53);
  eh::Stream st(seed, 0x44524D4154ULL /* "DRMAT" */);
  auto draw = [&](uint64_t lo, uint64_t hi, uint64_t* dst) {
#pragma omp parallel for schedule(static)
    for (int64_t k = (int64_t)lo; k < (int64_t)hi; k++) {
      uint64_t u = 0, v = 0;
      for (uint32_t l = 0; l < scale; l++) {
        uint64_t r = st.at((uint64_t)k * scale + l) >> 11;
        uint64_t bu = r >= t2, bv = (r >= t1 && r < t2) || r >= t3;
        u = (u << 1) | bu;
        v = (v << 1) | bv;
      }
      dst[k - lo] = (u == v) ? eh::kSelfLoop : (u << 32) | v;
    }
  };
  std::vector<uint64_t> keys;
  if (!eh::first_distinct(num_edges, num_edges + num_edges / 2, draw, keys))
    return set_error(EH_ERR_INVALID_ARGUMENT, "R-MAT could not reach %llu distinct edges",
                     (unsigned long long)num_edges);
  HostGraph* g = new (std::nothrow) HostGraph();
  if (!g) return set_error(EH_ERR_OUT_OF_MEMORY, "host graph allocation failed");
  g->directed = true;
  g->n = n;
  g->offsets.assign(n + 1, 0);
  g->nbrs.resize(keys.size());
  for (uint64_t k : keys) g->offsets[(k >> 32) + 1]++;
  for (uint64_t i = 0; i < n; i++) g->offsets[i + 1] += g->offsets[i];
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < (int64_t)keys.size(); e++) g->nbrs[e] = (uint32_t)keys[e];
  g->ext_ids.resize(n);
  std::iota(g->ext_ids.begin(), g->ext_ids.end(), 0);
  eh::build_in_csr(*g);
  g->max_nbrhood_size = std::max(eh::max_row(g->offsets), eh::max_row(g->in_offsets));
  *out = reinterpret_cast<eh_hgraph_t>(g);
  return EH_OK;
}

}  // extern "C"
