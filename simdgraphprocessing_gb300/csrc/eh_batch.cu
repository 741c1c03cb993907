// Many graphs in one launch, CUDA-graph replay, and the work-shape autotuner.
//
// A batch is the block-diagonal union of its graphs: graph g owns rows
// [graph_rows[g], graph_rows[g+1]) and its neighbour ids are global row ids
// inside that range.  The union is one encoded matrix (rows pruned to
// nbr < node, so each graph's rows stay within its own block), counted by one
// launch of the same kernels as a single graph; each pivot adds its count to
// out[graph_of(pivot)] instead of one global sum.  The reference has no
// batching; each graph's count equals what its apps compute for that graph
// alone (apps/undirected_triangle_counting.cpp:27-65, apps/n_clique.cpp:52-101).
//
// The autotuner picks the pivot kernel's work shape -- resident CTAs per SM,
// the pivot size above which a whole CTA takes a pivot (light_max), and the
// pivot positions per CTA unit (unit_span) -- by timing the count on the
// matrix itself, coordinate by coordinate, and caches the choice per (GPU,
// layout, size bucket) in the process and optionally in a file named by the
// EH_TUNE_CACHE environment variable.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "eh_internal.h"
#include "eh_kernels.cuh"
#include "eh_matrix.cuh"

namespace eh {

struct Batch {
  Matrix* m = nullptr;
  uint32_t num_graphs = 0;
  uint32_t* d_graph_rows = nullptr;
  cudaGraphExec_t exec = nullptr;  // captured triangle + 4-clique counts
  uint64_t* exec_tri = nullptr;
  uint64_t* exec_clq = nullptr;
};

namespace {

struct Shape {
  uint32_t light_max, unit_span, ctas, core, hot, filter;
};

std::mutex g_tune_mutex;
std::map<std::string, Shape> g_tune_cache;
bool g_tune_file_loaded = false;

std::string tune_key(const Matrix* m, bool batch) {
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, m->device);
  int lc = 0, lr = 0;
  while ((1ull << (lc + 1)) <= m->tot.cardinality) lc++;
  while ((1ull << (lr + 1)) <= m->n) lr++;
  char buf[512];
  snprintf(buf, sizeof(buf), "%.200s|sm%d|layout%d|sel%d|card2^%d|rows2^%d|%s", prop.name, prop.multiProcessorCount,
           m->layout, m->selection, lc, lr, batch ? "batch" : "single");
  std::string k = buf;
  for (char& ch : k)
    if (ch == ' ') ch = '_';
  return k;
}

void load_tune_file() {
  if (g_tune_file_loaded) return;
  g_tune_file_loaded = true;
  const char* path = getenv("EH_TUNE_CACHE");
  if (!path) return;
  FILE* f = fopen(path, "r");
  if (!f) return;
  char line[1024];
  while (fgets(line, sizeof(line), f)) {  // key light_max unit_span ctas core [hot [filter]]
    char key[512];
    unsigned lm, us, ct, co, hot = 0, filt = 0;
    if (sscanf(line, "%511s %u %u %u %u %u %u", key, &lm, &us, &ct, &co, &hot, &filt) >= 5)
      g_tune_cache[key] = Shape{lm, us, ct, co, hot, filt};
  }
  fclose(f);
}

void store_tune(const std::string& key, const Shape& s) {
  g_tune_cache[key] = s;
  const char* path = getenv("EH_TUNE_CACHE");
  if (!path) return;
  FILE* f = fopen(path, "a");
  if (!f) return;
  fprintf(f, "%s %u %u %u %u %u %u\n", key.c_str(), s.light_max, s.unit_span, s.ctas, s.core, s.hot, s.filter);
  fclose(f);
}

int max_ctas_per_sm(int device) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  return std::max(1, pivot_grid(device) / std::max(1, sms));
}

eh_status apply_shape(Matrix* m, const Shape& s, cudaStream_t st) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, m->device);
  m->light_max = s.light_max;
  m->unit_span = s.unit_span;
  m->core_limit = s.core;
  m->core_hot_words = s.hot;
  m->core_filter_words = s.filter;
  m->grid = sms * (int)s.ctas;
  m->shape_set = true;
  return ensure_plan(m, st);
}

// Host time of building the current shape's own plan parts from nothing (heavy
// units, dense core, row filters), as a matrix built for a few counts pays
// them: median of 3.
eh_status time_setup(Matrix* m, cudaStream_t st, float* ms) {
  std::vector<float> t;
  for (int r = 0; r < 3; r++) {
    eh_status s = drop_shape_parts(m, st);
    if (s == EH_OK && cudaStreamSynchronize(st) != cudaSuccess) s = set_error(EH_ERR_CUDA, "plan parts free");
    if (s != EH_OK) return s;
    const auto t0 = std::chrono::steady_clock::now();
    s = ensure_plan(m, st);
    if (s == EH_OK && cudaStreamSynchronize(st) != cudaSuccess) s = set_error(EH_ERR_CUDA, "plan parts build");
    if (s != EH_OK) return s;
    t.push_back(std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count());
  }
  std::sort(t.begin(), t.end());
  *ms = t[t.size() / 2];
  return EH_OK;
}

// Median of `reps` timed triangle counts (after one warm-up) for the matrix's current shape;
// counts under 2 ms get up to 15 repetitions, so that the median of short
// counts is not decided by launch noise.
eh_status time_shape(Matrix* m, const uint32_t* graph_rows, uint32_t num_graphs, unsigned long long* out,
                     cudaStream_t st, int reps, float* ms) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  std::vector<float> t;
  eh_status s = EH_OK;
  // A matrix of full rows (EH_SELECT_ALL) is tuned on the lollipop count, the
  // other use of the same pivot kernels; pruned matrices on the triangle count.
  const bool lolli = m->selection == EH_SELECT_ALL && !graph_rows;
  for (int r = 0; r <= reps && s == EH_OK; r++) {
    cudaEventRecord(e0, st);
    s = lolli ? launch_lollipop_count(m, out, st) : launch_triangle_count(m, out, graph_rows, num_graphs, st);
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float x = 0;
    cudaEventElapsedTime(&x, e0, e1);
    if (r > 0) t.push_back(x);
    if (r == 1 && x < 2.0f) reps = std::max(reps, 15);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (s != EH_OK) return s;
  std::sort(t.begin(), t.end());
  *ms = t[t.size() / 2];
  return EH_OK;
}

// per_build = 0 ranks shapes by the count's time alone (a matrix counted many
// times); per_build = k by the count's time plus the shape's one-shot plan
// cost (time_setup) / k (a matrix built for k counts).
eh_status tune(Matrix* m, const uint32_t* graph_rows, uint32_t num_graphs, cudaStream_t st, eh_tuning* res,
               uint32_t per_build) {
  // The first plan build looks up the shape cache itself (apply_cached_shape), so
  // it runs before this function takes the cache lock.
  eh_status s = ensure_plan(m, st);
  if (s != EH_OK) return s;
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  load_tune_file();
  std::string key = tune_key(m, graph_rows != nullptr);
  if (per_build) key += "|per_build" + std::to_string(per_build);
  unsigned long long* out = nullptr;
  const size_t outn = graph_rows ? num_graphs : 1;
  if (pool_alloc((void**)&out, outn * sizeof(unsigned long long), st) != cudaSuccess)
    return set_error(EH_ERR_OUT_OF_MEMORY, "tuner output allocation failed");
  auto it = g_tune_cache.find(key);
  Shape best{m->light_max, m->unit_span, (uint32_t)max_ctas_per_sm(m->device), m->core_limit, m->core_hot_words,
             m->core_filter_words};
  float best_ms = 0, best_score = 0;
  uint32_t tried = 0;
  // Count time of the current shape, and its rank (count time plus the
  // amortised one-shot plan cost when per_build is set).
  auto measure = [&](float* ms, float* score) {
    s = time_shape(m, graph_rows, num_graphs, out, st, 3, ms);
    *score = *ms;
    float setup = 0;
    if (s == EH_OK && per_build && (s = time_setup(m, st, &setup)) == EH_OK) *score += setup / (float)per_build;
  };
  if (it != g_tune_cache.end()) {
    best = it->second;
    s = apply_shape(m, best, st);
    if (s == EH_OK) s = time_shape(m, graph_rows, num_graphs, out, st, 3, &best_ms);
    tried = 1;
  } else {
    const int cmax = max_ctas_per_sm(m->device);
    s = apply_shape(m, best, st);
    if (s == EH_OK) measure(&best_ms, &best_score);
    tried = 1;
    auto consider = [&](Shape c) {
      if (s != EH_OK) return;
      s = apply_shape(m, c, st);
      float ms = 0, score = 0;
      if (s == EH_OK) measure(&ms, &score);
      tried++;
      if (s == EH_OK && score < best_score) {
        best_ms = ms;
        best_score = score;
        best = c;
      }
    };
    const Shape start = best;
    // Core size and filters together: a filter makes a larger core pay.
    for (uint32_t co : {0u, 16384u, 32768u, 65536u, 98304u, 131072u, 196608u, 262144u})
      for (uint32_t fw : {0u, 32u})
        if ((co != start.core || fw != start.filter) && co <= kCoreMaxK && (fw == 0 || co > kFilterLo))
          consider(Shape{start.light_max, start.unit_span, start.ctas, co, start.hot, fw});
    const Shape after_core0 = best;
    if (after_core0.core)
      for (uint32_t hot : {0u, 32u, 64u, 128u})
        if (hot != after_core0.hot)
          consider(Shape{after_core0.light_max, after_core0.unit_span, after_core0.ctas, after_core0.core, hot,
                         after_core0.filter});
    const Shape after_hot = best;
    if (after_hot.core > kFilterLo)
      for (uint32_t fw : {0u, 16u, 32u, 64u})
        if (fw != after_hot.filter)
          consider(Shape{after_hot.light_max, after_hot.unit_span, after_hot.ctas, after_hot.core, after_hot.hot, fw});
    const Shape after_core = best;
    for (int c = 1; c <= cmax; c++)
      if ((uint32_t)c != after_core.ctas)
        consider(Shape{after_core.light_max, after_core.unit_span, (uint32_t)c, after_core.core, after_core.hot,
                         after_core.filter});
    const Shape after_ctas = best;
    for (uint32_t lm : {32u, 64u, 96u, 128u, 160u})
      if (lm != after_ctas.light_max && lm <= kLightMax)
        consider(Shape{lm, after_ctas.unit_span, after_ctas.ctas, after_ctas.core, after_ctas.hot, after_ctas.filter});
    const Shape after_lm = best;
    for (uint32_t us : {32u, 128u, 256u, 512u, 1024u, 2048u})
      if (us != after_lm.unit_span) consider(Shape{after_lm.light_max, us, after_lm.ctas, after_lm.core, after_lm.hot, after_lm.filter});
    if (s == EH_OK) {
      s = apply_shape(m, best, st);
      store_tune(key, best);
    }
  }
  cudaFreeAsync(out, st);
  if (s != EH_OK) return s;
  if (res) {
    res->light_max = best.light_max;
    res->unit_span = best.unit_span;
    res->ctas_per_sm = best.ctas;
    res->core_rows = best.core;
    res->ms = best_ms;
    res->configs_tried = tried;
    res->core_hot_words = best.hot;
    res->core_filter_words = best.filter;
  }
  return EH_OK;
}

}  // namespace

// Applies a cached tuned shape for this matrix's size class, if one exists.
// Called when a matrix's plan is first built (before the plan's units exist).
void apply_cached_shape(Matrix* m) {
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  load_tune_file();
  auto it = g_tune_cache.find(tune_key(m, m->is_batch));
  if (it == g_tune_cache.end()) return;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, m->device);
  m->light_max = it->second.light_max;
  m->unit_span = it->second.unit_span;
  m->core_limit = it->second.core;
  m->core_hot_words = it->second.hot;
  m->core_filter_words = it->second.filter;
  m->grid = sms * (int)it->second.ctas;
}

}  // namespace eh

using eh::Batch;
using eh::set_error;

extern "C" {

eh_status eh_matrix_tune(eh_matrix_t mh, void* stream, eh_tuning* result) {
  if (!mh) return set_error(EH_ERR_INVALID_ARGUMENT, "matrix is NULL");
  eh::Matrix* m = reinterpret_cast<eh::Matrix*>(mh);
  cudaSetDevice(m->device);
  if (m->selection == EH_SELECT_MASK)
    return set_error(EH_ERR_UNSUPPORTED,
                     "tuning times the triangle count (EH_SELECT_LOWER) or the lollipop count (EH_SELECT_ALL)");
  return eh::tune(m, nullptr, 0, reinterpret_cast<cudaStream_t>(stream), result, 0);
}

eh_status eh_matrix_tune_for(eh_matrix_t mh, uint32_t counts_per_build, void* stream, eh_tuning* result) {
  if (!mh) return set_error(EH_ERR_INVALID_ARGUMENT, "matrix is NULL");
  eh::Matrix* m = reinterpret_cast<eh::Matrix*>(mh);
  cudaSetDevice(m->device);
  if (m->selection == EH_SELECT_MASK)
    return set_error(EH_ERR_UNSUPPORTED,
                     "tuning times the triangle count (EH_SELECT_LOWER) or the lollipop count (EH_SELECT_ALL)");
  return eh::tune(m, nullptr, 0, reinterpret_cast<cudaStream_t>(stream), result, counts_per_build);
}

eh_status eh_matrix_set_shape(eh_matrix_t mh, const eh_tuning* shape, void* stream) {
  EH_CHECK_ARG(mh && shape, "NULL argument");
  eh::Matrix* m = reinterpret_cast<eh::Matrix*>(mh);
  cudaSetDevice(m->device);
  EH_CHECK_ARG(shape->light_max >= 2 && shape->light_max <= eh::kLightMax, "light_max %u outside [2, %u]",
               shape->light_max, eh::kLightMax);
  EH_CHECK_ARG(shape->unit_span >= 1 && shape->unit_span <= 65536, "unit_span %u outside [1, 65536]",
               shape->unit_span);
  EH_CHECK_ARG(shape->ctas_per_sm >= 1 && (int)shape->ctas_per_sm <= eh::max_ctas_per_sm(m->device),
               "ctas_per_sm %u outside [1, %d]", shape->ctas_per_sm, eh::max_ctas_per_sm(m->device));
  EH_CHECK_ARG(shape->core_rows <= eh::kCoreMaxK, "core_rows %u above %u", shape->core_rows, eh::kCoreMaxK);
  const uint32_t fw = shape->core_filter_words;
  EH_CHECK_ARG(fw == 0 || fw == 16 || fw == 32 || fw == 64, "core_filter_words %u is not 0, 16, 32 or 64", fw);
  const eh::Shape s{shape->light_max, shape->unit_span, shape->ctas_per_sm, shape->core_rows, shape->core_hot_words,
                    fw};
  return eh::apply_shape(m, s, reinterpret_cast<cudaStream_t>(stream));
}

eh_status eh_batch_build(uint32_t num_graphs, const uint64_t* graph_rows, uint64_t n, const uint64_t* offsets,
                         const uint32_t* nbrs, eh_layout layout, void* stream, eh_batch_t* out) {
  EH_CHECK_ARG(out, "out is NULL");
  EH_CHECK_ARG(num_graphs > 0 && graph_rows, "a batch needs at least one graph");
  EH_CHECK_ARG(offsets, "offsets is NULL");
  EH_CHECK_ARG(n < (1ull << 32), "n=%llu exceeds the u32 vertex id space", (unsigned long long)n);
  EH_CHECK_ARG(graph_rows[0] == 0 && graph_rows[num_graphs] == n, "graph_rows must run from 0 to n");
  for (uint32_t g = 0; g < num_graphs; g++)
    EH_CHECK_ARG(graph_rows[g + 1] >= graph_rows[g], "graph_rows not ascending at graph %u", g);
  // Every edge must stay inside its graph's block of rows.
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 8) reduction(| : bad)
  for (int64_t g = 0; g < (int64_t)num_graphs; g++) {
    const uint64_t lo = graph_rows[g], hi = graph_rows[g + 1];
    for (uint64_t r = lo; r < hi && !bad; r++)
      for (uint64_t e = offsets[r]; e < offsets[r + 1]; e++)
        if (nbrs[e] < lo || nbrs[e] >= hi) {
          bad = 1;
          break;
        }
  }
  EH_CHECK_ARG(!bad, "an edge leaves its graph's block of rows");
  eh_matrix_t mh = nullptr;
  eh_status s = eh_matrix_build(n, offsets, nbrs, nullptr, EH_SELECT_LOWER, layout, stream, &mh);
  if (s != EH_OK) return s;
  Batch* b = new Batch();
  b->m = reinterpret_cast<eh::Matrix*>(mh);
  b->m->is_batch = true;
  b->num_graphs = num_graphs;
  std::vector<uint32_t> gr(num_graphs + 1);
  for (uint32_t g = 0; g <= num_graphs; g++) gr[g] = (uint32_t)graph_rows[g];
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (eh::pool_alloc((void**)&b->d_graph_rows, gr.size() * 4, st) != cudaSuccess) {
    eh_matrix_free(mh);
    delete b;
    return set_error(EH_ERR_OUT_OF_MEMORY, "batch allocation failed");
  }
  if (cudaMemcpyAsync(b->d_graph_rows, gr.data(), gr.size() * 4, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    eh_batch_free(reinterpret_cast<eh_batch_t>(b));
    return set_error(EH_ERR_CUDA, "batch graph boundaries upload failed");
  }
  s = eh::ensure_plan(b->m, st);
  if (s != EH_OK) {
    eh_batch_free(reinterpret_cast<eh_batch_t>(b));
    return s;
  }
  *out = reinterpret_cast<eh_batch_t>(b);
  return EH_OK;
}

eh_status eh_batch_matrix(eh_batch_t bh, eh_matrix_t* m) {
  EH_CHECK_ARG(bh && m, "NULL argument");
  *m = reinterpret_cast<eh_matrix_t>(reinterpret_cast<Batch*>(bh)->m);
  return EH_OK;
}

eh_status eh_batch_count(eh_batch_t bh, uint32_t k, uint64_t* d_counts, void* stream) {
  EH_CHECK_ARG(bh && d_counts, "NULL argument");
  Batch* b = reinterpret_cast<Batch*>(bh);
  cudaSetDevice(b->m->device);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  unsigned long long* out = reinterpret_cast<unsigned long long*>(d_counts);
  if (k == 3) return eh::launch_triangle_count(b->m, out, b->d_graph_rows, b->num_graphs, st);
  return eh::launch_cliques(b->m, k, out, b->d_graph_rows, b->num_graphs, st);
}

eh_status eh_batch_run(eh_batch_t bh, uint64_t* d_triangles, uint64_t* d_cliques4, int use_graph, void* stream) {
  EH_CHECK_ARG(bh && d_triangles && d_cliques4, "NULL argument");
  Batch* b = reinterpret_cast<Batch*>(bh);
  cudaSetDevice(b->m->device);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (!use_graph) {
    eh_status s = eh_batch_count(bh, 3, d_triangles, stream);
    return s != EH_OK ? s : eh_batch_count(bh, 4, d_cliques4, stream);
  }
  EH_CHECK_ARG(st != nullptr, "CUDA-graph replay needs a non-default stream");
  if (!b->exec || b->exec_tri != d_triangles || b->exec_clq != d_cliques4) {
    if (b->exec) {
      cudaGraphExecDestroy(b->exec);
      b->exec = nullptr;
    }
    // One direct run first: it builds the plan and any clique scratch, which
    // allocate and so cannot happen while the stream is being captured.
    eh_status s = eh_batch_run(bh, d_triangles, d_cliques4, 0, stream);
    if (s != EH_OK) return s;
    if (cudaStreamSynchronize(st) != cudaSuccess) return set_error(EH_ERR_CUDA, "batch warm-up failed");
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return set_error(EH_ERR_CUDA, "stream capture: %s", cudaGetErrorString(e));
    eh_status s1 = eh_batch_count(bh, 3, d_triangles, stream);
    eh_status s2 = s1 == EH_OK ? eh_batch_count(bh, 4, d_cliques4, stream) : s1;
    e = cudaStreamEndCapture(st, &g);
    if (s2 != EH_OK) {
      if (g) cudaGraphDestroy(g);
      return s2;
    }
    if (e != cudaSuccess) return set_error(EH_ERR_CUDA, "stream capture: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&b->exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return set_error(EH_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    b->exec_tri = d_triangles;
    b->exec_clq = d_cliques4;
  }
  const cudaError_t e = cudaGraphLaunch(b->exec, st);
  eh::note_use(b->m, st);
  return e == cudaSuccess ? EH_OK : set_error(EH_ERR_CUDA, "graph launch: %s", cudaGetErrorString(e));
}

eh_status eh_batch_tune(eh_batch_t bh, void* stream, eh_tuning* result) {
  EH_CHECK_ARG(bh, "batch is NULL");
  Batch* b = reinterpret_cast<Batch*>(bh);
  cudaSetDevice(b->m->device);
  if (b->exec) {  // the captured graph holds the old launch shape
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  return eh::tune(b->m, b->d_graph_rows, b->num_graphs, reinterpret_cast<cudaStream_t>(stream), result, 0);
}

void eh_batch_free(eh_batch_t bh) {
  Batch* b = reinterpret_cast<Batch*>(bh);
  if (!b) return;
  cudaSetDevice(b->m->device);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  // The graph boundaries go back to the pool once the matrix's recorded
  // launches are done (they read them), like the matrix's own buffers.
  cudaStream_t st = nullptr;
  if (b->d_graph_rows) {
    if (eh::upload_stream(&st) == cudaSuccess && eh::wait_uses(b->m, st) == cudaSuccess) {
      cudaFreeAsync(b->d_graph_rows, st);
    } else {
      cudaDeviceSynchronize();
      cudaFreeAsync(b->d_graph_rows, nullptr);
    }
  }
  eh_matrix_free(reinterpret_cast<eh_matrix_t>(b->m));
  delete b;
}

}  // extern "C"
