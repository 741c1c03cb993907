// C ABI over the device matrix: build orchestration, lazily built work plans,
// pattern counts, and host views of rows in the reference's flattened format.
#include <cstdint>
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include <cuda_runtime.h>

#include "eh_internal.h"
#include "eh_kernels.cuh"
#include "eh_matrix.cuh"

namespace eh {

static eh_status cuda_fail(cudaError_t e, const char* what) {
  return set_error(EH_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}
#define CU(call, what)                         \
  do {                                         \
    cudaError_t _e = (call);                   \
    if (_e != cudaSuccess) return eh::cuda_fail(_e, what); \
  } while (0)

static bool valid_layout(int l) { return l == 0 || l == 1 || l == 2 || l == 5 || l == 16; }
static bool is_hybrid(int l) { return l == 5 || l == 16; }

// Reference flattened byte count of a row (hybrid.hpp:132-166 and the inner
// build_flattened of each layout).
static uint64_t flattened_bytes(int layout, const RowDesc& d) {
  const uint32_t type = desc_type(d), len = desc_len(d);
  uint64_t inner;
  if (type == TY_UINT) inner = 4ull * d.card;
  else if (type == TY_BITSET) inner = d.card ? 4 + 8 + 8ull * len : 0;
  else inner = d.card ? 4 + 2ull * len : 0;
  return inner + (is_hybrid(layout) ? 8 : 0);
}

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_device_mu;
cudaMemPool_t g_pool[kMaxDevices][2] = {};
cudaStream_t g_upload_stream[kMaxDevices] = {};
}  // namespace

cudaError_t pool_alloc(void** p, size_t bytes, cudaStream_t st, PoolKind kind) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  cudaMemPool_t pool;
  {
    std::lock_guard<std::mutex> g(g_device_mu);
    if (!g_pool[dev][kind]) {
      cudaMemPoolProps props = {};
      props.allocType = cudaMemAllocationTypePinned;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = dev;
      cudaMemPool_t created = nullptr;
      if ((e = cudaMemPoolCreate(&created, &props)) != cudaSuccess) return e;
      uint64_t keep = kPoolKeep;
      if ((e = cudaMemPoolSetAttribute(created, cudaMemPoolAttrReleaseThreshold, &keep)) != cudaSuccess) {
        cudaMemPoolDestroy(created);
        return e;
      }
      g_pool[dev][kind] = created;
    }
    pool = g_pool[dev][kind];
  }
  return cudaMallocFromPoolAsync(p, bytes, pool, st);
}

cudaError_t upload_stream(cudaStream_t* out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> g(g_device_mu);
  if (!g_upload_stream[dev] &&
      (e = cudaStreamCreateWithFlags(&g_upload_stream[dev], cudaStreamNonBlocking)) != cudaSuccess) {
    g_upload_stream[dev] = nullptr;
    return e;
  }
  *out = g_upload_stream[dev];
  return cudaSuccess;
}

void note_use(Matrix* m, cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return;
  std::lock_guard<std::mutex> g(m->uses_mu);
  cudaEvent_t ev = nullptr;
  for (auto& u : m->uses)
    if (u.first == st) ev = u.second;
  if (!ev) {
    if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) return;
    m->uses.emplace_back(st, ev);
  }
  cudaEventRecord(ev, st);
}

cudaError_t wait_uses(Matrix* m, cudaStream_t st) {
  std::lock_guard<std::mutex> g(m->uses_mu);
  for (auto& u : m->uses) {
    if (u.first == st) continue;  // stream order covers it
    const cudaError_t e = cudaStreamWaitEvent(st, u.second, 0);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

eh_status build_device(uint64_t n, const uint64_t* d_off, const uint32_t* d_nbr, const uint8_t* d_mask,
                       int sel, int layout, cudaStream_t st, Matrix** out, uint64_t total, const UploadChunks* up) {
  EH_CHECK_ARG(out != nullptr, "out is NULL");
  EH_CHECK_ARG(valid_layout(layout), "unknown layout %d", layout);
  EH_CHECK_ARG(sel >= 0 && sel <= 2, "unknown selection %d", sel);
  EH_CHECK_ARG(sel != EH_SELECT_MASK || d_mask != nullptr || n == 0, "EH_SELECT_MASK needs an edge mask");
  EH_CHECK_ARG(n < (1ull << 32), "n=%llu exceeds the u32 vertex id space", (unsigned long long)n);
  EH_CHECK_ARG(n == 0 || (d_off != nullptr), "offsets is NULL");
  if (n && total == kTotalUnknown) {  // the neighbour array's length is offsets[n], on the device
    cudaError_t ce = cudaMemcpyAsync(&total, d_off + n, sizeof(uint64_t), cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) return set_error(EH_ERR_CUDA, "offsets read: %s", cudaGetErrorString(ce));
  }
  EH_CHECK_ARG(n == 0 || total == 0 || d_nbr != nullptr, "nbrs is NULL");
  Matrix* m = new Matrix();
  m->n = n;
  m->layout = layout;
  m->selection = sel;
  cudaGetDevice(&m->device);
  RowMeasure* meas = nullptr;
  BuildTotals* tot = nullptr;
  uint32_t* err = nullptr;
  uint32_t* off16 = nullptr;
  uint32_t* tmp = nullptr;
  // big: rows over 4,096 entries (big_cap slots), their count n_big, then
  // n_big as it stood after each uploaded chunk of rows (mark[0] = 0), so that
  // each chunk's long rows are measured right after it.
  uint32_t* big = nullptr;
  const uint64_t big_cap = big_row_capacity(n, total);
  const uint64_t n_marks = (up ? up->ready.size() : 0) + 1;
  auto cleanup = [&]() {
    cudaFreeAsync(meas, st);
    cudaFreeAsync(tot, st);
    cudaFreeAsync(err, st);
    cudaFreeAsync(off16, st);
    cudaFreeAsync(tmp, st);
    cudaFreeAsync(big, st);
  };
  auto fail = [&](eh_status s) {
    cleanup();
    cudaFreeAsync(m->desc, st);
    cudaFreeAsync(m->arena, st);
    cudaFreeAsync(m->counters, st);
    cudaStreamSynchronize(st);
    delete m;
    return s;
  };
  cudaError_t e;
  const uint64_t nn = n ? n : 1;
  if ((e = pool_alloc((void**)&meas, nn * sizeof(RowMeasure), st)) != cudaSuccess ||
      (e = pool_alloc((void**)&tot, sizeof(BuildTotals), st)) != cudaSuccess ||
      (e = pool_alloc((void**)&err, sizeof(uint32_t), st)) != cudaSuccess ||
      (e = pool_alloc((void**)&off16, nn * sizeof(uint32_t), st)) != cudaSuccess ||
      (e = pool_alloc((void**)&tmp, scan_tmp_words(nn) * sizeof(uint32_t), st)) != cudaSuccess ||
      (e = pool_alloc((void**)&big, (big_cap + 1 + n_marks) * sizeof(uint32_t), st)) != cudaSuccess)
    return fail(e == cudaErrorMemoryAllocation ? set_error(EH_ERR_OUT_OF_MEMORY, "build scratch allocation failed")
                                               : cuda_fail(e, "cudaMallocAsync"));
  cudaMemsetAsync(tot, 0, sizeof(BuildTotals), st);
  cudaMemsetAsync(err, 0, sizeof(uint32_t), st);
  uint32_t* n_big = big + big_cap;
  uint32_t* mark = n_big + 1;
  cudaMemsetAsync(n_big, 0, 2 * sizeof(uint32_t), st);  // n_big, mark[0]
  if (up) {
    for (size_t c = 0; c < up->ready.size(); c++) {
      if ((e = cudaStreamWaitEvent(st, up->ready[c], 0)) != cudaSuccess) return fail(cuda_fail(e, "upload wait"));
      if ((e = launch_measure_rows(n, total, up->rows[c], up->rows[c + 1], d_off, d_nbr, d_mask, sel, layout, meas,
                                   tot, err, big, n_big, st)) != cudaSuccess ||
          (e = cudaMemcpyAsync(mark + c + 1, n_big, sizeof(uint32_t), cudaMemcpyDeviceToDevice, st)) != cudaSuccess ||
          (e = launch_measure_big(n, d_off, d_nbr, d_mask, sel, layout, meas, tot, err, big, mark + c, mark + c + 1,
                                  st)) != cudaSuccess)
        return fail(cuda_fail(e, "measure kernel"));
    }
  } else if ((e = launch_measure_rows(n, total, 0, n, d_off, d_nbr, d_mask, sel, layout, meas, tot, err, big, n_big,
                                      st)) != cudaSuccess ||
             (e = launch_measure_big(n, d_off, d_nbr, d_mask, sel, layout, meas, tot, err, big, mark, n_big, st)) !=
                 cudaSuccess) {
    return fail(cuda_fail(e, "measure kernel"));
  }
  uint32_t herr = 0;
  cudaMemcpyAsync(&m->tot, tot, sizeof(BuildTotals), cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(&herr, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail(cuda_fail(e, "measure"));
  if (herr) {
    return fail(set_error(EH_ERR_INVALID_ARGUMENT, "adjacency rejected:%s%s%s%s",
                          (herr & ERRF_OFFSETS) ? " offsets fall or run past offsets[n];" : "",
                          (herr & ERRF_UNSORTED) ? " a row is not strictly ascending;" : "",
                          (herr & ERRF_RANGE) ? " a neighbour id is >= n;" : "",
                          (herr & ERRF_ROW_TOO_LONG) ? " a row has >= 2^28 selected entries;" : ""));
  }
  if (m->tot.payload_units >= (1ull << 32))
    return fail(set_error(EH_ERR_UNSUPPORTED, "encoded matrix exceeds 64 GiB"));
  if ((e = launch_scan_units(n, meas, off16, tmp, scan_tmp_words(nn), st)) != cudaSuccess)
    return fail(cuda_fail(e, "scan"));
  m->arena_units = m->tot.payload_units;
  if ((e = pool_alloc((void**)&m->desc, nn * sizeof(RowDesc), st)) != cudaSuccess ||
      (e = pool_alloc((void**)&m->arena, (m->arena_units + 1) * 16, st)) != cudaSuccess ||
      (e = pool_alloc((void**)&m->counters, 128, st)) != cudaSuccess)
    return fail(set_error(EH_ERR_OUT_OF_MEMORY, "matrix allocation (%llu bytes) failed: %s",
                          (unsigned long long)((m->arena_units + 1) * 16 + nn * 16), cudaGetErrorString(e)));
  // Words 0..15: work-queue counters; 16..17: the u64 result of the synchronous calls.
  m->result = reinterpret_cast<unsigned long long*>(m->counters + 16);
  m->device_bytes = nn * sizeof(RowDesc) + (m->arena_units + 1) * 16 + 128;
  cudaMemsetAsync(m->counters, 0, 128, st);
  cudaMemsetAsync(m->arena, 0, (m->arena_units + 1) * 16, st);
  if ((e = launch_encode(n, d_off, d_nbr, d_mask, sel, meas, off16, m->desc, m->arena, big, big + big_cap, st)) !=
      cudaSuccess)
    return fail(cuda_fail(e, "encode kernel"));
  cleanup();
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) {
    cudaFreeAsync(m->desc, st);
    cudaFreeAsync(m->arena, st);
    cudaFreeAsync(m->counters, st);
    delete m;
    return cuda_fail(e, "encode");
  }
  m->grid = pivot_grid(m->device);
  *out = m;
  return EH_OK;
}

// (Re)builds the heavy-unit list of the plan for (light_max, unit_span).
eh_status ensure_units(Matrix* m, uint32_t light_max, uint32_t unit_span, cudaStream_t st) {
  Plan& p = m->plan;
  if (p.units && p.light_max == light_max && p.unit_span == unit_span) return EH_OK;
  const uint32_t n_heavy = p.above(light_max);
  uint32_t* cnt = nullptr;
  uint32_t* start = nullptr;
  uint32_t* tmp = nullptr;
  const uint32_t nh = n_heavy ? n_heavy : 1;
  CU(pool_alloc((void**)&cnt, nh * sizeof(uint32_t), st), "unit scratch");
  CU(pool_alloc((void**)&start, nh * sizeof(uint32_t), st), "unit scratch");
  CU(pool_alloc((void**)&tmp, scan_tmp_words(nh) * sizeof(uint32_t), st), "unit scratch");
  CU(launch_pivot_units(m->desc, p.order, n_heavy, unit_span, cnt, st), "unit count");
  uint32_t n_units = 0;
  if (n_heavy) {
    CU(exclusive_scan_u32(cnt, n_heavy, start, tmp, st), "unit scan");
    uint32_t last_start = 0, last_cnt = 0;
    CU(cudaMemcpyAsync(&last_start, start + n_heavy - 1, 4, cudaMemcpyDeviceToHost, st), "unit copy");
    CU(cudaMemcpyAsync(&last_cnt, cnt + n_heavy - 1, 4, cudaMemcpyDeviceToHost, st), "unit copy");
    CU(cudaStreamSynchronize(st), "units");
    n_units = last_start + last_cnt;
  }
  if (!p.units || p.units_cap < (uint64_t)n_units) {
    if (p.units) {  // launches on other streams may still read them
      CU(wait_uses(m, st), "units");
      CU(cudaFreeAsync(p.units, st), "units");
      m->device_bytes -= p.units_cap * sizeof(uint2);
    }
    p.units_cap = n_units ? n_units : 1;
    CU(pool_alloc((void**)&p.units, p.units_cap * sizeof(uint2), st), "unit allocation");
    m->device_bytes += p.units_cap * sizeof(uint2);
  }
  CU(launch_pivot_unit_fill(cnt, start, n_heavy, p.units, st), "unit fill");
  cudaFreeAsync(cnt, st);
  cudaFreeAsync(start, st);
  cudaFreeAsync(tmp, st);
  CU(cudaStreamSynchronize(st), "unit build");
  p.n_heavy = n_heavy;
  p.n_units = n_units;
  p.light_max = light_max;
  p.unit_span = unit_span;
  return EH_OK;
}

// Dense core of the first min(n, core_limit) rows (rounded down to a multiple of
// 64); small graphs (under 4,096 rows) go without.
eh_status ensure_core(Matrix* m, cudaStream_t st) {
  Plan& p = m->plan;
  uint32_t want = (uint32_t)std::min<uint64_t>(m->n, m->core_limit) & ~63u;
  if (m->n < 4096) want = 0;
  // Row filters cover the core's rows from kFilterLo on.
  const uint32_t want_fw = (m->core_filter_words && want > kFilterLo) ? m->core_filter_words : 0u;
  const uint32_t want_fk = want_fw ? want : 0u;
  if (want == p.core_k && (want == 0 || p.core) && want_fw == p.filter_words && want_fk == p.filter_k)
    return EH_OK;
  if (p.core || p.filter) CU(wait_uses(m, st), "core");  // launches on other streams may still read them
  if (p.filter) {
    CU(cudaFreeAsync(p.filter, st), "row filters");
    m->device_bytes -= (uint64_t)(p.filter_k - kFilterLo) * p.filter_words * 8;
    p.filter = nullptr;
    p.filter_words = 0;
    p.filter_k = 0;
  }
  if (p.core && want != p.core_k) {
    CU(cudaFreeAsync(p.core, st), "core");
    m->device_bytes -= core_row_offset(p.core_k) * 8;
    p.core = nullptr;
    p.core_k = 0;
  }
  if (want && !p.core) {
    const uint64_t words = core_row_offset(want);
    CU(pool_alloc((void**)&p.core, words * 8, st, kPoolCore), "core allocation");
    m->device_bytes += words * 8;
    CU(launch_core_build(m->desc, m->arena, want, p.core, st), "core build");
    p.core_k = want;
  }
  if (want_fw) {
    const uint64_t fwords = (uint64_t)(want_fk - kFilterLo) * want_fw;
    CU(pool_alloc((void**)&p.filter, fwords * 8, st, kPoolCore), "row filter allocation");
    m->device_bytes += fwords * 8;
    CU(launch_filter_build(m->desc, m->arena, want_fk, want_fw, p.filter, st), "row filter build");
    p.filter_words = want_fw;
    p.filter_k = want_fk;
  }
  CU(cudaStreamSynchronize(st), "core build");
  return EH_OK;
}

eh_status drop_shape_parts(Matrix* m, cudaStream_t st) {
  Plan& p = m->plan;
  if (!p.units && !p.core && !p.filter) return EH_OK;
  CU(wait_uses(m, st), "plan parts");  // launches on other streams may still read them
  if (p.units) {
    CU(cudaFreeAsync(p.units, st), "units");
    m->device_bytes -= p.units_cap * sizeof(uint2);
    p.units = nullptr;
    p.units_cap = 0;
    p.n_units = 0;
  }
  if (p.filter) {
    CU(cudaFreeAsync(p.filter, st), "row filters");
    m->device_bytes -= (uint64_t)(p.filter_k - kFilterLo) * p.filter_words * 8;
    p.filter = nullptr;
    p.filter_words = 0;
    p.filter_k = 0;
  }
  if (p.core) {
    CU(cudaFreeAsync(p.core, st), "core");
    m->device_bytes -= core_row_offset(p.core_k) * 8;
    p.core = nullptr;
    p.core_k = 0;
  }
  return EH_OK;
}

// Row order (descending card) and decoded copies of the giant non-uint pivots,
// then the heavy units for the matrix's current work shape.
eh_status ensure_plan(Matrix* m, cudaStream_t st) {
  Plan& p = m->plan;
  if (!p.ready) {
    if (!m->shape_set) apply_cached_shape(m);
    uint32_t* hist = nullptr;
    uint32_t* cursor = nullptr;
    const uint64_t nn = m->n ? m->n : 1;
    CU(pool_alloc((void**)&p.order, nn * sizeof(uint32_t), st), "plan order allocation");
    m->device_bytes += nn * sizeof(uint32_t);
    CU(pool_alloc((void**)&hist, (65536 + scan_tmp_words(65536)) * sizeof(uint32_t), st), "plan scratch");
    CU(pool_alloc((void**)&cursor, 65536 * sizeof(uint32_t), st), "plan scratch");
    CU(launch_plan(m->n, m->desc, 2, hist, p.order, cursor, st), "plan kernels");
    std::vector<uint32_t> starts(65536);
    uint32_t total = 0;
    CU(cudaMemcpyAsync(starts.data(), hist, 65536 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st), "plan copy");
    CU(cudaMemcpyAsync(&total, cursor + 65535, sizeof(uint32_t), cudaMemcpyDeviceToHost, st), "plan copy");
    CU(cudaStreamSynchronize(st), "plan");
    cudaFreeAsync(hist, st);
    cudaFreeAsync(cursor, st);
    p.n_order = m->n ? total : 0;
    if (m->n) p.starts = starts;
    p.n_giant = p.above(kCtaListCap);
    // Giant pivots that are not uint rows get a decoded list.
    std::vector<uint32_t> grows(p.n_giant);
    std::vector<unsigned long long> goff(p.n_giant ? p.n_giant : 1, 0);
    uint64_t gtotal = 0;
    std::vector<uint32_t> dec_rows;
    std::vector<unsigned long long> dec_off;
    if (p.n_giant) {
      // The giant rows' ids and descriptors come back in one synchronisation:
      // a gather kernel collects their descriptors next to each other first.
      std::vector<RowDesc> gdesc(p.n_giant);
      RowDesc* d_gdesc = nullptr;
      CU(pool_alloc((void**)&d_gdesc, p.n_giant * sizeof(RowDesc), st), "giant scratch");
      CU(launch_gather_desc(m->desc, p.order, p.n_giant, d_gdesc, st), "giant gather");
      CU(cudaMemcpyAsync(grows.data(), p.order, p.n_giant * sizeof(uint32_t), cudaMemcpyDeviceToHost, st),
         "giant copy");
      CU(cudaMemcpyAsync(gdesc.data(), d_gdesc, p.n_giant * sizeof(RowDesc), cudaMemcpyDeviceToHost, st),
         "giant desc");
      cudaFreeAsync(d_gdesc, st);
      CU(cudaStreamSynchronize(st), "giant");
      for (uint32_t u = 0; u < p.n_giant; u++) {
        const RowDesc& d = gdesc[u];
        if (desc_type(d) != TY_UINT) {
          goff[u] = gtotal;
          dec_rows.push_back(grows[u]);
          dec_off.push_back(gtotal);
          gtotal += d.card;
        }
      }
    }
    CU(pool_alloc((void**)&p.giant_off, goff.size() * sizeof(unsigned long long), st), "giant allocation");
    CU(pool_alloc((void**)&p.giant_lists, (gtotal ? gtotal : 1) * sizeof(uint32_t), st), "giant allocation");
    m->device_bytes += goff.size() * 8 + (gtotal ? gtotal : 1) * 4;
    CU(cudaMemcpyAsync(p.giant_off, goff.data(), goff.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice,
                       st),
       "giant copy");
    if (!dec_rows.empty()) {
      uint32_t* d_rows = nullptr;
      unsigned long long* d_off = nullptr;
      CU(pool_alloc((void**)&d_rows, dec_rows.size() * 4, st), "giant scratch");
      CU(pool_alloc((void**)&d_off, dec_off.size() * 8, st), "giant scratch");
      CU(cudaMemcpyAsync(d_rows, dec_rows.data(), dec_rows.size() * 4, cudaMemcpyHostToDevice, st), "giant copy");
      CU(cudaMemcpyAsync(d_off, dec_off.data(), dec_off.size() * 8, cudaMemcpyHostToDevice, st), "giant copy");
      CU(launch_decode_rows(m->desc, m->arena, d_rows, d_off, (uint32_t)dec_rows.size(), p.giant_lists, st),
         "giant decode");
      cudaFreeAsync(d_rows, st);
      cudaFreeAsync(d_off, st);
    }
    CU(cudaStreamSynchronize(st), "plan build");
    p.ready = true;
  }
  eh_status s = ensure_core(m, st);
  if (s != EH_OK) return s;
  return ensure_units(m, m->light_max, m->unit_span, st);
}

PivotArgs pivot_args(Matrix* m, unsigned long long* out) {
  PivotArgs a;
  a.desc = m->desc;
  a.arena = m->arena;
  a.order = m->plan.order;
  a.n_order = m->plan.n_order;
  a.n_heavy = m->plan.n_heavy;
  a.n_giant = m->plan.n_giant;
  a.giant_lists = m->plan.giant_lists;
  a.giant_off = m->plan.giant_off;
  a.counters = m->counters;
  a.out = out;
  a.unit_span = m->plan.unit_span;
  a.graph_rows = nullptr;
  a.num_graphs = 0;
  a.core = m->plan.core;
  a.core_k = m->plan.core_k;
  a.core_hot_words = m->core_hot_words;
  a.filter = m->plan.filter;
  a.filter_words = m->plan.filter_words;
  a.filter_k = m->plan.filter_k;
  return a;
}

// Copies the result back and checks the kernels' device error flags
// (counters[15]; e.g. a bulk copy whose bounded wait ran out), which are
// cleared when reported.
static eh_status finish_sync(Matrix* m, unsigned long long* d_res, uint64_t* count, cudaStream_t st) {
  uint32_t flags = 0;
  CU(cudaMemcpyAsync(count, d_res, sizeof(uint64_t), cudaMemcpyDeviceToHost, st), "result copy");
  CU(cudaMemcpyAsync(&flags, m->counters + 15, sizeof(uint32_t), cudaMemcpyDeviceToHost, st), "flag copy");
  CU(cudaStreamSynchronize(st), "count");
  if (flags) {
    CU(cudaMemsetAsync(m->counters + 15, 0, sizeof(uint32_t), st), "flag reset");
    return set_error(EH_ERR_DEVICE_CHECK, "a device-side wait ran out (flags 0x%x); the count is not valid", flags);
  }
  return EH_OK;
}

eh_status launch_cliques(Matrix* m, uint32_t k, unsigned long long* out, const uint32_t* graph_rows,
                         uint32_t num_graphs, cudaStream_t st, Workspace* ws, bool list, uint32_t* tuples,
                         uint64_t capacity) {
  Workspace own;
  if (!ws) {
    own.counters = m->counters;
    own.clique_scratch = m->clique_scratch;
    own.clique_scratch_words = m->clique_scratch_words;
  }
  Workspace& w = ws ? *ws : own;
  if (m->selection != EH_SELECT_LOWER)
    return set_error(EH_ERR_UNSUPPORTED, "clique counting needs a matrix built with EH_SELECT_LOWER");
  if (k > kCliqueMaxK)
    return set_error(EH_ERR_UNSUPPORTED, "clique size %u above the supported maximum %u", k, kCliqueMaxK);
  CU(cudaMemsetAsync(out, 0, sizeof(uint64_t) * (graph_rows ? num_graphs : 1), st), "memset");
  // The reference's recursion only returns a count at depth n >= 3 (apps/n_clique.cpp:41-43);
  // for n < 3 it never reaches that depth and the count stays 0.
  if (k < 3) return EH_OK;
  if (m->tot.max_card >= kCliqueMaxPivot)
    return set_error(EH_ERR_UNSUPPORTED, "a row of %llu selected entries is above the clique kernels' limit of %u",
                     (unsigned long long)m->tot.max_card, kCliqueMaxPivot - 1);
  eh_status s = ensure_plan(m, st);
  if (s != EH_OK) return s;
  const Plan& p = m->plan;
  const uint32_t cap = clique_smem_cap(k, m->device);
  const uint32_t nG = p.above(cap);
  const uint32_t nB = p.above(32);
  const uint32_t nL = p.above(k - 2);
  CliqueArgs a{m->desc, m->arena, p.order, k, out, graph_rows, num_graphs, p.core, p.core_k, tuples, capacity};
  CU(cudaMemsetAsync(w.counters, 0, 16 * sizeof(uint32_t), st), "memset");
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, m->device);
  if (nG > 0) {
    const uint32_t cmax = (uint32_t)m->tot.max_card;
    int grid = (int)std::min<uint64_t>(nG, 2ull * sms);
    const uint64_t slot = clique_slot_words(cmax, k);
    if (slot * grid > w.clique_scratch_words) {
      if (ws) {  // a caller's workspace is never grown here: use the slots it has
        grid = (int)std::min<uint64_t>(grid, w.clique_scratch_words / slot);
        if (grid < 1) return set_error(EH_ERR_OUT_OF_MEMORY, "workspace too small for a %u-entry pivot", cmax);
      } else {
        if (m->clique_scratch) {  // earlier launches on any stream may still use it
          CU(wait_uses(m, st), "clique scratch");
          CU(cudaFreeAsync(m->clique_scratch, st), "clique scratch");
        }
        m->clique_scratch = nullptr;
        m->clique_scratch_words = 0;
        CU(pool_alloc((void**)&m->clique_scratch, slot * grid * 4, st), "clique scratch allocation");
        m->clique_scratch_words = slot * grid;
        w.clique_scratch = m->clique_scratch;
        w.clique_scratch_words = m->clique_scratch_words;
      }
    }
    CU(launch_clique_cta(a, 0, nG, w.counters + 2, cmax, w.clique_scratch, grid, st, list), "clique kernel (global)");
  }
  // The shared-memory tier runs in size bands, each launch sized for its own
  // largest pivot, so that the many small pivots are not held to the
  // occupancy of the largest one.  Band edges where the CTAs per SM change
  // (1 above 1,024 entries, 3 up to 1,024, 5 up to 768, 6 -- the register
  // limit -- up to 512); fewer bands mean fewer drained-GPU tails.
  const uint32_t bands[] = {cap, 1024, 768, 512, 32};
  for (int b = 0; b + 1 < (int)(sizeof(bands) / sizeof(bands[0])); b++) {
    if (bands[b] <= bands[b + 1]) continue;
    const uint32_t p0 = p.above(bands[b]), p1 = p.above(bands[b + 1]);
    if (p1 <= p0) continue;
    const uint32_t cmax = p.largest_at_most(bands[b]);
    CU(launch_clique_cta(a, p0, p1, w.counters + 3 + b, cmax, nullptr, 0, st, list), "clique kernel (shared)");
  }
  if (nL > nB) {
    const int grid = (int)std::min<uint64_t>((nL - nB + 63) / 64, 8ull * sms);
    CU(launch_clique_light(a, nB, nL, w.counters + 11, grid > 0 ? grid : 1, st, list), "clique kernel (warp)");
  }
  note_use(m, st);
  return EH_OK;
}

eh_status launch_lollipop_count(Matrix* m, unsigned long long* out, cudaStream_t st) {
  eh_status s = ensure_plan(m, st);
  if (s != EH_OK) return s;
  PivotArgs a = pivot_args(m, out);
  CU(launch_lollipops(a, m->plan.units, m->plan.n_units, m->grid, st), "lollipop kernel");
  note_use(m, st);
  return EH_OK;
}

eh_status launch_triangle_count(Matrix* m, unsigned long long* out, const uint32_t* graph_rows, uint32_t num_graphs,
                                cudaStream_t st, Workspace* ws) {
  if (m->selection != EH_SELECT_LOWER)
    return set_error(EH_ERR_UNSUPPORTED, "triangle counting needs a matrix built with EH_SELECT_LOWER");
  eh_status s = ensure_plan(m, st);
  if (s != EH_OK) return s;
  PivotArgs a = pivot_args(m, out);
  if (ws) a.counters = ws->counters;
  a.graph_rows = graph_rows;
  a.num_graphs = num_graphs;
  CU(launch_triangles(a, m->plan.units, m->plan.n_units, m->grid, st), "triangle kernel");
  note_use(m, st);
  return EH_OK;
}

}  // namespace eh

using eh::Matrix;
using eh::set_error;

static Matrix* MX(eh_matrix_t m) { return reinterpret_cast<Matrix*>(m); }
static cudaStream_t ST(void* s) { return reinterpret_cast<cudaStream_t>(s); }

#define CHECK_MATRIX(m)                                                      \
  do {                                                                       \
    if (!(m)) return set_error(EH_ERR_INVALID_ARGUMENT, "matrix is NULL");   \
    cudaSetDevice(MX(m)->device);                                            \
  } while (0)

extern "C" {

eh_status eh_matrix_build_device(uint64_t n, const uint64_t* d_offsets, const uint32_t* d_nbrs,
                                 const uint8_t* d_edge_mask, eh_selection sel, eh_layout layout,
                                 void* stream, eh_matrix_t* out) {
  Matrix* m = nullptr;
  eh_status s = eh::build_device(n, d_offsets, d_nbrs, d_edge_mask, (int)sel, (int)layout, ST(stream), &m,
                                 eh::kTotalUnknown);
  if (s == EH_OK) *out = reinterpret_cast<eh_matrix_t>(m);
  return s;
}

eh_status eh_matrix_build(uint64_t n, const uint64_t* offsets, const uint32_t* nbrs, const uint8_t* edge_mask,
                          eh_selection sel, eh_layout layout, void* stream, eh_matrix_t* out) {
  EH_CHECK_ARG(out != nullptr, "out is NULL");
  EH_CHECK_ARG(offsets != nullptr, "offsets is NULL");
  EH_CHECK_ARG(n < (1ull << 32), "n=%llu exceeds the u32 vertex id space", (unsigned long long)n);
  EH_CHECK_ARG(offsets[0] == 0, "offsets[0] must be 0");
  const uint64_t m = offsets[n];
  EH_CHECK_ARG(m == 0 || nbrs != nullptr, "nbrs is NULL");
  EH_CHECK_ARG(sel != EH_SELECT_MASK || edge_mask != nullptr || m == 0, "EH_SELECT_MASK needs an edge mask");
  // Offsets are checked on the device (each row must lie within [0, offsets[n])).
  cudaStream_t st = ST(stream);
  cudaStream_t cs = nullptr;
  uint64_t* d_off = nullptr;
  uint32_t* d_nbr = nullptr;
  uint8_t* d_mask = nullptr;
  cudaError_t e;
  if ((e = eh::upload_stream(&cs)) != cudaSuccess) return eh::cuda_fail(e, "upload stream");
  if ((e = eh::pool_alloc((void**)&d_off, (n + 1) * 8, st)) != cudaSuccess ||
      (e = eh::pool_alloc((void**)&d_nbr, (m ? m : 1) * 4, st)) != cudaSuccess ||
      (sel == EH_SELECT_MASK && (e = eh::pool_alloc((void**)&d_mask, m ? m : 1, st)) != cudaSuccess)) {
    cudaFreeAsync(d_off, st);
    cudaFreeAsync(d_nbr, st);
    return set_error(EH_ERR_OUT_OF_MEMORY, "input upload allocation failed: %s", cudaGetErrorString(e));
  }
  // The adjacency goes up in chunks of rows (about kUploadChunkEntries entries
  // each) on the upload stream, and the build's first pass measures each chunk
  // as soon as it has landed, so the copy over the host link and the measure
  // pass overlap.  Every entry is copied exactly once whatever the offsets
  // hold (rows with bad offsets are rejected by the measure pass).
  constexpr uint64_t kUploadChunkEntries = 16ull << 20;
  constexpr uint64_t kUploadMaxChunks = 16;
  const uint64_t chunks =
      std::max<uint64_t>(1, std::min<uint64_t>(kUploadMaxChunks, (m + kUploadChunkEntries - 1) / kUploadChunkEntries));
  eh::UploadChunks up;
  std::vector<uint64_t> upto;
  eh::plan_upload_chunks(n, offsets, m, chunks, up.rows, upto);
  eh_status s = EH_OK;
  cudaEvent_t allocated = nullptr;
  auto event = [](cudaEvent_t* ev) { return cudaEventCreateWithFlags(ev, cudaEventDisableTiming); };
  if ((e = event(&allocated)) != cudaSuccess) allocated = nullptr;
  if (e != cudaSuccess || (e = cudaEventRecord(allocated, st)) != cudaSuccess ||
      (e = cudaStreamWaitEvent(cs, allocated, 0)) != cudaSuccess ||
      (e = cudaMemcpyAsync(d_off, offsets, (n + 1) * 8, cudaMemcpyHostToDevice, cs)) != cudaSuccess)
    s = eh::cuda_fail(e, "upload");
  uint64_t copied = 0;
  for (uint64_t c = 0; c < chunks && s == EH_OK; c++) {
    if (upto[c] > copied) {
      if ((e = cudaMemcpyAsync(d_nbr + copied, nbrs + copied, (upto[c] - copied) * 4, cudaMemcpyHostToDevice,
                               cs)) != cudaSuccess ||
          (d_mask && (e = cudaMemcpyAsync(d_mask + copied, edge_mask + copied, upto[c] - copied,
                                          cudaMemcpyHostToDevice, cs)) != cudaSuccess)) {
        s = eh::cuda_fail(e, "upload");
        break;
      }
    }
    copied = upto[c];
    cudaEvent_t ev = nullptr;
    if ((e = event(&ev)) != cudaSuccess) {
      s = eh::cuda_fail(e, "upload event");
      break;
    }
    up.ready.push_back(ev);
    if ((e = cudaEventRecord(ev, cs)) != cudaSuccess) s = eh::cuda_fail(e, "upload event");
  }
  Matrix* mx = nullptr;
  if (s == EH_OK) s = eh::build_device(n, d_off, d_nbr, d_mask, (int)sel, (int)layout, st, &mx, m, &up);
  if (s == EH_OK) *out = reinterpret_cast<eh_matrix_t>(mx);
  // Every copy has landed before the upload buffers go back to the pool (after
  // a successful build the stream has already waited for all of them).
  if (allocated) cudaStreamSynchronize(cs);
  cudaFreeAsync(d_off, st);
  cudaFreeAsync(d_nbr, st);
  if (d_mask) cudaFreeAsync(d_mask, st);
  if (allocated) cudaEventDestroy(allocated);
  for (cudaEvent_t ev : up.ready) cudaEventDestroy(ev);
  return s;
}

eh_status eh_matrix_get_info(eh_matrix_t mh, eh_matrix_info* info) {
  CHECK_MATRIX(mh);
  EH_CHECK_ARG(info, "info is NULL");
  Matrix* m = MX(mh);
  info->matrix_size = m->n;
  info->cardinality = m->tot.cardinality;
  info->row_total_bytes_used = m->tot.ref_bytes;
  info->max_nbrhood_size = m->tot.max_full_degree;
  info->max_row_cardinality = m->tot.max_card;
  info->num_uint_rows = m->tot.num_uint;
  info->num_pshort_rows = m->tot.num_pshort;
  info->num_bitset_rows = m->tot.num_bitset;
  info->device_bytes = m->device_bytes;
  info->layout = m->layout;
  info->selection = m->selection;
  return EH_OK;
}

eh_status eh_matrix_row_meta(eh_matrix_t mh, uint8_t* types, uint32_t* cards, uint64_t* nbytes) {
  CHECK_MATRIX(mh);
  Matrix* m = MX(mh);
  std::vector<eh::RowDesc> d(m->n);
  if (m->n) CU(cudaMemcpy(d.data(), m->desc, m->n * sizeof(eh::RowDesc), cudaMemcpyDeviceToHost), "desc copy");
  for (uint64_t i = 0; i < m->n; i++) {
    if (types) types[i] = (uint8_t)eh::desc_type(d[i]);
    if (cards) cards[i] = d[i].card;
    if (nbytes) nbytes[i] = eh::flattened_bytes(m->layout, d[i]);
  }
  return EH_OK;
}

namespace eh {
// Writes row d's flattened bytes (payload = its arena bytes) to p; returns the size.
static uint64_t flatten_row(int layout, const RowDesc& d, const uint8_t* payload, uint8_t* p) {
  const uint32_t type = desc_type(d), len = desc_len(d);
  const uint64_t pbytes = type == TY_UINT ? 4ull * d.card : type == TY_BITSET ? 8ull * len : 2ull * len;
  uint8_t* q = p;
  if (is_hybrid(layout)) {
    const uint64_t tag = type;
    memcpy(q, &tag, 8);
    q += 8;
  }
  if (type == TY_UINT) {
    memcpy(q, payload, pbytes);
    q += pbytes;
  } else if (d.card) {
    const uint32_t nb = (uint32_t)(type == TY_BITSET ? 8 + pbytes : pbytes);
    memcpy(q, &nb, 4);
    q += 4;
    if (type == TY_BITSET) {
      const uint64_t first = d.aux;
      memcpy(q, &first, 8);
      q += 8;
    }
    memcpy(q, payload, pbytes);
    q += pbytes;
  }
  return (uint64_t)(q - p);
}
}  // namespace eh

eh_status eh_matrix_export_row(eh_matrix_t mh, uint32_t row, uint8_t* buf, uint64_t cap, uint64_t* nbytes) {
  CHECK_MATRIX(mh);
  Matrix* m = MX(mh);
  EH_CHECK_ARG(row < m->n, "row %u out of range", row);
  EH_CHECK_ARG(nbytes, "nbytes is NULL");
  eh::RowDesc d;
  CU(cudaMemcpy(&d, m->desc + row, sizeof(d), cudaMemcpyDeviceToHost), "desc copy");
  const uint64_t total = eh::flattened_bytes(m->layout, d);
  *nbytes = total;
  EH_CHECK_ARG(buf != nullptr && cap >= total, "buffer too small (%llu < %llu)", (unsigned long long)cap,
               (unsigned long long)total);
  const uint32_t type = eh::desc_type(d), len = eh::desc_len(d);
  const uint64_t payload = type == eh::TY_UINT ? 4ull * d.card : type == eh::TY_BITSET ? 8ull * len : 2ull * len;
  std::vector<uint8_t> pl(payload ? payload : 1);
  if (payload) CU(cudaMemcpy(pl.data(), m->arena + d.off16, payload, cudaMemcpyDeviceToHost), "payload copy");
  eh::flatten_row(m->layout, d, pl.data(), buf);
  return EH_OK;
}

eh_status eh_matrix_export_flattened(eh_matrix_t mh, uint8_t* buf, uint64_t cap, uint64_t* nbytes) {
  CHECK_MATRIX(mh);
  EH_CHECK_ARG(nbytes, "nbytes is NULL");
  Matrix* m = MX(mh);
  std::vector<eh::RowDesc> d(m->n);
  if (m->n) CU(cudaMemcpy(d.data(), m->desc, m->n * sizeof(eh::RowDesc), cudaMemcpyDeviceToHost), "desc copy");
  uint64_t total = 0;
  for (uint64_t i = 0; i < m->n; i++) total += eh::flattened_bytes(m->layout, d[i]);
  *nbytes = total;
  if (!buf) return EH_OK;
  EH_CHECK_ARG(cap >= total, "buffer too small (%llu < %llu)", (unsigned long long)cap, (unsigned long long)total);
  std::vector<uint8_t> arena((m->arena_units + 1) * 16);
  CU(cudaMemcpy(arena.data(), m->arena, arena.size(), cudaMemcpyDeviceToHost), "arena copy");
  uint64_t pos = 0;
  for (uint64_t i = 0; i < m->n; i++) pos += eh::flatten_row(m->layout, d[i], arena.data() + 16ull * d[i].off16, buf + pos);
  return EH_OK;
}

eh_status eh_matrix_get_max_row_id(eh_matrix_t mh, uint32_t* row) {
  CHECK_MATRIX(mh);
  EH_CHECK_ARG(row, "row is NULL");
  Matrix* m = MX(mh);
  if (m->vstar < 0) {
    CU(cudaMemset(m->result, 0, 8), "memset");
    CU(eh::launch_max_row(m->n, m->desc, m->result, 0), "max row kernel");
    unsigned long long key = 0;
    CU(cudaMemcpy(&key, m->result, 8, cudaMemcpyDeviceToHost), "max row copy");
    m->vstar = m->n ? (int64_t)(0xffffffffu - (uint32_t)(key & 0xffffffffu)) : 0;
  }
  *row = (uint32_t)m->vstar;
  return EH_OK;
}

eh_status eh_matrix_triangle_bytes(eh_matrix_t mh, uint64_t* bytes) {
  CHECK_MATRIX(mh);
  EH_CHECK_ARG(bytes, "bytes is NULL");
  Matrix* m = MX(mh);
  CU(cudaMemset(m->result, 0, 8), "memset");
  CU(eh::launch_triangle_bytes(m->n, m->desc, m->arena, m->result, 0), "bytes kernel");
  CU(cudaMemcpy(bytes, m->result, 8, cudaMemcpyDeviceToHost), "bytes copy");
  return EH_OK;
}

void eh_matrix_free(eh_matrix_t mh) {
  Matrix* m = MX(mh);
  if (!m) return;
  cudaSetDevice(m->device);
  // The buffers go back to the pool on the library's upload stream once every
  // launch recorded on the matrix (on any stream) has finished; neither the
  // host nor other streams wait.
  cudaStream_t st = nullptr;
  if (eh::upload_stream(&st) != cudaSuccess || eh::wait_uses(m, st) != cudaSuccess) {
    cudaDeviceSynchronize();  // no stream to order the frees on: fall back to waiting here
    st = nullptr;
  }
  void* bufs[] = {m->desc, m->arena, m->counters, m->plan.order, m->plan.units, m->plan.giant_lists,
                  m->plan.giant_off, m->plan.core, m->plan.filter, m->clique_scratch};
  for (void* b : bufs)
    if (b) cudaFreeAsync(b, st);
  for (auto& u : m->uses) cudaEventDestroy(u.second);
  delete m;
}

eh_status eh_count_triangles_async(eh_matrix_t mh, uint64_t* d_count, void* stream) {
  CHECK_MATRIX(mh);
  EH_CHECK_ARG(d_count, "d_count is NULL");
  return eh::launch_triangle_count(MX(mh), reinterpret_cast<unsigned long long*>(d_count), nullptr, 0, ST(stream));
}

eh_status eh_count_triangles(eh_matrix_t mh, uint64_t* count, void* stream) {
  CHECK_MATRIX(mh);
  EH_CHECK_ARG(count, "count is NULL");
  eh_status s = eh_count_triangles_async(mh, reinterpret_cast<uint64_t*>(MX(mh)->result), stream);
  if (s != EH_OK) return s;
  return eh::finish_sync(MX(mh), MX(mh)->result, count, ST(stream));
}

eh_status eh_count_lollipops_async(eh_matrix_t mh, uint64_t* d_count, void* stream) {
  CHECK_MATRIX(mh);
  EH_CHECK_ARG(d_count, "d_count is NULL");
  return eh::launch_lollipop_count(MX(mh), reinterpret_cast<unsigned long long*>(d_count), ST(stream));
}

eh_status eh_count_lollipops(eh_matrix_t mh, uint64_t* count, void* stream) {
  CHECK_MATRIX(mh);
  EH_CHECK_ARG(count, "count is NULL");
  eh_status s = eh_count_lollipops_async(mh, reinterpret_cast<uint64_t*>(MX(mh)->result), stream);
  if (s != EH_OK) return s;
  return eh::finish_sync(MX(mh), MX(mh)->result, count, ST(stream));
}

eh_status eh_similar_nodes_async(eh_matrix_t mh, uint32_t threshold, uint64_t* d_count, void* stream) {
  CHECK_MATRIX(mh);
  EH_CHECK_ARG(d_count, "d_count is NULL");
  Matrix* m = MX(mh);
  uint32_t vstar = 0;
  eh_status s = eh_matrix_get_max_row_id(mh, &vstar);
  if (s != EH_OK) return s;
  CU(eh::launch_similar(m->n, m->desc, m->arena, vstar, threshold, reinterpret_cast<unsigned long long*>(d_count),
                        ST(stream)),
     "similar_nodes kernel");
  eh::note_use(m, ST(stream));
  return EH_OK;
}

eh_status eh_similar_nodes(eh_matrix_t mh, uint32_t threshold, uint64_t* count, void* stream) {
  CHECK_MATRIX(mh);
  EH_CHECK_ARG(count, "count is NULL");
  eh_status s = eh_similar_nodes_async(mh, threshold, reinterpret_cast<uint64_t*>(MX(mh)->result), stream);
  if (s != EH_OK) return s;
  return eh::finish_sync(MX(mh), MX(mh)->result, count, ST(stream));
}

eh_status eh_intersect_rows(eh_matrix_t mh, const uint32_t* d_a, const uint32_t* d_b, uint64_t npairs,
                            uint32_t* d_counts, void* stream) {
  CHECK_MATRIX(mh);
  EH_CHECK_ARG(npairs == 0 || (d_a && d_b && d_counts), "NULL pair arrays");
  Matrix* m = MX(mh);
  CU(eh::launch_intersect_rows(m->n, m->desc, m->arena, d_a, d_b, npairs, d_counts, ST(stream)), "intersect kernel");
  eh::note_use(m, ST(stream));
  return EH_OK;
}

eh_status eh_count_cliques_async(eh_matrix_t mh, uint32_t k, uint64_t* d_count, void* stream) {
  CHECK_MATRIX(mh);
  EH_CHECK_ARG(d_count, "d_count is NULL");
  return eh::launch_cliques(MX(mh), k, reinterpret_cast<unsigned long long*>(d_count), nullptr, 0, ST(stream));
}

eh_status eh_list_cliques(eh_matrix_t mh, uint32_t k, uint32_t* d_out, uint64_t capacity, uint64_t* d_total,
                          void* stream) {
  CHECK_MATRIX(mh);
  EH_CHECK_ARG(d_total, "d_total is NULL");
  EH_CHECK_ARG(capacity == 0 || d_out, "d_out is NULL");
  if (k != 3 && k != 4) return set_error(EH_ERR_UNSUPPORTED, "clique tuples are written for k = 3 or 4, not %u", k);
  return eh::launch_cliques(MX(mh), k, reinterpret_cast<unsigned long long*>(d_total), nullptr, 0, ST(stream),
                            nullptr, true, d_out, capacity);
}

eh_status eh_count_cliques(eh_matrix_t mh, uint32_t k, uint64_t* count, void* stream) {
  CHECK_MATRIX(mh);
  EH_CHECK_ARG(count, "count is NULL");
  eh_status s = eh_count_cliques_async(mh, k, reinterpret_cast<uint64_t*>(MX(mh)->result), stream);
  if (s != EH_OK) return s;
  return eh::finish_sync(MX(mh), MX(mh)->result, count, ST(stream));
}

}  // extern "C"
