// k-clique counting that allocates no device memory when it is called.
//
// eh_count_cliques_async allocates a global scratch area the first time a
// matrix has pivot rows too large for shared memory (more than 1,024 entries),
// and grows it when a later call needs more.  Some callers cannot allow that:
// a serving loop that reserves its whole device-memory budget at start-up and
// must not grow its footprint or meet an allocation failure in the middle of a
// request, or a host framework that owns every device allocation and forbids
// libraries from calling cudaMalloc / cudaFree (cudaFree also synchronizes the
// device).  eh_count_cliques_noalloc runs the same kernels with their scratch
// taken from one fixed array in device memory instead.
//
// The array is a file-scope __device__ variable of kNoAllocScratchBytes
// (16 MiB): every GPU that loads this library holds it until the process
// exits.  Its first 64 words are the kernels' work-queue counters; the rest
// holds the per-CTA slots of the largest pivots.  A pivot whose slot does not
// fit is rejected with EH_ERR_UNSUPPORTED.  All calls share the array and it
// keeps the previous call's contents: the counters are cleared on every call,
// the slots are fully rewritten before they are read.  Calls whose kernels
// overlap on the GPU (for example on two streams) race on the array.
//
// Host code cannot use the array's name as a device address (in host code it
// is a host-side stand-in).  The first call on each device, with that device
// current, looks its address up once with cudaGetSymbolAddress; that first
// call should come before any stream capture.  The address is kept for the
// life of the process: a device reset (cudaDeviceReset) after the first call
// is not supported, since the module and its array are loaded again then.
//
// The shared-memory tier runs as one launch sized for its largest pivot
// (eh_count_cliques_async splits it into size bands with their own occupancy),
// so on skewed graphs this entry point can be slower.  It records no use on
// the matrix: eh_matrix_free does not wait for its launches, so the caller
// synchronizes their stream before freeing the matrix.
#include <algorithm>
#include <cstdint>
#include <mutex>

#include <cuda_runtime.h>

#include "eh_internal.h"
#include "eh_kernels.cuh"
#include "eh_matrix.cuh"

namespace eh {
namespace {

constexpr uint64_t kNoAllocScratchBytes = 16ull << 20;
constexpr uint64_t kNoAllocScratchWords = kNoAllocScratchBytes / 4;
constexpr uint64_t kCounterWords = 64;  // work counters, then slots from a 256-byte boundary
constexpr int kMaxDevices = 64;

static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocScratchWords];

std::mutex g_setup_mutex;
uint32_t* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on `device` (which must be current).
eh_status scratch_address(int device, uint32_t** out) {
  if (device < 0 || device >= kMaxDevices)
    return set_error(EH_ERR_UNSUPPORTED, "device ordinal %d above %d", device, kMaxDevices - 1);
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return set_error(EH_ERR_CUDA, "cudaGetSymbolAddress(clique scratch): %s", cudaGetErrorString(e));
    g_scratch_ptr[device] = static_cast<uint32_t*>(p);
  }
  *out = g_scratch_ptr[device];
  return EH_OK;
}

}  // namespace
}  // namespace eh

extern "C" eh_status eh_count_cliques_noalloc(eh_matrix_t mh, uint32_t k, uint64_t* d_count, void* stream) {
  using namespace eh;
  if (!mh) return set_error(EH_ERR_INVALID_ARGUMENT, "matrix is NULL");
  Matrix* m = reinterpret_cast<Matrix*>(mh);
  cudaSetDevice(m->device);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  EH_CHECK_ARG(d_count, "d_count is NULL");
  if (m->selection != EH_SELECT_LOWER)
    return set_error(EH_ERR_UNSUPPORTED, "clique counting needs a matrix built with EH_SELECT_LOWER");
  if (k > kCliqueMaxK)
    return set_error(EH_ERR_UNSUPPORTED, "clique size %u above the supported maximum %u", k, kCliqueMaxK);
  if (!m->plan.ready)
    return set_error(EH_ERR_INVALID_ARGUMENT,
                     "the matrix has no work plan yet; run one count on it (any eh_count_* call) "
                     "before the first no-allocation call");
  uint32_t* scratch = nullptr;
  eh_status s = scratch_address(m->device, &scratch);
  if (s != EH_OK) return s;
  cudaError_t e = cudaMemsetAsync(d_count, 0, sizeof(uint64_t), st);
  if (e != cudaSuccess) return set_error(EH_ERR_CUDA, "memset: %s", cudaGetErrorString(e));
  if (k < 3) return EH_OK;  // as eh_count_cliques: the reference returns 0 for n < 3
  if (m->tot.max_card >= kCliqueMaxPivot)
    return set_error(EH_ERR_UNSUPPORTED, "a row of %llu selected entries is above the clique kernels' limit of %u",
                     (unsigned long long)m->tot.max_card, kCliqueMaxPivot - 1);
  const Plan& p = m->plan;
  const uint32_t cap = clique_smem_cap(k, m->device);
  const uint32_t nG = p.above(cap);
  const uint32_t nB = p.above(32);
  const uint32_t nL = p.above(k - 2);
  uint32_t* counters = scratch;
  uint32_t* slots = scratch + kCounterWords;
  const uint64_t slot_capacity = kNoAllocScratchWords - kCounterWords;
  // No dense core here: the counts probe the rows themselves.
  CliqueArgs a{m->desc, m->arena, p.order, k, reinterpret_cast<unsigned long long*>(d_count), nullptr, 0,
               nullptr, 0};
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, m->device);
  uint64_t grid_g = 0;
  if (nG > 0) {
    const uint32_t cmax = (uint32_t)m->tot.max_card;
    const uint64_t slot = clique_slot_words(cmax, k);
    if (slot > slot_capacity)
      return set_error(EH_ERR_UNSUPPORTED,
                       "a pivot row of %u entries needs %llu bytes of clique scratch for k=%u; the fixed "
                       "scratch of eh_count_cliques_noalloc holds %llu bytes (use eh_count_cliques)",
                       cmax, (unsigned long long)(slot * 4), k, (unsigned long long)(slot_capacity * 4));
    grid_g = std::min<uint64_t>(std::min<uint64_t>(nG, 2ull * sms), slot_capacity / slot);
  }
  e = cudaMemsetAsync(counters, 0, kCounterWords * sizeof(uint32_t), st);
  if (e != cudaSuccess) return set_error(EH_ERR_CUDA, "memset: %s", cudaGetErrorString(e));
  if (nG > 0) {
    e = launch_clique_cta(a, 0, nG, counters + 2, (uint32_t)m->tot.max_card, slots, (int)grid_g, st);
    if (e != cudaSuccess) return set_error(EH_ERR_CUDA, "clique kernel (fixed scratch): %s", cudaGetErrorString(e));
  }
  if (nB > nG) {
    const uint32_t cmax = p.largest_at_most(cap);
    const int grid = (int)std::min<uint64_t>(nB - nG, 4ull * sms);
    e = launch_clique_cta(a, nG, nB, counters + 3, cmax, nullptr, grid, st);
    if (e != cudaSuccess) return set_error(EH_ERR_CUDA, "clique kernel (shared): %s", cudaGetErrorString(e));
  }
  if (nL > nB) {
    const int grid = (int)std::min<uint64_t>((nL - nB + 63) / 64, 8ull * sms);
    e = launch_clique_light(a, nB, nL, counters + 4, grid > 0 ? grid : 1, st);
    if (e != cudaSuccess) return set_error(EH_ERR_CUDA, "clique kernel (warp): %s", cudaGetErrorString(e));
  }
  return EH_OK;
}
