// Device ingestion of undirected edge lists: the work of
// MutableGraph::undirectedFromEdgeList (src/MutableGraph.hpp:517-599: both
// directions, rows sorted, duplicates removed, self-loops kept) and
// reorder_by_degree (:268-272 with OrderNeighborhoodByDegree, :20-32: relabel
// by descending degree, ties by ascending id, then sort every row), done on
// the device so that an end-to-end run can start from raw edges.
//
// Each directed entry is a u64 key (row << 32 | nbr); a radix sort plus a
// unique pass gives the sorted, deduplicated adjacency, and row offsets are
// lower bounds of (row << 32) in the key array.  Degree ordering sorts
// (~degree << 32 | id) keys for the new order, relabels every key and sorts
// again.  Vertex ids are dense (0 .. n-1); the host loader keeps the
// reference's arbitrary external ids.
#include <cstdint>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_select.cuh>
#include <cuda_runtime.h>

#include "eh_internal.h"
#include "eh_kernels.cuh"

namespace eh {

struct DCsr {
  int device = 0;
  uint64_t n = 0, entries = 0;
  uint64_t* offsets = nullptr;
  uint32_t* nbrs = nullptr;
  uint32_t* new2old = nullptr;  // null unless degree-ordered
};

namespace {

constexpr unsigned long long kDropped = ~0ull;

__global__ void k_edge_keys(uint64_t m, const uint32_t* __restrict__ src, const uint32_t* __restrict__ dst,
                            uint64_t n, int drop_self, unsigned long long* __restrict__ keys, uint32_t* err) {
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t u = src[e], v = dst[e];
    if (u >= n || v >= n) {
      atomicOr(err, 1u);
      keys[2 * e] = keys[2 * e + 1] = kDropped;
    } else if (u == v && drop_self) {
      keys[2 * e] = keys[2 * e + 1] = kDropped;
    } else {
      keys[2 * e] = ((unsigned long long)u << 32) | v;
      keys[2 * e + 1] = ((unsigned long long)v << 32) | u;
    }
  }
}

// offsets[r] = first position with key >= r << 32 (r in 0..n); nbrs = low words.
__global__ void k_csr_from_keys(uint64_t n, const unsigned long long* __restrict__ keys, uint64_t count,
                                uint64_t* __restrict__ offsets, uint32_t* __restrict__ nbrs) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r <= n; r += stride) {
    const unsigned long long target = (unsigned long long)r << 32;
    uint64_t lo = 0, hi = count;
    while (lo < hi) {
      const uint64_t mid = (lo + hi) >> 1;
      if (keys[mid] < target) lo = mid + 1; else hi = mid;
    }
    offsets[r] = lo;
  }
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride)
    nbrs[i] = (uint32_t)(keys[i] & 0xffffffffull);
}

__global__ void k_degree_keys(uint64_t n, const uint64_t* __restrict__ offsets, unsigned long long* __restrict__ keys) {
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t deg = offsets[r + 1] - offsets[r];
    keys[r] = ((unsigned long long)(0xffffffffu - (uint32_t)deg) << 32) | r;  // descending degree, then id
  }
}

__global__ void k_orders(uint64_t n, const unsigned long long* __restrict__ sorted, uint32_t* __restrict__ new2old,
                         uint32_t* __restrict__ old2new) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t old = (uint32_t)(sorted[i] & 0xffffffffull);
    new2old[i] = old;
    old2new[old] = (uint32_t)i;
  }
}

__global__ void k_relabel(uint64_t count, const unsigned long long* __restrict__ keys,
                          const uint32_t* __restrict__ old2new, unsigned long long* __restrict__ out) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (uint64_t)gridDim.x * blockDim.x) {
    const unsigned long long k = keys[i];
    out[i] = ((unsigned long long)old2new[k >> 32] << 32) | old2new[k & 0xffffffffull];
  }
}

int bits_for(uint64_t n) {
  int b = 1;
  while (b < 32 && (1ull << b) < n) b++;
  return b;
}

unsigned grid_of(uint64_t items) {
  uint64_t g = (items + 255) / 256;
  if (g < 1) g = 1;
  if (g > 152ull * 32) g = 152ull * 32;
  return (unsigned)g;
}

}  // namespace
}  // namespace eh

using eh::set_error;

extern "C" {

eh_status eh_dcsr_from_edges(uint64_t n, uint64_t num_edges, const uint32_t* d_src, const uint32_t* d_dst,
                             int drop_self_loops, int degree_order, void* stream, eh_dcsr_t* out) {
  EH_CHECK_ARG(out, "out is NULL");
  EH_CHECK_ARG(n >= 1 && n < (1ull << 32), "n out of range");
  EH_CHECK_ARG(num_edges == 0 || (d_src && d_dst), "edge arrays are NULL");
  EH_CHECK_ARG(num_edges < (1ull << 62), "too many edges");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  eh::DCsr* g = new eh::DCsr();
  cudaGetDevice(&g->device);
  g->n = n;
  const uint64_t m2 = 2 * num_edges;
  unsigned long long *a = nullptr, *b = nullptr;
  void* temp = nullptr;
  size_t temp_bytes = 0, t1 = 0, t2 = 0;
  uint32_t* err = nullptr;
  unsigned long long* d_count = nullptr;
  uint32_t* old2new = nullptr;
  cudaError_t e = cudaSuccess;
  const int row_bits = eh::bits_for(n);
  auto fail = [&](eh_status s) {
    cudaStreamSynchronize(st);
    cudaFree(a);
    cudaFree(b);
    cudaFree(temp);
    cudaFree(err);
    cudaFree(d_count);
    cudaFree(old2new);
    cudaFree(g->offsets);
    cudaFree(g->nbrs);
    cudaFree(g->new2old);
    delete g;
    return s;
  };
  const uint64_t cap = m2 > n ? m2 : n;
  if ((e = cudaMalloc((void**)&a, (cap ? cap : 1) * 8)) != cudaSuccess ||
      (e = cudaMalloc((void**)&b, (cap ? cap : 1) * 8)) != cudaSuccess ||
      (e = cudaMalloc((void**)&err, 4)) != cudaSuccess || (e = cudaMalloc((void**)&d_count, 8)) != cudaSuccess)
    return fail(set_error(EH_ERR_OUT_OF_MEMORY, "ingestion buffers (%llu bytes): %s",
                          (unsigned long long)(2 * cap * 8), cudaGetErrorString(e)));
  cub::DeviceRadixSort::SortKeys(nullptr, t1, a, b, (int64_t)cap, 0, 64, st);
  cub::DeviceSelect::Unique(nullptr, t2, b, a, d_count, (int64_t)cap, st);
  temp_bytes = t1 > t2 ? t1 : t2;
  if ((e = cudaMalloc(&temp, temp_bytes ? temp_bytes : 1)) != cudaSuccess)
    return fail(set_error(EH_ERR_OUT_OF_MEMORY, "sort scratch: %s", cudaGetErrorString(e)));
  cudaMemsetAsync(err, 0, 4, st);
  uint64_t count = 0;
  if (m2) {
    eh::k_edge_keys<<<eh::grid_of(num_edges), 256, 0, st>>>(num_edges, d_src, d_dst, n, drop_self_loops, a, err);
    // Sort all 64 bits: dropped entries are ~0 and must sort last.
    t1 = temp_bytes;
    cub::DeviceRadixSort::SortKeys(temp, t1, a, b, (int64_t)m2, 0, 64, st);
    t2 = temp_bytes;
    cub::DeviceSelect::Unique(temp, t2, b, a, d_count, (int64_t)m2, st);
    unsigned long long hc = 0, last = 0;
    uint32_t herr = 0;
    cudaMemcpyAsync(&hc, d_count, 8, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail(set_error(EH_ERR_CUDA, "ingestion: %s", cudaGetErrorString(e)));
    if (herr) return fail(set_error(EH_ERR_INVALID_ARGUMENT, "an edge endpoint is >= n"));
    if (hc) {
      cudaMemcpy(&last, a + hc - 1, 8, cudaMemcpyDeviceToHost);
      count = hc - (last == eh::kDropped ? 1 : 0);
    }
  }
  g->entries = count;
  if ((e = cudaMalloc((void**)&g->offsets, (n + 1) * 8)) != cudaSuccess ||
      (e = cudaMalloc((void**)&g->nbrs, (count ? count : 1) * 4)) != cudaSuccess)
    return fail(set_error(EH_ERR_OUT_OF_MEMORY, "CSR allocation: %s", cudaGetErrorString(e)));
  eh::k_csr_from_keys<<<eh::grid_of(n + 1 > count ? n + 1 : count), 256, 0, st>>>(n, a, count, g->offsets, g->nbrs);
  if (degree_order) {
    unsigned long long* order_keys = nullptr;
    if ((e = cudaMalloc((void**)&g->new2old, n * 4)) != cudaSuccess ||
        (e = cudaMalloc((void**)&old2new, n * 4)) != cudaSuccess ||
        (e = cudaMalloc((void**)&order_keys, n * 8)) != cudaSuccess) {
      cudaFree(order_keys);
      return fail(set_error(EH_ERR_OUT_OF_MEMORY, "order allocation: %s", cudaGetErrorString(e)));
    }
    // New order: sort (~degree << 32 | id) keys (b is free: the entries are in a).
    eh::k_degree_keys<<<eh::grid_of(n), 256, 0, st>>>(n, g->offsets, b);
    t1 = temp_bytes;
    cub::DeviceRadixSort::SortKeys(temp, t1, b, order_keys, (int64_t)n, 0, 64, st);
    eh::k_orders<<<eh::grid_of(n), 256, 0, st>>>(n, order_keys, g->new2old, old2new);
    if (count) {  // relabel every entry, then sort rows and neighbours again
      eh::k_relabel<<<eh::grid_of(count), 256, 0, st>>>(count, a, old2new, b);
      t1 = temp_bytes;
      cub::DeviceRadixSort::SortKeys(temp, t1, b, a, (int64_t)count, 0, 32 + row_bits, st);
    }
    eh::k_csr_from_keys<<<eh::grid_of(n + 1 > count ? n + 1 : count), 256, 0, st>>>(n, a, count, g->offsets, g->nbrs);
    cudaStreamSynchronize(st);
    cudaFree(order_keys);
  }
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess)
    return fail(set_error(EH_ERR_CUDA, "ingestion: %s", cudaGetErrorString(e)));
  cudaFree(a);
  cudaFree(b);
  cudaFree(temp);
  cudaFree(err);
  cudaFree(d_count);
  cudaFree(old2new);
  *out = reinterpret_cast<eh_dcsr_t>(g);
  return EH_OK;
}

eh_status eh_dcsr_view(eh_dcsr_t gh, uint64_t* n, uint64_t* num_entries, const uint64_t** d_offsets,
                       const uint32_t** d_nbrs, const uint32_t** d_new2old) {
  EH_CHECK_ARG(gh, "graph is NULL");
  eh::DCsr* g = reinterpret_cast<eh::DCsr*>(gh);
  if (n) *n = g->n;
  if (num_entries) *num_entries = g->entries;
  if (d_offsets) *d_offsets = g->offsets;
  if (d_nbrs) *d_nbrs = g->nbrs;
  if (d_new2old) *d_new2old = g->new2old;
  return EH_OK;
}

void eh_dcsr_free(eh_dcsr_t gh) {
  eh::DCsr* g = reinterpret_cast<eh::DCsr*>(gh);
  if (!g) return;
  cudaSetDevice(g->device);
  cudaFree(g->offsets);
  cudaFree(g->nbrs);
  cudaFree(g->new2old);
  delete g;
}

}  // extern "C"
