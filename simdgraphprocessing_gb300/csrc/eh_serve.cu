// Serving loop: device-resident graphs, pattern queries with continuous
// batching, HBM-footprint admission, per-query latency.  (The reference has no
// serving; each answer is what its apps compute for that graph.)
//
// A dispatcher thread owns `slots` CUDA streams, each with its own workspace
// (work-queue counters, clique scratch slots, pinned result word).  Queries
// wait in arrival order; whenever a slot is free and a query's scratch fits
// under the HBM cap (resident graphs + scratch held by slots), the query is
// launched on that slot at once, so queries that arrive while others run
// overlap with them on the device.  A query whose scratch does not fit yet
// waits while younger queries that fit pass it, at most kMaxBypass of them;
// then admission stops until it has started (a bounded wait for large
// queries, no head-of-line blocking for small ones).  A query that fills the
// GPU by itself (a triangle or clique count on a graph of at least
// kFillEdges pruned edges) runs only while no other such query does: two of
// them side by side are slower than one after the other (they compete for
// the SMs and thrash each other's rows in L2), while small queries fit in
// beside one.  Such a query waiting for the running one lets younger small
// queries pass without limit (it starts as soon as the running one ends) and
// keeps its place ahead of younger large ones.  Slot scratch comes from
// the library's stream-ordered pool on the slot's own stream (no device-wide
// synchronisation while other slots run).  Completion is detected by polling
// each slot's event (cudaEventQuery, never a blocking wait), and callers wait
// on their ticket with a timeout.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "eh_internal.h"
#include "eh_kernels.cuh"
#include "eh_matrix.cuh"

namespace eh {
namespace {

int64_t now_ns() {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

struct Query {
  uint32_t graph = 0, kind = 0, param = 0;
  int64_t submit_ns = 0, start_ns = 0, done_ns = 0;
  uint64_t count = 0;
  eh_status status = EH_OK;
  int32_t slot = -1;
  bool done = false;
};

struct Slot {
  cudaStream_t st = nullptr;
  cudaEvent_t ev = nullptr;
  Workspace ws;
  unsigned long long* d_out = nullptr;
  uint64_t* h_out = nullptr;  // pinned: [0] the count, [1] the query's device error flags
  uint64_t ticket = 0;
  bool busy = false;
  bool fills = false;  // the running query fills the GPU by itself
};

struct GraphEntry {
  Matrix* low = nullptr;  // nbr < node rows: triangles, cliques
  Matrix* all = nullptr;  // full rows: similar_nodes
  uint32_t vstar = 0;
  uint64_t bytes = 0;
};

}  // namespace

constexpr uint32_t kMaxBypass = 64;     // younger queries that may pass a waiting one
constexpr uint64_t kFillEdges = 8ull << 20;  // pruned edges from which a count fills the GPU
constexpr size_t kAdmissionWindow = 256;  // queued queries looked at per admission round

struct Server {
  int device = 0;
  uint32_t nslots = 0;
  uint64_t cap = 0;
  uint64_t resident = 0;      // matrices
  uint64_t scratch = 0;       // clique scratch held by slots
  std::vector<GraphEntry> graphs;
  std::vector<Slot> slots;
  std::deque<uint64_t> queue;
  std::unordered_map<uint64_t, Query> queries;
  uint64_t next_ticket = 1;
  uint64_t completed = 0, launched = 0, max_inflight = 0;
  uint64_t blocked_ticket = 0;  // oldest query waiting for memory, and how often it has been passed
  uint32_t bypassed = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  bool stop = false;
  std::thread dispatcher;
};

namespace {

// Clique scratch words a query on graph g needs (0 when its pivots fit shared memory).
uint64_t query_scratch_words(const GraphEntry& ge, uint32_t kind, uint32_t k, int sms) {
  if (kind != EH_QUERY_CLIQUES || k < 3) return 0;
  const Matrix* m = ge.low;
  const uint32_t nG = m->plan.above(clique_smem_cap(k, m->device));
  if (!nG) return 0;
  const uint64_t grid = std::min<uint64_t>(nG, 2ull * sms);
  return clique_slot_words((uint32_t)m->tot.max_card, k) * grid;
}

// Whether query q alone keeps every SM busy for its whole run.
bool fills_gpu(const Server* s, const Query& q) {
  return q.kind != EH_QUERY_SIMILAR_NODES && s->graphs[q.graph].low->tot.cardinality >= kFillEdges;
}

eh_status launch_query(Server* s, Slot& sl, const Query& q) {
  const GraphEntry& ge = s->graphs[q.graph];
  eh_status st = EH_OK;
  if (q.kind == EH_QUERY_TRIANGLES) {
    st = launch_triangle_count(ge.low, sl.d_out, nullptr, 0, sl.st, &sl.ws);
  } else if (q.kind == EH_QUERY_CLIQUES) {
    st = launch_cliques(ge.low, q.param, sl.d_out, nullptr, 0, sl.st, &sl.ws);
  } else {
    cudaError_t e = launch_similar(ge.all->n, ge.all->desc, ge.all->arena, ge.vstar, q.param, sl.d_out, sl.st);
    if (e != cudaSuccess) st = set_error(EH_ERR_CUDA, "similar_nodes kernel: %s", cudaGetErrorString(e));
  }
  if (st != EH_OK) return st;
  cudaMemcpyAsync(sl.h_out, sl.d_out, sizeof(uint64_t), cudaMemcpyDeviceToHost, sl.st);
  // The pivot kernels' flags word (a bounded wait that ran out), cleared for the slot's next query.
  sl.h_out[1] = 0;
  cudaMemcpyAsync(sl.h_out + 1, sl.ws.counters + 15, sizeof(uint32_t), cudaMemcpyDeviceToHost, sl.st);
  cudaMemsetAsync(sl.ws.counters + 15, 0, sizeof(uint32_t), sl.st);
  cudaEventRecord(sl.ev, sl.st);
  return EH_OK;
}

void dispatch_loop(Server* s) {
  cudaSetDevice(s->device);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device);
  std::unique_lock<std::mutex> lock(s->mu);
  for (;;) {
    bool progress = false;
    // Completions.
    uint32_t inflight = 0;
    for (uint32_t i = 0; i < s->nslots; i++) {
      Slot& sl = s->slots[i];
      if (!sl.busy) continue;
      const cudaError_t e = cudaEventQuery(sl.ev);
      if (e == cudaErrorNotReady) {
        inflight++;
        continue;
      }
      Query& q = s->queries[sl.ticket];
      q.done_ns = now_ns();
      q.count = *sl.h_out;
      q.status = e != cudaSuccess ? EH_ERR_CUDA : sl.h_out[1] ? EH_ERR_DEVICE_CHECK : EH_OK;
      q.done = true;
      sl.busy = false;
      s->completed++;
      progress = true;
    }
    if (progress) s->cv_done.notify_all();
    // Admission, oldest first: each queued query takes a free slot when its
    // scratch fits under the cap; one that does not fit lets younger queries
    // pass (at most kMaxBypass in all) while slots drain and free memory.
    size_t qi = 0;
    bool blocked = false;
    bool filling = false;  // a GPU-filling query is running, or the oldest waiting one is
    for (const Slot& o : s->slots) filling = filling || (o.busy && o.fills);
    while (qi < s->queue.size() && qi < kAdmissionWindow) {
      int free_slot = -1;
      const uint64_t ticket = s->queue[qi];
      Query& q = s->queries[ticket];
      const bool fills = fills_gpu(s, q);
      if (fills && filling) {  // waits for the running one; smaller queries go ahead
        filling = true;
        qi++;
        continue;
      }
      const uint64_t need = query_scratch_words(s->graphs[q.graph], q.kind, q.param, sms);
      for (uint32_t i = 0; i < s->nslots; i++) {  // a free slot, preferring one whose scratch already fits
        if (s->slots[i].busy) continue;
        if (free_slot < 0 || (s->slots[i].ws.clique_scratch_words >= need &&
                              s->slots[free_slot].ws.clique_scratch_words < need))
          free_slot = (int)i;
      }
      if (free_slot < 0) break;
      Slot& sl = s->slots[free_slot];
      if (need > sl.ws.clique_scratch_words) {
        const uint64_t grow = (need - sl.ws.clique_scratch_words) * 4;
        if (s->resident + s->scratch + grow > s->cap) {
          // Idle slots give their scratch back (stream-ordered, nothing waits).
          for (Slot& o : s->slots)
            if (!o.busy && &o != &sl && o.ws.clique_scratch) {
              cudaFreeAsync(o.ws.clique_scratch, o.st);
              s->scratch -= o.ws.clique_scratch_words * 4;
              o.ws.clique_scratch = nullptr;
              o.ws.clique_scratch_words = 0;
            }
        }
        if (s->resident + s->scratch + grow > s->cap) {
          if (s->resident + need * 4 > s->cap) {  // can never fit
            s->queue.erase(s->queue.begin() + qi);
            q.status = set_error(EH_ERR_ADMISSION, "query needs %llu scratch bytes above the HBM cap",
                                 (unsigned long long)(need * 4));
            q.done = true;
            q.done_ns = now_ns();
            s->cv_done.notify_all();
            progress = true;
            continue;
          }
          if (!blocked) {  // the oldest query waiting for memory
            blocked = true;
            if (s->blocked_ticket != ticket) {
              s->blocked_ticket = ticket;
              s->bypassed = 0;
            }
          }
          if (s->bypassed >= kMaxBypass) break;  // it has waited long enough: no more passing
          qi++;
          continue;
        }
        if (sl.ws.clique_scratch) {
          cudaFreeAsync(sl.ws.clique_scratch, sl.st);
          s->scratch -= sl.ws.clique_scratch_words * 4;
          sl.ws.clique_scratch = nullptr;
          sl.ws.clique_scratch_words = 0;
        }
        if (pool_alloc((void**)&sl.ws.clique_scratch, need * 4, sl.st) != cudaSuccess) {
          sl.ws.clique_scratch = nullptr;
          break;  // retried on the next round, when other slots may have released memory
        }
        sl.ws.clique_scratch_words = need;
        s->scratch += need * 4;
      }
      s->queue.erase(s->queue.begin() + qi);
      if (blocked) s->bypassed++;
      q.start_ns = now_ns();
      q.slot = free_slot;
      sl.ticket = ticket;
      sl.fills = fills;
      filling = filling || fills;
      const eh_status st = launch_query(s, sl, q);
      if (st != EH_OK) {
        q.status = st;
        q.done = true;
        q.done_ns = now_ns();
        s->cv_done.notify_all();
      } else {
        sl.busy = true;
        s->launched++;
        inflight++;
      }
      progress = true;
    }
    s->max_inflight = std::max<uint64_t>(s->max_inflight, inflight);
    if (s->stop && s->queue.empty() && inflight == 0) break;
    if (!progress) {
      // Bounded nap: new submissions wake us at once; running slots are re-polled soon.
      s->cv_work.wait_for(lock, std::chrono::microseconds(inflight ? 20 : 2000));
    }
  }
}

}  // namespace
}  // namespace eh

using eh::Server;
using eh::set_error;

extern "C" {

eh_status eh_server_create(const eh_server_config* cfg, eh_server_t* out) {
  EH_CHECK_ARG(cfg && out, "NULL argument");
  EH_CHECK_ARG(cfg->slots >= 1 && cfg->slots <= 64, "slots must be in [1, 64]");
  Server* s = new Server();
  cudaGetDevice(&s->device);
  s->nslots = cfg->slots;
  s->cap = cfg->hbm_cap_bytes;
  s->slots.resize(s->nslots);
  for (auto& sl : s->slots) {
    if (cudaStreamCreateWithFlags(&sl.st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaMalloc((void**)&sl.ws.counters, 64) != cudaSuccess ||
        cudaMemset(sl.ws.counters, 0, 64) != cudaSuccess ||
        cudaMalloc((void**)&sl.d_out, sizeof(unsigned long long)) != cudaSuccess ||
        cudaMallocHost((void**)&sl.h_out, 2 * sizeof(uint64_t)) != cudaSuccess) {
      eh_server_free(reinterpret_cast<eh_server_t>(s));
      return set_error(EH_ERR_OUT_OF_MEMORY, "server slot allocation failed");
    }
  }
  s->dispatcher = std::thread(eh::dispatch_loop, s);
  *out = reinterpret_cast<eh_server_t>(s);
  return EH_OK;
}

eh_status eh_server_add_graph(eh_server_t sh, uint64_t n, const uint64_t* offsets, const uint32_t* nbrs,
                              eh_layout layout, uint32_t* graph_id) {
  EH_CHECK_ARG(sh && graph_id, "NULL argument");
  Server* s = reinterpret_cast<Server*>(sh);
  cudaSetDevice(s->device);
  eh_matrix_t low = nullptr, all = nullptr;
  eh_status st = eh_matrix_build(n, offsets, nbrs, nullptr, EH_SELECT_LOWER, layout, nullptr, &low);
  if (st != EH_OK) return st;
  st = eh_matrix_build(n, offsets, nbrs, nullptr, EH_SELECT_ALL, layout, nullptr, &all);
  if (st != EH_OK) {
    eh_matrix_free(low);
    return st;
  }
  eh::GraphEntry ge;
  ge.low = reinterpret_cast<eh::Matrix*>(low);
  ge.all = reinterpret_cast<eh::Matrix*>(all);
  if ((st = eh::ensure_plan(ge.low, nullptr)) == EH_OK) st = eh_matrix_get_max_row_id(all, &ge.vstar);
  if (st != EH_OK) {
    eh_matrix_free(low);
    eh_matrix_free(all);
    return st;
  }
  ge.bytes = ge.low->device_bytes + ge.all->device_bytes;
  std::lock_guard<std::mutex> lock(s->mu);
  if (s->resident + s->scratch + ge.bytes > s->cap) {
    eh_matrix_free(low);
    eh_matrix_free(all);
    return set_error(EH_ERR_ADMISSION, "graph needs %llu device bytes; %llu of the %llu-byte cap are in use",
                     (unsigned long long)ge.bytes, (unsigned long long)(s->resident + s->scratch),
                     (unsigned long long)s->cap);
  }
  s->resident += ge.bytes;
  s->graphs.push_back(ge);
  *graph_id = (uint32_t)(s->graphs.size() - 1);
  return EH_OK;
}

eh_status eh_server_submit(eh_server_t sh, uint32_t graph_id, eh_query_kind kind, uint32_t param, uint64_t* ticket) {
  EH_CHECK_ARG(sh && ticket, "NULL argument");
  Server* s = reinterpret_cast<Server*>(sh);
  EH_CHECK_ARG(kind == EH_QUERY_TRIANGLES || kind == EH_QUERY_CLIQUES || kind == EH_QUERY_SIMILAR_NODES,
               "unknown query kind %d", (int)kind);
  EH_CHECK_ARG(kind != EH_QUERY_CLIQUES || param <= eh::kCliqueMaxK, "clique size %u above %u", param,
               eh::kCliqueMaxK);
  {
    std::lock_guard<std::mutex> lock(s->mu);
    EH_CHECK_ARG(graph_id < s->graphs.size(), "unknown graph %u", graph_id);
    EH_CHECK_ARG(!s->stop, "server is stopping");
    const uint64_t t = s->next_ticket++;
    eh::Query q;
    q.graph = graph_id;
    q.kind = (uint32_t)kind;
    q.param = param;
    q.submit_ns = eh::now_ns();
    s->queries.emplace(t, q);
    s->queue.push_back(t);
    *ticket = t;
  }
  s->cv_work.notify_one();
  return EH_OK;
}

eh_status eh_server_wait(eh_server_t sh, uint64_t ticket, uint32_t timeout_ms, eh_query_result* out) {
  EH_CHECK_ARG(sh && out, "NULL argument");
  Server* s = reinterpret_cast<Server*>(sh);
  std::unique_lock<std::mutex> lock(s->mu);
  auto it = s->queries.find(ticket);
  EH_CHECK_ARG(it != s->queries.end(), "unknown ticket %llu", (unsigned long long)ticket);
  const bool ok = s->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms),
                                      [&] { return s->queries[ticket].done; });
  if (!ok) return set_error(EH_ERR_TIMEOUT, "query %llu not done after %u ms", (unsigned long long)ticket, timeout_ms);
  const eh::Query& q = s->queries[ticket];
  out->count = q.count;
  out->status = q.status;
  out->slot = q.slot;
  out->submit_ns = q.submit_ns;
  out->start_ns = q.start_ns;
  out->done_ns = q.done_ns;
  const eh_status st = q.status;
  s->queries.erase(ticket);
  return st;
}

eh_status eh_server_run_alone(eh_server_t sh, uint32_t graph_id, eh_query_kind kind, uint32_t param, uint64_t* count) {
  EH_CHECK_ARG(sh && count, "NULL argument");
  Server* s = reinterpret_cast<Server*>(sh);
  eh::GraphEntry ge;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    EH_CHECK_ARG(graph_id < s->graphs.size(), "unknown graph %u", graph_id);
    ge = s->graphs[graph_id];
  }
  eh_matrix_t low = reinterpret_cast<eh_matrix_t>(ge.low), all = reinterpret_cast<eh_matrix_t>(ge.all);
  if (kind == EH_QUERY_TRIANGLES) return eh_count_triangles(low, count, nullptr);
  if (kind == EH_QUERY_CLIQUES) return eh_count_cliques(low, param, count, nullptr);
  if (kind == EH_QUERY_SIMILAR_NODES) return eh_similar_nodes(all, param, count, nullptr);
  return set_error(EH_ERR_INVALID_ARGUMENT, "unknown query kind %d", (int)kind);
}

eh_status eh_server_stats(eh_server_t sh, eh_server_counters* out) {
  EH_CHECK_ARG(sh && out, "NULL argument");
  Server* s = reinterpret_cast<Server*>(sh);
  std::lock_guard<std::mutex> lock(s->mu);
  out->graphs = (uint32_t)s->graphs.size();
  out->slots = s->nslots;
  out->queued = s->queue.size();
  out->completed = s->completed;
  out->launched = s->launched;
  out->max_inflight = s->max_inflight;
  out->resident_bytes = s->resident;
  out->scratch_bytes = s->scratch;
  out->hbm_cap_bytes = s->cap;
  return EH_OK;
}

void eh_server_free(eh_server_t sh) {
  Server* s = reinterpret_cast<Server*>(sh);
  if (!s) return;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->dispatcher.joinable()) s->dispatcher.join();
  cudaSetDevice(s->device);
  for (auto& sl : s->slots) {
    if (sl.st) cudaStreamSynchronize(sl.st);
    if (sl.ev) cudaEventDestroy(sl.ev);
    if (sl.st) cudaStreamDestroy(sl.st);
    cudaFree(sl.ws.counters);
    if (sl.ws.clique_scratch) cudaFreeAsync(sl.ws.clique_scratch, nullptr);
    cudaFree(sl.d_out);
    if (sl.h_out) cudaFreeHost(sl.h_out);
  }
  for (auto& g : s->graphs) {
    eh_matrix_free(reinterpret_cast<eh_matrix_t>(g.low));
    eh_matrix_free(reinterpret_cast<eh_matrix_t>(g.all));
  }
  delete s;
}

}  // extern "C"
