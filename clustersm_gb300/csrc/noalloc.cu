// noalloc.cu — a join entry point that allocates no memory.
//
// Some callers cannot call cudaMalloc while they match: code that runs
// between the graph capture and replay of a larger CUDA application, callers
// whose allocator is owned by a framework or a real-time loop that must not
// allocate after start-up.  smg_join_noalloc serves them: it runs the same
// persistent join kernel as smg_match, but its scratch (the task queue, its
// ready flags, the queue state, the query record and the counters) lives in
// file-scope __device__ arrays of fixed size, loaded with the library.  The
// caller passes the inputs (candidate masks and root candidates in device
// memory it owns) and receives the count.
//
// Host code must never hand the arrays' names to a kernel: in host code they
// are stand-ins, not device addresses.  The first call on each device looks
// the addresses up with cudaGetSymbolAddress (with that device current) and
// keeps them; make that first call before any stream capture.  All calls on a
// device share the one set of arrays: every call clears what must start at
// zero, and calls that overlap on the GPU (two host threads, two streams)
// race on them.
#include <cuda_runtime.h>

#include <cstring>
#include <map>
#include <mutex>

#include "api_internal.cuh"

namespace {

constexpr uint32_t kTW = 4 + smg::kMaxK;  // task words for queries of up to 32 vertices

__device__ __align__(256) uint32_t g_na_tasks[static_cast<size_t>(SMG_NOALLOC_MAX_TASKS) * kTW];
__device__ __align__(256) uint32_t g_na_ready[SMG_NOALLOC_MAX_TASKS];
__device__ __align__(256) smg::QueueState g_na_queue;
__device__ __align__(256) smg::JoinQuery g_na_query;
__device__ __align__(256) smg::QCounters g_na_counters;

struct Scratch {
  uint32_t *tasks = nullptr, *ready = nullptr;
  smg::QueueState *qs = nullptr;
  smg::JoinQuery *jq = nullptr;
  smg::QCounters *cnt = nullptr;
};

std::mutex g_mu;
std::map<int, Scratch> g_scratch;  // per device

smg_status scratch_for(int device, Scratch &out) {
  std::lock_guard<std::mutex> lock(g_mu);
  auto it = g_scratch.find(device);
  if (it != g_scratch.end()) {
    out = it->second;
    return SMG_OK;
  }
  Scratch s;
  SMG_CUDA(cudaGetSymbolAddress(reinterpret_cast<void **>(&s.tasks), g_na_tasks));
  SMG_CUDA(cudaGetSymbolAddress(reinterpret_cast<void **>(&s.ready), g_na_ready));
  SMG_CUDA(cudaGetSymbolAddress(reinterpret_cast<void **>(&s.qs), g_na_queue));
  SMG_CUDA(cudaGetSymbolAddress(reinterpret_cast<void **>(&s.jq), g_na_query));
  SMG_CUDA(cudaGetSymbolAddress(reinterpret_cast<void **>(&s.cnt), g_na_counters));
  g_scratch[device] = s;
  out = s;
  return SMG_OK;
}

}  // namespace

extern "C" smg_status smg_join_noalloc(smg_ctx *c, const smg_graph *G, const smg_plan *p, const uint32_t *candmask,
                                       const uint32_t *roots, uint32_t num_roots, uint64_t *count) {
  using namespace smg;
  if (!c || !G || !p || !count || (G->g.n && !candmask) || (num_roots && !roots))
    return fail(SMG_ERR_INVALID, "null argument");
  if (G->device != c->device) return fail(SMG_ERR_INVALID, "graph lives on another device");
  const Plan &P = p->p;
  if (P.k > kMaxK) return fail(SMG_ERR_LIMIT, "smg_join_noalloc takes queries of at most 32 vertices");
  if (num_roots > G->g.n) return fail(SMG_ERR_LIMIT, "more root candidates than data vertices");
  SMG_CUDA(cudaSetDevice(c->device));
  Scratch sc;
  smg_status st = scratch_for(c->device, sc);
  if (st) return st;
  cudaStream_t s = c->stream;
  // the query record and the root count go through the context's staging
  // buffer (page-locked when the context was opened)
  JoinQuery *hj = static_cast<JoinQuery *>(c->pinned);
  uint32_t *hroots = reinterpret_cast<uint32_t *>(hj + 1);
  std::memset(hj, 0, sizeof(*hj));
  hj->k = P.k;
  for (uint32_t l = 0; l < P.k; ++l) {
    hj->order[l] = P.order[l];
    hj->back_mask[l] = P.back_mask[l];
    hj->same_label[l] = P.same_label_mask[l];
  }
  hj->candmask = candmask;
  hj->roots = roots;
  hj->num_roots = &sc.cnt->num_roots;
  hj->count = &sc.cnt->count;
  hj->emb_count = &sc.cnt->emb_count;
  hj->over = &sc.cnt->over;
  hj->pending = &sc.cnt->pending;
  *hroots = num_roots;
  SMG_CUDA(cudaMemsetAsync(sc.qs, 0, sizeof(QueueState), s));
  SMG_CUDA(cudaMemsetAsync(sc.ready, 0, static_cast<size_t>(SMG_NOALLOC_MAX_TASKS) * sizeof(uint32_t), s));
  SMG_CUDA(cudaMemsetAsync(sc.cnt, 0, sizeof(QCounters), s));
  SMG_CUDA(cudaMemcpyAsync(sc.jq, hj, sizeof(JoinQuery), cudaMemcpyHostToDevice, s));
  SMG_CUDA(cudaMemcpyAsync(&sc.cnt->num_roots, hroots, sizeof(uint32_t), cudaMemcpyHostToDevice, s));
  JoinLaunch jl;
  std::memset(&jl, 0, sizeof(jl));
  set_graph(jl, G->g);
  jl.queries = sc.jq;
  jl.nq = 1;
  jl.kmax = kMaxK;
  jl.qs = sc.qs;
  jl.tasks = sc.tasks;
  jl.ready = sc.ready;
  jl.cap = SMG_NOALLOC_MAX_TASKS;
  jl.max_seed_tasks = SMG_NOALLOC_MAX_TASKS / 4;  // root tasks leave room for load balancing
  jl.donate_min = 2;
  jl.time_limit_ns = time_limit_ns();
  st = launch_join(jl, s, c->num_sms);
  if (st) return st;
  unsigned long long *hcount = reinterpret_cast<unsigned long long *>(hroots + 2);
  int *herr = reinterpret_cast<int *>(hcount + 1);
  SMG_CUDA(cudaMemcpyAsync(hcount, &sc.cnt->count, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
  SMG_CUDA(cudaMemcpyAsync(herr, &sc.qs->error, sizeof(int), cudaMemcpyDeviceToHost, s));
  SMG_CUDA(cudaStreamSynchronize(s));
  if (*herr) return fail(SMG_ERR_TIMEOUT, "join stopped at a bounded wait or its time limit");
  *count = *hcount;
  return SMG_OK;
}
