// noalloc.cu — a join entry point that allocates no memory.
//
// Some callers cannot call cudaMalloc while they match: code that runs
// between the graph capture and replay of a larger CUDA application, callers
// whose allocator is owned by a framework or a real-time loop that must not
// allocate after start-up.  smg_join_noalloc serves them: it runs the same
// persistent join kernel as smg_match, but its scratch (the task queue, its
// ready flags, the queue state, the query record and the counters) lives in
// file-scope __device__ arrays of fixed size (about 10 MB) in the library's
// device image.  The caller passes the inputs (candidate masks and root
// candidates in device memory it owns) and receives the count.
//
// Host code must never hand the arrays' names to a kernel: in host code they
// are stand-ins, not device addresses.  The first call on each device looks
// the addresses up with cudaGetSymbolAddress (with that device current) and
// keeps them.  Under lazy module loading (CUDA_MODULE_LOADING=LAZY, the
// default) that lookup is also what loads this file's device image, arrays
// included, onto the device; either way, make the first call on a device
// before any stream capture.  All calls on a device share the one set of
// arrays: every call clears what must start at zero, and calls that overlap
// on the GPU (two host threads, two streams) race on them.
//
// The queue is linear: its SMG_NOALLOC_MAX_TASKS slots are a budget for the
// whole call, not for the tasks waiting at one time.  Root tasks take at most
// an eighth of them; each task a busy warp splits off for an idle one takes
// another.  Once the slots are spent, warps stop splitting work and each
// finishes its own tasks: the count stays exact, but a skewed query then runs
// with less load balancing than under smg_match.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
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
// queue use of the last call per device: slots taken, tasks split off, and
// whether a split found the slots spent
std::map<int, std::array<unsigned long long, 3>> g_last;

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
  // tasks are 4 + k words: the array, sized for k = 32, holds the cap at any k
  jl.kmax = P.k;
  jl.qs = sc.qs;
  jl.tasks = sc.tasks;
  jl.ready = sc.ready;
  jl.cap = SMG_NOALLOC_MAX_TASKS;
  // root tasks: two per resident join warp (4 blocks of 8 warps per SM), at
  // most an eighth of the slots, so that most slots are left for splitting
  jl.max_seed_tasks = std::min<uint32_t>(SMG_NOALLOC_MAX_TASKS / 8, 2u * 32u * static_cast<uint32_t>(c->num_sms));
  jl.donate_min = 2;
  jl.time_limit_ns = time_limit_ns();
  st = launch_join(jl, s, c->num_sms);
  if (st) return st;
  unsigned long long *hcount = reinterpret_cast<unsigned long long *>(hroots + 2);
  // behind the query record, the root count and the count in the staging buffer
  QueueState *hq = reinterpret_cast<QueueState *>(static_cast<char *>(c->pinned) +
                                                  ((sizeof(JoinQuery) + 64 + 255) & ~static_cast<size_t>(255)));
  SMG_CUDA(cudaMemcpyAsync(hcount, &sc.cnt->count, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
  SMG_CUDA(cudaMemcpyAsync(hq, sc.qs, sizeof(QueueState), cudaMemcpyDeviceToHost, s));
  SMG_CUDA(cudaStreamSynchronize(s));
  {
    std::lock_guard<std::mutex> lock(g_mu);
    g_last[c->device] = {hq->tail.v, hq->donations, static_cast<unsigned long long>(hq->full)};
  }
  if (hq->error) {
    // the same statuses as smg_match (api.cu): a full queue is a size limit,
    // every other stop a bounded wait or the time limit running out
    const char *why = hq->error == JOIN_ERR_DEADLINE       ? "join exceeded its time limit (SMG_TIME_LIMIT_S)"
                      : hq->error == JOIN_ERR_IDLE_TIMEOUT ? "join made no progress for too long"
                      : hq->error == JOIN_ERR_QUEUE_FULL   ? "join task queue full"
                                                           : "a queued task was never published";
    return fail(hq->error == JOIN_ERR_QUEUE_FULL ? SMG_ERR_LIMIT : SMG_ERR_TIMEOUT, why);
  }
  if (hq->pending.v != 0) return fail(SMG_ERR_INTERNAL, "join ended with pending tasks");
  *count = *hcount;
  return SMG_OK;
}

// Test hook (not part of smg.h): queue use of the last smg_join_noalloc call
// on `device`: out[0] slots taken (root tasks and split-off tasks), out[1]
// tasks split off for idle warps, out[2] 1 when a split found the slots spent.
extern "C" int smg_debug_noalloc_queue(int device, unsigned long long *out) {
  std::lock_guard<std::mutex> lock(g_mu);
  auto it = g_last.find(device);
  if (!out || it == g_last.end()) return 1;
  for (int i = 0; i < 3; ++i) out[i] = it->second[i];
  return 0;
}
