// serve.cpp — continuous-batching request loop over a resident data graph.
//
// The reference has no serving mode: runClusterSM.sh starts one process per
// query and re-reads the data graph each time (runClusterSM.sh:9-13).  Here
// the data graph stays resident and requests flow through one shared,
// persistent work queue:
//
//   * a request is admitted into a slot when a slot is free and its device
//     state (candidate masks, cluster bitmap, candidate lists) fits the memory
//     budget; admission order is arrival order;
//   * newly admitted queries are filtered together and their root tasks are
//     appended to the live queue.  By default this happens while a slice
//     runs: on a second stream, the filter kernels take the SM room the join
//     leaves (3 of its 4 blocks per SM), and the seeds join the running
//     queue, whose waiting warps pick them up.  A host-mapped hold word keeps
//     the join's warps waiting, rather than leaving, while the queue is
//     empty but more work may be appended; the host clears it when nothing is
//     running or waiting.  Slots and memory a request frees during a slice
//     are reused only after the slice, so that no SM can hold a stale cached
//     line of the previous tenant's records or bitmaps.  SMG_SERVE_LIVE=0
//     admits only between slices;
//   * the join runs in slices.  A slice ends when its work is done, after
//     SMG_SLICE_MS (default 1,000 ms; 250 ms with SMG_SERVE_LIVE=0), or, once
//     SMG_SLICE_MIN_MS (default 2 ms) have passed, when the host rings a
//     doorbell in host-mapped memory: without live admission because
//     requests are waiting and slots are free, with it when the queue has
//     used half its slots, or when requests wait that no free slot or memory
//     can take while at least as many requests retired in the slice are held
//     as still run.  At the end of a slice every warp writes the
//     unfinished part of its depth-first stack into the next slice's queue,
//     and the untaken tasks follow;
//   * a query is finished when its count of queued and running tasks reaches
//     zero.  The warp that brings it there writes the final count to a
//     host-mapped completion record, so the host retires the request (and
//     frees its slot and memory) while the slice is still running.
//
// smg_server_step never blocks while a slice is on the device; between
// slices it synchronises once (counters, queue state, admission staging).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <string>
#include <memory>
#include <thread>
#include <unordered_set>

#include "api_internal.cuh"

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}


struct Request {
  uint64_t ticket;
  const smg::Plan *plan;
  double submit_s;
  uint64_t bytes;
};

struct Slot {
  bool used = false;
  bool held = false;         // retired during a live slice; free once it ends
  uint64_t ticket = 0;
  uint32_t gen = 0;          // admission number, echoed by the completion record
  const smg::Plan *plan = nullptr;
  size_t off = 0, size = 0;  // pool range
  double submit_s = 0, start_s = 0;
};

// Host-mapped completion record of one slot (written by the join).
struct alignas(16) Done {
  unsigned long long count;
  uint32_t gen;
  uint32_t pad;
};

// First-fit allocator over one device buffer, with coalescing frees.
struct Pool {
  char *base = nullptr;
  size_t size = 0;
  std::map<size_t, size_t> free_;  // offset -> length
  void init(char *b, size_t s) {
    base = b;
    size = s;
    free_.clear();
    free_[0] = s;
  }
  bool alloc(size_t n, size_t &off) {
    n = (n + 255) & ~size_t(255);
    for (auto it = free_.begin(); it != free_.end(); ++it)
      if (it->second >= n) {
        off = it->first;
        const size_t rest = it->second - n;
        free_.erase(it);
        if (rest) free_[off + n] = rest;
        return true;
      }
    return false;
  }
  void release(size_t off, size_t n) {
    n = (n + 255) & ~size_t(255);
    auto it = free_.emplace(off, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
};

}  // namespace

struct smg_server {
  smg_ctx *ctx = nullptr;
  int device = 0;
  const smg_graph *graph = nullptr;
  smg_server_config cfg{};
  uint64_t next_ticket = 1;
  uint32_t next_gen = 0;
  std::deque<Request> waiting;
  std::vector<Slot> slots;
  uint32_t free_slots = 0;
  uint32_t running = 0;      // admitted requests not yet retired
  std::map<uint64_t, smg_request_result> done;  // finished, not yet collected by smg_server_poll
  std::unordered_set<uint64_t> outstanding;     // submitted, not yet finished
  Pool pool;
  // device allocations
  char *pool_mem = nullptr;
  smg::FilterQuery *d_fq_new = nullptr;  // contiguous records of the newly admitted
  smg::JoinQuery *d_jq = nullptr;        // [max_inflight], indexed by slot
  smg::QCounters *d_cnt = nullptr;       // [max_inflight]
  uint32_t *d_seed = nullptr;            // slots to seed
  // what an admission clears (launch_zero_ranges): word prefix sums, then byte
  // offsets from zero_base, of up to zplan_cap ranges
  uint64_t *d_zplan = nullptr;
  size_t zplan_cap = 0;
  uint32_t *tasks[2] = {nullptr, nullptr};
  uint32_t *ready[2] = {nullptr, nullptr};
  unsigned int *next_count = nullptr;    // tasks preempted into the other queue
  uint32_t *xbuf = nullptr;              // the join warps' hoisted-set buffers
  smg::QueueState *qs = nullptr;
  unsigned int *walk_count = nullptr;
  uint4 *walk_items = nullptr;
  uint32_t cap = 0, cur = 0;
  // admission into the running slice (SMG_SERVE_LIVE, default on)
  bool live = true;
  cudaStream_t s2 = nullptr;        // its stream
  cudaEvent_t ev_admit = nullptr;   // the last admission's work on s2
  bool admitting = false;           // that work may still be running
  uint32_t join_blocks = 3;         // join blocks per SM while admitting live
  void *stage = nullptr;            // page-locked staging of admissions
  uint32_t *h_hold = nullptr, *d_hold = nullptr;
  unsigned long long *h_tail = nullptr;  // the live queue's tail, read after each admission
  std::vector<std::pair<size_t, size_t>> freed_mem;  // released at the end of the slice
  std::vector<uint32_t> freed_slots;
  uint32_t kmax = smg::kMaxK;  // task width: the largest query accepted
  uint32_t admit_batch = 1;    // free slots that ring the doorbell (SMG_ADMIT_BATCH; default an eighth)
  uint64_t slice_ns = 0, slice_min_ns = 0;
  cudaEvent_t ev = nullptr;
  bool inflight = false, bell_rung = false;
  double slice_start_s = 0;
  smg_server_stats stats{};
  uint64_t slices = 0;
  smg::FilterDev fdev;
  // page-locked host memory: counters and queue state read back between
  // slices; the doorbell and the completion records are also mapped into the
  // device's address space
  smg::QCounters *h_cnt = nullptr;
  smg::QueueState *h_qs = nullptr;
  uint32_t *h_bell = nullptr, *d_bell = nullptr;
  Done *h_done = nullptr, *d_done = nullptr;

  // The context may already be closed (closing it synchronised its stream),
  // so only the device is used here.
  ~smg_server() {
    cudaSetDevice(device);
    cudaDeviceSynchronize();
    for (void *p : {static_cast<void *>(pool_mem), static_cast<void *>(d_fq_new), static_cast<void *>(d_jq),
                    static_cast<void *>(d_cnt), static_cast<void *>(d_seed), static_cast<void *>(d_zplan),
                    static_cast<void *>(tasks[0]),
                    static_cast<void *>(tasks[1]), static_cast<void *>(ready[0]), static_cast<void *>(ready[1]),
                    static_cast<void *>(next_count), static_cast<void *>(qs), static_cast<void *>(walk_count),
                    static_cast<void *>(walk_items), static_cast<void *>(xbuf)})
      if (p) cudaFree(p);
    for (void *p : {static_cast<void *>(h_cnt), static_cast<void *>(h_qs), static_cast<void *>(h_bell),
                    static_cast<void *>(h_done), stage, static_cast<void *>(h_hold), static_cast<void *>(h_tail)})
      if (p) cudaFreeHost(p);
    if (ev) cudaEventDestroy(ev);
    if (ev_admit) cudaEventDestroy(ev_admit);
    if (s2) cudaStreamDestroy(s2);
  }
};

namespace {

using smg::fail;

uint32_t task_words(const smg_server *s) { return 4 + s->kmax; }

smg::WalkOverflow walk_overflow(smg_server *s) {
  smg::WalkOverflow w;
  w.count = s->walk_count;
  w.cap = smg::kWalkCap;
  w.items = s->walk_items;
  return w;
}

smg::JoinLaunch join_launch(smg_server *s) {
  const smg::DevGraph &g = s->graph->g;
  smg::JoinLaunch jl;
  std::memset(&jl, 0, sizeof(jl));
  smg::set_graph(jl, g);
  jl.queries = s->d_jq;
  jl.nq = s->cfg.max_inflight;
  jl.kmax = s->kmax;
  jl.qs = s->qs;
  jl.tasks = s->tasks[s->cur];
  jl.ready = s->ready[s->cur];
  jl.cap = s->cap;
  jl.max_seed_tasks = 256;
  jl.donate_min = 2;
  jl.time_limit_ns = smg::time_limit_ns();
  jl.slice_ns = s->slice_ns;
  jl.slice_min_ns = s->slice_min_ns;
  jl.bell = s->d_bell;
  jl.next_tasks = s->tasks[1 - s->cur];
  jl.next_ready = s->ready[1 - s->cur];
  jl.next_count = s->next_count;
  jl.xbuf = s->xbuf;
  jl.xcap = smg::hoist_global_cap();
  if (s->live) {
    jl.hold = s->d_hold;
    jl.max_blocks_per_sm = s->join_blocks;
  }
  return jl;
}

bool any_active(const smg_server *s) { return s->running > 0; }

// Empty queue: head = tail = pending = 0, every ready flag clear.
smg_status reset_queue(smg_server *s) {
  cudaStream_t st = s->ctx->stream;
  SMG_CUDA(cudaMemsetAsync(s->qs, 0, sizeof(smg::QueueState), st));
  SMG_CUDA(cudaMemsetAsync(s->ready[0], 0, static_cast<size_t>(s->cap) * 4, st));
  SMG_CUDA(cudaMemsetAsync(s->ready[1], 0, static_cast<size_t>(s->cap) * 4, st));
  SMG_CUDA(cudaMemsetAsync(s->next_count, 0, sizeof(unsigned int), st));
  s->cur = 0;
  return SMG_OK;
}

void retire(smg_server *s, Slot &sl, smg_status status, uint64_t count) {
  smg_request_result r{};
  r.status = status;
  r.count = status ? 0 : count;
  r.submit_s = sl.submit_s;
  r.start_s = sl.start_s;
  r.finish_s = now_s();
  s->done[sl.ticket] = r;
  s->outstanding.erase(sl.ticket);
  --s->running;
  if (s->live && s->inflight) {
    // the running join may have this slot's records and bitmaps cached:
    // they are reused only after the slice
    s->freed_mem.emplace_back(sl.off, sl.size);
    s->freed_slots.push_back(static_cast<uint32_t>(&sl - s->slots.data()));
    sl = Slot();
    sl.used = true;
    sl.held = true;
    return;
  }
  s->pool.release(sl.off, sl.size);
  sl = Slot();
  ++s->free_slots;
}

// Slots and memory retired during the slice just ended become free.
void release_freed(smg_server *s) {
  for (const auto &m : s->freed_mem) s->pool.release(m.first, m.second);
  for (uint32_t i : s->freed_slots) {
    s->slots[i] = Slot();
    ++s->free_slots;
  }
  s->freed_mem.clear();
  s->freed_slots.clear();
}

// Retires the requests whose completion records the join has published.
void poll_done(smg_server *s) {
  for (Slot &sl : s->slots) {
    if (!sl.used || sl.held) continue;
    const uint32_t i = static_cast<uint32_t>(&sl - s->slots.data());
    if (__atomic_load_n(&s->h_done[i].gen, __ATOMIC_ACQUIRE) != sl.gen) continue;
    retire(s, sl, SMG_OK, __atomic_load_n(&s->h_done[i].count, __ATOMIC_RELAXED));
    if (s->inflight) ++s->stats.retired_in_slice;
  }
}

// While a slice runs: ring the doorbell once requests wait and enough slots
// are free to admit them in a batch (SMG_ADMIT_BATCH, default an eighth of
// the slots), or any slot is
// free and the slice has run 10 ms, so that the slice closes and the next one
// admits them.  (The device closes a slice no earlier than SMG_SLICE_MIN_MS.)
void maybe_ring(smg_server *s) {
  if (s->bell_rung || s->waiting.empty() || s->free_slots == 0) return;
  const uint32_t want = s->admit_batch;
  if (s->free_slots >= want || now_s() - s->slice_start_s > 0.010) {
    __atomic_store_n(s->h_bell, 1u, __ATOMIC_RELEASE);
    s->bell_rung = true;
    ++s->stats.bells;
  }
}

// After a slice: move untaken and preempted tasks into the other queue (on
// the device; the one just run becomes the next preemption target).
smg_status end_slice(smg_server *s) {
  cudaStream_t st = s->ctx->stream;
  const uint32_t other = 1 - s->cur;
  smg_status rc = smg::launch_compact(s->tasks[s->cur], s->ready[s->cur], s->cap, task_words(s), s->tasks[other],
                                      s->ready[other], s->next_count, s->qs, st, s->ctx->num_sms);
  if (rc) return rc;
  SMG_CUDA(cudaMemsetAsync(s->ready[s->cur], 0, static_cast<size_t>(s->cap) * 4, st));
  s->cur = other;
  return SMG_OK;
}

// Admit waiting requests (arrival order) while slots and memory allow; filter
// them together and append their root tasks to the live queue.  Only
// enqueues: the caller synchronises once for admission and read-back.
smg_status admit(smg_server *s, cudaStream_t st) {
  const smg::DevGraph &g = s->graph->g;
  std::vector<uint32_t> fresh;
  std::vector<smg::QueryFootprint> fps;
  const double t = now_s();
  uint32_t idx = 0;
  while (!s->waiting.empty() && s->free_slots) {
    while (s->slots[idx].used) ++idx;
    const Request &r = s->waiting.front();
    const smg::QueryFootprint fp = smg::query_footprint(g, *r.plan);
    size_t off = 0;
    if (!s->pool.alloc(fp.total(), off)) break;  // wait for memory to free up
    Slot &sl = s->slots[idx];
    sl.used = true;
    sl.ticket = r.ticket;
    sl.gen = ++s->next_gen;
    sl.plan = r.plan;
    sl.off = off;
    sl.size = fp.total();
    sl.submit_s = r.submit_s;
    sl.start_s = t;
    --s->free_slots;
    ++s->running;
    ++s->stats.admitted;
    s->waiting.pop_front();
    fresh.push_back(idx);
    fps.push_back(fp);
  }
  if (fresh.empty()) return SMG_OK;
  const uint32_t n = static_cast<uint32_t>(fresh.size());
  smg::FilterQuery *hf = static_cast<smg::FilterQuery *>(s->stage);
  smg::JoinQuery *hj = reinterpret_cast<smg::JoinQuery *>(hf + n);
  uint32_t *hseed = reinterpret_cast<uint32_t *>(hj + n);
  // What the admitted requests' filter and join read must start at zero: the
  // counters, the candidate bitmaps, and the masks and cluster bitmap over
  // the positions of each request's label groups.  Offsets are from the
  // lower of the two allocations involved.
  char *const zbase = reinterpret_cast<uintptr_t>(s->pool.base) < reinterpret_cast<uintptr_t>(s->d_cnt)
                          ? s->pool.base
                          : reinterpret_cast<char *>(s->d_cnt);
  std::vector<std::pair<uint64_t, uint64_t>> zr;  // (byte offset from zbase, bytes)
  smg::FilterBatch fb;
  for (uint32_t i = 0; i < n; ++i) {
    const uint32_t idx = fresh[i];
    const Slot &sl = s->slots[idx];
    char *base = s->pool.base + sl.off;
    smg::QueryBuffers b;
    b.vmask = reinterpret_cast<uint32_t *>(base);
    b.enc = reinterpret_cast<uint32_t *>(base + fps[i].vmask);
    b.cand = reinterpret_cast<uint32_t *>(base + fps[i].vmask + fps[i].enc);
    b.roots = reinterpret_cast<uint32_t *>(base + fps[i].vmask + fps[i].enc + fps[i].cand);
    b.cbits = reinterpret_cast<uint32_t *>(base + fps[i].vmask + fps[i].enc + fps[i].cand + fps[i].roots);
    b.counters = s->d_cnt + idx;
    smg_status rc = smg::make_query_records(*sl.plan, g, b, 0, hf[i], hj[i]);
    if (rc) return rc;
    const smg::TuneSetting &tune = s->ctx->tuning[smg::plan_class(*sl.plan)];
    if (tune.valid) smg::apply_tuning(tune, hj[i]);
    hj[i].done_count = &s->d_done[idx].count;
    hj[i].done_gen = &s->d_done[idx].gen;
    hj[i].gen = sl.gen;
    rc = smg::append_filter_steps(*sl.plan, i, fb);
    if (rc) return rc;
    hseed[i] = idx;
    const uint64_t W = sl.plan->num_words;
    auto at = [&](const void *p) {
      return static_cast<uint64_t>(reinterpret_cast<uintptr_t>(p) - reinterpret_cast<uintptr_t>(zbase));
    };
    for (uint32_t gi = 0; gi < hf[i].ngrp; ++gi) {
      const uint64_t lo = hf[i].grp_lo[gi], hi = hf[i].grp_hi[gi];
      if (hi <= lo || hi > g.n) continue;
      zr.emplace_back(at(b.enc) + lo * W * 4, (hi - lo) * W * 4);
      zr.emplace_back(at(b.vmask) + lo * 4, (hi - lo) * 4);
    }
    if (fps[i].cbits) zr.emplace_back(at(b.cbits), fps[i].cbits);
    zr.emplace_back(at(b.counters), sizeof(smg::QCounters));
    SMG_CUDA(cudaMemcpyAsync(s->d_jq + idx, hj + i, sizeof(smg::JoinQuery), cudaMemcpyHostToDevice, st));
  }
  // one kernel clears them all, with 256-thread blocks that fit beside a
  // running join (live admission)
  std::sort(zr.begin(), zr.end());
  if (zr.size() > s->zplan_cap) return fail(SMG_ERR_INTERNAL, "admission clears more ranges than planned");
  {
    const uintptr_t pa = (reinterpret_cast<uintptr_t>(hseed + n) + 7) & ~static_cast<uintptr_t>(7);
    uint64_t *hz = reinterpret_cast<uint64_t *>(pa);
    const size_t nr = zr.size();
    hz[0] = 0;
    for (size_t r = 0; r < nr; ++r) {
      hz[r + 1] = hz[r] + zr[r].second / 4;
      hz[nr + 1 + r] = zr[r].first;
    }
    SMG_CUDA(cudaMemcpyAsync(s->d_zplan, hz, (2 * nr + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
    smg_status zrc = smg::launch_zero_ranges(zbase, s->d_zplan, s->d_zplan + nr + 1, static_cast<uint32_t>(nr), st,
                                             s->ctx->num_sms);
    if (zrc) return zrc;
  }
  smg_status rc = s->fdev.upload(fb, st);
  if (rc) return rc;
  SMG_CUDA(cudaMemcpyAsync(s->d_fq_new, hf, n * sizeof(smg::FilterQuery), cudaMemcpyHostToDevice, st));
  SMG_CUDA(cudaMemcpyAsync(s->d_seed, hseed, n * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
  rc = smg::launch_zero(s->walk_count, smg::kMaxWalkPhases * 2 * sizeof(unsigned int), st, s->ctx->num_sms);
  if (rc) return rc;
  rc = smg::launch_filter(g, s->d_fq_new, n, s->fdev, walk_overflow(s), st, s->ctx->num_sms);
  if (rc) return rc;
  smg::JoinLaunch jl = join_launch(s);
  jl.seed_list = s->d_seed;
  jl.seed_n = n;
  rc = smg::launch_join_prep(jl, st, s->ctx->num_sms);
  if (rc) return rc;
  return smg::launch_seed(jl, st);
}

// Between slices: admit, read every slot's counters and the queue state back
// (one synchronisation, which also releases the admission's pinned staging),
// retire what finished (queries without root candidates never run a task),
// and fail every active request if the join reported an error.
smg_status settle(smg_server *s) {
  cudaStream_t st = s->ctx->stream;
  release_freed(s);
  smg_status rc = admit(s, st);
  if (rc) return rc;
  SMG_CUDA(cudaMemcpyAsync(s->h_cnt, s->d_cnt, s->slots.size() * sizeof(smg::QCounters), cudaMemcpyDeviceToHost,
                           st));
  SMG_CUDA(cudaMemcpyAsync(s->h_qs, s->qs, sizeof(smg::QueueState), cudaMemcpyDeviceToHost, st));
  SMG_CUDA(cudaStreamSynchronize(st));
  s->stats.carried_tasks += s->h_qs->tail.v;  // the queue the next slice starts with
  poll_done(s);
  if (s->h_qs->error) {
    const smg_status why = s->h_qs->error == smg::JOIN_ERR_QUEUE_FULL ? SMG_ERR_LIMIT : SMG_ERR_TIMEOUT;
    for (Slot &sl : s->slots)
      if (sl.used && !sl.held) retire(s, sl, why, 0);
    return reset_queue(s);
  }
  for (size_t i = 0; i < s->slots.size(); ++i) {
    Slot &sl = s->slots[i];
    if (sl.used && !sl.held && s->h_cnt[i].pending == 0) retire(s, sl, SMG_OK, s->h_cnt[i].count);
  }
  if (!any_active(s)) return reset_queue(s);
  return SMG_OK;
}

smg_status launch_slice(smg_server *s) {
  cudaStream_t st = s->ctx->stream;
  __atomic_store_n(s->h_bell, 0u, __ATOMIC_RELEASE);
  s->bell_rung = false;
  if (s->live) __atomic_store_n(s->h_hold, 1u, __ATOMIC_RELEASE);  // live admission may append work
  smg_status rc = smg::launch_slice_begin(s->qs, st);
  if (rc) return rc;
  rc = smg::launch_join_only(join_launch(s), st, s->ctx->num_sms);
  if (rc) return rc;
  SMG_CUDA(cudaEventRecord(s->ev, st));
  s->inflight = true;
  s->slice_start_s = now_s();
  ++s->slices;
  return SMG_OK;
}

// While a slice runs with live admission: finish the last admission (and
// read the queue's tail it left), admit waiting requests into the running
// queue on the second stream, ring the doorbell when the queue has used half
// its slots, and clear the hold once nothing is running, waiting or being
// admitted (then the join leaves when its queue drains, and later requests
// start the next slice).
smg_status live_step(smg_server *s) {
  if (s->admitting) {
    const cudaError_t e = cudaEventQuery(s->ev_admit);
    if (e == cudaErrorNotReady) return SMG_OK;
    if (e != cudaSuccess) return smg::cuda_fail(e, "server admission");
    s->admitting = false;
    if (*s->h_tail > s->cap / 2 && !s->bell_rung) {
      __atomic_store_n(s->h_bell, 1u, __ATOMIC_RELEASE);
      s->bell_rung = true;
      ++s->stats.bells;
    }
  }
  const bool open = __atomic_load_n(s->h_hold, __ATOMIC_ACQUIRE) != 0;
  if (open && !s->bell_rung && !s->waiting.empty() && s->free_slots) {
    const uint64_t before = s->stats.admitted;
    smg_status rc = admit(s, s->s2);
    if (rc) return rc;
    if (s->stats.admitted != before) {
      s->stats.admitted_live += s->stats.admitted - before;
      SMG_CUDA(cudaMemcpyAsync(s->h_tail, &s->qs->tail.v, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s->s2));
      SMG_CUDA(cudaEventRecord(s->ev_admit, s->s2));
      s->admitting = true;
    }
  }
  // Slots retired during the slice are held until it ends.  When requests
  // still wait after the admission above (no free slot, or no memory), end
  // the slice once at least as many requests are held as still run: ending
  // a slice hands every running warp's stack back as tasks, so it pays only
  // once a good part of the admitted work is done (ringing at every eighth
  // of the slots held measured 449 queries/s under overload, against 634
  // for no ringing at all).
  if (open && !s->admitting && !s->bell_rung && !s->waiting.empty() && !s->freed_slots.empty() &&
      s->freed_slots.size() >= s->running) {
    __atomic_store_n(s->h_bell, 1u, __ATOMIC_RELEASE);
    s->bell_rung = true;
    ++s->stats.bells;
  }
  if (open && !s->admitting && s->waiting.empty() && s->running == 0)
    __atomic_store_n(s->h_hold, 0u, __ATOMIC_RELEASE);
  return SMG_OK;
}

smg_status step(smg_server *s) {
  SMG_CUDA(cudaSetDevice(s->ctx->device));
  if (s->inflight) {
    const cudaError_t e = cudaEventQuery(s->ev);
    if (e == cudaErrorNotReady) {
      poll_done(s);
      if (s->live) return live_step(s);
      maybe_ring(s);
      return SMG_OK;
    }
    if (e != cudaSuccess) return smg::cuda_fail(e, "server slice");
    s->inflight = false;
    s->stats.slice_s += now_s() - s->slice_start_s;
    if (s->admitting) {
      // its seeds may have landed after the join left: the compaction moves them
      SMG_CUDA(cudaStreamWaitEvent(s->ctx->stream, s->ev_admit, 0));
      s->admitting = false;
    }
    poll_done(s);  // completions written during the slice, before their slots are freed
    smg_status rc = end_slice(s);
    if (rc) return rc;
  } else if (s->waiting.empty() && !any_active(s)) {
    return SMG_OK;  // idle
  }
  const double t0 = now_s();
  smg_status rc = settle(s);
  if (rc) return rc;
  if (any_active(s)) rc = launch_slice(s);
  s->stats.between_s += now_s() - t0;
  return rc;
}

double env_ms(const char *name, double dflt) {
  const char *v = std::getenv(name);
  const double x = v ? std::atof(v) : dflt;
  return x > 0 ? x : dflt;
}

}  // namespace

extern "C" {

smg_status smg_server_create(smg_ctx *c, const smg_graph *g, const smg_server_config *cfg, smg_server **out) {
  if (!c || !g || !out) return fail(SMG_ERR_INVALID, "null argument");
  *out = nullptr;
  SMG_CUDA(cudaSetDevice(c->device));
  std::unique_ptr<smg_server> s(new smg_server);
  s->ctx = c;
  s->device = c->device;
  s->graph = g;
  if (cfg) s->cfg = *cfg;
  if (!s->cfg.max_inflight) s->cfg.max_inflight = 64;
  if (s->cfg.max_query_vertices) {
    if (s->cfg.max_query_vertices < 2 || s->cfg.max_query_vertices > smg::kMaxK)
      return fail(SMG_ERR_INVALID, "max_query_vertices must be 2..32 (0: 32)");
    s->kmax = s->cfg.max_query_vertices;
  }
  const size_t per_rec = sizeof(smg::FilterQuery) + sizeof(smg::JoinQuery) + 4;
  if (s->cfg.max_inflight * per_rec > smg::kPinnedBytes) return fail(SMG_ERR_LIMIT, "max_inflight too large");
  size_t free_b = 0, total_b = 0;
  SMG_CUDA(cudaMemGetInfo(&free_b, &total_b));
  if (!s->cfg.memory_budget_bytes) s->cfg.memory_budget_bytes = std::min<size_t>(64ull << 30, free_b / 3);
  {
    const char *lv = std::getenv("SMG_SERVE_LIVE");
    s->live = !(lv && std::string(lv) == "0");
    const char *jb = std::getenv("SMG_SERVE_JOIN_BLOCKS");
    if (jb) s->join_blocks = static_cast<uint32_t>(std::max(1, std::atoi(jb)));
  }
  s->slice_ns = static_cast<uint64_t>(env_ms("SMG_SLICE_MS", s->live ? 1000.0 : 250.0) * 1e6);
  s->slice_min_ns = std::min(s->slice_ns, static_cast<uint64_t>(env_ms("SMG_SLICE_MIN_MS", 2.0) * 1e6));
  // task slots of each of the two queues.  A slice's queue is linear and the
  // doorbell ends a slice once half of it is used, so the size sets how often
  // every running warp is preempted: at 1,000 requests/s on the 2^24 R-MAT
  // graph, 2^21 slots ended 20 slices in 2 s (p50 33.6 ms, p99 208 ms), 2^23
  // slots 11 (p50 12.1 ms, p99 98.9 ms) and 2^25 slots 4 (p50 9.7 ms, p99
  // 89.9 ms).  Default: 2^25 slots, at most 4 GiB per queue.
  {
    const double tw_bytes = 4.0 * (4 + s->kmax);
    const double dflt = std::min(static_cast<double>(1u << 25), std::floor((4.0 * (1ull << 30)) / tw_bytes));
    s->cap = static_cast<uint32_t>(std::min(env_ms("SMG_SERVE_QUEUE_TASKS", dflt), static_cast<double>(1u << 28)));
  }
  s->admit_batch = std::max<uint32_t>(1, static_cast<uint32_t>(env_ms("SMG_ADMIT_BATCH", s->cfg.max_inflight / 8.0)));
  const size_t tw = task_words(s.get());
  const uint32_t m = s->cfg.max_inflight;
  // the context's batch scratch may hold the memory the server needs (it
  // grows to what the largest batch used): free it first
  if (free_b < s->cfg.memory_budget_bytes + (8ull << 30)) smg::release_batch_memory(c);
  SMG_CUDA(cudaMalloc(&s->pool_mem, s->cfg.memory_budget_bytes));
  s->pool.init(s->pool_mem, s->cfg.memory_budget_bytes);
  SMG_CUDA(cudaMalloc(&s->d_fq_new, m * sizeof(smg::FilterQuery)));
  SMG_CUDA(cudaMalloc(&s->d_jq, m * sizeof(smg::JoinQuery)));
  SMG_CUDA(cudaMalloc(&s->d_cnt, m * sizeof(smg::QCounters)));
  SMG_CUDA(cudaMalloc(&s->d_seed, m * sizeof(uint32_t)));
  // per admitted request: two ranges per label group, its bitmaps and counters
  s->zplan_cap = static_cast<size_t>(m) * (2 * s->kmax + 2);
  SMG_CUDA(cudaMalloc(&s->d_zplan, (2 * s->zplan_cap + 1) * sizeof(uint64_t)));
  for (int i = 0; i < 2; ++i) {
    SMG_CUDA(cudaMalloc(&s->tasks[i], static_cast<size_t>(s->cap) * tw * 4));
    SMG_CUDA(cudaMalloc(&s->ready[i], static_cast<size_t>(s->cap) * 4));
  }
  SMG_CUDA(cudaMalloc(&s->next_count, sizeof(unsigned int)));
  SMG_CUDA(cudaMalloc(&s->xbuf, smg::hoist_buffer_bytes(c->num_sms)));
  SMG_CUDA(cudaMalloc(&s->qs, sizeof(smg::QueueState)));
  SMG_CUDA(cudaMalloc(&s->walk_count, smg::kMaxWalkPhases * 2 * sizeof(unsigned int)));
  SMG_CUDA(cudaMalloc(&s->walk_items, static_cast<size_t>(smg::kWalkCap) * sizeof(uint4)));
  SMG_CUDA(cudaHostAlloc(&s->h_cnt, m * sizeof(smg::QCounters), cudaHostAllocDefault));
  SMG_CUDA(cudaHostAlloc(&s->h_qs, sizeof(smg::QueueState), cudaHostAllocDefault));
  SMG_CUDA(cudaHostAlloc(&s->h_bell, sizeof(uint32_t), cudaHostAllocMapped));
  SMG_CUDA(cudaHostAlloc(&s->h_done, m * sizeof(Done), cudaHostAllocMapped));
  SMG_CUDA(cudaHostAlloc(&s->stage, m * per_rec + 4096 + (2 * s->zplan_cap + 1) * sizeof(uint64_t),
                         cudaHostAllocDefault));
  SMG_CUDA(cudaHostAlloc(&s->h_hold, sizeof(uint32_t), cudaHostAllocMapped));
  SMG_CUDA(cudaHostAlloc(&s->h_tail, sizeof(unsigned long long), cudaHostAllocDefault));
  SMG_CUDA(cudaHostGetDevicePointer(reinterpret_cast<void **>(&s->d_hold), s->h_hold, 0));
  *s->h_hold = 0;
  *s->h_tail = 0;
  SMG_CUDA(cudaStreamCreateWithFlags(&s->s2, cudaStreamNonBlocking));
  SMG_CUDA(cudaEventCreateWithFlags(&s->ev_admit, cudaEventDisableTiming));
  // the filter's step tables of up to max_inflight admissions at once, sized
  // now: growing them later would free memory under a running join
  {
    smg_status rc0 = s->fdev.reserve(static_cast<size_t>(m) * 64 * 1024 + (1u << 20));
    if (rc0) return rc0;
  }
  SMG_CUDA(cudaHostGetDevicePointer(reinterpret_cast<void **>(&s->d_bell), s->h_bell, 0));
  SMG_CUDA(cudaHostGetDevicePointer(reinterpret_cast<void **>(&s->d_done), s->h_done, 0));
  *s->h_bell = 0;
  std::memset(s->h_done, 0, m * sizeof(Done));
  SMG_CUDA(cudaMemsetAsync(s->d_cnt, 0, m * sizeof(smg::QCounters), c->stream));
  SMG_CUDA(cudaEventCreateWithFlags(&s->ev, cudaEventDisableTiming));
  s->slots.resize(m);
  s->free_slots = m;
  smg_status rc = reset_queue(s.get());
  if (rc) return rc;
  SMG_CUDA(cudaStreamSynchronize(c->stream));
  *out = s.release();
  return SMG_OK;
}

smg_status smg_server_submit(smg_server *s, const smg_plan *p, uint64_t *ticket) {
  if (!s || !p || !ticket) return fail(SMG_ERR_INVALID, "null argument");
  if (p->p.k > s->kmax) return fail(SMG_ERR_LIMIT, "query larger than the server's max_query_vertices");
  const uint64_t bytes = smg::query_footprint(s->graph->g, p->p).total();
  if (bytes > s->cfg.memory_budget_bytes) return fail(SMG_ERR_BUDGET, "query exceeds the server memory budget");
  for (uint32_t u = 0; u < p->p.k; ++u)
    if (p->p.label[u] >= smg::kMaxLabels) return fail(SMG_ERR_LIMIT, "query labels must be below 256");
  *ticket = s->next_ticket++;
  s->waiting.push_back({*ticket, &p->p, now_s(), bytes});
  s->outstanding.insert(*ticket);
  return SMG_OK;
}

smg_status smg_server_step(smg_server *s) {
  if (!s) return fail(SMG_ERR_INVALID, "null server");
  return step(s);
}

smg_status smg_server_poll(smg_server *s, uint64_t ticket, smg_request_result *out) {
  if (!s || !out) return fail(SMG_ERR_INVALID, "null argument");
  auto it = s->done.find(ticket);
  if (it == s->done.end()) {
    if (s->outstanding.count(ticket)) return SMG_ERR_NOT_READY;
    return fail(SMG_ERR_INVALID, "unknown ticket, or its result was already collected");
  }
  *out = it->second;
  s->done.erase(it);  // a result is handed out once, so a long-running server keeps no history
  return SMG_OK;
}

smg_status smg_server_cancel(smg_server *s, uint64_t ticket) {
  if (!s) return fail(SMG_ERR_INVALID, "null server");
  for (auto it = s->waiting.begin(); it != s->waiting.end(); ++it)
    if (it->ticket == ticket) {
      smg_request_result res{};
      res.status = SMG_ERR_CANCELLED;
      res.submit_s = it->submit_s;
      res.finish_s = now_s();
      s->done[ticket] = res;
      s->outstanding.erase(ticket);
      s->waiting.erase(it);
      return SMG_OK;
    }
  return fail(SMG_ERR_INVALID, "ticket is not waiting (unknown, running or finished)");
}

smg_status smg_server_drain(smg_server *s) {
  if (!s) return fail(SMG_ERR_INVALID, "null server");
  while (s->inflight || !s->waiting.empty() || any_active(s)) {
    smg_status rc = step(s);
    if (rc) return rc;
    // completions and the doorbell are served while the slice runs
    if (s->inflight) std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
  return SMG_OK;
}

smg_status smg_server_get_stats(const smg_server *s, smg_server_stats *out) {
  if (!s || !out) return fail(SMG_ERR_INVALID, "null argument");
  *out = s->stats;
  out->slices = s->slices;
  return SMG_OK;
}

void smg_server_destroy(smg_server *s) { delete s; }

}  // extern "C"
