// join.cuh — host interface of the join (join.cu).
#pragma once

#include "device.cuh"

namespace smg {

// One hot counter per 128-byte line, so that spinning readers of one do not
// slow the atomics on another.
struct alignas(128) QLine {
  unsigned long long v;
  unsigned long long pad[15];
};

// Work-queue state in device memory.  A warp wanting work takes a ticket
// (head++) and waits for slot `ticket` to be published; producers append at
// tail++.  head > tail therefore means warps are waiting, which is when busy
// warps split their work.  `pending` counts tasks pushed and not yet
// finished; the persistent kernel ends when it reaches zero.
struct QueueState {
  QLine head, tail, pending, progress;
  unsigned long long tasks_done, donations, start_ns, scanned, descents, probes;
  int error;  // JOIN_ERR_* below, first one wins
  int abort;  // set on error or deadline: every warp leaves
  int full;   // a donation found the queue full (load balance only)
  int pad;
};
constexpr int JOIN_ERR_READY_TIMEOUT = 1;  // a claimed task was never published
constexpr int JOIN_ERR_DEADLINE = 2;       // the run exceeded its time limit
constexpr int JOIN_ERR_IDLE_TIMEOUT = 3;   // no warp made progress for too long

struct JoinLaunch {
  const uint32_t *off, *adj;
  const uint32_t *hub_of;    // [n] hub index or kNone
  const uint32_t *hub_bits;  // [hubs][hub_words] neighbour bitmaps of hubs
  uint64_t hub_words;
  const JoinQuery *queries;  // device array
  uint32_t nq, kmax;
  QueueState *qs;            // device
  uint32_t *tasks;           // [cap][4 + kmax]
  uint32_t *ready;           // [cap], zero on entry
  uint32_t cap;
  uint32_t root_chunk;       // 0: derive from max_seed_tasks
  uint32_t max_seed_tasks;   // initial tasks per query at most
  uint32_t donate_min;       // shortest remaining list worth donating
  uint64_t time_limit_ns;    // device-side deadline for the whole run
  int emit;
};

// Bytes of queue storage for `cap` tasks of a batch whose largest query has
// kmax vertices.
size_t join_queue_bytes(uint32_t cap, uint32_t kmax);
// Seeds one task per chunk of root candidates of every query (device-side, so
// no host round trip sits between the filter and the join) and runs the
// persistent kernel.  QueueState must be zeroed on entry.
smg_status launch_join(const JoinLaunch &jl, cudaStream_t s, int num_sms);
// Neighbour bitmaps of the highest-degree vertices (degree >= min_degree,
// at most max_bytes of bitmaps), built once per resident graph.
smg_status build_hub_bitmaps(DevGraph &g, uint32_t min_degree, size_t max_bytes, cudaStream_t s,
                             const std::vector<uint32_t> &degrees_host);

}  // namespace smg
