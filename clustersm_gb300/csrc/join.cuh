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
  unsigned long long last_count_entries;  // list entries read by k_last_counts
  // bytes a breadth-first table join would move for the same partial
  // matches (JoinLaunch::count_model; the per-level model of the join's
  // minimum traffic)
  unsigned long long model_bytes;
  unsigned long long bfs_tasks;  // tasks queued by breadth-first levels (JoinQuery::bfs_depth)
  int error;  // JOIN_ERR_* below, first one wins
  int abort;  // set on error or deadline: every warp leaves
  int full;   // a donation found the queue full (load balance only)
  int closing;  // the time slice is over: warps hand their work back and leave
};
constexpr int JOIN_ERR_READY_TIMEOUT = 1;  // a claimed task was never published
constexpr int JOIN_ERR_DEADLINE = 2;       // the run exceeded its time limit
constexpr int JOIN_ERR_IDLE_TIMEOUT = 3;   // no warp made progress for too long
constexpr int JOIN_ERR_QUEUE_FULL = 4;     // a time slice's leftover tasks did not fit the next queue
// Queue slots kept free for tasks that racing warps push after a slice's
// preemptions sized the next queue (at most about 12 per resident warp).
constexpr uint32_t kPreemptSlack = 1u << 16;

struct JoinLaunch {
  const uint32_t *off, *adj;
  const uint32_t *hub_of;    // [n] hub index or kNone
  const uint32_t *hub_bits;  // [hubs][hub_words] neighbour bitmaps of hubs
  uint64_t hub_words;
  const uint32_t *adjl;      // label index (DevGraph::adjl, lab_of, lab_off)
  const uint32_t *lab_of, *lab_off;
  uint32_t lab_buckets;
  const uint32_t *adjr;      // rank of each adjl entry within its label (DevGraph::adjr; null: none)
  const uint32_t *label;     // vertex labels (bucket of a probed vertex without a level bucket)
  const uint32_t *lverts;    // vertex ids grouped by label (DevGraph::lverts)
  const uint32_t *lab_rank, *bucket_word_off;  // hub bitmap layout by label (null: by id)
  uint32_t probe_runs;       // membership probes search label runs (SMG_PROBE=runs)
  uint32_t hoist;            // hoisted last-level sets (count-only runs; SMG_HOIST=0: off)
  // how |X & N(v)| is counted for a stored hoisted set X: v's run is
  // scanned when 8 x its length <= hoist_scan_x8 x |X|, else X is walked
  // (SMG_HOIST_SCAN_RATIO, in eighths; 8 walks the shorter side)
  uint32_t hoist_scan_x8;
  // per resident warp, room for a stored hoisted set of xcap entries (global
  // memory, [blocks x warps per block][xcap]); null: the warp's shared
  // memory, 256 entries
  uint32_t *xbuf;
  uint32_t xcap;
  uint32_t n;                // data vertices (bounds of the self-checking build)
  uint64_t m2;               // adjacency entries
  uint32_t num_hubs;
  const JoinQuery *queries;  // device array
  uint32_t nq, kmax;
  QueueState *qs;            // device
  uint32_t *tasks;           // [cap][4 + kmax]
  uint32_t *ready;           // [cap], zero on entry
  uint32_t cap;
  uint32_t root_chunk;       // 0: derive from max_seed_tasks
  uint32_t max_seed_tasks;   // initial tasks per query at most
  uint32_t donate_min;       // shortest remaining list worth donating
  // a warp checks for waiting warps every (mask + 1) steps (SMG_DONATE_EVERY:
  // 1, 2, 4 or 8; default 2)
  uint32_t donate_every_mask;
  // Queue slots breadth-first levels may fill: a warp queues a batch of
  // partial matches only while the tail stays within this many slots, else
  // it descends into them itself, so the breadth-first frontier is bounded
  // by the queue (0: no breadth-first levels in this launch).
  uint64_t bfs_budget;
  uint64_t time_limit_ns;    // device-side deadline for the whole run
  int emit;
  // Time-sliced runs (serving).  A slice closes after slice_ns, or after
  // slice_min_ns once the host has rung `bell` (a host-mapped word: requests
  // are waiting and slots are free).  Then every warp writes what is left of
  // its stack into the next slice's queue and leaves.  slice_ns = 0: run to
  // completion.
  uint64_t slice_ns;
  uint64_t slice_min_ns;
  const volatile uint32_t *bell;
  uint32_t *next_tasks;      // [cap][4 + kmax]
  uint32_t *next_ready;      // [cap], zero on entry
  unsigned int *next_count;  // tasks written to the next queue, zero on entry
  const uint32_t *seed_list; // seed only these query indices (null: 0 .. nq-1)
  uint32_t seed_n;
  // Serving with admission into the running slice: while the host-mapped
  // word *hold is non-zero, warps keep waiting for work when the queue
  // drains instead of leaving (the host may still append root tasks), so no
  // claimed ticket is ever abandoned; the host clears it once nothing more
  // will be appended.  Null: leave when the queue drains.
  const volatile uint32_t *hold;
  // Join blocks per SM at most (0: as many as fit); the server leaves room
  // for the filter kernels of requests admitted into a running slice.
  uint32_t max_blocks_per_sm;
  // Accumulate QueueState::model_bytes (a measurement run; costs a few loads
  // per partial match).
  uint32_t count_model;
};

// The resident graph's arrays in a launch record (every launch site uses
// this, so the hub bitmap layout and the label index always travel together).
void set_graph(JoinLaunch &jl, const DevGraph &g);
// Entries of a warp's hoisted-set buffer in global memory (SMG_HOIST_CAP,
// default 4,096), and the bytes of such buffers for every warp a join launch
// on num_sms SMs can have.
uint32_t hoist_global_cap();
size_t hoist_buffer_bytes(int num_sms);
// Bytes of queue storage for `cap` tasks of a batch whose largest query has
// kmax vertices.
size_t join_queue_bytes(uint32_t cap, uint32_t kmax);
// Seeds one task per chunk of root candidates of every query (device-side, so
// no host round trip sits between the filter and the join) and runs the
// persistent kernel.  QueueState must be zeroed on entry.
smg_status launch_join(const JoinLaunch &jl, cudaStream_t s, int num_sms);
// Starts a time slice (clock and closing flag) without seeding.
smg_status launch_slice_begin(QueueState *qs, cudaStream_t s);
// Seeds the root tasks of jl.queries[0 .. jl.nq) (appending to the queue).
smg_status launch_seed(const JoinLaunch &jl, cudaStream_t s);
// Persistent join without seeding (tasks already queued).
smg_status launch_join_only(const JoinLaunch &jl, cudaStream_t s, int num_sms);
// Rebuilds the queue after a slice: appends the published-but-untaken tasks
// of the old queue (ready == 1) to the new one, behind the tasks preempted
// warps wrote there (new_count of them), then resets head/tail/pending to the
// new queue and clears new_count.  A whole grid; order is not kept.
smg_status launch_compact(const uint32_t *tasks_old, const uint32_t *ready_old, uint32_t cap, uint32_t tw,
                          uint32_t *tasks_new, uint32_t *ready_new, unsigned int *new_count, QueueState *qs,
                          cudaStream_t s, int num_sms);
// Join inputs built after the filter (which leaves the candidate bitmaps)
// for the queries jl.seed_list names (all jl.nq when it is null): unless the
// run emits embeddings, each fast_last query's last-level counts: for every
// candidate v of the last vertex's back neighbour, how many neighbours of v
// are candidates of the last vertex.  launch_join runs it itself.
smg_status launch_join_prep(const JoinLaunch &jl, cudaStream_t s, int num_sms);
// Label index of a resident graph (DevGraph::adjl, lab_of, lab_off) from the
// host's id-ordered lists: vertices of degree >= min_degree get a run table,
// highest degree first, up to max_bytes of tables.
smg_status build_label_index(DevGraph &g, const uint64_t *offsets, const uint32_t *adj, const uint32_t *labels,
                             uint32_t min_degree, size_t max_bytes, cudaStream_t s);
// Neighbour bitmaps of the highest-degree vertices (degree >= min_degree,
// at most max_bytes of bitmaps), built once per resident graph.
smg_status build_hub_bitmaps(DevGraph &g, uint32_t min_degree, size_t max_bytes, cudaStream_t s,
                             const std::vector<uint32_t> &degrees_host);

}  // namespace smg
