// api_internal.cuh — context, resident-graph and run structures behind the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <vector>

#include "device.cuh"
#include "filter.cuh"
#include "join.cuh"

namespace smg {

constexpr size_t kPinnedBytes = 32u << 20;

// Grow-only device buffer; each run carves its scratch out of it.
// Device memory a batch leaves free for what is allocated after its arena:
// kernels' local memory at launch, CUDA graph instantiation, filter tables.
constexpr size_t kHeadroomBytes = 8ull << 30;

struct Arena {
  char *base = nullptr;
  size_t cap = 0;
  smg_status reserve(size_t bytes);
  Arena() = default;
  Arena(const Arena &) = delete;
  Arena &operator=(const Arena &) = delete;
  ~Arena();
};

// Per-query counters (zeroed before each run).
struct QCounters {
  uint32_t cand_cnt[kMaxK];    // initial candidates appended per query vertex
  uint32_t num_roots;          // root candidates after the bitmap filter
  uint32_t over;               // count exceeded the run's count limit
  uint32_t pad[2];
  unsigned long long stat[4];  // [0] sum |C(u)| final, [1] walk list entries
  unsigned long long count;    // embeddings
  unsigned long long emb_count;
  unsigned long long pending;  // tasks of this query not yet finished
  unsigned long long work;     // join steps taken (counted only under a work limit)
  unsigned long long pad2[6];
};
static_assert(sizeof(QCounters) % 16 == 0, "QCounters must keep 16-byte alignment");

uint64_t time_limit_ns();

// Options of one run (plain path: one query; batched: many).
struct TuneSetting {
  uint32_t root_chunk = 0, donate_min = 0, split_len = 0, hoist_cap = 0, bfs_depth = 0;
  bool valid = false;
};
// The tuned knobs of a shape class into a query's join record.
inline void apply_tuning(const TuneSetting &t, JoinQuery &j) {
  j.root_chunk = t.root_chunk;
  j.donate_min = t.donate_min;
  j.split_len = t.split_len;
  j.hoist_cap = t.hoist_cap;
  j.bfs_depth = t.bfs_depth;
}
uint32_t plan_class(const Plan &P);

struct RunOpts {
  const TuneSetting *tuning = nullptr;  // per shape class, SMG_TUNE_CLASSES entries
  bool profile = false;
  uint32_t root_chunk = 0;
  uint32_t max_seed_tasks = 0;   // 0: derived from the device size
  uint32_t *emb_host = nullptr;  // plain path only
  uint64_t emb_cap = 0;
  bool use_graph = false;        // capture the launches in a CUDA graph
  uint64_t count_limit = 0;      // 0: none
  uint64_t work_limit = 0;       // 0: none
  bool model = false;            // count the breadth-first byte model
  uint32_t bfs_depth = 0;        // 0: the tuned depth (none when untuned)
};

struct QueryOut {
  uint64_t count = 0, emb_written = 0, cands = 0, walk_entries = 0;
  uint32_t num_roots = 0, overflow = 0, limit_hit = 0;
  uint64_t initial_cands = 0;
};

struct RunStats {
  float filter_ms = 0, join_ms = 0;
  uint64_t tasks = 0, donations = 0, scanned = 0, descents = 0, probes = 0, last_count_entries = 0;
  uint64_t bfs_tasks = 0;
  uint64_t model_bytes = 0;
  uint64_t filter_bytes = 0, join_bytes = 0;
  uint64_t launches = 0, h2d = 0, d2h = 0;
  uint32_t chunks = 0;
};

}  // namespace smg

struct smg_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  void *pinned = nullptr;  // kPinnedBytes of page-locked staging
  smg::Arena arena;
  std::unique_ptr<smg::FilterDev> fdev;
  smg::TuneSetting tuning[SMG_TUNE_CLASSES];
  // CUDA graph of the last single-chunk batch, valid while no other run has
  // touched the arena since (run_gen == graph_gen)
  cudaGraphExec_t graph_exec = nullptr;
  std::vector<const void *> graph_key;
  uint64_t run_gen = 0, graph_gen = ~0ull;
  uint64_t graph_launches = 0;
};

struct smg_graph {
  int device = 0;
  smg::DevGraph g;
};

namespace smg {
// Forgets the captured batch graph of a context.
void drop_graph(smg_ctx *c);
// Frees a context's batch scratch (the arena grows to what the largest batch
// needed, up to all free memory) and the captured batch graph; the next batch
// allocates again.
void release_batch_memory(smg_ctx *c);
// Device buffers holding one query's filter state and results.
struct QueryBuffers {
  uint32_t *vmask = nullptr, *enc = nullptr, *cand = nullptr, *roots = nullptr;
  uint32_t *cbits = nullptr;  // candidate bitmaps (null: the join tests vmask)
  QCounters *counters = nullptr;
  uint32_t *emb = nullptr;
  uint64_t emb_cap = 0;
};
// Sizes of those buffers for one plan (bytes, each rounded to 256).
struct QueryFootprint {
  size_t vmask, enc, cand, roots, cbits;
  size_t total() const { return vmask + enc + cand + roots + cbits; }
};
QueryFootprint query_footprint(const DevGraph &g, const Plan &P);
// Fills the filter and join records of one query whose state lives in `b`.
smg_status make_query_records(const Plan &P, const DevGraph &g, const QueryBuffers &b, uint64_t count_limit,
                              FilterQuery &f, JoinQuery &j, uint64_t work_limit = 0);
constexpr uint32_t kMaxWalkPhases = 2 * 100;  // 2 * MAX_LAYERS - 1 phases at most
constexpr uint32_t kWalkCap = 1u << 20;        // chunk-pass items per filter launch

// Sorted, duplicate-free CSR of an undirected edge list (host pairs), built
// on the device (graph_build.cu): 64-bit offsets [n + 1] and neighbours
// [*m2], both device allocations the caller frees.
smg_status build_csr_device(smg_ctx *c, uint32_t n, uint64_t np, const uint32_t *pairs_host,
                            unsigned long long **off64, uint32_t **adj, uint64_t *m2);
smg_status narrow_offsets(const unsigned long long *off64, uint32_t *off32, uint64_t n1, cudaStream_t s, int num_sms);
// Labels, label groups, neighbour-label counts, label index and hub bitmaps
// of a graph whose off/adj are on the device (the same CSR in host memory).
smg_status finish_resident(smg_ctx *c, DevGraph &g, const uint64_t *offsets, const uint32_t *adj,
                           const uint32_t *labels, uint32_t maxl, uint32_t maxd);
// Filter + join for `nq` plans against a resident graph; splits into chunks
// that fit the device memory.  out[i] receives plan i's results.
smg_status run_queries(smg_ctx *c, const DevGraph &g, const Plan *const *plans, uint32_t nq, const RunOpts &o,
                       QueryOut *out, RunStats *st);
}  // namespace smg
