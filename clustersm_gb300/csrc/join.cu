// join.cu — warp-parallel join of partial matches on sm_103a.
//
// The reference joins edge by edge breadth-first, materialising every level
// in two MAX_RES-row tables (join.cu:290-435): one warp per row expands over
// the anchor's neighbours (joinOneEdgeKernel, join.cu:100-177) and a thread
// per row scans an adjacency list for each non-tree edge
// (selectPartialMatchingsKernel, join.cu:16-68).  Its result is the set of
// injective mappings whose every vertex passes its candidate bit and whose
// every query edge is present.  This kernel computes the same set:
//
//  * vertices are matched in the order of JoinQuery::order (a cost-based
//    order chosen on the host; every connected order gives the same set);
//    each level checks, for a new vertex, every query edge back to a matched
//    vertex at once;
//  * a persistent grid pulls tasks (a matched prefix plus a slice of the next
//    level's list) from a device work queue and finishes each depth-first, so
//    memory stays bounded instead of growing with the level sizes;
//  * candidates of a level come from the neighbour list of the matched
//    neighbour with the fewest neighbours; 32 list entries are tested per
//    step (candidate bit, injectivity, membership in the other matched
//    neighbours' lists) and compacted with a warp ballot;
//  * membership in the list of a high-degree vertex is one bit of a
//    per-graph neighbour bitmap; other lists are binary-searched;
//  * the last level is counted, not materialised: one warp walks the
//    concatenated last-level lists of a whole batch of up to 32 candidates of
//    the level before it (a segmented scan), so short lists fill the warp;
//  * a warp with a long remaining list donates half of it to the queue while
//    more warps wait than tasks are queued (work splitting for hubs);
//  * the first JoinQuery::bfs_depth levels may run breadth-first, as the
//    reference's join does for every level: a warp queues each batch of
//    accepted candidates as tasks one level deeper instead of descending,
//    within a bounded number of queue slots (JoinLaunch::bfs_budget), so the
//    frontier kept in memory stays bounded and deeper levels run depth-first;
//  * every wait is bounded: a claimed-but-unpublished task, an idle grid and
//    the whole run have time limits after which the kernel records an error
//    and returns.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <numeric>
#include <string>
#include <vector>

#include "filter.cuh"  // kMaxLabels
#include "join.cuh"

namespace smg {
namespace {

constexpr int kWarpsPerBlock = 8;
constexpr uint64_t kIdleLimitNs = 30000000000ull;  // 30 s without any progress
constexpr unsigned long long kLimitFlush = 4096;    // count-limited joins publish at this many
constexpr uint32_t kSplitLen = 8192;                // last-level lists are cut into slices this long

__device__ __forceinline__ uint64_t now_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned long long vload(const QLine &l) {
  return *reinterpret_cast<const volatile unsigned long long *>(&l.v);
}

__device__ __forceinline__ void set_error(QueueState *qs, int code) {
  atomicCAS(&qs->error, 0, code);
  atomicExch(&qs->abort, 1);
}

// Waits for the task of `ticket` to be published.  Returns 1 when it is,
// 0 when the run is over (no task pending anywhere, so none can come) or
// aborted, -1 on a deadline / idle timeout (recorded in the queue state).
// Each waiter polls its own ready flag; the shared counters are read only
// every 16 polls.
__device__ int wait_ticket(const JoinLaunch &p, unsigned long long ticket, uint64_t &idle_mark, uint64_t &idle_t0) {
  QueueState *qs = p.qs;
  volatile uint32_t *r = ticket < p.cap ? p.ready + ticket : nullptr;
  uint32_t ns = 128, polls = 0;
  while (true) {
    if (r && *r) {
      __threadfence();
      return 1;
    }
    if ((polls++ & 15) == 0) {
      if (vload(qs->pending) == 0 && !(p.hold && *p.hold)) return 0;
      if (*reinterpret_cast<volatile int *>(&qs->abort)) return 0;
      if (*reinterpret_cast<volatile int *>(&qs->closing)) return 0;
      const uint64_t pr = vload(qs->progress), t = now_ns();
      if (pr != idle_mark || idle_t0 == 0) {
        idle_mark = pr;
        idle_t0 = t;
      } else if (t - idle_t0 > kIdleLimitNs) {
        set_error(qs, JOIN_ERR_IDLE_TIMEOUT);
        return -1;
      }
      const uint64_t el = t - *reinterpret_cast<volatile unsigned long long *>(&qs->start_ns);
      if (el > p.time_limit_ns) {
        set_error(qs, JOIN_ERR_DEADLINE);
        return -1;
      }
      // a time slice also ends for a waiting warp (under a hold, every warp
      // may be waiting when the slice time runs out or the bell rings)
      if (p.slice_ns && (el > p.slice_ns || (el > p.slice_min_ns && p.bell && *p.bell))) {
        atomicExch(&qs->closing, 1);
        return 0;
      }
    }
    __nanosleep(ns);
    ns = min(ns * 2, 2048u);
  }
}

// One block per seeded query: thread 0 reserves the query's root tasks (one
// per chunk of root candidates) at the queue's tail, then every thread writes
// and publishes its share of them (a query may have tens of thousands).
__global__ void __launch_bounds__(256) k_seed(JoinLaunch p) {
  __shared__ unsigned long long s_first;
  __shared__ uint32_t s_nt, s_chunk, s_nr;
  // a whole batch starts its clock here; seeds of admitted requests (a seed
  // list) join a slice whose clock k_slice_begin set
  if (!p.seed_list && blockIdx.y == 0 && threadIdx.x == 0) p.qs->start_ns = now_ns();
  const uint32_t nseed = p.seed_list ? p.seed_n : p.nq;
  const uint32_t tw = 4 + p.kmax;
  for (uint32_t si = blockIdx.y; si < nseed; si += gridDim.y) {
    const uint32_t q = p.seed_list ? p.seed_list[si] : si;
    if (threadIdx.x == 0) {
      const uint32_t nr = *p.queries[q].num_roots;
      const uint32_t rc = p.queries[q].root_chunk ? p.queries[q].root_chunk : p.root_chunk;
      uint32_t chunk = rc ? rc : 1, nt = 0;
      unsigned long long first = 0;
      if (nr) {
        chunk = max(chunk, (nr + p.max_seed_tasks - 1) / p.max_seed_tasks);
        nt = (nr + chunk - 1) / chunk;
        first = atomicAdd(&p.qs->tail.v, static_cast<unsigned long long>(nt));
        if (first + nt > p.cap) {  // no room: the run fails (batches size the queue for every seed)
          set_error(p.qs, JOIN_ERR_QUEUE_FULL);
          nt = 0;
        } else {
          atomicAdd(&p.qs->pending.v, static_cast<unsigned long long>(nt));
          atomicAdd(p.queries[q].pending, static_cast<unsigned long long>(nt));
        }
      }
      // a served query without root candidates never runs a task: its count
      // (zero) is final now
      if (nr == 0 && p.queries[q].done_gen) {
        const JoinQuery &Q = p.queries[q];
        *reinterpret_cast<volatile unsigned long long *>(Q.done_count) = 0ull;
        __threadfence_system();
        *reinterpret_cast<volatile uint32_t *>(Q.done_gen) = Q.gen;
      }
      s_first = first;
      s_nt = nt;
      s_chunk = chunk;
      s_nr = nr;
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < s_nt; i += blockDim.x) {
      uint32_t *t = p.tasks + (s_first + i) * tw;
      t[0] = q;
      t[1] = 0;
      t[2] = i * s_chunk;
      t[3] = min(s_nr, (i + 1) * s_chunk);
      __threadfence();
      p.ready[s_first + i] = 1;
    }
    __syncthreads();  // the shared values are rewritten for the next query
  }
}

// Block per hub: set one bit per neighbour, by id or (label, rank) layout.
__global__ void k_hub_bits(const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                           const uint32_t *__restrict__ hubs, uint64_t words, uint32_t *__restrict__ bits,
                           const uint32_t *__restrict__ label, const uint32_t *__restrict__ rank,
                           const uint32_t *__restrict__ bucket_word_off, uint32_t buckets) {
  const uint32_t v = hubs[blockIdx.x];
  uint32_t *row = bits + blockIdx.x * words;
  for (uint32_t e = off[v] + threadIdx.x; e < off[v + 1]; e += blockDim.x) {
    const uint32_t w = adj[e];
    if (rank) {
      const uint32_t r = rank[w];
      atomicOr(row + bucket_word_off[min(label[w], buckets - 1)] + (r >> 5), 1u << (r & 31));
    } else {
      atomicOr(row + (w >> 5), 1u << (w & 31));
    }
  }
}

// A word of a hub bitmap row.  The rows are large (n / 8 bytes each, up to
// 64 GB in all) and a probe touches one random word of one, so the load
// neither allocates in L1 nor keeps its line in L2 ahead of the lists, the
// candidate bitmaps and the queue, which are read again (evict-first
// policy).  Measured on the 2^22 R-MAT workload, same box, interleaved
// runs: join 144.6 / 143.8 ms per 1,024 queries with plain loads, 140.6 /
// 141.5 ms with this one.
__device__ __forceinline__ uint32_t ld_hub_word(const uint32_t *a) {
  uint32_t v;
  uint64_t policy;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(policy));
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(v) : "l"(a), "l"(policy));
  return v;
}

// Candidate test of data vertex w for query vertex u: one bit of u's row of
// the candidate bitmaps, or bit u of w's mask when a query has no bitmaps.
struct CandView {
  const uint32_t *bits;  // cbits
  uint64_t words;        // cwords
  const uint32_t *mask;  // candmask
  const uint32_t *crow;  // rank-indexed rows (null: none)
  __device__ __forceinline__ bool has(uint32_t u, uint32_t w) const {
    if (bits) return (__ldg(bits + u * words + (w >> 5)) >> (w & 31)) & 1u;
    return (__ldg(mask + w) >> u) & 1u;
  }
  // the same test for an entry of a label run of u's label, by its rank r
  // within that label's group
  __device__ __forceinline__ bool has_rank(uint32_t u, uint32_t r) const {
    return (__ldg(crow + u * words + (r >> 5)) >> (r & 31)) & 1u;
  }
  // rank array of the entries of `list` when the tests can use the
  // rank-indexed rows: the list is a label run in adjl (so every entry
  // carries the level's label) and the graph has entry ranks; else null
  __device__ __forceinline__ const uint32_t *ranks_of(const JoinLaunch &p, const uint32_t *list) const {
    if (!crow || !p.adjr || list < p.adjl || list >= p.adjl + p.m2) return nullptr;
    return p.adjr + (list - p.adjl);
  }
};

// Last-level counts.  In a count-only run, when the last query vertex u_L
// has a single edge back to the matched prefix (to level b), the last level
// of a prefix m[0..k-2] accepts exactly the neighbours w of m[b] that are
// candidates of u_L (which implies u_L's label) and differ from the matched
// vertices of u_L's label.  Its count is therefore the number of such
// neighbours of m[b], stored once per query for every candidate of order[b],
// less the same-label matched vertices among them.  The counts go to an
// id-indexed array (JoinQuery::lastcnt, over the query's cluster bitmap,
// which nothing reads after the filter); kNone marks a vertex whose count is
// not stored (degree above kLastCountMaxDeg), whose list the join scans as
// before.
constexpr uint32_t kLastCountMaxDeg = 8192;

// A warp takes 32 consecutive vertices, picks the candidates of order[b]
// with a ballot and counts each one's qualifying neighbours with its lanes
// (four independent list entries per lane per step).
__global__ void __launch_bounds__(256) k_last_counts(const JoinQuery *__restrict__ queries,
                                                     const uint32_t *__restrict__ list, uint32_t nq,
                                                     const uint32_t *__restrict__ lverts,
                                                     const uint32_t *__restrict__ off,
                                                     const uint32_t *__restrict__ adj,
                                                     const uint32_t *__restrict__ adjl,
                                                     const uint32_t *__restrict__ lab_of,
                                                     const uint32_t *__restrict__ lab_off, uint32_t lab_buckets,
                                                     uint32_t n, QueueState *qs) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warp = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
  unsigned long long read = 0;
  for (uint32_t qi = blockIdx.y; qi < nq; qi += gridDim.y) {
    const JoinQuery &Q = queries[list ? list[qi] : qi];
    if (!Q.fast_last) continue;
    const uint32_t ub = Q.order[Q.fast_last - 1], ul = Q.order[Q.k - 1];
    const uint32_t *row = Q.cbits + ul * Q.cwords;
    const uint32_t bk = Q.level_bucket[Q.k - 1];
    uint32_t *cnt = Q.lastcnt;  // by vertex id
    // the candidates of order[b] all carry its label: walk that label's group
    for (uint32_t t0 = Q.lc_lo + warp * 32; t0 < Q.lc_hi; t0 += nwarps * 32) {
      const uint32_t t = t0 + lane;
      const uint32_t v = t < Q.lc_hi ? __ldg(lverts + t) : 0u;
      const uint32_t mine = t < Q.lc_hi ? __ldg(Q.candmask + t) : 0u;  // the final mask, by position
      for (uint32_t bal = __ballot_sync(0xFFFFFFFFu, (mine >> ub) & 1u); bal; bal &= bal - 1) {
        const uint32_t src = __ffs(bal) - 1;
        const uint32_t x = __shfl_sync(0xFFFFFFFFu, v, src);
        // the neighbours of x with the last vertex's label bucket (its run
        // when x has a run table, else the whole list)
        uint32_t beg = __ldg(off + x), end = __ldg(off + x + 1);
        const uint32_t *lst = adj;
        if (Q.use_labels) {
          const uint32_t li = __ldg(lab_of + x);
          if (li != kNone) {
            const uint32_t *t = lab_off + static_cast<uint64_t>(li) * (lab_buckets + 1) + bk;
            const uint32_t lo = __ldg(t), hi = __ldg(t + 1);
            lst = adjl;
            end = beg + hi;
            beg += lo;
          }
        }
        uint32_t c = kNone;
        if (end - beg <= kLastCountMaxDeg) {
          uint32_t part = 0;
          for (uint32_t e = beg + lane; e < end; e += 128) {
            uint32_t w[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) w[i] = e + 32 * i < end ? __ldg(lst + e + 32 * i) : kNone;
#pragma unroll
            for (int i = 0; i < 4; ++i)
              if (w[i] != kNone && SMG_DCHECK(w[i] < n, 120, w[i], x)) part += (__ldg(row + (w[i] >> 5)) >> (w[i] & 31)) & 1u;
          }
          c = __reduce_add_sync(0xFFFFFFFFu, part);
          read += end - beg;
        }
        if (lane == src) cnt[x] = c;
      }
    }
  }
  if (lane == 0 && read) atomicAdd(&qs->last_count_entries, read);
}

// Is w in the neighbour list of matched vertex x (id-ordered list at beg,
// deg entries)?  `hub` selects x's bitmap when it has one.  With
// p.probe_runs, a vertex with a label run table is searched in its run of
// w's label bucket instead (bucket: that of the level w is a candidate for,
// kNone when the query has no label index): a short sorted range that all
// lanes of a warp search together, in place of a random bitmap word.
__device__ __forceinline__ bool is_neighbor(const JoinLaunch &p, uint32_t x, uint32_t beg, uint32_t deg,
                                            uint32_t hub, uint32_t bucket, uint32_t w, uint32_t &probes) {
  const uint32_t *a = p.adj + beg;
  uint32_t len = deg;
  bool run = false;
  if (p.probe_runs && bucket != kNone) {
    const uint32_t li = __ldg(p.lab_of + x);
    if (li != kNone) {
      const uint32_t *t = p.lab_off + static_cast<uint64_t>(li) * (p.lab_buckets + 1) + bucket;
      const uint32_t r0 = __ldg(t);
      len = __ldg(t + 1) - r0;
      a = p.adjl + beg + r0;
      run = true;
    }
  }
  if (!run && hub != kNone && SMG_DCHECK(hub < p.num_hubs, 102, hub, p.num_hubs) &&
      SMG_DCHECK(w < p.n, 103, w, p.n)) {
    ++probes;
    uint32_t word = w >> 5, bit = w & 31;
    if (p.lab_rank) {  // bitmap rows laid out by label bucket, then rank
      const uint32_t b = bucket != kNone ? bucket : min(__ldg(p.label + w), p.lab_buckets - 1);
      const uint32_t r = __ldg(p.lab_rank + w);
      word = __ldg(p.bucket_word_off + b) + (r >> 5);
      bit = r & 31;
    }
    return (ld_hub_word(p.hub_bits + hub * p.hub_words + word) >> bit) & 1u;
  }
  if (!SMG_DCHECK(static_cast<uint64_t>(beg) + deg <= p.m2, 104, beg, deg)) return false;
  uint32_t lo = 0, hi = len;
  while (lo < hi) {
    ++probes;
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(a + mid) < w)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo < len && __ldg(a + lo) == w;
}

// Per-warp shared state, K = largest query of the launch:
//   m, beg, deg, hub  matched data vertex per level, its list and bitmap
//   cur, end      cursor and end of the level's source list
//   bcnt, bidx    batch of up to 32 tested candidates of the level
//   piv           level whose matched vertex's list feeds this level
//   ord, bmask, slab  the task's query: vertex, backward-edge mask and
//                 same-label mask per level
//   lbk           the task's query: label bucket per level (label index)
//   lbase         base pointer of the level's source list
//   batch         [K][32] tested candidates
//   seg*          per-candidate segments of the segmented last level; bit 31
//                 of spiv marks a segment read from the label-ordered lists
__host__ __device__ inline uint32_t scalar_words(uint32_t K) { return (13 * K + 1) & ~1u; }
//   xs, xlen      the hoisted last-level set of the current prefix (see
//                 last_level): sorted, at most kHoistCap entries
constexpr uint32_t kHoistCap = 256;
constexpr uint32_t kHoistInvalid = 0xFFFFFFFFu;  // xlen: not built for this prefix
constexpr uint32_t kHoistTooBig = 0xFFFFFFFEu;   // xlen: larger than kHoistCap
__host__ __device__ inline uint32_t warp_words(uint32_t K) {
  return scalar_words(K) + 2 * K + 32 * K + 7 * 32 + kHoistCap + 2 + 32 * K;
}

struct WarpView {
  uint32_t *m, *beg, *deg, *hub, *cur, *end, *bcnt, *bidx, *piv, *ord, *bmask, *slab, *lbk, *batch;
  uint32_t *sv, *sbeg, *sdeg, *shub, *sbase, *spre, *spiv, *xs, *xlen, *bpos;
  uint32_t xcap = kHoistCap;  // entries xs holds (xs may be moved to a global buffer)
  const uint32_t **lbase;
  __device__ WarpView(uint32_t *W, uint32_t K) {
    m = W;
    beg = W + K;
    deg = W + 2 * K;
    hub = W + 3 * K;
    cur = W + 4 * K;
    end = W + 5 * K;
    bcnt = W + 6 * K;
    bidx = W + 7 * K;
    piv = W + 8 * K;
    ord = W + 9 * K;
    bmask = W + 10 * K;
    slab = W + 11 * K;
    lbk = W + 12 * K;
    const uint32_t s = scalar_words(K);
    lbase = reinterpret_cast<const uint32_t **>(W + s);
    batch = W + s + 2 * K;
    sv = batch + 32 * K;
    sbeg = sv + 32;
    sdeg = sbeg + 32;
    shub = sdeg + 32;
    sbase = shub + 32;
    spre = sbase + 32;
    spiv = spre + 32;
    xs = spiv + 32;
    xlen = xs + kHoistCap;
    bpos = xlen + 2;  // [K][32] list position of each batch entry
  }
};

constexpr uint32_t kFromLabelIndex = 1u << 31;  // spiv flag: segment in adjl
constexpr uint32_t kHoistScan = 1u << 30;       // spiv flag: keep entries found in the hoisted set
constexpr uint32_t kHoistSet = 1u << 29;        // spiv flag: the segment is the hoisted set itself

#ifdef SMG_CHECKED
// Self-checking build: does `e` point into adj or adjl?
__device__ __forceinline__ bool in_lists(const JoinLaunch &p, const uint32_t *e) {
  return (e >= p.adj && e < p.adj + p.m2) || (p.adjl && e >= p.adjl && e < p.adjl + p.m2);
}
#endif

// The list that level `level` scans: the neighbours of matched vertex x (its
// id-ordered list starts at beg and holds deg entries), narrowed to the run
// of the level's label bucket when x has a run table.  Every path that
// derives a level's list (task start, descent, last level, split slices)
// calls this, so a task's [lo, hi) means the same entries to every warp.
__device__ __forceinline__ const uint32_t *scan_list(const JoinLaunch &p, const WarpView &S, bool use_labels,
                                                     uint32_t level, uint32_t x, uint32_t beg, uint32_t deg,
                                                     uint32_t &len) {
  if (use_labels) {
    const uint32_t li = __ldg(p.lab_of + x);
    if (li != kNone) {
      const uint32_t *t = p.lab_off + static_cast<uint64_t>(li) * (p.lab_buckets + 1) + S.lbk[level];
      const uint32_t lo = __ldg(t);
      len = __ldg(t + 1) - lo;
      return p.adjl + beg + lo;
    }
  }
  len = deg;
  return p.adj + beg;
}

// Length of the list scan_list would give: the run of the level's label
// bucket when x has a run table, else its degree.
__device__ __forceinline__ uint32_t run_len(const JoinLaunch &p, const WarpView &S, bool use_labels,
                                            uint32_t level, uint32_t x, uint32_t deg) {
  if (use_labels) {
    const uint32_t li = __ldg(p.lab_of + x);
    if (li != kNone) {
      const uint32_t *t = p.lab_off + static_cast<uint64_t>(li) * (p.lab_buckets + 1) + S.lbk[level];
      return __ldg(t + 1) - __ldg(t);
    }
  }
  return deg;
}

// The pivot of `level`: the back neighbour whose list scan_list gives is
// shortest (ties to the lower level).  cand_level / cand_v / cand_deg stand
// in for the matched vertex of cand_level (the last level's candidate, not
// yet in S.m); pass kNone otherwise.  Every path that picks a level's pivot
// calls this, so donor and receiver of a task pick the same list.
__device__ __forceinline__ uint32_t choose_pivot(const JoinLaunch &p, const WarpView &S, bool use_labels,
                                                 uint32_t level, uint32_t cand_level = kNone, uint32_t cand_v = 0,
                                                 uint32_t cand_deg = 0) {
  uint32_t best = 0, bd = 0xFFFFFFFFu;
  for (uint32_t b = S.bmask[level]; b; b &= b - 1) {
    const uint32_t j = __ffs(b) - 1;
    const uint32_t d = j == cand_level ? run_len(p, S, use_labels, level, cand_v, cand_deg)
                                       : run_len(p, S, use_labels, level, S.m[j], S.deg[j]);
    if (d < bd) {
      bd = d;
      best = j;
    }
  }
  return best;
}

// The per-level byte model of a breadth-first join that keeps every partial
// match in a table (the reference's join.cu:290-435): a row of `level`
// mapped vertices is read (4 B per column), expanded along its anchor (the
// back neighbour of least degree: its offsets and its whole list, one
// candidate-bitmap word per entry, 8 + 8 B per entry) and checked against
// every other back edge by an adjacency scan (8 + 4 B per entry); the rows it
// produces are written (4 B per column, counted where they are produced).
// cand_level / cand_deg stand in for a level whose vertex is not in S.m yet.
__device__ __forceinline__ unsigned long long level_model(const WarpView &S, uint32_t level,
                                                          uint32_t cand_level = kNone, uint32_t cand_deg = 0) {
  uint32_t dmin = 0xFFFFFFFFu;
  unsigned long long scans = 0;
  for (uint32_t b = S.bmask[level]; b; b &= b - 1) {
    const uint32_t j = __ffs(b) - 1;
    const uint32_t d = j == cand_level ? cand_deg : S.deg[j];
    dmin = min(dmin, d);
    scans += 8ull + 4ull * d;
  }
  if (dmin == 0xFFFFFFFFu) return 4ull * level;
  return 4ull * level + 8ull + 8ull * dmin + (scans - 8ull - 4ull * dmin);
}

// Entries a lane tests per refill of an intermediate level.  The tests are
// chains of dependent loads (candidate bit, then a hub bitmap word or a
// binary search per back edge); a lane runs kWays chains in lockstep so that
// their loads are in flight together.
constexpr int kWays = 1;

// Candidate tests at an intermediate level (>= 1, not the last) for the kWays
// entries w[i] of a lane whose bit i of `live` is set: the candidate bit,
// injectivity against the matched vertices of the level's label, then
// membership in the lists of the back neighbours other than the pivot.
// Returns the entries that pass.  Every step is issued for all live entries
// before any of them is resolved.
__device__ __forceinline__ uint32_t accept_multi(const WarpView &S, const JoinLaunch &p, const CandView &cv,
                                                 bool use_labels, uint32_t level, const uint32_t (&w)[kWays],
                                                 const uint32_t (&r)[kWays], bool ranked, uint32_t live,
                                                 uint32_t &probes) {
  const uint32_t u = S.ord[level];
  // candidate bits
  uint32_t word[kWays];
#pragma unroll
  for (int i = 0; i < kWays; ++i) {
    word[i] = 0;
    if ((live >> i) & 1u) {
      if (!SMG_DCHECK(w[i] < p.n, 105, w[i], level)) {
        live &= ~(1u << i);
        continue;
      }
      if (ranked)
        word[i] = __ldg(cv.crow + u * cv.words + (r[i] >> 5));
      else
        word[i] = cv.bits ? __ldg(cv.bits + u * cv.words + (w[i] >> 5)) : __ldg(cv.mask + w[i]);
    }
  }
#pragma unroll
  for (int i = 0; i < kWays; ++i) {
    const uint32_t bit = ranked ? (r[i] & 31) : cv.bits ? (w[i] & 31) : u;
    if (!((word[i] >> bit) & 1u)) live &= ~(1u << i);
  }
  // injectivity against the matched vertices of the same label
  for (uint32_t b = S.slab[level]; b && live; b &= b - 1) {
    const uint32_t x = S.m[__ffs(b) - 1];
#pragma unroll
    for (int i = 0; i < kWays; ++i)
      if (w[i] == x) live &= ~(1u << i);
  }
  // membership in the lists of the back neighbours other than the pivot
  const uint32_t bucket = use_labels ? S.lbk[level] : kNone;
  for (uint32_t b = S.bmask[level] & ~(1u << S.piv[level]); b && live; b &= b - 1) {
    const uint32_t j = __ffs(b) - 1;
    const uint32_t hub = S.hub[j];
    if (p.probe_runs || p.lab_rank) {  // the rarer layouts: one entry at a time
#pragma unroll
      for (int i = 0; i < kWays; ++i)
        if (((live >> i) & 1u) && !is_neighbor(p, S.m[j], S.beg[j], S.deg[j], hub, bucket, w[i], probes))
          live &= ~(1u << i);
    } else if (hub != kNone && SMG_DCHECK(hub < p.num_hubs, 102, hub, p.num_hubs)) {
      const uint32_t *row = p.hub_bits + hub * p.hub_words;
#pragma unroll
      for (int i = 0; i < kWays; ++i) {
        word[i] = 0;
        if ((live >> i) & 1u) {
          ++probes;
          word[i] = ld_hub_word(row + (w[i] >> 5));
        }
      }
#pragma unroll
      for (int i = 0; i < kWays; ++i)
        if (!((word[i] >> (w[i] & 31)) & 1u)) live &= ~(1u << i);
    } else {
      // lockstep branchless lower bound over the id-ordered list: every
      // search takes the same steps for one list, so the loads of all live
      // entries go out together; an entry equal to w seen on the way, or at
      // the final position, is a hit
      const uint32_t *a = p.adj + S.beg[j];
      uint32_t len = S.deg[j];
      if (!SMG_DCHECK(static_cast<uint64_t>(S.beg[j]) + len <= p.m2, 104, S.beg[j], len)) len = 0;
      uint32_t base[kWays], hit = 0;
#pragma unroll
      for (int i = 0; i < kWays; ++i) base[i] = 0;
      for (uint32_t nn = len; nn > 1;) {
        const uint32_t half = nn >> 1;
#pragma unroll
        for (int i = 0; i < kWays; ++i) {
          if ((live >> i) & 1u) {
            ++probes;
            const uint32_t x = __ldg(a + base[i] + half);
            if (x < w[i]) base[i] += half;
            if (x == w[i]) hit |= 1u << i;
          }
        }
        nn -= half;
      }
#pragma unroll
      for (int i = 0; i < kWays; ++i) {
        if (((live >> i) & 1u) && !((hit >> i) & 1u)) {
          ++probes;
          if (!(len && __ldg(a + base[i]) == w[i])) live &= ~(1u << i);
        }
      }
    }
  }
  return live;
}

// A last-level list longer than the query's split length (split_len, default
// kSplitLen) is cut into slices of that length:
// the first stays with this lane, the others become tasks (level P + 1, range
// [lo, hi) of the list, prefix m[0..P-1] plus candidate v) when warps are
// waiting for work or the list is very long.  Returns the length this lane
// keeps (all of it when the queue has no room).
__device__ uint32_t split_last(const WarpView &S, const JoinLaunch &p, const JoinQuery &Q, uint32_t q, uint32_t P,
                               uint32_t v, uint32_t len) {
  QueueState *qs = p.qs;
  const uint32_t sl = Q.split_len ? Q.split_len : kSplitLen;
  const unsigned long long h = vload(qs->head), t = vload(qs->tail);
  if (!(h > t || len > 8 * sl)) return len;
  if (*reinterpret_cast<volatile int *>(&qs->closing)) return len;
  const uint32_t slices = (len - 1) / sl;  // beyond the first
  const unsigned long long first = atomicAdd(&qs->tail.v, static_cast<unsigned long long>(slices));
  if (first + slices > p.cap) {
    // no room: the slot numbers taken stay unpublished and are never waited
    // for beyond the end of the run (their tickets see pending reach zero)
    atomicExch(&qs->full, 1);
    return len;
  }
  atomicAdd(&qs->pending.v, static_cast<unsigned long long>(slices));
  atomicAdd(Q.pending, static_cast<unsigned long long>(slices));
  const uint32_t tw = 4 + p.kmax;
  for (uint32_t i = 0; i < slices; ++i) {
    uint32_t *T = p.tasks + (first + i) * tw;
    T[0] = q;
    T[1] = P + 1;
    T[2] = (i + 1) * sl;
    T[3] = min(len, (i + 2) * sl);
    for (uint32_t j = 0; j < P; ++j) T[4 + j] = S.m[j];
    T[4 + P] = v;
  }
  __threadfence();
  for (uint32_t i = 0; i < slices; ++i) atomicExch(p.ready + first + i, 1u);
  atomicAdd(&qs->donations, static_cast<unsigned long long>(slices));
  return sl;
}

// Counts (and optionally emits) the last level over entries [lo, hi) of one
// list: the prefix m[0..P] is matched, the list is that of the last vertex's
// back neighbour with the shortest list (the pivot last_level chose).
__device__ unsigned long long last_level_range(WarpView &S, const JoinLaunch &p, const JoinQuery &Q,
                                               const CandView &cv, uint32_t P, uint32_t lo,
                                               uint32_t hi, uint32_t lane, unsigned long long &scanned,
                                               uint32_t &probes) {
  const uint32_t L = P + 1;
  const uint32_t bucket = Q.use_labels ? S.lbk[L] : kNone;
  const uint32_t piv = choose_pivot(p, S, Q.use_labels, L);
  uint32_t len = 0;
  const uint32_t *base = scan_list(p, S, Q.use_labels, L, S.m[piv], S.beg[piv], S.deg[piv], len);
  hi = min(hi, len);
  if (lo >= hi) return 0;
  scanned += hi - lo;
  const uint32_t u = S.ord[L], back = S.bmask[L] & ~(1u << piv), same = S.slab[L];
  const uint32_t lt = (1u << lane) - 1;
  const uint32_t *rk = cv.ranks_of(p, base);
  unsigned long long cnt = 0;
  for (uint32_t t0 = lo; t0 < hi; t0 += 32) {
    const uint32_t t = t0 + lane;
    bool good = false;
    uint32_t w = 0;
    if (t < hi) {
      w = __ldg(base + t);
      good = SMG_DCHECK(w < p.n, 115, w, t) && (rk ? cv.has_rank(u, __ldg(rk + t)) : cv.has(u, w));
      for (uint32_t b = same; b && good; b &= b - 1) good = S.m[__ffs(b) - 1] != w;
      for (uint32_t b = back; b && good; b &= b - 1) {
        const uint32_t j = __ffs(b) - 1;
        good = is_neighbor(p, S.m[j], S.beg[j], S.deg[j], S.hub[j], bucket, w, probes);
      }
    }
    const uint32_t bal = __ballot_sync(0xFFFFFFFFu, good);
    cnt += __popc(bal);
    if (p.emit && bal) {
      unsigned long long pos = 0;
      if (lane == 0) pos = atomicAdd(Q.emb_count, static_cast<unsigned long long>(__popc(bal)));
      pos = __shfl_sync(0xFFFFFFFFu, pos, 0);
      const unsigned long long r = pos + __popc(bal & lt);
      if (good && r < Q.emb_cap) {
        uint32_t *row = Q.emb + r * Q.k;
        for (uint32_t j = 0; j <= P; ++j) row[S.ord[j]] = S.m[j];
        row[S.ord[L]] = w;
      }
    }
  }
  __syncwarp();
  return cnt;
}

// Is w in the hoisted set (sorted, n entries)?
__device__ __forceinline__ bool in_hoisted(const WarpView &S, uint32_t n, uint32_t w) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (S.xs[mid] < w)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo < n && S.xs[lo] == w;
}

// The hoisted last-level set of the prefix m[0..P-1]: the candidates w of the
// last vertex u_L adjacent to every back neighbour of u_L matched before level
// P (`fixed`), other than the matched vertices of u_L's label before P.  It
// does not depend on the level-P vertex, so a warp builds it once per prefix
// and every batch of level-P candidates reuses it.  It is the shortest fixed
// back neighbour's run filtered by the others, so it comes out sorted by id.
// Sets *S.xlen to its size, or kHoistTooBig past the warp's S.xcap entries.  With
// store false only its size is needed (the last vertex does not depend on
// level P) and there is no cap.
__device__ void build_hoisted(WarpView &S, const JoinLaunch &p, const JoinQuery &Q, const CandView &cv,
                              uint32_t P, uint32_t fixed, bool store, uint32_t lane, unsigned long long &scanned,
                              uint32_t &probes) {
  const uint32_t L = P + 1;
  const uint32_t bucket = Q.use_labels ? S.lbk[L] : kNone;
  uint32_t a = 0, best = 0xFFFFFFFFu;
  for (uint32_t b = fixed; b; b &= b - 1) {
    const uint32_t j = __ffs(b) - 1;
    const uint32_t d = run_len(p, S, Q.use_labels, L, S.m[j], S.deg[j]);
    if (d < best) {
      best = d;
      a = j;
    }
  }
  uint32_t len = 0;
  const uint32_t *lst = scan_list(p, S, Q.use_labels, L, S.m[a], S.beg[a], S.deg[a], len);
  const uint32_t u = S.ord[L], same = S.slab[L] & ((1u << P) - 1), others = fixed & ~(1u << a);
  const uint32_t lt = (1u << lane) - 1;
  const uint32_t *rk = cv.ranks_of(p, lst);
  uint32_t n = 0;
  scanned += len;
  for (uint32_t t0 = 0; t0 < len; t0 += 32) {
    const uint32_t t = t0 + lane;
    bool good = false;
    uint32_t w = 0;
    if (t < len) {
      w = __ldg(lst + t);
      good = SMG_DCHECK(w < p.n, 116, w, t) && (rk ? cv.has_rank(u, __ldg(rk + t)) : cv.has(u, w));
      for (uint32_t b = same; b && good; b &= b - 1) good = S.m[__ffs(b) - 1] != w;
      for (uint32_t b = others; b && good; b &= b - 1) {
        const uint32_t j = __ffs(b) - 1;
        good = is_neighbor(p, S.m[j], S.beg[j], S.deg[j], S.hub[j], bucket, w, probes);
      }
    }
    const uint32_t bal = __ballot_sync(0xFFFFFFFFu, good);
    if (store) {
      if (n + __popc(bal) > S.xcap) {
        n = kHoistTooBig;
        break;
      }
      if (good) S.xs[n + __popc(bal & lt)] = w;
    }
    n += __popc(bal);
  }
  __syncwarp();
  if (lane == 0) *S.xlen = n;
  __syncwarp();
}

// Which way |X & N(v)| is counted for a stored hoisted set X (xn entries,
// sorted) and a level-P candidate v whose run has rv entries: true scans v's
// run, testing each entry by a binary search of X; false walks X, probing
// N(v) for each member (a hub bitmap word or a binary search of v's list).
// The run is scanned while it is at most hoist_scan_x8 / 8 times as long as X.
__device__ __forceinline__ bool hoist_scan_run(const JoinLaunch &p, uint32_t rv, uint32_t xn) {
  return 8ull * rv <= static_cast<uint64_t>(p.hoist_scan_x8) * xn;
}

// Counts (and optionally emits) the last level for every candidate of the
// batch of level P = k-2: the candidates' last-level lists are concatenated
// and walked 32 entries at a time, each lane finding its candidate by binary
// search over the segment starts.  Returns the count (same in every lane).
__device__ unsigned long long last_level(WarpView &S, const JoinLaunch &p, const JoinQuery &Q, uint32_t q,
                                         const CandView &cv, uint32_t P, uint32_t bc,
                                         uint32_t lane, unsigned long long &scanned, uint32_t &probes) {
  const uint32_t L = P + 1;
  const uint32_t bucket = Q.use_labels ? S.lbk[L] : kNone;
  const uint32_t lt = (1u << lane) - 1;
  const bool fast_ok = Q.fast_last && !p.emit;  // k_last_counts ran only then
  // several back edges, some to levels before P: the hoisted set of the prefix
  const uint32_t fixed = S.bmask[L] & ((1u << P) - 1);
  const bool p_indep = !((S.bmask[L] >> P) & 1u);  // u_L not adjacent to level P: only |X| matters
  uint32_t xn = kHoistTooBig;
  if (p.hoist && !p.emit && !Q.fast_last && fixed) {
    if (*S.xlen == kHoistInvalid) build_hoisted(S, p, Q, cv, P, fixed, !p_indep, lane, scanned, probes);
    xn = *S.xlen;
  }
  const bool use_x = xn != kHoistTooBig;
  uint32_t len = 0, fast = 0;
  if (lane < bc) {
    uint32_t v = S.batch[P * 32 + lane];
    if (!SMG_DCHECK(v < p.n, 106, v, P)) v = 0;
    bool counted = false;
    if (use_x) {
      const uint32_t vb = __ldg(p.off + v), vd = __ldg(p.off + v + 1) - vb;
      if (p_indep) {
        // u_L is not adjacent to level P: every candidate sees the whole set,
        // less itself when it has u_L's label and belongs to the set (tested
        // directly: the set may be counted rather than stored)
        bool member = false;
        if ((S.slab[L] >> P) & 1u) {
          const uint32_t u = S.ord[L];
          member = cv.has(u, v);
          for (uint32_t b = S.slab[L] & ((1u << P) - 1); b && member; b &= b - 1) member = S.m[__ffs(b) - 1] != v;
          for (uint32_t b = fixed; b && member; b &= b - 1) {
            const uint32_t j = __ffs(b) - 1;
            member = is_neighbor(p, S.m[j], S.beg[j], S.deg[j], S.hub[j], bucket, v, probes);
          }
        }
        fast = xn - (member ? 1u : 0u);
        counted = true;
      } else {
        // |X & N(v)|: walk v's run keeping members of X, or walk X probing
        // N(v), whichever is shorter
        const uint32_t rv = run_len(p, S, Q.use_labels, L, v, vd);
        const uint32_t hv = __ldg(p.hub_of + v);
        uint32_t mode = kHoistSet, base = 0;
        if (hoist_scan_run(p, rv, xn)) {
          const uint32_t *lst = scan_list(p, S, Q.use_labels, L, v, vb, vd, len);
          const bool from_l = lst != p.adj + vb;
          base = static_cast<uint32_t>(lst - (from_l ? p.adjl : p.adj));
          mode = kHoistScan | (from_l ? kFromLabelIndex : 0u);
        } else {
          len = xn;
        }
        S.sv[lane] = v;
        S.sbeg[lane] = vb;
        S.sdeg[lane] = vd;
        S.shub[lane] = hv;
        S.sbase[lane] = base;
        S.spiv[lane] = P | mode;
        counted = true;
      }
    }
    if (!counted && fast_ok) {
      // one back edge, to level fb: the stored neighbour count of its vertex
      // a, less the matched vertices of the last vertex's label adjacent to a
      const uint32_t fb = Q.fast_last - 1;
      const uint32_t a = fb == P ? v : S.m[fb];
      const uint32_t c = __ldg(Q.lastcnt + a);
      if (c != kNone) {
        uint32_t corr = 0;
        if (S.slab[L]) {
          uint32_t ab, ad, ah;
          if (fb == P) {
            ab = __ldg(p.off + v);
            ad = __ldg(p.off + v + 1) - ab;
            ah = __ldg(p.hub_of + v);
          } else {
            ab = S.beg[fb];
            ad = S.deg[fb];
            ah = S.hub[fb];
          }
          const uint32_t u = S.ord[L];
          for (uint32_t b = S.slab[L]; b; b &= b - 1) {
            const uint32_t j = __ffs(b) - 1;
            const uint32_t x = j == P ? v : S.m[j];
            if (x != a && cv.has(u, x) && is_neighbor(p, a, ab, ad, ah, bucket, x, probes)) ++corr;
          }
        }
        fast = c - corr;
        counted = true;  // a zero-length segment: the scan below never visits it
      }
    }
    if (!counted) {
      const uint32_t vb = __ldg(p.off + v), vd = __ldg(p.off + v + 1) - vb;
      const uint32_t piv = choose_pivot(p, S, Q.use_labels, L, P, v, vd);
      const uint32_t pb = piv == P ? vb : S.beg[piv];
      const uint32_t *lst =
          scan_list(p, S, Q.use_labels, L, piv == P ? v : S.m[piv], pb, piv == P ? vd : S.deg[piv], len);
      const bool from_l = lst != p.adj + pb;
      if (len > (Q.split_len ? Q.split_len : kSplitLen)) len = split_last(S, p, Q, q, P, v, len);
      S.sv[lane] = v;
      S.sbeg[lane] = vb;
      S.sdeg[lane] = vd;
      S.shub[lane] = __ldg(p.hub_of + v);
      S.sbase[lane] = static_cast<uint32_t>(lst - (from_l ? p.adjl : p.adj));
      S.spiv[lane] = piv | (from_l ? kFromLabelIndex : 0u);
    }
  }
  uint32_t incl = len;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= static_cast<uint32_t>(o)) incl += t;
  }
  const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
  S.spre[lane] = incl - len;
  __syncwarp();
  scanned += total;
  unsigned long long cnt = (fast_ok || use_x) ? __reduce_add_sync(0xFFFFFFFFu, fast) : 0u;
  const uint32_t u = S.ord[L];
  const uint32_t back = S.bmask[L], same = S.slab[L];
  for (uint32_t t0 = 0; t0 < total; t0 += 32) {
    const uint32_t t = t0 + lane;
    bool good = false;
    uint32_t w = 0, i = 0;
    if (t < total) {
      uint32_t lo = 0, hi = bc;  // last segment starting at or before t
      while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (S.spre[mid] <= t)
          lo = mid;
        else
          hi = mid;
      }
      i = lo;
      const uint32_t vi = S.sv[i];
      const uint32_t sp = S.spiv[i];
      if (sp & kHoistSet) {  // a member of the hoisted set: is it a neighbour of v?
        w = S.xs[t - S.spre[i]];
        good = is_neighbor(p, vi, S.sbeg[i], S.sdeg[i], S.shub[i], bucket, w, probes);
      } else {
        const uint64_t ai = static_cast<uint64_t>(S.sbase[i]) + (t - S.spre[i]);
        const bool in_adj = SMG_DCHECK(ai < p.m2, 107, ai, i);
        w = in_adj ? __ldg(((sp & kFromLabelIndex) ? p.adjl : p.adj) + ai) : 0u;
        if (sp & kHoistScan) {  // a neighbour of v: is it in the hoisted set?
          good = in_adj && in_hoisted(S, xn, w);
        } else {
          good = in_adj && SMG_DCHECK(w < p.n, 108, w, ai) &&
                 ((sp & kFromLabelIndex) && cv.crow && p.adjr ? cv.has_rank(u, __ldg(p.adjr + ai)) : cv.has(u, w));
          for (uint32_t b = same; b && good; b &= b - 1) {
            const uint32_t j = __ffs(b) - 1;
            good = (j == P ? vi : S.m[j]) != w;
          }
          // back edges other than the pivot's (whose list w comes from)
          for (uint32_t b = back & ~(1u << (sp & 31u)); b && good; b &= b - 1) {
            const uint32_t j = __ffs(b) - 1;
            if (j == P)
              good = is_neighbor(p, vi, S.sbeg[i], S.sdeg[i], S.shub[i], bucket, w, probes);
            else
              good = is_neighbor(p, S.m[j], S.beg[j], S.deg[j], S.hub[j], bucket, w, probes);
          }
        }
      }
    }
    const uint32_t bal = __ballot_sync(0xFFFFFFFFu, good);
    cnt += __popc(bal);
    if (p.emit && bal) {
      unsigned long long pos = 0;
      if (lane == 0) pos = atomicAdd(Q.emb_count, static_cast<unsigned long long>(__popc(bal)));
      pos = __shfl_sync(0xFFFFFFFFu, pos, 0);
      const unsigned long long r = pos + __popc(bal & lt);
      if (good && r < Q.emb_cap) {
        uint32_t *row = Q.emb + r * Q.k;
        for (uint32_t j = 0; j < P; ++j) row[S.ord[j]] = S.m[j];
        row[S.ord[P]] = S.sv[i];
        row[S.ord[L]] = w;
      }
    }
  }
  __syncwarp();
  return cnt;
}

// While warps wait for work (tickets beyond the tail), split off the
// shallowest unexplored work of this warp's stack: the back half of a level's
// unscanned list, or else one untried candidate of a level's batch (which
// becomes a task one level deeper).  Returns true when something was pushed.
__device__ bool try_donate(WarpView &S, const JoinLaunch &p, uint32_t q, unsigned long long *qpending, uint32_t L0,
                           uint32_t level, uint32_t P, uint32_t lane, uint32_t min_rem) {
  int pushed = 0;
  if (lane == 0) {
    QueueState *qs = p.qs;
    const unsigned long long h = vload(qs->head), t = vload(qs->tail);
    {
      // tickets beyond the tail are warps waiting for work
      if (h > t && t < p.cap && !*reinterpret_cast<volatile int *>(&qs->closing)) {
        uint32_t tl = kNone, lo = 0, hi = 0, item = 0;
        for (uint32_t l = L0; l <= level && tl == kNone; ++l) {
          const uint32_t c = S.cur[l], e = S.end[l];
          const uint32_t rem = e > c ? e - c : 0;
          if (rem >= min_rem || (rem >= 1 && l < level)) {
            tl = l;
            lo = c + rem / 2;
            hi = e;
          } else if (l < P) {
            const uint32_t left = S.bcnt[l] - S.bidx[l];
            if (left >= 2 || (left == 1 && l < level)) {
              tl = l + 1;
              item = S.batch[l * 32 + S.bcnt[l] - 1];
              lo = 0;
              hi = kNone;
            }
          }
        }
        if (tl != kNone) {
          const unsigned long long slot = atomicAdd(&qs->tail.v, 1ull);
          if (slot < p.cap) {
            atomicAdd(&qs->pending.v, 1ull);
            atomicAdd(qpending, 1ull);
            uint32_t *T = p.tasks + slot * (4 + p.kmax);
            T[0] = q;
            T[1] = tl;
            T[2] = lo;
            T[3] = hi;
            if (hi == kNone) {  // a batch candidate: prefix m[0..tl-2] plus the candidate
              for (uint32_t j = 0; j + 1 < tl; ++j) T[4 + j] = S.m[j];
              T[4 + tl - 1] = item;
              --S.bcnt[tl - 1];
            } else {
              for (uint32_t j = 0; j < tl; ++j) T[4 + j] = S.m[j];
              S.end[tl] = lo;
            }
            __threadfence();
            atomicExch(p.ready + slot, 1u);
            atomicAdd(&qs->donations, 1ull);
            pushed = 1;
          } else {
            qs->full = 1;
          }
        }
      }
    }
  }
  pushed = __shfl_sync(0xFFFFFFFFu, pushed, 0);
  __syncwarp();
  return pushed != 0;
}

// Breadth-first level: the batch of `taken` accepted candidates of `level`
// (< P) becomes `taken` tasks one level deeper (prefix m[0..level-1] plus the
// candidate, the whole list of the next level), appended behind every task
// queued so far, instead of being descended into one by one.  Only while the
// queue's tail stays within the launch's breadth-first budget: past it the
// warp keeps its batch and goes on depth-first, so the frontier held in the
// queue is bounded.  Returns true when the batch was queued.
__device__ __noinline__ bool bfs_push(const WarpView &S, const JoinLaunch &p, uint32_t q,
                                      unsigned long long *qpending, uint32_t level, uint32_t taken, uint32_t lane) {
  QueueState *qs = p.qs;
  unsigned long long first = 0;
  int ok = 0;
  if (lane == 0 && !*reinterpret_cast<volatile int *>(&qs->closing) && vload(qs->tail) + taken <= p.bfs_budget) {
    first = atomicAdd(&qs->tail.v, static_cast<unsigned long long>(taken));
    if (first + taken <= p.cap) {
      ok = 1;
      atomicAdd(&qs->pending.v, static_cast<unsigned long long>(taken));
      atomicAdd(qpending, static_cast<unsigned long long>(taken));
    } else {
      // no room: the slot numbers taken stay unpublished and are never waited
      // for beyond the end of the run (their tickets see pending reach zero)
      atomicExch(&qs->full, 1);
    }
  }
  ok = __shfl_sync(0xFFFFFFFFu, ok, 0);
  if (!ok) return false;
  first = __shfl_sync(0xFFFFFFFFu, first, 0);
  if (lane < taken) {
    uint32_t *T = p.tasks + (first + lane) * (4 + p.kmax);
    T[0] = q;
    T[1] = level + 1;
    T[2] = 0;
    T[3] = kNone;
    for (uint32_t j = 0; j < level; ++j) T[4 + j] = S.m[j];
    T[4 + level] = S.batch[level * 32 + lane];
    __threadfence();
    atomicExch(p.ready + first + lane, 1u);
  }
  if (lane == 0) atomicAdd(&qs->bfs_tasks, static_cast<unsigned long long>(taken));
  __syncwarp();
  return true;
}

// End of a time slice: every part of this warp's stack that is not done
// becomes a task of the next slice's queue: the unscanned rest of each level's
// list, and each untried batch candidate (as a task one level deeper).  The
// next queue must also take this queue's untaken tasks (at most its tail) and
// what racing warps still push (kPreemptSlack).  Returns false (and the warp
// keeps working) when they would not fit.
__device__ bool preempt(WarpView &S, const JoinLaunch &p, uint32_t q, unsigned long long *qpending, uint32_t L0,
                        uint32_t level, uint32_t P, uint32_t lane) {
  int ok = 0;
  if (lane == 0) {
    // per level at most two tasks: the untried part of its batch, as the list
    // range from the first untried entry to just past the last one still in
    // the batch (entries in between that failed their tests fail again;
    // entries a donation took from the batch's end lie beyond it), and the
    // unscanned rest of the list
    uint32_t n = 0;
    for (uint32_t l = L0; l <= level; ++l) {
      if (S.cur[l] < S.end[l]) ++n;
      if (l < P && S.bidx[l] < S.bcnt[l]) ++n;
    }
    if (n == 0) {
      ok = 1;
    } else {
      const unsigned long long tail = vload(p.qs->tail);
      unsigned int old = *reinterpret_cast<volatile unsigned int *>(p.next_count);
      unsigned int base = kNone;
      while (static_cast<unsigned long long>(old) + n + tail + kPreemptSlack <= p.cap) {
        const unsigned int seen = atomicCAS(p.next_count, old, old + n);
        if (seen == old) {
          base = old;
          break;
        }
        old = seen;
      }
      if (base != kNone) {
        const uint32_t tw = 4 + p.kmax;
        uint32_t idx = base;
        for (uint32_t l = L0; l <= level; ++l) {
          if (S.cur[l] < S.end[l]) {
            uint32_t *T = p.next_tasks + static_cast<uint64_t>(idx) * tw;
            T[0] = q;
            T[1] = l;
            T[2] = S.cur[l];
            T[3] = S.end[l];
            for (uint32_t j = 0; j < l; ++j) T[4 + j] = S.m[j];
            p.next_ready[idx++] = 1;
          }
          if (l < P && S.bidx[l] < S.bcnt[l]) {
            uint32_t *T = p.next_tasks + static_cast<uint64_t>(idx) * tw;
            T[0] = q;
            T[1] = l;
            T[2] = S.bpos[l * 32 + S.bidx[l]];
            T[3] = S.bpos[l * 32 + S.bcnt[l] - 1] + 1;
            for (uint32_t j = 0; j < l; ++j) T[4 + j] = S.m[j];
            p.next_ready[idx++] = 1;
          }
        }
        atomicAdd(qpending, static_cast<unsigned long long>(n));
        ok = 1;
      }
    }
  }
  ok = __shfl_sync(0xFFFFFFFFu, ok, 0);
  __syncwarp();
  return ok != 0;
}

// The warp that took a served query's pending count to zero publishes the
// final count to the host-mapped completion record.  Every warp added its
// share to Q.count before a fence and its pending decrement, so the count
// read here after the last decrement is final.
__device__ __forceinline__ void notify_done(const JoinQuery &Q) {
  __threadfence();
  const unsigned long long total = atomicAdd(Q.count, 0ull);
  *reinterpret_cast<volatile unsigned long long *>(Q.done_count) = total;
  __threadfence_system();
  *reinterpret_cast<volatile uint32_t *>(Q.done_gen) = Q.gen;
}

__device__ __forceinline__ void join_body(const JoinLaunch &p) {
  extern __shared__ __align__(16) uint32_t smem[];
  const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const uint32_t K = p.kmax, tw = 4 + K;
  WarpView S(smem + wib * warp_words(K), K);
  if (p.xbuf) {  // a larger hoisted-set buffer of this warp's own in global memory
    S.xs = p.xbuf + (static_cast<uint64_t>(blockIdx.x) * kWarpsPerBlock + wib) * p.xcap;
    S.xcap = p.xcap;
  }
  const uint32_t lt = (1u << lane) - 1;
  QueueState *qs = p.qs;
  volatile int *vabort = &qs->abort;
  uint64_t idle_mark = 0, idle_t0 = 0;
  unsigned long long scanned = 0, descents = 0, model = 0;
  uint32_t probes = 0;

  while (true) {
    int got = 0;
    unsigned long long slot = 0;
    if (lane == 0) {
      if (!*reinterpret_cast<volatile int *>(&qs->closing)) {
        slot = atomicAdd(&qs->head.v, 1ull);
        got = wait_ticket(p, slot, idle_mark, idle_t0);
        if (got == 1) p.ready[slot] = 2;  // taken (a time-sliced run carries untaken ones over)
      }
    }
    got = __shfl_sync(0xFFFFFFFFu, got, 0);
    if (got != 1) break;
    slot = __shfl_sync(0xFFFFFFFFu, slot, 0);
    // Lane 0 acquired the task's ready flag; the barrier orders that before
    // every lane's reads, and the reads go to L2 (__ldcg): a donated task was
    // written during this launch by another SM, and this SM's L1 may hold an
    // older copy of the line from a neighbouring slot.
    __syncwarp();
    const uint32_t *T = p.tasks + static_cast<uint64_t>(slot) * tw;
    const uint32_t q = __ldcg(T), L0 = __ldcg(T + 1), lo = __ldcg(T + 2), hi = __ldcg(T + 3);
    if (!SMG_DCHECK(q < p.nq, 109, q, p.nq)) break;
    const JoinQuery &Q = p.queries[q];
    const uint32_t k = Q.k, P = k - 2;
    if (!SMG_DCHECK(L0 <= P + 1, 110, L0, k)) break;
    // the query's cap on stored hoisted sets, within this warp's buffer
    S.xcap = min(p.xbuf ? p.xcap : kHoistCap, Q.hoist_cap ? Q.hoist_cap : 0xFFFFFFFFu);
    int drop = 0;
    if (lane == 0) drop = (Q.count_limit || Q.work_limit) && *reinterpret_cast<volatile uint32_t *>(Q.over);
    drop = __shfl_sync(0xFFFFFFFFu, drop, 0);
    if (drop) {  // the query is over its count limit
      if (lane == 0) {
        atomicAdd(&qs->tasks_done, 1ull);
        atomicAdd(&qs->progress.v, 1ull);
        atomicAdd(Q.pending, ~0ull);
        atomicAdd(&qs->pending.v, ~0ull);
      }
      continue;
    }
    if (lane < k) {
      S.ord[lane] = Q.order[lane];
      S.bmask[lane] = Q.back_mask[lane];
      S.slab[lane] = Q.same_label[lane];
      S.lbk[lane] = Q.level_bucket[lane];
    }
    if (lane < L0) {
      uint32_t v = __ldcg(T + 4 + lane);
      if (!SMG_DCHECK(v < p.n, 111, v, lane)) v = 0;
      S.m[lane] = v;
      const uint32_t b = __ldg(p.off + v);
      S.beg[lane] = b;
      S.deg[lane] = __ldg(p.off + v + 1) - b;
      S.hub[lane] = __ldg(p.hub_of + v);
    }
    __syncwarp();
    CandView cv;
    cv.bits = Q.cbits;
    cv.words = Q.cwords;
    cv.mask = Q.candmask;
    cv.crow = Q.crow;
    unsigned long long cnt = 0;
    bool aborted = false, preempted = false;
    uint32_t iter = 0;  // steps of this task (work limit)
    if (L0 == P + 1) {
      // a slice of one last-level list, split off by last_level
      cnt = last_level_range(S, p, Q, cv, P, lo, hi, lane, scanned, probes);
    } else {
    if (lane == 0) {
      if (L0 == 0) {
        S.lbase[0] = Q.roots;
        S.cur[L0] = lo;
        S.end[L0] = hi;
      } else {
        const uint32_t pv = choose_pivot(p, S, Q.use_labels, L0);
        uint32_t len = 0;
        S.piv[L0] = pv;
        S.lbase[L0] = scan_list(p, S, Q.use_labels, L0, S.m[pv], S.beg[pv], S.deg[pv], len);
        S.cur[L0] = lo;
        S.end[L0] = hi == kNone ? len : min(hi, len);
        // a split-off batch candidate: its row was never expanded by the donor
        if (p.count_model && hi == kNone) model += 4ull * L0 + level_model(S, L0);
      }
      S.bcnt[L0] = 0;
      S.bidx[L0] = 0;
      *S.xlen = kHoistInvalid;  // a new prefix
    }
    __syncwarp();

    uint32_t level = L0, tick = 0;  // tick paces donation checks

    const uint32_t donate_min = max(2u, Q.donate_min ? Q.donate_min : p.donate_min);
    while (true) {
      if ((++iter & 255) == 0) {
        int stop = 0;
        if (lane == 0) {
          atomicAdd(&qs->progress.v, 1ull);
          if (Q.count_limit) {
            // publish the running count so that the limit sees every warp's share
            if (cnt) {
              const unsigned long long before = atomicAdd(Q.count, cnt);
              if (before + cnt > Q.count_limit) *Q.over = 1;
            }
          }
          if (Q.work_limit && atomicAdd(Q.work, 256ull) + 256ull > Q.work_limit) *Q.over = 1;
          if ((Q.count_limit || Q.work_limit) && *reinterpret_cast<volatile uint32_t *>(Q.over)) {
            stop = 2;  // this query is over its limit: drop the task, keep running
          } else if (*vabort) {
            stop = 1;
          } else if (now_ns() - *reinterpret_cast<volatile unsigned long long *>(&qs->start_ns) > p.time_limit_ns) {
            set_error(qs, JOIN_ERR_DEADLINE);
            stop = 1;
          }
        }
        stop = __shfl_sync(0xFFFFFFFFu, stop, 0);
        if (Q.count_limit) cnt = 0;  // flushed above
        if (stop == 2) {
          cnt = 0;
          break;
        }
        if (stop) {
          aborted = true;
          break;
        }
      }
      // time slice over (serving): hand the rest of this stack back and leave
      if (p.slice_ns && (iter & 31) == 0) {
        int close = 0;
        if (lane == 0) {
          if (*reinterpret_cast<volatile int *>(&qs->closing)) {
            close = 1;
          } else {
            const uint64_t el = now_ns() - *reinterpret_cast<volatile unsigned long long *>(&qs->start_ns);
            if (el > p.slice_ns || (el > p.slice_min_ns && p.bell && *p.bell)) {
              atomicExch(&qs->closing, 1);
              close = 1;
            }
          }
        }
        close = __shfl_sync(0xFFFFFFFFu, close, 0);
        if (close && !(level == P && S.bcnt[P] != 0) && preempt(S, p, q, Q.pending, L0, level, P, lane)) {
          preempted = true;
          break;
        }
      }
      // give the shallowest unexplored work of this stack to a waiting warp
      if ((++tick & p.donate_every_mask) == 0) {
        if (try_donate(S, p, q, Q.pending, L0, level, P, lane, donate_min)) continue;
      }
      if (level == P) {
        const uint32_t bc = S.bcnt[level];
        if (bc) {
          if (p.count_model) {
            // each candidate's row of P + 1 vertices, written and expanded
            // (complete embeddings are counted, not written)
            unsigned long long mb = 0;
            if (lane < bc) {
              const uint32_t v = S.batch[P * 32 + lane];
              const uint32_t vd = __ldg(p.off + v + 1) - __ldg(p.off + v);
              mb = 4ull * (P + 1) + level_model(S, P + 1, P, vd);
            }
            for (int o = 16; o; o >>= 1) mb += __shfl_down_sync(0xFFFFFFFFu, mb, o);
            if (lane == 0) model += mb;
          }
          cnt += last_level(S, p, Q, q, cv, P, bc, lane, scanned, probes);
          descents += bc;
          if (lane == 0) S.bcnt[level] = 0;
          __syncwarp();
          if (Q.count_limit && cnt >= kLimitFlush) {
            // publish early so that a query over its limit stops soon
            int over = 0;
            if (lane == 0) {
              const unsigned long long before = atomicAdd(Q.count, cnt);
              over = before + cnt > Q.count_limit;
              if (over) *Q.over = 1;
            }
            cnt = 0;
            if (__shfl_sync(0xFFFFFFFFu, over, 0)) break;
          }
          continue;
        }
      } else {
        const uint32_t bi = S.bidx[level], bc = S.bcnt[level];
        if (bi < bc) {
          // descend into the next tested candidate
          uint32_t v = S.batch[level * 32 + bi];
          if (!SMG_DCHECK(v < p.n, 113, v, level)) v = 0;
          __syncwarp();
          if (lane == 0) {
            S.bidx[level] = bi + 1;
            S.m[level] = v;
            const uint32_t b = __ldg(p.off + v);
            S.beg[level] = b;
            S.deg[level] = __ldg(p.off + v + 1) - b;
            S.hub[level] = __ldg(p.hub_of + v);
          }
          __syncwarp();
          const uint32_t nl = level + 1;
          if (lane == 0) {
            const uint32_t pv = choose_pivot(p, S, Q.use_labels, nl);
            uint32_t len = 0;
            S.piv[nl] = pv;
            S.lbase[nl] = scan_list(p, S, Q.use_labels, nl, S.m[pv], S.beg[pv], S.deg[pv], len);
            S.cur[nl] = 0;
            S.end[nl] = len;
            S.bcnt[nl] = 0;
            S.bidx[nl] = 0;
            if (nl == P) *S.xlen = kHoistInvalid;  // the prefix m[0..P-1] changed
            if (p.count_model) model += 4ull * nl + level_model(S, nl);  // the row written, then expanded
          }
          __syncwarp();
          ++descents;
          level = nl;
          continue;
        }
      }
      const uint32_t c = S.cur[level];
      uint32_t e = S.end[level];
      if (c < e) {
        // refill the batch: test the next 32 x kWays entries (entry c + 32 i
        // + lane in way i), keep the first 32 that pass in list order, and
        // resume after the last one kept (entries beyond it are tested again)
        const uint32_t n = min(32u * kWays, e - c);
        scanned += n;
        const uint32_t *base = S.lbase[level];
        const uint32_t *rk = level != 0 ? cv.ranks_of(p, base) : nullptr;
        uint32_t w[kWays], r[kWays], live = 0;
#pragma unroll
        for (int i = 0; i < kWays; ++i) {
          const uint32_t t = 32u * i + lane;
          w[i] = 0;
          r[i] = 0;
          if (t < n && SMG_DCHECK(level == 0 ? c + t < *Q.num_roots : in_lists(p, base + c + t), 114, c + t, level)) {
            w[i] = __ldg(base + c + t);
            if (rk) r[i] = __ldg(rk + c + t);
            if (SMG_DCHECK(w[i] < p.n, 112, w[i], level)) live |= 1u << i;
          }
        }
        if (level != 0) live = accept_multi(S, p, cv, Q.use_labels, level, w, r, rk != nullptr, live, probes);
        uint32_t taken = 0, stop = n;
#pragma unroll
        for (int i = 0; i < kWays; ++i) {
          const bool good = (live >> i) & 1u;
          const uint32_t bal = __ballot_sync(0xFFFFFFFFu, good);
          if (taken < 32 && bal) {
            const uint32_t room = 32 - taken;
            const uint32_t keep = __ballot_sync(0xFFFFFFFFu, good && __popc(bal & lt) < room);
            if ((keep >> lane) & 1u) {
              const uint32_t pos = taken + __popc(keep & lt);
              S.batch[level * 32 + pos] = w[i];
              S.bpos[level * 32 + pos] = c + 32u * i + lane;
            }
            taken += __popc(keep);
            if (taken == 32) stop = 32u * i + (31 - __clz(keep)) + 1;
          }
        }
        __syncwarp();
        // a breadth-first level queues the whole batch (one task per
        // candidate) and goes on scanning its list
        if (taken && p.bfs_budget && level < P && level < Q.bfs_depth &&
            bfs_push(S, p, q, Q.pending, level, taken, lane)) {
          descents += taken;
          taken = 0;
        }
        if (lane == 0) {
          S.bcnt[level] = taken;
          S.bidx[level] = 0;
          S.cur[level] = c + stop;
        }
        __syncwarp();
        continue;
      }
      if (level == L0) break;
      --level;
    }
    }  // L0 <= P
    unsigned long long pr = probes;
    probes = 0;
    for (int o = 16; o; o >>= 1) pr += __shfl_down_sync(0xFFFFFFFFu, pr, o);
    if (lane == 0) {
      if (cnt) {
        const unsigned long long before = atomicAdd(Q.count, cnt);
        if (Q.count_limit && before + cnt > Q.count_limit) *Q.over = 1;
      }
      // the steps of this task not yet charged in blocks of 256, plus one for
      // the task itself (a query split into many short tasks is charged too)
      if (Q.work_limit) {
        const unsigned long long w = (iter & 255u) + 1u;
        if (atomicAdd(Q.work, w) + w > Q.work_limit) *Q.over = 1;
      }
      atomicAdd(&qs->scanned, scanned);
      atomicAdd(&qs->descents, descents);
      if (model) atomicAdd(&qs->model_bytes, model);
      if (pr) atomicAdd(&qs->probes, pr);
      if (!aborted) {
        atomicAdd(&qs->tasks_done, 1ull);
        atomicAdd(&qs->progress.v, 1ull);
        if (Q.done_gen) __threadfence();  // this task's count before its pending decrement
        const unsigned long long left = atomicAdd(Q.pending, ~0ull);  // -1
        atomicAdd(&qs->pending.v, ~0ull);                             // -1
        if (left == 1 && Q.done_gen) notify_done(Q);
      }
    }
    scanned = 0;
    descents = 0;
    model = 0;
    if (aborted || preempted) break;
  }
}

// The join is bound by the latency of its scattered reads, so it trades
// registers for resident warps.  On the 2^22 R-MAT workload (scanning whole
// lists), 8 blocks of 8 warps per SM (32 registers, a 476-byte spill)
// measured 501 queries/s, 6 blocks (40 registers) 426 and 4 blocks (64
// registers) 357; the compiler's own choice, 80 registers, fits 3.  Once the
// label index, counted and hoisted last levels removed most of the list
// scanning, the spills cost more than the extra warps gain: 4 blocks (64
// registers, no spill to speak of) measured 3,647 queries/s, 6 blocks 3,453
// and 8 blocks 3,477, so 4 is the default.  A launch takes the most blocks
// its shared memory allows; SMG_JOIN_OCCUPANCY=4|6|8 caps it.
__global__ void __launch_bounds__(kWarpsPerBlock * 32, 8) k_join(JoinLaunch p) { join_body(p); }
__global__ void __launch_bounds__(kWarpsPerBlock * 32, 6) k_join6(JoinLaunch p) { join_body(p); }
__global__ void __launch_bounds__(kWarpsPerBlock * 32, 4) k_join4(JoinLaunch p) { join_body(p); }

__global__ void k_slice_begin(QueueState *qs) {
  qs->start_ns = now_ns();
  qs->closing = 0;
}

// Appends the published-but-untaken tasks of the old queue (ready == 1) to
// the new queue behind what preempted warps wrote there.  A warp takes 32
// slots, claims room for its kept tasks with one atomic and copies them with
// its lanes over the task's words.  A task that would not fit records
// JOIN_ERR_QUEUE_FULL (preempt leaves room for every untaken task, so this is
// a guard, not a path).
__global__ void k_compact(const uint32_t *__restrict__ tasks_old, const uint32_t *__restrict__ ready_old,
                          uint32_t cap, uint32_t tw, uint32_t *__restrict__ tasks_new,
                          uint32_t *__restrict__ ready_new, unsigned int *new_count, QueueState *qs) {
  const unsigned long long tail = *reinterpret_cast<volatile unsigned long long *>(&qs->tail.v);
  const uint32_t n_old = static_cast<uint32_t>(min(tail, static_cast<unsigned long long>(cap)));
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint64_t base = static_cast<uint64_t>(warp) * 32; base < n_old; base += static_cast<uint64_t>(nwarps) * 32) {
    const uint64_t i = base + lane;
    const bool keep = i < n_old && ready_old[i] == 1;
    const uint32_t bal = __ballot_sync(0xFFFFFFFFu, keep);
    if (!bal) continue;
    unsigned int first = 0;
    if (lane == 0) first = atomicAdd(new_count, static_cast<unsigned int>(__popc(bal)));
    first = __shfl_sync(0xFFFFFFFFu, first, 0);
    uint32_t r = 0;
    for (uint32_t bb = bal; bb; bb &= bb - 1, ++r) {
      const uint64_t src = base + __ffs(bb) - 1, dst = static_cast<uint64_t>(first) + r;
      if (dst >= cap) {
        if (lane == 0) atomicCAS(&qs->error, 0, JOIN_ERR_QUEUE_FULL);
        break;
      }
      for (uint32_t j = lane; j < tw; j += 32) tasks_new[dst * tw + j] = tasks_old[src * tw + j];
      if (lane == 0) ready_new[dst] = 1;
    }
  }
}

// The new queue holds new_count tasks: head 0, tail = pending = that count.
__global__ void k_compact_finish(QueueState *qs, unsigned int *new_count, uint32_t cap) {
  const unsigned long long n = min(static_cast<unsigned long long>(*new_count), static_cast<unsigned long long>(cap));
  qs->head.v = 0;
  qs->tail.v = n;
  qs->pending.v = n;
  qs->closing = 0;
  *new_count = 0;
}

}  // namespace

smg_status launch_slice_begin(QueueState *qs, cudaStream_t s) {
  k_slice_begin<<<1, 1, 0, s>>>(qs);
  SMG_CUDA(cudaGetLastError());
  return SMG_OK;
}

smg_status launch_compact(const uint32_t *tasks_old, const uint32_t *ready_old, uint32_t cap, uint32_t tw,
                          uint32_t *tasks_new, uint32_t *ready_new, unsigned int *new_count, QueueState *qs,
                          cudaStream_t s, int num_sms) {
  k_compact<<<std::max(num_sms, 1) * 4, 256, 0, s>>>(tasks_old, ready_old, cap, tw, tasks_new, ready_new, new_count,
                                                      qs);
  SMG_CUDA(cudaGetLastError());
  k_compact_finish<<<1, 1, 0, s>>>(qs, new_count, cap);
  SMG_CUDA(cudaGetLastError());
  return SMG_OK;
}

#ifdef SMG_CHECKED
extern "C" int smg_debug_check_join(unsigned long long *out) {
  return static_cast<int>(cudaMemcpyFromSymbol(out, g_check_record, 3 * sizeof(unsigned long long)));
}
#endif

void set_graph(JoinLaunch &jl, const DevGraph &g) {
  jl.off = g.off;
  jl.adj = g.adj;
  jl.hub_of = g.hub_of;
  jl.hub_bits = g.hub_bits;
  jl.hub_words = g.hub_words;
  jl.adjl = g.adjl;
  jl.lab_of = g.lab_of;
  jl.lab_off = g.lab_off;
  jl.lab_buckets = g.lab_buckets;
  jl.adjr = g.adjr;
  jl.label = g.label;
  jl.lverts = g.lverts;
  jl.lab_rank = g.hub_by_label ? g.lab_rank : nullptr;
  jl.bucket_word_off = g.hub_by_label ? g.bucket_word_off : nullptr;
  jl.n = g.n;
  jl.m2 = g.m2;
  jl.num_hubs = g.num_hubs;
}

uint32_t hoist_global_cap() {
  static const uint32_t v = [] {
    const char *e = std::getenv("SMG_HOIST_CAP");
    const long x = e ? std::atol(e) : 4096;
    return static_cast<uint32_t>(std::min<long>(std::max<long>(x, 256), 1 << 20));
  }();
  return v;
}

size_t hoist_buffer_bytes(int num_sms) {
  // at most 8 resident blocks of kWarpsPerBlock warps per SM
  return static_cast<size_t>(std::max(num_sms, 1)) * 8 * kWarpsPerBlock * hoist_global_cap() * sizeof(uint32_t);
}

size_t join_queue_bytes(uint32_t cap, uint32_t kmax) {
  return static_cast<size_t>(cap) * (4 + kmax) * sizeof(uint32_t) + static_cast<size_t>(cap) * sizeof(uint32_t);
}

namespace {

using JoinKernel = void (*)(JoinLaunch);

uint32_t occupancy_cap() {
  static const uint32_t cap = [] {
    const char *e = std::getenv("SMG_JOIN_OCCUPANCY");
    const int v = e ? std::atoi(e) : 4;
    return static_cast<uint32_t>(v >= 8 ? 8 : v >= 6 ? 6 : 4);
  }();
  return cap;
}

// The variant whose register budget matches the blocks that fit: 8 or 6 only
// when that many blocks' shared memory fits an SM.
JoinKernel join_kernel(size_t smem_per_block) {
  const size_t sm_bytes = 227 * 1024;
  const uint32_t cap = occupancy_cap();
  if (cap >= 8 && 8 * (smem_per_block + 1024) <= sm_bytes) return k_join;
  if (cap >= 6 && 6 * (smem_per_block + 1024) <= sm_bytes) return k_join6;
  return k_join4;
}

// Membership probes: hub bitmaps and id-ordered lists (default), or, with
// SMG_PROBE=runs, binary searches of label runs where a vertex has them.
bool probe_runs() {
  static const bool v = [] {
    const char *e = std::getenv("SMG_PROBE");
    return e && std::string(e) == "runs";
  }();
  return v;
}

// The hoisted last-level set (SMG_HOIST=0 turns it off).
bool hoist_enabled() {
  static const bool v = [] {
    const char *e = std::getenv("SMG_HOIST");
    return !(e && std::string(e) == "0");
  }();
  return v;
}

// How much longer than a hoisted set X a candidate's run may be and still be
// scanned against X rather than X walked against the candidate's list, in
// eighths (SMG_HOIST_SCAN_RATIO; default 8: the shorter side is walked).
uint32_t hoist_scan_x8() {
  static const uint32_t v = [] {
    const char *e = std::getenv("SMG_HOIST_SCAN_RATIO");
    const long c = e ? std::strtol(e, nullptr, 10) : 8;
    return static_cast<uint32_t>(std::min(std::max(c, 1L), 1024L));
  }();
  return v;
}

smg_status launch_persistent(const JoinLaunch &jl_in, cudaStream_t s, int num_sms) {
  JoinLaunch jl = jl_in;
  jl.probe_runs = probe_runs() && jl.adjl != nullptr;
  // How often a warp looks for waiting warps to split work off to: every
  // second step.  On 1,024 R-MAT 2^22 queries, same box, join 134.7-137.2 ms
  // against 137.6-142.2 ms every fourth step, 146-154 ms every eighth and
  // 158-159 ms every step; served at 1,000 requests/s on the 2^24 graph, p99
  // 52.7 ms against 87.6 ms every fourth step.
  static const long donate_env = [] {
    const char *e = std::getenv("SMG_DONATE_EVERY");
    return e ? std::atol(e) : 0L;
  }();
  const long every = donate_env > 0 ? donate_env : 2;
  jl.donate_every_mask = static_cast<uint32_t>(every >= 8 ? 7 : every >= 4 ? 3 : every >= 2 ? 1 : 0);
  jl.hoist = hoist_enabled();
  jl.hoist_scan_x8 = hoist_scan_x8();
  const size_t smem = static_cast<size_t>(kWarpsPerBlock) * warp_words(jl.kmax) * sizeof(uint32_t);
  const JoinKernel kern = join_kernel(smem);
  if (smem > 48 * 1024)
    SMG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  int per_sm = 0;
  SMG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWarpsPerBlock * 32, smem));
  if (jl.max_blocks_per_sm) per_sm = std::min(per_sm, static_cast<int>(jl.max_blocks_per_sm));
  per_sm = std::max(1, per_sm);
  kern<<<num_sms * per_sm, kWarpsPerBlock * 32, smem, s>>>(jl);
  SMG_CUDA(cudaGetLastError());
  return SMG_OK;
}

}  // namespace

smg_status launch_join(const JoinLaunch &jl, cudaStream_t s, int num_sms) {
  if (jl.nq == 0) return SMG_OK;
  const uint32_t seed_threads = 256;
  const uint32_t nseed = jl.seed_list ? jl.seed_n : jl.nq;
  smg_status rc = launch_join_prep(jl, s, num_sms);
  if (rc) return rc;
  k_seed<<<dim3(1, std::min<uint32_t>(nseed, 65535)), seed_threads, 0, s>>>(jl);
  SMG_CUDA(cudaGetLastError());
  return launch_persistent(jl, s, num_sms);
}

smg_status launch_join_only(const JoinLaunch &jl, cudaStream_t s, int num_sms) {
  return launch_persistent(jl, s, num_sms);
}

smg_status launch_join_prep(const JoinLaunch &jl, cudaStream_t s, int num_sms) {
  const uint32_t nq = jl.seed_list ? jl.seed_n : jl.nq;
  if (!nq || !jl.n || jl.emit) return SMG_OK;
  const uint32_t want = std::max<uint32_t>(1, static_cast<uint32_t>(std::max(num_sms, 1)) * 16 / nq);
  const uint32_t span = static_cast<uint32_t>((static_cast<uint64_t>(jl.n) + 255) / 256);  // 32 vertices a warp
  const dim3 g2(std::min(span, want), std::min<uint32_t>(nq, 65535));
  k_last_counts<<<g2, 256, 0, s>>>(jl.queries, jl.seed_list, nq, jl.lverts, jl.off, jl.adj, jl.adjl, jl.lab_of,
                                    jl.lab_off, jl.lab_buckets, jl.n, jl.qs);
  SMG_CUDA(cudaGetLastError());
  return SMG_OK;
}

smg_status launch_seed(const JoinLaunch &jl, cudaStream_t s) {
  const uint32_t n = jl.seed_list ? jl.seed_n : jl.nq;
  if (!n) return SMG_OK;
  k_seed<<<dim3(1, std::min<uint32_t>(n, 65535)), 256, 0, s>>>(jl);
  SMG_CUDA(cudaGetLastError());
  return SMG_OK;
}

smg_status build_label_index(DevGraph &g, const uint64_t *offsets, const uint32_t *adj, const uint32_t *labels,
                             uint32_t min_degree, size_t max_bytes, cudaStream_t s) {
  const uint32_t n = g.n;
  g.lab_buckets = std::max<uint32_t>(1, std::min<uint32_t>(g.num_labels, kMaxLabels));
  const uint32_t B = g.lab_buckets;
  if (!n || !g.m2) return SMG_OK;
  auto bucket = [&](uint32_t w) { return std::min(labels[w], B - 1); };
  // lists ordered by (bucket, id): a stable counting pass per vertex over the
  // id-ordered list keeps ids ascending within a bucket
  std::vector<uint32_t> adjl(g.m2);
#pragma omp parallel
  {
    std::vector<uint32_t> cnt(B + 1);
#pragma omp for schedule(dynamic, 1024)
    for (int64_t v = 0; v < static_cast<int64_t>(n); ++v) {
      const uint64_t a = offsets[v], b = offsets[v + 1];
      if (b - a < 2) {
        if (b > a) adjl[a] = adj[a];
        continue;
      }
      std::fill(cnt.begin(), cnt.end(), 0u);
      for (uint64_t e = a; e < b; ++e) ++cnt[bucket(adj[e]) + 1];
      for (uint32_t i = 0; i < B; ++i) cnt[i + 1] += cnt[i];
      for (uint64_t e = a; e < b; ++e) adjl[a + cnt[bucket(adj[e])]++] = adj[e];
    }
  }
  // run tables for the highest-degree vertices
  std::vector<uint32_t> cand;
  for (uint32_t v = 0; v < n; ++v)
    if (offsets[v + 1] - offsets[v] >= std::max<uint32_t>(min_degree, 1)) cand.push_back(v);
  std::stable_sort(cand.begin(), cand.end(),
                   [&](uint32_t x, uint32_t y) { return offsets[x + 1] - offsets[x] > offsets[y + 1] - offsets[y]; });
  const size_t row = static_cast<size_t>(B + 1) * 4;
  if (cand.size() > max_bytes / row) cand.resize(max_bytes / row);
  g.lab_indexed = static_cast<uint32_t>(cand.size());
  std::vector<uint32_t> lab_of(n, kNone), lab_off(std::max<size_t>(cand.size(), 1) * (B + 1));
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < static_cast<int64_t>(cand.size()); ++i) {
    const uint32_t v = cand[i];
    lab_of[v] = static_cast<uint32_t>(i);
    uint32_t *t = lab_off.data() + static_cast<size_t>(i) * (B + 1);
    std::fill(t, t + B + 1, 0u);
    const uint64_t a = offsets[v], b = offsets[v + 1];
    for (uint64_t e = a; e < b; ++e) ++t[bucket(adj[e]) + 1];
    for (uint32_t j = 0; j < B; ++j) t[j + 1] += t[j];  // t[j] = start of bucket j, t[B] = degree
  }
  // rank of each vertex within its bucket, and where each bucket's words
  // start in a hub bitmap row: only the label layout of the hub bitmaps
  // (SMG_HUB_LAYOUT=label) reads them
  std::vector<uint32_t> rank, bwo;
  const char *layout = std::getenv("SMG_HUB_LAYOUT");
  if (layout && std::string(layout) == "label") {
    rank.resize(n);
    bwo.assign(B + 1, 0);
    std::vector<uint32_t> cnt(B, 0);
    for (uint32_t v = 0; v < n; ++v) rank[v] = cnt[std::min(labels[v], B - 1)]++;
    for (uint32_t b = 0; b < B; ++b) bwo[b + 1] = bwo[b] + (cnt[b] + 31) / 32;
    g.hub_row_words = bwo[B];
    SMG_CUDA(cudaMalloc(&g.lab_rank, static_cast<size_t>(n) * 4));
    SMG_CUDA(cudaMalloc(&g.bucket_word_off, (B + 1) * 4));
    SMG_CUDA(cudaMemcpyAsync(g.lab_rank, rank.data(), static_cast<size_t>(n) * 4, cudaMemcpyHostToDevice, s));
    SMG_CUDA(cudaMemcpyAsync(g.bucket_word_off, bwo.data(), (B + 1) * 4, cudaMemcpyHostToDevice, s));
    g.bytes += static_cast<size_t>(n) * 4 + (B + 1) * 4;
  }
  // each entry's rank within its label's vertex group (ids ascending, as
  // lverts orders them), when every bucket is one label; SMG_RANK_ROWS=0
  // leaves it out (every candidate test reads the id-indexed rows)
  std::vector<uint32_t> adjr;
  const char *rr = std::getenv("SMG_RANK_ROWS");
  if (g.num_labels <= B && !(rr && std::string(rr) == "0")) {
    std::vector<uint32_t> lrank(n), cnt(B, 0);
    for (uint32_t v = 0; v < n; ++v) lrank[v] = cnt[labels[v]]++;
    adjr.resize(g.m2);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < static_cast<int64_t>(g.m2); ++e) adjr[e] = lrank[adjl[e]];
  }
  SMG_CUDA(cudaMalloc(&g.adjl, g.m2 * 4));
  SMG_CUDA(cudaMalloc(&g.lab_of, static_cast<size_t>(n) * 4));
  SMG_CUDA(cudaMalloc(&g.lab_off, lab_off.size() * 4));
  SMG_CUDA(cudaMemcpyAsync(g.adjl, adjl.data(), g.m2 * 4, cudaMemcpyHostToDevice, s));
  SMG_CUDA(cudaMemcpyAsync(g.lab_of, lab_of.data(), static_cast<size_t>(n) * 4, cudaMemcpyHostToDevice, s));
  SMG_CUDA(cudaMemcpyAsync(g.lab_off, lab_off.data(), lab_off.size() * 4, cudaMemcpyHostToDevice, s));
  if (!adjr.empty()) {
    SMG_CUDA(cudaMalloc(&g.adjr, g.m2 * 4));
    SMG_CUDA(cudaMemcpyAsync(g.adjr, adjr.data(), g.m2 * 4, cudaMemcpyHostToDevice, s));
    g.bytes += g.m2 * 4;
  }
  SMG_CUDA(cudaStreamSynchronize(s));  // the host vectors go out of scope
  g.bytes += g.m2 * 4 + static_cast<size_t>(n) * 4 + lab_off.size() * 4;
  return SMG_OK;
}

smg_status build_hub_bitmaps(DevGraph &g, uint32_t min_degree, size_t max_bytes, cudaStream_t s,
                             const std::vector<uint32_t> &deg) {
  // rows by id; SMG_HUB_LAYOUT=label lays them out by label then rank (needs
  // the label index).  On the 2^22 R-MAT workload the label layout measured
  // slower (join 371 ms against 335 ms per 1,024 queries): the extra
  // dependent rank load costs more than the smaller per-label footprint saves.
  const char *layout = std::getenv("SMG_HUB_LAYOUT");
  g.hub_by_label = g.lab_rank && layout && std::string(layout) == "label";
  g.hub_words = g.hub_by_label ? g.hub_row_words : (static_cast<uint64_t>(g.n) + 31) / 32;
  std::vector<uint32_t> cand;
  for (uint32_t v = 0; v < g.n; ++v)
    if (deg[v] >= min_degree) cand.push_back(v);
  std::stable_sort(cand.begin(), cand.end(), [&](uint32_t a, uint32_t b) { return deg[a] > deg[b]; });
  const uint64_t per = g.hub_words * 4;
  const uint64_t fit = per ? max_bytes / per : 0;
  if (cand.size() > fit) cand.resize(fit);
  g.num_hubs = static_cast<uint32_t>(cand.size());
  std::vector<uint32_t> hub_of(std::max<uint32_t>(g.n, 1), kNone);
  for (uint32_t i = 0; i < g.num_hubs; ++i) hub_of[cand[i]] = i;
  SMG_CUDA(cudaMalloc(&g.hub_of, hub_of.size() * 4));
  SMG_CUDA(cudaMemcpyAsync(g.hub_of, hub_of.data(), hub_of.size() * 4, cudaMemcpyHostToDevice, s));
  g.bytes += hub_of.size() * 4;
  if (g.num_hubs) {
    uint32_t *d_hubs = nullptr;
    SMG_CUDA(cudaMalloc(&g.hub_bits, per * g.num_hubs));
    SMG_CUDA(cudaMalloc(&d_hubs, g.num_hubs * 4));
    SMG_CUDA(cudaMemsetAsync(g.hub_bits, 0, per * g.num_hubs, s));
    SMG_CUDA(cudaMemcpyAsync(d_hubs, cand.data(), g.num_hubs * 4, cudaMemcpyHostToDevice, s));
    k_hub_bits<<<g.num_hubs, 256, 0, s>>>(g.off, g.adj, d_hubs, g.hub_words, g.hub_bits, g.label,
                                          g.hub_by_label ? g.lab_rank : nullptr, g.bucket_word_off, g.lab_buckets);
    SMG_CUDA(cudaGetLastError());
    SMG_CUDA(cudaStreamSynchronize(s));
    cudaFree(d_hubs);
    g.bytes += per * g.num_hubs;
  }
  return SMG_OK;
}

}  // namespace smg
