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
//  * vertices are matched in the order the reference's edge order first
//    reaches them; each level checks, for a new vertex, its tree edge and
//    every non-tree edge back to a matched vertex at once;
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
//  * every wait is bounded: a claimed-but-unpublished task, an idle grid and
//    the whole run have time limits after which the kernel records an error
//    and returns.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <numeric>
#include <string>

#include "join.cuh"

namespace smg {
namespace {

constexpr int kWarpsPerBlock = 8;
constexpr uint64_t kReadyWaitNs = 2000000000ull;   // 2 s for a producer to publish
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
      if (vload(qs->pending) == 0) return 0;
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
      if (t - *reinterpret_cast<volatile unsigned long long *>(&qs->start_ns) > p.time_limit_ns) {
        set_error(qs, JOIN_ERR_DEADLINE);
        return -1;
      }
    }
    __nanosleep(ns);
    ns = min(ns * 2, 2048u);
  }
}

__global__ void k_seed(JoinLaunch p) {
  if (blockIdx.x == 0 && threadIdx.x == 0) p.qs->start_ns = now_ns();
  const uint32_t nseed = p.seed_list ? p.seed_n : p.nq;
  for (uint32_t si = blockIdx.x * blockDim.x + threadIdx.x; si < nseed; si += gridDim.x * blockDim.x) {
    const uint32_t q = p.seed_list ? p.seed_list[si] : si;
    const uint32_t nr = *p.queries[q].num_roots;
    if (nr == 0) continue;
    const uint32_t rc = p.queries[q].root_chunk ? p.queries[q].root_chunk : p.root_chunk;
    uint32_t chunk = rc ? rc : 1;
    chunk = max(chunk, (nr + p.max_seed_tasks - 1) / p.max_seed_tasks);
    const uint32_t nt = (nr + chunk - 1) / chunk;
    atomicAdd(&p.qs->pending.v, static_cast<unsigned long long>(nt));
    atomicAdd(p.queries[q].pending, static_cast<unsigned long long>(nt));
    const unsigned long long first = atomicAdd(&p.qs->tail.v, static_cast<unsigned long long>(nt));
    const uint32_t tw = 4 + p.kmax;
    if (!SMG_DCHECK(first + nt <= p.cap, 101, first + nt, p.cap)) continue;
    for (uint32_t i = 0; i < nt; ++i) {
      uint32_t *t = p.tasks + (first + i) * tw;
      t[0] = q;
      t[1] = 0;
      t[2] = i * chunk;
      t[3] = min(nr, (i + 1) * chunk);
    }
    __threadfence();
    for (uint32_t i = 0; i < nt; ++i) p.ready[first + i] = 1;
  }
}

// Block per hub: set one bit per neighbour.
__global__ void k_hub_bits(const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                           const uint32_t *__restrict__ hubs, uint64_t words, uint32_t *__restrict__ bits) {
  const uint32_t v = hubs[blockIdx.x];
  uint32_t *row = bits + blockIdx.x * words;
  for (uint32_t e = off[v] + threadIdx.x; e < off[v + 1]; e += blockDim.x) {
    const uint32_t w = adj[e];
    atomicOr(row + (w >> 5), 1u << (w & 31));
  }
}

// Is w in the neighbour list (beg, deg) of a matched vertex?  `hub` selects
// its bitmap when it has one.
__device__ __forceinline__ bool is_neighbor(const JoinLaunch &p, uint32_t beg, uint32_t deg, uint32_t hub,
                                            uint32_t w, uint32_t &probes) {
  if (hub != kNone && SMG_DCHECK(hub < p.num_hubs, 102, hub, p.num_hubs) && SMG_DCHECK(w < p.n, 103, w, p.n)) {
    ++probes;
    return (__ldg(p.hub_bits + hub * p.hub_words + (w >> 5)) >> (w & 31)) & 1u;
  }
  if (!SMG_DCHECK(static_cast<uint64_t>(beg) + deg <= p.m2, 104, beg, deg)) return false;
  const uint32_t *a = p.adj + beg;
  uint32_t lo = 0, hi = deg;
  while (lo < hi) {
    ++probes;
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(a + mid) < w)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo < deg && __ldg(a + lo) == w;
}

// Per-warp shared state, K = largest query of the launch:
//   m, beg, deg, hub  matched data vertex per level, its list and bitmap
//   cur, end      cursor and end of the level's source list
//   bcnt, bidx    batch of up to 32 tested candidates of the level
//   piv           level whose matched vertex's list feeds this level
//   ord, bmask, slab  the task's query: vertex, backward-edge mask and
//                 same-label mask per level
//   lbase         base pointer of the level's source list
//   batch         [K][32] tested candidates
//   seg*          per-candidate segments of the segmented last level
__host__ __device__ inline uint32_t scalar_words(uint32_t K) { return (12 * K + 1) & ~1u; }
__host__ __device__ inline uint32_t warp_words(uint32_t K) { return scalar_words(K) + 2 * K + 32 * K + 7 * 32; }

struct WarpView {
  uint32_t *m, *beg, *deg, *hub, *cur, *end, *bcnt, *bidx, *piv, *ord, *bmask, *slab, *batch;
  uint32_t *sv, *sbeg, *sdeg, *shub, *sbase, *spre, *spiv;
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
  }
};

__device__ __forceinline__ uint32_t choose_pivot(const WarpView &S, uint32_t level) {
  uint32_t best = 0, bd = 0xFFFFFFFFu;
  for (uint32_t b = S.bmask[level]; b; b &= b - 1) {
    const uint32_t j = __ffs(b) - 1;
    if (S.deg[j] < bd) {
      bd = S.deg[j];
      best = j;
    }
  }
  return best;
}

// Candidate test for list entry w at `level` (>= 1, not the last level).
__device__ __forceinline__ bool accept(const WarpView &S, const JoinLaunch &p, const uint32_t *__restrict__ candmask,
                                       uint32_t level, uint32_t w, uint32_t &probes) {
  if (!SMG_DCHECK(w < p.n, 105, w, level)) return false;
  if (!((__ldg(candmask + w) >> S.ord[level]) & 1u)) return false;
  for (uint32_t b = S.slab[level]; b; b &= b - 1)
    if (S.m[__ffs(b) - 1] == w) return false;
  for (uint32_t b = S.bmask[level] & ~(1u << S.piv[level]); b; b &= b - 1) {
    const uint32_t j = __ffs(b) - 1;
    if (!is_neighbor(p, S.beg[j], S.deg[j], S.hub[j], w, probes)) return false;
  }
  return true;
}

// A last-level list longer than kSplitLen is cut into slices of that length:
// the first stays with this lane, the others become tasks (level P + 1, range
// [lo, hi) of the list, prefix m[0..P-1] plus candidate v) when warps are
// waiting for work or the list is very long.  Returns the length this lane
// keeps (all of it when the queue has no room).
__device__ uint32_t split_last(const WarpView &S, const JoinLaunch &p, const JoinQuery &Q, uint32_t q, uint32_t P,
                               uint32_t v, uint32_t len) {
  QueueState *qs = p.qs;
  const unsigned long long h = vload(qs->head), t = vload(qs->tail);
  if (!(h > t || len > 8 * kSplitLen)) return len;
  const uint32_t slices = (len - 1) / kSplitLen;  // beyond the first
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
    T[2] = (i + 1) * kSplitLen;
    T[3] = min(len, (i + 2) * kSplitLen);
    for (uint32_t j = 0; j < P; ++j) T[4 + j] = S.m[j];
    T[4 + P] = v;
  }
  __threadfence();
  for (uint32_t i = 0; i < slices; ++i) atomicExch(p.ready + first + i, 1u);
  atomicAdd(&qs->donations, static_cast<unsigned long long>(slices));
  return kSplitLen;
}

// Counts (and optionally emits) the last level over entries [lo, hi) of one
// list: the prefix m[0..P] is matched, the list is that of the last vertex's
// back neighbour with the shortest list (the pivot last_level chose).
__device__ unsigned long long last_level_range(WarpView &S, const JoinLaunch &p, const JoinQuery &Q,
                                               const uint32_t *__restrict__ candmask, uint32_t P, uint32_t lo,
                                               uint32_t hi, uint32_t lane, unsigned long long &scanned,
                                               uint32_t &probes) {
  const uint32_t L = P + 1;
  uint32_t piv = 0, bd = 0xFFFFFFFFu;
  for (uint32_t b = S.bmask[L]; b; b &= b - 1) {
    const uint32_t j = __ffs(b) - 1;
    if (S.deg[j] < bd) {
      bd = S.deg[j];
      piv = j;
    }
  }
  hi = min(hi, bd);
  if (lo >= hi) return 0;
  scanned += hi - lo;
  const uint32_t *base = p.adj + S.beg[piv];
  const uint32_t u = S.ord[L], back = S.bmask[L] & ~(1u << piv), same = S.slab[L];
  const uint32_t lt = (1u << lane) - 1;
  unsigned long long cnt = 0;
  for (uint32_t t0 = lo; t0 < hi; t0 += 32) {
    const uint32_t t = t0 + lane;
    bool good = false;
    uint32_t w = 0;
    if (t < hi) {
      w = __ldg(base + t);
      good = SMG_DCHECK(w < p.n, 115, w, t) && ((__ldg(candmask + w) >> u) & 1u);
      for (uint32_t b = same; b && good; b &= b - 1) good = S.m[__ffs(b) - 1] != w;
      for (uint32_t b = back; b && good; b &= b - 1) {
        const uint32_t j = __ffs(b) - 1;
        good = is_neighbor(p, S.beg[j], S.deg[j], S.hub[j], w, probes);
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

// Counts (and optionally emits) the last level for every candidate of the
// batch of level P = k-2: the candidates' last-level lists are concatenated
// and walked 32 entries at a time, each lane finding its candidate by binary
// search over the segment starts.  Returns the count (same in every lane).
__device__ unsigned long long last_level(WarpView &S, const JoinLaunch &p, const JoinQuery &Q, uint32_t q,
                                         const uint32_t *__restrict__ candmask, uint32_t P, uint32_t bc,
                                         uint32_t lane, unsigned long long &scanned, uint32_t &probes) {
  const uint32_t L = P + 1;
  const uint32_t lt = (1u << lane) - 1;
  uint32_t len = 0;
  if (lane < bc) {
    uint32_t v = S.batch[P * 32 + lane];
    if (!SMG_DCHECK(v < p.n, 106, v, P)) v = 0;
    const uint32_t vb = __ldg(p.off + v), vd = __ldg(p.off + v + 1) - vb;
    uint32_t piv = 0, bd = 0xFFFFFFFFu;
    for (uint32_t b = S.bmask[L]; b; b &= b - 1) {
      const uint32_t j = __ffs(b) - 1;
      const uint32_t d = j == P ? vd : S.deg[j];
      if (d < bd) {
        bd = d;
        piv = j;
      }
    }
    len = bd;
    if (len > kSplitLen) len = split_last(S, p, Q, q, P, v, len);
    S.sv[lane] = v;
    S.sbeg[lane] = vb;
    S.sdeg[lane] = vd;
    S.shub[lane] = __ldg(p.hub_of + v);
    S.sbase[lane] = piv == P ? vb : S.beg[piv];
    S.spiv[lane] = piv;
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
  unsigned long long cnt = 0;
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
      const uint64_t ai = static_cast<uint64_t>(S.sbase[i]) + (t - S.spre[i]);
      const bool in_adj = SMG_DCHECK(ai < p.m2, 107, ai, i);
      w = in_adj ? __ldg(p.adj + ai) : 0u;
      good = in_adj && SMG_DCHECK(w < p.n, 108, w, ai) && ((__ldg(candmask + w) >> u) & 1u);
      for (uint32_t b = same; b && good; b &= b - 1) {
        const uint32_t j = __ffs(b) - 1;
        good = (j == P ? vi : S.m[j]) != w;
      }
      // back edges other than the pivot's (whose list w comes from)
      for (uint32_t b = back & ~(1u << S.spiv[i]); b && good; b &= b - 1) {
        const uint32_t j = __ffs(b) - 1;
        if (j == P)
          good = is_neighbor(p, S.sbeg[i], S.sdeg[i], S.shub[i], w, probes);
        else
          good = is_neighbor(p, S.beg[j], S.deg[j], S.hub[j], w, probes);
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
      if (h > t && t < p.cap) {
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

// End of a time slice: every part of this warp's stack that is not done
// becomes a carry-over task: the unscanned rest of each level's list, and each
// untried batch candidate (as a task one level deeper).  Returns false (and
// the warp keeps working) if the carry buffer cannot take them all.
__device__ bool preempt(WarpView &S, const JoinLaunch &p, uint32_t q, unsigned long long *qpending, uint32_t L0,
                        uint32_t level, uint32_t P, uint32_t lane) {
  int ok = 0;
  if (lane == 0) {
    uint32_t n = 0;
    for (uint32_t l = L0; l <= level; ++l) {
      if (S.cur[l] < S.end[l]) ++n;
      if (l < P) n += S.bcnt[l] - S.bidx[l];
    }
    if (n == 0) {
      ok = 1;
    } else {
      unsigned int old = *reinterpret_cast<volatile unsigned int *>(p.carry_count);
      unsigned int base = kNone;
      while (old + n <= p.carry_cap) {
        const unsigned int seen = atomicCAS(p.carry_count, old, old + n);
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
            uint32_t *T = p.carry + static_cast<uint64_t>(idx++) * tw;
            T[0] = q;
            T[1] = l;
            T[2] = S.cur[l];
            T[3] = S.end[l];
            for (uint32_t j = 0; j < l; ++j) T[4 + j] = S.m[j];
          }
          if (l < P)
            for (uint32_t b = S.bidx[l]; b < S.bcnt[l]; ++b) {
              uint32_t *T = p.carry + static_cast<uint64_t>(idx++) * tw;
              T[0] = q;
              T[1] = l + 1;
              T[2] = 0;
              T[3] = kNone;
              for (uint32_t j = 0; j < l; ++j) T[4 + j] = S.m[j];
              T[4 + l] = S.batch[l * 32 + b];
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

__device__ __forceinline__ void join_body(const JoinLaunch &p) {
  extern __shared__ __align__(16) uint32_t smem[];
  const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const uint32_t K = p.kmax, tw = 4 + K;
  WarpView S(smem + wib * warp_words(K), K);
  const uint32_t lt = (1u << lane) - 1;
  QueueState *qs = p.qs;
  volatile int *vabort = &qs->abort;
  uint64_t idle_mark = 0, idle_t0 = 0;
  unsigned long long scanned = 0, descents = 0;
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
    int drop = 0;
    if (lane == 0) drop = Q.count_limit && *reinterpret_cast<volatile uint32_t *>(Q.over);
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
    unsigned long long cnt = 0;
    bool aborted = false, preempted = false;
    if (L0 == P + 1) {
      // a slice of one last-level list, split off by last_level
      cnt = last_level_range(S, p, Q, Q.candmask, P, lo, hi, lane, scanned, probes);
    } else {
    if (lane == 0) {
      if (L0 == 0) {
        S.lbase[0] = Q.roots;
      } else {
        const uint32_t pv = choose_pivot(S, L0);
        S.piv[L0] = pv;
        S.lbase[L0] = p.adj + S.beg[pv];
      }
      S.cur[L0] = lo;
      S.end[L0] = (hi == kNone && L0 > 0) ? S.deg[S.piv[L0]] : hi;
      S.bcnt[L0] = 0;
      S.bidx[L0] = 0;
    }
    __syncwarp();

    uint32_t level = L0, iter = 0, tick = 0;  // tick paces donation checks
    const uint32_t *const candmask = Q.candmask;
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
          if (Q.count_limit && *reinterpret_cast<volatile uint32_t *>(Q.over)) {
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
          } else if (now_ns() - *reinterpret_cast<volatile unsigned long long *>(&qs->start_ns) > p.slice_ns) {
            atomicExch(&qs->closing, 1);
            close = 1;
          }
        }
        close = __shfl_sync(0xFFFFFFFFu, close, 0);
        if (close && !(level == P && S.bcnt[P] != 0) && preempt(S, p, q, Q.pending, L0, level, P, lane)) {
          preempted = true;
          break;
        }
      }
      // give the shallowest unexplored work of this stack to a waiting warp
      if ((++tick & 3) == 0) {
        if (try_donate(S, p, q, Q.pending, L0, level, P, lane, donate_min)) continue;
      }
      if (level == P) {
        const uint32_t bc = S.bcnt[level];
        if (bc) {
          cnt += last_level(S, p, Q, q, candmask, P, bc, lane, scanned, probes);
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
            const uint32_t pv = choose_pivot(S, nl);
            S.piv[nl] = pv;
            S.lbase[nl] = p.adj + S.beg[pv];
            S.cur[nl] = 0;
            S.end[nl] = S.deg[pv];
            S.bcnt[nl] = 0;
            S.bidx[nl] = 0;
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
        // refill the batch with the next 32 tested entries
        const uint32_t n = min(32u, e - c);
        scanned += n;
        const uint32_t *base = S.lbase[level];
        bool good = false;
        uint32_t w = 0;
        if (lane < n && SMG_DCHECK(level == 0 ? c + lane < *Q.num_roots
                                                : static_cast<uint64_t>(base - p.adj) + c + lane < p.m2,
                                   114, c + lane, level)) {
          w = __ldg(base + c + lane);
          good = SMG_DCHECK(w < p.n, 112, w, level) && (level == 0 || accept(S, p, candmask, level, w, probes));
        }
        const uint32_t bal = __ballot_sync(0xFFFFFFFFu, good);
        if (good) S.batch[level * 32 + __popc(bal & lt)] = w;
        __syncwarp();
        if (lane == 0) {
          S.bcnt[level] = __popc(bal);
          S.bidx[level] = 0;
          S.cur[level] = c + n;
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
      atomicAdd(&qs->scanned, scanned);
      atomicAdd(&qs->descents, descents);
      if (pr) atomicAdd(&qs->probes, pr);
      if (!aborted) {
        atomicAdd(&qs->tasks_done, 1ull);
        atomicAdd(&qs->progress.v, 1ull);
        atomicAdd(Q.pending, ~0ull);       // -1
        atomicAdd(&qs->pending.v, ~0ull);  // -1
      }
    }
    scanned = 0;
    descents = 0;
    if (aborted || preempted) break;
  }
}

// The join at the compiler's register choice (fewer, fatter warps) and
// bounded to 6 resident blocks per SM (more warps to hide latency, a small
// spill).  SMG_JOIN_OCCUPANCY=high selects the second.
__global__ void __launch_bounds__(kWarpsPerBlock * 32) k_join(JoinLaunch p) { join_body(p); }
__global__ void __launch_bounds__(kWarpsPerBlock * 32, 6) k_join_hi(JoinLaunch p) { join_body(p); }

__global__ void k_slice_begin(QueueState *qs) {
  qs->start_ns = now_ns();
  qs->closing = 0;
}

// Single block: keep the published-but-untaken tasks of the old queue
// (ready == 1) in order, then append the carry-over tasks.
__global__ void __launch_bounds__(1024) k_compact(const uint32_t *__restrict__ tasks_old,
                                                  const uint32_t *__restrict__ ready_old, uint32_t n_old,
                                                  const uint32_t *__restrict__ carry,
                                                  const unsigned int *__restrict__ carry_count, uint32_t carry_cap,
                                                  uint32_t tw, uint32_t *__restrict__ tasks_new,
                                                  uint32_t *__restrict__ ready_new, QueueState *qs) {
  __shared__ uint32_t warp_sum[32];
  __shared__ uint32_t running;
  const uint32_t tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  if (tid == 0) running = 0;
  __syncthreads();
  for (uint32_t base = 0; base < n_old; base += blockDim.x) {
    const uint32_t i = base + tid;
    const bool keep = i < n_old && ready_old[i] == 1;
    const uint32_t bal = __ballot_sync(0xFFFFFFFFu, keep);
    if (lane == 0) warp_sum[wid] = __popc(bal);
    __syncthreads();
    uint32_t before = running;
    for (uint32_t w = 0; w < wid; ++w) before += warp_sum[w];
    if (keep) {
      const uint32_t dst = before + __popc(bal & ((1u << lane) - 1));
      for (uint32_t j = 0; j < tw; ++j) tasks_new[static_cast<uint64_t>(dst) * tw + j] = tasks_old[static_cast<uint64_t>(i) * tw + j];
      ready_new[dst] = 1;
    }
    __syncthreads();
    if (tid == 0) {
      uint32_t tot = 0;
      for (uint32_t w = 0; w < blockDim.x / 32; ++w) tot += warp_sum[w];
      running += tot;
    }
    __syncthreads();
  }
  const uint32_t kept = running;
  const uint32_t nc = min(*carry_count, carry_cap);
  for (uint32_t i = tid; i < nc; i += blockDim.x) {
    for (uint32_t j = 0; j < tw; ++j) tasks_new[static_cast<uint64_t>(kept + i) * tw + j] = carry[static_cast<uint64_t>(i) * tw + j];
    ready_new[kept + i] = 1;
  }
  if (tid == 0) {
    qs->head.v = 0;
    qs->tail.v = kept + nc;
    qs->pending.v = kept + nc;
    qs->closing = 0;
  }
}

}  // namespace

smg_status launch_slice_begin(QueueState *qs, cudaStream_t s) {
  k_slice_begin<<<1, 1, 0, s>>>(qs);
  SMG_CUDA(cudaGetLastError());
  return SMG_OK;
}

smg_status launch_compact(const uint32_t *tasks_old, const uint32_t *ready_old, uint32_t n_old,
                          const uint32_t *carry, const unsigned int *carry_count, uint32_t carry_cap, uint32_t tw,
                          uint32_t *tasks_new, uint32_t *ready_new, QueueState *qs, cudaStream_t s) {
  k_compact<<<1, 1024, 0, s>>>(tasks_old, ready_old, n_old, carry, carry_count, carry_cap, tw, tasks_new, ready_new,
                               qs);
  SMG_CUDA(cudaGetLastError());
  return SMG_OK;
}

#ifdef SMG_CHECKED
extern "C" int smg_debug_check_join(unsigned long long *out) {
  return static_cast<int>(cudaMemcpyFromSymbol(out, g_check_record, 3 * sizeof(unsigned long long)));
}
#endif

size_t join_queue_bytes(uint32_t cap, uint32_t kmax) {
  return static_cast<size_t>(cap) * (4 + kmax) * sizeof(uint32_t) + static_cast<size_t>(cap) * sizeof(uint32_t);
}

namespace {

bool high_occupancy() {
  static const bool hi = [] {
    const char *e = std::getenv("SMG_JOIN_OCCUPANCY");
    return e && std::string(e) == "high";
  }();
  return hi;
}

smg_status launch_persistent(const JoinLaunch &jl, cudaStream_t s, int num_sms) {
  const size_t smem = static_cast<size_t>(kWarpsPerBlock) * warp_words(jl.kmax) * sizeof(uint32_t);
  void (*kern)(JoinLaunch) = high_occupancy() ? k_join_hi : k_join;
  if (smem > 48 * 1024)
    SMG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  int per_sm = 0;
  SMG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWarpsPerBlock * 32, smem));
  per_sm = std::max(1, per_sm);
  kern<<<num_sms * per_sm, kWarpsPerBlock * 32, smem, s>>>(jl);
  SMG_CUDA(cudaGetLastError());
  return SMG_OK;
}

}  // namespace

smg_status launch_join(const JoinLaunch &jl, cudaStream_t s, int num_sms) {
  if (jl.nq == 0) return SMG_OK;
  const uint32_t seed_threads = 128;
  const uint32_t nseed = jl.seed_list ? jl.seed_n : jl.nq;
  k_seed<<<(nseed + seed_threads - 1) / seed_threads, seed_threads, 0, s>>>(jl);
  SMG_CUDA(cudaGetLastError());
  return launch_persistent(jl, s, num_sms);
}

smg_status launch_join_only(const JoinLaunch &jl, cudaStream_t s, int num_sms) {
  return launch_persistent(jl, s, num_sms);
}

smg_status launch_seed(const JoinLaunch &jl, cudaStream_t s) {
  const uint32_t n = jl.seed_list ? jl.seed_n : jl.nq;
  if (!n) return SMG_OK;
  k_seed<<<(n + 127) / 128, 128, 0, s>>>(jl);
  SMG_CUDA(cudaGetLastError());
  return SMG_OK;
}

smg_status build_hub_bitmaps(DevGraph &g, uint32_t min_degree, size_t max_bytes, cudaStream_t s,
                             const std::vector<uint32_t> &deg) {
  g.hub_words = (static_cast<uint64_t>(g.n) + 31) / 32;
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
    k_hub_bits<<<g.num_hubs, 256, 0, s>>>(g.off, g.adj, d_hubs, g.hub_words, g.hub_bits);
    SMG_CUDA(cudaGetLastError());
    SMG_CUDA(cudaStreamSynchronize(s));
    cudaFree(d_hubs);
    g.bytes += per * g.num_hubs;
  }
  return SMG_OK;
}

}  // namespace smg
