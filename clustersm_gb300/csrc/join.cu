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
//    step (candidate bit, injectivity, binary search in the other matched
//    neighbours' sorted lists) and compacted with a warp ballot;
//  * the last level is counted with popcounts of ballots, not materialised;
//  * a warp whose remaining list is long donates half of it to the queue
//    while the queue runs low (work splitting for hub-heavy graphs);
//  * every wait is bounded: a claimed-but-unpublished task, an idle grid and
//    the whole run have time limits after which the kernel records an error
//    and returns.
#include <cuda_runtime.h>

#include <algorithm>

#include "join.cuh"

namespace smg {
namespace {

constexpr int kWarpsPerBlock = 8;
constexpr uint64_t kReadyWaitNs = 2000000000ull;   // 2 s for a producer to publish
constexpr uint64_t kIdleLimitNs = 30000000000ull;  // 30 s without any progress

__host__ __device__ inline uint32_t warp_words(uint32_t K) {
  const uint32_t p = (11 * K + 1) & ~1u;
  return p + 2 * K + 32 * K;
}

__device__ __forceinline__ uint64_t now_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool sorted_contains(const uint32_t *a, uint32_t n, uint32_t x, uint32_t &probes) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    ++probes;
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(a + mid) < x)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo < n && __ldg(a + lo) == x;
}

__device__ __forceinline__ void set_error(QueueState *qs, int code) {
  atomicCAS(&qs->error, 0, code);
  atomicExch(&qs->abort, 1);
}

// Claims the next published task index, or -1 if the queue is empty.
__device__ long long pop_task(const JoinLaunch &p) {
  volatile QueueState *s = p.qs;
  for (int tries = 0; tries < 32; ++tries) {
    const unsigned long long h = s->head;
    unsigned long long t = s->tail;
    if (t > p.cap) t = p.cap;
    if (h >= t) return -1;
    if (atomicCAS(&p.qs->head, h, h + 1) == h) return static_cast<long long>(h);
  }
  return -1;
}

// Bounded wait until the producer of `slot` has written it.
__device__ bool wait_ready(const JoinLaunch &p, uint64_t slot) {
  volatile uint32_t *r = p.ready + slot;
  if (*r) {
    __threadfence();
    return true;
  }
  const uint64_t t0 = now_ns();
  uint32_t ns = 32;
  while (!*r) {
    if (now_ns() - t0 > kReadyWaitNs) return false;
    __nanosleep(ns);
    ns = min(ns * 2, 1024u);
  }
  __threadfence();
  return true;
}

__global__ void k_seed(JoinLaunch p) {
  if (blockIdx.x == 0 && threadIdx.x == 0) p.qs->start_ns = now_ns();
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < p.nq; q += gridDim.x * blockDim.x) {
    const uint32_t nr = *p.queries[q].num_roots;
    if (nr == 0) continue;
    uint32_t chunk = p.root_chunk ? p.root_chunk : 1;
    chunk = max(chunk, (nr + p.max_seed_tasks - 1) / p.max_seed_tasks);
    const uint32_t nt = (nr + chunk - 1) / chunk;
    atomicAdd(&p.qs->pending, static_cast<unsigned long long>(nt));
    const unsigned long long first = atomicAdd(&p.qs->tail, static_cast<unsigned long long>(nt));
    const uint32_t tw = 4 + p.kmax;
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

// Per-warp shared state, K = largest query of the launch:
//   m, beg, deg   matched data vertex per level, its list offset and degree
//   cur, end      cursor and end of the level's candidate source list
//   bcnt, bidx    batch of up to 32 tested candidates of the level
//   piv           level whose matched vertex's list feeds this level
//   ord, bmask, slab  the task's query: vertex, backward-edge mask and
//                 same-label mask per level
//   lbase         base pointer of the level's source list
//   batch         [K][32] tested candidates
struct WarpView {
  uint32_t *m, *beg, *deg, *cur, *end, *bcnt, *bidx, *piv, *ord, *bmask, *slab, *batch;
  const uint32_t **lbase;
  __device__ WarpView(uint32_t *W, uint32_t K) {
    m = W;
    beg = W + K;
    deg = W + 2 * K;
    cur = W + 3 * K;
    end = W + 4 * K;
    bcnt = W + 5 * K;
    bidx = W + 6 * K;
    piv = W + 7 * K;
    ord = W + 8 * K;
    bmask = W + 9 * K;
    slab = W + 10 * K;
    const uint32_t p = (11 * K + 1) & ~1u;
    lbase = reinterpret_cast<const uint32_t **>(W + p);
    batch = W + p + 2 * K;
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

// Candidate test for list entry w at `level` (>= 1).
__device__ __forceinline__ bool accept(const WarpView &S, const uint32_t *__restrict__ adj,
                                       const uint32_t *__restrict__ candmask, uint32_t level, uint32_t w,
                                       uint32_t &probes) {
  if (!((__ldg(candmask + w) >> S.ord[level]) & 1u)) return false;
  for (uint32_t b = S.slab[level]; b; b &= b - 1)
    if (S.m[__ffs(b) - 1] == w) return false;
  for (uint32_t b = S.bmask[level] & ~(1u << S.piv[level]); b; b &= b - 1) {
    const uint32_t j = __ffs(b) - 1;
    if (!sorted_contains(adj + S.beg[j], S.deg[j], w, probes)) return false;
  }
  return true;
}

__global__ void __launch_bounds__(kWarpsPerBlock * 32) k_join(JoinLaunch p) {
  extern __shared__ __align__(16) uint32_t smem[];
  const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const uint32_t K = p.kmax, tw = 4 + K;
  WarpView S(smem + wib * warp_words(K), K);
  const uint32_t lt = (1u << lane) - 1;
  volatile QueueState *vqs = p.qs;
  uint64_t idle_mark = 0, idle_t0 = 0;
  uint32_t idle_ns = 64;

  while (true) {
    long long slot = -1;
    if (lane == 0) slot = pop_task(p);
    slot = __shfl_sync(0xFFFFFFFFu, slot, 0);
    if (slot < 0) {
      int stop = 0;
      if (lane == 0) {
        if (vqs->pending == 0 || vqs->abort) {
          stop = 1;
        } else {
          const uint64_t pr = vqs->progress, t = now_ns();
          if (pr != idle_mark || idle_t0 == 0) {
            idle_mark = pr;
            idle_t0 = t;
          } else if (t - idle_t0 > kIdleLimitNs) {
            set_error(p.qs, JOIN_ERR_IDLE_TIMEOUT);
            stop = 1;
          }
          if (t - vqs->start_ns > p.time_limit_ns) {
            set_error(p.qs, JOIN_ERR_DEADLINE);
            stop = 1;
          }
          __nanosleep(idle_ns);
          idle_ns = min(idle_ns * 2, 4096u);
        }
      }
      if (__shfl_sync(0xFFFFFFFFu, stop, 0)) break;
      continue;
    }
    idle_ns = 64;
    int ok = 1;
    if (lane == 0 && !wait_ready(p, static_cast<uint64_t>(slot))) {
      set_error(p.qs, JOIN_ERR_READY_TIMEOUT);
      ok = 0;
    }
    if (!__shfl_sync(0xFFFFFFFFu, ok, 0)) break;

    const uint32_t *T = p.tasks + static_cast<uint64_t>(slot) * tw;
    const uint32_t q = T[0], L0 = T[1], lo = T[2], hi = T[3];
    const JoinQuery &Q = p.queries[q];
    const uint32_t k = Q.k;
    if (lane < k) {
      S.ord[lane] = Q.order[lane];
      S.bmask[lane] = Q.back_mask[lane];
      S.slab[lane] = Q.same_label[lane];
    }
    if (lane < L0) {
      const uint32_t v = T[4 + lane];
      S.m[lane] = v;
      const uint32_t b = __ldg(p.off + v);
      S.beg[lane] = b;
      S.deg[lane] = __ldg(p.off + v + 1) - b;
    }
    __syncwarp();
    if (lane == 0) {
      if (L0 == 0) {
        S.lbase[0] = Q.roots;
      } else {
        const uint32_t pv = choose_pivot(S, L0);
        S.piv[L0] = pv;
        S.lbase[L0] = p.adj + S.beg[pv];
      }
      S.cur[L0] = lo;
      S.end[L0] = hi;
      S.bcnt[L0] = 0;
      S.bidx[L0] = 0;
    }
    __syncwarp();

    unsigned long long cnt = 0, scanned = 0, descents = 0;
    uint32_t probes = 0;
    uint32_t level = L0, iter = 0;
    const uint32_t *const candmask = Q.candmask;
    bool aborted = false;
    while (true) {
      if ((++iter & 1023) == 0) {
        int stop = 0;
        if (lane == 0) {
          atomicAdd(&p.qs->progress, 1ull);
          if (vqs->abort) stop = 1;
          else if (now_ns() - vqs->start_ns > p.time_limit_ns) {
            set_error(p.qs, JOIN_ERR_DEADLINE);
            stop = 1;
          }
        }
        if (__shfl_sync(0xFFFFFFFFu, stop, 0)) {
          aborted = true;
          break;
        }
      }
      if (level == k - 1) {
        // last level: count (and optionally emit) without materialising
        const uint32_t *base = S.lbase[level];
        const uint32_t e = S.end[level];
        if (e > S.cur[level]) scanned += e - S.cur[level];
        for (uint32_t c = S.cur[level]; c < e; c += 32) {
          const uint32_t idx = c + lane;
          bool good = false;
          uint32_t w = 0;
          if (idx < e) {
            w = __ldg(base + idx);
            good = level == 0 || accept(S, p.adj, candmask, level, w, probes);
          }
          const uint32_t bal = __ballot_sync(0xFFFFFFFFu, good);
          cnt += __popc(bal);
          if (p.emit && bal) {
            unsigned long long pos = 0;
            if (lane == 0) pos = atomicAdd(Q.emb_count, static_cast<unsigned long long>(__popc(bal)));
            pos = __shfl_sync(0xFFFFFFFFu, pos, 0);
            const unsigned long long r = pos + __popc(bal & lt);
            if (good && r < Q.emb_cap) {
              uint32_t *row = Q.emb + r * k;
              for (uint32_t j = 0; j < level; ++j) row[S.ord[j]] = S.m[j];
              row[S.ord[level]] = w;
            }
          }
        }
        if (level == L0) break;
        --level;
        continue;
      }
      const uint32_t bi = S.bidx[level], bc = S.bcnt[level];
      if (bi < bc) {
        // descend into the next tested candidate
        const uint32_t v = S.batch[level * 32 + bi];
        __syncwarp();
        if (lane == 0) {
          S.bidx[level] = bi + 1;
          S.m[level] = v;
          const uint32_t b = __ldg(p.off + v);
          S.beg[level] = b;
          S.deg[level] = __ldg(p.off + v + 1) - b;
        }
        __syncwarp();
        ++descents;
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
        level = nl;
        continue;
      }
      const uint32_t c = S.cur[level];
      uint32_t e = S.end[level];
      if (c < e) {
        // donate the back half of a long list while the queue runs low
        if (e - c >= p.donate_min) {
          long long ds = -1;
          uint32_t mid = 0;
          if (lane == 0) {
            const unsigned long long h = vqs->head, t = vqs->tail;
            const unsigned long long queued = t > h ? t - h : 0;
            if (queued < gridDim.x * kWarpsPerBlock && t < p.cap) {
              const unsigned long long s = atomicAdd(&p.qs->tail, 1ull);
              if (s < p.cap) {
                atomicAdd(&p.qs->pending, 1ull);
                ds = static_cast<long long>(s);
                mid = c + ((e - c) >> 1);
              } else {
                p.qs->full = 1;
              }
            }
          }
          ds = __shfl_sync(0xFFFFFFFFu, ds, 0);
          if (ds >= 0) {
            mid = __shfl_sync(0xFFFFFFFFu, mid, 0);
            uint32_t *t = p.tasks + static_cast<uint64_t>(ds) * tw;
            if (lane < level) t[4 + lane] = S.m[lane];
            if (lane == 0) {
              t[0] = q;
              t[1] = level;
              t[2] = mid;
              t[3] = e;
            }
            __threadfence();
            __syncwarp();
            if (lane == 0) {
              atomicExch(p.ready + ds, 1u);
              atomicAdd(&p.qs->donations, 1ull);
              S.end[level] = mid;
            }
            e = mid;
            __syncwarp();
          }
        }
        // refill the batch with the next 32 tested entries
        scanned += min(32u, e - c);
        const uint32_t *base = S.lbase[level];
        const uint32_t idx = c + lane;
        bool good = false;
        uint32_t w = 0;
        if (idx < e) {
          w = __ldg(base + idx);
          good = level == 0 || accept(S, p.adj, candmask, level, w, probes);
        }
        const uint32_t bal = __ballot_sync(0xFFFFFFFFu, good);
        if (good) S.batch[level * 32 + __popc(bal & lt)] = w;
        __syncwarp();
        if (lane == 0) {
          S.bcnt[level] = __popc(bal);
          S.bidx[level] = 0;
          S.cur[level] = c + 32;
        }
        __syncwarp();
        continue;
      }
      if (level == L0) break;
      --level;
    }
    unsigned long long pr = probes;
    for (int o = 16; o; o >>= 1) pr += __shfl_down_sync(0xFFFFFFFFu, pr, o);
    if (lane == 0) {
      if (cnt) atomicAdd(Q.count, cnt);
      atomicAdd(&p.qs->scanned, scanned);
      atomicAdd(&p.qs->descents, descents);
      if (pr) atomicAdd(&p.qs->probes, pr);
      if (!aborted) {
        atomicAdd(&p.qs->tasks_done, 1ull);
        atomicAdd(&p.qs->progress, 1ull);
        atomicAdd(&p.qs->pending, ~0ull);  // -1
      }
    }
    if (aborted) break;
  }
}

}  // namespace

size_t join_queue_bytes(uint32_t cap, uint32_t kmax) {
  return static_cast<size_t>(cap) * (4 + kmax) * sizeof(uint32_t) + static_cast<size_t>(cap) * sizeof(uint32_t);
}

smg_status launch_join(const JoinLaunch &jl, cudaStream_t s, int num_sms) {
  if (jl.nq == 0) return SMG_OK;
  const size_t smem = static_cast<size_t>(kWarpsPerBlock) * warp_words(jl.kmax) * sizeof(uint32_t);
  if (smem > 48 * 1024) SMG_CUDA(cudaFuncSetAttribute(k_join, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                      static_cast<int>(smem)));
  int per_sm = 0;
  SMG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_join, kWarpsPerBlock * 32, smem));
  per_sm = std::max(1, per_sm);
  const uint32_t seed_threads = 128;
  k_seed<<<(jl.nq + seed_threads - 1) / seed_threads, seed_threads, 0, s>>>(jl);
  SMG_CUDA(cudaGetLastError());
  k_join<<<num_sms * per_sm, kWarpsPerBlock * 32, smem, s>>>(jl);
  SMG_CUDA(cudaGetLastError());
  return SMG_OK;
}

}  // namespace smg
