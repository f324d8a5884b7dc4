// filter.cu — the bitmap-encoded cluster candidate filter on sm_103a.
//
//   k_build_nlc     per-vertex neighbour-label counts, once per resident graph
//   k_nlc_filter    label / degree / NLC test (filter.cu:404-539 of the reference)
//   k_cluster_walk  star encode, merge and combine steps of one layer
//                   (encodeKernel filter.cu:585-653, mergeKernel 656-746,
//                   combineMultipleClustersKernel 749-873)
//   k_collect       final per-vertex candidate masks and the root list
//                   (collectCandidatesKernel filter.cu:1158-1232)
//
// All of it is integer, HBM-bound work: coalesced sweeps over the vertex
// arrays, warp-per-candidate walks over neighbour lists, and warp-aggregated
// atomics for appends.  Differences from the reference, all on purpose:
//  * neighbour-label counts of data vertices are computed once per graph
//    (saturated at 255 >= any query count) instead of once per query;
//  * every kernel is sized to the device (the reference launches the encode
//    kernels with a single block because the host count it sizes them by is
//    still zero, filter.cu:982-983 vs main.cu:102-103);
//  * the steps of one layer run in one launch per phase, and each combine runs
//    at the end of its own layer with the intended AND semantics (the
//    reference negates the combined bit and strides by the wrong width,
//    filter.cu:858-863, and runs new-cluster combines one layer late);
//  * labels of any value below 256 are supported (the reference overflows its
//    shared NLC table for query labels >= 16, filter.cu:425-426).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>

#include "device.cuh"
#include "filter.cuh"

namespace smg {

namespace {

__device__ __forceinline__ bool enc_bit(const uint32_t *enc, uint32_t W, uint32_t v, uint32_t s) {
  return (enc[static_cast<size_t>(v) * W + (s >> 5)] >> (s & 31)) & 1u;
}

__device__ __forceinline__ void enc_set(uint32_t *enc, uint32_t W, uint32_t v, uint32_t word, uint32_t mask) {
  uint32_t *p = enc + static_cast<size_t>(v) * W + word;
  if ((*p & mask) != mask) atomicOr(p, mask);
}

__device__ __forceinline__ void enc_clear(uint32_t *enc, uint32_t W, uint32_t v, uint32_t s) {
  uint32_t *p = enc + static_cast<size_t>(v) * W + (s >> 5);
  const uint32_t b = 1u << (s & 31);
  if (*p & b) atomicAnd(p, ~b);
}

// ---------------------------------------------------------------- NLC table
// One warp per position p of the label groups (vertex v = lverts[p]): lanes
// stride v's neighbour list and count labels in a per-warp shared histogram,
// then write saturated bytes to row p and v's degree to ldeg[p].  Rows follow
// the label groups so that the initial filter, which sweeps a group, reads
// consecutive rows and degrees instead of one scattered row per vertex.
__global__ void k_build_nlc(uint32_t n, const uint32_t *__restrict__ off, const uint32_t *__restrict__ adj,
                            const uint32_t *__restrict__ label, const uint32_t *__restrict__ lverts, uint32_t ncols,
                            uint32_t stride, uint8_t *__restrict__ nlc, uint32_t *__restrict__ ldeg) {
  extern __shared__ uint32_t hist[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  uint32_t *h = hist + wib * ncols;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t pos = blockIdx.x * (blockDim.x >> 5) + wib; pos < n; pos += warps) {
    const uint32_t v = lverts[pos];
    for (uint32_t c = lane; c < ncols; c += 32) h[c] = 0;
    __syncwarp();
    const uint32_t e0 = off[v], e1 = off[v + 1];
    for (uint32_t e = e0 + lane; e < e1; e += 32) {
      const uint32_t l = label[adj[e]];
      if (l < ncols) atomicAdd_block(&h[l], 1u);
    }
    __syncwarp();
    uint8_t *row = nlc + static_cast<size_t>(pos) * stride;
    for (uint32_t c = lane; c < stride; c += 32) row[c] = c < ncols ? static_cast<uint8_t>(min(h[c], 255u)) : 0;
    if (lane == 0) ldeg[pos] = e1 - e0;
    __syncwarp();
  }
}

// ------------------------------------------------------------ initial filter
// A query's vertices to visit: its label groups laid end to end.  Returns the
// vertex at position t (< total), the query vertices carrying its label, its
// rank within its label's group and its position in lverts.
__device__ __forceinline__ uint32_t group_vertex(const FilterQuery &Q, const uint32_t *__restrict__ lverts, uint32_t t,
                                                 uint32_t &same, uint32_t &rank, uint32_t &pos) {
  uint32_t i = 0;
  while (t >= Q.grp_hi[i] - Q.grp_lo[i]) {
    t -= Q.grp_hi[i] - Q.grp_lo[i];
    ++i;
  }
  same = Q.grp_mask[i];
  rank = t;
  pos = Q.grp_lo[i] + t;
  return lverts[pos];
}

__device__ __forceinline__ uint32_t group_total(const FilterQuery &Q) {
  uint32_t total = 0;
  for (uint32_t i = 0; i < Q.ngrp; ++i) total += Q.grp_hi[i] - Q.grp_lo[i];
  return total;
}

// Thread per data vertex of the query's labels (the masks start at zero, so
// other vertices are never touched).  Candidates are appended to per-u lists
// with one atomic per warp and query vertex.
__global__ void __launch_bounds__(256) k_nlc_filter(const uint32_t *__restrict__ lverts,
                                                    const uint32_t *__restrict__ ldeg,
                                                    const uint8_t *__restrict__ nlc, uint32_t stride,
                                                    const FilterQuery *__restrict__ qs) {
  __shared__ FilterQuery Q;
  const FilterQuery *src = qs + blockIdx.y;
  for (uint32_t i = threadIdx.x; i < sizeof(FilterQuery) / 4; i += blockDim.x)
    reinterpret_cast<uint32_t *>(&Q)[i] = reinterpret_cast<const uint32_t *>(src)[i];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const uint32_t total = group_total(Q);
  const uint32_t step = gridDim.x * blockDim.x;
  for (uint32_t base = blockIdx.x * blockDim.x; base < total; base += step) {
    const uint32_t t = base + threadIdx.x;
    uint32_t mask = 0, pos = 0;
    if (t < total) {
      uint32_t same = 0, rank = 0;
      group_vertex(Q, lverts, t, same, rank, pos);
      const uint32_t dv = ldeg[pos];
      const uint8_t *row = nlc + static_cast<size_t>(pos) * stride;
      for (uint32_t b = same; b; b &= b - 1) {
        const uint32_t u = __ffs(b) - 1;
        if (Q.deg[u] > dv) continue;
        bool ok = true;
        for (uint32_t i = 0; i < Q.nnlc[u] && ok; ++i) ok = row[Q.nlc_label[u][i]] >= Q.nlc_count[u][i];
        if (ok) mask |= 1u << u;
      }
      if (mask) Q.vmask[pos] = mask;
    }
    // warp-aggregated appends of positions, one atomic per query vertex
    // present in the warp
    uint32_t any = __reduce_or_sync(0xFFFFFFFFu, mask);
    for (; any; any &= any - 1) {
      const uint32_t u = __ffs(any) - 1;
      const uint32_t bal = __ballot_sync(0xFFFFFFFFu, (mask >> u) & 1u);
      uint32_t first = 0;
      if (lane == 0) first = atomicAdd(Q.cand_cnt + u, __popc(bal));
      first = __shfl_sync(0xFFFFFFFFu, first, 0);
      if ((mask >> u) & 1u) {
        const uint64_t at = Q.cand_off[u] + first + __popc(bal & ((1u << lane) - 1));
        if (SMG_DCHECK(at < Q.cand_off[u + 1], 201, at, u)) Q.cand[at] = pos;
      }
    }
  }
}

// ----------------------------------------------------- cluster bitmap steps
// Grid: x strides the candidates of the group's core, y indexes the group.
// One warp per candidate v of the core:
//   star    set the core slot on v, then the neighbour slots on N(v)
//   merge   for each merge of the group in cluster order: v keeps going only
//           while both connection slots are set; failing v become holes
//   combine core slot = AND of the other clusters' core slots; neighbour
//           slot = AND of the same vertex's slots in the other clusters
__device__ __forceinline__ void spread_slots(const ClusterStep &st, uint32_t xm, uint32_t *enc, uint32_t W,
                                             uint32_t w) {
  for (uint32_t gi = 0; gi < st.num_groups; ++gi) {
    const WordGroup &gr = st.groups[gi];
    uint32_t y = xm & gr.qmask, mask = 0;
    for (; y; y &= y - 1) mask |= 1u << gr.pos[__ffs(y) - 1];
    if (mask) enc_set(enc, W, w, gr.word, mask);
  }
}

// One neighbour of a candidate, at position w of the label groups, that
// passed steps `pass` of its group: set the neighbour slots of those steps
// (star / merge), or apply the combine rule (AND of the other clusters'
// slots) to it.
__device__ __forceinline__ void walk_entry(uint32_t w, const StepGroup &G, const ClusterStep *__restrict__ steps,
                                           const uint32_t *__restrict__ aux, const FilterQuery &Q, uint32_t kind,
                                           uint32_t pass) {
  const uint32_t W = Q.words;
  uint32_t *const enc = Q.enc;
  if (kind != 2) {
    const uint32_t xm = Q.vmask[w];
    if (!xm) return;
    for (uint32_t p = pass; p; p &= p - 1) spread_slots(steps[G.first + __ffs(p) - 1], xm, enc, W, w);
  } else {
    const ClusterStep &st = steps[G.first];
    uint32_t t = st.targets_off;
    for (uint32_t ti = 0; ti < st.num_targets; ++ti) {
      const uint32_t slot = aux[t], nsrc = aux[t + 1];
      bool fin = true;
      for (uint32_t s = 0; s < nsrc && fin; ++s) fin = enc_bit(enc, W, w, aux[t + 2 + s]);
      t += 2 + nsrc;
      if (st.type == 0) {
        if (fin) enc_set(enc, W, w, slot >> 5, 1u << (slot & 31));
      } else if (!fin) {
        enc_clear(enc, W, w, slot);
      }
    }
  }
}

// Neighbour part of a step group for candidate v over adj[e0, e1), one
// entry per lane (each neighbour's position looked up in pos_of).
__device__ __forceinline__ void walk_neighbors(const uint32_t *__restrict__ adj, const StepGroup &G,
                                               const ClusterStep *__restrict__ steps,
                                               const uint32_t *__restrict__ aux, const FilterQuery &Q,
                                               uint32_t kind, uint32_t pass, uint32_t e0, uint32_t e1,
                                               uint32_t lane, uint32_t n, const uint32_t *__restrict__ pos_of) {
  for (uint32_t e = e0 + lane; e < e1; e += 32) {
    const uint32_t w = adj[e];
    if (!SMG_DCHECK(w < n, 207, w, e)) continue;
    walk_entry(__ldg(pos_of + w), G, steps, aux, Q, kind, pass);
  }
}

// Queues entries [e0 + kWalkChunk, e1) of candidate v for the chunk pass,
// one item per kWalkChunk entries; returns the end the caller keeps (e1 when
// the queue has no room).  Called by single lanes.
__device__ __forceinline__ uint32_t queue_tail_chunks(uint32_t tag, uint32_t v, uint32_t pass, uint32_t e0,
                                                      uint32_t e1, const WalkOverflow &ov) {
  if (e1 - e0 <= kWalkChunk) return e1;
  const uint32_t extra = (e1 - e0 - 1) / kWalkChunk;
  unsigned int old = *(volatile unsigned int *)ov.count;
  while (old + extra <= ov.cap) {
    const unsigned int seen = atomicCAS(ov.count, old, old + extra);
    if (seen == old) {
      for (uint32_t c = 0; c < extra; ++c)
        if (SMG_DCHECK(old + c < ov.cap, 205, old + c, ov.cap))
          ov.items[old + c] = make_uint4(tag, v, pass, e0 + (c + 1) * kWalkChunk);
      return e0 + kWalkChunk;
    }
    old = seen;
  }
  return e1;
}

// Candidates of a group's core that its step group walks, clamped to the
// core's segment of the candidate list.
__device__ __forceinline__ uint32_t group_candidates(const StepGroup &G, const FilterQuery &Q) {
  uint32_t cnt = *(volatile const uint32_t *)(Q.cand_cnt + G.core);
  if (!SMG_DCHECK(Q.cand_off[G.core] + cnt <= Q.cand_off[G.core + 1], 202, cnt, G.core)) cnt = 0;
  return cnt;
}

// The walk's work list of one phase: group g owns 32-candidate chunks
// [chunk_start[g], chunk_start[g + 1]); chunk_start[ng] is the total.  The
// groups of a phase differ in size by orders of magnitude (a frequent label's
// core has millions of candidates, a rare one's a few), so the walk's warps
// take chunks from one counter instead of a fixed share of blocks per group.
__global__ void __launch_bounds__(256) k_walk_plan(const StepGroup *__restrict__ groups, uint32_t ng,
                                                    const FilterQuery *__restrict__ qs,
                                                    uint32_t *__restrict__ chunk_start) {
  __shared__ uint32_t warp_sum[32];
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t per = (ng + blockDim.x - 1) / blockDim.x;
  const uint32_t lo = min(ng, threadIdx.x * per), hi = min(ng, lo + per);
  uint32_t own = 0;
  for (uint32_t g = lo; g < hi; ++g) own += (group_candidates(groups[g], qs[groups[g].query]) + 31) / 32;
  uint32_t incl = own;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= static_cast<uint32_t>(o)) incl += t;
  }
  if (lane == 31) warp_sum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const uint32_t w = lane < (blockDim.x >> 5) ? warp_sum[lane] : 0u;
    uint32_t wi = w;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, wi, o);
      if (lane >= static_cast<uint32_t>(o)) wi += t;
    }
    warp_sum[lane] = wi - w;
    if (lane == 31) chunk_start[ng] = wi;
  }
  __syncthreads();
  uint32_t run = warp_sum[warp] + incl - own;
  for (uint32_t g = lo; g < hi; ++g) {
    chunk_start[g] = run;
    run += (group_candidates(groups[g], qs[groups[g].query]) + 31) / 32;
  }
}

// A warp takes a chunk of 32 candidates of one group's core, one per lane:
// each lane applies the group's steps to its own candidate (core slot, merge
// tests, combine rule), then the warp walks the neighbour runs of all 32 as
// one segmented stream (an entry finds its candidate by a binary search over
// the lanes' run offsets), so short runs still fill the warp.  Runs longer
// than kWalkChunk hand their tail to the chunk pass.  Chunks come from one
// counter over the whole phase (k_walk_plan's work list).
__global__ void __launch_bounds__(256) k_cluster_walk(const uint32_t *__restrict__ off,
                                                      const uint32_t *__restrict__ adj,
                                                      const StepGroup *__restrict__ groups, uint32_t ng,
                                                      const uint32_t *__restrict__ chunk_start,
                                                      unsigned int *next,
                                                      const ClusterStep *__restrict__ steps,
                                                      const uint32_t *__restrict__ aux,
                                                      const FilterQuery *__restrict__ qs, WalkOverflow ov) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t chunks = chunk_start[ng];
  while (true) {
  uint32_t item = 0;
  if (lane == 0) item = atomicAdd(next, 1u);
  item = __shfl_sync(0xFFFFFFFFu, item, 0);
  if (item >= chunks) break;
  // the group owning the chunk: the last g with chunk_start[g] <= item
  uint32_t glo = 0, ghi = ng;
  while (ghi - glo > 1) {
    const uint32_t mid = (glo + ghi) >> 1;
    if (chunk_start[mid] <= item) glo = mid;
    else ghi = mid;
  }
  const uint32_t gi = glo;
  const StepGroup G = groups[gi];
  const FilterQuery &Q = qs[G.query];
  const uint32_t W = Q.words;
  uint32_t *const enc = Q.enc;
  uint32_t *const list = Q.cand + Q.cand_off[G.core];
  const uint32_t cnt = group_candidates(G, Q);
  const uint32_t kind = steps[G.first].kind;
  const bool by_label = G.nlab && ov.adjl;
  const uint32_t nruns = by_label ? G.nlab : 1;
  unsigned long long scanned = 0;
  {
    const uint64_t i0 = static_cast<uint64_t>(item - chunk_start[gi]) * 32;
    const uint64_t i = i0 + lane;
    uint32_t v = 0, pass = 0;
    bool act = false;
    if (i < cnt) {
      // the list holds the candidates' positions; v is the vertex itself
      const uint32_t pv = list[i];
      if (pv != kNone && SMG_DCHECK(pv < ov.n, 203, pv, i)) {
        v = __ldg(ov.lverts + pv);
        if (kind == 0) {
          const ClusterStep &st = steps[G.first];
          enc_set(enc, W, pv, st.core_slot >> 5, 1u << (st.core_slot & 31));
          pass = 1;
          act = true;
        } else if (kind == 1) {
          bool alive = true;
          for (uint32_t j = 0; j < G.count && alive; ++j) {
            const ClusterStep &st = steps[G.first + j];
            if (enc_bit(enc, W, pv, st.left_pos) && enc_bit(enc, W, pv, st.right_pos)) {
              pass |= 1u << j;
              enc_set(enc, W, pv, st.core_slot >> 5, 1u << (st.core_slot & 31));
            } else {
              alive = false;
            }
          }
          if (!alive) list[i] = kNone;  // removed by this merge group
          act = pass != 0;
        } else {
          const ClusterStep &st = steps[G.first];
          bool all = true;
          for (uint32_t o = 0; o < st.num_others && all; ++o) all = enc_bit(enc, W, pv, aux[st.others_off + o]);
          if (st.type == 0) {
            if (all) enc_set(enc, W, pv, st.core_slot >> 5, 1u << (st.core_slot & 31));
          } else if (!all) {
            enc_clear(enc, W, pv, st.core_slot);
          }
          act = true;
        }
      }
    }
    uint32_t e0 = 0, e1 = 0, li = kNone;
    if (act) {
      e0 = off[v];
      e1 = off[v + 1];
      if (!SMG_DCHECK(e0 <= e1 && e1 <= ov.m2, 204, e0, e1)) act = false;
      else if (by_label) li = __ldg(ov.lab_of + v);
    }
    for (uint32_t r = 0; r < nruns; ++r) {
      // an entry of the run of the group's r-th label sits at position
      // lvstart[label] + its rank (adjr) when each bucket is one label
      const uint32_t lab_r = by_label ? static_cast<uint32_t>(G.lab[r]) : kNone;
      const bool ranked = ov.adjr && lab_r < ov.num_groups_l && lab_r < ov.lab_buckets;
      const uint32_t run_base = ranked ? __ldg(ov.lvstart + lab_r) : 0u;
      // this lane's segment: the run of the group's r-th label when its
      // candidate has a run table (only those neighbours can change), else
      // (r = 0 only) its whole list
      uint32_t s0 = 0, s1 = 0;
      bool from_l = false;
      if (act) {
        if (li != kNone) {
          const uint32_t *t = ov.lab_off + static_cast<uint64_t>(li) * (ov.lab_buckets + 1) +
                              min(static_cast<uint32_t>(G.lab[r]), ov.lab_buckets - 1);
          s0 = e0 + __ldg(t);
          s1 = e0 + __ldg(t + 1);
          from_l = true;
        } else if (r == 0) {
          s0 = e0;
          s1 = e1;
        }
      }
      scanned += s1 - s0;
      if (s1 - s0 > kWalkChunk) s1 = queue_tail_chunks(gi | (from_l ? 0x80000000u : 0u), v, pass, s0, s1, ov);
      const uint32_t len = s1 - s0;
      uint32_t incl = len;
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t x = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= static_cast<uint32_t>(o)) incl += x;
      }
      const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31), pre = incl - len;
      const uint32_t fl = from_l ? 1u : 0u;
      for (uint32_t t0 = 0; t0 < total; t0 += 32) {
        const uint32_t t = t0 + lane;
        uint32_t src = 0;  // the last lane whose segment starts at or before t
        for (uint32_t step = 16; step; step >>= 1) {
          const uint32_t c = src + step;
          if (__shfl_sync(0xFFFFFFFFu, pre, c) <= t) src = c;
        }
        const uint32_t sb = __shfl_sync(0xFFFFFFFFu, s0, src), sp = __shfl_sync(0xFFFFFFFFu, pre, src);
        const uint32_t spass = __shfl_sync(0xFFFFFFFFu, pass, src), sfl = __shfl_sync(0xFFFFFFFFu, fl, src);
        if (t < total) {
          const uint32_t e = sb + (t - sp);
          const uint32_t w = (sfl ? ov.adjl : adj)[e];
          if (SMG_DCHECK(w < ov.n, 207, w, sb)) {
            const uint32_t pw = sfl && ranked ? run_base + __ldg(ov.adjr + e) : __ldg(ov.pos_of + w);
            if (SMG_DCHECK(pw < ov.n, 209, pw, w)) walk_entry(pw, G, steps, aux, Q, kind, spass);
          }
        }
      }
    }
  }
  for (int o = 16; o; o >>= 1) scanned += __shfl_down_sync(0xFFFFFFFFu, scanned, o);
  if (lane == 0 && scanned) atomicAdd(Q.stat + 1, scanned);
  }  // chunks
}

// Chunks of long neighbour lists queued by k_cluster_walk: one warp each.
__global__ void __launch_bounds__(256) k_walk_chunks(const uint32_t *__restrict__ off,
                                                     const uint32_t *__restrict__ adj,
                                                     const StepGroup *__restrict__ groups,
                                                     const ClusterStep *__restrict__ steps,
                                                     const uint32_t *__restrict__ aux,
                                                     const FilterQuery *__restrict__ qs, WalkOverflow ov) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t n = min(*ov.count, ov.cap);
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
    const uint4 it = ov.items[i];
    const uint32_t gi = it.x & 0x7FFFFFFFu;
    if (!SMG_DCHECK(gi < ov.num_groups && it.y < ov.n && it.w < ov.m2, 206, i, it.x)) continue;
    const StepGroup G = groups[gi];
    const FilterQuery &Q = qs[G.query];
    const uint32_t kind = steps[G.first].kind;
    // a chunk of a label run may run past the run's end into the vertex's
    // next runs: those neighbours carry none of the group's labels, so their
    // slots do not change
    const uint32_t e1 = min(it.w + kWalkChunk, off[it.y + 1]);
    walk_neighbors((it.x >> 31) ? ov.adjl : adj, G, steps, aux, Q, kind, it.z, it.w, e1, lane, ov.n, ov.pos_of);
  }
}

// --------------------------------------------------------------- collect
// Thread per vertex of the query's labels: bit u of the final mask is the
// bit of u's last slot.  Vertices with no initial candidate bit are skipped
// (the bitmap can only hold bits the initial filter allowed).  Root candidates are appended with
// a warp-aggregated atomic.
__global__ void __launch_bounds__(256) k_collect(const uint32_t *__restrict__ lverts,
                                                 const FilterQuery *__restrict__ qs) {
  __shared__ uint32_t last_slot[kMaxK];
  const FilterQuery &Q = qs[blockIdx.y];
  if (threadIdx.x < kMaxK) last_slot[threadIdx.x] = Q.last_slot[threadIdx.x];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const uint32_t W = Q.words, root = Q.root;
  uint32_t *const vmask = Q.vmask;
  const uint32_t *const enc = Q.enc;
  unsigned long long ncand = 0;
  const uint32_t total = group_total(Q);
  const uint32_t step = gridDim.x * blockDim.x;
  for (uint32_t base = blockIdx.x * blockDim.x; base < total; base += step) {
    const uint32_t t = base + threadIdx.x;
    uint32_t cm = 0, v = 0;
    if (t < total) {
      uint32_t same = 0, rank = 0, pos = 0;
      v = group_vertex(Q, lverts, t, same, rank, pos);
      const uint32_t m0 = vmask[pos];
      for (uint32_t b = m0; b; b &= b - 1) {
        const uint32_t u = __ffs(b) - 1;
        if (enc_bit(enc, W, pos, last_slot[u])) cm |= 1u << u;
      }
      if (m0 != cm) vmask[pos] = cm;
      ncand += __popc(cm);
      // the join's candidate bitmaps (zero on entry): one bit per (u, v)
      if (Q.cbits)
        for (uint32_t b = cm; b; b &= b - 1) {
          const uint32_t u = __ffs(b) - 1;
          atomicOr(Q.cbits + u * Q.cwords + (v >> 5), 1u << (v & 31));
          // u's rank-indexed row: u carries v's label, so rank is v's place in that group
          if (Q.rank_rows) atomicOr(Q.cbits + (Q.k + u) * Q.cwords + (rank >> 5), 1u << (rank & 31));
        }
    }
    const bool is_root = (cm >> root) & 1u;
    const uint32_t bal = __ballot_sync(0xFFFFFFFFu, is_root);
    if (bal) {
      uint32_t pos = 0;
      if (lane == 0) pos = atomicAdd(Q.num_roots, __popc(bal));
      pos = __shfl_sync(0xFFFFFFFFu, pos, 0);
      if (is_root) {
        const uint64_t at = pos + __popc(bal & ((1u << lane) - 1));
        if (SMG_DCHECK(at < Q.root_cap, 208, at, Q.root_cap)) Q.roots[at] = v;
      }
    }
  }
  for (int o = 16; o; o >>= 1) ncand += __shfl_down_sync(0xFFFFFFFFu, ncand, o);
  if (lane == 0 && ncand) atomicAdd(Q.stat, ncand);
}

}  // namespace

// ======================================================================
// host side
// ======================================================================

smg_status launch_build_nlc(DevGraph &g, cudaStream_t s, int num_sms) {
  const uint32_t ncols = std::min<uint32_t>(g.num_labels, kMaxLabels);
  const int threads = 256;
  const size_t smem = static_cast<size_t>(threads / 32) * ncols * sizeof(uint32_t);
  const uint32_t blocks = std::max<uint32_t>(1, std::min<uint64_t>((g.n + 7) / 8, static_cast<uint64_t>(num_sms) * 16));
  if (g.n) k_build_nlc<<<blocks, threads, smem, s>>>(g.n, g.off, g.adj, g.label, g.lverts, ncols, g.nlc_stride, g.nlc,
                                                     g.ldeg);
  SMG_CUDA(cudaGetLastError());
  return SMG_OK;
}

smg_status fill_filter_query(const Plan &P, const DevGraph &g, FilterQuery &fq) {
  std::memset(&fq, 0, sizeof(fq));
  const uint32_t ncols = std::min<uint32_t>(g.num_labels, kMaxLabels);
  fq.k = P.k;
  fq.words = P.num_words;
  fq.nvlq = P.nvlq;
  fq.root = P.root;
  for (uint32_t u = 0; u < P.k; ++u) {
    if (P.label[u] >= kMaxLabels) return fail(SMG_ERR_LIMIT, "query labels must be below 256");
    fq.label[u] = P.label[u];
    fq.deg[u] = P.deg[u];
    fq.last_slot[u] = P.last_slot[u];
    uint32_t c = 0;
    for (uint32_t l = 0; l < P.nvlq; ++l) {
      const uint32_t cnt = P.nlc[u * P.nvlq + l];
      if (!cnt) continue;
      if (l >= ncols) fq.deg[u] = kNone;  // no data vertex carries label l: u has no candidate
      fq.nlc_label[u][c] = static_cast<uint16_t>(l < ncols ? l : 0);
      fq.nlc_count[u][c] = static_cast<uint8_t>(cnt);
      ++c;
    }
    fq.nnlc[u] = c;
  }
  // the vertex groups of the query's labels (a label the graph lacks, or
  // carries on no vertex, has none)
  uint32_t grp_label[kMaxK];
  for (uint32_t u = 0; u < P.k; ++u) {
    const uint32_t l = P.label[u];
    if (l + 1 >= g.lvert_start.size() || g.lvert_start[l] == g.lvert_start[l + 1]) continue;
    uint32_t i = 0;
    while (i < fq.ngrp && grp_label[i] != l) ++i;
    if (i == fq.ngrp) {
      grp_label[i] = l;
      fq.grp_lo[i] = g.lvert_start[l];
      fq.grp_hi[i] = g.lvert_start[l + 1];
      fq.grp_mask[i] = 0;
      ++fq.ngrp;
    }
    fq.grp_mask[i] |= 1u << u;
  }
  return SMG_OK;
}

namespace {

void word_groups(const Plan &P, uint32_t c, ClusterStep &st) {
  st.num_groups = 0;
  for (uint32_t s = P.cl_off[c] + 1; s < P.cl_off[c + 1]; ++s) {
    const uint32_t word = s >> 5;
    WordGroup *gr = nullptr;
    for (uint32_t i = 0; i < st.num_groups; ++i)
      if (st.groups[i].word == word) gr = &st.groups[i];
    if (!gr) {
      gr = &st.groups[st.num_groups++];
      gr->word = word;
      gr->qmask = 0;
    }
    const uint32_t u = P.slots[s];
    gr->qmask |= 1u << u;
    gr->pos[u] = static_cast<uint8_t>(s & 31);
  }
}

}  // namespace

#ifdef SMG_CHECKED
extern "C" int smg_debug_check_filter(unsigned long long *out) {
  return static_cast<int>(cudaMemcpyFromSymbol(out, g_check_record, 3 * sizeof(unsigned long long)));
}
#endif

// Adds the labels of cluster c's neighbour slots to a group's label set
// (nlab = 0 once more than four distinct labels are needed).
static void add_neighbor_labels(const Plan &P, uint32_t c, StepGroup &g, bool &overflow) {
  for (uint32_t s = P.cl_off[c] + 1; s < P.cl_off[c + 1] && !overflow; ++s) {
    const uint32_t l = P.label[P.slots[s]];
    bool have = false;
    for (uint32_t i = 0; i < g.nlab; ++i) have |= g.lab[i] == l;
    if (have) continue;
    if (g.nlab == 4 || l >= kMaxLabels) {
      overflow = true;
    } else {
      g.lab[g.nlab++] = static_cast<uint8_t>(l);
    }
  }
  if (overflow) g.nlab = 0;
}

static StepGroup make_group(uint32_t qi, uint32_t core, uint32_t first, uint32_t count) {
  StepGroup g;
  std::memset(&g, 0, sizeof(g));
  g.query = qi;
  g.core = core;
  g.first = first;
  g.count = count;
  return g;
}

smg_status append_filter_steps(const Plan &P, uint32_t qi, FilterBatch &fb) {
  const uint32_t phases = 2 * P.num_layers - 1;
  if (fb.phases.size() < phases) fb.phases.resize(phases);
  std::vector<int64_t> merge_of(P.clusters.size(), -1);
  for (size_t r = 0; r < P.mg_cluster.size(); ++r) merge_of[P.mg_cluster[r]] = static_cast<int64_t>(r);
  auto base_step = [&](uint32_t c, uint32_t kind) {
    ClusterStep st;
    std::memset(&st, 0, sizeof(st));
    st.kind = kind;
    st.core_slot = P.cl_off[c];
    st.core = P.slots[st.core_slot];
    word_groups(P, c, st);
    return st;
  };
  // phase 0: stars of layer 0, one group each
  for (uint32_t c = P.layer_begin[0]; c < P.layer_begin[1]; ++c) {
    ClusterStep st = base_step(c, 0);
    StepGroup g = make_group(qi, st.core, static_cast<uint32_t>(fb.steps.size()), 1);
    bool over = false;
    add_neighbor_labels(P, c, g, over);
    fb.phases[0].push_back(g);
    fb.steps.push_back(st);
  }
  for (uint32_t layer = 1; layer < P.num_layers; ++layer) {
    // merges of this layer grouped by core, clusters in index order
    std::vector<uint32_t> cores;
    std::map<uint32_t, std::vector<uint32_t>> by_core;
    for (uint32_t c = P.layer_begin[layer]; c < P.layer_begin[layer + 1]; ++c) {
      if (P.cl_kind[c] != 1) continue;
      const uint32_t core = P.slots[P.cl_off[c]];
      if (!by_core.count(core)) cores.push_back(core);
      by_core[core].push_back(c);
    }
    for (uint32_t core : cores) {
      StepGroup gr = make_group(qi, core, static_cast<uint32_t>(fb.steps.size()), 0);
      bool over = false;
      for (uint32_t c : by_core[core]) {
        add_neighbor_labels(P, c, gr, over);
        const int64_t r = merge_of[c];
        if (r < 0) return fail(SMG_ERR_INTERNAL, "merge cluster without a merge record");
        ClusterStep st = base_step(c, 1);
        st.left_pos = P.mg_left_pos[r];
        st.right_pos = P.mg_right_pos[r];
        fb.steps.push_back(st);
        ++gr.count;
      }
      if (gr.count > 32) return fail(SMG_ERR_LIMIT, "more than 32 merges share a core in one layer");
      fb.phases[2 * layer - 1].push_back(gr);
    }
    // combines of this layer
    for (const CombineRec &rec : P.combines) {
      if (rec.layer != layer) continue;
      ClusterStep st = base_step(rec.out, 2);
      st.type = rec.type;
      st.num_others = static_cast<uint32_t>(rec.others.size());
      st.others_off = static_cast<uint32_t>(fb.aux.size());
      for (uint32_t o : rec.others) fb.aux.push_back(P.cl_off[o]);
      st.targets_off = static_cast<uint32_t>(fb.aux.size());
      st.num_targets = 0;
      for (uint32_t s = P.cl_off[rec.out] + 1; s < P.cl_off[rec.out + 1]; ++s) {
        const uint32_t u = P.slots[s];
        fb.aux.push_back(s);
        const size_t nsrc_at = fb.aux.size();
        fb.aux.push_back(0);
        for (uint32_t o : rec.others)
          for (uint32_t t = P.cl_off[o]; t < P.cl_off[o + 1]; ++t)
            if (P.slots[t] == u) {
              fb.aux.push_back(t);
              ++fb.aux[nsrc_at];
              break;
            }
        ++st.num_targets;
      }
      StepGroup g = make_group(qi, st.core, static_cast<uint32_t>(fb.steps.size()), 1);
      bool over = false;
      add_neighbor_labels(P, rec.out, g, over);
      fb.phases[2 * layer].push_back(g);
      fb.steps.push_back(st);
    }
  }
  return SMG_OK;
}

smg_status FilterDev::upload(const FilterBatch &fb, cudaStream_t s) {
  phase_first.clear();
  phase_count.clear();
  std::vector<StepGroup> flat;
  for (const auto &ph : fb.phases) {
    phase_first.push_back(static_cast<uint32_t>(flat.size()));
    phase_count.push_back(static_cast<uint32_t>(ph.size()));
    flat.insert(flat.end(), ph.begin(), ph.end());
  }
  const size_t bytes_steps = fb.steps.size() * sizeof(ClusterStep);
  const size_t bytes_groups = flat.size() * sizeof(StepGroup);
  const size_t bytes_aux = fb.aux.size() * sizeof(uint32_t);
  const size_t bytes_cs = (flat.size() + phase_count.size()) * sizeof(uint32_t);  // walk work lists
  auto al256 = [](size_t x) { return (x + 255) & ~size_t(255); };
  const size_t need = al256(bytes_steps) + al256(bytes_groups) + al256(bytes_aux) + al256(bytes_cs) + 256;
  if (need > cap) {
    if (buf) cudaFree(buf);
    buf = nullptr;
    cap = 0;
    SMG_CUDA(cudaMalloc(&buf, need));
    cap = need;
  }
  host.resize(need);
  size_t o = 0;
  auto put = [&](const void *src, size_t n) {
    size_t at = o;
    if (n) std::memcpy(host.data() + o, src, n);
    o = (o + n + 255) & ~size_t(255);
    return at;
  };
  const size_t os = put(fb.steps.data(), bytes_steps);
  const size_t og = put(flat.data(), bytes_groups);
  const size_t oa = put(fb.aux.data(), bytes_aux);
  const size_t oc = o;  // written on the device by k_walk_plan
  std::memset(host.data() + oc, 0, bytes_cs);
  o = (o + bytes_cs + 255) & ~size_t(255);
  steps = reinterpret_cast<ClusterStep *>(static_cast<char *>(buf) + os);
  groups = reinterpret_cast<StepGroup *>(static_cast<char *>(buf) + og);
  aux = reinterpret_cast<uint32_t *>(static_cast<char *>(buf) + oa);
  chunk_start = reinterpret_cast<uint32_t *>(static_cast<char *>(buf) + oc);
  SMG_CUDA(cudaMemcpyAsync(buf, host.data(), o, cudaMemcpyHostToDevice, s));
  // the staging buffer must outlive the copy
  SMG_CUDA(cudaStreamSynchronize(s));
  return SMG_OK;
}

smg_status FilterDev::reserve(size_t bytes) {
  if (bytes <= cap) return SMG_OK;
  if (buf) cudaFree(buf);
  buf = nullptr;
  cap = 0;
  SMG_CUDA(cudaMalloc(&buf, bytes));
  cap = bytes;
  return SMG_OK;
}

FilterDev::~FilterDev() {
  if (buf) cudaFree(buf);
}

static uint32_t vertex_blocks(const DevGraph &g, uint32_t nq, int num_sms) {
  const uint32_t vblocks = static_cast<uint32_t>((static_cast<uint64_t>(g.n) + 255) / 256);
  return std::max<uint32_t>(1, std::min<uint32_t>(vblocks, (num_sms * 16u + nq - 1) / nq));
}

smg_status launch_nlc_filter(const DevGraph &g, const FilterQuery *d_qs, uint32_t nq, cudaStream_t s, int num_sms) {
  if (!nq || !g.n) return SMG_OK;
  for (uint32_t y0 = 0; y0 < nq; y0 += 65535) {
    const uint32_t ny = std::min<uint32_t>(65535, nq - y0);
    k_nlc_filter<<<dim3(vertex_blocks(g, nq, num_sms), ny), 256, 0, s>>>(g.lverts, g.ldeg, g.nlc, g.nlc_stride,
                                                                         d_qs + y0);
    SMG_CUDA(cudaGetLastError());
  }
  return SMG_OK;
}

smg_status launch_walks(const DevGraph &g, const FilterQuery *d_qs, const FilterDev &fd, WalkOverflow ov,
                        cudaStream_t s, int num_sms) {
  for (size_t p = 0; p < fd.phase_count.size(); ++p) {
    const uint32_t ng = fd.phase_count[p];
    if (!ng) continue;
    WalkOverflow po = ov;
    po.count = ov.count + 2 * p;  // one zeroed counter per phase
    po.n = g.n;
    po.m2 = g.m2;
    po.num_groups = fd.phase_count[p];
    po.adjl = g.adjl;
    po.lab_of = g.lab_of;
    po.lab_off = g.lab_off;
    po.lab_buckets = g.lab_buckets;
    po.lverts = g.lverts;
    po.pos_of = g.pos_of;
    po.lvstart = g.lvstart;
    po.adjr = g.adjl ? g.adjr : nullptr;
    po.num_groups_l = static_cast<uint32_t>(g.lvert_start.size()) - 1;
    uint32_t *cs = fd.chunk_start + fd.phase_first[p] + p;  // ng + 1 entries per phase
    // 256 threads, so that a served request's plan fits beside a running join
    k_walk_plan<<<1, 256, 0, s>>>(fd.groups + fd.phase_first[p], ng, d_qs, cs);
    SMG_CUDA(cudaGetLastError());
    // the phase's second zeroed counter hands out the chunks
    k_cluster_walk<<<num_sms * 8, 256, 0, s>>>(g.off, g.adj, fd.groups + fd.phase_first[p], ng, cs, po.count + 1,
                                               fd.steps, fd.aux, d_qs, po);
    SMG_CUDA(cudaGetLastError());
    k_walk_chunks<<<num_sms * 8, 256, 0, s>>>(g.off, g.adj, fd.groups + fd.phase_first[p], fd.steps, fd.aux,
                                                d_qs, po);
    SMG_CUDA(cudaGetLastError());
  }
  return SMG_OK;
}

// Zeroes `bytes` (a multiple of 16) at p with 256-thread blocks: a server
// zeroes an admitted request's buffers on its admission stream while the
// join runs, and the driver's memset may not fit beside the join's blocks.
__global__ void __launch_bounds__(256) k_zero(uint4 *p, uint64_t n16) {
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n16;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    p[i] = make_uint4(0u, 0u, 0u, 0u);
}

// Zeroes a list of disjoint byte ranges of `base` (offsets and lengths
// multiples of 4): prefix[r] is the first 4-byte word of range r counted over
// all ranges (prefix[nr] the total), off[r] its byte offset.  Each block takes
// chunks of `chunk` consecutive words, finds the range holding the first by
// binary search and walks on from there, so ranges of any size cost only
// their words.
__global__ void __launch_bounds__(256) k_zero_ranges(char *base, const uint64_t *__restrict__ prefix,
                                                     const uint64_t *__restrict__ off, uint32_t nr, uint64_t chunk) {
  const uint64_t total = prefix[nr];
  for (uint64_t c0 = blockIdx.x * chunk; c0 < total; c0 += static_cast<uint64_t>(gridDim.x) * chunk) {
    const uint64_t c1 = min(total, c0 + chunk);
    uint32_t lo = 0, hi = nr;  // the last range starting at or before c0
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (prefix[mid] <= c0)
        lo = mid;
      else
        hi = mid;
    }
    for (uint32_t r = lo; r < nr && prefix[r] < c1; ++r) {
      const uint64_t a = max(c0, prefix[r]), b = min(c1, prefix[r + 1]);
      uint32_t *w = reinterpret_cast<uint32_t *>(base + off[r]);
      for (uint64_t t = a + threadIdx.x; t < b; t += blockDim.x) w[t - prefix[r]] = 0u;
    }
  }
}

smg_status launch_zero_ranges(char *base, const uint64_t *prefix, const uint64_t *off, uint32_t nr, cudaStream_t s,
                              int num_sms) {
  if (!nr) return SMG_OK;
  k_zero_ranges<<<static_cast<uint32_t>(std::max(num_sms, 1)) * 8, 256, 0, s>>>(base, prefix, off, nr, 1u << 16);
  SMG_CUDA(cudaGetLastError());
  return SMG_OK;
}

smg_status launch_zero(void *p, size_t bytes, cudaStream_t s, int num_sms) {
  if (!bytes) return SMG_OK;
  if (bytes % 16 || reinterpret_cast<uintptr_t>(p) % 16) return fail(SMG_ERR_INTERNAL, "launch_zero: unaligned range");
  const uint64_t n16 = bytes / 16;
  const uint32_t blocks = static_cast<uint32_t>(std::min<uint64_t>((n16 + 255) / 256, static_cast<uint64_t>(num_sms) * 4));
  k_zero<<<blocks, 256, 0, s>>>(static_cast<uint4 *>(p), n16);
  SMG_CUDA(cudaGetLastError());
  return SMG_OK;
}

smg_status launch_collect(const DevGraph &g, const FilterQuery *d_qs, uint32_t nq, cudaStream_t s, int num_sms) {
  if (!nq || !g.n) return SMG_OK;
  for (uint32_t y0 = 0; y0 < nq; y0 += 65535) {
    const uint32_t ny = std::min<uint32_t>(65535, nq - y0);
    k_collect<<<dim3(vertex_blocks(g, nq, num_sms), ny), 256, 0, s>>>(g.lverts, d_qs + y0);
    SMG_CUDA(cudaGetLastError());
  }
  return SMG_OK;
}

smg_status launch_filter(const DevGraph &g, const FilterQuery *d_qs, uint32_t nq, const FilterDev &fd,
                         WalkOverflow ov, cudaStream_t s, int num_sms) {
  smg_status st = launch_nlc_filter(g, d_qs, nq, s, num_sms);
  if (st) return st;
  st = launch_walks(g, d_qs, fd, ov, s, num_sms);
  if (st) return st;
  return launch_collect(g, d_qs, nq, s, num_sms);
}

}  // namespace smg
