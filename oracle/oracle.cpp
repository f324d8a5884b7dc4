// oracle.cpp — CPU restatement of the reference's filter and join semantics.
// TEST INFRASTRUCTURE ONLY: the checker for tests/, smoke() and the CPU
// baseline of bench.py.  The product library never links or calls this file.
#include "oracle.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct QueryInfo {
  uint32_t k = 0;
  std::vector<uint32_t> label, deg;
  uint32_t adj[32] = {0};          // adjacency bitmask per query vertex
  std::vector<uint32_t> order;      // matching order of the oracle
  std::vector<uint32_t> level_of;
  std::vector<uint32_t> back;       // per level: mask of earlier levels adjacent
};

// The oracle's own order: start at the vertex of largest degree, then keep
// adding the unmapped vertex with the most mapped neighbours (ties: larger
// degree, then smaller id).  Independent of the library's plan.
bool make_query(const smg_query_desc *q, QueryInfo &Q) {
  if (!q || q->num_vertices < 1 || q->num_vertices > 32) return false;
  Q.k = q->num_vertices;
  Q.label.assign(q->labels, q->labels + Q.k);
  Q.deg.assign(Q.k, 0);
  for (uint32_t i = 0; i < q->num_edges; ++i) {
    uint32_t a = q->edges[2 * i], b = q->edges[2 * i + 1];
    if (a >= Q.k || b >= Q.k || a == b) return false;
    Q.adj[a] |= 1u << b;
    Q.adj[b] |= 1u << a;
  }
  for (uint32_t u = 0; u < Q.k; ++u) Q.deg[u] = __builtin_popcount(Q.adj[u]);
  uint32_t start = 0;
  for (uint32_t u = 1; u < Q.k; ++u)
    if (Q.deg[u] > Q.deg[start]) start = u;
  Q.order = {start};
  uint32_t mapped = 1u << start;
  while (Q.order.size() < Q.k) {
    int best = -1, best_c = -1;
    for (uint32_t u = 0; u < Q.k; ++u) {
      if (mapped >> u & 1) continue;
      int c = __builtin_popcount(Q.adj[u] & mapped);
      if (c == 0) continue;
      if (c > best_c || (c == best_c && Q.deg[u] > Q.deg[best])) {
        best = static_cast<int>(u);
        best_c = c;
      }
    }
    if (best < 0) return false;  // disconnected
    Q.order.push_back(static_cast<uint32_t>(best));
    mapped |= 1u << best;
  }
  Q.level_of.assign(Q.k, 0);
  for (uint32_t i = 0; i < Q.k; ++i) Q.level_of[Q.order[i]] = i;
  Q.back.assign(Q.k, 0);
  for (uint32_t i = 0; i < Q.k; ++i)
    for (uint32_t j = 0; j < i; ++j)
      if (Q.adj[Q.order[i]] >> Q.order[j] & 1) Q.back[i] |= 1u << j;
  return true;
}

inline bool has_edge(const smg_csr *g, uint32_t a, uint32_t b) {
  const uint32_t *lo = g->neighbors + g->offsets[a], *hi = g->neighbors + g->offsets[a + 1];
  return std::binary_search(lo, hi, b);
}

struct Matcher {
  const smg_csr *g;
  const QueryInfo &Q;
  const uint32_t *candmask;
  uint32_t m[32];  // image per level
  uint64_t count = 0;
  std::vector<uint32_t> *rows = nullptr;
  uint64_t max_rows = 0;
  // optional work budget shared by all threads (partial matches created)
  uint64_t *budget_used = nullptr;
  uint64_t budget = 0, local = 0;
  bool aborted = false;
  // level 1 scans only entries [l1_lo, l1_hi) of the root's list (its only
  // back neighbour is the root), so that one root's work can be split
  uint64_t l1_lo = 0, l1_hi = ~0ull;

  bool ok_vertex(uint32_t lvl, uint32_t v) const {
    uint32_t u = Q.order[lvl];
    if (g->labels[v] != Q.label[u]) return false;
    if (g->offsets[v + 1] - g->offsets[v] < Q.deg[u]) return false;
    if (candmask && !(candmask[v] >> u & 1)) return false;
    return true;
  }

  void extend(uint32_t lvl) {
    // pivot: mapped neighbour whose image has the fewest neighbours
    uint32_t bm = Q.back[lvl], pivot = 0;
    uint64_t best = ~0ull;
    for (uint32_t b = bm; b; b &= b - 1) {
      uint32_t j = __builtin_ctz(b);
      uint64_t d = g->offsets[m[j] + 1] - g->offsets[m[j]];
      if (d < best) {
        best = d;
        pivot = j;
      }
    }
    const uint32_t pv = m[pivot];
    uint64_t e0 = g->offsets[pv], e1 = g->offsets[pv + 1];
    if (lvl == 1) {
      e1 = std::min(e1, e0 + std::min(l1_hi, e1 - e0));
      e0 += std::min(l1_lo, e1 - e0);
    }
    for (uint64_t e = e0; e < e1; ++e) {
      uint32_t w = g->neighbors[e];
      if (!ok_vertex(lvl, w)) continue;
      bool good = true;
      for (uint32_t j = 0; j < lvl && good; ++j) good = m[j] != w;
      for (uint32_t b = bm & ~(1u << pivot); b && good; b &= b - 1)
        good = has_edge(g, m[__builtin_ctz(b)], w);
      if (!good) continue;
      m[lvl] = w;
      if (budget_used && ++local == 4096) {
        if (__atomic_add_fetch(budget_used, local, __ATOMIC_RELAXED) > budget) aborted = true;
        local = 0;
      }
      if (aborted) return;
      if (lvl + 1 == Q.k) {
        ++count;
        if (rows && rows->size() / Q.k < max_rows) {
          for (uint32_t u = 0; u < Q.k; ++u) rows->push_back(m[Q.level_of[u]]);
        }
      } else {
        extend(lvl + 1);
      }
    }
  }
};

void root_candidates(const smg_csr *g, const QueryInfo &Q, const uint32_t *candmask,
                     std::vector<uint32_t> &roots) {
  Matcher mt{g, Q, candmask};
  for (uint32_t v = 0; v < g->num_vertices; ++v)
    if (mt.ok_vertex(0, v)) roots.push_back(v);
}

uint64_t count_range(const smg_csr *g, const QueryInfo &Q, const uint32_t *candmask,
                     const std::vector<uint32_t> &roots, uint64_t lo, uint64_t hi, int threads) {
  uint64_t total = 0;
  if (Q.k == 1) return hi - lo;
  int nt = threads;
#ifdef _OPENMP
  if (nt <= 0) nt = omp_get_max_threads();
#else
  nt = 1;
#endif
  // units of work: a root, or a slice of a long root list at level 1 (the
  // counts of disjoint slices add up), so that hub roots spread over threads
  constexpr uint64_t kSlice = 256;
  struct Unit {
    uint32_t root;
    uint64_t lo, hi;
  };
  std::vector<Unit> units;
  for (uint64_t r = lo; r < hi; ++r) {
    const uint32_t v = roots[r];
    const uint64_t d = g->offsets[v + 1] - g->offsets[v];
    if (d <= 2 * kSlice) {
      units.push_back({v, 0, ~0ull});
    } else {
      for (uint64_t a = 0; a < d; a += kSlice) units.push_back({v, a, std::min(d, a + kSlice)});
    }
  }
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total) num_threads(nt)
  for (int64_t i = 0; i < static_cast<int64_t>(units.size()); ++i) {
    Matcher mt{g, Q, candmask};
    mt.m[0] = units[i].root;
    mt.l1_lo = units[i].lo;
    mt.l1_hi = units[i].hi;
    mt.extend(1);
    total += mt.count;
  }
  return total;
}

}  // namespace

extern "C" {

int oracle_count(const smg_csr *g, const smg_query_desc *q, const uint32_t *candmask, int threads,
                 uint64_t *count) {
  QueryInfo Q;
  if (!g || !count || !make_query(q, Q)) return 1;
  std::vector<uint32_t> roots;
  root_candidates(g, Q, candmask, roots);
  *count = count_range(g, Q, candmask, roots, 0, roots.size(), threads);
  return 0;
}

int oracle_count_budget(const smg_csr *g, const smg_query_desc *q, const uint32_t *candmask, int threads,
                        uint64_t budget, uint64_t *count, uint64_t *used) {
  QueryInfo Q;
  if (!g || !count || !used || !make_query(q, Q) || Q.k < 2) return 1;
  std::vector<uint32_t> roots;
  root_candidates(g, Q, candmask, roots);
  uint64_t total = 0, spent = 0;
  bool aborted = false;
  int nt = threads;
#ifdef _OPENMP
  if (nt <= 0) nt = omp_get_max_threads();
#else
  nt = 1;
#endif
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total) reduction(|| : aborted) num_threads(nt)
  for (int64_t r = 0; r < static_cast<int64_t>(roots.size()); ++r) {
    if (__atomic_load_n(&spent, __ATOMIC_RELAXED) > budget) {
      aborted = true;
      continue;
    }
    Matcher mt{g, Q, candmask};
    mt.budget_used = &spent;
    mt.budget = budget;
    mt.m[0] = roots[r];
    mt.extend(1);
    __atomic_add_fetch(&spent, mt.local, __ATOMIC_RELAXED);
    total += mt.count;
    aborted = aborted || mt.aborted;
  }
  *count = total;
  *used = aborted ? ~0ull : spent;
  return 0;
}

int oracle_count_roots(const smg_csr *g, const smg_query_desc *q, int threads, uint64_t root_lo,
                       uint64_t root_hi, uint64_t *count, uint64_t *num_roots) {
  QueryInfo Q;
  if (!g || !count || !make_query(q, Q)) return 1;
  std::vector<uint32_t> roots;
  root_candidates(g, Q, nullptr, roots);
  if (num_roots) *num_roots = roots.size();
  root_hi = std::min<uint64_t>(root_hi, roots.size());
  root_lo = std::min(root_lo, root_hi);
  *count = count_range(g, Q, nullptr, roots, root_lo, root_hi, threads);
  return 0;
}

int oracle_embeddings(const smg_csr *g, const smg_query_desc *q, uint64_t max_rows, uint32_t *emb,
                      uint64_t *rows, uint64_t *count) {
  QueryInfo Q;
  if (!g || !count || !make_query(q, Q)) return 1;
  std::vector<uint32_t> roots;
  root_candidates(g, Q, nullptr, roots);
  std::vector<uint32_t> all;
  Matcher mt{g, Q, nullptr};
  mt.rows = &all;
  mt.max_rows = max_rows;
  for (uint32_t r : roots) {
    mt.m[0] = r;
    if (Q.k == 1) {
      ++mt.count;
      if (all.size() < max_rows) all.push_back(r);
    } else {
      mt.extend(1);
    }
  }
  *count = mt.count;
  const uint32_t k = Q.k;
  const uint64_t n = all.size() / k;
  std::vector<uint64_t> idx(n);
  for (uint64_t i = 0; i < n; ++i) idx[i] = i;
  std::sort(idx.begin(), idx.end(), [&](uint64_t a, uint64_t b) {
    return std::lexicographical_compare(all.begin() + a * k, all.begin() + a * k + k,
                                        all.begin() + b * k, all.begin() + b * k + k);
  });
  uint64_t w = std::min<uint64_t>(n, max_rows);
  if (emb)
    for (uint64_t i = 0; i < w; ++i) std::memcpy(emb + i * k, all.data() + idx[i] * k, k * sizeof(uint32_t));
  if (rows) *rows = emb ? w : 0;
  return 0;
}

// Rows of the reference's breadth-first join tables, level by level
// (join.cu:290-435): rows[0] = |C(first vertex of the edge order)|
// (firstJoinKernel join.cu:71-97), then after each edge (a -> b) of the
// order: b unmapped, every row r and neighbour w of r[a] with bit b of
// candmask[w] set and w not yet in r gives a row (joinOneEdgeKernel
// join.cu:100-177); b mapped, r is kept when r[b] is a neighbour of r[a]
// (selectPartialMatchingsKernel join.cu:16-68).  Depth-first over the same
// rows.  Gives up once a level holds more than `limit` rows: that level and
// the later ones then read UINT64_MAX.
int oracle_ref_rows(const smg_csr *g, uint32_t k, uint32_t num_edges, const uint32_t *first,
                    const uint32_t *second, const uint32_t *candmask, int threads, uint64_t limit,
                    uint64_t *rows) {
  if (!g || !first || !second || !candmask || !rows || k < 2 || k > 32 || num_edges < 1) return 1;
  const uint32_t E = num_edges, root = first[0];
  // an edge extends the rows when its second vertex is new at that point
  std::vector<char> extends(E, 0);
  {
    uint32_t mapped = 1u << root;
    for (uint32_t e = 0; e < E; ++e) {
      if (first[e] >= k || second[e] >= k || !(mapped >> first[e] & 1)) return 1;
      extends[e] = !(mapped >> second[e] & 1);
      mapped |= 1u << second[e];
    }
  }
  std::vector<uint32_t> roots;
  for (uint32_t v = 0; v < g->num_vertices; ++v)
    if (candmask[v] >> root & 1) roots.push_back(v);
  std::vector<uint64_t> total(E + 1, 0);
  total[0] = roots.size();
  bool over = total[0] > limit;
  int nt = threads;
#ifdef _OPENMP
  if (nt <= 0) nt = omp_get_max_threads();
#else
  nt = 1;
#endif
#pragma omp parallel num_threads(nt)
  {
    std::vector<uint64_t> local(E + 1, 0);
    uint64_t pending = 0;
    uint32_t m[32];
    auto flush = [&]() {
      for (uint32_t j = 1; j <= E; ++j) {
        if (!local[j]) continue;
        if (__atomic_add_fetch(&total[j], local[j], __ATOMIC_RELAXED) > limit)
          __atomic_store_n(&over, true, __ATOMIC_RELAXED);
        local[j] = 0;
      }
      pending = 0;
    };
    // per level j < E: next neighbour position and end of the anchor's list
    // (extending edge), or whether the single adjacency test is still to do
    std::vector<uint64_t> pos(E), end(E);
#pragma omp for schedule(dynamic, 1)
    for (int64_t r = 0; r < static_cast<int64_t>(roots.size()); ++r) {
      if (__atomic_load_n(&over, __ATOMIC_RELAXED)) continue;
      for (uint32_t u = 0; u < k; ++u) m[u] = UINT32_MAX;
      m[root] = roots[r];
      int64_t j = 0;  // rows at depth j have edges [0, j) applied
      bool enter = true;
      while (j >= 0) {
        if (j == static_cast<int64_t>(E)) {  // a full row: back up
          --j;
          enter = false;
          continue;
        }
        const uint32_t a = first[j], b = second[j];
        if (enter) {
          if (extends[j]) {
            pos[j] = g->offsets[m[a]];
            end[j] = g->offsets[m[a] + 1];
          } else {
            pos[j] = 0;
            end[j] = 1;
          }
        }
        bool down = false;
        if (extends[j]) {
          while (pos[j] < end[j]) {
            const uint32_t w = g->neighbors[pos[j]++];
            if (!(candmask[w] >> b & 1)) continue;
            bool used = false;
            for (uint32_t u = 0; u < k && !used; ++u) used = u != b && m[u] == w;
            if (used) continue;
            m[b] = w;
            down = true;
            break;
          }
          if (!down) m[b] = UINT32_MAX;
        } else if (pos[j] < end[j]) {
          pos[j] = end[j];
          down = has_edge(g, m[a], m[b]);
        }
        if (++pending >= 4096) {
          flush();
          if (__atomic_load_n(&over, __ATOMIC_RELAXED)) break;
        }
        if (down) {
          ++local[j + 1];
          ++j;
          enter = true;
        } else {
          --j;
          enter = false;
        }
      }
      flush();
    }
  }
  for (uint32_t j = 0; j <= E; ++j) rows[j] = total[j];
  if (over) {
    uint32_t j = 0;
    while (j <= E && total[j] <= limit) ++j;
    for (; j <= E; ++j) rows[j] = UINT64_MAX;
  }
  return 0;
}

// filter.cu:404-539 restated: one pass over the data vertices.
int oracle_nlc_filter(const smg_csr *g, const smg_plan_view *p, uint32_t *vmask0) {
  if (!g || !p || !vmask0) return 1;
  const uint32_t nvlq = p->nvlq, k = p->k;
#pragma omp parallel
  {
    std::vector<uint32_t> nlc(nvlq);
#pragma omp for schedule(dynamic, 4096)
    for (int64_t vi = 0; vi < static_cast<int64_t>(g->num_vertices); ++vi) {
      const uint32_t v = static_cast<uint32_t>(vi);
      uint32_t mask = 0;
      const uint32_t lv = g->labels[v];
      if (lv < nvlq) {  // filter.cu:463-467
        std::fill(nlc.begin(), nlc.end(), 0);
        for (uint64_t e = g->offsets[v]; e < g->offsets[v + 1]; ++e) {
          uint32_t l = g->labels[g->neighbors[e]];
          if (l < nvlq) ++nlc[l];
        }
        const uint64_t dv = g->offsets[v + 1] - g->offsets[v];
        for (uint32_t u = 0; u < k; ++u) {
          if (p->degrees[u] > dv || p->labels[u] != lv) continue;  // filter.cu:489-490
          bool ok = true;
          for (uint32_t l = 0; l < nvlq && ok; ++l) ok = nlc[l] >= p->nlc[u * nvlq + l];
          if (ok) mask |= 1u << u;
        }
      }
      vmask0[v] = mask;
    }
  }
  return 0;
}

int oracle_encode(const smg_csr *g, const smg_plan_view *p, const uint32_t *vmask0, uint32_t *enc,
                  uint32_t *candmask) {
  if (!g || !p || !vmask0 || !enc) return 1;
  const uint32_t n = g->num_vertices, B = p->num_words, k = p->k;
  std::memset(enc, 0, sizeof(uint32_t) * static_cast<size_t>(n) * B);
  auto bit = [&](uint32_t v, uint32_t s) -> bool { return enc[static_cast<size_t>(v) * B + s / 32] >> (s % 32) & 1; };
  auto set = [&](uint32_t v, uint32_t s) { enc[static_cast<size_t>(v) * B + s / 32] |= 1u << (s % 32); };
  auto clr = [&](uint32_t v, uint32_t s) { enc[static_cast<size_t>(v) * B + s / 32] &= ~(1u << (s % 32)); };
  // candidate lists of the initial filter; merges punch holes (filter.cu:718)
  std::vector<std::vector<char>> alive(k, std::vector<char>(n, 0));
  for (uint32_t v = 0; v < n; ++v)
    for (uint32_t u = 0; u < k; ++u)
      if (vmask0[v] >> u & 1) alive[u][v] = 1;
  // neighbour slots of cluster c set on w when w passed the initial filter
  // for that slot's vertex (filter.cu:633-647, 724-740)
  auto spread = [&](uint32_t c, uint32_t v) {
    const uint32_t s0 = p->cluster_offsets[c], s1 = p->cluster_offsets[c + 1];
    for (uint64_t e = g->offsets[v]; e < g->offsets[v + 1]; ++e) {
      uint32_t w = g->neighbors[e];
      for (uint32_t s = s0 + 1; s < s1; ++s)
        if (vmask0[w] >> p->slots[s] & 1) set(w, s);
    }
  };
  const uint32_t C = p->num_clusters;
  // merge record per cluster
  std::vector<int64_t> merge_of(C, -1);
  for (uint32_t r = 0; r < p->num_merges; ++r) merge_of[p->merge_cluster[r]] = r;
  for (uint32_t layer = 0; layer < p->num_layers; ++layer) {
    for (uint32_t c = 0; c < C; ++c) {
      if (p->cluster_layer[c] != layer) continue;
      const uint32_t s0 = p->cluster_offsets[c], core = p->slots[s0];
      if (p->cluster_kind[c] == 0) {  // encodeKernel filter.cu:585-653
        for (uint32_t v = 0; v < n; ++v) {
          if (!alive[core][v]) continue;
          set(v, s0);
          spread(c, v);
        }
      } else if (p->cluster_kind[c] == 1) {  // mergeKernel filter.cu:656-746
        const int64_t r = merge_of[c];
        if (r < 0) return 2;
        uint32_t lp = 0, rp = 0;
        for (uint32_t s = p->cluster_offsets[p->merge_left[r]];; ++s)
          if (p->slots[s] == core) { lp = s; break; }
        for (uint32_t s = p->cluster_offsets[p->merge_right[r]];; ++s)
          if (p->slots[s] == core) { rp = s; break; }
        for (uint32_t v = 0; v < n; ++v) {
          if (!alive[core][v]) continue;
          if (bit(v, lp) && bit(v, rp)) {
            set(v, s0);
            spread(c, v);
          } else {
            alive[core][v] = 0;
          }
        }
      }
    }
    // combines of this layer (filter.cu:749-873 with the intended semantics:
    // a slot of the combined cluster holds the AND of the same vertex's slots
    // in the other clusters of the group)
    for (uint32_t r = 0; r < p->num_combines; ++r) {
      if (p->combine_layer[r] != layer) continue;
      const uint32_t out = p->combine_out[r], type = p->combine_type[r];
      const uint32_t s0 = p->cluster_offsets[out], s1 = p->cluster_offsets[out + 1], core = p->slots[s0];
      const uint32_t *oth = p->combine_others + p->combine_other_offsets[r];
      const uint32_t no = p->combine_other_offsets[r + 1] - p->combine_other_offsets[r];
      // slot of target vertex in each other cluster (or none)
      std::vector<std::vector<uint32_t>> tslots(s1 - s0);
      for (uint32_t s = s0 + 1; s < s1; ++s)
        for (uint32_t o = 0; o < no; ++o)
          for (uint32_t t = p->cluster_offsets[oth[o]]; t < p->cluster_offsets[oth[o] + 1]; ++t)
            if (p->slots[t] == p->slots[s]) {
              tslots[s - s0].push_back(t);
              break;
            }
      for (uint32_t v = 0; v < n; ++v) {
        if (!alive[core][v]) continue;
        bool all = true;
        for (uint32_t o = 0; o < no; ++o) all = all && bit(v, p->cluster_offsets[oth[o]]);
        if (type == 0) {
          if (all) set(v, s0);
        } else if (!all) {
          clr(v, s0);
        }
        for (uint64_t e = g->offsets[v]; e < g->offsets[v + 1]; ++e) {
          uint32_t w = g->neighbors[e];
          for (uint32_t s = s0 + 1; s < s1; ++s) {
            bool fin = true;
            for (uint32_t t : tslots[s - s0]) fin = fin && bit(w, t);
            if (type == 0) {
              if (fin) set(w, s);
            } else if (!fin) {
              clr(w, s);
            }
          }
        }
      }
    }
  }
  if (candmask)  // collectCandidatesKernel filter.cu:1158-1232
    for (uint32_t v = 0; v < n; ++v) {
      uint32_t m = 0;
      for (uint32_t u = 0; u < k; ++u)
        if (bit(v, p->last_slot[u])) m |= 1u << u;
      candmask[v] = m;
    }
  return 0;
}

}  // extern "C"

// ------------------------------------------------------------------ inputs
// The seeded synthetic graphs of the workloads, restated here so that the
// CPU baseline needs nothing from the library: a counter-seeded xoshiro256**
// stream (splitmix64 seeding), R-MAT quadrants on a 16-bit grid with
// (a, a+b, a+b+c) = (0.57, 0.76, 0.95), Zipf(s=1) labels as integer weights
// floor(2^40 / (l + 1)), and a symmetrised, sorted, duplicate- and loop-free
// CSR.  tests/test_oracle.py checks them bit for bit against the library's
// generator.
namespace {

uint64_t sm64(uint64_t &x) {
  uint64_t z = (x += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

struct Xs {
  uint64_t s[4];
  explicit Xs(uint64_t seed) {
    uint64_t x = seed;
    for (auto &w : s) w = sm64(x);
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  uint64_t below(uint64_t bound) { return static_cast<uint64_t>((static_cast<unsigned __int128>(next()) * bound) >> 64); }
};

uint64_t stream_of(uint64_t seed, uint64_t stream, uint64_t chunk) {
  uint64_t x = seed ^ (stream * 0xD1B54A32D192ED03ull);
  const uint64_t a = sm64(x);
  x = a ^ (chunk * 0x8CB92BA72F3D8DD7ull);
  return sm64(x);
}

void gen_labels(uint32_t n, uint32_t L, bool zipf, uint64_t seed, uint32_t *label) {
  std::vector<uint64_t> cum;
  uint64_t acc = 0;
  for (uint32_t l = 0; l < L; ++l) {
    acc += zipf ? ((1ull << 40) / (l + 1)) : (1ull << 32);
    cum.push_back(acc);
  }
  const int64_t chunk = 1 << 16, nchunks = (static_cast<int64_t>(n) + chunk - 1) / chunk;
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < nchunks; ++c) {
    Xs r(stream_of(seed, 2, static_cast<uint64_t>(c)));
    const int64_t e = std::min<int64_t>(n, (c + 1) * chunk);
    for (int64_t v = c * chunk; v < e; ++v)
      label[v] = static_cast<uint32_t>(std::upper_bound(cum.begin(), cum.end(), r.below(cum.back())) - cum.begin());
  }
}

// CSR of a directed pair list, symmetrised, sorted, without loops or repeats.
void to_csr(uint32_t n, const std::vector<uint32_t> &a, const std::vector<uint32_t> &b, std::vector<uint64_t> &off,
            std::vector<uint32_t> &adj) {
  std::vector<uint64_t> cnt(static_cast<size_t>(n) + 1, 0);
  for (size_t i = 0; i < a.size(); ++i)
    if (a[i] != b[i]) {
      ++cnt[a[i] + 1];
      ++cnt[b[i] + 1];
    }
  for (uint32_t v = 0; v < n; ++v) cnt[v + 1] += cnt[v];
  std::vector<uint32_t> tmp(cnt[n]);
  std::vector<uint64_t> at(cnt.begin(), cnt.end() - 1);
  for (size_t i = 0; i < a.size(); ++i)
    if (a[i] != b[i]) {
      tmp[at[a[i]]++] = b[i];
      tmp[at[b[i]]++] = a[i];
    }
  off.assign(static_cast<size_t>(n) + 1, 0);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t v = 0; v < static_cast<int64_t>(n); ++v) {
    auto lo = tmp.begin() + static_cast<int64_t>(cnt[v]), hi = tmp.begin() + static_cast<int64_t>(cnt[v + 1]);
    std::sort(lo, hi);
    off[v + 1] = static_cast<uint64_t>(std::unique(lo, hi) - lo);
  }
  for (uint32_t v = 0; v < n; ++v) off[v + 1] += off[v];
  adj.resize(off[n]);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t v = 0; v < static_cast<int64_t>(n); ++v)
    std::copy(tmp.begin() + static_cast<int64_t>(cnt[v]),
              tmp.begin() + static_cast<int64_t>(cnt[v] + (off[v + 1] - off[v])), adj.begin() + static_cast<int64_t>(off[v]));
}

int hand_out(const std::vector<uint64_t> &off, const std::vector<uint32_t> &adj, const std::vector<uint32_t> &lab,
             uint64_t **o_off, uint32_t **o_adj, uint32_t **o_lab, uint64_t *o_m2) {
  *o_off = static_cast<uint64_t *>(std::malloc(off.size() * 8));
  *o_adj = static_cast<uint32_t *>(std::malloc(std::max<size_t>(adj.size(), 1) * 4));
  *o_lab = static_cast<uint32_t *>(std::malloc(std::max<size_t>(lab.size(), 1) * 4));
  if (!*o_off || !*o_adj || !*o_lab) return 1;
  std::memcpy(*o_off, off.data(), off.size() * 8);
  if (!adj.empty()) std::memcpy(*o_adj, adj.data(), adj.size() * 4);
  if (!lab.empty()) std::memcpy(*o_lab, lab.data(), lab.size() * 4);
  *o_m2 = adj.size();
  return 0;
}

}  // namespace

extern "C" {

int oracle_gen_rmat(uint32_t scale, uint32_t avg_degree, uint32_t num_labels, uint32_t zipf, uint64_t seed,
                    uint64_t **off, uint32_t **adj, uint32_t **labels, uint64_t *m2) {
  if (!off || !adj || !labels || !m2 || scale < 1 || scale > 31 || !avg_degree || !num_labels) return 1;
  const uint32_t n = 1u << scale;
  const uint64_t draws = static_cast<uint64_t>(n) * avg_degree / 2;
  const uint32_t TA = 37356, TB = 49807, TC = 62259;
  std::vector<uint32_t> a(draws), b(draws);
  const int64_t chunk = 1 << 20, nchunks = static_cast<int64_t>((draws + chunk - 1) / chunk);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t c = 0; c < nchunks; ++c) {
    Xs r(stream_of(seed, 3, static_cast<uint64_t>(c)));
    const int64_t e = std::min<int64_t>(static_cast<int64_t>(draws), (c + 1) * chunk);
    for (int64_t i = c * chunk; i < e; ++i) {
      uint32_t u = 0, v = 0;
      uint64_t bits = 0;
      int left = 0;
      for (uint32_t lvl = 0; lvl < scale; ++lvl) {
        if (left == 0) {
          bits = r.next();
          left = 4;
        }
        const uint32_t x = static_cast<uint32_t>(bits & 0xFFFF);
        bits >>= 16;
        --left;
        u = (u << 1) | (x >= TB ? 1u : 0u);
        v = (v << 1) | (((x >= TA && x < TB) || x >= TC) ? 1u : 0u);
      }
      a[i] = u;
      b[i] = v;
    }
  }
  std::vector<uint64_t> o;
  std::vector<uint32_t> d, lab(n);
  to_csr(n, a, b, o, d);
  gen_labels(n, num_labels, zipf != 0, seed, lab.data());
  return hand_out(o, d, lab, off, adj, labels, m2);
}

int oracle_gen_er(uint32_t n, uint64_t m, uint32_t num_labels, uint32_t zipf, uint64_t seed, uint64_t **off,
                  uint32_t **adj, uint32_t **labels, uint64_t *m2) {
  if (!off || !adj || !labels || !m2 || n < 2 || !num_labels || m > static_cast<uint64_t>(n) * (n - 1) / 2) return 1;
  Xs r(stream_of(seed, 1, 0));
  std::vector<uint32_t> a, b;
  a.reserve(m);
  b.reserve(m);
  // distinct unordered pairs in draw order: an open-addressing set of the
  // keys (min, max) + 1, so that 0 marks an empty cell
  std::vector<uint64_t> table;
  size_t mask = 0, filled = 0;
  auto grow = [&]() {
    std::vector<uint64_t> old;
    old.swap(table);
    table.assign(old.size() * 2, 0);
    mask = table.size() - 1;
    for (uint64_t k : old)
      if (k) {
        size_t h = static_cast<size_t>(k * 0x9E3779B97F4A7C15ull) & mask;
        while (table[h]) h = (h + 1) & mask;
        table[h] = k;
      }
  };
  table.assign(1024, 0);
  mask = 1023;
  while (a.size() < m) {
    const uint32_t x = static_cast<uint32_t>(r.below(n)), y = static_cast<uint32_t>(r.below(n));
    if (x == y) continue;
    // +1 so that the key is never 0 (the empty marker)
    const uint64_t k = ((static_cast<uint64_t>(std::min(x, y)) << 32) | std::max(x, y)) + 1;
    if (2 * (filled + 1) > table.size()) grow();
    size_t h = static_cast<size_t>(k * 0x9E3779B97F4A7C15ull) & mask;
    bool dup = false;
    while (table[h]) {
      if (table[h] == k) {
        dup = true;
        break;
      }
      h = (h + 1) & mask;
    }
    if (dup) continue;
    table[h] = k;
    ++filled;
    a.push_back(x);
    b.push_back(y);
  }
  std::vector<uint64_t> o;
  std::vector<uint32_t> d, lab(n);
  to_csr(n, a, b, o, d);
  gen_labels(n, num_labels, zipf != 0, seed, lab.data());
  return hand_out(o, d, lab, off, adj, labels, m2);
}

void oracle_free(void *p) { std::free(p); }

}  // extern "C"
