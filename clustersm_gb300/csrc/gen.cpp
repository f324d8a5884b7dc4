// gen.cpp — seeded synthetic data graphs and queries.
//
// The reference's own datasets (github / gowalla / dblp, runClusterSM.sh:9-27)
// are not available, so workloads are generated.  Every generator uses only
// integer arithmetic on a counter-seeded xoshiro256** stream, so a seed gives
// bit-identical graphs on every host and for every thread count.
#include <algorithm>
#include <atomic>
#include <memory>
#include <unordered_set>

#include "host.h"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace smg {
namespace {

inline uint64_t splitmix64(uint64_t &x) {
  uint64_t z = (x += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

struct Rng {
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    uint64_t x = seed;
    for (auto &w : s) w = splitmix64(x);
  }
  static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    uint64_t r = rotl(s[1] * 5, 7) * 9;
    uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  // uniform in [0, bound) by 64x64->128 multiply (Lemire, no rejection:
  // bias below 2^-32 for the bounds used here)
  uint64_t below(uint64_t bound) {
    return static_cast<uint64_t>((static_cast<unsigned __int128>(next()) * bound) >> 64);
  }
};

inline uint64_t stream_seed(uint64_t seed, uint64_t stream, uint64_t chunk) {
  uint64_t x = seed ^ (stream * 0xD1B54A32D192ED03ull);
  uint64_t a = splitmix64(x);
  x = a ^ (chunk * 0x8CB92BA72F3D8DD7ull);
  return splitmix64(x);
}

// Zipf(s=1) over L labels, P(l) proportional to 1/(l+1), as integer weights.
struct LabelSampler {
  std::vector<uint64_t> cum;
  uint32_t L;
  uint32_t dist;
  LabelSampler(uint32_t L_, uint32_t dist_) : L(L_), dist(dist_) {
    uint64_t acc = 0;
    for (uint32_t l = 0; l < L; ++l) {
      acc += (dist == SMG_LABELS_ZIPF1) ? ((1ull << 40) / (l + 1)) : (1ull << 32);
      cum.push_back(acc);
    }
  }
  uint32_t draw(Rng &r) const {
    uint64_t x = r.below(cum.back());
    return static_cast<uint32_t>(std::upper_bound(cum.begin(), cum.end(), x) - cum.begin());
  }
};

void draw_labels_into(uint32_t n, uint32_t L, uint32_t dist, uint64_t seed, uint32_t *label) {
  LabelSampler ls(L, dist);
  const int64_t chunk = 1 << 16;
  const int64_t nchunks = (static_cast<int64_t>(n) + chunk - 1) / chunk;
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < nchunks; ++c) {
    Rng r(stream_seed(seed, 2, static_cast<uint64_t>(c)));
    int64_t e = std::min<int64_t>(n, (c + 1) * chunk);
    for (int64_t v = c * chunk; v < e; ++v) label[v] = ls.draw(r);
  }
}

void draw_labels(HostGraph &g, uint32_t L, uint32_t dist, uint64_t seed) {
  g.label.resize(g.n);
  draw_labels_into(g.n, L, dist, seed, g.label.data());
}

// Symmetrise a directed edge list into a CSR with sorted, duplicate-free
// neighbour lists and no self-loops.
void build_simple_csr(uint32_t n, const std::vector<uint32_t> &src, const std::vector<uint32_t> &dst,
                      HostGraph &g) {
  const int64_t D = static_cast<int64_t>(src.size());
  std::vector<uint64_t> cnt(static_cast<size_t>(n) + 1, 0);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < D; ++i) {
    if (src[i] == dst[i]) continue;
    __atomic_fetch_add(&cnt[src[i] + 1], 1, __ATOMIC_RELAXED);
    __atomic_fetch_add(&cnt[dst[i] + 1], 1, __ATOMIC_RELAXED);
  }
  for (uint32_t v = 0; v < n; ++v) cnt[v + 1] += cnt[v];
  std::vector<uint32_t> tmp(cnt[n]);
  std::vector<uint64_t> cur(cnt.begin(), cnt.end() - 1);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < D; ++i) {
    uint32_t a = src[i], b = dst[i];
    if (a == b) continue;
    tmp[__atomic_fetch_add(&cur[a], 1, __ATOMIC_RELAXED)] = b;
    tmp[__atomic_fetch_add(&cur[b], 1, __ATOMIC_RELAXED)] = a;
  }
  std::vector<uint64_t> uniq(static_cast<size_t>(n) + 1, 0);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t v = 0; v < static_cast<int64_t>(n); ++v) {
    auto b = tmp.begin() + static_cast<int64_t>(cnt[v]);
    auto e = tmp.begin() + static_cast<int64_t>(cnt[v + 1]);
    std::sort(b, e);
    uniq[v + 1] = static_cast<uint64_t>(std::unique(b, e) - b);
  }
  for (uint32_t v = 0; v < n; ++v) uniq[v + 1] += uniq[v];
  g.n = n;
  g.off = uniq;
  g.adj.resize(uniq[n]);
  g.m = uniq[n] / 2;
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t v = 0; v < static_cast<int64_t>(n); ++v)
    std::copy(tmp.begin() + static_cast<int64_t>(cnt[v]),
              tmp.begin() + static_cast<int64_t>(cnt[v] + (uniq[v + 1] - uniq[v])),
              g.adj.begin() + static_cast<int64_t>(uniq[v]));
}

// R-MAT edge draws of stream 3: draw i goes to src[i * stride], dst[i * stride].
void rmat_draws(uint32_t scale, uint64_t draws, uint64_t seed, uint32_t *src, uint32_t *dst, uint64_t stride) {
  // (a, a+b, a+b+c) = (0.57, 0.76, 0.95) on a 16-bit grid
  const uint32_t TA = 37356, TB = 49807, TC = 62259;
  const int64_t chunk = 1 << 20;
  const int64_t nchunks = static_cast<int64_t>((draws + chunk - 1) / chunk);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t c = 0; c < nchunks; ++c) {
    Rng r(stream_seed(seed, 3, static_cast<uint64_t>(c)));
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
        uint32_t x = static_cast<uint32_t>(bits & 0xFFFF);
        bits >>= 16;
        --left;
        uint32_t bu = x >= TB, bv = (x >= TA && x < TB) || x >= TC;
        u = (u << 1) | bu;
        v = (v << 1) | bv;
      }
      src[static_cast<uint64_t>(i) * stride] = u;
      dst[static_cast<uint64_t>(i) * stride] = v;
    }
  }
}

bool adjacent(const smg_csr &g, uint32_t a, uint32_t b) {
  // lists of generated and uploaded graphs are sorted; file graphs may not be
  const uint32_t *lo = g.neighbors + g.offsets[a], *hi = g.neighbors + g.offsets[a + 1];
  if (hi - lo > 64 && std::is_sorted(lo, hi)) return std::binary_search(lo, hi, b);
  return std::find(lo, hi, b) != hi;
}

}  // namespace
}  // namespace smg

using namespace smg;

extern "C" {

smg_status smg_gen_er(uint32_t n, uint64_t m, uint32_t num_labels, uint32_t label_dist,
                      uint64_t seed, smg_host_graph **out) {
  if (!out || n < 2 || num_labels == 0) return fail(SMG_ERR_INVALID, "bad ER arguments");
  *out = nullptr;
  const uint64_t maxm = static_cast<uint64_t>(n) * (n - 1) / 2;
  if (m > maxm) return fail(SMG_ERR_INVALID, "more edges than vertex pairs");
  if (m > (1ull << 28)) return fail(SMG_ERR_LIMIT, "ER generator is meant for small graphs");
  Rng r(stream_seed(seed, 1, 0));
  std::unordered_set<uint64_t> seen;
  seen.reserve(static_cast<size_t>(m) * 2);
  std::vector<uint32_t> src, dst;
  src.reserve(m);
  dst.reserve(m);
  while (src.size() < m) {
    uint32_t a = static_cast<uint32_t>(r.below(n)), b = static_cast<uint32_t>(r.below(n));
    if (a == b) continue;
    uint64_t key = (static_cast<uint64_t>(std::min(a, b)) << 32) | std::max(a, b);
    if (!seen.insert(key).second) continue;
    src.push_back(a);
    dst.push_back(b);
  }
  std::unique_ptr<smg_host_graph> h(new smg_host_graph);
  build_simple_csr(n, src, dst, h->g);
  draw_labels(h->g, num_labels, label_dist, seed);
  *out = h.release();
  return SMG_OK;
}

smg_status smg_gen_rmat(uint32_t scale, uint32_t avg_degree, uint32_t num_labels, uint32_t label_dist,
                        uint64_t seed, int threads, smg_host_graph **out) {
  if (!out || scale < 1 || scale > 31 || avg_degree == 0 || num_labels == 0)
    return fail(SMG_ERR_INVALID, "bad R-MAT arguments");
  *out = nullptr;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
  const uint32_t n = 1u << scale;
  const uint64_t draws = static_cast<uint64_t>(n) * avg_degree / 2;
  std::vector<uint32_t> src(draws), dst(draws);
  rmat_draws(scale, draws, seed, src.data(), dst.data(), 1);
  std::unique_ptr<smg_host_graph> h(new smg_host_graph);
  build_simple_csr(n, src, dst, h->g);
  std::vector<uint32_t>().swap(src);
  std::vector<uint32_t>().swap(dst);
  draw_labels(h->g, num_labels, label_dist, seed);
  *out = h.release();
  return SMG_OK;
}

smg_status smg_gen_rmat_pairs(uint32_t scale, uint32_t avg_degree, uint64_t seed, int threads, uint32_t *pairs,
                              uint64_t *num_pairs) {
  if (!num_pairs || scale < 1 || scale > 31 || avg_degree == 0) return fail(SMG_ERR_INVALID, "bad R-MAT arguments");
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
  const uint64_t draws = (static_cast<uint64_t>(1) << scale) * avg_degree / 2;
  *num_pairs = draws;
  if (pairs) rmat_draws(scale, draws, seed, pairs, pairs + 1, 2);
  return SMG_OK;
}

smg_status smg_gen_labels(uint32_t num_vertices, uint32_t num_labels, uint32_t label_dist, uint64_t seed,
                          uint32_t *labels) {
  if ((num_vertices && !labels) || num_labels == 0) return fail(SMG_ERR_INVALID, "bad label arguments");
  draw_labels_into(num_vertices, num_labels, label_dist, seed, labels);
  return SMG_OK;
}

smg_status smg_gen_query(const smg_csr *gc, uint32_t k, uint32_t shape, uint64_t seed,
                         smg_host_query **out, uint32_t *out_data_vertices) {
  if (!gc || !out || k < 2 || k > SMG_MAX_QUERY_VERTICES || shape > SMG_SHAPE_INDUCED)
    return fail(SMG_ERR_INVALID, "bad query-generator arguments");
  *out = nullptr;
  const smg_csr &g = *gc;
  Rng r(stream_seed(seed, 4, k * 3 + shape));
  const int max_attempts = 20000000;
  for (int attempt = 0; attempt < max_attempts; ++attempt) {
    uint32_t start = 0;
    bool found = false;
    for (int t = 0; t < 4096; ++t) {
      start = static_cast<uint32_t>(r.below(g.num_vertices));
      if (g.offsets[start + 1] > g.offsets[start]) {
        found = true;
        break;
      }
    }
    if (!found) return fail(SMG_ERR_INVALID, "graph has (almost) no edges");
    std::vector<uint32_t> vis{start};
    std::vector<uint32_t> tree;  // query-index pairs
    uint32_t cur = start, cur_idx = 0;
    for (uint32_t step = 0; step < 100 * k && vis.size() < k; ++step) {
      uint64_t d = g.offsets[cur + 1] - g.offsets[cur];
      uint32_t nxt = g.neighbors[g.offsets[cur] + r.below(d)];
      auto it = std::find(vis.begin(), vis.end(), nxt);
      uint32_t nxt_idx;
      if (it == vis.end()) {
        nxt_idx = static_cast<uint32_t>(vis.size());
        vis.push_back(nxt);
        tree.push_back(cur_idx);
        tree.push_back(nxt_idx);
      } else {
        nxt_idx = static_cast<uint32_t>(it - vis.begin());
      }
      cur = nxt;
      cur_idx = nxt_idx;
    }
    if (vis.size() < k) continue;
    // induced non-tree edges in (i, j) order
    std::vector<uint32_t> extra;
    for (uint32_t i = 0; i < k; ++i)
      for (uint32_t j = i + 1; j < k; ++j) {
        bool is_tree = false;
        for (size_t t = 0; t < tree.size(); t += 2)
          if ((tree[t] == i && tree[t + 1] == j) || (tree[t] == j && tree[t + 1] == i)) is_tree = true;
        if (!is_tree && adjacent(g, vis[i], vis[j])) {
          extra.push_back(i);
          extra.push_back(j);
        }
      }
    std::vector<uint32_t> edges = tree;
    if (shape == SMG_SHAPE_SPARSE) {
      const uint64_t c = extra.size() / 2;
      if (c < 2) continue;
      uint64_t a = r.below(c), b = r.below(c - 1);
      if (b >= a) ++b;
      edges.insert(edges.end(), {extra[2 * a], extra[2 * a + 1], extra[2 * b], extra[2 * b + 1]});
    } else if (shape == SMG_SHAPE_DENSE) {
      edges.insert(edges.end(), extra.begin(), extra.end());
      if (edges.size() < 3ull * k) continue;  // average degree 2|E|/k >= 3
    } else if (shape == SMG_SHAPE_INDUCED) {
      edges.insert(edges.end(), extra.begin(), extra.end());
    }
    std::unique_ptr<smg_host_query> h(new smg_host_query);
    h->q.n = k;
    h->q.label.resize(k);
    for (uint32_t i = 0; i < k; ++i) h->q.label[i] = gc->labels[vis[i]];
    h->q.edges = std::move(edges);
    if (out_data_vertices) std::copy(vis.begin(), vis.end(), out_data_vertices);
    *out = h.release();
    return SMG_OK;
  }
  return fail(SMG_ERR_LIMIT, "no query of the requested shape found by the random walk");
}

}  // extern "C"
