// api.cu — the C ABI of libsmg: device context, resident graph, plain and
// batched matching, filter inspection.
//
// The reference's main (main.cu:24-175) runs one query per process: it reads
// both graphs, copies them to the device, filters, joins and prints
// num_res.  Here the data graph is uploaded once and stays resident; a query
// costs one filter pass (filter.cu) and one persistent join launch (join.cu)
// on the context's stream, with scratch taken from a grow-only device arena
// instead of per-query cudaMalloc/cudaMemset of 2 x k x 2 GB result tables
// (join.cu:313-319).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "api_internal.cuh"
#include "filter.cuh"
#include "join.cuh"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace smg {

smg_status cuda_fail(cudaError_t e, const char *what) {
  cudaGetLastError();  // clear a sticky-free error so the context stays usable
  const smg_status s = (e == cudaErrorMemoryAllocation) ? SMG_ERR_OOM
                       : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? SMG_ERR_NO_DEVICE
                                                                                        : SMG_ERR_CUDA;
  return fail(s, std::string(what) + ": " + cudaGetErrorName(e) + " " + cudaGetErrorString(e));
}

// ------------------------------------------------------------------ arena
smg_status Arena::reserve(size_t bytes) {
  if (bytes <= cap) return SMG_OK;
  if (base) cudaFree(base);
  base = nullptr;
  cap = 0;
  // grow by a quarter for the next, larger batch, but never into the headroom
  // that kernel launches (local memory), graphs and the filter's step tables
  // need
  size_t free_b = 0, total_b = 0;
  SMG_CUDA(cudaMemGetInfo(&free_b, &total_b));
  const size_t spare = free_b > kHeadroomBytes ? free_b - kHeadroomBytes : 0;
  const size_t want = std::max(bytes, std::min(bytes + bytes / 4 + (1 << 20), spare));
  cudaError_t e = cudaMalloc(&base, want);
  if (e != cudaSuccess) {
    e = cudaMalloc(&base, bytes);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(arena)");
    cap = bytes;
  } else {
    cap = want;
  }
  return SMG_OK;
}

Arena::~Arena() {
  if (base) cudaFree(base);
}

// Vertices of at least this degree get a neighbour bitmap (one-load
// membership tests in the join), up to hub_max_bytes of bitmaps per graph.
uint32_t hub_min_degree() {
  const char *s = std::getenv("SMG_HUB_MIN_DEGREE");
  return s ? static_cast<uint32_t>(std::atol(s)) : 128u;
}

// SMG_HUB_BYTES, else min(64 GB, a quarter of free memory).  On the 2^22
// R-MAT workload (n / 8 = 512 KB a row) 2 GB covers the 4,096 vertices of
// highest degree and every other probe binary-searches a list; 64 GB covers
// all 109,643 vertices of degree >= 128 (57 GB) and cut the join from 159 to
// 145 ms per 1,024 queries (16 GB: 4% less than 2 GB on the dense class).
size_t hub_max_bytes() {
  if (const char *s = std::getenv("SMG_HUB_BYTES")) return static_cast<size_t>(std::atoll(s));
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return 2ull << 30;
  return std::min<size_t>(64ull << 30, free_b / 4);
}

// Vertices of at least this degree get a label run table (the join scans
// only the neighbours of the label it needs), up to 1 GB of tables, highest
// degree first.  SMG_LABEL_INDEX=0 leaves the index out (whole lists are
// scanned).  On the 2^22 R-MAT workload (32 labels, 132 B of table a
// vertex) a threshold of 64 measured join 142.8 / 145.1 ms per 1,024
// queries, 16 measured 139.1 / 139.5 and 4 measured 137.4 / 138.4: shorter
// lists then also come as label runs, with their entries' ranks.
uint32_t label_index_min_degree() {
  const char *s = std::getenv("SMG_LABEL_INDEX_MIN_DEGREE");
  return s ? static_cast<uint32_t>(std::atol(s)) : 4u;
}

bool label_index_enabled() {
  const char *s = std::getenv("SMG_LABEL_INDEX");
  return !(s && std::strcmp(s, "0") == 0);
}

void drop_graph(smg_ctx *c) {
  if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
  c->graph_exec = nullptr;
  c->graph_key.clear();
  c->graph_gen = ~0ull;
}

void release_batch_memory(smg_ctx *c) {
  if (c->stream) cudaStreamSynchronize(c->stream);
  drop_graph(c);
  c->arena.~Arena();
  new (&c->arena) Arena();
}

uint64_t time_limit_ns() {
  const char *s = std::getenv("SMG_TIME_LIMIT_S");
  double v = s ? std::atof(s) : 120.0;
  if (v <= 0) v = 120.0;
  return static_cast<uint64_t>(v * 1e9);
}

}  // namespace smg

using namespace smg;

namespace smg {
// Everything a resident graph holds besides off/adj (already on the device):
// labels, vertices grouped by label, neighbour-label counts, the label index
// and the hub bitmaps.  offsets/adj/labels are the same CSR in host memory.
smg_status finish_resident(smg_ctx *c, DevGraph &g, const uint64_t *offsets, const uint32_t *adj_src,
                           const uint32_t *labels, uint32_t maxl, uint32_t maxd) {
  const uint32_t n = g.n;
  g.num_labels = n ? maxl + 1 : 0;
  g.max_degree = maxd;
  g.label_count.assign(std::min<uint32_t>(g.num_labels, kMaxLabels), 0);
  for (uint32_t v = 0; v < n; ++v)
    if (labels[v] < kMaxLabels) ++g.label_count[labels[v]];
  // vertex ids grouped by label (labels >= kMaxLabels, which no query has, at the end)
  std::vector<uint32_t> lverts(std::max<uint32_t>(n, 1));
  {
    const size_t nl = g.label_count.size();
    g.lvert_start.assign(nl + 1, 0);
    for (size_t l = 0; l < nl; ++l) g.lvert_start[l + 1] = g.lvert_start[l] + static_cast<uint32_t>(g.label_count[l]);
    std::vector<uint32_t> at(g.lvert_start.begin(), g.lvert_start.end() - 1);
    uint32_t tail = g.lvert_start[nl];
    for (uint32_t v = 0; v < n; ++v) {
      const uint32_t l = labels[v];
      lverts[l < nl ? at[l]++ : tail++] = v;
    }
  }
  const uint32_t ncols = std::min<uint32_t>(g.num_labels, kMaxLabels);
  g.nlc_stride = std::max<uint32_t>(16, (ncols + 15) & ~15u);
  const size_t b_lab = std::max<size_t>(n, 1) * 4, b_nlc = std::max<size_t>(n, 1) * g.nlc_stride;
  SMG_CUDA(cudaMalloc(&g.label, b_lab));
  SMG_CUDA(cudaMalloc(&g.nlc, b_nlc));
  SMG_CUDA(cudaMalloc(&g.lverts, b_lab));
  SMG_CUDA(cudaMalloc(&g.ldeg, b_lab));
  SMG_CUDA(cudaMalloc(&g.pos_of, b_lab));
  SMG_CUDA(cudaMalloc(&g.lvstart, g.lvert_start.size() * 4));
  g.bytes += 4 * b_lab + b_nlc + g.lvert_start.size() * 4;
  std::vector<uint32_t> pos_of(std::max<uint32_t>(n, 1));
  for (uint32_t p = 0; p < n; ++p) pos_of[lverts[p]] = p;
  if (n) SMG_CUDA(cudaMemcpyAsync(g.label, labels, static_cast<size_t>(n) * 4, cudaMemcpyHostToDevice, c->stream));
  if (n) SMG_CUDA(cudaMemcpyAsync(g.lverts, lverts.data(), static_cast<size_t>(n) * 4, cudaMemcpyHostToDevice, c->stream));
  if (n) SMG_CUDA(cudaMemcpyAsync(g.pos_of, pos_of.data(), static_cast<size_t>(n) * 4, cudaMemcpyHostToDevice, c->stream));
  SMG_CUDA(cudaMemcpyAsync(g.lvstart, g.lvert_start.data(), g.lvert_start.size() * 4, cudaMemcpyHostToDevice,
                           c->stream));
  smg_status st = launch_build_nlc(g, c->stream, c->num_sms);
  if (st) return st;
  if (label_index_enabled()) {
    // the id-ordered lists the device got; built first: the hub bitmaps take
    // its label layout
    st = build_label_index(g, offsets, adj_src, labels, label_index_min_degree(), 1ull << 30, c->stream);
    if (st) return st;
  }
  {
    std::vector<uint32_t> deg(n);
#pragma omp parallel for schedule(static)
    for (int64_t v = 0; v < static_cast<int64_t>(n); ++v)
      deg[v] = static_cast<uint32_t>(offsets[v + 1] - offsets[v]);
    st = build_hub_bitmaps(g, hub_min_degree(), hub_max_bytes(), c->stream, deg);
    if (st) return st;
  }
  SMG_CUDA(cudaStreamSynchronize(c->stream));
  return SMG_OK;
}
}  // namespace smg

extern "C" {

smg_status smg_open(int device, smg_ctx **out) {
  if (!out) return fail(SMG_ERR_INVALID, "null out");
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    cudaGetLastError();
    return fail(SMG_ERR_NO_DEVICE, "no CUDA device visible");
  }
  if (device < 0 || device >= count) return fail(SMG_ERR_INVALID, "device index out of range");
  std::unique_ptr<smg_ctx> c(new smg_ctx);
  c->device = device;
  SMG_CUDA(cudaSetDevice(device));
  cudaDeviceProp prop;
  SMG_CUDA(cudaGetDeviceProperties(&prop, device));
  c->num_sms = prop.multiProcessorCount;
  SMG_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  SMG_CUDA(cudaEventCreate(&c->ev[0]));
  SMG_CUDA(cudaEventCreate(&c->ev[1]));
  SMG_CUDA(cudaEventCreate(&c->ev[2]));
  SMG_CUDA(cudaMallocHost(&c->pinned, kPinnedBytes));
  *out = c.release();
  return SMG_OK;
}

void *smg_ctx_stream(smg_ctx *c) { return c ? static_cast<void *>(c->stream) : nullptr; }

void smg_close(smg_ctx *c) {
  if (!c) return;
  cudaSetDevice(c->device);
  release_batch_memory(c);
  c->fdev.reset();
  for (auto &e : c->ev)
    if (e) cudaEventDestroy(e);
  if (c->pinned) cudaFreeHost(c->pinned);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

smg_status smg_graph_upload(smg_ctx *c, const smg_csr *in, smg_graph **out) {
  if (!c || !in || !out) return fail(SMG_ERR_INVALID, "null argument");
  *out = nullptr;
  const uint32_t n = in->num_vertices;
  const uint64_t m2 = 2 * in->num_edges;
  if (n && (!in->offsets || !in->labels || (m2 && !in->neighbors))) return fail(SMG_ERR_INVALID, "null arrays");
  if (m2 >= (1ull << 32)) return fail(SMG_ERR_LIMIT, "more than 2^32-1 adjacency entries");
  if (n == 0xFFFFFFFFu) return fail(SMG_ERR_LIMIT, "too many vertices");
  if (in->offsets[0] != 0 || in->offsets[n] != m2) return fail(SMG_ERR_INVALID, "offsets do not span 2*num_edges");
  SMG_CUDA(cudaSetDevice(c->device));
  std::unique_ptr<smg_graph> G(new smg_graph);
  DevGraph &g = G->g;
  g.n = n;
  g.m2 = m2;
  // host checks and the sorted copy the device needs
  std::vector<uint32_t> off32(static_cast<size_t>(n) + 1);
  bool bad = false, unsorted = false;
  uint32_t maxl = 0, maxd = 0;
#pragma omp parallel for schedule(static) reduction(|| : bad) reduction(max : maxl, maxd)
  for (int64_t v = 0; v < static_cast<int64_t>(n); ++v) {
    const uint64_t a = in->offsets[v], b = in->offsets[v + 1];
    off32[v] = static_cast<uint32_t>(a);
    if (b < a) {
      bad = true;
      continue;
    }
    maxd = std::max<uint32_t>(maxd, static_cast<uint32_t>(b - a));
    maxl = std::max(maxl, in->labels[v]);
  }
  off32[n] = static_cast<uint32_t>(m2);
  if (bad) return fail(SMG_ERR_INVALID, "offsets are not monotone");
#pragma omp parallel for schedule(dynamic, 4096) reduction(|| : bad, unsorted)
  for (int64_t v = 0; v < static_cast<int64_t>(n); ++v) {
    for (uint64_t e = in->offsets[v]; e < in->offsets[v + 1]; ++e) {
      const uint32_t w = in->neighbors[e];
      if (w >= n || w == static_cast<uint32_t>(v)) bad = true;
      if (e > in->offsets[v] && in->neighbors[e - 1] >= w) unsorted = true;
    }
  }
  if (bad) return fail(SMG_ERR_INVALID, "neighbour id out of range or self-loop");
  std::vector<uint32_t> sorted;
  const uint32_t *adj_src = in->neighbors;
  if (unsorted) {
    sorted.assign(in->neighbors, in->neighbors + m2);
#pragma omp parallel for schedule(dynamic, 4096) reduction(|| : bad)
    for (int64_t v = 0; v < static_cast<int64_t>(n); ++v) {
      auto b = sorted.begin() + static_cast<int64_t>(in->offsets[v]);
      auto e = sorted.begin() + static_cast<int64_t>(in->offsets[v + 1]);
      std::sort(b, e);
      if (std::adjacent_find(b, e) != e) bad = true;
    }
    if (bad) return fail(SMG_ERR_INVALID, "repeated edge");
    adj_src = sorted.data();
  }
  const size_t b_off = (static_cast<size_t>(n) + 1) * 4, b_adj = std::max<uint64_t>(m2, 1) * 4;
  SMG_CUDA(cudaMalloc(&g.off, b_off));
  SMG_CUDA(cudaMalloc(&g.adj, b_adj));
  g.bytes = b_off + b_adj;
  SMG_CUDA(cudaMemcpyAsync(g.off, off32.data(), b_off, cudaMemcpyHostToDevice, c->stream));
  if (m2) SMG_CUDA(cudaMemcpyAsync(g.adj, adj_src, m2 * 4, cudaMemcpyHostToDevice, c->stream));
  smg_status st = finish_resident(c, g, in->offsets, adj_src, in->labels, maxl, maxd);
  if (st) return st;
  G->device = c->device;
  *out = G.release();
  return SMG_OK;
}

smg_status smg_graph_build(smg_ctx *c, uint32_t num_vertices, uint64_t num_pairs, const uint32_t *pairs,
                           const uint32_t *labels, smg_graph **out, uint64_t *num_edges) {
  if (!c || !out || (num_vertices && !labels) || (num_pairs && !pairs)) return fail(SMG_ERR_INVALID, "null argument");
  *out = nullptr;
  const uint32_t n = num_vertices;
  if (n == 0xFFFFFFFFu) return fail(SMG_ERR_LIMIT, "too many vertices");
  if (num_pairs >= (1ull << 31)) return fail(SMG_ERR_LIMIT, "2^31 or more edge pairs");
  SMG_CUDA(cudaSetDevice(c->device));
  std::unique_ptr<smg_graph> G(new smg_graph);
  DevGraph &g = G->g;
  g.n = n;
  unsigned long long *off64 = nullptr;
  uint32_t *adj = nullptr;
  uint64_t m2 = 0;
  smg_status st = build_csr_device(c, n, num_pairs, pairs, &off64, &adj, &m2);
  if (st) return st;
  g.m2 = m2;
  g.adj = adj;
  // the join indexes lists with 32-bit offsets; 2|E| < 2^32 holds here
  // because the pairs are fewer than 2^31
  const size_t b_off = (static_cast<size_t>(n) + 1) * 4;
  SMG_CUDA(cudaMalloc(&g.off, b_off));
  g.bytes = b_off + std::max<uint64_t>(m2, 1) * 4;
  st = narrow_offsets(off64, g.off, static_cast<uint64_t>(n) + 1, c->stream, c->num_sms);
  if (st) {
    cudaFree(off64);
    return st;
  }
  // the host copy of the CSR the label index and the hub selection read
  std::vector<uint64_t> offsets(static_cast<size_t>(n) + 1);
  std::vector<uint32_t> adj_host(std::max<uint64_t>(m2, 1));
  SMG_CUDA(cudaMemcpyAsync(offsets.data(), off64, offsets.size() * 8, cudaMemcpyDeviceToHost, c->stream));
  if (m2) SMG_CUDA(cudaMemcpyAsync(adj_host.data(), adj, m2 * 4, cudaMemcpyDeviceToHost, c->stream));
  SMG_CUDA(cudaStreamSynchronize(c->stream));
  cudaFree(off64);
  uint32_t maxl = 0, maxd = 0;
#pragma omp parallel for schedule(static) reduction(max : maxl, maxd)
  for (int64_t v = 0; v < static_cast<int64_t>(n); ++v) {
    maxd = std::max<uint32_t>(maxd, static_cast<uint32_t>(offsets[v + 1] - offsets[v]));
    maxl = std::max(maxl, labels[v]);
  }
  st = finish_resident(c, g, offsets.data(), adj_host.data(), labels, maxl, maxd);
  if (st) return st;
  if (num_edges) *num_edges = m2 / 2;
  G->device = c->device;
  *out = G.release();
  return SMG_OK;
}

smg_status smg_graph_download(smg_ctx *c, const smg_graph *G, uint64_t *offsets, uint32_t *neighbors) {
  if (!c || !G || !offsets || (G->g.m2 && !neighbors)) return fail(SMG_ERR_INVALID, "null argument");
  if (G->device != c->device) return fail(SMG_ERR_INVALID, "graph lives on another device");
  SMG_CUDA(cudaSetDevice(c->device));
  const DevGraph &g = G->g;
  std::vector<uint32_t> off32(static_cast<size_t>(g.n) + 1);
  SMG_CUDA(cudaMemcpyAsync(off32.data(), g.off, off32.size() * 4, cudaMemcpyDeviceToHost, c->stream));
  if (g.m2) SMG_CUDA(cudaMemcpyAsync(neighbors, g.adj, g.m2 * 4, cudaMemcpyDeviceToHost, c->stream));
  SMG_CUDA(cudaStreamSynchronize(c->stream));
  for (size_t i = 0; i < off32.size(); ++i) offsets[i] = off32[i];
  return SMG_OK;
}

void smg_graph_free(smg_graph *G) {
  if (!G) return;
  cudaSetDevice(G->device);
  DevGraph &g = G->g;
  if (g.off) cudaFree(g.off);
  if (g.adj) cudaFree(g.adj);
  if (g.label) cudaFree(g.label);
  if (g.nlc) cudaFree(g.nlc);
  if (g.lverts) cudaFree(g.lverts);
  if (g.ldeg) cudaFree(g.ldeg);
  if (g.pos_of) cudaFree(g.pos_of);
  if (g.lvstart) cudaFree(g.lvstart);
  if (g.hub_of) cudaFree(g.hub_of);
  if (g.hub_bits) cudaFree(g.hub_bits);
  if (g.adjr) cudaFree(g.adjr);
  if (g.adjl) cudaFree(g.adjl);
  if (g.lab_of) cudaFree(g.lab_of);
  if (g.lab_off) cudaFree(g.lab_off);
  if (g.lab_rank) cudaFree(g.lab_rank);
  if (g.bucket_word_off) cudaFree(g.bucket_word_off);
  delete G;
}

smg_status smg_graph_get_stats(const smg_graph *G, smg_graph_stats *out) {
  if (!G || !out) return fail(SMG_ERR_INVALID, "null argument");
  out->num_vertices = G->g.n;
  out->num_edges = G->g.m2 / 2;
  out->num_labels = G->g.num_labels;
  out->max_degree = G->g.max_degree;
  out->device_bytes = G->g.bytes;
  return SMG_OK;
}

}  // extern "C"

namespace smg {
namespace {

inline size_t al(size_t x) { return (x + 255) & ~size_t(255); }

// Device layout of one chunk of queries inside the arena.  Everything that
// must start at zero (queue state, ready flags, counters, cluster bitmaps) is
// one contiguous region cleared with a single memset.
struct Chunk {
  uint32_t a = 0, b = 0, kmax = 0, cap = 0;
  size_t zero_bytes = 0, total = 0;
  QueueState *qs = nullptr;
  uint32_t *ready = nullptr, *tasks = nullptr, *emb = nullptr, *xbuf = nullptr;
  QCounters *counters = nullptr;
  unsigned int *walk_count = nullptr;  // one zeroed counter pair per walk phase
  uint4 *walk_items = nullptr;
  uint32_t walk_cap = 0;
  FilterQuery *fq = nullptr;
  JoinQuery *jq = nullptr;
  std::vector<uint32_t *> vmask, enc, cand, roots, cbits;
  // What a batch clears before the filter: the queue state, ready flags and
  // counters, each query's candidate bitmaps, and its masks and cluster
  // bitmap only over the positions of its own label groups (the filter and
  // the join read nothing else of them).  A device plan for k_zero_ranges:
  // zero_plan[0 .. nr] word prefix sums, zero_plan[nr + 1 ..] byte offsets.
  std::vector<size_t> o_enc, o_vm, o_cb;
  size_t head_bytes = 0, zero_plan_cap = 0;
  uint64_t *zero_plan = nullptr;
  uint32_t zero_ranges = 0;
  std::vector<uint64_t> cand_total;
};

// k id-indexed rows, and k rank-indexed ones when the graph has entry ranks
size_t cbits_bytes(const DevGraph &g, uint32_t k) {
  return static_cast<size_t>(k) * ((g.n + 31ull) / 32) * 4 * (g.adjr ? 2 : 1);
}

}  // namespace

uint32_t plan_class(const Plan &P) {
  const uint32_t shape = P.m + 1 == P.k ? 0u : (2 * P.m >= 3 * P.k ? 2u : 1u);
  const uint32_t size = P.k <= 5 ? 0u : P.k <= 8 ? 1u : P.k <= 12 ? 2u : 3u;
  return 4 * shape + size;
}

namespace {

uint64_t label_cands(const DevGraph &g, uint32_t l) { return l < g.label_count.size() ? g.label_count[l] : 0; }

uint32_t order_mode() {  // 0 cost-based with counted endings, 1 greedy only, 2 the reference's
  static const uint32_t v = [] {
    const char *e = std::getenv("SMG_JOIN_ORDER");
    if (e && std::strcmp(e, "plan") == 0) return 2u;
    if (e && std::strcmp(e, "greedy") == 0) return 1u;
    return 0u;
  }();
  return v;
}

// Greedy order of the query vertices in `allowed` (a connected set): first
// the one with the fewest label candidates per query edge, then repeatedly
// the one with the most edges back to those placed, then the fewest
// candidates, then the highest degree.  Writes order[at ..] and returns the
// next position.
uint32_t greedy_order(const Plan &P, const DevGraph &g, uint32_t allowed, uint32_t *order, uint32_t at) {
  const uint32_t k = P.k;
  uint32_t root = kNone;
  for (uint32_t u = 0; u < k; ++u)
    if ((allowed >> u) & 1u)
      if (root == kNone || label_cands(g, P.label[u]) * P.deg[root] < label_cands(g, P.label[root]) * P.deg[u])
        root = u;
  uint32_t placed = 1u << root;
  order[at++] = root;
  while (placed != allowed) {
    uint32_t best = kNone, best_back = 0;
    for (uint32_t u = 0; u < k; ++u) {
      if (!((allowed >> u) & 1u) || ((placed >> u) & 1u)) continue;
      uint32_t nb = 0;
      for (uint32_t e = P.q_off[u]; e < P.q_off[u + 1]; ++e) nb += (placed >> P.q_nbr[e]) & 1u;
      if (!nb) continue;
      bool better = best == kNone || nb > best_back;
      if (!better && nb == best_back) {
        const uint64_t cu = label_cands(g, P.label[u]), cb = label_cands(g, P.label[best]);
        better = cu < cb || (cu == cb && P.deg[u] > P.deg[best]);
      }
      if (better) {
        best = u;
        best_back = nb;
      }
    }
    order[at++] = best;  // `allowed` is connected, so one is adjacent
    placed |= 1u << best;
  }
  return at;
}

uint32_t nbr_mask(const Plan &P, uint32_t u) {
  uint32_t m = 0;
  for (uint32_t e = P.q_off[u]; e < P.q_off[u + 1]; ++e) m |= 1u << P.q_nbr[e];
  return m;
}

bool connected(const Plan &P, uint32_t set) {
  if (!set) return false;
  uint32_t seen = set & (~set + 1), frontier = seen;
  while (frontier) {
    uint32_t next = 0;
    for (uint32_t f = frontier; f; f &= f - 1) next |= nbr_mask(P, __builtin_ctz(f)) & set;
    frontier = next & ~seen;
    seen |= next;
  }
  return seen == set;
}

// The join's matching order (every connected order yields the same
// embeddings).  It ends, where the query allows, so that the last level is
// counted rather than enumerated: with a leaf (one back edge: per-vertex
// neighbour counts), else with two non-adjacent vertices (the last vertex
// does not depend on the level before it: one hoisted set per prefix);
// among several, the ending vertex with the most candidates.  The rest, and
// queries with neither, take the greedy order.  SMG_JOIN_ORDER=greedy keeps
// the greedy order throughout, =plan the order the reference's edge order
// (order.cpp getBFSEdgeOrder) reaches the vertices in.
void compute_order(const Plan &P, const DevGraph &g, uint32_t *order) {
  const uint32_t k = P.k, all = k >= 32 ? 0xFFFFFFFFu : (1u << k) - 1;
  if (order_mode() == 2) {
    for (uint32_t l = 0; l < k; ++l) order[l] = P.order[l];
    return;
  }
  if (order_mode() == 0 && k >= 3) {
    uint32_t leaf = kNone;
    for (uint32_t u = 0; u < k; ++u)
      if (P.deg[u] == 1 && (leaf == kNone || label_cands(g, P.label[u]) > label_cands(g, P.label[leaf]))) leaf = u;
    if (leaf != kNone) {
      greedy_order(P, g, all & ~(1u << leaf), order, 0);
      order[k - 1] = leaf;
      return;
    }
    if (k >= 4) {
      uint32_t bx = kNone, by = kNone;
      for (uint32_t y = 0; y < k; ++y)
        for (uint32_t x = 0; x < k; ++x) {
          if (x == y || ((nbr_mask(P, y) >> x) & 1u)) continue;
          if (!connected(P, all & ~(1u << x) & ~(1u << y))) continue;
          const uint64_t cy = label_cands(g, P.label[y]), cx = label_cands(g, P.label[x]);
          if (by == kNone || cy > label_cands(g, P.label[by]) ||
              (cy == label_cands(g, P.label[by]) && cx > label_cands(g, P.label[bx]))) {
            bx = x;
            by = y;
          }
        }
      if (by != kNone) {
        greedy_order(P, g, all & ~(1u << bx) & ~(1u << by), order, 0);
        order[k - 2] = bx;
        order[k - 1] = by;
        return;
      }
    }
  }
  greedy_order(P, g, all, order, 0);
}

}  // namespace

// The first vertex of the join's matching order (its candidates are the root list).
uint32_t join_root(const Plan &P, const DevGraph &g) {
  uint32_t order[kMaxK];
  compute_order(P, g, order);
  return order[0];
}

void join_order(const Plan &P, const DevGraph &g, uint32_t *order, uint32_t *back, uint32_t *same) {
  const uint32_t k = P.k;
  std::vector<uint32_t> level(k, kNone);
  compute_order(P, g, order);
  for (uint32_t l = 0; l < k; ++l) level[order[l]] = l;
  for (uint32_t l = 0; l < k; ++l) {
    const uint32_t u = order[l];
    back[l] = 0;
    same[l] = 0;
    for (uint32_t e = P.q_off[u]; e < P.q_off[u + 1]; ++e)
      if (level[P.q_nbr[e]] < l) back[l] |= 1u << level[P.q_nbr[e]];
    for (uint32_t lw = 0; lw < l; ++lw)
      if (P.label[order[lw]] == P.label[u]) same[l] |= 1u << lw;
  }
}

QueryFootprint query_footprint(const DevGraph &g, const Plan &P) {
  QueryFootprint f;
  uint64_t cand = 0;
  for (uint32_t u = 0; u < P.k; ++u) cand += label_cands(g, P.label[u]);
  const uint64_t rc = label_cands(g, P.label[join_root(P, g)]);
  f.vmask = al(static_cast<size_t>(g.n) * 4);
  f.enc = al(static_cast<size_t>(g.n) * P.num_words * 4);
  f.cand = al(std::max<uint64_t>(cand, 1) * 4);
  f.roots = al(std::max<uint64_t>(rc, 1) * 4);
  f.cbits = al(cbits_bytes(g, P.k));
  return f;
}

smg_status make_query_records(const Plan &P, const DevGraph &g, const QueryBuffers &b, uint64_t count_limit,
                              FilterQuery &f, JoinQuery &j, uint64_t work_limit) {
  smg_status st = fill_filter_query(P, g, f);
  if (st) return st;
  uint64_t acc = 0;
  for (uint32_t u = 0; u < P.k; ++u) {
    f.cand_off[u] = acc;
    acc += P.label[u] < g.label_count.size() ? g.label_count[P.label[u]] : 0;
  }
  f.cand_off[P.k] = acc;
  f.vmask = b.vmask;
  f.enc = b.enc;
  f.cand = b.cand;
  f.cand_cnt = b.counters->cand_cnt;
  f.roots = b.roots;
  std::memset(&j, 0, sizeof(j));
  join_order(P, g, j.order, j.back_mask, j.same_label);
  f.root = j.order[0];  // k_collect gathers the join's first vertex's candidates
  f.root_cap = label_cands(g, P.label[f.root]);
  f.num_roots = &b.counters->num_roots;
  f.stat = b.counters->stat;
  j.k = P.k;
  j.candmask = b.vmask;
  if (g.adjl) {
    j.use_labels = 1;
    for (uint32_t l = 0; l < P.k; ++l) j.level_bucket[l] = std::min(P.label[j.order[l]], g.lab_buckets - 1);
  }
  if (b.cbits) {
    f.cbits = b.cbits;  // k_collect writes them with the final masks
    f.cwords = (g.n + 31ull) / 32;
    f.rank_rows = g.adjr ? 1u : 0u;
    j.cbits = b.cbits;
    j.cwords = (g.n + 31ull) / 32;
    j.crow = g.adjr ? b.cbits + static_cast<size_t>(P.k) * j.cwords : nullptr;
    j.lastcnt = b.enc;
    const uint32_t last_back = j.back_mask[P.k - 1];
    if (last_back && !(last_back & (last_back - 1))) {
      j.fast_last = static_cast<uint32_t>(__builtin_ctz(last_back)) + 1;
      const uint32_t l = P.label[j.order[j.fast_last - 1]];  // its candidates all carry this label
      if (l + 1 < g.lvert_start.size()) {
        j.lc_lo = g.lvert_start[l];
        j.lc_hi = g.lvert_start[l + 1];
      }
    }
  }
  j.roots = b.roots;
  j.num_roots = &b.counters->num_roots;
  j.count = &b.counters->count;
  j.emb = b.emb;
  j.emb_cap = b.emb_cap;
  j.emb_count = &b.counters->emb_count;
  j.count_limit = count_limit;
  j.over = &b.counters->over;
  j.work_limit = work_limit;
  j.work = &b.counters->work;
  j.pending = &b.counters->pending;
  return SMG_OK;
}

namespace {

WalkOverflow walk_overflow(const Chunk &ch) {
  WalkOverflow w;
  w.count = ch.walk_count;
  w.cap = ch.walk_cap;
  w.items = ch.walk_items;
  return w;
}

size_t query_bytes(const DevGraph &g, const Plan &P, uint64_t &cand_total) {
  cand_total = 0;
  for (uint32_t u = 0; u < P.k; ++u)
    cand_total += P.label[u] < g.label_count.size() ? g.label_count[P.label[u]] : 0;
  const uint64_t rc = label_cands(g, P.label[join_root(P, g)]);
  return al(static_cast<size_t>(g.n) * 4) + al(static_cast<size_t>(g.n) * P.num_words * 4) + al(cand_total * 4) +
         al(rc * 4) + al(cbits_bytes(g, P.k)) + sizeof(QCounters) + al(sizeof(FilterQuery)) + al(sizeof(JoinQuery));
}

uint32_t seed_tasks(const smg_ctx *c, const RunOpts &o, uint32_t nq) {
  if (o.max_seed_tasks) return o.max_seed_tasks;
  const uint32_t warps = static_cast<uint32_t>(c->num_sms) * 64;
  return std::max<uint32_t>(16, (8 * warps) / std::max<uint32_t>(nq, 1));
}

smg_status layout_chunk(smg_ctx *c, const DevGraph &g, const Plan *const *plans, Chunk &ch, const RunOpts &o) {
  const uint32_t nq = ch.b - ch.a;
  ch.kmax = 0;
  for (uint32_t i = ch.a; i < ch.b; ++i) ch.kmax = std::max(ch.kmax, plans[i]->k);
  const uint32_t seeds = seed_tasks(c, o, nq);
  const uint64_t cap64 = static_cast<uint64_t>(nq) * seeds + (4u << 20);
  ch.cap = static_cast<uint32_t>(std::min<uint64_t>(cap64, 0x7FFFFFFFu));
  ch.cand_total.resize(nq);
  // zero region
  size_t off = 0;
  const size_t o_qs = off;
  off += al(sizeof(QueueState));
  const size_t o_ready = off;
  off += al(static_cast<size_t>(ch.cap) * 4);
  const size_t o_cnt = off;
  off += al(nq * sizeof(QCounters));
  const size_t o_wcnt = off;
  off += al(kMaxWalkPhases * 2 * sizeof(unsigned int));
  ch.head_bytes = off;
  std::vector<size_t> &o_enc = ch.o_enc, &o_vm = ch.o_vm, &o_cb = ch.o_cb;
  o_enc.assign(nq, 0);
  o_vm.assign(nq, 0);
  o_cb.assign(nq, 0);
  std::vector<size_t> o_cand(nq), o_root(nq);
  // the filter writes masks and candidate bitmaps only for vertices of the
  // query's labels: they start at zero with the cluster bitmaps
  for (uint32_t i = 0; i < nq; ++i) {
    o_enc[i] = off;
    off += al(static_cast<size_t>(g.n) * plans[ch.a + i]->num_words * 4);
    o_vm[i] = off;
    off += al(static_cast<size_t>(g.n) * 4);
    o_cb[i] = off;
    off += al(cbits_bytes(g, plans[ch.a + i]->k));
  }
  ch.zero_bytes = off;
  for (uint32_t i = 0; i < nq; ++i) {
    const Plan &P = *plans[ch.a + i];
    query_bytes(g, P, ch.cand_total[i]);
    o_cand[i] = off;
    off += al(ch.cand_total[i] * 4);
    o_root[i] = off;
    const uint64_t rc = label_cands(g, P.label[join_root(P, g)]);
    off += al(std::max<uint64_t>(rc, 1) * 4);
  }
  const size_t o_tasks = off;
  off += al(static_cast<size_t>(ch.cap) * (4 + ch.kmax) * 4);
  const size_t o_xbuf = off;  // the join warps' hoisted-set buffers
  off += al(hoist_buffer_bytes(c->num_sms));
  ch.walk_cap = kWalkCap;
  const size_t o_witems = off;
  off += al(static_cast<size_t>(ch.walk_cap) * sizeof(uint4));
  const size_t o_fq = off;
  off += al(nq * sizeof(FilterQuery));
  const size_t o_jq = off;
  off += al(nq * sizeof(JoinQuery));
  // the zero plan: at most the head, then per query its bitmaps and two
  // ranges per label group
  ch.zero_plan_cap = 1 + static_cast<size_t>(nq) * (2 * kMaxK + 1);
  const size_t o_zplan = off;
  off += al((2 * ch.zero_plan_cap + 1) * sizeof(uint64_t));
  const size_t o_emb = off;
  if (o.emb_host && o.emb_cap) off += al(o.emb_cap * ch.kmax * 4);
  ch.total = off;
  smg_status st = c->arena.reserve(ch.total);
  if (st) return st;
  char *B = c->arena.base;
  ch.qs = reinterpret_cast<QueueState *>(B + o_qs);
  ch.ready = reinterpret_cast<uint32_t *>(B + o_ready);
  ch.counters = reinterpret_cast<QCounters *>(B + o_cnt);
  ch.walk_count = reinterpret_cast<unsigned int *>(B + o_wcnt);
  ch.walk_items = reinterpret_cast<uint4 *>(B + o_witems);
  ch.tasks = reinterpret_cast<uint32_t *>(B + o_tasks);
  ch.xbuf = reinterpret_cast<uint32_t *>(B + o_xbuf);
  ch.fq = reinterpret_cast<FilterQuery *>(B + o_fq);
  ch.jq = reinterpret_cast<JoinQuery *>(B + o_jq);
  ch.zero_plan = reinterpret_cast<uint64_t *>(B + o_zplan);
  ch.emb = (o.emb_host && o.emb_cap) ? reinterpret_cast<uint32_t *>(B + o_emb) : nullptr;
  ch.vmask.resize(nq);
  ch.enc.resize(nq);
  ch.cand.resize(nq);
  ch.roots.resize(nq);
  ch.cbits.resize(nq);
  for (uint32_t i = 0; i < nq; ++i) {
    ch.cbits[i] = reinterpret_cast<uint32_t *>(B + o_cb[i]);
    ch.enc[i] = reinterpret_cast<uint32_t *>(B + o_enc[i]);
    ch.vmask[i] = reinterpret_cast<uint32_t *>(B + o_vm[i]);
    ch.cand[i] = reinterpret_cast<uint32_t *>(B + o_cand[i]);
    ch.roots[i] = reinterpret_cast<uint32_t *>(B + o_root[i]);
  }
  return SMG_OK;
}

// Host-side query records of a chunk, staged in pinned memory and uploaded.
smg_status stage_chunk(smg_ctx *c, const DevGraph &g, const Plan *const *plans, Chunk &ch, const RunOpts &o) {
  const uint32_t nq = ch.b - ch.a;
  const size_t need = nq * (sizeof(FilterQuery) + sizeof(JoinQuery));
  if (need > kPinnedBytes) return fail(SMG_ERR_INTERNAL, "chunk exceeds the pinned staging buffer");
  FilterQuery *hf = static_cast<FilterQuery *>(c->pinned);
  JoinQuery *hj = reinterpret_cast<JoinQuery *>(static_cast<char *>(c->pinned) + nq * sizeof(FilterQuery));
  FilterBatch fb;
  for (uint32_t i = 0; i < nq; ++i) {
    const Plan &P = *plans[ch.a + i];
    QueryBuffers b;
    b.vmask = ch.vmask[i];
    b.enc = ch.enc[i];
    b.cand = ch.cand[i];
    b.roots = ch.roots[i];
    b.cbits = ch.cbits[i];
    b.counters = ch.counters + i;
    b.emb = ch.emb;
    b.emb_cap = ch.emb ? o.emb_cap : 0;
    smg_status st = make_query_records(P, g, b, o.count_limit, hf[i], hj[i], o.work_limit);
    if (st) return st;
    if (o.tuning && !o.root_chunk) {
      const TuneSetting &t = o.tuning[plan_class(P)];
      if (t.valid) apply_tuning(t, hj[i]);
    }
    if (o.bfs_depth) hj[i].bfs_depth = o.bfs_depth;
    st = append_filter_steps(P, i, fb);
    if (st) return st;
  }
  if (!c->fdev) c->fdev.reset(new FilterDev);
  smg_status st = c->fdev->upload(fb, c->stream);
  if (st) return st;
  SMG_CUDA(cudaMemcpyAsync(ch.fq, hf, nq * sizeof(FilterQuery), cudaMemcpyHostToDevice, c->stream));
  SMG_CUDA(cudaMemcpyAsync(ch.jq, hj, nq * sizeof(JoinQuery), cudaMemcpyHostToDevice, c->stream));
  // The zero plan (see Chunk): the head, then per query the positions of its
  // label groups in its cluster bitmap and masks, and its candidate bitmaps
  // whole.  SMG_ZERO=full clears the whole region instead.
  ch.zero_ranges = 0;
  static const bool full_zero = [] {
    const char *e = std::getenv("SMG_ZERO");
    return e && std::string(e) == "full";
  }();
  if (!full_zero) {
    std::vector<std::pair<uint64_t, uint64_t>> rg;  // (byte offset, bytes)
    rg.emplace_back(0, ch.head_bytes);
    for (uint32_t i = 0; i < nq; ++i) {
      const Plan &P = *plans[ch.a + i];
      const uint64_t W = P.num_words;
      for (uint32_t gi = 0; gi < hf[i].ngrp; ++gi) {
        const uint64_t lo = hf[i].grp_lo[gi], hi = hf[i].grp_hi[gi];
        if (hi <= lo || hi > g.n) continue;
        rg.emplace_back(ch.o_enc[i] + lo * W * 4, (hi - lo) * W * 4);
        rg.emplace_back(ch.o_vm[i] + lo * 4, (hi - lo) * 4);
      }
      rg.emplace_back(ch.o_cb[i], cbits_bytes(g, P.k));
    }
    std::sort(rg.begin(), rg.end());
    const size_t plan_bytes = (2 * rg.size() + 1) * sizeof(uint64_t);
    uint64_t *hz = reinterpret_cast<uint64_t *>(hj + nq);
    if (rg.size() <= ch.zero_plan_cap && need + plan_bytes <= kPinnedBytes) {
      const size_t nr = rg.size();
      hz[0] = 0;
      for (size_t r = 0; r < nr; ++r) {
        hz[r + 1] = hz[r] + rg[r].second / 4;
        hz[nr + 1 + r] = rg[r].first;
      }
      SMG_CUDA(cudaMemcpyAsync(ch.zero_plan, hz, plan_bytes, cudaMemcpyHostToDevice, c->stream));
      ch.zero_ranges = static_cast<uint32_t>(nr);
    }
  }
  // the staging buffer is reused by the read-back: finish the copies first
  SMG_CUDA(cudaStreamSynchronize(c->stream));
  return SMG_OK;
}

JoinLaunch make_join_launch(smg_ctx *c, const DevGraph &g, Chunk &ch, const RunOpts &o) {
  const uint32_t nq = ch.b - ch.a;
  JoinLaunch jl;
  std::memset(&jl, 0, sizeof(jl));
  set_graph(jl, g);
  jl.queries = ch.jq;
  jl.nq = nq;
  jl.kmax = ch.kmax;
  jl.qs = ch.qs;
  jl.tasks = ch.tasks;
  jl.ready = ch.ready;
  jl.cap = ch.cap;
  jl.root_chunk = o.root_chunk;
  jl.max_seed_tasks = seed_tasks(c, o, nq);
  jl.donate_min = 2;
  // breadth-first levels may queue a few tasks per resident join warp beyond
  // the root tasks (SMG_BFS_SLOTS_PER_WARP, default 16), at most half the
  // queue: enough to spread every query's first levels over the grid, while
  // the deeper levels stay depth-first and split on demand
  static const uint64_t per_warp = [] {
    const char *e = std::getenv("SMG_BFS_SLOTS_PER_WARP");
    return static_cast<uint64_t>(e ? std::max(0L, std::atol(e)) : 16L);
  }();
  jl.bfs_budget = std::min<uint64_t>(ch.cap / 2, static_cast<uint64_t>(nq) * jl.max_seed_tasks +
                                                     per_warp * 32u * static_cast<uint64_t>(c->num_sms));
  jl.time_limit_ns = time_limit_ns();
  jl.emit = ch.emb != nullptr;
  jl.xbuf = ch.xbuf;
  jl.xcap = hoist_global_cap();
  jl.count_model = o.model ? 1u : 0u;
  return jl;
}

// Zeroing memset, filter, seeding and join of a staged chunk on the stream
// (also what a captured graph holds).  A profiled run brackets the filter and
// the join with events; under capture they become event-record nodes
// (cudaEventRecordExternal), recorded at every replay.
smg_status enqueue_chunk(smg_ctx *c, const DevGraph &g, Chunk &ch, const RunOpts &o, bool capturing) {
  const uint32_t nq = ch.b - ch.a;
  const unsigned ev_flags = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
  if (ch.zero_ranges) {
    smg_status z = launch_zero_ranges(c->arena.base, ch.zero_plan, ch.zero_plan + ch.zero_ranges + 1, ch.zero_ranges,
                                      c->stream, c->num_sms);
    if (z) return z;
  } else {
    SMG_CUDA(cudaMemsetAsync(c->arena.base, 0, ch.zero_bytes, c->stream));
  }
  if (o.profile) SMG_CUDA(cudaEventRecordWithFlags(c->ev[0], c->stream, ev_flags));
  smg_status s = launch_filter(g, ch.fq, nq, *c->fdev, walk_overflow(ch), c->stream, c->num_sms);
  if (s) return s;
  if (o.profile) SMG_CUDA(cudaEventRecordWithFlags(c->ev[1], c->stream, ev_flags));
  s = launch_join(make_join_launch(c, g, ch, o), c->stream, c->num_sms);
  if (s) return s;
  if (o.profile) SMG_CUDA(cudaEventRecordWithFlags(c->ev[2], c->stream, ev_flags));
  return SMG_OK;
}

smg_status run_chunk(smg_ctx *c, const DevGraph &g, const Plan *const *plans, Chunk &ch, const RunOpts &o,
                     QueryOut *out, RunStats *st, const std::vector<const void *> *key) {
  const uint32_t nq = ch.b - ch.a;
  const bool replay = key && c->graph_exec && c->graph_gen == c->run_gen && c->graph_key == *key;
  ++c->run_gen;
  if (replay) {
    SMG_CUDA(cudaGraphLaunch(c->graph_exec, c->stream));
    c->graph_gen = c->run_gen;
    st->launches += c->graph_launches;
  } else {
    smg_status s = stage_chunk(c, g, plans, ch, o);
    if (s) return s;
    st->h2d += c->fdev->host.size() + nq * (sizeof(FilterQuery) + sizeof(JoinQuery));
    uint64_t walk_launches = 0;
    for (uint32_t ng : c->fdev->phase_count)
      if (ng) walk_launches += 3;  // work list, walk, chunk pass
    const uint64_t launches = 2 * ((nq + 65534) / 65535) + walk_launches + 2 + (ch.zero_ranges ? 1 : 0);
    st->launches += launches;
    if (key) {
      drop_graph(c);
      cudaGraph_t graph = nullptr;
      SMG_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      s = enqueue_chunk(c, g, ch, o, true);
      cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
      if (s) {
        if (graph) cudaGraphDestroy(graph);
        return s;
      }
      if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
      e = cudaGraphInstantiate(&c->graph_exec, graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
      c->graph_key = *key;
      c->graph_launches = launches;
      SMG_CUDA(cudaGraphLaunch(c->graph_exec, c->stream));
      c->graph_gen = c->run_gen;
    } else {
      s = enqueue_chunk(c, g, ch, o, false);
      if (s) return s;
    }
  }
  st->d2h += nq * sizeof(QCounters) + sizeof(QueueState);
  QCounters *hc = static_cast<QCounters *>(c->pinned);
  QueueState *hq = reinterpret_cast<QueueState *>(static_cast<char *>(c->pinned) + al(nq * sizeof(QCounters)));
  SMG_CUDA(cudaMemcpyAsync(hc, ch.counters, nq * sizeof(QCounters), cudaMemcpyDeviceToHost, c->stream));
  SMG_CUDA(cudaMemcpyAsync(hq, ch.qs, sizeof(QueueState), cudaMemcpyDeviceToHost, c->stream));
  SMG_CUDA(cudaStreamSynchronize(c->stream));
  if (hq->error) {
    drop_graph(c);
    const char *why = hq->error == JOIN_ERR_DEADLINE       ? "join exceeded its time limit (SMG_TIME_LIMIT_S)"
                      : hq->error == JOIN_ERR_IDLE_TIMEOUT ? "join made no progress for too long"
                      : hq->error == JOIN_ERR_QUEUE_FULL   ? "join task queue full"
                                                           : "a queued task was never published";
    char msg[320];
    std::snprintf(msg, sizeof(msg), "%s; queue: head %llu tail %llu pending %llu tasks done %llu donations %llu "
                  "progress %llu full %d", why, hq->head.v, hq->tail.v, hq->pending.v, hq->tasks_done,
                  hq->donations, hq->progress.v, hq->full);
    return fail(hq->error == JOIN_ERR_QUEUE_FULL ? SMG_ERR_LIMIT : SMG_ERR_TIMEOUT, msg);
  }
  if (hq->pending.v != 0) return fail(SMG_ERR_INTERNAL, "join ended with pending tasks");
  for (uint32_t i = 0; i < nq; ++i) {
    QueryOut &q = out[ch.a + i];
    q.count = hc[i].count;
    q.limit_hit = hc[i].over;
    q.num_roots = hc[i].num_roots;
    q.cands = hc[i].stat[0];
    q.walk_entries = hc[i].stat[1];
    q.initial_cands = 0;
    for (uint32_t u = 0; u < plans[ch.a + i]->k; ++u) q.initial_cands += hc[i].cand_cnt[u];
    q.emb_written = ch.emb ? std::min<uint64_t>(hc[i].emb_count, o.emb_cap) : 0;
    q.overflow = ch.emb ? (hc[i].emb_count > o.emb_cap) : 0;
    // algorithmic bytes of the filter: each array touched once, 4 B per id or
    // word (the per-kernel units are itemised below)
    const Plan &P = *plans[ch.a + i];
    uint64_t lab = 0;
    std::vector<char> seen(kMaxLabels, 0);
    for (uint32_t u = 0; u < P.k; ++u)
      if (P.label[u] < g.label_count.size() && !seen[P.label[u]]) {
        seen[P.label[u]] = 1;
        lab += g.label_count[P.label[u]];
      }
    // masks cleared (4 B a vertex); per vertex of the query's labels: group
    // entry, degree, NLC row, mask write, then group entry and mask read in
    // collect; per candidate appended, per walked entry, per root
    st->filter_bytes += 4ull * g.n + lab * (4 + 4 + g.nlc_stride + 4 + 4 + 4) + 8ull * q.initial_cands +
                        8ull * q.walk_entries + 4ull * q.num_roots;
    // candidate bitmap rows written by collect: k id-indexed rows of n bits,
    // and with entry ranks k rank-indexed rows of the label's group size
    st->filter_bytes += static_cast<uint64_t>(P.k) * ((g.n + 31ull) / 32) * 4;
    if (g.adjr)
      for (uint32_t u = 0; u < P.k; ++u)
        if (P.label[u] < g.label_count.size()) st->filter_bytes += (g.label_count[P.label[u]] + 31) / 32 * 4;
  }
  st->tasks += hq->tasks_done;
  st->donations += hq->donations;
  st->bfs_tasks += hq->bfs_tasks;
  st->scanned += hq->scanned;
  st->descents += hq->descents;
  st->probes += hq->probes;
  st->last_count_entries += hq->last_count_entries;
  st->model_bytes += hq->model_bytes;
  st->join_bytes += 8ull * hq->scanned + 8ull * hq->descents + 4ull * hq->probes + 8ull * hq->last_count_entries;
  if (o.profile) {
    float f = 0, j = 0;
    SMG_CUDA(cudaEventElapsedTime(&f, c->ev[0], c->ev[1]));
    SMG_CUDA(cudaEventElapsedTime(&j, c->ev[1], c->ev[2]));
    st->filter_ms += f;
    st->join_ms += j;
  }
  if (ch.emb) {
    const uint64_t rows = out[ch.a].emb_written;
    if (rows) SMG_CUDA(cudaMemcpy(o.emb_host, ch.emb, rows * plans[ch.a]->k * 4, cudaMemcpyDeviceToHost));
    st->d2h += rows * plans[ch.a]->k * 4;
  }
  ++st->chunks;
  return SMG_OK;
}

}  // namespace

smg_status run_queries(smg_ctx *c, const DevGraph &g, const Plan *const *plans, uint32_t nq, const RunOpts &o,
                       QueryOut *out, RunStats *st) {
  SMG_CUDA(cudaSetDevice(c->device));
  if (o.emb_host && nq != 1) return fail(SMG_ERR_INVALID, "embeddings are returned by the plain path only");
  // queue storage of a chunk (bound) and the join warps' hoisted-set buffers
  const size_t per_chunk_fixed = (64ull << 20) * 4 + hoist_buffer_bytes(c->num_sms);
  // device memory is asked for only when the batch may not fit the arena
  // (cudaMemGetInfo is a driver round trip, too slow for every plain call)
  size_t need = per_chunk_fixed;
  for (uint32_t i = 0; i < nq && need <= c->arena.cap; ++i) {
    uint64_t ct;
    need += query_bytes(g, *plans[i], ct);
  }
  size_t budget = c->arena.cap;
  if (need > c->arena.cap) {
    size_t free_b = 0, total_b = 0;
    SMG_CUDA(cudaMemGetInfo(&free_b, &total_b));
    budget += free_b > kHeadroomBytes ? free_b - kHeadroomBytes : free_b / 2;
  }
  // SMG_MAX_BATCH_BYTES caps what one chunk may use (a chunk holds at least
  // one query whatever the cap)
  if (const char *cap = std::getenv("SMG_MAX_BATCH_BYTES")) {
    const unsigned long long v = std::strtoull(cap, nullptr, 10);
    if (v) budget = std::min<size_t>(budget, v);
  }
  const size_t max_q = kPinnedBytes / (sizeof(FilterQuery) + sizeof(JoinQuery) + sizeof(QCounters));
  uint32_t a = 0;
  while (a < nq) {
    uint32_t b = a;
    size_t used = per_chunk_fixed;
    while (b < nq && b - a < max_q) {
      uint64_t ct;
      const size_t qb = query_bytes(g, *plans[b], ct);
      if (b > a && used + qb > budget) break;
      used += qb;
      ++b;
    }
    Chunk ch;
    ch.a = a;
    ch.b = b;
    const size_t cap_before = c->arena.cap;
    smg_status s = layout_chunk(c, g, plans, ch, o);
    if (s) return s;
    if (c->arena.cap != cap_before) drop_graph(c);  // arena moved: captured pointers are stale
    std::vector<const void *> key;
    const bool whole = a == 0 && b == nq;
    if (o.use_graph && whole) {
      key.push_back(&g);
      key.push_back(reinterpret_cast<const void *>(static_cast<uintptr_t>(o.root_chunk)));
      key.push_back(reinterpret_cast<const void *>(static_cast<uintptr_t>(o.count_limit)));
      key.push_back(reinterpret_cast<const void *>(static_cast<uintptr_t>(o.work_limit)));
      key.push_back(reinterpret_cast<const void *>(static_cast<uintptr_t>(o.profile)));
      key.push_back(reinterpret_cast<const void *>(static_cast<uintptr_t>(o.model)));
      key.push_back(reinterpret_cast<const void *>(static_cast<uintptr_t>(o.bfs_depth)));
      for (uint32_t i = 0; i < nq; ++i) key.push_back(plans[i]);
    }
    s = run_chunk(c, g, plans, ch, o, out, st, key.empty() ? nullptr : &key);
    if (s) return s;
    a = b;
  }
  return SMG_OK;
}

}  // namespace smg

extern "C" {

smg_status smg_match(smg_ctx *c, const smg_graph *G, const smg_plan *p, const smg_match_opts *opts,
                     smg_match_result *out) {
  if (!c || !G || !p || !out) return fail(SMG_ERR_INVALID, "null argument");
  if (G->device != c->device) return fail(SMG_ERR_INVALID, "graph lives on another device");
  std::memset(out, 0, sizeof(*out));
  RunOpts o;
  o.tuning = c->tuning;
  if (opts) {
    o.profile = (opts->flags & SMG_FLAG_PROFILE) != 0;
    o.root_chunk = opts->root_chunk;
    o.bfs_depth = opts->bfs_depth;
    o.count_limit = opts->max_count;
    o.work_limit = opts->max_work;
    if (opts->flags & SMG_FLAG_EMIT) {
      if (!opts->embeddings && opts->max_embeddings) return fail(SMG_ERR_INVALID, "null embeddings buffer");
      o.emb_host = opts->embeddings;
      o.emb_cap = opts->max_embeddings;
    }
  }
  const Plan *pl = &p->p;
  QueryOut q;
  RunStats st;
  smg_status s = run_queries(c, G->g, &pl, 1, o, &q, &st);
  if (s) return s;
  out->count = q.count;
  out->embeddings_written = q.emb_written;
  out->overflow = q.overflow;
  out->num_candidates_root = q.num_roots;
  out->candidates_total = q.cands;
  out->filter_ms = st.filter_ms;
  out->join_ms = st.join_ms;
  out->tasks = st.tasks;
  out->filter_bytes = st.filter_bytes;
  out->join_bytes = st.join_bytes;
  out->limit_hit = q.limit_hit;
  return SMG_OK;
}

smg_status smg_match_batch(smg_ctx *c, const smg_graph *G, const smg_plan *const *plans, uint32_t n,
                           const smg_match_opts *opts, uint64_t *counts, smg_batch_stats *stats) {
  if (!c || !G || (n && (!plans || !counts))) return fail(SMG_ERR_INVALID, "null argument");
  if (G->device != c->device) return fail(SMG_ERR_INVALID, "graph lives on another device");
  if (opts && (opts->flags & SMG_FLAG_EMIT)) return fail(SMG_ERR_INVALID, "the batched path returns counts only");
  std::vector<const Plan *> pl(n);
  for (uint32_t i = 0; i < n; ++i) {
    if (!plans[i]) return fail(SMG_ERR_INVALID, "null plan in batch");
    pl[i] = &plans[i]->p;
  }
  RunOpts o;
  o.tuning = c->tuning;
  o.use_graph = true;
  if (opts) {
    o.profile = (opts->flags & SMG_FLAG_PROFILE) != 0;
    o.root_chunk = opts->root_chunk;
    o.bfs_depth = opts->bfs_depth;
    o.count_limit = opts->max_count;
    o.work_limit = opts->max_work;
    o.use_graph = (opts->flags & SMG_FLAG_NO_GRAPH) == 0;
    o.model = (opts->flags & SMG_FLAG_MODEL) != 0;
  }
  std::vector<QueryOut> q(n);
  RunStats st;
  smg_status s = run_queries(c, G->g, pl.data(), n, o, q.data(), &st);
  if (s) return s;
  uint64_t tot = 0;
  for (uint32_t i = 0; i < n; ++i) {
    counts[i] = q[i].limit_hit ? ~0ull : q[i].count;
    if (!q[i].limit_hit) tot += q[i].count;
  }
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->filter_ms = st.filter_ms;
    stats->join_ms = st.join_ms;
    stats->tasks = st.tasks;
    stats->total_embeddings = tot;
    stats->kernel_launches = st.launches;
    stats->h2d_bytes = st.h2d;
    stats->d2h_bytes = st.d2h;
    stats->filter_bytes = st.filter_bytes;
    stats->join_bytes = st.join_bytes;
    stats->chunks = st.chunks;
    stats->scanned = st.scanned;
    stats->descents = st.descents;
    stats->probes = st.probes;
    stats->last_count_entries = st.last_count_entries;
    stats->donations = st.donations;
    stats->bfs_tasks = st.bfs_tasks;
    stats->model_bytes = st.model_bytes;
  }
  return SMG_OK;
}

smg_status smg_filter_inspect(smg_ctx *c, const smg_graph *G, const smg_plan *p, uint32_t *vmask0,
                              uint32_t *encodings, uint32_t *candmask) {
  if (!c || !G || !p) return fail(SMG_ERR_INVALID, "null argument");
  SMG_CUDA(cudaSetDevice(c->device));
  const Plan *pl = &p->p;
  const DevGraph &g = G->g;
  RunOpts o;
  Chunk ch;
  ch.a = 0;
  ch.b = 1;
  smg_status s = layout_chunk(c, g, &pl, ch, o);
  if (s) return s;
  ++c->run_gen;  // invalidates a captured batch graph
  s = stage_chunk(c, g, &pl, ch, o);
  if (s) return s;
  // the filter keeps its masks and bitmap by position in the label groups;
  // the caller gets them by vertex id
  const size_t n = g.n, W = pl->num_words;
  std::vector<uint32_t> lv(std::max<size_t>(n, 1)), m0(vmask0 ? n : 0), enc(encodings ? n * W : 0),
      cm(candmask ? n : 0);
  SMG_CUDA(cudaMemsetAsync(c->arena.base, 0, ch.zero_bytes, c->stream));
  s = launch_nlc_filter(g, ch.fq, 1, c->stream, c->num_sms);
  if (s) return s;
  if (vmask0 && n)
    SMG_CUDA(cudaMemcpyAsync(m0.data(), ch.vmask[0], n * 4, cudaMemcpyDeviceToHost, c->stream));
  s = launch_walks(g, ch.fq, *c->fdev, walk_overflow(ch), c->stream, c->num_sms);
  if (s) return s;
  s = launch_collect(g, ch.fq, 1, c->stream, c->num_sms);
  if (s) return s;
  if (encodings && n) SMG_CUDA(cudaMemcpyAsync(enc.data(), ch.enc[0], n * W * 4, cudaMemcpyDeviceToHost, c->stream));
  if (candmask && n) SMG_CUDA(cudaMemcpyAsync(cm.data(), ch.vmask[0], n * 4, cudaMemcpyDeviceToHost, c->stream));
  if (n) SMG_CUDA(cudaMemcpyAsync(lv.data(), g.lverts, n * 4, cudaMemcpyDeviceToHost, c->stream));
  SMG_CUDA(cudaStreamSynchronize(c->stream));
  for (size_t q = 0; q < n; ++q) {
    const uint32_t v = lv[q];
    if (vmask0) vmask0[v] = m0[q];
    if (candmask) candmask[v] = cm[q];
    if (encodings) std::memcpy(encodings + static_cast<size_t>(v) * W, enc.data() + q * W, W * 4);
  }
  return SMG_OK;
}

}  // extern "C"

extern "C" {

uint32_t smg_plan_class(const smg_plan *p) { return p ? plan_class(p->p) : 0u; }

smg_status smg_set_tuning(smg_ctx *c, const smg_tune_entry *e, uint32_t n) {
  if (!c || (n && !e)) return fail(SMG_ERR_INVALID, "null argument");
  for (uint32_t i = 0; i < n; ++i) {
    if (e[i].shape_class >= SMG_TUNE_CLASSES) return fail(SMG_ERR_INVALID, "bad shape class");
    TuneSetting &t = c->tuning[e[i].shape_class];
    t.root_chunk = e[i].root_chunk;
    t.donate_min = e[i].donate_min;
    t.split_len = e[i].split_len;
    t.hoist_cap = e[i].hoist_cap;
    t.bfs_depth = e[i].bfs_depth;
    t.valid = e[i].samples > 0;
  }
  ++c->run_gen;  // the settings are staged into the query records: a captured batch is stale
  return SMG_OK;
}

smg_status smg_autotune(smg_ctx *c, const smg_graph *G, const smg_plan *const *plans, uint32_t n,
                        smg_tune_entry *out) {
  if (!c || !G || (n && !plans)) return fail(SMG_ERR_INVALID, "null argument");
  static const uint32_t kChunks[] = {1, 8, 64};
  static const uint32_t kDonate[] = {2, 33, 129};
  static const uint32_t kSplits[] = {8192, 2048, 32768};
  static const uint32_t kHoists[] = {4096, 1024, 256};
  static const uint32_t kBfs[] = {0, 2, 3};
  std::vector<std::vector<const Plan *>> by_class(SMG_TUNE_CLASSES);
  for (uint32_t i = 0; i < n; ++i)
    if (plans[i] && by_class[plan_class(plans[i]->p)].size() < 32) by_class[plan_class(plans[i]->p)].push_back(&plans[i]->p);
  for (uint32_t cls = 0; cls < SMG_TUNE_CLASSES; ++cls) {
    smg_tune_entry e{};
    e.shape_class = cls;
    const auto &sample = by_class[cls];
    if (!sample.empty()) {
      // device time of the sample under setting `cand` (second of two runs)
      auto time_of = [&](const TuneSetting &cand, float &ms) -> smg_status {
        TuneSetting t[SMG_TUNE_CLASSES];
        t[cls] = cand;
        t[cls].valid = true;
        RunOpts o;
        o.tuning = t;
        o.profile = true;
        std::vector<QueryOut> q(sample.size());
        for (int rep = 0; rep < 2; ++rep) {  // the first run warms the caches
          RunStats st;
          smg_status s = run_queries(c, G->g, sample.data(), static_cast<uint32_t>(sample.size()), o, q.data(), &st);
          if (s) return s;
          ms = st.filter_ms + st.join_ms;
        }
        return SMG_OK;
      };
      TuneSetting best;
      best.root_chunk = kChunks[0];
      best.donate_min = kDonate[0];
      best.split_len = kSplits[0];
      best.hoist_cap = kHoists[0];
      best.bfs_depth = kBfs[0];
      float best_ms = -1.f;
      // one knob group at a time, each from the best of the groups before
      for (int group = 0; group < 4; ++group) {
        std::vector<TuneSetting> cands;
        if (group == 0) {
          for (uint32_t rc : kChunks)
            for (uint32_t dm : kDonate) {
              TuneSetting t = best;
              t.root_chunk = rc;
              t.donate_min = dm;
              cands.push_back(t);
            }
        } else {
          const uint32_t *vals = group == 1 ? kSplits : group == 2 ? kHoists : kBfs;
          for (int vi = 0; vi < 3; ++vi) {
            TuneSetting t = best;
            (group == 1 ? t.split_len : group == 2 ? t.hoist_cap : t.bfs_depth) = vals[vi];
            cands.push_back(t);
          }
        }
        TuneSetting group_best = best;
        float group_ms = best_ms;
        for (size_t ci = 0; ci < cands.size(); ++ci) {
          if (group > 0 && ci == 0) continue;  // the incumbent, timed already
          float ms = 0.f;
          smg_status s = time_of(cands[ci], ms);
          if (s) return s;
          if (group == 0 && ci == 0) e.default_ms = ms;
          if (group_ms < 0 || ms < group_ms) {
            group_ms = ms;
            group_best = cands[ci];
          }
        }
        best = group_best;
        best_ms = group_ms;
      }
      e.root_chunk = best.root_chunk;
      e.donate_min = best.donate_min;
      e.split_len = best.split_len;
      e.hoist_cap = best.hoist_cap;
      e.bfs_depth = best.bfs_depth;
      e.samples = static_cast<uint32_t>(sample.size());
      e.best_ms = best_ms;
      TuneSetting &t = c->tuning[cls];
      t = best;
      t.valid = true;
    }
    if (out) out[cls] = e;
  }
  ++c->run_gen;
  return SMG_OK;
}

}  // extern "C"
