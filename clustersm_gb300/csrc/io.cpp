// io.cpp — status strings, .in reading/writing, host graph objects.
//
// The .in dialect is the one readGraphToCPU2 parses (io.cu:24-108):
//   t <n> <m>
//   v <id> <label> <deg>      one per vertex
//   e <a> <b>                 once per undirected edge
// Neighbour lists are filled in edge order (io.cu:86-93), so a vertex's list
// keeps the order in which its edges appear in the file.  Unlike the
// reference, malformed input is reported as a status instead of exit(1), and
// declared degrees, ids, self-loops and repeated edges are checked because the
// reference would write out of bounds or build a multigraph on them.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <memory>
#include <numeric>

#include "host.h"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace smg {

static thread_local std::string g_last_error;

smg_status fail(smg_status s, const std::string &msg) {
  g_last_error = msg;
  return s;
}

namespace {

struct Reader {
  const char *p, *end;
  void skip() {
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n')) ++p;
  }
  bool type(char &c) {
    skip();
    if (p >= end) return false;
    c = *p++;
    return true;
  }
  bool u64(uint64_t &v) {
    skip();
    if (p >= end || *p < '0' || *p > '9') return false;
    uint64_t x = 0;
    while (p < end && *p >= '0' && *p <= '9') {
      uint64_t nx = x * 10 + static_cast<uint64_t>(*p - '0');
      if (nx < x) return false;
      x = nx;
      ++p;
    }
    v = x;
    return true;
  }
};

smg_status slurp(const char *path, std::vector<char> &buf) {
  if (!path) return fail(SMG_ERR_INVALID, "null path");
  FILE *f = std::fopen(path, "rb");
  if (!f) return fail(SMG_ERR_IO, std::string("Unable to open file ") + path);
  std::fseek(f, 0, SEEK_END);
  long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if (sz < 0) {
    std::fclose(f);
    return fail(SMG_ERR_IO, std::string("cannot size file ") + path);
  }
  buf.resize(static_cast<size_t>(sz));
  size_t got = sz ? std::fread(buf.data(), 1, static_cast<size_t>(sz), f) : 0;
  std::fclose(f);
  if (got != static_cast<size_t>(sz)) return fail(SMG_ERR_IO, std::string("short read on ") + path);
  return SMG_OK;
}

}  // namespace

smg_status read_in_file(const char *path, uint32_t &n, std::vector<uint32_t> &label,
                        std::vector<uint32_t> &deg, std::vector<uint32_t> &edges) {
  std::vector<char> buf;
  smg_status s = slurp(path, buf);
  if (s) return s;
  Reader r{buf.data(), buf.data() + buf.size()};
  char c;
  uint64_t nv, ne;
  if (!r.type(c) || c != 't')
    return fail(SMG_ERR_FORMAT, std::string("Expected 't' at the beginning of ") + path);
  if (!r.u64(nv) || !r.u64(ne)) return fail(SMG_ERR_FORMAT, "bad 't' line");
  if (nv > 0xFFFFFFFEull) return fail(SMG_ERR_LIMIT, "more than 2^32-2 vertices");
  n = static_cast<uint32_t>(nv);
  label.assign(n, 0);
  deg.assign(n, 0);
  std::vector<uint8_t> seen(n, 0);
  edges.clear();
  edges.reserve(static_cast<size_t>(ne) * 2);
  uint64_t nvert = 0;
  while (r.type(c)) {
    if (c == 'v') {
      uint64_t id, l, d;
      if (!r.u64(id) || !r.u64(l) || !r.u64(d)) return fail(SMG_ERR_FORMAT, "bad 'v' line");
      if (id >= n) return fail(SMG_ERR_FORMAT, "vertex id out of range in 'v' line");
      if (seen[id]) return fail(SMG_ERR_FORMAT, "vertex declared twice");
      if (l > 0xFFFFFFFEull || d > 0xFFFFFFFFull) return fail(SMG_ERR_FORMAT, "label/degree too large");
      seen[id] = 1;
      label[id] = static_cast<uint32_t>(l);
      deg[id] = static_cast<uint32_t>(d);
      ++nvert;
    } else if (c == 'e') {
      uint64_t a, b;
      if (!r.u64(a) || !r.u64(b)) return fail(SMG_ERR_FORMAT, "bad 'e' line");
      if (a >= n || b >= n) return fail(SMG_ERR_FORMAT, "edge endpoint out of range");
      if (a == b) return fail(SMG_ERR_FORMAT, "self-loop in edge list");
      edges.push_back(static_cast<uint32_t>(a));
      edges.push_back(static_cast<uint32_t>(b));
    } else {
      return fail(SMG_ERR_FORMAT, std::string("unexpected line type '") + c + "'");
    }
  }
  if (nvert != n) return fail(SMG_ERR_FORMAT, "not every vertex has a 'v' line");
  if (edges.size() / 2 != ne) return fail(SMG_ERR_FORMAT, "edge count differs from the 't' line");
  // declared degrees must agree with the edges (io.cu:75 builds offsets from them)
  std::vector<uint32_t> cnt(n, 0);
  for (size_t i = 0; i < edges.size(); ++i) ++cnt[edges[i]];
  for (uint32_t v = 0; v < n; ++v)
    if (cnt[v] != deg[v]) return fail(SMG_ERR_FORMAT, "declared degree differs from the edge list at vertex " + std::to_string(v));
  return SMG_OK;
}

smg_status csr_from_edges(uint32_t n, const std::vector<uint32_t> &edges, bool sort_lists,
                          HostGraph &g) {
  g.n = n;
  g.m = edges.size() / 2;
  g.off.assign(static_cast<size_t>(n) + 1, 0);
  for (uint32_t x : edges) ++g.off[x + 1];
  for (uint32_t v = 0; v < n; ++v) g.off[v + 1] += g.off[v];
  g.adj.resize(edges.size());
  std::vector<uint64_t> cur(g.off.begin(), g.off.end() - 1);
  for (size_t i = 0; i + 1 < edges.size(); i += 2) {
    uint32_t a = edges[i], b = edges[i + 1];
    g.adj[cur[a]++] = b;
    g.adj[cur[b]++] = a;
  }
  if (sort_lists) {
    bool dup = false;
#pragma omp parallel for schedule(dynamic, 4096) reduction(|| : dup)
    for (int64_t v = 0; v < static_cast<int64_t>(n); ++v) {
      auto b = g.adj.begin() + static_cast<int64_t>(g.off[v]);
      auto e = g.adj.begin() + static_cast<int64_t>(g.off[v + 1]);
      std::sort(b, e);
      if (std::adjacent_find(b, e) != e) dup = true;
    }
    if (dup) return fail(SMG_ERR_FORMAT, "repeated edge in the edge list");
  }
  return SMG_OK;
}

}  // namespace smg

using namespace smg;

extern "C" {

const char *smg_strerror(smg_status s) {
  switch (s) {
    case SMG_OK: return "ok";
    case SMG_ERR_INVALID: return "invalid argument";
    case SMG_ERR_IO: return "i/o error";
    case SMG_ERR_FORMAT: return "malformed graph file";
    case SMG_ERR_QUERY: return "unsupported query graph";
    case SMG_ERR_LIMIT: return "size limit exceeded";
    case SMG_ERR_CUDA: return "CUDA error";
    case SMG_ERR_OOM: return "out of memory";
    case SMG_ERR_TIMEOUT: return "device wait timed out";
    case SMG_ERR_NO_DEVICE: return "no CUDA device";
    case SMG_ERR_BUDGET: return "memory budget exceeded";
    case SMG_ERR_CANCELLED: return "cancelled";
    case SMG_ERR_NOT_READY: return "not ready";
    case SMG_ERR_INTERNAL: return "internal error";
    default: return "unknown status";
  }
}

const char *smg_last_error(void) { return smg::g_last_error.c_str(); }

smg_status smg_read_graph(const char *path, smg_host_graph **out) {
  if (!out) return fail(SMG_ERR_INVALID, "null out");
  *out = nullptr;
  uint32_t n;
  std::vector<uint32_t> label, deg, edges;
  smg_status s = read_in_file(path, n, label, deg, edges);
  if (s) return s;
  std::unique_ptr<smg_host_graph> h(new smg_host_graph);
  s = csr_from_edges(n, edges, false, h->g);
  if (s) return s;
  h->g.label = std::move(label);
  // repeated edges are checked on a sorted copy so that file order is kept
  {
    std::vector<uint32_t> tmp(h->g.adj);
    bool dup = false;
#pragma omp parallel for schedule(dynamic, 4096) reduction(|| : dup)
    for (int64_t v = 0; v < static_cast<int64_t>(n); ++v) {
      auto b = tmp.begin() + static_cast<int64_t>(h->g.off[v]);
      auto e = tmp.begin() + static_cast<int64_t>(h->g.off[v + 1]);
      std::sort(b, e);
      if (std::adjacent_find(b, e) != e) dup = true;
    }
    if (dup) return fail(SMG_ERR_FORMAT, "repeated edge in the edge list");
  }
  *out = h.release();
  return SMG_OK;
}

smg_status smg_read_query(const char *path, smg_host_query **out) {
  if (!out) return fail(SMG_ERR_INVALID, "null out");
  *out = nullptr;
  uint32_t n;
  std::vector<uint32_t> label, deg, edges;
  smg_status s = read_in_file(path, n, label, deg, edges);
  if (s) return s;
  std::unique_ptr<smg_host_query> h(new smg_host_query);
  h->q.n = n;
  h->q.label = std::move(label);
  h->q.edges = std::move(edges);
  *out = h.release();
  return SMG_OK;
}

static void put_u64(std::string &s, uint64_t v) {
  char tmp[24];
  int i = 0;
  do {
    tmp[i++] = static_cast<char>('0' + v % 10);
    v /= 10;
  } while (v);
  while (i) s.push_back(tmp[--i]);
}

static smg_status write_all(const char *path, const std::string &s) {
  FILE *f = std::fopen(path, "wb");
  if (!f) return fail(SMG_ERR_IO, std::string("cannot open ") + path + " for writing");
  size_t w = std::fwrite(s.data(), 1, s.size(), f);
  int c = std::fclose(f);
  if (w != s.size() || c != 0) return fail(SMG_ERR_IO, std::string("short write on ") + path);
  return SMG_OK;
}

smg_status smg_write_graph(const char *path, const smg_csr *g) {
  if (!path || !g || (!g->offsets && g->num_vertices)) return fail(SMG_ERR_INVALID, "null argument");
  std::string s;
  s.reserve(static_cast<size_t>(g->num_vertices) * 16 + static_cast<size_t>(g->num_edges) * 20 + 32);
  s += "t ";
  put_u64(s, g->num_vertices);
  s += ' ';
  put_u64(s, g->num_edges);
  s += '\n';
  for (uint32_t v = 0; v < g->num_vertices; ++v) {
    s += "v ";
    put_u64(s, v);
    s += ' ';
    put_u64(s, g->labels[v]);
    s += ' ';
    put_u64(s, g->offsets[v + 1] - g->offsets[v]);
    s += '\n';
  }
  uint64_t written = 0;
  for (uint32_t v = 0; v < g->num_vertices; ++v)
    for (uint64_t e = g->offsets[v]; e < g->offsets[v + 1]; ++e)
      if (g->neighbors[e] > v) {
        s += "e ";
        put_u64(s, v);
        s += ' ';
        put_u64(s, g->neighbors[e]);
        s += '\n';
        ++written;
      }
  if (written != g->num_edges) return fail(SMG_ERR_INVALID, "CSR is not symmetric");
  return write_all(path, s);
}

smg_status smg_write_query(const char *path, const smg_query_desc *q) {
  if (!path || !q) return fail(SMG_ERR_INVALID, "null argument");
  std::vector<uint32_t> deg(q->num_vertices, 0);
  for (uint32_t i = 0; i < 2 * q->num_edges; ++i) {
    if (q->edges[i] >= q->num_vertices) return fail(SMG_ERR_INVALID, "edge endpoint out of range");
    ++deg[q->edges[i]];
  }
  std::string s = "t ";
  put_u64(s, q->num_vertices);
  s += ' ';
  put_u64(s, q->num_edges);
  s += '\n';
  for (uint32_t v = 0; v < q->num_vertices; ++v) {
    s += "v ";
    put_u64(s, v);
    s += ' ';
    put_u64(s, q->labels[v]);
    s += ' ';
    put_u64(s, deg[v]);
    s += '\n';
  }
  for (uint32_t i = 0; i < q->num_edges; ++i) {
    s += "e ";
    put_u64(s, q->edges[2 * i]);
    s += ' ';
    put_u64(s, q->edges[2 * i + 1]);
    s += '\n';
  }
  return write_all(path, s);
}

smg_status smg_host_graph_view(const smg_host_graph *g, smg_csr *out) {
  if (!g || !out) return fail(SMG_ERR_INVALID, "null argument");
  *out = g->g.view();
  return SMG_OK;
}

smg_status smg_host_query_view(const smg_host_query *q, smg_query_desc *out) {
  if (!q || !out) return fail(SMG_ERR_INVALID, "null argument");
  *out = q->q.view();
  return SMG_OK;
}

smg_status smg_host_graph_from_csr(const smg_csr *in, smg_host_graph **out) {
  if (!in || !out) return fail(SMG_ERR_INVALID, "null argument");
  *out = nullptr;
  const uint32_t n = in->num_vertices;
  if (n && (!in->offsets || !in->labels)) return fail(SMG_ERR_INVALID, "null arrays");
  if (in->offsets[0] != 0 || in->offsets[n] != 2 * in->num_edges)
    return fail(SMG_ERR_INVALID, "offsets do not span 2*num_edges");
  std::unique_ptr<smg_host_graph> h(new smg_host_graph);
  HostGraph &g = h->g;
  g.n = n;
  g.m = in->num_edges;
  g.off.assign(in->offsets, in->offsets + n + 1);
  g.adj.assign(in->neighbors, in->neighbors + 2 * in->num_edges);
  g.label.assign(in->labels, in->labels + n);
  bool bad = false;
#pragma omp parallel for schedule(dynamic, 4096) reduction(|| : bad)
  for (int64_t v = 0; v < static_cast<int64_t>(n); ++v) {
    if (g.off[v] > g.off[v + 1]) {
      bad = true;
      continue;
    }
    auto b = g.adj.begin() + static_cast<int64_t>(g.off[v]);
    auto e = g.adj.begin() + static_cast<int64_t>(g.off[v + 1]);
    std::sort(b, e);
    if (std::adjacent_find(b, e) != e) bad = true;
    for (auto it = b; it != e; ++it)
      if (*it >= n || *it == static_cast<uint32_t>(v)) bad = true;
  }
  if (bad) return fail(SMG_ERR_INVALID, "CSR has out-of-range ids, self-loops or repeated edges");
  // symmetry: every (v,w) has (w,v)
#pragma omp parallel for schedule(dynamic, 4096) reduction(|| : bad)
  for (int64_t v = 0; v < static_cast<int64_t>(n); ++v)
    for (uint64_t e = g.off[v]; e < g.off[v + 1]; ++e) {
      uint32_t w = g.adj[e];
      auto b = g.adj.begin() + static_cast<int64_t>(g.off[w]);
      auto en = g.adj.begin() + static_cast<int64_t>(g.off[w + 1]);
      if (!std::binary_search(b, en, static_cast<uint32_t>(v))) bad = true;
    }
  if (bad) return fail(SMG_ERR_INVALID, "CSR is not symmetric");
  *out = h.release();
  return SMG_OK;
}

void smg_host_graph_free(smg_host_graph *g) { delete g; }
void smg_host_query_free(smg_host_query *q) { delete q; }

}  // extern "C"
