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
#include <cstdlib>
#include <cstring>
#include <memory>
#include <numeric>

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

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

// A whole file in memory: mapped read-only where the system allows it, so
// that the parsing threads fault its pages in in parallel and nothing is
// copied; read into a buffer otherwise (empty files, pipes).
struct FileText {
  const char *p = nullptr;
  size_t n = 0;
  void *map = nullptr;
  std::vector<char> buf;
  FileText() = default;
  FileText(const FileText &) = delete;
  FileText &operator=(const FileText &) = delete;
  ~FileText() {
    if (map) munmap(map, n);
  }
};

smg_status slurp(const char *path, FileText &ft) {
  if (!path) return fail(SMG_ERR_INVALID, "null path");
  int fd = open(path, O_RDONLY);
  if (fd < 0) return fail(SMG_ERR_IO, std::string("Unable to open file ") + path);
  struct stat st;
  if (fstat(fd, &st) == 0 && S_ISREG(st.st_mode) && st.st_size > 0) {
    void *m = mmap(nullptr, static_cast<size_t>(st.st_size), PROT_READ, MAP_PRIVATE, fd, 0);
    if (m != MAP_FAILED) {
      close(fd);
      ft.map = m;
      ft.p = static_cast<const char *>(m);
      ft.n = static_cast<size_t>(st.st_size);
      return SMG_OK;
    }
  }
  close(fd);
  FILE *f = std::fopen(path, "rb");
  if (!f) return fail(SMG_ERR_IO, std::string("Unable to open file ") + path);
  char chunk[1 << 16];
  size_t got;
  while ((got = std::fread(chunk, 1, sizeof chunk, f)) > 0) ft.buf.insert(ft.buf.end(), chunk, chunk + got);
  const bool err = std::ferror(f) != 0;
  std::fclose(f);
  if (err) return fail(SMG_ERR_IO, std::string("short read on ") + path);
  ft.p = ft.buf.data();
  ft.n = ft.buf.size();
  return SMG_OK;
}

}  // namespace

namespace {

// One piece of the body of a .in file, parsed by one thread.  Vertex records
// are applied to the shared label/degree arrays directly (ids are distinct or
// the file is rejected); edges stay local until the pieces are joined in file
// order.
struct Piece {
  const char *b = nullptr, *e = nullptr;
  std::vector<uint32_t> edges;
  uint64_t nvert = 0;
  smg_status st = SMG_OK;
  std::string err;
};

bool is_letter(char c) { return (c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z'); }

// Pieces start at a line whose first character is a letter.  Letters only
// ever begin a record (every other token is a decimal number), so a piece
// boundary is a record boundary: a record cut short or run long at a boundary
// fails inside one piece exactly as it fails in a single pass.
std::vector<Piece> split_body(const char *b, const char *e, size_t want) {
  std::vector<Piece> pieces;
  const size_t len = static_cast<size_t>(e - b);
  // smallest piece worth a thread (SMG_IO_PIECE_BYTES, default 1 MiB)
  size_t min_piece = 1 << 20;
  if (const char *env = std::getenv("SMG_IO_PIECE_BYTES")) {
    const long long v = std::atoll(env);
    if (v > 0) min_piece = static_cast<size_t>(v);
  }
  size_t np = std::max<size_t>(1, std::min(want, len / min_piece));
  const char *at = b;
  for (size_t i = 1; i <= np; ++i) {
    const char *q = i == np ? e : b + len / np * i;
    if (q < at) q = at;
    while (q < e && !(q > b && q[-1] == '\n' && is_letter(*q))) ++q;
    if (q > at || i == np) {
      Piece p;
      p.b = at;
      p.e = q;
      pieces.push_back(std::move(p));
      at = q;
    }
  }
  return pieces;
}

void parse_piece(Piece &pc, uint32_t n, uint32_t *label, uint32_t *deg, uint8_t *seen) {
  Reader r{pc.b, pc.e};
  char c;
  auto bad = [&](const std::string &msg) {
    pc.st = SMG_ERR_FORMAT;
    pc.err = msg;
  };
  pc.edges.reserve(static_cast<size_t>(pc.e - pc.b) / 6);
  while (r.type(c)) {
    if (c == 'e') {
      uint64_t a, b;
      if (!r.u64(a) || !r.u64(b)) return bad("bad 'e' line");
      if (a >= n || b >= n) return bad("edge endpoint out of range");
      if (a == b) return bad("self-loop in edge list");
      pc.edges.push_back(static_cast<uint32_t>(a));
      pc.edges.push_back(static_cast<uint32_t>(b));
    } else if (c == 'v') {
      uint64_t id, l, d;
      if (!r.u64(id) || !r.u64(l) || !r.u64(d)) return bad("bad 'v' line");
      if (id >= n) return bad("vertex id out of range in 'v' line");
      if (l > 0xFFFFFFFEull || d > 0xFFFFFFFFull) return bad("label/degree too large");
      if (__atomic_exchange_n(&seen[id], static_cast<uint8_t>(1), __ATOMIC_RELAXED))
        return bad("vertex declared twice");
      label[id] = static_cast<uint32_t>(l);
      deg[id] = static_cast<uint32_t>(d);
      ++pc.nvert;
    } else {
      return bad(std::string("unexpected line type '") + c + "'");
    }
  }
}

int num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // namespace

std::vector<uint32_t> count_degrees(uint32_t n, const RawU32 &edges) {
  std::vector<uint32_t> cnt(n, 0);
  uint32_t *c = cnt.data();
  const int64_t m2 = static_cast<int64_t>(edges.size());
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < m2; ++i) __atomic_fetch_add(&c[edges[i]], 1u, __ATOMIC_RELAXED);
  return cnt;
}

smg_status read_in_file(const char *path, uint32_t &n, std::vector<uint32_t> &label,
                        std::vector<uint32_t> &deg, RawU32 &edges) {
  FileText ft;
  smg_status s = slurp(path, ft);
  if (s) return s;
  Reader r{ft.p, ft.p + ft.n};
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
  // the body is parsed in pieces, one per thread task; the first failing
  // piece in file order gives the error
  std::vector<Piece> pieces = split_body(r.p, r.end, static_cast<size_t>(num_threads()) * 4);
  const int64_t np = static_cast<int64_t>(pieces.size());
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t i = 0; i < np; ++i) parse_piece(pieces[i], n, label.data(), deg.data(), seen.data());
  uint64_t nvert = 0, nent = 0;
  std::vector<uint64_t> at(pieces.size() + 1, 0);
  for (size_t i = 0; i < pieces.size(); ++i) {
    if (pieces[i].st) return fail(pieces[i].st, pieces[i].err);
    nvert += pieces[i].nvert;
    at[i + 1] = at[i] + pieces[i].edges.size();
  }
  nent = at.back();
  if (nvert != n) return fail(SMG_ERR_FORMAT, "not every vertex has a 'v' line");
  if (nent / 2 != ne) return fail(SMG_ERR_FORMAT, "edge count differs from the 't' line");
  edges.resize(nent);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t i = 0; i < np; ++i) {
    if (!pieces[i].edges.empty())
      std::memcpy(edges.data() + at[i], pieces[i].edges.data(), pieces[i].edges.size() * sizeof(uint32_t));
    std::vector<uint32_t>().swap(pieces[i].edges);
  }
  // declared degrees must agree with the edges (io.cu:75 builds offsets from them)
  std::vector<uint32_t> cnt = count_degrees(n, edges);
  int64_t first_bad = -1;
  for (uint32_t v = 0; v < n && first_bad < 0; ++v)
    if (cnt[v] != deg[v]) first_bad = v;
  if (first_bad >= 0)
    return fail(SMG_ERR_FORMAT, "declared degree differs from the edge list at vertex " + std::to_string(first_bad));
  return SMG_OK;
}

smg_status csr_from_edges(uint32_t n, const RawU32 &edges, bool sort_lists,
                          HostGraph &g, const std::vector<uint32_t> *degrees) {
  g.n = n;
  g.m = edges.size() / 2;
  const uint64_t m2 = edges.size();
  std::vector<uint32_t> counted;
  if (!degrees) {
    counted = count_degrees(n, edges);
    degrees = &counted;
  }
  g.off.assign(static_cast<size_t>(n) + 1, 0);
  for (uint32_t v = 0; v < n; ++v) g.off[v + 1] = g.off[v] + (*degrees)[v];
  if (g.off[n] != m2) return fail(SMG_ERR_INVALID, "degree counts do not match the edge list");
  g.adj.resize(m2);
  // Stable parallel scatter.  Vertices are split into R ranges of about equal
  // adjacency; edge pairs into P pieces in file order.  Pass 1 counts each
  // piece's entries per range, pass 2 moves them into range-major,
  // piece-minor order, and pass 3 has one thread per range fill its vertices'
  // lists.  Every list therefore receives its entries in file order, as the
  // sequential fill of io.cu:86-93 does.
  const uint64_t pairs = g.m;
  const int T = num_threads();
  const size_t R = static_cast<size_t>(std::max(1, std::min(T * 2, 250)));
  const size_t P = static_cast<size_t>(std::max(1, T * 2));
  // lists shorter in total than SMG_IO_SCATTER_MIN entries (default 2^20)
  // are filled by one thread
  uint64_t scatter_min = 1u << 20;
  if (const char *env = std::getenv("SMG_IO_SCATTER_MIN")) scatter_min = std::strtoull(env, nullptr, 10);
  if (m2 < scatter_min || R == 1) {
    std::vector<uint64_t> cur(g.off.begin(), g.off.end() - 1);
    for (uint64_t i = 0; i < pairs; ++i) {
      uint32_t a = edges[2 * i], b = edges[2 * i + 1];
      g.adj[cur[a]++] = b;
      g.adj[cur[b]++] = a;
    }
  } else {
    std::vector<uint32_t> rstart(R + 1, n);
    rstart[0] = 0;
    for (size_t r = 1; r < R; ++r)
      rstart[r] = static_cast<uint32_t>(std::lower_bound(g.off.begin(), g.off.end() - 1, m2 / R * r) - g.off.begin());
    std::vector<uint8_t> range_of(n);
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < static_cast<int64_t>(R); ++r)
      std::fill(range_of.begin() + rstart[r], range_of.begin() + rstart[r + 1], static_cast<uint8_t>(r));
    std::vector<uint64_t> cnt(P * R, 0);  // [piece][range]
    auto piece_lo = [&](size_t p) { return pairs / P * p + std::min<uint64_t>(p, pairs % P); };
#pragma omp parallel for schedule(static, 1)
    for (int64_t p = 0; p < static_cast<int64_t>(P); ++p) {
      uint64_t *c = &cnt[static_cast<size_t>(p) * R];
      for (uint64_t i = piece_lo(p); i < piece_lo(p + 1); ++i) {
        ++c[range_of[edges[2 * i]]];
        ++c[range_of[edges[2 * i + 1]]];
      }
    }
    std::vector<uint64_t> pos(P * R), rbeg(R + 1, 0);
    uint64_t at = 0;
    for (size_t r = 0; r < R; ++r) {
      rbeg[r] = at;
      for (size_t p = 0; p < P; ++p) {
        pos[p * R + r] = at;
        at += cnt[p * R + r];
      }
    }
    rbeg[R] = at;
    RawU32 src(m2), dst(m2);
#pragma omp parallel for schedule(static, 1)
    for (int64_t p = 0; p < static_cast<int64_t>(P); ++p) {
      uint64_t *q = &pos[static_cast<size_t>(p) * R];
      for (uint64_t i = piece_lo(p); i < piece_lo(p + 1); ++i) {
        const uint32_t a = edges[2 * i], b = edges[2 * i + 1];
        uint64_t &qa = q[range_of[a]];
        src[qa] = a;
        dst[qa++] = b;
        uint64_t &qb = q[range_of[b]];
        src[qb] = b;
        dst[qb++] = a;
      }
    }
    std::vector<uint64_t> cur(g.off.begin(), g.off.end() - 1);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t r = 0; r < static_cast<int64_t>(R); ++r)
      for (uint64_t k = rbeg[r]; k < rbeg[r + 1]; ++k) g.adj[cur[src[k]]++] = dst[k];
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
  std::vector<uint32_t> label, deg;
  RawU32 edges;
  smg_status s = read_in_file(path, n, label, deg, edges);
  if (s) return s;
  std::unique_ptr<smg_host_graph> h(new smg_host_graph);
  s = csr_from_edges(n, edges, false, h->g, &deg);
  if (s) return s;
  RawU32().swap(edges);
  h->g.label = std::move(label);
  // repeated edges are checked on a sorted copy so that file order is kept
  {
    RawU32 tmp(h->g.adj.size());
    bool dup = false;
#pragma omp parallel for schedule(dynamic, 4096) reduction(|| : dup)
    for (int64_t v = 0; v < static_cast<int64_t>(n); ++v) {
      auto b = tmp.begin() + static_cast<int64_t>(h->g.off[v]);
      auto e = tmp.begin() + static_cast<int64_t>(h->g.off[v + 1]);
      std::copy(h->g.adj.begin() + static_cast<int64_t>(h->g.off[v]),
                h->g.adj.begin() + static_cast<int64_t>(h->g.off[v + 1]), b);
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
  std::vector<uint32_t> label, deg;
  RawU32 edges;
  smg_status s = read_in_file(path, n, label, deg, edges);
  if (s) return s;
  std::unique_ptr<smg_host_query> h(new smg_host_query);
  h->q.n = n;
  h->q.label = std::move(label);
  h->q.edges.assign(edges.begin(), edges.end());
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
