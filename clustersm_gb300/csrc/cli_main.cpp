// cli_main.cpp — drop-in replacement for the reference's ClusterSM binary.
//
//   ClusterSM -q <query.in> -d <data.in> [--gpu <int>=0]        (main.cu:26-34)
//   stdout, last line:  num_res: <count>                          (main.cu:172)
//
// The count is uint64 (the reference's is uint32 and wraps, defs.h:33).
// Extra options:  --emit <file>  write every embedding, sorted; --max-emit <rows>
//                 caps the rows kept (the count stays exact); --emit-format
//                 text (default: one embedding per line, k data-vertex ids in
//                 query-vertex order) or bin (the binary layout below).
//
// Binary embedding file (--emit-format bin), little-endian:
//   bytes  0..7   magic "SMGEMB01"
//          8..11  uint32 k (query vertices)
//         12..15  uint32 0 (reserved)
//         16..23  uint64 count: the exact number of embeddings
//         24..31  uint64 rows stored (min(count, --max-emit))
//         32..    rows x k uint32 data-vertex ids, row r = the embedding's
//                 image of query vertices 0..k-1, rows sorted lexicographically
// The reference prints only the count (main.cu:172); it never writes its
// result table out (main.cu:155-170).
// Exit status: 0; 106 for a missing required option (CLI11's RequiredError);
// otherwise the smg_status of the failing call (SMG_ERR_IO / SMG_ERR_FORMAT
// for unreadable or malformed files, where the reference exits with 1).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "smg.h"

namespace {

int usage(const char *argv0, int code) {
  std::fprintf(code ? stderr : stdout,
               "Usage: %s -q <query graph path> -d <data graph path> [--gpu <gpu number>]\n"
               "          [--emit <file>] [--max-emit <rows>] [--emit-format text|bin]\n",
               argv0);
  return code;
}

int die(const char *what, smg_status s) {
  std::fprintf(stderr, "Error: %s: %s (%s)\n", what, smg_strerror(s), smg_last_error());
  return static_cast<int>(s);
}

// little-endian store of the low `bytes` bytes of v
void put_le(unsigned char *p, uint64_t v, int bytes) {
  for (int i = 0; i < bytes; ++i) p[i] = static_cast<unsigned char>(v >> (8 * i));
}

bool take(int &i, int argc, char **argv, const char *name, std::string &val) {
  const size_t n = std::strlen(name);
  if (std::strcmp(argv[i], name) == 0) {
    if (i + 1 >= argc) return false;
    val = argv[++i];
    return true;
  }
  if (std::strncmp(argv[i], name, n) == 0 && argv[i][n] == '=') {
    val = argv[i] + n + 1;
    return true;
  }
  return false;
}

}  // namespace

int main(int argc, char **argv) {
  std::string qpath, dpath, gpu = "0", emit, max_emit = "100000000", emit_format = "text";
  for (int i = 1; i < argc; ++i) {
    if (!std::strcmp(argv[i], "-h") || !std::strcmp(argv[i], "--help")) return usage(argv[0], 0);
    if (take(i, argc, argv, "-q", qpath) || take(i, argc, argv, "-d", dpath) ||
        take(i, argc, argv, "--gpu", gpu) || take(i, argc, argv, "--emit", emit) ||
        take(i, argc, argv, "--max-emit", max_emit) || take(i, argc, argv, "--emit-format", emit_format))
      continue;
    std::fprintf(stderr, "The following argument was not expected: %s\n", argv[i]);
    return usage(argv[0], 109);
  }
  if (qpath.empty() || dpath.empty()) {
    std::fprintf(stderr, "%s is required\n", qpath.empty() ? "-q" : "-d");
    return usage(argv[0], 106);
  }
  if (emit_format != "text" && emit_format != "bin") {
    std::fprintf(stderr, "--emit-format: %s is not one of text, bin\n", emit_format.c_str());
    return 105;
  }
  char *endp = nullptr;
  const long dev = std::strtol(gpu.c_str(), &endp, 10);
  if (*endp || dev < 0) {
    std::fprintf(stderr, "--gpu: value %s is not a non-negative integer\n", gpu.c_str());
    return 105;
  }

  smg_host_query *hq = nullptr;
  smg_host_graph *hg = nullptr;
  smg_status s = smg_read_query(qpath.c_str(), &hq);
  if (s) return die("reading the query graph", s);
  s = smg_read_graph(dpath.c_str(), &hg);
  if (s) return die("reading the data graph", s);
  smg_query_desc qd;
  smg_csr csr;
  smg_host_query_view(hq, &qd);
  smg_host_graph_view(hg, &csr);
  smg_plan *plan = nullptr;
  s = smg_plan_create(&qd, &plan);
  if (s) return die("preparing the query", s);
  smg_ctx *ctx = nullptr;
  s = smg_open(static_cast<int>(dev), &ctx);
  if (s) return die("opening the device", s);
  smg_graph *g = nullptr;
  s = smg_graph_upload(ctx, &csr, &g);
  if (s) return die("uploading the data graph", s);

  smg_match_opts opts;
  std::memset(&opts, 0, sizeof(opts));
  std::vector<uint32_t> rows;
  const uint32_t k = qd.num_vertices;
  smg_match_result res;
  s = smg_match(ctx, g, plan, &opts, &res);
  if (s) return die("matching", s);
  if (!emit.empty()) {
    // a second pass writes the rows into a buffer sized by the exact count
    opts.flags = SMG_FLAG_EMIT;
    opts.max_embeddings = std::min<uint64_t>(res.count, std::strtoull(max_emit.c_str(), nullptr, 10));
    uint64_t n = 0;
    if (opts.max_embeddings) {
      rows.resize(opts.max_embeddings * k);
      opts.embeddings = rows.data();
      s = smg_match(ctx, g, plan, &opts, &res);
      if (s) return die("matching", s);
      n = res.embeddings_written;
    }
    std::vector<uint64_t> idx(n);
    for (uint64_t i = 0; i < n; ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](uint64_t a, uint64_t b) {
      return std::lexicographical_compare(rows.begin() + a * k, rows.begin() + a * k + k, rows.begin() + b * k,
                                          rows.begin() + b * k + k);
    });
    FILE *f = std::fopen(emit.c_str(), emit_format == "bin" ? "wb" : "w");
    if (!f) return die("opening the embedding file", SMG_ERR_IO);
    bool ok = true;
    if (emit_format == "bin") {
      unsigned char head[32] = {'S', 'M', 'G', 'E', 'M', 'B', '0', '1'};
      put_le(head + 8, k, 4);
      put_le(head + 16, res.count, 8);
      put_le(head + 24, n, 8);
      ok = std::fwrite(head, 1, sizeof(head), f) == sizeof(head);
      std::vector<unsigned char> buf(static_cast<size_t>(k) * 4);
      for (uint64_t i = 0; i < n && ok; ++i) {
        for (uint32_t j = 0; j < k; ++j) put_le(buf.data() + 4 * j, rows[idx[i] * k + j], 4);
        ok = std::fwrite(buf.data(), 1, buf.size(), f) == buf.size();
      }
    } else {
      for (uint64_t i = 0; i < n && ok; ++i)
        for (uint32_t j = 0; j < k; ++j)
          ok = std::fprintf(f, "%u%c", rows[idx[i] * k + j], j + 1 == k ? '\n' : ' ') > 0;
    }
    if (std::fclose(f) != 0 || !ok) return die("writing the embedding file", SMG_ERR_IO);
    if (res.overflow) std::fprintf(stderr, "warning: embeddings truncated to %llu rows\n",
                                   static_cast<unsigned long long>(n));
  }
  std::printf("num_res: %llu\n", static_cast<unsigned long long>(res.count));
  smg_graph_free(g);
  smg_close(ctx);
  smg_plan_free(plan);
  smg_host_graph_free(hg);
  smg_host_query_free(hq);
  return 0;
}
