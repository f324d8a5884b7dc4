// cli_main.cpp — drop-in replacement for the reference's ClusterSM binary.
//
//   ClusterSM -q <query.in> -d <data.in> [--gpu <int>=0]        (main.cu:26-34)
//   stdout, last line:  num_res: <count>                          (main.cu:172)
//
// The count is uint64 (the reference's is uint32 and wraps, defs.h:33).
// Extra options:  --emit <file>  write every embedding, sorted, one per line
//                 (k data-vertex ids in query-vertex order); --max-emit <rows>
//                 caps the rows kept (the count stays exact).
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
               "          [--emit <file>] [--max-emit <rows>]\n",
               argv0);
  return code;
}

int die(const char *what, smg_status s) {
  std::fprintf(stderr, "Error: %s: %s (%s)\n", what, smg_strerror(s), smg_last_error());
  return static_cast<int>(s);
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
  std::string qpath, dpath, gpu = "0", emit, max_emit = "100000000";
  for (int i = 1; i < argc; ++i) {
    if (!std::strcmp(argv[i], "-h") || !std::strcmp(argv[i], "--help")) return usage(argv[0], 0);
    if (take(i, argc, argv, "-q", qpath) || take(i, argc, argv, "-d", dpath) ||
        take(i, argc, argv, "--gpu", gpu) || take(i, argc, argv, "--emit", emit) ||
        take(i, argc, argv, "--max-emit", max_emit))
      continue;
    std::fprintf(stderr, "The following argument was not expected: %s\n", argv[i]);
    return usage(argv[0], 109);
  }
  if (qpath.empty() || dpath.empty()) {
    std::fprintf(stderr, "%s is required\n", qpath.empty() ? "-q" : "-d");
    return usage(argv[0], 106);
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
  if (!emit.empty()) {
    opts.flags = SMG_FLAG_EMIT;
    opts.max_embeddings = std::strtoull(max_emit.c_str(), nullptr, 10);
    rows.resize(opts.max_embeddings * k);
    opts.embeddings = rows.data();
  }
  smg_match_result res;
  s = smg_match(ctx, g, plan, &opts, &res);
  if (s) return die("matching", s);
  if (!emit.empty()) {
    const uint64_t n = res.embeddings_written;
    std::vector<uint64_t> idx(n);
    for (uint64_t i = 0; i < n; ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](uint64_t a, uint64_t b) {
      return std::lexicographical_compare(rows.begin() + a * k, rows.begin() + a * k + k, rows.begin() + b * k,
                                          rows.begin() + b * k + k);
    });
    FILE *f = std::fopen(emit.c_str(), "w");
    if (!f) return die("opening the embedding file", SMG_ERR_IO);
    for (uint64_t i = 0; i < n; ++i)
      for (uint32_t j = 0; j < k; ++j) std::fprintf(f, "%u%c", rows[idx[i] * k + j], j + 1 == k ? '\n' : ' ');
    std::fclose(f);
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
