// serve.cpp — request loop over a resident data graph.
//
// The reference has no serving mode: runClusterSM.sh starts one process per
// query and re-reads the data graph each time (runClusterSM.sh:9-13).  Here
// requests are queued, admitted against a device-memory budget estimated from
// each query's filter footprint, and run together as one batch (one filter
// pass and one persistent join launch for the admitted set).
#include <chrono>
#include <deque>
#include <map>
#include <memory>

#include "api_internal.cuh"

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Request {
  uint64_t ticket;
  const smg::Plan *plan;
  double submit_s;
  uint64_t bytes;
};

}  // namespace

struct smg_server {
  smg_ctx *ctx = nullptr;
  const smg_graph *graph = nullptr;
  smg_server_config cfg{};
  uint64_t next_ticket = 1;
  std::deque<Request> queue;
  std::map<uint64_t, smg_request_result> done;
};

namespace {

uint64_t footprint(const smg::DevGraph &g, const smg::Plan &P) {
  uint64_t cand = 0;
  for (uint32_t u = 0; u < P.k; ++u) cand += P.label[u] < g.label_count.size() ? g.label_count[P.label[u]] : 0;
  return static_cast<uint64_t>(g.n) * 4 * (1 + P.num_words) + cand * 8 + 4096;
}

smg_status run_admitted(smg_server *s) {
  if (s->queue.empty()) return SMG_OK;
  std::vector<Request> batch;
  uint64_t used = 0;
  while (!s->queue.empty() && batch.size() < s->cfg.max_inflight) {
    const Request &r = s->queue.front();
    if (!batch.empty() && used + r.bytes > s->cfg.memory_budget_bytes) break;
    used += r.bytes;
    batch.push_back(r);
    s->queue.pop_front();
  }
  const double start = now_s();
  std::vector<const smg::Plan *> plans;
  for (auto &r : batch) plans.push_back(r.plan);
  std::vector<smg::QueryOut> out(batch.size());
  smg::RunStats st;
  smg::RunOpts o;
  smg_status rc = smg::run_queries(s->ctx, s->graph->g, plans.data(), static_cast<uint32_t>(plans.size()), o,
                                   out.data(), &st);
  const double fin = now_s();
  for (size_t i = 0; i < batch.size(); ++i) {
    smg_request_result res{};
    res.status = rc;
    res.count = rc ? 0 : out[i].count;
    res.submit_s = batch[i].submit_s;
    res.start_s = start;
    res.finish_s = fin;
    s->done[batch[i].ticket] = res;
  }
  return rc;
}

}  // namespace

extern "C" {

smg_status smg_server_create(smg_ctx *c, const smg_graph *g, const smg_server_config *cfg, smg_server **out) {
  if (!c || !g || !out) return smg::fail(SMG_ERR_INVALID, "null argument");
  std::unique_ptr<smg_server> s(new smg_server);
  s->ctx = c;
  s->graph = g;
  if (cfg) s->cfg = *cfg;
  if (!s->cfg.max_inflight) s->cfg.max_inflight = 256;
  if (!s->cfg.memory_budget_bytes) s->cfg.memory_budget_bytes = 32ull << 30;
  *out = s.release();
  return SMG_OK;
}

smg_status smg_server_submit(smg_server *s, const smg_plan *p, uint64_t *ticket) {
  if (!s || !p || !ticket) return smg::fail(SMG_ERR_INVALID, "null argument");
  const uint64_t bytes = footprint(s->graph->g, p->p);
  if (bytes > s->cfg.memory_budget_bytes) return smg::fail(SMG_ERR_BUDGET, "query exceeds the server memory budget");
  *ticket = s->next_ticket++;
  s->queue.push_back({*ticket, &p->p, now_s(), bytes});
  return SMG_OK;
}

smg_status smg_server_step(smg_server *s) {
  if (!s) return smg::fail(SMG_ERR_INVALID, "null server");
  return run_admitted(s);
}

smg_status smg_server_poll(smg_server *s, uint64_t ticket, smg_request_result *out) {
  if (!s || !out) return smg::fail(SMG_ERR_INVALID, "null argument");
  auto it = s->done.find(ticket);
  if (it == s->done.end()) {
    if (ticket == 0 || ticket >= s->next_ticket) return smg::fail(SMG_ERR_INVALID, "unknown ticket");
    return SMG_ERR_NOT_READY;
  }
  *out = it->second;
  return SMG_OK;
}

smg_status smg_server_cancel(smg_server *s, uint64_t ticket) {
  if (!s) return smg::fail(SMG_ERR_INVALID, "null server");
  for (auto it = s->queue.begin(); it != s->queue.end(); ++it)
    if (it->ticket == ticket) {
      smg_request_result res{};
      res.status = SMG_ERR_CANCELLED;
      res.submit_s = it->submit_s;
      res.finish_s = now_s();
      s->done[ticket] = res;
      s->queue.erase(it);
      return SMG_OK;
    }
  return smg::fail(SMG_ERR_INVALID, "ticket is not queued");
}

smg_status smg_server_drain(smg_server *s) {
  if (!s) return smg::fail(SMG_ERR_INVALID, "null server");
  while (!s->queue.empty()) {
    smg_status rc = run_admitted(s);
    if (rc) return rc;
  }
  return SMG_OK;
}

void smg_server_destroy(smg_server *s) { delete s; }

}  // extern "C"
