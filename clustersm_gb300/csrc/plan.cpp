// plan.cpp — host-side query preprocessing.
//
// Each step reproduces the reference's host algorithm exactly (same vertex,
// cluster and edge numbering), because the cluster bitmap and the matching
// order depend on it:
//   decycle            decycle.cpp:6-134
//   vertex cover       filter.cu:23-112 (getVertexCover / dfs_cvc)
//   clustering         filter.cu:127-401
//   cluster CSR        structure.cu:219-239 (encodingMeta::init)
//   last slot per u    filter.cu:1290-1307, join.cu:242-250
//   first vertex       main.cu:144 (core of the last cluster)
//   edge order         order.cpp:150-206 (getBFSEdgeOrder)
// The reference's fixed-size tables (MAX_CLUSTERS = 150, MAX_LAYERS = 100,
// defs.h:15-16) become vectors; the layer count is still capped at 100.
#include <algorithm>
#include <memory>
#include <queue>
#include <set>

#include "host.h"

namespace smg {
namespace {

constexpr uint32_t NONE = 0xFFFFFFFFu;
constexpr uint32_t MAX_LAYERS = 100;
constexpr uint32_t MAX_CLUSTERS = 1u << 16;

// Tree DP for a minimum vertex cover (filter.cu:23-41).
void cover_dp(const Plan &P, uint32_t cur, uint32_t father, std::vector<int> &f0, std::vector<int> &f1) {
  f0[cur] = 0;
  f1[cur] = 1;
  for (uint32_t e = P.t_off[cur]; e < P.t_off[cur + 1]; ++e) {
    uint32_t w = P.t_nbr[e];
    if (w == father) continue;
    cover_dp(P, w, cur, f0, f1);
    f0[cur] += f1[w];
    f1[cur] += std::min(f0[w], f1[w]);
  }
}

}  // namespace

smg_status build_plan(const smg_query_desc &q, Plan &P) {
  const uint32_t n = q.num_vertices, m = q.num_edges;
  if (n < 2 || n > SMG_MAX_QUERY_VERTICES)
    return fail(SMG_ERR_QUERY, "query must have 2..32 vertices");
  if (m < 1 || m > SMG_MAX_QUERY_EDGES) return fail(SMG_ERR_QUERY, "query must have 1..496 edges");
  if (!q.labels || !q.edges) return fail(SMG_ERR_INVALID, "null query arrays");
  P = Plan();
  P.k = n;
  P.m = m;
  P.label.assign(q.labels, q.labels + n);
  // directed edge ids as readGraphToCPU2 assigns them (io.cu:82-94)
  std::vector<uint32_t> eid(n * n, NONE);
  P.evv_first.resize(2 * m);
  P.evv_second.resize(2 * m);
  std::vector<uint32_t> cnt(n + 1, 0);
  for (uint32_t i = 0; i < m; ++i) {
    uint32_t a = q.edges[2 * i], b = q.edges[2 * i + 1];
    if (a >= n || b >= n) return fail(SMG_ERR_QUERY, "query edge endpoint out of range");
    if (a == b) return fail(SMG_ERR_QUERY, "query has a self-loop");
    if (eid[a * n + b] != NONE) return fail(SMG_ERR_QUERY, "query has a repeated edge");
    eid[a * n + b] = 2 * i;
    eid[b * n + a] = 2 * i + 1;
    P.evv_first[2 * i] = a;
    P.evv_second[2 * i] = b;
    P.evv_first[2 * i + 1] = b;
    P.evv_second[2 * i + 1] = a;
    ++cnt[a + 1];
    ++cnt[b + 1];
  }
  for (uint32_t v = 0; v < n; ++v) cnt[v + 1] += cnt[v];
  P.q_off = cnt;
  P.q_nbr.resize(2 * m);
  P.q_eid.resize(2 * m);
  {
    std::vector<uint32_t> cur(cnt.begin(), cnt.end() - 1);
    for (uint32_t i = 0; i < m; ++i) {
      uint32_t a = q.edges[2 * i], b = q.edges[2 * i + 1];
      P.q_nbr[cur[a]] = b;
      P.q_eid[cur[a]++] = 2 * i;
      P.q_nbr[cur[b]] = a;
      P.q_eid[cur[b]++] = 2 * i + 1;
    }
  }
  P.deg.resize(n);
  for (uint32_t v = 0; v < n; ++v) P.deg[v] = P.q_off[v + 1] - P.q_off[v];
  // connectivity
  {
    std::vector<char> seen(n, 0);
    std::vector<uint32_t> st{0};
    seen[0] = 1;
    uint32_t reached = 1;
    while (!st.empty()) {
      uint32_t u = st.back();
      st.pop_back();
      for (uint32_t e = P.q_off[u]; e < P.q_off[u + 1]; ++e)
        if (!seen[P.q_nbr[e]]) {
          seen[P.q_nbr[e]] = 1;
          ++reached;
          st.push_back(P.q_nbr[e]);
        }
    }
    if (reached != n) return fail(SMG_ERR_QUERY, "query graph is disconnected");
  }
  // neighbour-label counts of the full query (filter.cu:555-564)
  uint32_t maxl = 0;
  for (uint32_t v = 0; v < n; ++v) maxl = std::max(maxl, P.label[v]);
  if (maxl >= (1u << 16)) return fail(SMG_ERR_LIMIT, "query labels must be below 65536");
  P.nvlq = maxl + 1;
  P.nlc.assign(static_cast<size_t>(n) * P.nvlq, 0);
  for (uint32_t u = 0; u < n; ++u)
    for (uint32_t e = P.q_off[u]; e < P.q_off[u + 1]; ++e) ++P.nlc[u * P.nvlq + P.label[P.q_nbr[e]]];

  // ---- decycle (decycle.cpp:6-134): BFS spanning tree from the first
  // vertex of maximum degree; non-tree edges are dropped from the tree only.
  P.t_deg = P.deg;
  {
    uint32_t root = 0;
    for (uint32_t u = 1; u < n; ++u)
      if (P.t_deg[u] > P.t_deg[root]) root = u;
    std::vector<char> keep(2 * m, 0), vis(n, 0);
    std::queue<uint32_t> qu;
    qu.push(root);
    vis[root] = 1;
    while (!qu.empty()) {
      uint32_t top = qu.front();
      qu.pop();
      for (uint32_t e = P.q_off[top]; e < P.q_off[top + 1]; ++e) {
        uint32_t w = P.q_nbr[e];
        if (!vis[w]) {
          vis[w] = 1;
          qu.push(w);
          keep[eid[top * n + w]] = 1;
        }
      }
    }
    for (uint32_t e = 0; e < 2 * m; e += 2) {
      if (keep[e] || keep[e + 1]) {
        keep[e] = keep[e + 1] = 1;
      } else {
        --P.t_deg[P.evv_first[e]];
        --P.t_deg[P.evv_second[e]];
      }
    }
    P.t_off.assign(n + 1, 0);
    for (uint32_t u = 0; u < n; ++u) {
      for (uint32_t e = P.q_off[u]; e < P.q_off[u + 1]; ++e)
        if (keep[P.q_eid[e]]) P.t_nbr.push_back(P.q_nbr[e]);
      P.t_off[u + 1] = static_cast<uint32_t>(P.t_nbr.size());
    }
  }

  // ---- minimum vertex cover of the tree (filter.cu:43-112)
  {
    uint32_t root = 0;
    for (uint32_t u = 1; u < n; ++u)
      if (P.t_deg[u] > P.t_deg[root]) root = u;
    std::vector<int> f0(n, 0), f1(n, 0);
    cover_dp(P, root, NONE, f0, f1);
    const uint32_t want = static_cast<uint32_t>(std::min(f0[root], f1[root]));
    struct Item {
      uint32_t v, father;
      bool father_selected;
    };
    std::vector<Item> st{{root, NONE, false}};
    while (!st.empty()) {
      Item it = st.back();
      st.pop_back();
      bool push_sel;
      if (f1[it.v] <= f0[it.v]) {
        P.cover.push_back(it.v);
        push_sel = true;
      } else if (it.father_selected || it.father == NONE) {
        push_sel = false;
      } else {
        P.cover.push_back(it.v);
        push_sel = true;
      }
      for (uint32_t e = P.t_off[it.v]; e < P.t_off[it.v + 1]; ++e) {
        uint32_t w = P.t_nbr[e];
        if (w == it.father) continue;
        st.push_back({w, it.v, push_sel});
      }
    }
    if (P.cover.size() != want) return fail(SMG_ERR_INTERNAL, "vertex cover size differs from the DP optimum");
  }

  // ---- clustering (filter.cu:127-401)
  std::vector<std::vector<uint32_t>> &C = P.clusters;
  std::vector<char> valid;
  uint32_t num_clusters = static_cast<uint32_t>(P.cover.size());
  for (uint32_t c = 0; c < num_clusters; ++c) {
    uint32_t core = P.cover[c];
    std::vector<uint32_t> cl{core};
    cl.insert(cl.end(), P.t_nbr.begin() + P.t_off[core], P.t_nbr.begin() + P.t_off[core + 1]);
    C.push_back(cl);
    P.cl_layer.push_back(0);
    P.cl_kind.push_back(0);
  }
  valid.assign(num_clusters, 1);
  auto ensure = [&](uint32_t idx) {
    if (C.size() <= idx) {
      C.resize(idx + 1);
      P.cl_layer.resize(idx + 1, 0);
      P.cl_kind.resize(idx + 1, 0);
      valid.resize(idx + 1, 1);
    }
  };
  std::vector<uint32_t> per_layer{num_clusters};
  uint32_t layer = 0;
  uint32_t i = 0;
  int64_t actual_new;
  do {
    uint32_t num_new = 0;
    for (; i < num_clusters; ++i) {
      if (!valid[i]) continue;
      const uint32_t core_i = C[i][0];
      for (uint32_t j = i + 1; j < num_clusters; ++j) {
        if (!valid[j]) continue;
        const uint32_t core_j = C[j][0];
        for (size_t ip = 1; ip < C[i].size(); ++ip) {
          const uint32_t ui = C[i][ip];
          for (size_t jp = 0; jp < C[j].size(); ++jp) {
            if (ui != C[j][jp]) continue;
            ++num_new;
            const uint32_t idx = num_clusters + num_new - 1;
            if (idx >= MAX_CLUSTERS) return fail(SMG_ERR_LIMIT, "too many clusters");
            ensure(idx);
            valid[idx] = 1;
            if (jp != 0)
              C[idx] = core_i == core_j ? std::vector<uint32_t>{ui, core_i}
                                        : std::vector<uint32_t>{ui, core_i, core_j};
            else
              C[idx] = {ui, core_i};
            P.cl_layer[idx] = layer + 1;
            P.cl_kind[idx] = 1;
            P.mg_cluster.push_back(idx);
            P.mg_left.push_back(i);
            P.mg_right.push_back(j);
            P.mg_vertex.push_back(ui);
          }
        }
      }
    }
    ++layer;
    if (layer >= MAX_LAYERS) return fail(SMG_ERR_LIMIT, "too many cluster layers");
    actual_new = num_new;
    // combine clusters of this layer that share a core (filter.cu:270-366)
    for (uint32_t out = num_clusters; out < num_clusters + num_new; ++out) {
      if (!valid[out]) continue;
      const uint32_t core = C[out][0];
      bool dup = false;
      std::set<uint32_t> group{out};
      std::set<uint32_t> nbrs(C[out].begin() + 1, C[out].end());
      for (uint32_t in = out + 1; in < num_clusters + num_new; ++in) {
        if (!valid[in] || C[in][0] != core) continue;
        dup = true;
        group.insert(in);
        nbrs.insert(C[in].begin() + 1, C[in].end());
      }
      if (!dup) continue;
      CombineRec rec;
      rec.layer = layer;
      uint32_t holder = NONE;  // first cluster of the group holding every neighbour
      for (uint32_t c : group)
        if (C[c].size() == nbrs.size() + 1) {
          holder = c;
          break;
        }
      if (holder != NONE) {
        group.erase(holder);
        rec.type = 1;
        rec.out = holder;
      } else {
        ++num_new;
        ++actual_new;
        const uint32_t idx = num_clusters + num_new - 1;
        if (idx >= MAX_CLUSTERS) return fail(SMG_ERR_LIMIT, "too many clusters");
        ensure(idx);
        valid[idx] = 1;
        C[idx] = {core};
        C[idx].insert(C[idx].end(), nbrs.begin(), nbrs.end());
        P.cl_layer[idx] = layer;
        P.cl_kind[idx] = 2;
        rec.type = 0;
        rec.out = idx;
      }
      rec.others.assign(group.begin(), group.end());
      actual_new -= static_cast<int64_t>(group.size());
      for (uint32_t c : group) valid[c] = 0;
      P.combines.push_back(rec);
    }
    num_clusters += num_new;
    per_layer.push_back(num_new);
  } while (actual_new > 1);
  C.resize(num_clusters);
  P.cl_layer.resize(num_clusters);
  P.cl_kind.resize(num_clusters);
  P.num_layers = layer + 1;
  P.layer_begin.assign(P.num_layers + 1, 0);
  for (uint32_t l = 1; l <= layer; ++l) P.layer_begin[l] = P.layer_begin[l - 1] + per_layer[l - 1];
  P.layer_begin[P.num_layers] = num_clusters;

  // ---- cluster CSR (structure.cu:219-239)
  P.cl_off.assign(num_clusters + 1, 0);
  for (uint32_t c = 0; c < num_clusters; ++c) {
    P.cl_off[c + 1] = P.cl_off[c] + static_cast<uint32_t>(C[c].size());
    P.slots.insert(P.slots.end(), C[c].begin(), C[c].end());
  }
  P.num_words = (static_cast<uint32_t>(P.slots.size()) + 31) / 32;
  auto first_slot_of = [&](uint32_t c, uint32_t u) -> uint32_t {
    for (uint32_t s = P.cl_off[c]; s < P.cl_off[c + 1]; ++s)
      if (P.slots[s] == u) return s;
    return NONE;
  };
  for (size_t r = 0; r < P.mg_cluster.size(); ++r) {
    uint32_t lp = first_slot_of(P.mg_left[r], P.mg_vertex[r]);
    uint32_t rp = first_slot_of(P.mg_right[r], P.mg_vertex[r]);
    if (lp == NONE || rp == NONE) return fail(SMG_ERR_INTERNAL, "merge vertex missing from its clusters");
    P.mg_left_pos.push_back(lp);
    P.mg_right_pos.push_back(rp);
  }
  P.cb_oth_off.push_back(0);
  for (const CombineRec &r : P.combines) {
    P.cb_out.push_back(r.out);
    P.cb_type.push_back(r.type);
    P.cb_layer.push_back(r.layer);
    P.cb_oth.insert(P.cb_oth.end(), r.others.begin(), r.others.end());
    P.cb_oth_off.push_back(static_cast<uint32_t>(P.cb_oth.size()));
  }
  // slot whose bit gives the final candidates of u: the last one holding u
  P.last_slot.assign(n, NONE);
  for (uint32_t s = static_cast<uint32_t>(P.slots.size()); s-- > 0;)
    if (P.last_slot[P.slots[s]] == NONE) P.last_slot[P.slots[s]] = s;
  for (uint32_t u = 0; u < n; ++u)
    if (P.last_slot[u] == NONE) return fail(SMG_ERR_INTERNAL, "query vertex in no cluster");
  P.root = P.slots[P.cl_off[num_clusters - 1]];

  // ---- BFS edge order over the full query (order.cpp:150-206)
  {
    const uint32_t start = P.root, start_nbr = P.q_nbr[P.q_off[start]];
    std::vector<uint32_t> order{eid[start * n + start_nbr]};
    std::vector<char> vis(n, 0), used(n * n, 0);
    used[start * n + start_nbr] = 1;
    std::queue<uint32_t> qu;
    qu.push(start);
    while (!qu.empty()) {
      uint32_t u = qu.front();
      qu.pop();
      vis[u] = 1;
      for (uint32_t e = P.q_off[u]; e < P.q_off[u + 1]; ++e) {
        uint32_t w = P.q_nbr[e];
        if (!vis[w]) qu.push(w);
        if (!used[w * n + u] && !used[u * n + w]) {
          order.push_back(P.q_eid[e]);
          used[u * n + w] = 1;
        }
      }
    }
    if (order.size() != m) return fail(SMG_ERR_INTERNAL, "edge order does not cover the query");
    for (uint32_t e : order) {
      P.eo_first.push_back(P.evv_first[e]);
      P.eo_second.push_back(P.evv_second[e]);
    }
  }
  // ---- vertex-level order: a vertex is matched by the first edge that
  // reaches it (join.cu:348-370); every other edge becomes a check.
  P.level_of.assign(n, NONE);
  P.order.push_back(P.root);
  P.level_of[P.root] = 0;
  P.anchor_level.assign(n, 0);
  for (uint32_t t = 0; t < m; ++t) {
    uint32_t f = P.eo_first[t], s = P.eo_second[t];
    if (P.level_of[s] != NONE) continue;
    if (P.level_of[f] == NONE) return fail(SMG_ERR_INTERNAL, "edge order extends from an unmapped vertex");
    P.level_of[s] = static_cast<uint32_t>(P.order.size());
    P.anchor_level[P.order.size()] = P.level_of[f];
    P.order.push_back(s);
  }
  if (P.order.size() != n) return fail(SMG_ERR_INTERNAL, "matching order misses a vertex");
  P.back_mask.assign(n, 0);
  P.same_label_mask.assign(n, 0);
  for (uint32_t lv = 0; lv < n; ++lv) {
    uint32_t u = P.order[lv];
    for (uint32_t e = P.q_off[u]; e < P.q_off[u + 1]; ++e) {
      uint32_t lw = P.level_of[P.q_nbr[e]];
      if (lw < lv) P.back_mask[lv] |= 1u << lw;
    }
    for (uint32_t lw = 0; lw < lv; ++lw)
      if (P.label[P.order[lw]] == P.label[u]) P.same_label_mask[lv] |= 1u << lw;
  }
  return SMG_OK;
}

}  // namespace smg

using namespace smg;

extern "C" {

smg_status smg_plan_create(const smg_query_desc *q, smg_plan **out) {
  if (!q || !out) return fail(SMG_ERR_INVALID, "null argument");
  *out = nullptr;
  std::unique_ptr<smg_plan> p(new smg_plan);
  smg_status s = build_plan(*q, p->p);
  if (s) return s;
  *out = p.release();
  return SMG_OK;
}

void smg_plan_free(smg_plan *p) { delete p; }

smg_status smg_plan_create_batch(const smg_query_desc *queries, uint32_t n, smg_plan **out) {
  if (n && (!queries || !out)) return fail(SMG_ERR_INVALID, "null argument");
  std::vector<smg_status> st(n, SMG_OK);
  // the plans are independent: one per thread
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t i = 0; i < static_cast<int64_t>(n); ++i) {
    out[i] = nullptr;
    std::unique_ptr<smg_plan> p(new smg_plan);
    st[i] = build_plan(queries[i], p->p);
    if (!st[i]) out[i] = p.release();
  }
  for (uint32_t i = 0; i < n; ++i) {
    if (!st[i]) continue;
    // the first failing query again, on this thread, so that smg_last_error
    // (thread-local) names its reason; then nothing is handed out
    smg_plan *tmp = nullptr;
    const smg_status s = smg_plan_create(queries + i, &tmp);
    smg_plan_free(tmp);
    for (uint32_t j = 0; j < n; ++j) {
      smg_plan_free(out[j]);
      out[j] = nullptr;
    }
    return s ? s : st[i];
  }
  return SMG_OK;
}

smg_status smg_plan_get(const smg_plan *pp, smg_plan_view *v) {
  if (!pp || !v) return fail(SMG_ERR_INVALID, "null argument");
  const Plan &P = pp->p;
  v->k = P.k;
  v->num_edges = P.m;
  v->nvlq = P.nvlq;
  v->root = P.root;
  v->labels = P.label.data();
  v->degrees = P.deg.data();
  v->nlc = P.nlc.data();
  v->tree_offsets = P.t_off.data();
  v->tree_neighbors = P.t_nbr.data();
  v->cover_size = static_cast<uint32_t>(P.cover.size());
  v->cover = P.cover.data();
  v->num_clusters = static_cast<uint32_t>(P.clusters.size());
  v->num_slots = static_cast<uint32_t>(P.slots.size());
  v->num_words = P.num_words;
  v->cluster_offsets = P.cl_off.data();
  v->slots = P.slots.data();
  v->cluster_layer = P.cl_layer.data();
  v->cluster_kind = P.cl_kind.data();
  v->num_layers = P.num_layers;
  v->num_merges = static_cast<uint32_t>(P.mg_cluster.size());
  v->merge_cluster = P.mg_cluster.data();
  v->merge_left = P.mg_left.data();
  v->merge_right = P.mg_right.data();
  v->merge_vertex = P.mg_vertex.data();
  v->num_combines = static_cast<uint32_t>(P.combines.size());
  v->combine_out = P.cb_out.data();
  v->combine_type = P.cb_type.data();
  v->combine_layer = P.cb_layer.data();
  v->combine_other_offsets = P.cb_oth_off.data();
  v->combine_others = P.cb_oth.data();
  v->last_slot = P.last_slot.data();
  v->edge_order_first = P.eo_first.data();
  v->edge_order_second = P.eo_second.data();
  v->order = P.order.data();
  v->anchor_level = P.anchor_level.data();
  v->back_mask = P.back_mask.data();
  return SMG_OK;
}

}  // extern "C"
