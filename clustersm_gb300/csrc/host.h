// host.h — host-side structures shared by the library's C++ translation units.
#pragma once

#include <cstdint>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "smg.h"

namespace smg {

// Allocator whose resize() leaves new elements uninitialised, so that large
// host arrays are first touched by the parallel loops that fill them instead
// of by one thread writing zeros.
template <class T>
struct NoInitAlloc : std::allocator<T> {
  template <class U>
  struct rebind {
    using other = NoInitAlloc<U>;
  };
  NoInitAlloc() = default;
  template <class U>
  NoInitAlloc(const NoInitAlloc<U> &) noexcept {}
  template <class U>
  void construct(U *p) noexcept {
    ::new (static_cast<void *>(p)) U;
  }
  template <class U, class... A>
  void construct(U *p, A &&...a) {
    ::new (static_cast<void *>(p)) U(std::forward<A>(a)...);
  }
};
using RawU32 = std::vector<uint32_t, NoInitAlloc<uint32_t>>;

// Records `msg` as the calling thread's last error detail and returns `s`.
smg_status fail(smg_status s, const std::string &msg);

// Undirected labelled graph in CSR form.  Data graphs keep sorted neighbour
// lists; a graph read from a file keeps file order until it is uploaded.
struct HostGraph {
  uint32_t n = 0;
  uint64_t m = 0;  // undirected edges
  std::vector<uint64_t> off;
  RawU32 adj;
  std::vector<uint32_t> label;
  smg_csr view() const {
    smg_csr c;
    c.num_vertices = n;
    c.num_edges = m;
    c.offsets = off.data();
    c.neighbors = adj.data();
    c.labels = label.data();
    return c;
  }
};

// Query graph: labels and the undirected edge list in file order.
struct HostQuery {
  uint32_t n = 0;
  std::vector<uint32_t> label;
  std::vector<uint32_t> edges;  // 2 per edge
  smg_query_desc view() const {
    smg_query_desc d;
    d.num_vertices = n;
    d.num_edges = static_cast<uint32_t>(edges.size() / 2);
    d.labels = label.data();
    d.edges = edges.data();
    return d;
  }
};

// One combine record (filter.cu:262-366): the clusters of `others` that share
// the core of `out` are intersected into `out`.
struct CombineRec {
  uint32_t out = 0;
  uint32_t type = 0;  // 0: `out` is a new cluster, 1: `out` already existed
  uint32_t layer = 0;
  std::vector<uint32_t> others;  // ascending cluster indices
};

// Host-side query plan: everything the device filter and join need, derived
// by the same steps and in the same order as the reference's host code.
struct Plan {
  uint32_t k = 0, m = 0, nvlq = 0, root = 0;
  std::vector<uint32_t> label, deg;
  std::vector<uint32_t> nlc;  // k * nvlq
  // full query CSR in file order, directed edge ids 2i / 2i+1 per file edge i
  std::vector<uint32_t> q_off, q_nbr, q_eid;
  std::vector<uint32_t> evv_first, evv_second;  // [2m]
  // spanning tree (decycle)
  std::vector<uint32_t> t_off, t_nbr, t_deg;
  std::vector<uint32_t> cover;
  // clusters
  std::vector<std::vector<uint32_t>> clusters;
  std::vector<uint32_t> cl_off, slots, cl_layer, cl_kind;
  uint32_t num_layers = 0, num_words = 0;
  std::vector<uint32_t> layer_begin;  // [num_layers + 1] first cluster of layer
  std::vector<uint32_t> mg_cluster, mg_left, mg_right, mg_vertex;
  std::vector<uint32_t> mg_left_pos, mg_right_pos;  // slot of the vertex
  std::vector<CombineRec> combines;
  std::vector<uint32_t> cb_out, cb_type, cb_layer, cb_oth_off, cb_oth;
  std::vector<uint32_t> last_slot;  // [k]
  // reference edge order
  std::vector<uint32_t> eo_first, eo_second;
  // vertex-level matching order
  std::vector<uint32_t> order, level_of, anchor_level, back_mask;
  // per-level mask of earlier levels with the same label (injectivity)
  std::vector<uint32_t> same_label_mask;
};

smg_status build_plan(const smg_query_desc &q, Plan &out);

// .in parsing (io.cu:24-108 dialect)
smg_status read_in_file(const char *path, uint32_t &n, std::vector<uint32_t> &label,
                        std::vector<uint32_t> &deg, RawU32 &edges);

// Degree of every vertex in a flat (a, b) edge-pair list, counted in parallel.
std::vector<uint32_t> count_degrees(uint32_t n, const RawU32 &edges);

// CSR from an edge-pair list; each list keeps file order unless sort_lists.
// `degrees`, when given, must be the counts count_degrees would return.
smg_status csr_from_edges(uint32_t n, const RawU32 &edges, bool sort_lists,
                          HostGraph &g, const std::vector<uint32_t> *degrees = nullptr);

}  // namespace smg

struct smg_host_graph {
  smg::HostGraph g;
};
struct smg_host_query {
  smg::HostQuery q;
};
struct smg_plan {
  smg::Plan p;
};
