/*
 * oracle.h — CPU restatement of ClusterSM's filter and join, used ONLY as a
 * checker by tests/, by __graft_entry__.smoke() and by bench.py's CPU
 * baseline.  Nothing in the library links or calls it.
 *
 * Parity status: pinned.  The count semantics are pinned by the reference's
 * example (dataset/example_q_01.in in dataset/example_g_01.in = 4
 * embeddings), and the query plan the filter consumes is pinned against the
 * reference's own host code (decycle.cpp, filter.cu clustering, order.cpp),
 * compiled from its sources by oracle/build_ref.sh into golden fixtures.
 *
 * All graphs are CSR with sorted neighbour lists.  The plan arguments are the
 * arrays of an smg_plan_view (include/smg.h); the oracle only reads them.
 */
#ifndef SMG_ORACLE_H
#define SMG_ORACLE_H
#include <stdint.h>

#include "smg.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Exact number of injective, label-preserving, non-induced embeddings of q
 * in g by backtracking (join.cu:142-166 semantics: injective, every query
 * edge present; filter.cu:489-490: labels equal).  If candmask is non-NULL,
 * vertex v may only take query vertex u when bit u of candmask[v] is set.
 * threads <= 0 uses all cores.  max_rows/emb: if emb is non-NULL, up to
 * max_rows embeddings (k ids each, in query-vertex order, lexicographically
 * sorted) are written; *rows receives how many.  When the count exceeds
 * max_rows the rows written are the first ones found, not the smallest. */
int oracle_count(const smg_csr *g, const smg_query_desc *q, const uint32_t *candmask,
                 int threads, uint64_t *count);
int oracle_embeddings(const smg_csr *g, const smg_query_desc *q, uint64_t max_rows,
                      uint32_t *emb, uint64_t *rows, uint64_t *count);

/* As oracle_count, but gives up once more than `budget` partial matches have
 * been created: then *used = UINT64_MAX and *count is a lower bound.
 * Otherwise *used is the number of partial matches created. */
int oracle_count_budget(const smg_csr *g, const smg_query_desc *q, const uint32_t *candmask,
                        int threads, uint64_t budget, uint64_t *count, uint64_t *used);

/* Backtracking count limited to root candidates [root_lo, root_hi) of the
 * oracle's own order (for timing a bounded sample).  *num_roots receives
 * the total number of root candidates. */
int oracle_count_roots(const smg_csr *g, const smg_query_desc *q, int threads,
                       uint64_t root_lo, uint64_t root_hi, uint64_t *count,
                       uint64_t *num_roots);

/* Initial filter (filter.cu:404-539): bit u of vmask0[v] iff L(v)=L(u),
 * deg(v) >= deg(u) and NLC_v[l] >= NLC_u[l] for every l < nvlq. */
int oracle_nlc_filter(const smg_csr *g, const smg_plan_view *p, uint32_t *vmask0);

/* Cluster bitmap (filter.cu:585-873, driven per layer as in filter.cu:976-1141
 * with every combine applied at the end of its own layer) and final
 * candidates (filter.cu:1158-1232).  enc: [num_vertices * num_words],
 * candmask: [num_vertices]. */
int oracle_encode(const smg_csr *g, const smg_plan_view *p, const uint32_t *vmask0,
                  uint32_t *enc, uint32_t *candmask);

/* Rows of the reference's breadth-first join tables after each step of its
 * edge order (join.cu:290-435): rows[0] = candidates of first[0], rows[e+1] =
 * rows after edge (first[e] -> second[e]).  candmask: final candidates
 * (bit u of candmask[v]).  Gives up once a level holds more than `limit`
 * rows; that level and the later ones then read UINT64_MAX.  rows: [num_edges + 1]. */
int oracle_ref_rows(const smg_csr *g, uint32_t k, uint32_t num_edges, const uint32_t *first,
                    const uint32_t *second, const uint32_t *candmask, int threads, uint64_t limit,
                    uint64_t *rows);

/* The workloads' seeded graphs (R-MAT and Erdos-Renyi, with uniform or
 * Zipf(s=1) labels), restated from the same integer generator so that the
 * CPU baseline needs nothing from the library.  The arrays are malloc'd;
 * release them with oracle_free.  *m2 = entries of adj (2 x edges). */
int oracle_gen_rmat(uint32_t scale, uint32_t avg_degree, uint32_t num_labels, uint32_t zipf, uint64_t seed,
                    uint64_t **offsets, uint32_t **adj, uint32_t **labels, uint64_t *m2);
int oracle_gen_er(uint32_t n, uint64_t m, uint32_t num_labels, uint32_t zipf, uint64_t seed,
                  uint64_t **offsets, uint32_t **adj, uint32_t **labels, uint64_t *m2);
void oracle_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
