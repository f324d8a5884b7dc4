/*
 * smg.h — C ABI of the GB300-native subgraph-matching library (libsmg).
 *
 * The library counts (and optionally lists) the injective, label-preserving,
 * non-induced embeddings of a small labelled query graph in a large labelled
 * undirected data graph, with the same semantics and the same host-side
 * query preprocessing as ClusterSM:
 *
 *   reference seam                         replaced here by
 *   -------------------------------------  ---------------------------------
 *   readGraphToCPU2   io.cu:24-108          smg_read_graph / smg_read_query
 *   copyMeta + copyGraphToGPU io.cu:235,265 smg_graph_upload
 *   decycle decycle.cpp:6, clustering       smg_plan_create (host C++)
 *     filter.cu:127, getBFSEdgeOrder
 *     order.cpp:150, encodingMeta::init
 *     structure.cu:219
 *   clusterFilter  filter.cuh:130-144       smg_filter_inspect (filter only)
 *   clusterFilter + join  main.cu:123-172   smg_match (one query per call)
 *   runClusterSM.sh:9-13 (one process per   smg_match_batch (many queries,
 *     query)                                  one persistent launch)
 *   (none: no serving mode)                 smg_server_*
 *
 * Conventions: every call returns an smg_status; no call exits the process.
 * Vertex ids are uint32, offsets and counts uint64.  A context is bound to
 * one device and one CUDA stream; it is thread-compatible, not thread-safe.
 * Objects returned through an out-pointer are owned by the caller and freed
 * with the matching *_free / *_destroy call.
 */
#ifndef SMG_H
#define SMG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
typedef int32_t smg_status;
#define SMG_OK 0
#define SMG_ERR_INVALID 1    /* bad argument (null pointer, size mismatch)       */
#define SMG_ERR_IO 2         /* cannot open / read / write a file (io.cu:29-33)  */
#define SMG_ERR_FORMAT 3     /* malformed .in text (io.cu:37-41)                 */
#define SMG_ERR_QUERY 4      /* unsupported query: disconnected, <2 or >32
                                vertices, self-loop or repeated edge           */
#define SMG_ERR_LIMIT 5      /* a size limit of this build was exceeded          */
#define SMG_ERR_CUDA 6       /* a CUDA runtime call failed                       */
#define SMG_ERR_OOM 7        /* device or host allocation failed                 */
#define SMG_ERR_TIMEOUT 8    /* a bounded device-side wait gave up               */
#define SMG_ERR_NO_DEVICE 9  /* no usable CUDA device                            */
#define SMG_ERR_BUDGET 10    /* request exceeds the server memory budget         */
#define SMG_ERR_CANCELLED 11 /* request cancelled before it ran                  */
#define SMG_ERR_NOT_READY 12 /* request still in flight (smg_server_poll)        */
#define SMG_ERR_INTERNAL 13  /* invariant violated inside the library            */

/* Static string for a status code; never NULL. */
const char *smg_strerror(smg_status s);
/* Detail text of the last error raised on this host thread ("" if none). */
const char *smg_last_error(void);

/* Limits of this build. */
#define SMG_MAX_QUERY_VERTICES 32u /* u-bitmasks are 32 bits (filter.cu:501) */
#define SMG_MAX_QUERY_EDGES 496u   /* complete graph on 32 vertices          */

/* ------------------------------------------------------- host-side graphs */
/* Read-only view of an undirected labelled graph in CSR form (host memory).
 * neighbors holds every undirected edge twice, once in each endpoint's list. */
typedef struct smg_csr {
  uint32_t num_vertices;
  uint64_t num_edges;        /* undirected edges                          */
  const uint64_t *offsets;   /* [num_vertices + 1]                        */
  const uint32_t *neighbors; /* [2 * num_edges]                           */
  const uint32_t *labels;    /* [num_vertices]                            */
} smg_csr;

/* Read-only view of a query graph: labels plus the undirected edge list in
 * file order.  File order matters: it fixes neighbour order in the query CSR,
 * which fixes the spanning tree, the clusters and the matching order. */
typedef struct smg_query_desc {
  uint32_t num_vertices;
  uint32_t num_edges;
  const uint32_t *labels; /* [num_vertices]                                  */
  const uint32_t *edges;  /* [2 * num_edges]: (a0,b0, a1,b1, ...) file order */
} smg_query_desc;

typedef struct smg_host_graph smg_host_graph; /* library-owned host CSR   */
typedef struct smg_host_query smg_host_query; /* library-owned query      */

/* Parse a .in data graph: "t n m", then "v id label deg" lines, then
 * "e a b" once per undirected edge (io.cu:24-108).  Declared degrees must
 * match the edges.  Neighbour lists keep file order. */
smg_status smg_read_graph(const char *path, smg_host_graph **out);
/* Parse a .in query graph (same format), keeping the edge list in file order. */
smg_status smg_read_query(const char *path, smg_host_query **out);
/* Write a graph / query in the same .in dialect. */
smg_status smg_write_graph(const char *path, const smg_csr *g);
smg_status smg_write_query(const char *path, const smg_query_desc *q);

/* Views into library-owned objects (valid until the object is freed). */
smg_status smg_host_graph_view(const smg_host_graph *g, smg_csr *out);
smg_status smg_host_query_view(const smg_host_query *q, smg_query_desc *out);
/* Build a host graph from a caller's CSR (copies; neighbour lists are
 * sorted and checked for self-loops / duplicates / asymmetry). */
smg_status smg_host_graph_from_csr(const smg_csr *in, smg_host_graph **out);
void smg_host_graph_free(smg_host_graph *g);
void smg_host_query_free(smg_host_query *q);

/* Seeded synthetic inputs (deterministic on every host: integer-only RNG).
 * label_dist: SMG_LABELS_UNIFORM or SMG_LABELS_ZIPF1 (P(l) ~ 1/(l+1)).     */
#define SMG_LABELS_UNIFORM 0
#define SMG_LABELS_ZIPF1 1
/* Erdos-Renyi G(n, m): m distinct unordered pairs, no self-loops. */
smg_status smg_gen_er(uint32_t n, uint64_t m, uint32_t num_labels,
                      uint32_t label_dist, uint64_t seed, smg_host_graph **out);
/* R-MAT (a,b,c,d)=(0.57,0.19,0.19,0.05) on n = 2^scale vertices:
 * n*avg_degree/2 edge draws, symmetrised, self-loops and duplicates dropped,
 * neighbour lists sorted.  threads<=0 uses all host cores. */
smg_status smg_gen_rmat(uint32_t scale, uint32_t avg_degree, uint32_t num_labels,
                        uint32_t label_dist, uint64_t seed, int threads,
                        smg_host_graph **out);
/* The raw edge draws of smg_gen_rmat (same seed, same draws, before they are
 * symmetrised and de-duplicated) as pairs (a0, b0, a1, b1, ...) in
 * pairs[2 * *num_pairs]; with pairs == NULL only *num_pairs is set.  With the
 * labels of smg_gen_labels (same seed) they make the same graph through
 * smg_graph_build. */
smg_status smg_gen_rmat_pairs(uint32_t scale, uint32_t avg_degree, uint64_t seed, int threads,
                              uint32_t *pairs, uint64_t *num_pairs);
/* The vertex labels smg_gen_er / smg_gen_rmat draw for a seed. */
smg_status smg_gen_labels(uint32_t num_vertices, uint32_t num_labels, uint32_t label_dist,
                          uint64_t seed, uint32_t *labels);
/* Random-walk query extraction: k distinct vertices reached by a seeded walk,
 * labels copied, so at least one embedding exists.  shape: */
#define SMG_SHAPE_TREE 0   /* first-visit edges only                       */
#define SMG_SHAPE_SPARSE 1 /* tree + 2 random induced non-tree edges       */
#define SMG_SHAPE_DENSE 2  /* all induced edges, average query degree >= 3 */
#define SMG_SHAPE_INDUCED 3 /* all induced edges, no density requirement    */
smg_status smg_gen_query(const smg_csr *g, uint32_t k, uint32_t shape,
                         uint64_t seed, smg_host_query **out,
                         uint32_t *out_data_vertices /* [k] or NULL */);

/* ------------------------------------------------------------ query plans */
typedef struct smg_plan smg_plan;

/* Host-side preprocessing of one query: spanning tree (decycle.cpp:6-134),
 * minimum vertex cover (filter.cu:23-112), clustering (filter.cu:127-401),
 * cluster CSR (structure.cu:219-239), BFS edge order (order.cpp:150-206)
 * from the core of the last cluster (main.cu:144). */
smg_status smg_plan_create(const smg_query_desc *q, smg_plan **out);
void smg_plan_free(smg_plan *p);
/* smg_plan_create for queries[0 .. n) on all host threads: out[i] receives
 * the plan of queries[i].  On the first failing query (in index order) it
 * frees every plan, sets every out[i] to NULL and returns that query's
 * status (smg_last_error names the reason).  The reference plans one query
 * per process (runClusterSM.sh:9-13, main.cu:93-144). */
smg_status smg_plan_create_batch(const smg_query_desc *queries, uint32_t n, smg_plan **out);

/* Read-only view of a plan (arrays owned by the plan). */
typedef struct smg_plan_view {
  uint32_t k;              /* query vertices                                 */
  uint32_t num_edges;      /* query edges                                    */
  uint32_t nvlq;           /* largest query label + 1 (io.cu:269)            */
  uint32_t root;           /* first vertex of the matching order             */
  const uint32_t *labels;  /* [k]                                            */
  const uint32_t *degrees; /* [k] full-query degrees                         */
  const uint32_t *nlc;     /* [k * nvlq] neighbour-label counts (filter.cu:555) */
  /* spanning tree CSR (decycle) */
  const uint32_t *tree_offsets;   /* [k + 1]                               */
  const uint32_t *tree_neighbors; /* [tree_offsets[k]]                     */
  /* vertex cover in selection order */
  uint32_t cover_size;
  const uint32_t *cover;
  /* cluster CSR (encodingMeta) */
  uint32_t num_clusters;
  uint32_t num_slots;              /* num_total_us                          */
  uint32_t num_words;              /* ceil(num_slots / 32), num_blocks      */
  const uint32_t *cluster_offsets; /* [num_clusters + 1]                    */
  const uint32_t *slots;           /* [num_slots] query vertex per slot     */
  const uint32_t *cluster_layer;   /* [num_clusters]                        */
  const uint32_t *cluster_kind;    /* [num_clusters] 0 star, 1 merge, 2 combine */
  uint32_t num_layers;
  /* merge records, one per merge cluster, in cluster order */
  uint32_t num_merges;
  const uint32_t *merge_cluster; /* [num_merges] cluster index created      */
  const uint32_t *merge_left;    /* [num_merges]                            */
  const uint32_t *merge_right;   /* [num_merges]                            */
  const uint32_t *merge_vertex;  /* [num_merges] connection vertex          */
  /* combine records in creation order */
  uint32_t num_combines;
  const uint32_t *combine_out;          /* [num_combines]                   */
  const uint32_t *combine_type;         /* [num_combines] 0 new, 1 in-place  */
  const uint32_t *combine_layer;        /* [num_combines]                   */
  const uint32_t *combine_other_offsets;/* [num_combines + 1]               */
  const uint32_t *combine_others;       /* [combine_other_offsets[n]]       */
  const uint32_t *last_slot;            /* [k] slot read for candidates     */
  /* reference edge order: directed edges (first -> second), first mapped */
  const uint32_t *edge_order_first;  /* [num_edges]                        */
  const uint32_t *edge_order_second; /* [num_edges]                        */
  /* vertex-level matching order derived from the edge order */
  const uint32_t *order;         /* [k] query vertex matched at each level  */
  const uint32_t *anchor_level;  /* [k] level of the tree parent (0 for root) */
  const uint32_t *back_mask;     /* [k] bit j: edge to the vertex of level j<i */
} smg_plan_view;
smg_status smg_plan_get(const smg_plan *p, smg_plan_view *out);

/* ---------------------------------------------------- device context/graph */
typedef struct smg_ctx smg_ctx;
typedef struct smg_graph smg_graph;

/* Bind a context to CUDA device `device` (main.cu:36-43) on its own stream. */
smg_status smg_open(int device, smg_ctx **out);
void smg_close(smg_ctx *ctx);
/* The context's CUDA stream (a cudaStream_t), for callers that time or order
 * their own work against the library's launches. */
void *smg_ctx_stream(smg_ctx *ctx);

/* Upload a data graph: CSR with sorted neighbour lists, labels and the
 * per-vertex neighbour-label counts become device-resident until freed. */
smg_status smg_graph_upload(smg_ctx *ctx, const smg_csr *g, smg_graph **out);
void smg_graph_free(smg_graph *g);
/* Build a data graph on the device from an undirected edge list in host
 * memory, pairs[2 * num_pairs] = (a0, b0, a1, b1, ...): any order, repeats
 * and both orientations allowed, self-loops dropped, every endpoint below
 * num_vertices (else SMG_ERR_INVALID); fewer than 2^31 pairs.  The device
 * writes both directions of every pair, radix-sorts them by (source,
 * target), keeps one of each and scans the degrees into 64-bit offsets; the
 * resident graph is then the same as smg_graph_upload of that CSR.  Replaces
 * the reference's host CSR build (readGraphToCPU2 io.cu:60-96, one std::map
 * insert per edge).  *num_edges (may be NULL) receives the distinct
 * undirected edges. */
smg_status smg_graph_build(smg_ctx *ctx, uint32_t num_vertices, uint64_t num_pairs,
                           const uint32_t *pairs, const uint32_t *labels, smg_graph **out,
                           uint64_t *num_edges);
/* Copy a resident graph's CSR to host memory: offsets[num_vertices + 1] and
 * neighbors[2 * num_edges], lists sorted by id. */
smg_status smg_graph_download(smg_ctx *ctx, const smg_graph *g, uint64_t *offsets,
                              uint32_t *neighbors);

typedef struct smg_graph_stats {
  uint32_t num_vertices;
  uint64_t num_edges;
  uint32_t num_labels;   /* largest label + 1                              */
  uint32_t max_degree;
  uint64_t device_bytes; /* HBM held by the resident graph               */
} smg_graph_stats;
smg_status smg_graph_get_stats(const smg_graph *g, smg_graph_stats *out);

/* ------------------------------------------------------------------ match */
#define SMG_FLAG_EMIT 1u      /* write embeddings to opts->embeddings        */
#define SMG_FLAG_PROFILE 2u   /* record per-phase device times (adds syncs)  */
#define SMG_FLAG_NO_GRAPH 4u  /* batched path: launch directly instead of
                                 capturing the launches in a CUDA graph    */
#define SMG_FLAG_MODEL 8u     /* batched path: also count model_bytes, the
                                 bytes a breadth-first table join (the
                                 reference's, join.cu:290-435) would move
                                 for the same partial matches (costs a few
                                 loads per partial match)                 */

typedef struct smg_match_opts {
  uint32_t flags;
  uint32_t bfs_depth;     /* breadth-first levels before the join turns
                             depth-first: a warp queues every partial
                             match of the first bfs_depth levels as a
                             task, while the queue holds at most the root
                             tasks plus SMG_BFS_SLOTS_PER_WARP (16) slots
                             per resident join warp; past that it
                             descends itself.  0 = the tuned depth of the
                             query's shape class, none when untuned.
                             Counts do not depend on it.  The reference
                             joins every level breadth-first
                             (join.cu:290-435).                            */
  uint32_t root_chunk;    /* root candidates per initial task; 0 = auto    */
  uint32_t reserved;
  uint64_t max_embeddings; /* rows of k ids the embeddings buffer can hold */
  uint32_t *embeddings;    /* host buffer [max_embeddings * k], row r holds
                              the data vertex of query vertex 0..k-1       */
  uint64_t max_count;      /* 0 = none; otherwise a query stops as soon as
                              its count is known to exceed max_count, and
                              reports UINT64_MAX (batch) / limit_hit = 1   */
  uint64_t max_work;       /* 0 = none; otherwise a query stops once its
                              join warps have taken more than max_work
                              steps (one step: one pass of a warp's task
                              loop, a batch of list entries or one
                              descent), reported like max_count: a bound
                              on the work of queries whose count may be
                              out of reach                                 */
} smg_match_opts;

typedef struct smg_match_result {
  uint64_t count;               /* exact number of embeddings             */
  uint64_t embeddings_written;  /* rows written (<= max_embeddings)       */
  uint32_t overflow;            /* 1 if more embeddings than rows         */
  uint32_t num_candidates_root; /* candidates of the first matched vertex */
  uint64_t candidates_total;    /* sum over u of |C(u)| after the filter  */
  float filter_ms;              /* device time of the filter (PROFILE)    */
  float join_ms;                /* device time of the join (PROFILE)      */
  uint64_t tasks;               /* depth-first tasks processed            */
  uint64_t filter_bytes;        /* algorithmic bytes of the filter        */
  uint64_t join_bytes;          /* algorithmic bytes of the join          */
  uint32_t limit_hit;           /* 1: count exceeded opts->max_count      */
  uint32_t reserved;
} smg_match_result;

/* Plain path: one query, filter then join, synchronous. */
smg_status smg_match(smg_ctx *ctx, const smg_graph *g, const smg_plan *p,
                     const smg_match_opts *opts, smg_match_result *out);

/* Batched path: all queries in one persistent launch fed by a device work
 * queue; counts[i] receives the exact count of plans[i].  The launches of a
 * batch are captured in a CUDA graph; calling again with the same plans (same
 * handles, same order) on the same context replays the graph without
 * re-staging the query records, unless another call ran in between. */
typedef struct smg_batch_stats {
  float filter_ms;           /* device time of the filters (PROFILE)       */
  float join_ms;             /* device time of the joins (PROFILE)         */
  uint64_t tasks;            /* depth-first tasks processed                */
  uint64_t total_embeddings; /* sum of the counts                          */
  uint64_t kernel_launches;  /* kernels this call launched                 */
  uint64_t h2d_bytes;        /* host-to-device bytes this call copied      */
  uint64_t d2h_bytes;        /* device-to-host bytes this call copied      */
  uint64_t filter_bytes;     /* algorithmic bytes of the filters           */
  uint64_t join_bytes;       /* algorithmic bytes of the joins             */
  uint32_t chunks;           /* memory-bounded sub-batches                 */
  uint32_t reserved;
  uint64_t scanned;          /* join list entries tested                   */
  uint64_t descents;         /* partial matches extended (and counted ends)*/
  uint64_t probes;           /* membership probes (bitmap words, searches) */
  uint64_t last_count_entries; /* list entries read to build last counts   */
  uint64_t donations;        /* tasks split off to idle warps              */
  uint64_t model_bytes;      /* with SMG_FLAG_MODEL: per row of r mapped
                                vertices, 4r read + 8 + 8 x the anchor's
                                degree + (8 + 4 x degree) per other back
                                edge, plus 4r written where a row is made;
                                0 otherwise                               */
  uint64_t bfs_tasks;        /* tasks queued by breadth-first levels       */
} smg_batch_stats;
smg_status smg_match_batch(smg_ctx *ctx, const smg_graph *g,
                           const smg_plan *const *plans, uint32_t n,
                           const smg_match_opts *opts, uint64_t *counts,
                           smg_batch_stats *stats);

/* Autotuning.  Queries fall into shape classes: class = 4 * shape + size,
 * shape 0 tree (m = k-1), 2 dense (2m >= 3k), 1 sparse otherwise; size 0 for
 * k <= 5, 1 for 6..8, 2 for 9..12, 3 for 13+.  smg_autotune times up to 32
 * sample plans of each class (filter + join device time) under the join's
 * settings, one knob group at a time from the defaults: root candidates per
 * seeded task x shortest list worth splitting off to an idle warp (3 x 3),
 * then the slice length of long last-level lists (2,048 / 8,192 / 32,768),
 * then the cap on stored hoisted sets (256 / 1,024 / 4,096 entries), then
 * the breadth-first depth before the join turns depth-first (0 / 2 / 3).  It
 * keeps the fastest setting per class in the context and reports it; later
 * smg_match / smg_match_batch calls and servers on this context apply it. */
#define SMG_TUNE_CLASSES 12u
typedef struct smg_tune_entry {
  uint32_t shape_class;
  uint32_t root_chunk;
  uint32_t donate_min;
  uint32_t samples;  /* sample queries timed for this class (0: untuned) */
  float best_ms;     /* device time of the sample under the kept setting */
  float default_ms;  /* device time of the sample under the default setting */
  uint32_t split_len; /* last-level list slice length (0: 8,192)           */
  uint32_t hoist_cap; /* entries of a stored hoisted set (0: the warp's buffer) */
  uint32_t bfs_depth; /* breadth-first levels before depth-first (0: none) */
  uint32_t reserved;
} smg_tune_entry;
smg_status smg_autotune(smg_ctx *ctx, const smg_graph *g, const smg_plan *const *plans, uint32_t n,
                        smg_tune_entry *out /* [SMG_TUNE_CLASSES] or NULL */);
smg_status smg_set_tuning(smg_ctx *ctx, const smg_tune_entry *entries, uint32_t n);
/* Shape class of a plan (see above). */
uint32_t smg_plan_class(const smg_plan *p);

/* Filter only (for inspection): copies to host the per-vertex initial
 * candidate masks (bit u, filter.cu:529-535), the cluster bitmap
 * (num_vertices x num_words words, filter.cu:585-873) and the final
 * per-vertex candidate masks (filter.cu:1158-1232).  Any pointer may be
 * NULL. */
smg_status smg_filter_inspect(smg_ctx *ctx, const smg_graph *g,
                              const smg_plan *p, uint32_t *vmask0,
                              uint32_t *encodings, uint32_t *candmask);

/* ------------------------------------------------- allocation-free join */
/* No counterpart in the reference.  For callers that cannot call cudaMalloc
 * while they match: code running between the capture and the replay of a
 * larger application's CUDA graphs, callers whose device memory belongs to a
 * framework allocator, or real-time loops that must not allocate after
 * start-up.  Counts the embeddings of plan p from caller-owned device inputs:
 * candmask[num_vertices] (bit u set when data vertex v may take query vertex u,
 * as smg_filter_inspect's final masks) and roots[num_roots] (the candidates of
 * the plan's first matched vertex, view.root).  The join's scratch (a queue of
 * SMG_NOALLOC_MAX_TASKS tasks, its state, the query record and counters, about
 * 10 MB) is a fixed array in the library's device image; no call allocates.
 * The first call on a device looks that array up (cudaGetSymbolAddress) and
 * must come before any stream capture.  All calls on a device share the
 * array: each call clears it first, and calls that overlap on the GPU race.
 * Rejects more roots than data vertices (SMG_ERR_LIMIT). */
#define SMG_NOALLOC_MAX_TASKS 65536u
smg_status smg_join_noalloc(smg_ctx *ctx, const smg_graph *g, const smg_plan *p,
                            const uint32_t *candmask, const uint32_t *roots,
                            uint32_t num_roots, uint64_t *count);

/* ---------------------------------------------------------------- serving */
typedef struct smg_server smg_server;
typedef struct smg_server_config {
  uint64_t memory_budget_bytes; /* HBM for per-request state; 0 = auto      */
  uint32_t max_inflight;        /* queries resident at once; 0 = auto        */
  uint32_t max_query_vertices;  /* largest query accepted (2..32); 0 = 32.
                                   Smaller values give the join smaller task
                                   records and more resident warps.          */
} smg_server_config;
typedef struct smg_request_result {
  smg_status status;
  uint32_t reserved;
  uint64_t count;
  double submit_s;   /* host clock at submit                              */
  double start_s;    /* host clock at admission                           */
  double finish_s;   /* host clock when the count was read back           */
} smg_request_result;
smg_status smg_server_create(smg_ctx *ctx, const smg_graph *g,
                             const smg_server_config *cfg, smg_server **out);
smg_status smg_server_submit(smg_server *s, const smg_plan *p, uint64_t *ticket);
/* SMG_ERR_NOT_READY while the request is queued or running.  A finished
 * request's result is returned once: the server then forgets it, and a later
 * poll of the same ticket fails with SMG_ERR_INVALID. */
smg_status smg_server_poll(smg_server *s, uint64_t ticket, smg_request_result *out);
smg_status smg_server_cancel(smg_server *s, uint64_t ticket);
/* Drive the server until every submitted request has finished. */
smg_status smg_server_drain(smg_server *s);
/* Make progress once without blocking (admit, launch, retire). */
smg_status smg_server_step(smg_server *s);
/* Counters since creation (host clock for the times). */
typedef struct smg_server_stats {
  uint64_t slices;          /* join slices launched                          */
  uint64_t bells;           /* slices the doorbell asked to end early        */
  uint64_t admitted;        /* requests admitted                             */
  uint64_t retired_in_slice;/* requests retired from completion records     */
  uint64_t carried_tasks;   /* tasks moved into the next slice's queue       */
  double slice_s;           /* time from a slice's launch to its end seen    */
  double between_s;         /* time between slices (compaction, admission,
                               read-back) with requests active or waiting    */
  uint64_t admitted_live;   /* requests admitted into a running slice       */
} smg_server_stats;
smg_status smg_server_get_stats(const smg_server *s, smg_server_stats *out);
void smg_server_destroy(smg_server *s);

#ifdef __cplusplus
}
#endif
#endif /* SMG_H */
