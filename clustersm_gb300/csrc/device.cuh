// device.cuh — device-side data layout shared by the filter, the join and the
// C-ABI implementation.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "host.h"

namespace smg {

constexpr uint32_t kMaxK = SMG_MAX_QUERY_VERTICES;  // query vertices (u-bitmask width)
constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr int kWarp = 32;

// Bounds checks of the self-checking build (-DSMG_CHECKED): a failed check
// records (site, value, limit) in a per-translation-unit device word (first
// failure wins) and the caller skips the access.  In normal builds every
// check is `true` and compiles away.
#ifdef SMG_CHECKED
#define SMG_DCHECK(cond, site, a, b) ::smg::dcheck((cond), (site), (a), (b))
#else
#define SMG_DCHECK(cond, site, a, b) true
#endif

// CUDA status -> smg_status with a message naming the call site.
smg_status cuda_fail(cudaError_t e, const char *what);
#define SMG_CUDA(call)                                                  \
  do {                                                                  \
    cudaError_t e_ = (call);                                            \
    if (e_ != cudaSuccess) return ::smg::cuda_fail(e_, #call);          \
  } while (0)

// ------------------------------------------------------------ resident graph
// The data graph lives in HBM for as long as the smg_graph handle.  Neighbour
// lists are sorted so that non-tree edges are checked by binary search.
struct DevGraph {
  uint32_t n = 0;
  uint64_t m2 = 0;            // directed adjacency entries (2|E|)
  uint32_t num_labels = 0;    // largest label + 1
  uint32_t nlc_stride = 0;    // bytes per vertex in `nlc` (multiple of 16)
  uint32_t max_degree = 0;
  uint32_t *off = nullptr;    // [n+1]  (2|E| < 2^32 is required)
  uint32_t *adj = nullptr;    // [2|E|] sorted per vertex
  uint32_t *label = nullptr;  // [n]
  // [n][nlc_stride] neighbour-label counts, saturated at 255, one row per
  // position of `lverts` (row p: vertex lverts[p]), so that a sweep over a
  // label group reads consecutive rows; ldeg[p] is that vertex's degree
  uint8_t *nlc = nullptr;
  uint32_t *ldeg = nullptr;   // [n]
  uint32_t *hub_of = nullptr; // [n] index of the vertex's neighbour bitmap, or kNone
  uint32_t *hub_bits = nullptr;  // [num_hubs][hub_words]
  uint32_t num_hubs = 0;
  uint64_t hub_words = 0;
  // Label index: every neighbour list again, ordered by (label bucket, id),
  // where bucket(l) = min(l, lab_buckets - 1); and, for the vertices of high
  // degree, where each bucket's run starts (relative to off[v]; lab_buckets + 1
  // entries, the last = degree).  The join scans only the run of the label it
  // needs; membership tests keep the id-ordered `adj`.
  uint32_t *adjl = nullptr;     // [2|E|]
  uint32_t *lab_of = nullptr;   // [n] row of the vertex's run table, or kNone
  uint32_t *lab_off = nullptr;  // [indexed][lab_buckets + 1]
  uint32_t lab_buckets = 0, lab_indexed = 0;
  // When every bucket holds one label (at most kMaxLabels labels): the rank of
  // each adjl entry within its label's vertex group (its position in lverts
  // after the group's start).  A join level that scans a label run tests its
  // entries in the query's rank-indexed candidate rows (JoinQuery::crow),
  // whose rows are only as long as the label's group.  Null: not built.
  uint32_t *adjr = nullptr;     // [2|E|]
  // Optional hub bitmap layout by label bucket (SMG_HUB_LAYOUT=label, with
  // the label index): the bit of neighbour w sits at word
  // bucket_word_off[bucket(w)] + lab_rank[w] / 32 of the hub's row, where
  // lab_rank[w] is w's index among the vertices of its bucket (in id order).
  // A probe for a candidate of one label then touches that label's
  // n_label / 8 bytes of the row instead of all n / 8, at the price of one
  // more dependent load.
  uint32_t *lab_rank = nullptr;         // [n]
  uint32_t *bucket_word_off = nullptr;  // [lab_buckets + 1]
  uint64_t hub_row_words = 0;           // bucket_word_off[lab_buckets]
  bool hub_by_label = false;            // hub rows use the layout above (else by id)
  std::vector<uint64_t> label_count;  // vertices per label (host copy)
  // Vertex ids grouped by label (ascending within a label) for labels below
  // kMaxLabels, and where each label's group starts (host and device copies):
  // the per-query filter sweeps visit only the vertices of the query's labels.
  uint32_t *lverts = nullptr;              // [n]
  std::vector<uint32_t> lvert_start;       // [min(num_labels, kMaxLabels) + 1]
  // Device copies for the filter, whose per-query masks and cluster bitmaps
  // are indexed by position in lverts: where each label's group starts
  // (lvert_start), and each vertex's position (the inverse of lverts).
  uint32_t *lvstart = nullptr;             // [lvert_start.size()]
  uint32_t *pos_of = nullptr;              // [n]
  uint64_t bytes = 0;
};

// ------------------------------------------------------ per-query filter plan
// One star / merge / combine step of the cluster bitmap, flattened for the
// device.  Slot bits of a cluster are set per 32-bit word: for a word group,
// `qmask` holds the query vertices whose slot lies in that word and `pos[u]`
// the bit of u's slot inside it.
struct WordGroup {
  uint32_t word;   // word index within a vertex's num_words words
  uint32_t qmask;  // query vertices with a slot in this word (neighbour slots)
  uint8_t pos[kMaxK];
};

struct ClusterStep {
  uint32_t kind;          // 0 star, 1 merge, 2 combine
  uint32_t core;          // query vertex whose candidates are walked
  uint32_t core_slot;     // slot of the core in this cluster
  uint32_t left_pos, right_pos;  // merge: slots tested on the candidate
  uint32_t type;          // combine: 0 new cluster, 1 in place
  uint32_t num_groups;    // word groups of the neighbour slots (<= 2)
  WordGroup groups[2];
  // combine only, in the batch's aux array:
  //   aux[others_off + o]  core slot of the o-th other cluster
  //   from aux[targets_off], per neighbour slot of this cluster:
  //     slot, nsrc, then the nsrc slots holding the same vertex in the others
  uint32_t num_others, others_off;
  uint32_t num_targets, targets_off;
};

// Kernels of one launch walk the candidates of a group of steps sharing a
// core: merges with the same core in one layer must see each other's
// removals in cluster order (filter.cu:718).
struct StepGroup {
  uint32_t query;        // index into the batch
  uint32_t core;
  uint32_t first, count; // steps [first, first+count) of the step array
  // Labels of the query vertices whose slots the group's steps set or test on
  // neighbours (one byte each, nlab of them; nlab = 0: too many, walk whole
  // lists).  Only neighbours with these labels can change, so a candidate
  // with a label run table walks just those runs.
  uint32_t nlab;
  uint8_t lab[4];
};

// Per-query device state (filter scratch and join inputs).
struct QueryDev {
  uint32_t k = 0, words = 0, nvlq = 0;
  uint32_t *vmask = nullptr;   // [n]: initial masks, overwritten by final masks
  uint32_t *enc = nullptr;     // [n * words] cluster bitmap
  uint32_t *cand = nullptr;    // candidate lists of the initial filter, [k] segments
  uint32_t *cand_cnt = nullptr;// [k] (device), entries used per segment
  std::vector<uint64_t> cand_off;  // [k+1] segment offsets (host)
  uint32_t *roots = nullptr;   // root candidate list (after the bitmap filter)
};

// Query-side constants the filter kernels read (one per query in a batch).
struct FilterQuery {
  uint32_t k, words, nvlq;
  uint32_t label[kMaxK];
  uint32_t deg[kMaxK];
  uint32_t nnlc[kMaxK];          // non-zero neighbour-label counts of u
  uint16_t nlc_label[kMaxK][kMaxK];
  uint8_t nlc_count[kMaxK][kMaxK];
  uint32_t last_slot[kMaxK];
  uint32_t root;
  uint64_t cand_off[kMaxK + 1];
  // vmask (initial, then final candidate masks) and enc (the cluster
  // bitmap, `words` per vertex) are indexed by the vertex's position in
  // DevGraph::lverts, so that a sweep over a label group reads and writes them
  // in order; cand holds positions too; roots holds vertex ids (the join's)
  uint32_t *vmask, *enc, *cand, *cand_cnt, *roots, *num_roots;
  uint64_t root_cap;             // entries `roots` can hold
  unsigned long long *stat;       // [0] sum over u of final |C(u)|, [1] walk list entries
  uint32_t *cbits;               // the join's candidate bitmaps, written by collect (null: none)
  uint64_t cwords;               // words per bitmap row, ceil(n / 32)
  // rank-indexed rows after the k id-indexed ones (cbits + (k + u) * cwords,
  // bit r: the r-th vertex of u's label group is a candidate of u); 0: none
  uint32_t rank_rows;
  // the query's distinct labels present in the graph: their vertex groups in
  // DevGraph::lverts ([grp_lo, grp_hi)) and the query vertices carrying them
  uint32_t ngrp;
  uint32_t grp_lo[kMaxK], grp_hi[kMaxK], grp_mask[kMaxK];
};

// Query-side constants the join reads.
struct JoinQuery {
  uint32_t k;
  uint32_t order[kMaxK];      // query vertex matched at each level
  uint32_t back_mask[kMaxK];  // earlier levels adjacent to the level's vertex
  uint32_t same_label[kMaxK]; // earlier levels with the same label (injectivity)
  // [n] final candidate masks (bit u: may take query vertex u); by vertex id
  // when the caller provides them (smg_join_noalloc), by position in
  // DevGraph::lverts when the filter wrote them (the join then tests cbits)
  const uint32_t *candmask;
  // The same candidates as one bitmap per query vertex, cbits[u * cwords +
  // v / 32] bit v % 32, built after the filter: a random candidate test then
  // reads a 512 KB row (at 2^22 vertices) instead of a 16 MB mask array, so
  // the rows of many concurrent queries stay in L2.  Null: the join tests
  // candmask (caller-provided masks, smg_join_noalloc).
  uint32_t *cbits;
  uint64_t cwords;
  // The same candidates by rank within the query vertex's label group:
  // crow[u * cwords + r / 32] bit r % 32 for the r-th vertex of u's label
  // (DevGraph::lverts order).  Only the first |label group| / 32 words of a
  // row are used, so the rows a query's label runs touch are a fraction of
  // cbits' (a tenth on average under Zipf labels) and stay in L2 longer.
  // Null: every test reads cbits.
  const uint32_t *crow;
  // Count-only runs with fast_last set: the last level's per-vertex
  // neighbour counts by vertex id (see k_last_counts), written over the
  // query's cluster bitmap, which nothing reads after the filter.
  uint32_t *lastcnt;
  const uint32_t *roots;      // root candidates
  const uint32_t *num_roots;  // device counter
  unsigned long long *count;  // result
  uint32_t *emb;              // optional embedding rows [emb_cap][k]
  unsigned long long emb_cap;
  unsigned long long *emb_count;
  unsigned long long count_limit;  // 0: none; else stop once the count exceeds it
  uint32_t *over;             // set to 1 when the count exceeded count_limit (or the work work_limit)
  unsigned long long work_limit;   // 0: none; else stop once the join has taken more steps
  unsigned long long *work;   // join steps taken (under a work limit)
  unsigned long long *pending;  // tasks of this query queued or running
  uint32_t root_chunk;        // root candidates per seeded task (0: from max_seed_tasks)
  uint32_t donate_min;        // shortest list worth splitting off (0: launch default)
  uint32_t split_len;         // last-level lists are cut into slices this long (0: 8,192)
  uint32_t hoist_cap;         // stored hoisted sets hold at most this many (0: the warp's buffer)
  // Breadth-first prefix: a warp that fills a batch of accepted candidates
  // at a level below bfs_depth (and below the last two levels) queues every
  // one as a task instead of descending into it, while the launch's
  // breadth-first budget of queue slots lasts; deeper levels run depth-first.
  // 0: depth-first from the root tasks.
  uint32_t bfs_depth;
  // Completion notice (serving; null: none).  The warp that finishes the
  // query's last task writes the final count to done_count and then `gen` to
  // done_gen, both in host-mapped memory, so the host sees the result while
  // the slice is still running.
  unsigned long long *done_count;
  uint32_t *done_gen;
  uint32_t gen;
  // Label bucket of each level's query vertex, for the label index (valid
  // when use_labels is set; otherwise the join scans whole lists).
  uint32_t level_bucket[kMaxK];
  uint32_t use_labels;
  // the vertex group (DevGraph::lverts range) of the label of the fast_last
  // back neighbour's query vertex: its candidates all lie there
  uint32_t lc_lo, lc_hi;
  // 1 + the level of the last vertex's only back neighbour when the last
  // level can be counted from per-vertex neighbour counts (one back edge and
  // cbits present); 0: the last level is always scanned.
  uint32_t fast_last;
};

#if defined(SMG_CHECKED) && defined(__CUDACC__)
// Defined once per translation unit that includes this header.
static __device__ unsigned long long g_check_record[4];
__device__ __forceinline__ bool dcheck(bool ok, int site, unsigned long long a, unsigned long long b) {
  if (ok) return true;
  if (atomicCAS(&g_check_record[0], 0ull, static_cast<unsigned long long>(site)) == 0ull) {
    g_check_record[1] = a;
    g_check_record[2] = b;
  }
  return false;
}
#endif

}  // namespace smg
