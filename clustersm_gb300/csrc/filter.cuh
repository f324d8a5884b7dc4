// filter.cuh — host interface of the candidate filter (filter.cu).
#pragma once

#include <vector>

#include "device.cuh"

namespace smg {

// Neighbour-label counts are kept for labels below this bound.
constexpr uint32_t kMaxLabels = 256;
// Neighbour lists longer than this are walked by several warps, one chunk each.
constexpr uint32_t kWalkChunk = 2048;

// Chunks of long neighbour lists queued by one walk phase for the chunk pass.
// `count` points at this phase's counter (zeroed before the run; the walk
// launcher gives each phase its own); items are (group, vertex, passed-step
// mask, first adjacency index).  Bit 31 of an item's group marks an index
// into the label-ordered lists (adjl) rather than the id-ordered ones.
struct WalkOverflow {
  unsigned int *count;
  uint32_t cap;
  uint4 *items;
  uint32_t n, num_groups;  // data vertices and the phase's step groups (bounds checks)
  uint64_t m2;             // adjacency entries
  // the graph's label index (set by launch_walks; adjl null: none)
  const uint32_t *adjl, *lab_of, *lab_off;
  uint32_t lab_buckets;
  // positions in the label groups (set by launch_walks): lverts, its inverse
  // pos_of, the groups' starts lvstart (num_groups_l + 1 entries) and the
  // entries' ranks within their label adjr (null: look positions up in pos_of)
  const uint32_t *lverts, *pos_of, *lvstart, *adjr;
  uint32_t num_groups_l;
};

// Steps of the cluster bitmap for a batch of queries, grouped into phases:
// phase 0 = stars of layer 0; phase 2l-1 = merges of layer l; phase 2l =
// combines of layer l.  Queries of a batch share the phases, so a batch runs
// 2 * max_layers - 1 walk launches whatever its size.
struct FilterBatch {
  std::vector<ClusterStep> steps;
  std::vector<uint32_t> aux;
  std::vector<std::vector<StepGroup>> phases;
};

// The steps of a batch in device memory.
struct FilterDev {
  void *buf = nullptr;
  size_t cap = 0;
  std::vector<char> host;
  ClusterStep *steps = nullptr;
  StepGroup *groups = nullptr;
  uint32_t *aux = nullptr;
  uint32_t *chunk_start = nullptr;  // per phase: its walk work list (k_walk_plan), ng + 1 entries
  std::vector<uint32_t> phase_first, phase_count;
  smg_status upload(const FilterBatch &fb, cudaStream_t s);
  // Grows the device buffer ahead of time, so that an upload of at most
  // `bytes` allocates nothing (a cudaFree would wait for every running kernel).
  smg_status reserve(size_t bytes);
  FilterDev() = default;
  FilterDev(const FilterDev &) = delete;
  FilterDev &operator=(const FilterDev &) = delete;
  ~FilterDev();
};

smg_status launch_build_nlc(DevGraph &g, cudaStream_t s, int num_sms);
// Zeroes bytes (a multiple of 16, 16-byte aligned) with 256-thread blocks.
smg_status launch_zero(void *p, size_t bytes, cudaStream_t s, int num_sms);
// Zeroes nr disjoint byte ranges of base, sorted by offset: range r starts at
// byte off[r] and holds prefix[r + 1] - prefix[r] 4-byte words (both arrays
// in device memory, prefix[0] = 0).
smg_status launch_zero_ranges(char *base, const uint64_t *prefix, const uint64_t *off, uint32_t nr, cudaStream_t s,
                              int num_sms);
// Query constants (not the device pointers) of one plan.
smg_status fill_filter_query(const Plan &P, const DevGraph &g, FilterQuery &fq);
smg_status append_filter_steps(const Plan &P, uint32_t query_index, FilterBatch &fb);
// NLC filter, every walk phase, then collect, for `nq` queries whose
// FilterQuery records are at d_qs (device).  Candidate counters, the bitmap
// and the root counters must be zero on entry.
smg_status launch_nlc_filter(const DevGraph &g, const FilterQuery *d_qs, uint32_t nq, cudaStream_t s, int num_sms);
smg_status launch_walks(const DevGraph &g, const FilterQuery *d_qs, const FilterDev &fd, WalkOverflow ov,
                        cudaStream_t s, int num_sms);
smg_status launch_collect(const DevGraph &g, const FilterQuery *d_qs, uint32_t nq, cudaStream_t s, int num_sms);
smg_status launch_filter(const DevGraph &g, const FilterQuery *d_qs, uint32_t nq, const FilterDev &fd,
                         WalkOverflow ov, cudaStream_t s, int num_sms);

}  // namespace smg
