// ref_plan_harness.cpp — drives the reference's own host-side query
// preprocessing and prints what it produced, one JSON object per query file.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build_ref.sh compiles this file together
// with the reference's sources, where they lie, into oracle/_ref/ref_plan.
// Calls (reference file:line):
//   readGraphToCPU2   io.cu:24       (query read twice, as main.cu:55-56)
//   decycle           decycle.cpp:6
//   clustering        filter.cu:127  (vertex cover filter.cu:43, cluster CSR structure.cu:219)
//   getBFSEdgeOrder   order.cpp:150, root as main.cu:144
// No CUDA API is called, so the binary runs on a host without a GPU.  The
// globals copyMeta would set (io.cu:267-269) are assigned directly.
#include <cstdio>
#include <set>

#include "cpuGraph.h"
#include "decycle.h"
#include "filter.cuh"
#include "globals.cuh"
#include "io.cuh"
#include "order.h"
#include "structure.cuh"

template <typename T>
static void arr(const char *name, const T *a, long n, bool comma = true) {
  std::printf("\"%s\":[", name);
  for (long i = 0; i < n; ++i) std::printf("%s%ld", i ? "," : "", static_cast<long>(a[i]));
  std::printf("]%s", comma ? "," : "");
}

int main(int argc, char **argv) {
  std::printf("[");
  for (int a = 1; a < argc; ++a) {
    cpuGraph hq_backup, hq;
    readGraphToCPU2(&hq_backup, argv[a]);
    readGraphToCPU2(&hq, argv[a]);
    NUM_VQ = hq_backup.num_v;
    NUM_EQ = hq_backup.num_e;
    NUM_VLQ = hq_backup.largest_l + 1;
    decycle(&hq);
    cpuCluster *clusters = nullptr;
    encodingMeta meta;
    clustering(&hq, clusters, &meta);
    const vtype root = meta.query_us_compact_[meta.cluster_offsets_[meta.num_clusters - 1]];
    etype *order = new etype[NUM_EQ];
    getBFSEdgeOrder(&hq_backup, order, root);

    std::printf("%s{\"file\":\"%s\",", a > 1 ? "," : "", argv[a]);
    arr("tree_offsets", hq.offsets_, hq.num_v + 1);
    arr("tree_neighbors", hq.neighbors_, hq.offsets_[hq.num_v]);
    arr("tree_degrees", hq.outdeg_, hq.num_v);
    std::printf("\"num_clusters\":%u,\"num_layers\":%u,", meta.num_clusters, meta.num_layers);
    arr("cluster_offsets", meta.cluster_offsets_, meta.num_clusters + 1);
    arr("slots", meta.query_us_compact_, meta.num_total_us);
    arr("num_clusters_per_layer", meta.num_clusters_per_layer_, meta.num_layers);
    arr("layer_offsets", meta.layer_offsets_, meta.num_layers + 1);
    arr("merge_layer", meta.merged_cluster_layer_, meta.merge_count);
    arr("merge_left", meta.merged_cluster_left_, meta.merge_count);
    arr("merge_right", meta.merged_cluster_right_, meta.merge_count);
    arr("merge_vertex", meta.merged_cluster_vertex_, meta.merge_count);
    arr("combine_out", meta.combine_cluster_out_, meta.combine_cnt);
    arr("combine_type", meta.combine_type_, meta.combine_cnt);
    std::printf("\"combine_others\":[");
    for (unsigned c = 0; c < meta.combine_cnt; ++c) {
      std::printf("%s[", c ? "," : "");
      bool first = true;
      for (int x : meta.combine_clusters_other_[c]) {
        std::printf("%s%d", first ? "" : ",", x);
        first = false;
      }
      std::printf("]");
    }
    std::printf("],\"root\":%u,\"edge_order\":[", root);
    for (unsigned e = 0; e < NUM_EQ; ++e)
      std::printf("%s[%u,%u]", e ? "," : "", hq_backup.evv[order[e]].first, hq_backup.evv[order[e]].second);
    std::printf("]}\n");
    delete[] order;
  }
  std::printf("]\n");
  return 0;
}
