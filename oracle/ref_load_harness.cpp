// ref_load_harness.cpp — times the reference's own data-graph loader,
// readGraphToCPU2 (io.cu:24-108: token reads plus four std::map inserts per
// edge), on .in files, for comparison with the library's smg_read_graph.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build_ref.sh compiles this file together
// with the reference's sources, where they lie, into oracle/_ref/ref_load,
// at -O3 (the reference's CMakeLists.txt:10 builds Debug; -O3 is the faster
// build of its loader).  No CUDA API is called.
//
//   oracle/_ref/ref_load data.in [more.in ...]
// prints one JSON object per file: vertices, edges and wall seconds.
#include <chrono>
#include <cstdio>

#include "cpuGraph.h"
#include "io.cuh"

int main(int argc, char **argv) {
  for (int a = 1; a < argc; ++a) {
    const auto t0 = std::chrono::steady_clock::now();
    cpuGraph *g = new cpuGraph;
    readGraphToCPU2(g, argv[a]);
    const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf("{\"file\": \"%s\", \"num_v\": %lu, \"num_e\": %lu, \"seconds\": %.3f}\n", argv[a],
                static_cast<unsigned long>(g->num_v), static_cast<unsigned long>(g->num_e), s);
    std::fflush(stdout);
    // the graph is left allocated, as main.cu leaves its graphs (freeing its
    // maps would add their teardown to nothing measured here)
  }
  return 0;
}
