/* ref_bfs <csr> <out.bin> <src>...  — runs the reference's runCPUBFS
 * (BFS/cpu_BFS/main.cpp:114-209) once per source and appends each depth array
 * (u32 x V, unreached = 0xFFFFFFFF) to out.bin.  Prints "ms <total>" on stderr.
 * OG_REF_SRC is the path of the reference's main.cpp (set by build_oracle.py). */
#include "ref_common.hpp"
#define main og_ref_unused_main
#include OG_REF_SRC
#undef main

int main(int argc, char **argv) {
  if (argc < 4) {
    fprintf(stderr, "usage: ref_bfs <csr> <out.bin> <src>...\n");
    return 2;
  }
  Graph<myEdgeType> G;
  G.readDataFromFile(argv[1]);
  std::ofstream sink("/dev/null");
  std::vector<uint> dist(G.vertexArrSize);
  double ms = 0;
  for (int a = 3; a < argc; a++) {
    uint *d = dist.data();
    const double t0 = og_ref_now_ms();
    runCPUBFS(G, (uint)strtoul(argv[a], nullptr, 10), d, 0xFFFFFFFFu, sink);
    ms += og_ref_now_ms() - t0;
    og_ref_write(argv[2], d, sizeof(uint) * G.vertexArrSize);
  }
  fprintf(stderr, "ms %.3f\n", ms);
  return 0;
}
