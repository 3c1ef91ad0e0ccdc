/* ref_pr <pr-csr> <out.bin>  — runs the reference's CPU PageRank
 * (PR/cpu/pr.cpp:112-165, pr_init + pr_cal<double>) and appends the f64 rank
 * array followed by the u32 round count.  OG_REF_SRC is the path of pr.cpp. */
#include "ref_common.hpp"
#define main og_ref_unused_main
#include OG_REF_SRC
#undef main

int main(int argc, char **argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: ref_pr <pr-csr> <out.bin>\n");
    return 2;
  }
  Graph<uint> G;
  G.readDataFromFile(argv[1]);
  double *out = (double *)calloc(G.vertexArrSize, sizeof(double));
  pr_init(G.vertexArrSize, (uint)G.edgeArrSize, G.edgeArray, G.nodePointers,
          G.degree, out);
  int round = 0;
  const double t0 = og_ref_now_ms();
  pr_cal<double>(G.vertexArrSize, G.edgeArray, G.nodePointers, G.degree,
                 G.outDegree, round, 0.85, out);
  const double ms = og_ref_now_ms() - t0;
  og_ref_write(argv[2], out, sizeof(double) * G.vertexArrSize);
  unsigned r = (unsigned)round;
  og_ref_write(argv[2], &r, sizeof(r));
  fprintf(stderr, "ms %.3f\n", ms);
  return 0;
}
