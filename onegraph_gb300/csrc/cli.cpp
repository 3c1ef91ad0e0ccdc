// cli.cpp — the per-algorithm programs BFS_OneGraph / SSSP_OneGraph /
// CC_OneGraph / PR_OneGraph (one source, OG_CLI_ALGO selects the program).
//
// Argument handling follows ArgumentParser::Parse (BFS/oneGraph_BFS/
// ArgumentParser.h:40-73): argv is read in (flag, value) pairs from index 1.
// Accepted flags: -f <csr>, --type/-type <bfs|sssp|cc|pr>, -r <source>,
// --method/-method <0 OneGraph | 1 Subway | 2 USM> (parsed but unused by the
// reference), --adviseK/-adviseK/--advisek/-advisek <ratio>,
// plus --budget <bytes|NNG|NNM>, --dump <file>, --sources <n>,
// --direct <0|1>, --json <0|1>, --threshold <pr delta>, --device <ordinal>,
// --symmetric <1|0|check> (1 asserts that every edge has its reverse, which
// lets CC use union-find and BFS expand large levels bottom-up; "check"
// verifies it on the host first; without the flag a loaded file counts as
// not known to be symmetric and the reference's algorithms run).
// Differences from the reference, on purpose: a --type naming another
// algorithm is an error (exit 2) instead of a silent exit 0 (main.cpp:9-13),
// and -r is honoured by BFS when given (the reference BFS always walks
// findbignode, CalculateOpt.h:26-31; that remains the behaviour without -r).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/onegraph.h"

#ifndef OG_CLI_ALGO
#define OG_CLI_ALGO 0
#endif

static const char *kNames[] = {"bfs", "sssp", "cc", "pr"};

static uint64_t parse_bytes(const char *s) {
  char *end = nullptr;
  double v = strtod(s, &end);
  if (end && (*end == 'G' || *end == 'g')) v *= 1024.0 * 1024.0 * 1024.0;
  else if (end && (*end == 'M' || *end == 'm')) v *= 1024.0 * 1024.0;
  else if (end && (*end == 'K' || *end == 'k')) v *= 1024.0;
  return (uint64_t)v;
}

struct Args {
  std::string input, algo, dump, symmetric;
  int source = 0;
  bool has_source = false;
  double advisek = 0.0;
  uint64_t budget = 0;
  int sources = 5;  // CalculateOpt.h:7 testTimes
  int direct = 0, json = 0, device = 0;
  int method = 0;  // 0 OneGraph/Ascetic, 1 Subway (no static region, staged), 2 USM (no static region, pageable host reads)
  double threshold = 0.001;
};

static bool parse(int argc, char **argv, Args &a) {
  for (int i = 1; i < argc - 1; i += 2) {
    const char *k = argv[i], *v = argv[i + 1];
    if (!strcmp(k, "-f")) a.input = v;
    else if (!strcmp(k, "--type") || !strcmp(k, "-type")) a.algo = v;
    else if (!strcmp(k, "-r")) {
      a.source = atoi(v);
      a.has_source = true;
    } else if (!strcmp(k, "--method") || !strcmp(k, "-method")) {
      a.method = atoi(v);
    } else if (!strcmp(k, "--adviseK") || !strcmp(k, "-adviseK") || !strcmp(k, "--advisek") ||
               !strcmp(k, "-advisek"))
      a.advisek = atof(v);
    else if (!strcmp(k, "--budget")) a.budget = parse_bytes(v);
    else if (!strcmp(k, "--dump")) a.dump = v;
    else if (!strcmp(k, "--sources")) a.sources = atoi(v);
    else if (!strcmp(k, "--direct")) a.direct = atoi(v);
    else if (!strcmp(k, "--json")) a.json = atoi(v);
    else if (!strcmp(k, "--threshold")) a.threshold = atof(v);
    else if (!strcmp(k, "--device")) a.device = atoi(v);
    else if (!strcmp(k, "--symmetric")) a.symmetric = v;
    else {
      fprintf(stderr, "unknown flag %s\n", k);
      return false;
    }
  }
  return !a.input.empty();
}

static int die(const char *what, int rc) {
  fprintf(stderr, "%s failed (status %d): %s\n", what, rc, og_last_error());
  return 1;
}

static void print_stats(const og_stats &st, uint32_t eb, bool json, const char *algo, long src) {
  printf("totalProcess %.3f ms\n", st.ms_total);
  printf("staticProcess %.3f ms\noverloadProcess %.3f ms\npreProcess %.3f ms\n", st.ms_static,
         st.ms_dynamic, st.ms_compact);
  printf("iterations : %u\nnodeSum : %llu\nstaticnodeSum : %llu\n", st.iterations,
         (unsigned long long)st.frontier_sum, (unsigned long long)st.static_vertices);
  printf("move overload size : %llu MB\n", (unsigned long long)(st.edges_dynamic * eb / 1024 / 1024));
  if (json)
    printf("{\"algo\": \"%s\", \"source\": %ld, \"ms_total\": %.4f, \"ms_static\": %.4f, "
           "\"ms_dynamic\": %.4f, \"ms_compact\": %.4f, \"iterations\": %u, \"node_sum\": %llu, "
           "\"edges_static\": %llu, \"edges_dynamic\": %llu, \"link_bytes\": %llu, "
           "\"chunks\": %u, \"residual\": %.3e}\n",
           algo, src, st.ms_total, st.ms_static, st.ms_dynamic, st.ms_compact, st.iterations,
           (unsigned long long)st.frontier_sum, (unsigned long long)st.edges_static,
           (unsigned long long)st.edges_dynamic, (unsigned long long)st.link_bytes, st.chunks,
           st.residual);
}

int main(int argc, char **argv) {
  Args a;
  const char *own = kNames[OG_CLI_ALGO];
  if (!parse(argc, argv, a)) {
    fprintf(stderr,
            "usage: %s -f <csr> [--type %s] [-r <source>] [--advisek <ratio>] [--budget <bytes>] "
            "[--dump <file>] [--sources <n>] [--direct 0|1] [--json 0|1]\n",
            argv[0], own);
    return 2;
  }
  if (a.algo.empty()) a.algo = own;
  if (a.algo != own) {
    fprintf(stderr, "%s: --type %s is not this program's algorithm (%s)\n", argv[0], a.algo.c_str(), own);
    return 2;
  }
  printf("arguments.algo %s\n", own);
  const int kind = OG_CLI_ALGO == OG_ALGO_SSSP ? OG_GRAPH_WEIGHTED
                   : OG_CLI_ALGO == OG_ALGO_PR ? OG_GRAPH_PR
                                               : OG_GRAPH_PLAIN;
  og_graph *g = nullptr;
  int rc = og_graph_load(a.input.c_str(), kind, &g);
  if (rc) return die("og_graph_load", rc);
  if (a.symmetric == "1" || a.symmetric == "0") {
    og_graph_set_symmetric(g, a.symmetric == "1" ? 1 : 0);
  } else if (a.symmetric == "check") {
    int sym = 0;
    rc = og_graph_symmetric(g, &sym);
    if (rc) return die("og_graph_symmetric", rc);
    printf("symmetric %d\n", sym);
  } else if (!a.symmetric.empty()) {
    fprintf(stderr, "--symmetric takes 1, 0 or check\n");
    return 2;
  }
  uint64_t V = 0, E = 0;
  og_graph_info(g, &V, &E, nullptr, nullptr, nullptr, nullptr);
  printf("vertexArrSize = %llu edgeArrSize = %llu\n", (unsigned long long)V, (unsigned long long)E);
  og_config cfg;
  memset(&cfg, 0, sizeof cfg);
  cfg.budget_bytes = a.budget;
  cfg.advisek = a.advisek;
  cfg.flags = a.direct ? OG_CFG_DIRECT : 0;
  if (a.method == 1) cfg.flags = OG_CFG_NO_STATIC;
  if (a.method == 2) cfg.flags = OG_CFG_NO_STATIC | OG_CFG_DIRECT | OG_CFG_NO_PIN;
  cfg.device = a.device;
  og_engine *e = nullptr;
  rc = og_engine_create(g, &cfg, &e);
  if (rc) return die("og_engine_create", rc);
  og_plan plan;
  og_engine_plan(e, &plan);
  printf("availMemory %llu adviseK %f max_partition_size %llu static vertices %u static edges %llu "
         "chunk %llu\n",
         (unsigned long long)plan.budget_bytes, plan.advisek, (unsigned long long)plan.max_partition,
         plan.static_vertices, (unsigned long long)plan.static_edges,
         (unsigned long long)plan.chunk_edges);
  std::vector<uint32_t> out(V);
  og_stats st;
  FILE *dump = nullptr;
  if (!a.dump.empty() && !(dump = fopen(a.dump.c_str(), "wb"))) {
    fprintf(stderr, "cannot create %s\n", a.dump.c_str());
    return 1;
  }
  if (OG_CLI_ALGO == OG_ALGO_BFS || OG_CLI_ALGO == OG_ALGO_SSSP) {
    std::vector<uint32_t> srcs;
    if (a.has_source || OG_CLI_ALGO == OG_ALGO_SSSP) {
      srcs.push_back((uint32_t)a.source);
    } else {
      uint32_t last = 0;  // CalculateOpt.h:25-31
      for (int i = 0; i < a.sources; i++) srcs.push_back(last = og_graph_findbignode(g, last));
    }
    for (size_t t = 0; t < srcs.size(); t++) {
      printf("----------testIndex = %zu-----------\nsourceNode %u\n", t, srcs[t]);
      rc = OG_CLI_ALGO == OG_ALGO_BFS ? og_bfs(e, srcs[t], out.data(), &st)
                                      : og_sssp(e, srcs[t], out.data(), &st);
      if (rc) return die(own, rc);
      print_stats(st, plan.edge_bytes, a.json, own, (long)srcs[t]);
      if (OG_CLI_ALGO == OG_ALGO_SSSP) {  // SSSP/oneGraph/CalculateOpt.h:173-178
        for (uint32_t i = 0; i < 10 && i < V; i++) printf("%u\t", out[i]);
        printf("...%u\n", out[V - 1]);
      }
      if (dump) fwrite(out.data(), 4, V, dump);
    }
  } else if (OG_CLI_ALGO == OG_ALGO_CC) {
    rc = og_cc(e, out.data(), &st);
    if (rc) return die(own, rc);
    print_stats(st, plan.edge_bytes, a.json, own, -1);
    if (dump) fwrite(out.data(), 4, V, dump);
  } else {
    std::vector<float> rank(V);
    rc = og_pr(e, rank.data(), a.threshold, 0, &st);
    if (rc) return die(own, rc);
    print_stats(st, plan.edge_bytes, a.json, own, -1);
    if (dump) fwrite(rank.data(), 4, V, dump);
  }
  if (dump) fclose(dump);
  og_engine_destroy(e);
  og_graph_free(g);
  return 0;
}
