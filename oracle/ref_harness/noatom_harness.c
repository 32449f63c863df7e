/*
 * noatom_harness.c -- drives the reference Seq-kClist++ program's own functions
 * (kCDensestNoAtom.c, compiled from the reference sources where they lie, with
 * its main() renamed) and prints exact results for golden vectors.
 *
 * TEST INFRASTRUCTURE ONLY (builds into oracle/_ref/, never shipped).
 *
 * usage: noatom_harness p T k edgelist mode
 *   mode "seq":   the reference's CDF_CliqueEnum(FRANK_WOLFE) loop (:381-396) with
 *                 p threads; at each power of two prints CDF_FindDensestSubset.
 *   mode "edge":  per-root-edge streams: each root edge's chain runs from the
 *                 pass-start r through the reference's MakeSubgraph and
 *                 CDF_CliqueEnumThread; the per-edge increments are summed.
 * output lines:  "graph n e core", "info T n m density(%a) ub(%a)", "rho v0 v1 ...",
 *                "edge s t" (the DAG root edges, sorted).
 */
#define main kclpp_reference_main
#include "kCDensestNoAtom.c"
#undef main

static void dump_info(unsigned T, DensestSubsetInfo info) {
  printf("info %u %u %u %a %a\n", T, info.n, info.m, info.density, info.ub);
}

int main(int argc, char **argv) {
  if (argc < 6) { fprintf(stderr, "usage: %s p T k edgelist seq|edge\n", argv[0]); return 2; }
  unsigned p = atoi(argv[1]);
  unsigned num_iter = atoi(argv[2]);
  unsigned char k = atoi(argv[3]);
  char *file_name = argv[4];
  int edge_mode = strcmp(argv[5], "edge") == 0;
  omp_set_num_threads(edge_mode ? 1 : p);
  EdgeList *el = ReadEdgeList(file_name);
  SortByCore(el);
  Relabel(el);
  Graph *g = MakeGraph(el);
  printf("graph %u %u %u\n", g->n, g->e, g->core);
  for (unsigned i = 0; i < g->e; ++i) printf("edge %u %u\n", g->edges[i].s, g->edges[i].t);
  AllocCdf(g, k);
  for (unsigned i = 0; i < g->n; ++i) rho[i] = 0;
  unsigned long long *next = calloc(g->n + 1, sizeof(unsigned long long));
  Subgraph *sg = AllocSubgraph(g, k);
  for (unsigned T = 1, t = 1; T <= num_iter; T <<= 1) {
    for (; t <= T; ++t) {
      if (!edge_mode) {
        CDF_CliqueEnum(g, k, FRANK_WOLFE);
        continue;
      }
      for (unsigned i = 0; i < g->n; ++i) { rho_p[i] = rho[i]; next[i] = rho[i]; }
      for (unsigned i = 0; i < g->e; ++i) {
        unsigned s = g->edges[i].s, tt = g->edges[i].t;
        unsigned ngw = rho_p[tt] < rho_p[s] ? tt : s;
        MakeSubgraph(g, g->edges[i], sg, k);
        CDF_CliqueEnumThread(sg, k, k - 2, FRANK_WOLFE, ngw);
        next[s] += rho_p[s] - rho[s]; rho_p[s] = rho[s];
        next[tt] += rho_p[tt] - rho[tt]; rho_p[tt] = rho[tt];
        for (unsigned j = 0; j < sg->n[k - 2]; ++j) {
          unsigned x = id_sg2g[j];
          next[x] += rho_p[x] - rho[x];
          rho_p[x] = rho[x];
        }
      }
      for (unsigned i = 0; i < g->n; ++i) rho[i] = next[i];
    }
    for (unsigned i = 0; i < g->n; ++i) rho_tentative[i] = 0;
    DensestSubsetInfo info = CDF_FindDensestSubset(g, k, T);
    dump_info(T, info);
    printf("rho");
    for (unsigned i = 0; i < g->n; ++i) printf(" %llu", rho[i]);
    printf("\n");
  }
  return 0;
}
