/*
 * cmpsync_harness.c -- drives the reference Sim-kClist++ program's own functions
 * (kCDensestCmpSync.c, compiled from the reference sources where they lie, with
 * its main() renamed) and prints exact results for golden vectors.
 *
 * TEST INFRASTRUCTURE ONLY (builds into oracle/_ref/, never shipped).
 *
 * usage: cmpsync_harness p T k edgelist
 * output lines: "graph n e core", "info T n m density(%a) ub(%a)",
 *               "rho <%a per vertex>", "add <rho_add of the last pass>".
 */
#define main kclpp_reference_main
#include "kCDensestCmpSync.c"
#undef main

int main(int argc, char **argv) {
  if (argc < 5) { fprintf(stderr, "usage: %s p T k edgelist\n", argv[0]); return 2; }
  unsigned p = atoi(argv[1]);
  unsigned num_iter = atoi(argv[2]);
  unsigned char k = atoi(argv[3]);
  omp_set_num_threads(p);
  EdgeList *el = ReadEdgeList(argv[4]);
  SortByCore(el);
  Relabel(el);
  Graph *g = MakeGraph(el);
  printf("graph %u %u %u\n", g->n, g->e, g->core);
  AllocCdf(g, k);
  qsort(g->edges, g->e, sizeof(Edge), EdgeCmp);
  for (unsigned i = 0; i < g->n; ++i) rho[i] = 0;
  for (unsigned T = 1, t = 1; T <= num_iter; T <<= 1) {
    for (; t <= T; ++t) {
      for (unsigned i = 0; i < g->n; ++i) rho_add[i] = 0;
      CDF_CliqueEnum(g, k, FRANK_WOLFE);
      for (unsigned i = 0; i < g->n; ++i) rho[i] = (t * rho[i] + 2.0 * rho_add[i]) / (t + 2.0);
    }
    for (unsigned i = 0; i < g->n; ++i) rho_tentative[i] = 0;
    DensestSubsetInfo info = CDF_FindDensestSubset(g, k);
    printf("info %u %u %u %a %a\n", T, info.n, info.m, info.density, info.ub);
    printf("rho");
    for (unsigned i = 0; i < g->n; ++i) printf(" %a", rho[i]);
    printf("\n");
    printf("add");
    for (unsigned i = 0; i < g->n; ++i) printf(" %.0f", rho_add[i]);
    printf("\n");
  }
  return 0;
}
