/*
 * sampling_harness.c -- drives the reference Seq-Sampling++ program's own
 * functions (kCDensestSamplingKclistpp.c, compiled from the reference sources
 * where they lie, with its main() renamed) on a clique sample read from a
 * file, and prints exact results for golden vectors.
 *
 * TEST INFRASTRUCTURE ONLY (builds into oracle/_ref/, never shipped).
 *
 * usage: sampling_harness k edgelist samplefile seed
 *   samplefile: "S prob" on the first line, then S rows of k vertex ids (the
 *   graph's relabelled ids, ascending in each row).
 * output lines:
 *   "graph n e core"
 *   "count C"                      KCLIST_CliqueEnum COUNT
 *   "all S", then S lines "row ..." KCLIST_CliqueEnum SAMPLING with p = 1
 *   "order q_0 q_1 ..."            rows in the order one InMemoryFrankWolfe call
 *                                  visits them after srand(seed)
 *   "rho v_0 v_1 ..."              the loads after that call, from zero
 *   "info n m density ub"          ExtractDensest(T = 1) on them (%a)
 * and then Solve(num_iter = 1) after srand(seed) prints its own report line
 * ("Approximate densest subgraph: ..."), which starts from the same zero loads
 * and the same random sequence.
 */
#define main kclpp_reference_main
#include "kCDensestSamplingKclistpp.c"
#undef main

int main(int argc, char **argv) {
  if (argc < 5) {
    fprintf(stderr, "usage: %s k edgelist samplefile seed\n", argv[0]);
    return 2;
  }
  unsigned char k = (unsigned char)atoi(argv[1]);
  unsigned seed = (unsigned)strtoul(argv[4], NULL, 10);
  omp_set_num_threads(1);
  EdgeList *el = ReadEdgeList(argv[2]);
  SortByCore(el);
  Relabel(el);
  Graph *g = MakeGraph(el);
  printf("graph %u %u %u\n", g->n, g->e, g->core);

  KCLIST_CliqueEnum(g, k, COUNT);
  printf("count %llu\n", cnt_clique);
  /* p = 1 (target = the clique count): every clique is stored. */
  CLIQUES_TO_SAMPLE = (unsigned)cnt_clique;
  KCLIST_CliqueEnum(g, k, SAMPLING);
  printf("all %llu\n", cnt_sampled_clique);
  for (unsigned long long i = 0; i < cnt_sampled_clique; ++i) {
    printf("row");
    for (unsigned j = 0; j < k; ++j) printf(" %u", ck[i * k + j]);
    printf("\n");
  }
  free(ck);

  FILE *f = fopen(argv[3], "r");
  if (!f) {
    fprintf(stderr, "cannot open %s\n", argv[3]);
    return 2;
  }
  unsigned long long S = 0;
  double prob = 1;
  if (fscanf(f, "%llu %lf", &S, &prob) != 2) return 2;
  ck = (unsigned *)malloc((S * k + 1) * sizeof(unsigned));
  for (unsigned long long i = 0; i < S * k; ++i)
    if (fscanf(f, "%u", &ck[i]) != 1) return 2;
  fclose(f);
  cnt_sampled_clique = S;
  sampling_prob = prob;

  perm = (unsigned *)malloc((S + 1) * sizeof(unsigned));
  for (unsigned long long i = 0; i < S; ++i) perm[i] = (unsigned)i;
  rho = (unsigned *)calloc(g->n, sizeof(unsigned));
  is_in_densest_subgraph = (bool *)malloc(g->n * sizeof(bool));
  ordered_dec_rho = (unsigned *)malloc(g->n * sizeof(unsigned));
  rank_of_rho = (unsigned *)malloc(g->n * sizeof(unsigned));
  rho_pushed_to_max_rank = (unsigned *)calloc(g->n, sizeof(unsigned));
  srand(seed);
  InMemoryFrankWolfe(g, k);
  /* Step i of the call settles perm[i] for good (later steps swap only below
   * i), and steps run from S - 1 down to 0. */
  printf("order");
  for (unsigned long long i = S; i-- > 0;) printf(" %u", perm[i]);
  printf("\nrho");
  for (unsigned i = 0; i < g->n; ++i) printf(" %u", rho[i]);
  printf("\n");
  DensestSubsetInfo info = ExtractDensest(g, k, 1);
  printf("info %u %u %a %a\n", info.n, info.m, info.density, info.ub);
  fflush(stdout);
  free(perm);
  free(rho);
  free(is_in_densest_subgraph);
  free(ordered_dec_rho);
  free(rank_of_rho);
  free(rho_pushed_to_max_rank);

  srand(seed);
  Solve(g, k, 1, clock());
  fflush(stdout);
  return 0;
}
