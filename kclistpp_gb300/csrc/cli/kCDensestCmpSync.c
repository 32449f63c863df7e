/*
 * kCDensestCmpSync -- drop-in for the reference's Sim-kClist++ program
 * (kCDensestCmpSync.c:421-468), running on the GPU through libkclpp.
 *
 *   ./kCDensestCmpSync p T k edgeListFileName tag
 *
 * Writes stat_cmpsync_<tag>_<p>_<T>_<k>.txt with the reference's header and
 * one line per power of two (kCDensestCmpSync.c:386-387, 411) and prints the
 * same progress line on stderr (:410).  p is accepted and ignored.
 * KCLPP_ORDER=fast in the environment builds the DAG from the bin-sort core
 * order (same degeneracy and clique counts, other ties) instead of SortByCore;
 * KCLPP_TUNE=file keeps the autotuned launch schedule in that file (tuned and
 * written on the first run, loaded on the next ones; no result changes).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "kclpp.h"

#define CHECK(call)                                                                   \
  do {                                                                                \
    kclpp_status s_ = (call);                                                         \
    if (s_ != KCLPP_OK) {                                                             \
      fprintf(stderr, "%s failed: %s (%s)\n", #call, kclpp_status_string(s_),         \
              kclpp_last_error());                                                    \
      return 1;                                                                       \
    }                                                                                 \
  } while (0)

int main(int argc, char **argv) {
  if (argc < 6) {
    fprintf(stderr, "usage: %s p T k edgeListFileName tag\n", argv[0]);
    return 2;
  }
  unsigned num_iter = (unsigned)atoi(argv[2]);
  int k = atoi(argv[3]);
  time_t t0 = time(NULL);
  kclpp_ctx *ctx;
  CHECK(kclpp_create(0, NULL, &ctx));
  printf("Reading edgelist from file %s\n", argv[4]);
  kclpp_edge_list *el;
  CHECK(kclpp_read_edge_list(argv[4], &el));
  uint32_t n;
  uint64_t e, m;
  uint32_t core;
  CHECK(kclpp_edge_list_info(el, &n, &e));
  printf("Number of nodes = %u\nNumber of edges = %llu\n", n, (unsigned long long)e);
  printf("Building the graph structure\n");
  kclpp_graph *g;
  const char *order = getenv("KCLPP_ORDER");  /* "fast": the bin-sort peel */
  const int order_mode = order && !strcmp(order, "fast") ? KCLPP_ORDER_FAST : KCLPP_ORDER_EXACT;
  CHECK(kclpp_build_graph_mode(ctx, el, order_mode, &g));
  const char *tune = getenv("KCLPP_TUNE");  /* schedule cache: loaded when it matches, else tuned and written */
  if (tune && *tune) {
    uint64_t h;
    CHECK(kclpp_edge_list_hash(el, &h));
    h ^= (uint64_t)order_mode * 0x9E3779B97F4A7C15ull;
    kclpp_schedule sp;
    if (kclpp_schedule_load(tune, h, k, KCLPP_KERNEL_ORDER, &sp) == KCLPP_OK) {
      CHECK(kclpp_graph_set_schedule(ctx, g, &sp));
    } else {
      kclpp_tune_result tr;
      CHECK(kclpp_autotune(ctx, g, k, KCLPP_KERNEL_ORDER, &tr));
      CHECK(kclpp_schedule_save(tune, h, k, KCLPP_KERNEL_ORDER, &tr.best));
    }
  }
  CHECK(kclpp_graph_info(g, &n, &m, &core));
  printf("Core value (max truncated degree) = %u\n", core);
  printf("Number of nodes (degree > 0) = %u\n", n);
  printf("Iterate over all cliques\n");
  char name[512];
  snprintf(name, sizeof name, "stat_cmpsync_%s_%s_%s_%s.txt", argv[5], argv[1], argv[2], argv[3]);
  FILE *ofp = fopen(name, "w");
  if (!ofp) {
    fprintf(stderr, "cannot open %s\n", name);
    return 1;
  }
  fprintf(ofp, "[Number of Iterations]\t[Number of Nodes]\t[Number of Edges]\t[k-Clique Density]\t"
               "[Upper Bound of Maximum Density]\t[Time (seconds)]\n");
  double *rho = (double *)calloc((size_t)n + 1, sizeof(double));
  uint32_t done = 0;
  for (uint32_t T = 1; T <= num_iter; T <<= 1) {
    CHECK(kclpp_sim_passes(ctx, g, k, done + 1, T - done, rho));
    done = T;
    kclpp_densest_info info;
    CHECK(kclpp_extract_densest_sim(ctx, g, k, rho, &info, NULL));
    time_t t1 = time(NULL);
    fprintf(stderr, "Approximate densest subgraph: %u nodes, density = %f, upper bound = %f. %ld seconds.\n",
            info.n, info.density, info.ub, (long)(t1 - t0));
    fprintf(ofp, "%u\t%u\t%u\t%.12f\t%.12f\t%ld\n", T, info.n, info.m, info.density, info.ub, (long)(t1 - t0));
    fflush(ofp);
    if (T > 0x7fffffffu) break;
  }
  fclose(ofp);
  free(rho);
  kclpp_graph_free(g);
  kclpp_edge_list_free(el);
  kclpp_destroy(ctx);
  return 0;
}
