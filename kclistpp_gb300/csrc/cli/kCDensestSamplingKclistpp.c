/*
 * kCDensestSamplingKclistpp -- drop-in for the reference's Seq-Sampling++
 * program (kCDensestSamplingKclistpp.c:491-536), running on the GPU through
 * libkclpp.
 *
 *   ./kCDensestSamplingKclistpp p T k edgeListFileName
 *
 * Same arguments and the same printed lines as the reference: the graph, the
 * clique count, the sample size, then one "Approximate densest subgraph" line
 * per power of two up to T (Solve, :446-489).  p is accepted and ignored.
 * Where the reference samples with rand() seeded by the time of day, the
 * library keeps a clique by a counter-based draw from a seed, and runs its
 * "++" passes in waves; both come from the environment:
 *   KCLPP_SEED            seed of the sample (default 1)
 *   KCLPP_WAVES           waves per pass, 1..256 (default 8)
 *   KCLPP_SAMPLE_TARGET   cliques to sample (default 10^7, CLIQUES_TO_SAMPLE)
 *   KCLPP_ORDER=fast      the bin-sort core order instead of SortByCore's
 * Times are wall-clock milliseconds.
 */
#define _POSIX_C_SOURCE 199309L /* clock_gettime under a strict C standard */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "kclpp.h"

static double now_ms(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

static void print_time(const char *what, double ms) {
  long t = (long)ms;
  printf("- %s = %ldh%ldm%lds%ldms\n", what, t / 3600000, (t / 60000) % 60, (t / 1000) % 60, t % 1000);
}

static unsigned long long env_u64(const char *name, unsigned long long dflt) {
  const char *v = getenv(name);
  return v && *v ? strtoull(v, NULL, 10) : dflt;
}

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
  if (argc < 5) {
    fprintf(stderr, "usage: %s p T k edgeListFileName\n", argv[0]);
    return 2;
  }
  unsigned num_iter = (unsigned)atoi(argv[2]);
  int k = atoi(argv[3]);
  const char *file_name = argv[4];
  unsigned long long seed = env_u64("KCLPP_SEED", 1);
  unsigned waves = (unsigned)env_u64("KCLPP_WAVES", 8);
  unsigned long long target = env_u64("KCLPP_SAMPLE_TARGET", KCLPP_SAMPLE_TARGET);
  double t0 = now_ms(), t1 = t0, t2;
  kclpp_ctx *ctx;
  CHECK(kclpp_create(0, NULL, &ctx));

  printf("Reading edgelist from file %s\n", file_name);
  kclpp_edge_list *el;
  CHECK(kclpp_read_edge_list(file_name, &el));
  uint32_t n;
  uint64_t e;
  CHECK(kclpp_edge_list_info(el, &n, &e));
  printf("Number of nodes = %u\nNumber of edges = %llu\n", n, (unsigned long long)e);
  t2 = now_ms();
  print_time("Time", t2 - t1);
  t1 = t2;

  printf("Building the graph structure\n");
  kclpp_graph *g;
  const char *order = getenv("KCLPP_ORDER");  /* "fast": the bin-sort peel */
  CHECK(kclpp_build_graph_mode(ctx, el, order && !strcmp(order, "fast") ? KCLPP_ORDER_FAST : KCLPP_ORDER_EXACT,
                               &g));
  uint64_t m;
  uint32_t core;
  CHECK(kclpp_graph_info(g, &n, &m, &core));
  printf("Core value (max truncated degree) = %u\n", core);
  printf("Number of nodes (degree > 0) = %u\n", n);
  t2 = now_ms();
  print_time("Time", t2 - t1);
  t1 = t2;

  kclpp_sampling *s;
  CHECK(kclpp_sampling_create(ctx, g, k, target, seed, waves, &s));
  kclpp_sampling_info info;
  CHECK(kclpp_sampling_info_get(s, &info));
  printf("Number of %d-cliques: %llu\n", k, (unsigned long long)info.cliques_total);
  printf("Number of sampled %d-cliques: %llu\n", k, (unsigned long long)info.sampled);
  t2 = now_ms();
  print_time("Time", t2 - t1);
  t1 = t2;

  uint32_t done = 0;
  for (unsigned long long T = 1; T <= num_iter; T <<= 1) {
    CHECK(kclpp_sampling_passes(ctx, s, (uint32_t)T - done));
    done = (uint32_t)T;
    kclpp_sampling_report rep;
    CHECK(kclpp_sampling_extract(ctx, s, (uint32_t)T, &rep, NULL));
    printf("Core value (max truncated degree) = %u\n", rep.sub_core);
    printf("Approximate densest subgraph: %u nodes, %llu edges, edge density = %f, k-clique density = %f, "
           "upper bound = %f. %ld milliseconds.\n",
           rep.sub_n, (unsigned long long)rep.sub_e, rep.edge_density, rep.clique_density, rep.upper_bound,
           (long)(now_ms() - t0));
    fflush(stdout);
  }
  t2 = now_ms();
  print_time("Time", t2 - t1);
  print_time("Overall time", t2 - t0);

  kclpp_sampling_free(s);
  kclpp_graph_free(g);
  kclpp_edge_list_free(el);
  kclpp_destroy(ctx);
  return 0;
}
