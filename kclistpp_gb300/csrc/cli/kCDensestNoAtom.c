/*
 * kCDensestNoAtom -- drop-in for the reference's Seq-kClist++ program
 * (kCDensestNoAtom.c:404-452), running on the GPU through libkclpp.
 *
 *   ./kCDensestNoAtom p T k edgeListFileName tag
 *
 * Same arguments and the same report line per power of two as the reference
 * (kCDensestNoAtom.c:393).  p is accepted and ignored (the passes run on the
 * GPU); Seq-kClist++ runs with one stream per root edge, the deterministic
 * ordering of the library.  Times are wall-clock milliseconds.
 * KCLPP_ORDER=fast in the environment builds the DAG from the bin-sort core
 * order (same degeneracy and clique counts, other ties) instead of SortByCore;
 * KCLPP_DET=waves runs the passes in the wave ordering (KCLPP_SEQ_WAVES, fewer
 * passes to the same certified gap) instead of per-root-edge streams, and
 * KCLPP_DET=shared on one shared load vector (KCLPP_SEQ_SHARED, fewer passes
 * still; not deterministic);
 * KCLPP_TUNE=file keeps the autotuned launch schedule in that file (tuned and
 * written on the first run, loaded on the next ones; no result changes).
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
  const char *file_name = argv[4];
  double t0 = now_ms();
  kclpp_ctx *ctx;
  CHECK(kclpp_create(0, NULL, &ctx));
  printf("Reading edgelist from file %s\n", file_name);
  kclpp_edge_list *el;
  CHECK(kclpp_read_edge_list(file_name, &el));
  uint32_t n;
  uint64_t e;
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
    if (kclpp_schedule_load(tune, h, k, KCLPP_KERNEL_SEQ, &sp) == KCLPP_OK) {
      CHECK(kclpp_graph_set_schedule(ctx, g, &sp));
    } else {
      kclpp_tune_result tr;
      CHECK(kclpp_autotune(ctx, g, k, KCLPP_KERNEL_SEQ, &tr));
      CHECK(kclpp_schedule_save(tune, h, k, KCLPP_KERNEL_SEQ, &tr.best));
    }
  }
  uint64_t m;
  uint32_t core;
  CHECK(kclpp_graph_info(g, &n, &m, &core));
  printf("Core value (max truncated degree) = %u\n", core);
  printf("Number of nodes (degree > 0) = %u\n", n);
  printf("Iterate over all cliques\n");
  uint64_t *r = (uint64_t *)calloc((size_t)n + 1, sizeof(uint64_t));
  const char *det = getenv("KCLPP_DET");  /* "waves": KCLPP_SEQ_WAVES; "shared": KCLPP_SEQ_SHARED */
  const int det_mode = det && !strcmp(det, "waves")    ? KCLPP_SEQ_WAVES
                       : det && !strcmp(det, "shared") ? KCLPP_SEQ_SHARED
                                                       : KCLPP_SEQ_EDGE_STREAMS;
  uint32_t done = 0;
  for (uint32_t T = 1; T <= num_iter; T <<= 1) {
    CHECK(kclpp_seq_passes(ctx, g, k, T - done, det_mode, r));
    done = T;
    kclpp_densest_info info;
    CHECK(kclpp_extract_densest_seq(ctx, g, k, T, r, &info, NULL));
    printf("Approximate densest subgraph: %u nodes, %u edges, edge density = %f, k-clique density = %f, "
           "upper bound = %f. %ld milliseconds.\n",
           info.n, info.m, info.m * 2.0 / info.n / (info.n - 1), info.density, info.ub,
           (long)(now_ms() - t0));
    fflush(stdout);
    if (T > 0x7fffffffu) break;
  }
  free(r);
  kclpp_graph_free(g);
  kclpp_edge_list_free(el);
  kclpp_destroy(ctx);
  return 0;
}
