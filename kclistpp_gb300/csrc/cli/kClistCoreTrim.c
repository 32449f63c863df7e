/*
 * kClistCoreTrim -- drop-in for the reference's k-clique core trim
 * (kClistCoreTrim.c:707-775): k-clique degrees on the GPU, the exact peel on
 * the host, the same output files.
 *
 *   ./kClistCoreTrim k edgelist.txt ckdeg.txt ckcore.txt ckdens.txt tag
 *
 * Writes ckdeg ("origid nck", :419-429), ckcore ("origid core" along the peel,
 * :672-676), ckdens (:678-684), trimmed_<tag>_<k>.txt (:686-699) and
 * stat_trim_<tag>_<k>.txt (:701-704).  KCLPP_TRIM=fast selects the GPU
 * density-threshold trim (no core numbers).
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
  if (argc < 7) {
    fprintf(stderr, "usage: %s k edgelist.txt ckdeg.txt ckcore.txt ckdens.txt tag\n", argv[0]);
    return 2;
  }
  int kmax = atoi(argv[1]);
  const char *fast = getenv("KCLPP_TRIM");
  int mode = (fast && strcmp(fast, "fast") == 0) ? KCLPP_TRIM_FAST : KCLPP_TRIM_EXACT;
  time_t t0 = time(NULL);
  kclpp_ctx *ctx;
  CHECK(kclpp_create(0, NULL, &ctx));
  printf("Reading edgelist from file %s\n", argv[2]);
  kclpp_edge_list *el;
  CHECK(kclpp_read_edge_list(argv[2], &el));
  kclpp_trim_result *tr;
  CHECK(kclpp_trim(ctx, el, kmax, mode, &tr));
  kclpp_trim_info I;
  CHECK(kclpp_trim_info_get(tr, &I));
  printf("Number of nodes: %u\n", I.n);
  printf("Number of edges: %llu\n", (unsigned long long)I.e);
  printf("Number of nodes (with core value > %u): %u\n", kmax - 2, I.n2);
  printf("Number of edges (between nodes with core value > %u): %llu\n", kmax - 2, (unsigned long long)I.e2);
  printf("Core number = %u\n", I.core);
  printf("Number of %u-cliques: %llu\n", kmax, (unsigned long long)I.total);
  uint32_t *map = malloc(((size_t)I.n2 + 1) * 4), *order = malloc(((size_t)I.n2 + 1) * 4);
  uint64_t *nck = malloc(((size_t)I.n2 + 1) * 8), *core = malloc(((size_t)I.n2 + 1) * 8);
  CHECK(kclpp_trim_copy(tr, map, nck, order, core));
  FILE *f = fopen(argv[3], "w");
  if (!f) return 1;
  for (uint32_t i = 0; i < I.n2; ++i) fprintf(f, "%u %llu\n", map[i], (unsigned long long)nck[i]);
  fclose(f);
  printf("%u-clique core number of the graph = %llu\n", kmax, (unsigned long long)I.ckcore);
  printf("%u-clique density of the dense subgraph = %lf\n", kmax, I.ckrho);
  printf("Edge density of the found dense subgraph = %lf\n", I.rho);
  printf("Size of the found dense subgraph = %u\n", I.size);
  f = fopen(argv[4], "w");
  if (!f) return 1;
  for (uint32_t i = 0; i < I.n2; ++i) fprintf(f, "%u %llu\n", map[order[i]], (unsigned long long)core[i]);
  fclose(f);
  f = fopen(argv[5], "w");
  if (!f) return 1;
  fprintf(f, "%lf %lf %u", I.ckrho, I.rho, I.size);
  /* the reference's unsigned loop bound lists nobody when size == n2 */
  for (uint32_t i = I.n2 - 1; I.size < I.n2 && i > I.n2 - I.size - 1; i--) fprintf(f, " %u", map[order[i]]);
  fprintf(f, "\n");
  fclose(f);
  char name[512];
  snprintf(name, sizeof name, "trimmed_%s_%s.txt", argv[6], argv[1]);
  kclpp_edge_list *te;
  CHECK(kclpp_trim_edges(tr, &te));
  CHECK(kclpp_write_edge_list(te, name));
  printf("The trimmed graph has %u nodes, %llu edges and %llu k-cliques.\n", I.ntrim,
         (unsigned long long)I.mtrim, (unsigned long long)I.ncktrim);
  snprintf(name, sizeof name, "stat_trim_%s_%s.txt", argv[6], argv[1]);
  f = fopen(name, "w");
  if (!f) return 1;
  fprintf(f, "[Number of Nodes]\t[Number of Edges]\t[Number of k-Cliques]\t[Time (seconds)]\n");
  fprintf(f, "%u\t%llu\t%llu\t%ld\n", I.ntrim, (unsigned long long)I.mtrim, (unsigned long long)I.ncktrim,
          (long)(time(NULL) - t0));
  fclose(f);
  free(map); free(order); free(nck); free(core);
  kclpp_edge_list_free(te);
  kclpp_trim_free(tr);
  kclpp_edge_list_free(el);
  kclpp_destroy(ctx);
  return 0;
}
