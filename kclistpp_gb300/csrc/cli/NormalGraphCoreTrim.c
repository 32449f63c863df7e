/*
 * NormalGraphCoreTrim -- drop-in for the reference's k = 2 core trim
 * (NormalGraphCoreTrim.c:112-143): the degree peel on the host, the same output
 * files; no GPU is used.
 *
 *   ./NormalGraphCoreTrim edgelist.txt tag
 *
 * Writes trimmed_<tag>_2.txt (the kept edges, input order, :95-99) and
 * stat_trim_<tag>_2.txt (header, "vertices edges 2-cliques" and the seconds,
 * :86-91, :138-140).
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
  if (argc < 3) {
    fprintf(stderr, "usage: %s edgelist.txt tag\n", argv[0]);
    return 2;
  }
  time_t t0 = time(NULL), t1 = t0, t2;
  printf("Reading edgelist from file %s\n", argv[1]);
  kclpp_edge_list *el;
  CHECK(kclpp_read_edge_list(argv[1], &el));
  uint32_t n;
  uint64_t e;
  CHECK(kclpp_edge_list_info(el, &n, &e));
  printf("Number of nodes = %u\n", n);
  printf("Number of edges = %llu\n", (unsigned long long)e);
  t2 = time(NULL);
  printf("- Time = %ldh%ldm%lds\n", (long)(t2 - t1) / 3600, ((long)(t2 - t1) % 3600) / 60, ((long)(t2 - t1) % 60));
  t1 = t2;

  char trim_name[256], stat_name[256];
  snprintf(trim_name, sizeof trim_name, "trimmed_%s_2.txt", argv[2]);
  snprintf(stat_name, sizeof stat_name, "stat_trim_%s_2.txt", argv[2]);
  printf("Trimming the graph by core decomposition\n");
  kclpp_trim_result *tr;
  CHECK(kclpp_trim(NULL, el, 2, KCLPP_TRIM_EXACT, &tr));
  kclpp_trim_info info;
  CHECK(kclpp_trim_info_get(tr, &info));
  FILE *ofp = fopen(stat_name, "w");
  if (!ofp) {
    fprintf(stderr, "cannot open %s\n", stat_name);
    return 1;
  }
  if (info.ntrim) {
    fprintf(ofp, "[Number of Nodes]\t[Number of Edges]\t[Number of k-Cliques]\t[Time (seconds)]\n");
    fprintf(ofp, "%u\t%llu\t%llu\t", info.ntrim, (unsigned long long)info.mtrim, (unsigned long long)info.ncktrim);
  }
  fclose(ofp);
  kclpp_edge_list *kept;
  CHECK(kclpp_trim_edges(tr, &kept));
  CHECK(kclpp_write_edge_list(kept, trim_name));

  t2 = time(NULL);
  printf("- Overall time = %ldh%ldm%lds\n", (long)(t2 - t0) / 3600, ((long)(t2 - t0) % 3600) / 60, ((long)(t2 - t0) % 60));
  ofp = fopen(stat_name, "a");
  if (ofp) {
    fprintf(ofp, "%ld\n", (long)(t2 - t0));
    fclose(ofp);
  }
  kclpp_edge_list_free(kept);
  kclpp_trim_free(tr);
  kclpp_edge_list_free(el);
  return 0;
}
