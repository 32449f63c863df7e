/*
 * kclpp_oracle.h -- CPU restatement of the KClist++ reference algorithms.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the GPU path is
 * compared against (tests/, __graft_entry__.smoke()) and the timed CPU baseline
 * in bench.py.  Nothing in the shipped library (kclistpp_gb300/) links, loads or
 * calls it.  Every function names the reference file:line it restates; the
 * restatement was pinned against the reference programs themselves compiled
 * from source (oracle/Makefile, target "ref") and against the golden vectors in
 * tests/golden/.
 *
 * Conventions follow the reference: vertex ids are uint32, after orientation an
 * edge is s->t with s > t, out-lists are ascending.  Counters that the
 * reference keeps in `unsigned` are widened to 64 bits where the reference's
 * 32-bit value would wrap only on inputs larger than the reference can read.
 */
#ifndef KCLPP_ORACLE_H_
#define KCLPP_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { uint32_t s, t; } orc_edge;

/* Directed (degeneracy-oriented) graph, Graph.h:20-27. */
typedef struct {
  uint32_t n;        /* number of vertices (max source + 1) */
  uint64_t e;        /* number of edges */
  orc_edge *edges;   /* root edges sorted by (s, t) */
  uint64_t *cd;      /* out-CSR offsets, n + 1 */
  uint32_t *adj;     /* out-lists, ascending */
  uint32_t core;     /* max out-degree */
} orc_graph;

/* Densest-prefix report, kCDensestNoAtom.c:315-320. */
typedef struct {
  uint32_t n;
  uint32_t m;
  uint64_t cliques;  /* prefix clique count S(n*) (exact numerator of density) */
  double density;
  double ub;
} orc_info;

/* Seq-kClist++ pass orderings. */
enum {
  ORC_SEQ_SEQUENTIAL = 0,  /* one chain over all root edges: the reference at p = 1 */
  ORC_SEQ_EDGE_STREAMS = 1,/* each root edge its own chain from the pass-start r   */
  ORC_SEQ_THREADS = 2,     /* the reference's own p-thread dynamic schedule (timing only) */
  ORC_SEQ_VERTEX_STREAMS = 3 /* each root vertex's root edges in one chain from the pass-start r */
};

/* ---- A1-A4: graph input, degeneracy order, DAG ------------------------- */
int orc_read_edge_list(const char *path, uint32_t *n, uint64_t *e, orc_edge **edges);
int orc_write_edge_list(const char *path, uint64_t e, const orc_edge *edges);
void orc_sort_by_core(uint32_t n, uint64_t e, const orc_edge *edges, uint32_t *rank);
orc_graph *orc_make_graph(uint32_t n, uint64_t e, const orc_edge *edges, const uint32_t *rank);
void orc_free_graph(orc_graph *g);
uint32_t orc_count_edges(const orc_graph *g, uint32_t num_nodes, const uint32_t *nodes);

/* ---- k-clique counts --------------------------------------------------- */
uint64_t orc_count_cliques(const orc_graph *g, int k, uint64_t *per_vertex /* n or NULL */);

/* ---- Seq-kClist++ (kCDensestNoAtom.c) ---------------------------------- */
int orc_seq_pass(const orc_graph *g, int k, uint64_t *rho, int mode, int threads);
void orc_seq_pava(const orc_graph *g, int k, const uint32_t *level, uint64_t *tentative, int threads);
orc_info orc_seq_find_densest(const orc_graph *g, int k, uint32_t T, const uint64_t *rho,
                              uint32_t *reordered, uint32_t *level, int threads);
void orc_sort_by_r_u64(uint32_t n, const uint64_t *rho, uint32_t *reordered);
/* Sampled pass for the timed CPU baseline: every stride-th root edge; returns cliques visited. */
uint64_t orc_seq_pass_sample(const orc_graph *g, int k, uint64_t *rho, int mode, int threads, uint64_t stride);

/* Wave ordering of a Seq pass (the library's KCLPP_SEQ_WAVES). */
int orc_seq_pass_waves(const orc_graph *g, int k, uint64_t *rho, uint32_t waves, int threads);
/* One shard of a split pass: only root edges whose source is marked. */
int orc_seq_delta_masked(const orc_graph *g, int k, const uint64_t *rho, const uint8_t *root_mask, int threads,
                         uint64_t *delta);

/* ---- Sim-kClist++ (kCDensestCmpSync.c) --------------------------------- */
void orc_sim_counts(const orc_graph *g, int k, const double *rho, uint64_t *cnt, int threads);
uint64_t orc_sim_counts_sample(const orc_graph *g, int k, const double *rho, uint64_t *cnt, int threads,
                               uint64_t stride);
void orc_sim_counts_masked(const orc_graph *g, int k, const double *rho, const uint8_t *root_mask, int threads,
                           uint64_t *cnt);
void orc_sim_update(uint32_t n, uint32_t t, double *rho, const uint64_t *cnt);
void orc_sim_pava(const orc_graph *g, int k, const uint32_t *level, uint64_t *tentative, int threads);
orc_info orc_sim_find_densest(const orc_graph *g, int k, const double *rho,
                              uint32_t *reordered, uint32_t *level, int threads);
void orc_sort_by_r_f64(uint32_t n, const double *rho, uint32_t *reordered);

/* ---- k-clique core trim (kClistCoreTrim.c) ----------------------------- */
typedef struct {
  uint32_t n;            /* vertices in the input edge list (max id + 1) */
  uint64_t e;            /* input edges */
  uint32_t n2;           /* vertices with core >= k - 1 */
  uint64_t e2;           /* edges among them */
  uint32_t core;         /* degeneracy of the input */
  uint32_t *map;         /* n2: new label -> original id */
  uint64_t *nck;         /* n2: k-clique degree per new label */
  uint64_t total;        /* number of k-cliques */
  uint32_t *order;       /* n2: peel order, new labels */
  uint64_t *core_num;    /* n2: k-clique core number along the peel order */
  uint64_t ckcore;       /* k-clique core number of the graph */
  double ckrho;          /* best suffix k-clique density */
  double rho;            /* its edge density */
  uint32_t size;         /* its size */
  uint32_t ntrim;        /* vertices kept by the trim */
  uint64_t ncktrim;      /* k-cliques in the trimmed graph */
  uint64_t mtrim;        /* edges in the trimmed graph */
  orc_edge *trimmed;     /* mtrim edges, original ids, in input order */
} orc_trim_result;

int orc_trim(uint32_t n, uint64_t e, const orc_edge *edges, int k, orc_trim_result *out);
void orc_free_trim(orc_trim_result *r);

/* ---- Seq-Sampling++ (kCDensestSamplingKclistpp.c), with the library's
 * counter-based sample in place of rand() ---------------------------------- */
typedef struct {
  uint32_t n;       /* densest prefix by the stored cliques (info.n) */
  uint64_t m;       /* stored cliques pushed inside it (info.m)      */
  double density;
  double ub;
} orc_sampling_info;
uint64_t orc_sample_key(uint64_t seed, uint32_t v);
/* Every k-clique in enumeration order; the kept ones go to rows (ascending
 * ids, up to cap rows) with their wave.  Returns the number kept. */
uint64_t orc_sampling_collect(const orc_graph *g, int k, uint64_t seed, uint64_t threshold, int all,
                              uint32_t waves, uint32_t *rows, uint8_t *wave, uint64_t cap);
/* InMemoryFrankWolfe's update with a given visiting order. */
void orc_sampling_pass_order(int k, uint64_t S, const uint32_t *rows, const uint32_t *order, uint32_t *rho);
/* The library's wave-ordered pass. */
void orc_sampling_pass(uint32_t n, int k, uint64_t S, const uint32_t *rows, const uint8_t *wave, uint32_t waves,
                       uint32_t *rho);
/* ExtractDensest; ordered gets the n vertices by decreasing load. */
orc_sampling_info orc_sampling_extract(uint32_t n, int k, uint64_t S, const uint32_t *rows, const uint32_t *rho,
                                       uint32_t T, uint32_t *ordered);

/* ---- whole-program drivers (CDF_Main) ---------------------------------- */
/* Runs passes 1..2^floor(log2 num_iter) and writes one orc_info per power of two
 * into infos (capacity max_infos); returns the number of infos written. */
int orc_seq_main(const orc_graph *g, int k, uint32_t num_iter, int mode, int threads,
                 uint64_t *rho_out, orc_info *infos, int max_infos);
int orc_sim_main(const orc_graph *g, int k, uint32_t num_iter, int threads,
                 double *rho_out, orc_info *infos, int max_infos);

/* ---- the benchmark's input graph ----------------------------------------
 * The library's seeded RMAT generator (kclistpp_gb300/csrc/kclpp_gen.cpp,
 * KCLPP_GEN_RMAT), restated so that the CPU legs build the benchmark workload
 * without loading the library: a SplitMix64 stream seeded with
 * seed * 0x2545F4914F6CDD1D + 0x1234567; per sample, `scale` quadrant draws
 * (uniform = top 53 bits / 2^53; a, a+b, a+b+c thresholds), self loops
 * dropped; then a Fisher-Yates permutation of the 2^scale ids (swap i-1 with
 * below(i) = next() % i, i from n down to 2) applied to both ends; pairs
 * canonicalised (min, max), sorted and deduplicated; n = max id + 1.
 * *pairs is malloc'd (2 * *e entries); returns 0 on success. */
int orc_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
             uint32_t **pairs, uint64_t *e, uint32_t *n);
void orc_free(void *p);

/* ---- timing helper for the CPU baseline -------------------------------- */
double orc_wtime(void);
int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
