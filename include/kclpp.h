/*
 * kclpp.h -- C ABI of the GB300 KClist++ library (libkclpp.so).
 *
 * The reference (btsun/kclistpp) is a set of stand-alone C programs with no
 * library interface; these entry points replace the C functions those programs
 * call, keeping their meaning, and add the status codes, explicit buffers and
 * device residency the reference lacks.  Every declaration cites the reference
 * function it replaces (file:line in the reference tree).
 *
 * Conventions
 *  - Every call returns kclpp_status (0 = KCLPP_OK).  kclpp_last_error() gives a
 *    thread-local message for the last failure.  No exception crosses the ABI.
 *  - Host buffers are caller-owned.  Device buffers (the *_dev entry points)
 *    are caller-owned device pointers on the context's device.  Handles
 *    (kclpp_ctx, kclpp_edge_list, kclpp_graph, kclpp_trim_result,
 *    kclpp_batch, kclpp_warm_model, kclpp_sampling) are owned by the library
 *    and released with their *_free / kclpp_destroy call.
 *  - A context owns one CUDA stream (the caller's, if one is given) and is
 *    meant for one host thread at a time.
 *  - Graphs must be simple: no self loops and no repeated edges (the
 *    reference reads such input but counts cliques with multiplicity).
 *  - Vertex ids are uint32; CSR offsets are uint64.  After orientation an edge
 *    is s -> t with s > t and out-lists are ascending (Graph.c:95-156).
 */
#ifndef KCLPP_H_
#define KCLPP_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status ---------------------------------------------------------- */
typedef int kclpp_status;
#define KCLPP_OK 0
#define KCLPP_ERR_INVALID 1     /* bad argument, or input graph not simple      */
#define KCLPP_ERR_IO 2          /* file cannot be opened / written              */
#define KCLPP_ERR_NOMEM 3       /* host or device allocation failed             */
#define KCLPP_ERR_CUDA 4        /* CUDA runtime error                           */
#define KCLPP_ERR_UNSUPPORTED 5 /* k or out-degree beyond the compiled limits   */
#define KCLPP_ERR_OVERFLOW 6    /* a device counter would have wrapped          */
#define KCLPP_ERR_NODEVICE 7    /* no CUDA device                               */

#define KCLPP_MAX_K 8           /* largest clique size compiled in              */
#define KCLPP_MAX_OUTDEG 2048   /* largest out-degree a root may have           */

const char *kclpp_status_string(kclpp_status s);
const char *kclpp_last_error(void);
const char *kclpp_version(void);

/* ---- context ---------------------------------------------------------- */
typedef struct kclpp_ctx kclpp_ctx;
/* stream: a cudaStream_t to run on, or NULL for a stream the context creates. */
kclpp_status kclpp_create(int device, void *stream, kclpp_ctx **ctx);
kclpp_status kclpp_destroy(kclpp_ctx *ctx);
kclpp_status kclpp_synchronize(kclpp_ctx *ctx);
/* Number of kernels this context has launched since creation. */
uint64_t kclpp_launch_count(const kclpp_ctx *ctx);

/* Per-kernel timing (no reference counterpart; the reference prints clock()
 * totals only, kCDensestNoAtom.c:392).  While enabled, every clique-kernel
 * launch is bracketed by CUDA events on the context's stream.
 * kclpp_profile_read synchronises, returns one record per (mode, tier) seen
 * since the previous read, and starts a new period. */
#define KCLPP_KERNEL_COUNT 0    /* k-clique degrees          */
#define KCLPP_KERNEL_ORDER 1    /* Sim rho_add / PAVA counts */
#define KCLPP_KERNEL_SEQ 2      /* Seq "++" chains           */
typedef struct {
  int mode;          /* KCLPP_KERNEL_*                         */
  int tier;          /* 0 = S, 1 = M, 2 = L                    */
  uint32_t dmax;     /* largest out-degree in the tier         */
  uint32_t launches;
  double ms;         /* summed event time                      */
} kclpp_kernel_time;
kclpp_status kclpp_profile_enable(kclpp_ctx *ctx, int on);
kclpp_status kclpp_profile_read(kclpp_ctx *ctx, kclpp_kernel_time *out, int cap, int *count);

/* ---- edge lists (A1) --------------------------------------------------- */
typedef struct kclpp_edge_list kclpp_edge_list;
/* ReadEdgeList, Graph.c:34-53: "u v" per line, n = max id + 1. */
kclpp_status kclpp_read_edge_list(const char *path, kclpp_edge_list **out);
/* The same with `threads` host threads (0: one below 8 MB, else up to 16):
 * identical results for any count (the numbers are split at whitespace and
 * the first stop ends the file, as in the one-thread scan). */
kclpp_status kclpp_read_edge_list_mt(const char *path, int threads, kclpp_edge_list **out);
/* Binary edge lists (no reference counterpart): a checksummed cache of a
 * parsed file -- n, the pairs in input order -- read back without parsing.  A
 * truncated or altered file returns KCLPP_ERR_IO. */
kclpp_status kclpp_write_edge_list_bin(const kclpp_edge_list *el, const char *path);
kclpp_status kclpp_read_edge_list_bin(const char *path, kclpp_edge_list **out);
/* pairs = s0 t0 s1 t1 ... (2*e entries); n = max id + 1 as in ReadEdgeList. */
kclpp_status kclpp_edge_list_create(const uint32_t *pairs, uint64_t e, kclpp_edge_list **out);
kclpp_status kclpp_edge_list_info(const kclpp_edge_list *el, uint32_t *n, uint64_t *e);
kclpp_status kclpp_edge_list_copy(const kclpp_edge_list *el, uint32_t *pairs_out);
kclpp_status kclpp_write_edge_list(const kclpp_edge_list *el, const char *path);
void kclpp_edge_list_free(kclpp_edge_list *el);

/* Seeded synthetic inputs (no reference counterpart: the paper's datasets are
 * not distributed).  Undirected, deduplicated, no self loops, sorted (u < v). */
#define KCLPP_GEN_CHUNG_LU 1
#define KCLPP_GEN_RMAT 2
#define KCLPP_GEN_ER 3
#define KCLPP_GEN_PLANTED 4     /* Chung-Lu base plus planted G(n_c, p) communities */
#define KCLPP_GEN_RMAT_PLANTED 5 /* RMAT base plus planted G(n_c, p) communities   */
typedef struct {
  int kind;
  uint32_t n;                   /* vertices (CHUNG_LU, ER, PLANTED)             */
  double avg_degree;            /* CHUNG_LU, ER, PLANTED                        */
  double gamma;                 /* power-law exponent (CHUNG_LU, PLANTED)       */
  uint32_t scale;               /* RMAT: n = 2^scale                            */
  uint32_t edge_factor;         /* RMAT: samples = edge_factor * n              */
  double a, b, c;               /* RMAT quadrant probabilities (d = 1-a-b-c)    */
  uint32_t communities;         /* PLANTED, RMAT_PLANTED                        */
  uint32_t comm_min, comm_max;  /* PLANTED: sizes log-uniform in [min, max]     */
  double p_in;                  /* PLANTED: edge probability inside             */
  uint64_t seed;
} kclpp_gen_params;
kclpp_status kclpp_generate(const kclpp_gen_params *p, kclpp_edge_list **out);

/* ---- degeneracy order and DAG (A2-A4) ---------------------------------- */
typedef struct kclpp_graph kclpp_graph;
/* SortByCore, Graph.c:57-91 (same binary-heap tie order, BinaryHeap.c:6-90):
 * rank[v] = n - 1 - (pop index of v).  rank_out has n entries. */
kclpp_status kclpp_core_order(const kclpp_edge_list *el, uint32_t *rank_out);
/* Relabel + MakeGraph, Graph.c:95-156: orient by rank, sort, out-CSR, upload. */
kclpp_status kclpp_make_graph(kclpp_ctx *ctx, const kclpp_edge_list *el, const uint32_t *rank,
                              kclpp_graph **g);
/* kclpp_core_order followed by kclpp_make_graph (main, kCDensestNoAtom.c:425-427). */
kclpp_status kclpp_build_graph(kclpp_ctx *ctx, const kclpp_edge_list *el, kclpp_graph **g);
/* The order by mode.  EXACT is SortByCore (as above).  FAST is the bin-sort
 * min-degree peel of Batagelj and Zaversnik, O(n + m): the same core numbers
 * and degeneracy (the DAG's largest out-degree) and the same clique counts,
 * but its own tie order, so Seq-kClist++'s r differs from the reference's. */
#define KCLPP_ORDER_EXACT 0
#define KCLPP_ORDER_FAST 1
kclpp_status kclpp_core_order_mode(const kclpp_edge_list *el, int mode, uint32_t *rank_out);
kclpp_status kclpp_build_graph_mode(kclpp_ctx *ctx, const kclpp_edge_list *el, int mode, kclpp_graph **g);
/* A DAG given directly as host CSR (out-lists strictly below the source and
 * ascending), e.g. one made by another tool from the same edge list. */
kclpp_status kclpp_graph_from_csr(kclpp_ctx *ctx, uint32_t n, uint64_t m, const uint64_t *offsets,
                                  const uint32_t *cols, kclpp_graph **g);
/* n, m and core (max out-degree; "Core value" printed at Graph.c:137). */
kclpp_status kclpp_graph_info(const kclpp_graph *g, uint32_t *n, uint64_t *m, uint32_t *core);
kclpp_status kclpp_graph_copy_csr(const kclpp_graph *g, uint64_t *offsets, uint32_t *cols);
void kclpp_graph_free(kclpp_graph *g);
/* CountEdges, Graph.c:158-166: edges with both ends among nodes[0..num). */
kclpp_status kclpp_count_edges(kclpp_ctx *ctx, const kclpp_graph *g, uint32_t num_nodes,
                               const uint32_t *nodes, uint32_t *m_out);

/* Schedule knobs of a device graph (no reference counterpart; none changes a
 * result).  Roots are split into tiers by out-degree: tier S (a warp per
 * root, out-degree <= tier_s_max / tier_s_max_seq), tier M (a CTA per root,
 * rows in shared memory, out-degree <= 1024, launched in three groups bounded
 * by the two splits of each kernel so that smaller roots get a smaller
 * shared-memory footprint and more CTAs per SM), tier L (beyond, up to 2048).
 * Work stealing lets CTAs without a root of their own join the roots other
 * CTAs are working on.  Defaults: tier_s_max 64, tier_s_max_seq 16, splits
 * 256 / 512, Seq stealing on, counting stealing off, 4 waves, widths 0 (auto),
 * concurrent groups on. */
typedef struct {
  uint32_t tier_s_max;      /* counting kernels (k-clique degrees, Sim, PAVA): tier S bound, <= 64 */
  uint32_t tier_s_max_seq;  /* Seq kernel: tier S bound, <= 64                                    */
  uint32_t m_split1, m_split2; /* counting kernels' tier M groups: (S, split1], (split1, split2],  */
                               /* (split2, 1024]                                                  */
  int steal_seq;            /* work stealing in the Seq kernel                                    */
  int steal_count;          /* work stealing in the counting kernels                              */
  uint32_t seq_waves;       /* waves of KCLPP_SEQ_WAVES, 1..1024 (default 4)                      */
  uint32_t seq_warps[4];    /* Seq kernel, warps per CTA of the M1 (<= seq_split1), M2 (<= split2), */
                            /* M3 (<= 1024) and L root groups: 2, 4, 8, 12, 16, 20 or 24 (2 and 4:  */
                            /* many small CTAs, for groups of small roots); 0 = the width of 8..24 */
                            /* that keeps the most warps resident per SM                           */
  int concurrent_tiers;     /* Seq kernel: launch a pass's root groups on forked streams (def. 1)  */
  uint32_t count_warps[4];  /* the counting / Sim kernels' widths of the same four groups:         */
                            /* 8, 16, 24 or 32; 0 = the most resident warps per SM                 */
  uint32_t seq_split1, seq_split2; /* the Seq kernel's tier M groups (as m_split1, m_split2)        */
  int concurrent_count;     /* the counting / Sim kernels' root groups on forked streams (def. 1)  */
} kclpp_schedule;
kclpp_status kclpp_graph_get_schedule(const kclpp_graph *g, kclpp_schedule *sp);
kclpp_status kclpp_graph_set_schedule(kclpp_ctx *ctx, kclpp_graph *g, const kclpp_schedule *sp);
/* Autotuner: times one pass of `kernel` (KCLPP_KERNEL_SEQ or KCLPP_KERNEL_ORDER)
 * at clique size k under each candidate schedule (that kernel's tier bound,
 * splits and stealing; then its CTA width per group, timed per launch; then
 * its concurrent groups on / off), keeps the fastest on g and reports it.
 * Seq is timed on the pass after one pass from zero, the counting kernels from
 * zero; only the chosen kernel's fields change, so tuning both kernels of a
 * step on one graph keeps each one's choice. */
typedef struct {
  kclpp_schedule best;
  double best_ms;           /* one pass under the chosen schedule   */
  double default_ms;        /* one pass under the default schedule  */
  int candidates;
} kclpp_tune_result;
kclpp_status kclpp_autotune(kclpp_ctx *ctx, kclpp_graph *g, int k, int kernel, kclpp_tune_result *out);
/* Schedule cache (no reference counterpart): a tuned schedule stored with the
 * input's kclpp_edge_list_hash, k and kernel, so that later runs skip the
 * autotuner.  Host only.  Loading checks the file (magic, size, checksum:
 * KCLPP_ERR_IO) and the key (KCLPP_ERR_INVALID for another graph, k or
 * kernel); kclpp_graph_set_schedule validates the values. */
kclpp_status kclpp_schedule_save(const char *path, uint64_t graph_hash, int k, int kernel, const kclpp_schedule *sp);
kclpp_status kclpp_schedule_load(const char *path, uint64_t graph_hash, int k, int kernel, kclpp_schedule *sp);

/* ---- batches (no reference counterpart) ----------------------------------
 * Many graphs of uneven size as one disjoint union on the device (each graph
 * keeps its own degeneracy order), run for several k values at once: every
 * pass of every k is recorded into one CUDA graph (one concurrent branch per
 * k, each pass one launch per tier over all graphs' roots) that is launched
 * with a single call.  Results equal separate runs of each graph. */
typedef struct kclpp_batch kclpp_batch;
kclpp_status kclpp_batch_create(kclpp_ctx *ctx, const kclpp_edge_list *const *els, uint32_t count,
                                kclpp_batch **out);
/* union_graph (borrowed, may be NULL) can be tuned with kclpp_autotune; the
 * next kclpp_batch_run then captures its graph again with the new schedule. */
kclpp_status kclpp_batch_info(const kclpp_batch *b, uint32_t *graphs, uint32_t *total_n, uint64_t *total_m,
                              kclpp_graph **union_graph);
/* offsets[i] = first union vertex of graph i (graphs + 1 entries). */
kclpp_status kclpp_batch_vertex_offsets(const kclpp_batch *b, uint32_t *offsets);
/* `passes` Seq (KCLPP_KERNEL_SEQ, r u64) or Sim (KCLPP_KERNEL_ORDER, rho f64)
 * passes from zero for each of ks[0..nk); out (host) receives nk vectors of
 * total_n entries, k-major.  The captured graph is reused while kernel, ks
 * and passes stay the same. */
kclpp_status kclpp_batch_run(kclpp_ctx *ctx, kclpp_batch *b, int kernel, const int *ks, int nk,
                             uint32_t passes, void *out);
void kclpp_batch_free(kclpp_batch *b);

/* ---- k-clique counts (A16 on the DAG) ----------------------------------- */
/* Number of k-cliques and, if per_vertex != NULL, the k-clique degree of every
 * vertex (onepass/recursion, kClistCoreTrim.c:368-416). */
kclpp_status kclpp_count_cliques(kclpp_ctx *ctx, const kclpp_graph *g, int k,
                                 uint64_t *per_vertex, uint64_t *total);
/* The same k-clique degrees for callers that cannot allocate device memory
 * (no counterpart in the reference): code inside a memory pool or arena that
 * owns the device's memory, pipelines that must not take the allocator's
 * locks or implicit synchronisation, plug-in hosts that hand over only the
 * buffers the library may touch.  No context and no allocation: the caller
 * passes its stream (NULL = the legacy default stream), the DAG as device CSR
 * (the layout kclpp_graph_copy_csr returns: rows ascending, every column below
 * its row) and a device output nck_dev[n], which the call clears and fills;
 * *total (host, optional) receives the number of k-cliques.  The scheduler's
 * counters live in a static device array of fixed size, so n is limited to
 * 2,097,152 vertices and out-degrees to 1024 (KCLPP_ERR_UNSUPPORTED beyond).
 * The call ends by reading its status back and synchronising `stream`, so it
 * must not be called while any stream is being captured: it returns
 * KCLPP_ERR_INVALID when `stream` reports a capture in progress.  Calls share
 * the array, so calls whose kernels overlap on the GPU race. */
kclpp_status kclpp_count_cliques_noalloc(void *stream, uint32_t n, uint64_t m, const uint64_t *offsets_dev,
                                         const uint32_t *cols_dev, int k, uint64_t *nck_dev,
                                         uint64_t *total);

/* ---- Seq-kClist++ (A7) --------------------------------------------------- */
/* Deterministic pass orderings.  EDGE_STREAMS: every root edge runs the
 * reference's in-place "++" chain (kCDensestNoAtom.c:155-268) from the
 * pass-start r, and the per-edge increments are summed -- the reference's
 * CDF_CliqueEnum (kCDensestNoAtom.c:270-295) with one thread per root edge. */
#define KCLPP_SEQ_EDGE_STREAMS 1
/* WAVES: the root vertices are split into waves by a fixed hash of their id,
 * wave w = (uint32_t)(s * 2654435761) % W with W = the graph's
 * kclpp_schedule.seq_waves (default 4); the waves run one after another and
 * every root edge of a wave runs its chain from r as the earlier waves left
 * it.  A block Gauss-Seidel ordering: the pass's load is balanced across
 * waves, so the upper bound converges in several times fewer passes than
 * with EDGE_STREAMS, at the cost of W ordered launches per pass. */
#define KCLPP_SEQ_WAVES 2
/* SHARED (not deterministic): the root-edge streams share the pass's one load
 * vector, updated in place: a stream starts from the vector as the streams
 * closed before it left it (and sees its CTA's other streams as they close),
 * and adds its increments back when it closes.  Its cliques see far fresher
 * loads than with EDGE_STREAMS (closer to the reference's sequential p = 1
 * order), so the certified gap closes in several times fewer passes.  Every
 * clique still gives exactly one unit to one of its members, so r / T stays
 * a feasible load and the upper bound of kCDensestNoAtom.c:352-369 stays a
 * certificate; which member gets the unit depends on timing, so r differs
 * from run to run. */
#define KCLPP_SEQ_SHARED 3
/* `passes` FRANK_WOLFE passes (CDF_CliqueEnum, kCDensestNoAtom.c:270-295) on
 * r (n entries, u64 as in kCDensestNoAtom.c:124). */
kclpp_status kclpp_seq_passes(kclpp_ctx *ctx, const kclpp_graph *g, int k, uint32_t passes,
                              int det_mode, uint64_t *r_inout);
kclpp_status kclpp_seq_passes_dev(kclpp_ctx *ctx, const kclpp_graph *g, int k, uint32_t passes,
                                  int det_mode, uint64_t *r_inout_dev);
/* One-shot call for callers that hold only a host CSR: uploads the DAG, runs
 * `passes` passes on host r, and downloads r (the reference's data stays on
 * the host in the same way). */
kclpp_status kclpp_seq_passes_csr(kclpp_ctx *ctx, uint32_t n, uint64_t m, const uint64_t *offsets,
                                  const uint32_t *cols, int k, uint32_t passes, int det_mode,
                                  uint64_t *r_inout);

/* ---- Sim-kClist++ (A8, A9) ------------------------------------------------ */
/* rho_add of one FRANK_WOLFE pass (kCDensestCmpSync.c:138-146, 298-325): cnt[v]
 * = number of k-cliques whose (rho, id)-smallest member is v. */
kclpp_status kclpp_sim_counts(kclpp_ctx *ctx, const kclpp_graph *g, int k, const double *rho,
                              uint64_t *cnt);
/* Passes t_first .. t_first+passes-1 of CDF_Main's loop (kCDensestCmpSync.c:396-404):
 * rho = (t*rho + 2*rho_add) / (t + 2), IEEE double, no fused multiply-add. */
kclpp_status kclpp_sim_passes(kclpp_ctx *ctx, const kclpp_graph *g, int k, uint32_t t_first,
                              uint32_t passes, double *rho_inout);
kclpp_status kclpp_sim_passes_dev(kclpp_ctx *ctx, const kclpp_graph *g, int k, uint32_t t_first,
                                  uint32_t passes, double *rho_inout_dev);
kclpp_status kclpp_sim_passes_csr(kclpp_ctx *ctx, uint32_t n, uint64_t m, const uint64_t *offsets,
                                  const uint32_t *cols, int k, uint32_t t_first, uint32_t passes,
                                  double *rho_inout);

/* ---- exact k-clique densest subgraph (host; the reference's certifier,
 * MaxFlow.cpp / kCDensestMem.c, needs Boost, which this build does not use).
 * The published max-flow construction for the k-clique densest subgraph
 * (Goldberg's network with a node per (k-1)-clique), solved by Dinic's
 * algorithm and iterated from the whole graph's density to the optimum.  For
 * graphs with up to 2e7 k-cliques (KCLPP_ERR_UNSUPPORTED beyond); members, if
 * not NULL, gets n flags (original ids) marking one densest set. */
typedef struct {
  uint64_t num, den;       /* the optimum density num / den, reduced          */
  double density;
  uint32_t size;           /* vertices of the densest set found               */
  uint64_t cliques;        /* its k-cliques (cliques / size = num / den)      */
  uint64_t cliques_total;  /* k-cliques of the graph                          */
  int iterations;          /* max-flow solves                                 */
} kclpp_exact_info;
kclpp_status kclpp_densest_exact(const kclpp_edge_list *el, int k, kclpp_exact_info *info, uint8_t *members);

/* The exact algorithm's certificate (kCDensestMem.c:329-432: PAVA, the
 * stability check and the Goldberg-type integrality test), restated with
 * per-vertex loads from GPU passes so that no clique is stored.  The candidate
 * S is the first block of the isotonic regression of the prefix clique counts
 * in the order of r (any Seq run's loads); then, in up to max_passes shared-
 * load passes (KCLPP_SEQ_SHARED, doubling): "inside" holds when the loads of
 * passes on G[S] alone show, by integer arithmetic, that no subset of S has a
 * density above m / n; "outside" when passes on the graph with S's members out
 * of reach give no vertex outside S more than m / n per pass.  Both together
 * prove that S has the largest k-clique density of the graph, exactly m / n.
 * Where the loads do not settle "inside" within max_passes and G[S] has at
 * most 2e7 k-cliques, the host max-flow (kclpp_densest_exact) on G[S] decides
 * it, as the reference falls back to its max-flow (kCDensestMem.c:434-467).
 * members (n entries, or NULL) gets S's vertices. */
typedef struct {
  uint32_t n;              /* vertices of the candidate S                      */
  uint64_t cliques;        /* its k-cliques m (density = m / n exactly)        */
  double density;
  int inside;              /* no subset of S is denser                         */
  int inside_method;       /* 1: by the loads; 2: by max-flow on G[S]          */
  int outside;             /* no set with a vertex outside S is denser         */
  int certified;           /* inside and outside: S is a densest subgraph      */
  uint32_t passes_inside;  /* passes after which each condition held          */
  uint32_t passes_outside;
} kclpp_certify_info;
kclpp_status kclpp_certify_densest(kclpp_ctx *ctx, const kclpp_graph *g, int k, const uint64_t *r,
                                   uint32_t max_passes, kclpp_certify_info *info, uint32_t *members);

/* ---- checkpoints (no reference counterpart: its dump of r is commented out,
 * kCDensestNoAtom.c:398-401).  Host only: a run's vector -- Seq r (u64) or
 * Sim rho (f64, by bit pattern) -- with the passes done, k and a hash of its
 * input, so that it resumes where it stopped (for Sim, t_first = passes + 1).
 * A loaded file is checked (magic, size, checksum): a truncated or altered
 * checkpoint returns KCLPP_ERR_IO. */
typedef struct {
  int kind;             /* KCLPP_KERNEL_SEQ (r) or KCLPP_KERNEL_ORDER (Sim rho) */
  int k;
  uint32_t passes;      /* passes done                                        */
  uint32_t n;           /* vector length                                      */
  uint64_t graph_hash;  /* kclpp_edge_list_hash of the input, or 0            */
} kclpp_state_info;
kclpp_status kclpp_save_state(const char *path, const kclpp_state_info *info, const void *vec);
/* info receives the header; vec (nullable: header only) holds cap entries. */
kclpp_status kclpp_load_state(const char *path, kclpp_state_info *info, void *vec, uint32_t cap);
/* FNV-1a of an edge list's n and pairs (as read or generated). */
kclpp_status kclpp_edge_list_hash(const kclpp_edge_list *el, uint64_t *hash);

/* ---- sharded passes (roots split over ranks; no reference counterpart) -----
 * A pass splits over devices by root: every rank builds the same graph,
 * restricts it to its share of roots with kclpp_graph_shard, computes its
 * part with the *_delta / *_counts entry points below, and the ranks sum the
 * n-vectors (an all-reduce).  Root edges are independent within a pass, so the
 * sum equals the unsharded pass exactly (integers). */
/* owner[v] = rank that processes root v (greedy by out-degree squared). */
kclpp_status kclpp_shard_plan(uint32_t n, const uint64_t *offsets, uint32_t world, uint32_t *owner);
/* Restrict g's root schedule to `rank`'s share (world = 1 restores all roots).
 * While g is sharded (world > 1) only kclpp_seq_delta_dev and
 * kclpp_sim_counts_dev accept it; every other entry point that runs over the
 * graph's roots returns KCLPP_ERR_INVALID rather than a partial result. */
kclpp_status kclpp_graph_shard(kclpp_ctx *ctx, kclpp_graph *g, uint32_t rank, uint32_t world);
/* Seq pass increments of g's roots from r (device): delta = r_after - r, for
 * this shard only (CDF_CliqueEnum FRANK_WOLFE, kCDensestNoAtom.c:270-295). */
kclpp_status kclpp_seq_delta_dev(kclpp_ctx *ctx, const kclpp_graph *g, int k, const uint64_t *r_dev,
                                 uint64_t *delta_dev);
/* Sim rho_add of g's roots (device), and the rho update on a summed rho_add
 * (kCDensestCmpSync.c:298-325, 402-403). */
kclpp_status kclpp_sim_counts_dev(kclpp_ctx *ctx, const kclpp_graph *g, int k, const double *rho_dev,
                                  uint64_t *cnt_dev);
kclpp_status kclpp_sim_update_dev(kclpp_ctx *ctx, uint32_t n, uint32_t t, double *rho_dev,
                                  const uint64_t *cnt_dev);

/* ---- sort by r, PAVA pass, densest prefix (A10-A13) ------------------------ */
/* CDF_NodeCmp + qsort (kCDensestNoAtom.c:322-337): vertices by r descending,
 * ties by ascending id; level[reordered[i]] = i.  Either output may be NULL. */
kclpp_status kclpp_sort_by_r_u64(kclpp_ctx *ctx, uint32_t n, const uint64_t *r, uint32_t *reordered,
                                 uint32_t *level);
/* Sim's key truncates r to unsigned long long first (kCDensestCmpSync.c:334-340). */
kclpp_status kclpp_sort_by_r_f64(kclpp_ctx *ctx, uint32_t n, const double *r, uint32_t *reordered,
                                 uint32_t *level);
/* PAVA_PREPROCESS pass (kCDensestNoAtom.c:191-213, 296-309): tentative[i] =
 * cliques whose largest-level member has level i. */
kclpp_status kclpp_pava(kclpp_ctx *ctx, const kclpp_graph *g, int k, const uint32_t *level,
                        uint64_t *tentative);
typedef struct {
  uint32_t n;        /* vertices in the densest prefix                    */
  uint32_t m;        /* edges among them (CountEdges)                     */
  uint64_t cliques;  /* k-cliques among them: density = cliques / n       */
  double density;
  double ub;         /* upper bound on the maximum k-clique density       */
} kclpp_densest_info;
/* CDF_FindDensestSubset, kCDensestNoAtom.c:330-371 (T = passes behind r). */
kclpp_status kclpp_extract_densest_seq(kclpp_ctx *ctx, const kclpp_graph *g, int k, uint32_t T,
                                       const uint64_t *r, kclpp_densest_info *info,
                                       uint32_t *reordered_out);
/* CDF_FindDensestSubset, kCDensestCmpSync.c:342-383. */
kclpp_status kclpp_extract_densest_sim(kclpp_ctx *ctx, const kclpp_graph *g, int k,
                                       const double *rho, kclpp_densest_info *info,
                                       uint32_t *reordered_out);

/* ---- whole runs (A14) ------------------------------------------------------ */
/* CDF_Main (kCDensestNoAtom.c:373-402): passes 1..2^floor(log2 num_iter), one
 * info per power of two (at most max_infos stored; *n_infos = number made). */
kclpp_status kclpp_seq_main(kclpp_ctx *ctx, const kclpp_graph *g, int k, uint32_t num_iter,
                            int det_mode, uint64_t *r_out, kclpp_densest_info *infos,
                            int max_infos, int *n_infos);
/* CDF_Main (kCDensestCmpSync.c:385-419). */
kclpp_status kclpp_sim_main(kclpp_ctx *ctx, const kclpp_graph *g, int k, uint32_t num_iter,
                            double *rho_out, kclpp_densest_info *infos, int max_infos,
                            int *n_infos);

/* ---- learned warm start (no reference counterpart) ------------------------------
 * A 4 -> 64 (ReLU) -> 1 MLP, bf16 weights with fp32 accumulation, predicts
 * each vertex's Seq-kClist++ load log1p(r / T) from the features
 * log1p([degree, core number, triangles, 4-cliques capped at 2^24]).  The
 * forward, backward and Adam kernels are the library's own.  A warm start
 * begins the passes at r0 = round(t0 * predicted load); its upper bound must
 * come from the increments r - r0 (kclpp_extract_densest_seq_warm), which
 * remain a feasible load, while the plain zero-start run stays the fallback. */
typedef struct kclpp_warm_model kclpp_warm_model;
#define KCLPP_WARM_FEATURES 4
#define KCLPP_WARM_HIDDEN 64
#define KCLPP_WARM_PARAMS (KCLPP_WARM_HIDDEN * KCLPP_WARM_FEATURES + 2 * KCLPP_WARM_HIDDEN + 1)
kclpp_status kclpp_warm_create(kclpp_ctx *ctx, uint64_t seed, kclpp_warm_model **out);
void kclpp_warm_free(kclpp_warm_model *m);
/* fp32 master parameters, KCLPP_WARM_PARAMS floats: W1 (64 x 4, row-major), b1, W2, b2. */
kclpp_status kclpp_warm_get_params(const kclpp_warm_model *m, float *params);
kclpp_status kclpp_warm_set_params(kclpp_ctx *ctx, kclpp_warm_model *m, const float *params);
/* Features of every vertex of g into X_dev (n x 4 floats, device). */
kclpp_status kclpp_warm_features(kclpp_ctx *ctx, const kclpp_graph *g, float *X_dev);
kclpp_status kclpp_warm_features_dev(kclpp_ctx *ctx, uint32_t n, const uint32_t *deg_dev, const uint32_t *core_dev,
                                     const uint64_t *tri_dev, const uint64_t *k4_dev, float *X_dev);
/* Y_dev[i] = model(X_dev[i]) (device, enqueued). */
kclpp_status kclpp_warm_predict_dev(kclpp_ctx *ctx, const kclpp_warm_model *m, const float *X_dev, uint32_t n,
                                    float *Y_dev);
/* Gradient of the mean squared error over the n rows (host outputs, either may be NULL). */
kclpp_status kclpp_warm_grad_dev(kclpp_ctx *ctx, kclpp_warm_model *m, const float *X_dev, const float *Y_dev,
                                 uint32_t n, float *grad_host, float *loss_host);
/* `steps` full-batch Adam steps (learning rate lr); loss_host gets the final loss. */
kclpp_status kclpp_warm_train(kclpp_ctx *ctx, kclpp_warm_model *m, const float *X_dev, const float *Y_dev,
                              uint32_t n, uint32_t steps, float lr, float *loss_host);
kclpp_status kclpp_warm_r0_dev(kclpp_ctx *ctx, const float *Y_dev, uint32_t n, float t0, uint64_t *r0_dev);
/* features + prediction + r0 for g in one call (r0_dev: n entries, device). */
kclpp_status kclpp_warm_start_r(kclpp_ctx *ctx, const kclpp_graph *g, const kclpp_warm_model *m, float t0,
                                uint64_t *r0_dev);
/* Densest prefix in the order of r (host) with the upper bound of the T
 * passes' increments r - r0 (host), for runs that started at r0. */
kclpp_status kclpp_extract_densest_seq_warm(kclpp_ctx *ctx, const kclpp_graph *g, int k, uint32_t T,
                                            const uint64_t *r, const uint64_t *r0, kclpp_densest_info *info);

/* ---- k-clique core trim (A15-A18) ------------------------------------------ */
#define KCLPP_TRIM_EXACT 0  /* the reference's heap peel: core numbers, peel order,
                               best suffix and trimmed set identical to it */
#define KCLPP_TRIM_FAST 1   /* GPU density-threshold trimming: the rho-core for the
                               best density seen; no core numbers */
#define KCLPP_TRIM_EXACT_HOST 2 /* the same peel as EXACT with every recount on the
                               host, one pop at a time (the reference's own loop;
                               kept as the check of EXACT) */
typedef struct kclpp_trim_result kclpp_trim_result;
typedef struct {
  uint32_t n, n2;        /* input vertices; vertices with core >= k-1          */
  uint64_t e, e2;        /* input edges; edges among the n2                    */
  uint32_t core;         /* degeneracy of the input                            */
  uint64_t total;        /* k-cliques in the graph                             */
  uint64_t ckcore;       /* k-clique core number of the graph (EXACT)          */
  double ckrho;          /* best k-clique density found along the peel         */
  double rho;            /* its edge density                                   */
  uint32_t size;         /* its size                                           */
  uint32_t ntrim;        /* vertices kept                                      */
  uint64_t mtrim;        /* edges kept                                         */
  uint64_t ncktrim;      /* k-cliques kept                                     */
} kclpp_trim_info;
/* main of kClistCoreTrim.c:707-775: kcore (:242-272), relabelnodes (:274-294),
 * mkspecial (:306-331), onepass (:394-416), kcliquecore (:605-666).  k = 2 is
 * NormalGraphCoreTrim.c (TrimByCoreDecomp, :41-110): a host-only degree peel
 * (ctx may be NULL); its statistics are ntrim, mtrim = ncktrim, and ckrho =
 * rho = the best edge density along the peel; map is the identity. */
kclpp_status kclpp_trim(kclpp_ctx *ctx, const kclpp_edge_list *el, int k, int mode,
                        kclpp_trim_result **out);
kclpp_status kclpp_trim_info_get(const kclpp_trim_result *t, kclpp_trim_info *info);
/* Per surviving vertex (new labels 0..n2-1): original id (map), k-clique degree
 * (the ckdeg file, :419-429), and along the peel order: vertex and core number
 * (the ckcore file, :672-676).  Any output may be NULL. */
kclpp_status kclpp_trim_copy(const kclpp_trim_result *t, uint32_t *map, uint64_t *nck,
                             uint32_t *order, uint64_t *core_num);
/* How the EXACT peel's recounts ran (no reference counterpart): the heap's pops
 * are the reference's, one at a time on the host; the recounts of a batch of
 * predicted pops run together on the GPU and a pop commits only when it is the
 * predicted one.  batches: GPU rounds; predicted / committed: pops predicted and
 * committed; gpu_roots / host_roots: committed pops recounted on the GPU / on the
 * host (more than 2048 live neighbours); seconds: wall time of the peel. */
typedef struct {
  uint64_t batches, predicted, committed, gpu_roots, host_roots;
  double seconds;
} kclpp_peel_stats;
kclpp_status kclpp_trim_peel_stats(const kclpp_trim_result *t, kclpp_peel_stats *st);
/* The trimmed graph in original ids and input order (printdensest, :686-699). */
kclpp_status kclpp_trim_edges(const kclpp_trim_result *t, kclpp_edge_list **out);
void kclpp_trim_free(kclpp_trim_result *t);

/* ---- Seq-Sampling++ (kCDensestSamplingKclistpp.c) -------------------------
 * Keeps a sample of the k-cliques in device memory, runs the "++" passes over
 * the sample only and reports the densest prefix of the sampled loads, its
 * exact k-clique count and the scaled upper bound (Solve, :446-489).
 *
 * Sampling: p = target / (k-cliques of the graph), at most 1 (:272; the
 * reference's target is CLIQUES_TO_SAMPLE = 10^7, :138).  Where the reference
 * draws rand() per clique (:160, :198), a clique Q is kept iff
 * mix64(sum of key(v), v in Q) < floor(p * 2^64), key(v) = mix64(seed + (v + 1)
 * * 0x9E3779B97F4A7C15), mix64 = SplitMix64's output function: the same
 * sample on every run, device and schedule.
 *
 * "++" pass: where the reference updates the sample one clique at a time in a
 * fresh random order (InMemoryFrankWolfe, :345-361), the sample is split into
 * `waves` fixed groups (by the same key sum); the waves run one after another
 * and the cliques of a wave all compare the values the earlier waves left
 * (each gives its unit to its member of smallest value, ties to the smallest
 * id, as the reference).  waves = 1 is a synchronous pass; results do not
 * depend on the order in which the GPU visits the cliques.
 *
 * The graph must outlive the sampling object.  k in [3, 8], out-degree up to
 * 2048, target in [1, 2^31 - 1], waves in [1, 256]. */
#define KCLPP_SAMPLE_TARGET 10000000u
typedef struct kclpp_sampling kclpp_sampling;
typedef struct {
  uint64_t cliques_total; /* k-cliques of the graph (the COUNT task, :153-157)      */
  uint64_t sampled;       /* cliques kept                                         */
  double prob;            /* sampling probability (sampling_prob, :272)           */
  uint64_t threshold;     /* floor(prob * 2^64) (0 when every clique is kept)     */
  int all;                /* prob = 1: every clique kept                          */
  uint32_t waves;
  uint32_t passes;        /* "++" passes applied so far                           */
} kclpp_sampling_info;
typedef struct {
  uint32_t T;             /* passes the loads stand for (ExtractDensest's T)       */
  uint32_t n;             /* densest prefix by the sampled loads (info.n, :385-394) */
  uint64_t m;             /* sampled cliques pushed inside it (info.m)              */
  double density;         /* m / n                                                  */
  double ub;              /* bound from the sampled loads (info.ub, :400-417)       */
  uint32_t sub_n;         /* the densest subgraph's vertices with an edge (:467-470) */
  uint64_t sub_e;         /* its edges                                              */
  uint32_t sub_core;      /* its core value (max out-degree of its DAG)             */
  uint64_t sub_cliques;   /* its k-cliques, counted exactly on the GPU (:471)       */
  double edge_density;    /* sub_e * 2.0 / sub_n / (sub_n - 1)         (:475)       */
  double clique_density;  /* sub_cliques / sub_n                       (:476)       */
  double upper_bound;     /* ub / prob / (1 - sqrt(6 ln n / ub))       (:477)       */
} kclpp_sampling_report;
/* KCLIST_CliqueEnum COUNT then SAMPLING (SampleCliques, :438-444). */
kclpp_status kclpp_sampling_create(kclpp_ctx *ctx, const kclpp_graph *g, int k, uint64_t target, uint64_t seed,
                                   uint32_t waves, kclpp_sampling **out);
kclpp_status kclpp_sampling_info_get(const kclpp_sampling *s, kclpp_sampling_info *info);
/* The kept cliques, k ascending ids per row (the ck[] rows, :160-170), rows in
 * lexicographic order of (largest member, next largest, ...); waves gets each
 * row's wave.  rows holds sampled * k ids; either output may be NULL. */
kclpp_status kclpp_sampling_cliques(kclpp_ctx *ctx, const kclpp_sampling *s, uint32_t *rows, uint8_t *waves);
kclpp_status kclpp_sampling_passes(kclpp_ctx *ctx, kclpp_sampling *s, uint32_t passes);
/* The loads (rho, u32 per vertex, :328) and the passes they stand for. */
kclpp_status kclpp_sampling_get_rho(kclpp_ctx *ctx, const kclpp_sampling *s, uint32_t *rho);
kclpp_status kclpp_sampling_set_rho(kclpp_ctx *ctx, kclpp_sampling *s, const uint32_t *rho, uint32_t passes);
/* ExtractDensest (:364-419) for loads that stand for T passes, then the exact
 * count in the densest prefix's induced subgraph (:420-435, :467-471).  order, if not
 * NULL, gets the n vertices by decreasing load (ties: ascending id). */
kclpp_status kclpp_sampling_extract(kclpp_ctx *ctx, kclpp_sampling *s, uint32_t T, kclpp_sampling_report *rep,
                                    uint32_t *order);
void kclpp_sampling_free(kclpp_sampling *s);
/* Solve (:444-489): sample, then passes 1..2^floor(log2 num_iter) with one
 * report per power of two (cap reports at most; *count gets how many). */
kclpp_status kclpp_sampling_main(kclpp_ctx *ctx, const kclpp_graph *g, int k, uint32_t num_iter, uint64_t target,
                                 uint64_t seed, uint32_t waves, kclpp_sampling_report *reps, int cap, int *count);

#ifdef __cplusplus
}
#endif
#endif
