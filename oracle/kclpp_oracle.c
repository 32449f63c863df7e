/*
 * kclpp_oracle.c -- CPU restatement of the KClist++ reference algorithms.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU path and the timed CPU
 * baseline.  The shipped library never links or loads this file.
 *
 * Each function cites the reference file:line whose algorithm it restates.
 * Where the reference's result depends on an order (heap tie breaking, the
 * in-place "++" chain of Seq-kClist++, the floating-point summation order of
 * Sim-kClist++), the restatement performs the same steps in the same order.
 * Build with -ffp-contract=off so that no multiply-add is fused.
 */
#include "kclpp_oracle.h"

#include <limits.h>
#include <omp.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define ORC_MAXK 16
#define NIL32 UINT32_MAX
#define MARK32 (UINT32_MAX - 1u)

static void *xmalloc(size_t sz) {
  void *p = malloc(sz ? sz : 1);
  if (!p) { fprintf(stderr, "oracle: out of memory (%zu bytes)\n", sz); abort(); }
  return p;
}
static void *xcalloc(size_t n, size_t sz) {
  void *p = calloc(n ? n : 1, sz ? sz : 1);
  if (!p) { fprintf(stderr, "oracle: out of memory\n"); abort(); }
  return p;
}

double orc_wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
int orc_max_threads(void) { return omp_get_max_threads(); }

/* ------------------------------------------------------------------------ */
/* Indexed binary min-heap: the exact operation sequence of BinaryHeap.c:6-90
 * (and of the copies in kClistCoreTrim.c:64-133, 445-533), so that ties pop in
 * the reference's order.                                                     */
typedef struct { uint32_t key; uint64_t value; } orc_kv;
typedef struct { uint32_t n; uint32_t *p; orc_kv *kv; } orc_heap;

static void heap_init(orc_heap *h, uint32_t nmax) {
  h->n = 0;
  h->p = (uint32_t *)xmalloc((size_t)nmax * sizeof(uint32_t));
  for (uint32_t i = 0; i < nmax; ++i) h->p[i] = NIL32;
  h->kv = (orc_kv *)xmalloc((size_t)nmax * sizeof(orc_kv));
}
static void heap_free(orc_heap *h) { free(h->p); free(h->kv); }
static void heap_swap(orc_heap *h, uint32_t i, uint32_t j) {  /* BinaryHeap.c:15-22 */
  orc_kv tmp = h->kv[i];
  uint32_t pt = h->p[tmp.key];
  h->p[h->kv[i].key] = h->p[h->kv[j].key];
  h->kv[i] = h->kv[j];
  h->p[h->kv[j].key] = pt;
  h->kv[j] = tmp;
}
static void heap_up(orc_heap *h, uint32_t i) {  /* BinaryHeap.c:24-34 */
  while (i > 0) {
    uint32_t j = (i - 1) >> 1;
    if (h->kv[j].value > h->kv[i].value) { heap_swap(h, i, j); i = j; }
    else break;
  }
}
static void heap_down(orc_heap *h) {  /* BinaryHeap.c:36-49 */
  uint32_t i = 0, j1 = 1, j2 = 2, j;
  while (j1 < h->n) {
    j = ((j2 < h->n) && (h->kv[j2].value < h->kv[j1].value)) ? j2 : j1;
    if (h->kv[j].value < h->kv[i].value) {
      heap_swap(h, i, j);
      i = j; j1 = (i << 1) + 1; j2 = j1 + 1;
      continue;
    }
    break;
  }
}
static void heap_insert(orc_heap *h, uint32_t key, uint64_t value) {  /* BinaryHeap.c:51-55 */
  h->p[key] = h->n++;
  h->kv[h->n - 1].key = key;
  h->kv[h->n - 1].value = value;
  heap_up(h, h->n - 1);
}
static void heap_dec(orc_heap *h, uint32_t key, uint64_t delta) {  /* BinaryHeap.c:57-63 */
  uint32_t i = h->p[key];
  if (i != NIL32) { h->kv[i].value -= delta; heap_up(h, i); }
}
static orc_kv heap_pop(orc_heap *h) {  /* BinaryHeap.c:65-72 */
  orc_kv kv = h->kv[0];
  h->p[kv.key] = NIL32;
  h->kv[0] = h->kv[--(h->n)];
  h->p[h->kv[0].key] = 0;
  heap_down(h);
  return kv;
}

/* ------------------------------------------------------------------------ */
/* A1: ReadEdgeList, Graph.c:34-53.  n = max id + 1 (1 for an empty file). */
int orc_read_edge_list(const char *path, uint32_t *n, uint64_t *e, orc_edge **edges) {
  FILE *f = fopen(path, "r");
  if (!f) return -1;
  uint64_t cap = 1u << 20, m = 0;
  uint32_t mx = 0;
  orc_edge *E = (orc_edge *)xmalloc(cap * sizeof(orc_edge));
  unsigned a, b;
  while (fscanf(f, "%u %u", &a, &b) == 2) {
    if (m == cap) { cap *= 2; E = (orc_edge *)realloc(E, cap * sizeof(orc_edge)); if (!E) abort(); }
    E[m].s = a; E[m].t = b; ++m;
    if (a > mx) mx = a;
    if (b > mx) mx = b;
  }
  fclose(f);
  *n = mx + 1;
  *e = m;
  *edges = E;
  return 0;
}

int orc_write_edge_list(const char *path, uint64_t e, const orc_edge *edges) {
  FILE *f = fopen(path, "w");
  if (!f) return -1;
  for (uint64_t i = 0; i < e; ++i) fprintf(f, "%u %u\n", edges[i].s, edges[i].t);
  fclose(f);
  return 0;
}

/* A2: SortByCore, Graph.c:57-91.  rank[v] = n - (pop index + 1). */
void orc_sort_by_core(uint32_t n, uint64_t e, const orc_edge *edges, uint32_t *rank) {
  uint64_t *cd = (uint64_t *)xmalloc(((size_t)n + 1) * sizeof(uint64_t));
  uint32_t *d = (uint32_t *)xcalloc(n, sizeof(uint32_t));
  uint32_t *adj = (uint32_t *)xmalloc((size_t)(2 * e) * sizeof(uint32_t));
  for (uint64_t i = 0; i < e; ++i) { ++d[edges[i].s]; ++d[edges[i].t]; }
  cd[0] = 0;
  for (uint32_t i = 1; i <= n; ++i) { cd[i] = cd[i - 1] + d[i - 1]; d[i - 1] = 0; }
  for (uint64_t i = 0; i < e; ++i) {
    uint32_t s = edges[i].s, t = edges[i].t;
    adj[cd[s] + d[s]++] = t;
    adj[cd[t] + d[t]++] = s;
  }
  orc_heap h;
  heap_init(&h, n);
  for (uint32_t i = 0; i < n; ++i) heap_insert(&h, i, d[i]);
  uint32_t r = 0;
  for (uint32_t i = 0; i < n; ++i) {
    orc_kv kv = heap_pop(&h);
    rank[kv.key] = n - (++r);
    for (uint64_t j = cd[kv.key]; j < cd[kv.key + 1]; ++j) heap_dec(&h, adj[j], 1);
  }
  heap_free(&h);
  free(cd); free(d); free(adj);
}

static int edge_cmp(const void *a, const void *b) {
  const orc_edge *x = (const orc_edge *)a, *y = (const orc_edge *)b;
  if (x->s != y->s) return x->s < y->s ? -1 : 1;
  if (x->t != y->t) return x->t < y->t ? -1 : 1;
  return 0;
}

/* A3 + A4: Relabel (Graph.c:95-112) and MakeGraph (Graph.c:114-156). */
orc_graph *orc_make_graph(uint32_t n_in, uint64_t e, const orc_edge *edges, const uint32_t *rank) {
  (void)n_in;
  orc_graph *g = (orc_graph *)xcalloc(1, sizeof(orc_graph));
  g->e = e;
  g->edges = (orc_edge *)xmalloc((size_t)e * sizeof(orc_edge));
  uint32_t n = 0;
  for (uint64_t i = 0; i < e; ++i) {
    uint32_t s = rank[edges[i].s], t = rank[edges[i].t];
    if (s < t) { uint32_t tmp = s; s = t; t = tmp; }
    if (s + 1 > n) n = s + 1;
    g->edges[i].s = s; g->edges[i].t = t;
  }
  g->n = n;
  qsort(g->edges, (size_t)e, sizeof(orc_edge), edge_cmp);
  g->cd = (uint64_t *)xcalloc((size_t)n + 1, sizeof(uint64_t));
  g->adj = (uint32_t *)xmalloc((size_t)e * sizeof(uint32_t));
  for (uint64_t i = 0; i < e; ++i) g->cd[g->edges[i].s + 1]++;
  uint32_t mx = 0;
  for (uint32_t i = 1; i <= n; ++i) {
    if (g->cd[i] > mx) mx = (uint32_t)g->cd[i];
    g->cd[i] += g->cd[i - 1];
  }
  for (uint64_t i = 0; i < e; ++i) g->adj[i] = g->edges[i].t;  /* edges are sorted by (s,t) */
  g->core = mx;
  return g;
}

void orc_free_graph(orc_graph *g) {
  if (!g) return;
  free(g->edges); free(g->cd); free(g->adj); free(g);
}

/* CountEdges, Graph.c:158-166. */
uint32_t orc_count_edges(const orc_graph *g, uint32_t num_nodes, const uint32_t *nodes) {
  char *inc = (char *)xcalloc(g->n, 1);
  for (uint32_t i = 0; i < num_nodes; ++i) inc[nodes[i]] = 1;
  uint32_t m = 0;
  for (uint64_t i = 0; i < g->e; ++i) m += (inc[g->edges[i].s] && inc[g->edges[i].t]);
  free(inc);
  return m;
}

/* ------------------------------------------------------------------------ */
/* Per-thread induced-subgraph workspace: the structure of Subgraph
 * (GraphDupAdj.h:22-29, one adjacency array per level) built by
 * MakeSubgraph (kCDensestNoAtom.c:71-118).                                  */
typedef struct {
  int k;
  uint32_t core;
  uint32_t *g2sg;               /* n: global -> local id (NIL32 = absent) */
  uint32_t *sg2g;               /* core: local -> global id */
  uint8_t *label;               /* core */
  uint32_t nn[ORC_MAXK];        /* nodes per level */
  uint32_t *nodes[ORC_MAXK];
  uint32_t *deg[ORC_MAXK];
  uint32_t *adj[ORC_MAXK];      /* core * core per level */
} orc_ws;

static orc_ws *ws_new(const orc_graph *g, int k) {
  orc_ws *w = (orc_ws *)xcalloc(1, sizeof(orc_ws));
  uint32_t c = g->core ? g->core : 1;
  w->k = k;
  w->core = c;
  w->g2sg = (uint32_t *)xmalloc(((size_t)g->n + 1) * sizeof(uint32_t));
  for (uint32_t i = 0; i < g->n; ++i) w->g2sg[i] = NIL32;
  w->sg2g = (uint32_t *)xmalloc((size_t)c * sizeof(uint32_t));
  w->label = (uint8_t *)xcalloc(c, 1);
  for (int l = 1; l < k; ++l) {
    w->nodes[l] = (uint32_t *)xmalloc((size_t)c * sizeof(uint32_t));
    w->deg[l] = (uint32_t *)xmalloc((size_t)c * sizeof(uint32_t));
    w->adj[l] = (uint32_t *)xmalloc((size_t)c * c * sizeof(uint32_t));
  }
  return w;
}
static void ws_free(orc_ws *w) {
  for (int l = 1; l < w->k; ++l) { free(w->nodes[l]); free(w->deg[l]); free(w->adj[l]); }
  free(w->g2sg); free(w->sg2g); free(w->label); free(w);
}

/* MakeSubgraph, kCDensestNoAtom.c:71-118: C = N+(s) ∩ N+(t) with local ids in
 * ascending global order, induced adjacency at level k-2 in N+(x) order.   */
static void make_subgraph(orc_ws *w, const orc_graph *g, uint32_t s, uint32_t t) {
  const int L = w->k - 2;
  const uint32_t core = w->core;
  for (uint64_t i = g->cd[t]; i < g->cd[t + 1]; ++i) w->g2sg[g->adj[i]] = MARK32;
  uint32_t j = 0;
  for (uint64_t i = g->cd[s]; i < g->cd[s + 1]; ++i) {
    uint32_t x = g->adj[i];
    if (w->g2sg[x] == MARK32) {
      w->g2sg[x] = j;
      w->sg2g[j] = x;
      w->label[j] = (uint8_t)L;
      w->nodes[L][j] = j;
      w->deg[L][j] = 0;
      ++j;
    }
  }
  w->nn[L] = j;
  for (uint32_t i = 0; i < w->nn[L]; ++i) {
    uint32_t x = w->sg2g[i];
    for (uint64_t l = g->cd[x]; l < g->cd[x + 1]; ++l) {
      uint32_t jj = w->g2sg[g->adj[l]];
      if (jj < MARK32) w->adj[L][(size_t)core * i + w->deg[L][i]++] = jj;
    }
  }
  for (uint64_t i = g->cd[t]; i < g->cd[t + 1]; ++i) w->g2sg[g->adj[i]] = NIL32;
}

/* Level step of CDF_CliqueEnumThread (kCDensestNoAtom.c:235-259): children
 * of local node u at level l, relabelled l-1, adjacency filtered in order.  */
static void descend(orc_ws *w, int l, uint32_t u) {
  const uint32_t core = w->core;
  w->nn[l - 1] = 0;
  const uint32_t *au = w->adj[l] + (size_t)core * u;
  for (uint32_t j = 0; j < w->deg[l][u]; ++j) {
    uint32_t v = au[j];
    if (w->label[v] == l) {
      w->label[v] = (uint8_t)(l - 1);
      w->nodes[l - 1][w->nn[l - 1]++] = v;
      w->deg[l - 1][v] = 0;
    }
  }
  for (uint32_t j = 0; j < w->nn[l - 1]; ++j) {
    uint32_t v = w->nodes[l - 1][j];
    const uint32_t *av = w->adj[l] + (size_t)core * v;
    uint32_t *dst = w->adj[l - 1] + (size_t)core * v;
    for (uint32_t q = 0; q < w->deg[l][v]; ++q) {
      uint32_t x = av[q];
      if (w->label[x] == l - 1) dst[w->deg[l - 1][v]++] = x;
    }
  }
}
static void ascend(orc_ws *w, int l) {  /* kCDensestNoAtom.c:263-266 */
  for (uint32_t j = 0; j < w->nn[l - 1]; ++j) w->label[w->nodes[l - 1][j]] = (uint8_t)l;
}

/* ---- Seq-kClist++ chain: CDF_CliqueEnumThread FRANK_WOLFE,
 * kCDensestNoAtom.c:155-190 and 218-268.  The prefix argmin is cached as a
 * vertex id; its value is re-read from the live array at each comparison.  */
static uint64_t seq_rec(orc_ws *w, uint64_t *cur, int l, uint32_t ngw) {
  uint64_t cl = 0;
  if (w->k == 3) {                              /* :162-171 */
    for (uint32_t i = 0; i < w->nn[1]; ++i) {
      uint32_t x = w->sg2g[w->nodes[1][i]];
      uint32_t g2 = cur[x] < cur[ngw] ? x : ngw;
      ++cur[g2];
    }
    return w->nn[1];
  }
  if (l == 2) {                                 /* :173-188 */
    for (uint32_t i = 0; i < w->nn[2]; ++i) {
      uint32_t u = w->nodes[2][i];
      uint32_t x = w->sg2g[u];
      uint32_t g2 = cur[x] < cur[ngw] ? x : ngw;
      const uint32_t *au = w->adj[2] + (size_t)w->core * u;
      for (uint32_t j = 0; j < w->deg[2][u]; ++j) {
        uint32_t y = w->sg2g[au[j]];
        uint32_t g3 = cur[y] < cur[g2] ? y : g2;
        ++cur[g3];
      }
      cl += w->deg[2][u];
    }
    return cl;
  }
  if (w->nn[l] < (uint32_t)l) return 0;         /* :218 */
  for (uint32_t i = 0; i < w->nn[l]; ++i) {     /* :220-267 */
    uint32_t u = w->nodes[l][i];
    uint32_t x = w->sg2g[u];
    uint32_t g2 = cur[x] < cur[ngw] ? x : ngw;
    descend(w, l, u);
    cl += seq_rec(w, cur, l - 1, g2);
    ascend(w, l);
  }
  return cl;
}

/* ---- order-free clique visits: per clique, the member that minimises a
 * key (Sim: (rho, id), kCDensestCmpSync.c:138-146; PAVA: largest level,
 * kCDensestNoAtom.c:191-213) receives one unit.  The prefix extremum is
 * carried down the recursion; with a fixed key this equals the reference's
 * k-way scan.                                                              */
typedef struct {
  int kind;                  /* 0 = sim key, 1 = pava (max level), 2 = all members */
  const double *rho;
  const uint32_t *level;
  uint64_t *cnt;             /* per vertex (kind 0, 2) or per level (kind 1) */
  uint32_t pre[ORC_MAXK];    /* kind 2: current prefix of global ids */
} visit_t;

static inline int sim_less(const double *rho, uint32_t a, uint32_t b) {
  return rho[a] < rho[b] || (rho[a] == rho[b] && a < b);
}
static inline uint32_t pick(const visit_t *v, uint32_t a, uint32_t b) {
  if (v->kind == 0) return sim_less(v->rho, a, b) ? a : b;
  return v->level[a] > v->level[b] ? a : b;
}
static inline void credit(visit_t *v, uint32_t x) {
  if (v->kind == 0) v->cnt[x]++;
  else v->cnt[v->level[x]]++;
}

static uint64_t visit_rec(orc_ws *w, visit_t *vt, int l, uint32_t best, int depth) {
  uint64_t cl = 0;
  if (w->k == 3) {
    for (uint32_t i = 0; i < w->nn[1]; ++i) {
      uint32_t x = w->sg2g[w->nodes[1][i]];
      if (vt->kind == 2) {
        vt->cnt[x]++;
      } else {
        credit(vt, pick(vt, x, best));
      }
    }
    if (vt->kind == 2) for (int q = 0; q < depth; ++q) vt->cnt[vt->pre[q]] += w->nn[1];
    return w->nn[1];
  }
  if (l == 2) {
    for (uint32_t i = 0; i < w->nn[2]; ++i) {
      uint32_t u = w->nodes[2][i];
      uint32_t x = w->sg2g[u];
      const uint32_t *au = w->adj[2] + (size_t)w->core * u;
      uint32_t du = w->deg[2][u];
      if (vt->kind == 2) {
        for (uint32_t j = 0; j < du; ++j) vt->cnt[w->sg2g[au[j]]]++;
        vt->cnt[x] += du;
        for (int q = 0; q < depth; ++q) vt->cnt[vt->pre[q]] += du;
      } else {
        uint32_t b2 = pick(vt, x, best);
        for (uint32_t j = 0; j < du; ++j) credit(vt, pick(vt, w->sg2g[au[j]], b2));
      }
      cl += du;
    }
    return cl;
  }
  if (w->nn[l] < (uint32_t)l) return 0;
  for (uint32_t i = 0; i < w->nn[l]; ++i) {
    uint32_t u = w->nodes[l][i];
    uint32_t x = w->sg2g[u];
    uint32_t b2 = vt->kind == 2 ? x : pick(vt, x, best);
    vt->pre[depth] = x;
    descend(w, l, u);
    cl += visit_rec(w, vt, l - 1, b2, depth + 1);
    ascend(w, l);
  }
  return cl;
}

/* Shared driver for order-free passes (CDF_CliqueEnum, kCDensestNoAtom.c:270-313
 * and kCDensestCmpSync.c:298-325): dynamic schedule over root edges, per-thread
 * counters merged at the end (integers, so the merge order is immaterial).  */
static uint64_t visit_all_masked(const orc_graph *g, int k, visit_t proto, uint64_t nout,
                                 uint64_t *out, int threads, uint64_t stride, const uint8_t *root_mask) {
  uint64_t total = 0;
  if (stride == 0) stride = 1;
  memset(out, 0, (size_t)nout * sizeof(uint64_t));
  if (g->e == 0) return 0;
  #pragma omp parallel num_threads(threads > 0 ? threads : 1) reduction(+:total)
  {
    orc_ws *w = ws_new(g, k);
    visit_t vt = proto;
    vt.cnt = (uint64_t *)xcalloc((size_t)nout + 1, sizeof(uint64_t));
    int64_t ne = (int64_t)((g->e + stride - 1) / stride);
    #pragma omp for schedule(dynamic, 1) nowait
    for (int64_t q = 0; q < ne; ++q) {
      uint64_t i = (uint64_t)q * stride;
      uint32_t s = g->edges[i].s, t = g->edges[i].t;
      if (root_mask && !root_mask[s]) continue;
      uint32_t b;
      if (vt.kind == 2) {
        b = 0;
        vt.pre[0] = s;
        vt.pre[1] = t;
      } else if (vt.kind == 0) {
        /* kCDensestCmpSync.c:310 compares rho[t] < rho[s]; the clique-level
         * scan (:138-146) then settles ties toward the smaller id. */
        b = sim_less(vt.rho, t, s) ? t : s;
      } else {
        b = vt.level[t] > vt.level[s] ? t : s;
      }
      make_subgraph(w, g, s, t);
      total += visit_rec(w, &vt, k - 2, b, 2);
    }
    #pragma omp critical
    for (uint64_t x = 0; x < nout; ++x) out[x] += vt.cnt[x];
    free(vt.cnt);
    ws_free(w);
  }
  return total;
}

static uint64_t visit_all(const orc_graph *g, int k, visit_t proto, uint64_t nout,
                          uint64_t *out, int threads, uint64_t stride) {
  return visit_all_masked(g, k, proto, nout, out, threads, stride, NULL);
}

uint64_t orc_count_cliques(const orc_graph *g, int k, uint64_t *per_vertex) {
  visit_t p;
  memset(&p, 0, sizeof p);
  p.kind = 2;
  uint64_t *tmp = per_vertex ? per_vertex : (uint64_t *)xcalloc((size_t)g->n + 1, sizeof(uint64_t));
  uint64_t c = visit_all(g, k, p, g->n, tmp, omp_get_max_threads(), 1);
  if (!per_vertex) free(tmp);
  return c;
}

/* ---- Seq-kClist++ pass, CDF_CliqueEnum FRANK_WOLFE, kCDensestNoAtom.c:270-295. */
static uint64_t seq_pass_impl_masked(const orc_graph *g, int k, uint64_t *rho, int mode, int threads,
                                     uint64_t stride, const uint8_t *root_mask) {
  const uint32_t n = g->n;
  uint64_t total = 0;
  if (stride == 0) stride = 1;
  if (g->e == 0) return 0;
  const int64_t ne = (int64_t)((g->e + stride - 1) / stride);
  if (mode == ORC_SEQ_SEQUENTIAL) {
    orc_ws *w = ws_new(g, k);
    for (int64_t q = 0; q < ne; ++q) {
      uint64_t i = (uint64_t)q * stride;
      uint32_t s = g->edges[i].s, t = g->edges[i].t;
      uint32_t ngw = rho[t] < rho[s] ? t : s;              /* :287 */
      make_subgraph(w, g, s, t);
      total += seq_rec(w, rho, k - 2, ngw);
    }
    ws_free(w);
    return total;
  }
  uint64_t *delta = (uint64_t *)xcalloc((size_t)n + 1, sizeof(uint64_t));
  uint64_t *rho_old = NULL;
  if (mode == ORC_SEQ_THREADS) {                             /* :271-273 */
    rho_old = (uint64_t *)xmalloc((size_t)n * sizeof(uint64_t));
    memcpy(rho_old, rho, (size_t)n * sizeof(uint64_t));
  }
  #pragma omp parallel num_threads(threads > 0 ? threads : 1) reduction(+:total)
  {
    orc_ws *w = ws_new(g, k);
    uint64_t *cur = (uint64_t *)xmalloc(((size_t)n + 1) * sizeof(uint64_t));
    memcpy(cur, rho, (size_t)n * sizeof(uint64_t));          /* :281-282 */
    uint64_t *acc = NULL;
    if (mode == ORC_SEQ_EDGE_STREAMS) acc = (uint64_t *)xcalloc((size_t)n + 1, sizeof(uint64_t));
    #pragma omp for schedule(dynamic, 1) nowait
    for (int64_t q = 0; q < ne; ++q) {
      uint64_t i = (uint64_t)q * stride;
      uint32_t s = g->edges[i].s, t = g->edges[i].t;
      if (root_mask && !root_mask[s]) continue;
      uint32_t ngw = cur[t] < cur[s] ? t : s;
      make_subgraph(w, g, s, t);
      total += seq_rec(w, cur, k - 2, ngw);
      if (mode == ORC_SEQ_EDGE_STREAMS) {
        /* Close this root edge's stream: its increments fell on {s, t} ∪ C. */
        acc[s] += cur[s] - rho[s]; cur[s] = rho[s];
        acc[t] += cur[t] - rho[t]; cur[t] = rho[t];
        for (uint32_t j = 0; j < w->nn[k - 2]; ++j) {
          uint32_t x = w->sg2g[j];
          acc[x] += cur[x] - rho[x];
          cur[x] = rho[x];
        }
      }
    }
    #pragma omp critical                                     /* :291-293 */
    {
      if (mode == ORC_SEQ_EDGE_STREAMS) {
        for (uint32_t x = 0; x < n; ++x) delta[x] += acc[x];
      } else {
        for (uint32_t x = 0; x < n; ++x) delta[x] += cur[x] - rho_old[x];
      }
    }
    free(acc);
    free(cur);
    ws_free(w);
  }
  for (uint32_t x = 0; x < n; ++x) rho[x] += delta[x];
  free(delta);
  free(rho_old);
  return total;
}

/* Per-root-vertex streams: every root edge of one root vertex s, in (s, t)
 * order, in one chain from the pass-start r (its increments stay visible to
 * the later root edges of s); the roots' chains are independent and summed.
 * Every vertex a chain touches lies in {s} ∪ N+(s). */
static uint64_t seq_pass_vertex_streams(const orc_graph *g, int k, uint64_t *rho, int threads) {
  const uint32_t n = g->n;
  uint64_t total = 0;
  if (g->e == 0) return 0;
  uint64_t *delta = (uint64_t *)xcalloc((size_t)n + 1, sizeof(uint64_t));
  #pragma omp parallel num_threads(threads > 0 ? threads : 1) reduction(+:total)
  {
    orc_ws *w = ws_new(g, k);
    uint64_t *cur = (uint64_t *)xmalloc(((size_t)n + 1) * sizeof(uint64_t));
    memcpy(cur, rho, (size_t)n * sizeof(uint64_t));
    uint64_t *acc = (uint64_t *)xcalloc((size_t)n + 1, sizeof(uint64_t));
    #pragma omp for schedule(dynamic, 1) nowait
    for (int64_t sv = 0; sv < (int64_t)n; ++sv) {
      const uint32_t s = (uint32_t)sv;
      if (g->cd[s] == g->cd[s + 1]) continue;
      for (uint64_t i = g->cd[s]; i < g->cd[s + 1]; ++i) {
        const uint32_t t = g->adj[i];
        const uint32_t ngw = cur[t] < cur[s] ? t : s;
        make_subgraph(w, g, s, t);
        total += seq_rec(w, cur, k - 2, ngw);
      }
      acc[s] += cur[s] - rho[s];
      cur[s] = rho[s];
      for (uint64_t i = g->cd[s]; i < g->cd[s + 1]; ++i) {
        const uint32_t x = g->adj[i];
        acc[x] += cur[x] - rho[x];
        cur[x] = rho[x];
      }
    }
    #pragma omp critical
    for (uint32_t x = 0; x < n; ++x) delta[x] += acc[x];
    free(acc);
    free(cur);
    ws_free(w);
  }
  for (uint32_t x = 0; x < n; ++x) rho[x] += delta[x];
  free(delta);
  return total;
}

static uint64_t seq_pass_impl(const orc_graph *g, int k, uint64_t *rho, int mode, int threads,
                              uint64_t stride) {
  if (mode == ORC_SEQ_VERTEX_STREAMS) return seq_pass_vertex_streams(g, k, rho, threads);
  return seq_pass_impl_masked(g, k, rho, mode, threads, stride, NULL);
}

/* Per-root-edge-stream increments of the root edges whose source is marked
 * in root_mask (one shard of a split pass): delta = r_after - r. */
int orc_seq_delta_masked(const orc_graph *g, int k, const uint64_t *rho, const uint8_t *root_mask, int threads,
                         uint64_t *delta) {
  if (k < 3 || k >= ORC_MAXK) return -1;
  uint64_t *tmp = (uint64_t *)xmalloc(((size_t)g->n + 1) * sizeof(uint64_t));
  memcpy(tmp, rho, (size_t)g->n * sizeof(uint64_t));
  seq_pass_impl_masked(g, k, tmp, ORC_SEQ_EDGE_STREAMS, threads, 1, root_mask);
  for (uint32_t x = 0; x < g->n; ++x) delta[x] = tmp[x] - rho[x];
  free(tmp);
  return 0;
}

/* Sim rho_add of the marked roots' cliques. */
void orc_sim_counts_masked(const orc_graph *g, int k, const double *rho, const uint8_t *root_mask, int threads,
                           uint64_t *cnt) {
  visit_t p;
  memset(&p, 0, sizeof p);
  p.kind = 0;
  p.rho = rho;
  visit_all_masked(g, k, p, g->n, cnt, threads, 1, root_mask);
}

/* Wave ordering: root vertices grouped by (uint32)(s * 2654435761) % waves;
 * the waves run in order, each one's root-edge streams starting from r as the
 * earlier waves left it. */
int orc_seq_pass_waves(const orc_graph *g, int k, uint64_t *rho, uint32_t waves, int threads) {
  if (k < 3 || k >= ORC_MAXK || waves == 0) return -1;
  uint8_t *mask = (uint8_t *)xmalloc((size_t)g->n + 1);
  uint64_t *delta = (uint64_t *)xmalloc(((size_t)g->n + 1) * sizeof(uint64_t));
  for (uint32_t w = 0; w < waves; ++w) {
    for (uint32_t s = 0; s < g->n; ++s) mask[s] = ((uint32_t)(s * 2654435761u) % waves) == w;
    orc_seq_delta_masked(g, k, rho, mask, threads, delta);
    for (uint32_t x = 0; x < g->n; ++x) rho[x] += delta[x];
  }
  free(mask);
  free(delta);
  return 0;
}

int orc_seq_pass(const orc_graph *g, int k, uint64_t *rho, int mode, int threads) {
  if (k < 3 || k >= ORC_MAXK) return -1;
  seq_pass_impl(g, k, rho, mode, threads, 1);
  return 0;
}

/* Sampled pass for the timed CPU baseline: every stride-th root edge. */
uint64_t orc_seq_pass_sample(const orc_graph *g, int k, uint64_t *rho, int mode, int threads,
                             uint64_t stride) {
  if (k < 3 || k >= ORC_MAXK) return 0;
  return seq_pass_impl(g, k, rho, mode, threads, stride);
}

/* PAVA_PREPROCESS pass, kCDensestNoAtom.c:191-213, 296-309 (and the Sim copy,
 * kCDensestCmpSync.c:217-245): tentative[level] = cliques whose largest level
 * member has that level.                                                    */
void orc_seq_pava(const orc_graph *g, int k, const uint32_t *level, uint64_t *tentative, int threads) {
  visit_t p;
  memset(&p, 0, sizeof p);
  p.kind = 1;
  p.level = level;
  visit_all(g, k, p, g->n, tentative, threads, 1);
}
void orc_sim_pava(const orc_graph *g, int k, const uint32_t *level, uint64_t *tentative, int threads) {
  orc_seq_pava(g, k, level, tentative, threads);
}

/* Sim-kClist++ FRANK_WOLFE pass, kCDensestCmpSync.c:138-146, 188-216, 298-325:
 * cnt[v] = number of cliques whose (rho, id)-smallest member is v.          */
void orc_sim_counts(const orc_graph *g, int k, const double *rho, uint64_t *cnt, int threads) {
  visit_t p;
  memset(&p, 0, sizeof p);
  p.kind = 0;
  p.rho = rho;
  visit_all(g, k, p, g->n, cnt, threads, 1);
}
uint64_t orc_sim_counts_sample(const orc_graph *g, int k, const double *rho, uint64_t *cnt,
                               int threads, uint64_t stride) {
  visit_t p;
  memset(&p, 0, sizeof p);
  p.kind = 0;
  p.rho = rho;
  return visit_all(g, k, p, g->n, cnt, threads, stride);
}

/* kCDensestCmpSync.c:402-403, no fused multiply-add. */
void orc_sim_update(uint32_t n, uint32_t t, double *rho, const uint64_t *cnt) {
  for (uint32_t i = 0; i < n; ++i) {
    double add = (double)cnt[i];
    rho[i] = (t * rho[i] + 2.0 * add) / (t + 2.0);
  }
}

/* ---- A10: sort by r.  glibc's qsort is a stable merge sort for these sizes,
 * and reordered starts as the identity, so ties keep ascending ids
 * (kCDensestNoAtom.c:322-337, kCDensestCmpSync.c:334-349).                  */
typedef struct { uint64_t key; uint32_t id; } keyid_t;
static int keyid_desc(const void *a, const void *b) {
  const keyid_t *x = (const keyid_t *)a, *y = (const keyid_t *)b;
  if (x->key != y->key) return x->key > y->key ? -1 : 1;
  return x->id < y->id ? -1 : (x->id > y->id);
}
void orc_sort_by_r_u64(uint32_t n, const uint64_t *rho, uint32_t *reordered) {
  keyid_t *a = (keyid_t *)xmalloc((size_t)n * sizeof(keyid_t));
  for (uint32_t i = 0; i < n; ++i) { a[i].key = rho[i]; a[i].id = i; }
  qsort(a, n, sizeof(keyid_t), keyid_desc);
  for (uint32_t i = 0; i < n; ++i) reordered[i] = a[i].id;
  free(a);
}
void orc_sort_by_r_f64(uint32_t n, const double *rho, uint32_t *reordered) {
  keyid_t *a = (keyid_t *)xmalloc((size_t)n * sizeof(keyid_t));
  for (uint32_t i = 0; i < n; ++i) { a[i].key = (unsigned long long)rho[i]; a[i].id = i; }
  qsort(a, n, sizeof(keyid_t), keyid_desc);
  for (uint32_t i = 0; i < n; ++i) reordered[i] = a[i].id;
  free(a);
}

/* CDF_FindDensestSubset, kCDensestNoAtom.c:330-371. */
orc_info orc_seq_find_densest(const orc_graph *g, int k, uint32_t T, const uint64_t *rho,
                              uint32_t *reordered, uint32_t *level, int threads) {
  orc_info info;
  memset(&info, 0, sizeof info);
  info.density = -1;
  const uint32_t n = g->n;
  if (n == 0) { info.density = 0; return info; }
  orc_sort_by_r_u64(n, rho, reordered);
  for (uint32_t i = 0; i < n; ++i) level[reordered[i]] = i;
  uint64_t *tent = (uint64_t *)xcalloc(n, sizeof(uint64_t));
  orc_seq_pava(g, k, level, tent, threads);
  unsigned long long sum = 0;
  for (uint32_t i = 0; i < n; ++i) {
    sum += tent[i];
    if ((double)sum / (i + 1) > info.density) {
      info.density = (double)sum / (i + 1);
      info.n = i + 1;
      info.cliques = sum;
    }
  }
  free(tent);
  info.m = orc_count_edges(g, info.n, reordered);
  sum = 0;
  info.ub = 0;
  double ip1ck = 1;
  for (uint32_t i = 0; i < n; ++i) {
    sum += rho[reordered[i]];
    if (i + 1 == (uint32_t)k) ip1ck = 1;
    else if (i + 1 > (uint32_t)k) ip1ck = (ip1ck * (i + 1)) / (i + 1 - k);
    if (ip1ck < (double)sum / T) info.ub = ip1ck / (i + 1);
    else {
      if (info.ub < (double)sum / T / (i + 1)) info.ub = (double)sum / T / (i + 1);
      break;
    }
  }
  return info;
}

/* CDF_FindDensestSubset, kCDensestCmpSync.c:342-383 (double accumulators). */
orc_info orc_sim_find_densest(const orc_graph *g, int k, const double *rho,
                              uint32_t *reordered, uint32_t *level, int threads) {
  orc_info info;
  memset(&info, 0, sizeof info);
  info.density = -1;
  const uint32_t n = g->n;
  if (n == 0) { info.density = 0; return info; }
  orc_sort_by_r_f64(n, rho, reordered);
  for (uint32_t i = 0; i < n; ++i) level[reordered[i]] = i;
  uint64_t *tent = (uint64_t *)xcalloc(n, sizeof(uint64_t));
  orc_sim_pava(g, k, level, tent, threads);
  double sum = 0;
  uint64_t isum = 0;
  for (uint32_t i = 0; i < n; ++i) {
    sum += (double)tent[i];
    isum += tent[i];
    if (sum / (i + 1) > info.density) {
      info.density = (double)sum / (i + 1);
      info.n = i + 1;
      info.cliques = isum;
    }
  }
  free(tent);
  info.m = orc_count_edges(g, info.n, reordered);
  sum = 0;
  info.ub = 0;
  double ip1ck = 1;
  for (uint32_t i = 0; i < n; ++i) {
    sum += rho[reordered[i]];
    if (i + 1 == (uint32_t)k) ip1ck = 1;
    else if (i + 1 > (uint32_t)k) ip1ck = (ip1ck * (i + 1)) / (i + 1 - k);
    if (ip1ck < sum) info.ub = ip1ck / (i + 1);
    else {
      if (info.ub < sum / (i + 1)) info.ub = sum / (i + 1);
      break;
    }
  }
  return info;
}

/* CDF_Main, kCDensestNoAtom.c:373-402. */
int orc_seq_main(const orc_graph *g, int k, uint32_t num_iter, int mode, int threads,
                 uint64_t *rho_out, orc_info *infos, int max_infos) {
  if (k < 3 || k >= ORC_MAXK) return -1;
  const uint32_t n = g->n;
  uint64_t *rho = (uint64_t *)xcalloc((size_t)n + 1, sizeof(uint64_t));
  uint32_t *reordered = (uint32_t *)xmalloc(((size_t)n + 1) * sizeof(uint32_t));
  uint32_t *level = (uint32_t *)xmalloc(((size_t)n + 1) * sizeof(uint32_t));
  int c = 0;
  for (uint32_t T = 1, t = 1; T <= num_iter; T <<= 1) {
    for (; t <= T; ++t) orc_seq_pass(g, k, rho, mode, threads);
    orc_info info = orc_seq_find_densest(g, k, T, rho, reordered, level, threads);
    if (c < max_infos) infos[c] = info;
    ++c;
  }
  if (rho_out) memcpy(rho_out, rho, (size_t)n * sizeof(uint64_t));
  free(rho); free(reordered); free(level);
  return c;
}

/* CDF_Main, kCDensestCmpSync.c:385-419. */
int orc_sim_main(const orc_graph *g, int k, uint32_t num_iter, int threads,
                 double *rho_out, orc_info *infos, int max_infos) {
  if (k < 2 || k >= ORC_MAXK) return -1;
  const uint32_t n = g->n;
  double *rho = (double *)xcalloc((size_t)n + 1, sizeof(double));
  uint64_t *cnt = (uint64_t *)xcalloc((size_t)n + 1, sizeof(uint64_t));
  uint32_t *reordered = (uint32_t *)xmalloc(((size_t)n + 1) * sizeof(uint32_t));
  uint32_t *level = (uint32_t *)xmalloc(((size_t)n + 1) * sizeof(uint32_t));
  int c = 0;
  for (uint32_t T = 1, t = 1; T <= num_iter; T <<= 1) {
    for (; t <= T; ++t) {
      if (k == 2) {
        /* clique_size == 2 (kCDensestCmpSync.c:189-192): each root edge is a clique. */
        memset(cnt, 0, (size_t)n * sizeof(uint64_t));
        for (uint64_t i = 0; i < g->e; ++i) {
          uint32_t s = g->edges[i].s, tt = g->edges[i].t;
          cnt[sim_less(rho, tt, s) ? tt : s]++;
        }
      } else {
        orc_sim_counts(g, k, rho, cnt, threads);
      }
      orc_sim_update(n, t, rho, cnt);
    }
    orc_info info;
    if (k == 2) {
      memset(&info, 0, sizeof info);
      orc_sort_by_r_f64(n, rho, reordered);
      for (uint32_t i = 0; i < n; ++i) level[reordered[i]] = i;
      uint64_t *tent = (uint64_t *)xcalloc((size_t)n + 1, sizeof(uint64_t));
      for (uint64_t i = 0; i < g->e; ++i) {
        uint32_t s = g->edges[i].s, tt = g->edges[i].t;
        tent[level[level[tt] > level[s] ? tt : s]]++;
      }
      double sum = 0; uint64_t isum = 0;
      info.density = -1;
      for (uint32_t i = 0; i < n; ++i) {
        sum += (double)tent[i]; isum += tent[i];
        if (sum / (i + 1) > info.density) { info.density = sum / (i + 1); info.n = i + 1; info.cliques = isum; }
      }
      free(tent);
      info.m = orc_count_edges(g, info.n, reordered);
      sum = 0; info.ub = 0;
      double ip1ck = 1;
      for (uint32_t i = 0; i < n; ++i) {
        sum += rho[reordered[i]];
        if (i + 1 == (uint32_t)k) ip1ck = 1;
        else if (i + 1 > (uint32_t)k) ip1ck = (ip1ck * (i + 1)) / (i + 1 - k);
        if (ip1ck < sum) info.ub = ip1ck / (i + 1);
        else { if (info.ub < sum / (i + 1)) info.ub = sum / (i + 1); break; }
      }
    } else {
      info = orc_sim_find_densest(g, k, rho, reordered, level, threads);
    }
    if (c < max_infos) infos[c] = info;
    ++c;
  }
  if (rho_out) memcpy(rho_out, rho, (size_t)n * sizeof(double));
  free(rho); free(cnt); free(reordered); free(level);
  return c;
}

/* ------------------------------------------------------------------------ */
/* k-clique core trim, kClistCoreTrim.c.                                     */

/* Sorted-list intersection (kClistCoreTrim.c:348-365), without the reference's
 * one-past-the-end reads. */
static uint32_t intersect(const uint32_t *a, uint32_t na, const uint32_t *b, uint32_t nb, uint32_t *out) {
  uint32_t i = 0, j = 0, s = 0;
  while (i < na && j < nb) {
    if (a[i] < b[j]) ++i;
    else if (b[j] < a[i]) ++j;
    else { out[s++] = a[i]; ++i; ++j; }
  }
  return s;
}

typedef struct {
  uint32_t kmax, core;
  const uint64_t *cd;   /* sorted DAG out-CSR (mkspecial) */
  const uint32_t *adj;
  uint32_t *merge, *size, *ck;
  uint64_t *nck;
} trim_rec_t;

/* recursion, kClistCoreTrim.c:368-391 */
static void trim_recursion(trim_rec_t *r, uint32_t k) {
  uint32_t t = (k - 3) * r->core, t2 = t + r->core;
  if (r->size[k - 3] < r->kmax - k) return;
  if (k == r->kmax) {
    for (uint32_t i = 0; i < r->kmax - 1; ++i) r->nck[r->ck[i]] += r->size[k - 3];
    for (uint32_t i = 0; i < r->size[k - 3]; ++i) r->nck[r->merge[t + i]]++;
    return;
  }
  for (uint32_t i = 0; i < r->size[k - 3]; ++i) {
    uint32_t x = r->merge[t + i];
    r->ck[k - 1] = x;
    r->size[k - 2] = intersect(r->adj + r->cd[x], (uint32_t)(r->cd[x + 1] - r->cd[x]),
                               r->merge + t, r->size[k - 3], r->merge + t2);
    trim_recursion(r, k + 1);
  }
}

static int u32cmp(const void *a, const void *b) {
  uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
  return x < y ? -1 : (x > y);
}

int orc_trim(uint32_t n, uint64_t e, const orc_edge *edges_in, int kmax, orc_trim_result *out) {
  memset(out, 0, sizeof *out);
  if (kmax < 3 || kmax >= ORC_MAXK) return -1;
  out->n = n;
  out->e = e;
  /* mkgraph, kClistCoreTrim.c:198-220 */
  uint32_t *d0 = (uint32_t *)xcalloc(n, sizeof(uint32_t));
  uint64_t *cd0 = (uint64_t *)xmalloc(((size_t)n + 1) * sizeof(uint64_t));
  uint32_t *adj0 = (uint32_t *)xmalloc((size_t)(2 * e) * sizeof(uint32_t));
  for (uint64_t i = 0; i < e; ++i) { d0[edges_in[i].s]++; d0[edges_in[i].t]++; }
  cd0[0] = 0;
  for (uint32_t i = 1; i <= n; ++i) { cd0[i] = cd0[i - 1] + d0[i - 1]; d0[i - 1] = 0; }
  for (uint64_t i = 0; i < e; ++i) {
    uint32_t s = edges_in[i].s, t = edges_in[i].t;
    adj0[cd0[s] + d0[s]++] = t;
    adj0[cd0[t] + d0[t]++] = s;
  }
  /* kcore, kClistCoreTrim.c:242-272 */
  uint32_t *rank = (uint32_t *)xmalloc((size_t)n * sizeof(uint32_t));
  uint32_t *map = (uint32_t *)xmalloc((size_t)n * sizeof(uint32_t));
  {
    orc_heap h;
    heap_init(&h, n);
    for (uint32_t i = 0; i < n; ++i) heap_insert(&h, i, d0[i]);
    uint32_t r = 0, nn = n, c = 0, kk = (uint32_t)kmax - 1;
    for (uint32_t i = 0; i < n; ++i) {
      orc_kv kv = heap_pop(&h);
      if (kv.value > c) c = (uint32_t)kv.value;
      if (c < kk) { rank[kv.key] = NIL32; nn--; }
      else { map[nn - (++r)] = kv.key; rank[kv.key] = nn - r; }
      for (uint64_t j = cd0[kv.key]; j < cd0[kv.key + 1]; ++j) heap_dec(&h, adj0[j], 1);
    }
    heap_free(&h);
    out->core = c;
    out->n2 = nn;
  }
  free(d0); free(cd0); free(adj0);
  const uint32_t n2 = out->n2;
  /* relabelnodes, kClistCoreTrim.c:274-294 */
  orc_edge *E = (orc_edge *)xmalloc((size_t)e * sizeof(orc_edge));
  uint64_t e2 = 0;
  for (uint64_t i = 0; i < e; ++i) {
    uint32_t s = rank[edges_in[i].s], t = rank[edges_in[i].t];
    if (s == NIL32 || t == NIL32) continue;
    if (s < t) { E[e2].s = t; E[e2].t = s; }
    else { E[e2].s = s; E[e2].t = t; }
    ++e2;
  }
  out->e2 = e2;
  free(rank);
  out->map = (uint32_t *)xmalloc(((size_t)n2 + 1) * sizeof(uint32_t));
  memcpy(out->map, map, (size_t)n2 * sizeof(uint32_t));
  free(map);
  out->nck = (uint64_t *)xcalloc((size_t)n2 + 1, sizeof(uint64_t));
  out->order = (uint32_t *)xcalloc((size_t)n2 + 1, sizeof(uint32_t));
  out->core_num = (uint64_t *)xcalloc((size_t)n2 + 1, sizeof(uint64_t));
  if (n2 == 0) {
    out->trimmed = (orc_edge *)xmalloc(sizeof(orc_edge));
    free(E);
    return 0;
  }
  /* mkspecial, kClistCoreTrim.c:306-331 */
  uint64_t *cd = (uint64_t *)xcalloc((size_t)n2 + 1, sizeof(uint64_t));
  uint32_t *adj = (uint32_t *)xmalloc((size_t)e2 * sizeof(uint32_t) + 4);
  uint32_t *dd = (uint32_t *)xcalloc(n2, sizeof(uint32_t));
  for (uint64_t i = 0; i < e2; ++i) cd[E[i].s + 1]++;
  for (uint32_t i = 1; i <= n2; ++i) cd[i] += cd[i - 1];
  for (uint64_t i = 0; i < e2; ++i) adj[cd[E[i].s] + dd[E[i].s]++] = E[i].t;
  for (uint32_t i = 0; i < n2; ++i) qsort(adj + cd[i], dd[i], sizeof(uint32_t), u32cmp);
  free(dd);
  /* onepass, kClistCoreTrim.c:394-416 */
  const uint32_t core = out->core ? out->core : 1;
  trim_rec_t R;
  R.kmax = (uint32_t)kmax;
  R.core = core;
  R.cd = cd;
  R.adj = adj;
  R.merge = (uint32_t *)xmalloc((size_t)(kmax - 2) * core * sizeof(uint32_t));
  R.size = (uint32_t *)xcalloc(kmax, sizeof(uint32_t));
  R.ck = (uint32_t *)xcalloc(kmax, sizeof(uint32_t));
  R.nck = out->nck;
  for (uint64_t i = 0; i < e2; ++i) {
    uint32_t s = E[i].s, t = E[i].t;
    R.ck[0] = s; R.ck[1] = t;
    R.size[0] = intersect(adj + cd[s], (uint32_t)(cd[s + 1] - cd[s]), adj + cd[t],
                          (uint32_t)(cd[t + 1] - cd[t]), R.merge);
    trim_recursion(&R, 3);
  }
  uint64_t tot = 0;
  for (uint32_t i = 0; i < n2; ++i) tot += out->nck[i];
  tot /= (uint64_t)kmax;                                 /* :741-742 */
  out->total = tot;
  /* mkgraph2, kClistCoreTrim.c:547-573: undirected sorted CSR of survivors */
  uint64_t *cu = (uint64_t *)xcalloc((size_t)n2 + 1, sizeof(uint64_t));
  uint32_t *au = (uint32_t *)xmalloc((size_t)(2 * e2) * sizeof(uint32_t) + 4);
  uint32_t *du = (uint32_t *)xcalloc(n2, sizeof(uint32_t));
  for (uint64_t i = 0; i < e2; ++i) { cu[E[i].s + 1]++; cu[E[i].t + 1]++; }
  for (uint32_t i = 1; i <= n2; ++i) cu[i] += cu[i - 1];
  for (uint64_t i = 0; i < e2; ++i) {
    au[cu[E[i].s] + du[E[i].s]++] = E[i].t;
    au[cu[E[i].t] + du[E[i].t]++] = E[i].s;
  }
  for (uint32_t i = 0; i < n2; ++i) qsort(au + cu[i], du[i], sizeof(uint32_t), u32cmp);
  free(du);
  /* kcliquecore, kClistCoreTrim.c:605-666 */
  {
    orc_heap h;
    heap_init(&h, n2);
    for (uint32_t i = 0; i < n2; ++i) heap_insert(&h, i, out->nck[i]);
    uint64_t c = 0, ncktot = tot;
    uint32_t ecount = (uint32_t)e2;  /* `unsigned e` in the reference */
    uint64_t *whendel = (uint64_t *)xcalloc((size_t)n2 + 1, sizeof(uint64_t));
    uint64_t *nck2 = (uint64_t *)xcalloc((size_t)n2 + 1, sizeof(uint64_t));
    uint32_t *live = (uint32_t *)xmalloc(((size_t)n2 + 1) * sizeof(uint32_t));
    out->ncktrim = tot;
    out->ckrho = ((double)ncktot) / ((double)n2);
    out->size = n2;
    out->rho = ((double)(2 * ecount)) / ((double)(n2 * (n2 - 1)));
    R.nck = nck2;
    uint32_t i;
    for (i = 0; i < n2 - 1; ++i) {
      orc_kv kv = heap_pop(&h);
      uint32_t u = kv.key;
      if (kv.value > c) c = kv.value;
      out->order[i] = u;
      out->core_num[i] = c;
      /* oneshortpass, kClistCoreTrim.c:577-603 */
      uint32_t s = 0;
      for (uint64_t j = cu[u]; j < cu[u + 1]; ++j) {
        uint32_t v = au[j];
        if (h.p[v] != NIL32) live[s++] = v;
      }
      if (s > (uint32_t)kmax - 2) {
        R.ck[0] = u;
        for (uint32_t q = 0; q < s; ++q) {
          uint32_t v = live[q];
          R.ck[1] = v;
          R.size[0] = intersect(live, s, adj + cd[v], (uint32_t)(cd[v + 1] - cd[v]), R.merge);
          trim_recursion(&R, 3);
        }
      }
      uint64_t ncktot2 = 0;
      for (uint64_t j = cu[u]; j < cu[u + 1]; ++j) {
        uint32_t v = au[j];
        if (h.p[v] != NIL32) {
          ecount--;
          heap_dec(&h, v, nck2[v]);
          ncktot2 += nck2[v];
          nck2[v] = 0;
        }
      }
      uint32_t size_tmp = n2 - i - 1;
      whendel[size_tmp] = ncktot2 / ((uint64_t)(kmax - 1));
      ncktot -= whendel[size_tmp];
      double ckrho_tmp = ((double)ncktot) / ((double)size_tmp);
      if (ckrho_tmp > out->ckrho) {
        out->ckrho = ckrho_tmp;
        out->size = size_tmp;
        out->rho = ((double)(2 * ecount)) / ((double)(size_tmp * (size_tmp - 1)));
      }
    }
    out->ntrim = n2;  /* the reference leaves this unset when n2 == 1 */
    for (uint32_t j = n2 - 1; j >= 1; --j) {
      if ((double)whendel[j] >= out->ckrho) { out->ntrim = j + 1; break; }
      out->ncktrim -= whendel[j];
    }
    orc_kv kv = heap_pop(&h);
    out->order[i] = kv.key;
    out->core_num[i] = c;
    out->ckcore = c;
    heap_free(&h);
    free(whendel); free(nck2); free(live);
  }
  /* printdensest trimmed graph, kClistCoreTrim.c:686-699 */
  {
    char *alive = (char *)xcalloc(n2, 1);
    for (uint32_t i = n2 - 1; i != n2 - out->ntrim - 1; --i) alive[out->order[i]] = 1;
    out->trimmed = (orc_edge *)xmalloc(((size_t)e2 + 1) * sizeof(orc_edge));
    uint64_t m = 0;
    for (uint64_t i = 0; i < e2; ++i) {
      if (alive[E[i].s] && alive[E[i].t]) {
        out->trimmed[m].s = out->map[E[i].s];
        out->trimmed[m].t = out->map[E[i].t];
        ++m;
      }
    }
    out->mtrim = m;
    free(alive);
  }
  free(R.merge); free(R.size); free(R.ck);
  free(cd); free(adj); free(cu); free(au); free(E);
  return 0;
}

void orc_free_trim(orc_trim_result *r) {
  free(r->map); free(r->nck); free(r->order); free(r->core_num); free(r->trimmed);
  memset(r, 0, sizeof *r);
}

/* ======================================================================== */
/* Seq-Sampling++ (kCDensestSamplingKclistpp.c) with the library's
 * counter-based sample in place of rand(): a clique Q is kept iff
 * mix64(sum of key(v), v in Q) < threshold (or every clique with all), key(v)
 * = mix64(seed + (v + 1) * 0x9E3779B97F4A7C15), mix64 = SplitMix64's output
 * function (Steele, Lea and Flood, OOPSLA 2014); its wave is
 * ((mix64(sum ^ 0xD1B54A32D192ED03) >> 32) * waves) >> 32.                  */
static inline uint64_t smp_mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
uint64_t orc_sample_key(uint64_t seed, uint32_t v) {
  return smp_mix64(seed + ((uint64_t)v + 1ull) * 0x9E3779B97F4A7C15ull);
}

typedef struct {
  uint64_t seed, threshold;
  int all;
  uint32_t waves;
  uint32_t *rows;
  uint8_t *wave;
  uint64_t cap, kept;
  uint32_t pre[ORC_MAXK];  /* global ids of the prefix: s, t, then deeper members */
} sample_t;

/* One clique: the prefix pre[0, depth) plus the members in last[0, nl)
 * (deepest last). */
static void sample_one(sample_t *st, int k, int depth, const uint32_t *last, int nl) {
  uint64_t h = 0;
  for (int q = 0; q < depth; ++q) h += orc_sample_key(st->seed, st->pre[q]);
  for (int q = 0; q < nl; ++q) h += orc_sample_key(st->seed, last[q]);
  if (!st->all && !(smp_mix64(h) < st->threshold)) return;
  if (st->kept < st->cap) {
    /* ascending ids: deepest member first (the ck[] rows,
     * kCDensestSamplingKclistpp.c:166-170 and 204-209) */
    uint32_t *row = st->rows + st->kept * (uint64_t)k;
    int j = 0;
    for (int q = nl - 1; q >= 0; --q) row[j++] = last[q];
    for (int q = depth - 1; q >= 0; --q) row[j++] = st->pre[q];
    st->wave[st->kept] = (uint8_t)(((smp_mix64(h ^ 0xD1B54A32D192ED03ull) >> 32) * (uint64_t)st->waves) >> 32);
  }
  st->kept++;
}

/* KCLIST_CliqueEnumThread with the SAMPLING task
 * (kCDensestSamplingKclistpp.c:148-258), on the workspace of the other
 * passes: every clique in enumeration order.                              */
static void sample_rec(orc_ws *w, sample_t *st, int l, int depth) {
  if (w->k == 3) {
    for (uint32_t i = 0; i < w->nn[1]; ++i) {
      uint32_t x = w->sg2g[w->nodes[1][i]];
      sample_one(st, 3, depth, &x, 1);
    }
    return;
  }
  if (l == 2) {
    for (uint32_t i = 0; i < w->nn[2]; ++i) {
      uint32_t u = w->nodes[2][i];
      const uint32_t *au = w->adj[2] + (size_t)w->core * u;
      for (uint32_t j = 0; j < w->deg[2][u]; ++j) {
        uint32_t last[2] = {w->sg2g[u], w->sg2g[au[j]]};
        sample_one(st, w->k, depth, last, 2);
      }
    }
    return;
  }
  if (w->nn[l] < (uint32_t)l) return;
  for (uint32_t i = 0; i < w->nn[l]; ++i) {
    uint32_t u = w->nodes[l][i];
    st->pre[depth] = w->sg2g[u];
    descend(w, l, u);
    sample_rec(w, st, l - 1, depth + 1);
    ascend(w, l);
  }
}

uint64_t orc_sampling_collect(const orc_graph *g, int k, uint64_t seed, uint64_t threshold, int all,
                              uint32_t waves, uint32_t *rows, uint8_t *wave, uint64_t cap) {
  if (k < 3 || k > ORC_MAXK || g->e == 0) return 0;
  sample_t st;
  memset(&st, 0, sizeof st);
  st.seed = seed;
  st.threshold = threshold;
  st.all = all;
  st.waves = waves;
  st.rows = rows;
  st.wave = wave;
  st.cap = cap;
  orc_ws *w = ws_new(g, k);
  for (uint64_t i = 0; i < g->e; ++i) {  /* root edges in (s, t) order, :287-292 */
    st.pre[0] = g->edges[i].s;
    st.pre[1] = g->edges[i].t;
    make_subgraph(w, g, g->edges[i].s, g->edges[i].t);
    sample_rec(w, &st, k - 2, 2);
  }
  ws_free(w);
  return st.kept;
}

/* The member of a stored clique that takes its unit: the smallest value,
 * ties to the earliest member of the row (InMemoryFrankWolfe,
 * kCDensestSamplingKclistpp.c:353-359). */
static inline uint32_t smp_argmin(const uint32_t *row, int k, const uint32_t *rho) {
  uint32_t g = row[0];
  for (int j = 1; j < k; ++j)
    if (rho[row[j]] < rho[g]) g = row[j];
  return g;
}

/* InMemoryFrankWolfe's update (:345-361) with the visiting order given:
 * order[q] is the row taken at step q. */
void orc_sampling_pass_order(int k, uint64_t S, const uint32_t *rows, const uint32_t *order, uint32_t *rho) {
  for (uint64_t q = 0; q < S; ++q) ++rho[smp_argmin(rows + (uint64_t)order[q] * k, k, rho)];
}

/* The library's wave pass: waves one after another; the rows of a wave all
 * read the values the earlier waves left. */
void orc_sampling_pass(uint32_t n, int k, uint64_t S, const uint32_t *rows, const uint8_t *wave, uint32_t waves,
                       uint32_t *rho) {
  uint32_t *delta = (uint32_t *)xcalloc((size_t)n + 1, sizeof(uint32_t));
  for (uint32_t w = 0; w < waves; ++w) {
    for (uint64_t i = 0; i < S; ++i)
      if (wave[i] == w) ++delta[smp_argmin(rows + i * (uint64_t)k, k, rho)];
    for (uint32_t v = 0; v < n; ++v) {
      rho[v] += delta[v];
      delta[v] = 0;
    }
  }
  free(delta);
}

static const uint32_t *smp_sort_rho;
static int smp_rho_desc(const void *a, const void *b) {
  uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
  if (smp_sort_rho[x] != smp_sort_rho[y]) return smp_sort_rho[x] > smp_sort_rho[y] ? -1 : 1;
  return x < y ? -1 : (x > y);
}

/* ExtractDensest (kCDensestSamplingKclistpp.c:364-419): vertices by
 * decreasing load (ties: ascending id), each stored clique to its last vertex
 * in that order, the first strictly densest prefix, and the bound from the
 * loads.  Counters are 64-bit where the reference's unsigned would wrap. */
orc_sampling_info orc_sampling_extract(uint32_t n, int k, uint64_t S, const uint32_t *rows, const uint32_t *rho,
                                       uint32_t T, uint32_t *ordered) {
  orc_sampling_info info;
  memset(&info, 0, sizeof info);
  if (n == 0) return info;
  uint32_t *rank = (uint32_t *)xmalloc((size_t)n * sizeof(uint32_t));
  uint64_t *push = (uint64_t *)xcalloc(n, sizeof(uint64_t));
  for (uint32_t i = 0; i < n; ++i) ordered[i] = i;
  smp_sort_rho = rho;
  qsort(ordered, n, sizeof(uint32_t), smp_rho_desc);
  for (uint32_t i = 0; i < n; ++i) rank[ordered[i]] = i;
  for (uint64_t i = 0; i < S; ++i) {
    const uint32_t *row = rows + i * (uint64_t)k;
    uint32_t top = row[0];
    for (int j = 1; j < k; ++j)
      if (rank[row[j]] > rank[top]) top = row[j];
    ++push[rank[top]];
  }
  info.density = -1;
  uint64_t cnt = 0;
  for (uint32_t i = 0; i < n; ++i) {
    cnt += push[i];
    if (info.density < (double)cnt / (i + 1)) {
      info.n = i + 1;
      info.m = cnt;
      info.density = (double)cnt / (i + 1);
    }
  }
  uint64_t sum = 0;
  double ip1ck = 0;
  info.ub = 0;
  for (uint32_t i = 0; i < n; ++i) {
    sum += rho[ordered[i]];
    if (i + 1 == (uint32_t)k) ip1ck = 1;
    else if (i + 1 > (uint32_t)k) ip1ck = (ip1ck * (i + 1)) / (i + 1 - k);
    if (ip1ck < (double)sum / T) {
      info.ub = ip1ck / (i + 1);
    } else {
      if (info.ub < (double)sum / T / (i + 1)) info.ub = (double)sum / T / (i + 1);
      break;
    }
  }
  free(rank);
  free(push);
  return info;
}

/* ---- the benchmark's input graph (see kclpp_oracle.h) ------------------- */
typedef struct { uint64_t x; } orc_splitmix;
static inline uint64_t sm_next(orc_splitmix *r) {
  uint64_t z = (r->x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static inline double sm_uniform(orc_splitmix *r) { return (double)(sm_next(r) >> 11) * (1.0 / 9007199254740992.0); }
static inline uint64_t sm_below(orc_splitmix *r, uint64_t m) { return m ? sm_next(r) % m : 0; }
static inline uint64_t orc_pack(uint32_t u, uint32_t v) {
  if (u > v) { uint32_t t = u; u = v; v = t; }
  return ((uint64_t)u << 32) | v;
}

static void radix_u64(uint64_t *k, uint64_t n) {
  uint64_t *tmp = (uint64_t *)malloc((n ? n : 1) * sizeof(uint64_t));
  size_t *cnt = (size_t *)malloc((1u << 16) * sizeof(size_t));
  for (int sh = 0; sh < 64; sh += 16) {
    memset(cnt, 0, (1u << 16) * sizeof(size_t));
    for (uint64_t i = 0; i < n; ++i) cnt[(k[i] >> sh) & 0xFFFF]++;
    size_t sum = 0;
    for (uint32_t d = 0; d < (1u << 16); ++d) { size_t t = cnt[d]; cnt[d] = sum; sum += t; }
    for (uint64_t i = 0; i < n; ++i) tmp[cnt[(k[i] >> sh) & 0xFFFF]++] = k[i];
    memcpy(k, tmp, n * sizeof(uint64_t));
  }
  free(cnt);
  free(tmp);
}

int orc_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
             uint32_t **pairs, uint64_t *e, uint32_t *n_out) {
  if (scale < 1 || scale > 31 || edge_factor < 1) return -1;
  orc_splitmix r = {seed * 0x2545F4914F6CDD1Dull + 0x1234567ull};
  const double ab = a + b, abc = a + b + c;
  const uint32_t n = 1u << scale;
  const uint64_t samples = (uint64_t)edge_factor << scale;
  uint64_t *keys = (uint64_t *)malloc(samples * sizeof(uint64_t));
  uint64_t m = 0;
  for (uint64_t i = 0; i < samples; ++i) {
    uint32_t u = 0, v = 0;
    for (uint32_t l = 0; l < scale; ++l) {
      const double x = sm_uniform(&r);
      uint32_t bu = 0, bv = 0;
      if (x < a) {
      } else if (x < ab) {
        bv = 1;
      } else if (x < abc) {
        bu = 1;
      } else {
        bu = 1;
        bv = 1;
      }
      u = (u << 1) | bu;
      v = (v << 1) | bv;
    }
    if (u != v) keys[m++] = ((uint64_t)u << 32) | v;  /* ends mapped before canonicalising */
  }
  uint32_t *perm = (uint32_t *)malloc((size_t)n * sizeof(uint32_t));
  for (uint32_t i = 0; i < n; ++i) perm[i] = i;
  for (uint32_t i = n; i > 1; --i) {
    const uint64_t j = sm_below(&r, i);
    const uint32_t t = perm[i - 1];
    perm[i - 1] = perm[j];
    perm[j] = t;
  }
  for (uint64_t i = 0; i < m; ++i) keys[i] = orc_pack(perm[(uint32_t)(keys[i] >> 32)], perm[(uint32_t)keys[i]]);
  free(perm);
  radix_u64(keys, m);
  uint64_t w = 0;
  for (uint64_t i = 0; i < m; ++i)
    if (w == 0 || keys[i] != keys[w - 1]) keys[w++] = keys[i];
  uint32_t *P = (uint32_t *)malloc((w ? 2 * w : 2) * sizeof(uint32_t));
  uint32_t mx = 0;
  for (uint64_t i = 0; i < w; ++i) {
    P[2 * i] = (uint32_t)(keys[i] >> 32);
    P[2 * i + 1] = (uint32_t)keys[i];
    if (P[2 * i + 1] > mx) mx = P[2 * i + 1];
  }
  free(keys);
  *pairs = P;
  *e = w;
  *n_out = w ? mx + 1 : 1;
  return 0;
}

void orc_free(void *p) { free(p); }
