/*
 * ordering_study.c -- pass orderings of Seq-kClist++ that the library does
 * not ship, for the convergence study in oracle/ordering_study.py.
 *
 * TEST INFRASTRUCTURE ONLY: built into oracle/_build/libordering_study.so
 * (make -C oracle study), never linked into the library.  It includes the
 * oracle's own source so that the orderings below reuse its induced-subgraph
 * workspace and chain (make_subgraph, descend, seq_rec), which restate
 * kCDensestNoAtom.c:71-118 and 155-268.
 */
#include "kclpp_oracle.c"

/* Per-root-edge streams whose starting values extrapolate the pass: stream e
 * starts from r(x) + floor(tau_e * dprev(x)), tau_e = scale * e / |E|, dprev
 * the previous pass's increments. */
void orc_seq_pass_extrap(const orc_graph *g, int k, uint64_t *rho, const uint64_t *dprev, double scale,
                         int threads) {
  const uint32_t n = g->n;
  if (g->e == 0) return;
  uint64_t *delta = (uint64_t *)xcalloc((size_t)n + 1, sizeof(uint64_t));
  #pragma omp parallel num_threads(threads > 0 ? threads : 1)
  {
    orc_ws *w = ws_new(g, k);
    uint64_t *cur = (uint64_t *)xmalloc(((size_t)n + 1) * sizeof(uint64_t));
    uint64_t *base = (uint64_t *)xmalloc(((size_t)n + 1) * sizeof(uint64_t));
    uint64_t *acc = (uint64_t *)xcalloc((size_t)n + 1, sizeof(uint64_t));
    memcpy(cur, rho, (size_t)n * sizeof(uint64_t));
    #pragma omp for schedule(dynamic, 64) nowait
    for (int64_t q = 0; q < (int64_t)g->e; ++q) {
      const uint32_t s = g->edges[q].s, t = g->edges[q].t;
      make_subgraph(w, g, s, t);
      const double tau = scale * (double)q / (double)g->e;
      uint32_t touched[2] = {s, t};
      for (int a = 0; a < 2; ++a) {
        const uint32_t x = touched[a];
        cur[x] = rho[x] + (uint64_t)(tau * (double)dprev[x]);
        base[x] = cur[x];
      }
      for (uint32_t j = 0; j < w->nn[k - 2]; ++j) {
        const uint32_t x = w->sg2g[j];
        cur[x] = rho[x] + (uint64_t)(tau * (double)dprev[x]);
        base[x] = cur[x];
      }
      const uint32_t ngw = cur[t] < cur[s] ? t : s;
      seq_rec(w, cur, k - 2, ngw);
      for (int a = 0; a < 2; ++a) {
        const uint32_t x = touched[a];
        acc[x] += cur[x] - base[x];
        cur[x] = rho[x];
      }
      for (uint32_t j = 0; j < w->nn[k - 2]; ++j) {
        const uint32_t x = w->sg2g[j];
        acc[x] += cur[x] - base[x];
        cur[x] = rho[x];
      }
    }
    #pragma omp critical
    for (uint32_t x = 0; x < n; ++x) delta[x] += acc[x];
    free(acc);
    free(base);
    free(cur);
    ws_free(w);
  }
  for (uint32_t x = 0; x < n; ++x) rho[x] += delta[x];
  free(delta);
}

/* Every root vertex its own wave, roots in ascending order; the root's edges
 * are independent streams from r as the earlier roots left it. */
void orc_seq_pass_rootwaves(const orc_graph *g, int k, uint64_t *rho) {
  const uint32_t n = g->n;
  orc_ws *w = ws_new(g, k);
  uint64_t *cur = (uint64_t *)xmalloc(((size_t)n + 1) * sizeof(uint64_t));
  uint64_t *acc = (uint64_t *)xcalloc((size_t)n + 1, sizeof(uint64_t));
  memcpy(cur, rho, (size_t)n * sizeof(uint64_t));
  for (uint32_t s = 0; s < n; ++s) {
    if (g->cd[s] == g->cd[s + 1]) continue;
    for (uint64_t i = g->cd[s]; i < g->cd[s + 1]; ++i) {
      const uint32_t t = g->adj[i];
      make_subgraph(w, g, s, t);
      const uint32_t ngw = cur[t] < cur[s] ? t : s;
      seq_rec(w, cur, k - 2, ngw);
      acc[s] += cur[s] - rho[s];
      cur[s] = rho[s];
      acc[t] += cur[t] - rho[t];
      cur[t] = rho[t];
      for (uint32_t j = 0; j < w->nn[k - 2]; ++j) {
        const uint32_t x = w->sg2g[j];
        acc[x] += cur[x] - rho[x];
        cur[x] = rho[x];
      }
    }
    rho[s] += acc[s];
    cur[s] = rho[s];
    acc[s] = 0;
    for (uint64_t i = g->cd[s]; i < g->cd[s + 1]; ++i) {
      const uint32_t x = g->adj[i];
      rho[x] += acc[x];
      cur[x] = rho[x];
      acc[x] = 0;
    }
  }
  free(acc);
  free(cur);
  ws_free(w);
}

/* The root edges of roots s < cut in one sequential chain (in place), then
 * the other root edges as independent streams from the result. */
void orc_seq_pass_hybrid(const orc_graph *g, int k, uint64_t *rho, uint32_t cut, int threads) {
  const uint32_t n = g->n;
  orc_ws *w = ws_new(g, k);
  for (uint64_t i = 0; i < g->e; ++i) {
    const uint32_t s = g->edges[i].s, t = g->edges[i].t;
    if (s >= cut) break;  /* root edges are sorted by s */
    const uint32_t ngw = rho[t] < rho[s] ? t : s;
    make_subgraph(w, g, s, t);
    seq_rec(w, rho, k - 2, ngw);
  }
  ws_free(w);
  uint8_t *mask = (uint8_t *)xcalloc((size_t)n + 1, 1);
  for (uint32_t s = cut; s < n; ++s) mask[s] = 1;
  uint64_t *delta = (uint64_t *)xcalloc((size_t)n + 1, sizeof(uint64_t));
  orc_seq_delta_masked(g, k, rho, mask, threads, delta);
  for (uint32_t x = 0; x < n; ++x) rho[x] += delta[x];
  free(delta);
  free(mask);
}

/* Every k-clique in the sequential enumeration order, members in the
 * reference's comparison order (s, t, then deeper), for simulations that
 * replay a pass clique by clique. */
typedef struct {
  uint32_t *buf;
  uint64_t cnt, cap;
  uint32_t pre[ORC_MAXK];
} clique_list_t;

static void list_rec(orc_ws *w, clique_list_t *L, int l, int depth) {
  const int k = w->k;
  if (k == 3) {
    for (uint32_t i = 0; i < w->nn[1]; ++i) {
      if (L->cnt < L->cap) {
        uint32_t *r = L->buf + L->cnt * 3;
        r[0] = L->pre[0];
        r[1] = L->pre[1];
        r[2] = w->sg2g[w->nodes[1][i]];
      }
      L->cnt++;
    }
    return;
  }
  if (l == 2) {
    for (uint32_t i = 0; i < w->nn[2]; ++i) {
      const uint32_t u = w->nodes[2][i];
      const uint32_t *au = w->adj[2] + (size_t)w->core * u;
      for (uint32_t j = 0; j < w->deg[2][u]; ++j) {
        if (L->cnt < L->cap) {
          uint32_t *r = L->buf + L->cnt * (uint64_t)k;
          for (int q = 0; q < depth; ++q) r[q] = L->pre[q];
          r[depth] = w->sg2g[u];
          r[depth + 1] = w->sg2g[au[j]];
        }
        L->cnt++;
      }
    }
    return;
  }
  if (w->nn[l] < (uint32_t)l) return;
  for (uint32_t i = 0; i < w->nn[l]; ++i) {
    const uint32_t u = w->nodes[l][i];
    L->pre[depth] = w->sg2g[u];
    descend(w, l, u);
    list_rec(w, L, l - 1, depth + 1);
    ascend(w, l);
  }
}

/* Returns the number of k-cliques; fills buf (up to cap cliques of k ids)
 * and edge_first[0..e] (the index of every root edge's first clique). */
uint64_t orc_list_cliques(const orc_graph *g, int k, uint32_t *buf, uint64_t cap, uint64_t *edge_first) {
  clique_list_t L;
  memset(&L, 0, sizeof L);
  L.buf = buf;
  L.cap = cap;
  orc_ws *w = ws_new(g, k);
  for (uint64_t i = 0; i < g->e; ++i) {
    if (edge_first) edge_first[i] = L.cnt;
    L.pre[0] = g->edges[i].s;
    L.pre[1] = g->edges[i].t;
    make_subgraph(w, g, g->edges[i].s, g->edges[i].t);
    list_rec(w, &L, k - 2, 2);
  }
  if (edge_first) edge_first[g->e] = L.cnt;
  ws_free(w);
  return L.cnt;
}

/* One pass of P streams sharing one load vector, simulated: stream j walks
 * its root edges (stream_edges[stream_first[j] .. stream_first[j + 1]), each
 * edge's cliques cl[ef[e] .. ef[e + 1]) in order).  The streams advance in
 * steps of `chunk` cliques; inside a step a stream sees the loads as the
 * previous step left them plus its own increments of this step, and gives
 * each clique's unit to its member of smallest load (ties to the earlier
 * member of the row); the step's increments are added at its end.  The
 * result does not depend on the order in which the streams of a step run. */
void orc_sim_shared_pass(int k, const uint32_t *cl, const uint64_t *ef, const uint32_t *stream_edges,
                         const uint64_t *stream_first, uint32_t P, uint32_t chunk, uint64_t *loads, int threads) {
  uint64_t *pos_edge = (uint64_t *)xmalloc((size_t)P * sizeof(uint64_t));  /* index into stream_edges */
  uint64_t *pos_cl = (uint64_t *)xmalloc((size_t)P * sizeof(uint64_t));    /* next clique of that edge */
  uint32_t *inc = (uint32_t *)xmalloc((size_t)P * chunk * sizeof(uint32_t));
  uint32_t *ninc = (uint32_t *)xcalloc(P, sizeof(uint32_t));
  for (uint32_t j = 0; j < P; ++j) {
    pos_edge[j] = stream_first[j];
    pos_cl[j] = pos_edge[j] < stream_first[j + 1] ? ef[stream_edges[pos_edge[j]]] : 0;
  }
  int active = 1;
  while (active) {
    active = 0;
    #pragma omp parallel for num_threads(threads > 0 ? threads : 1) schedule(dynamic, 64) reduction(|:active)
    for (int64_t jj = 0; jj < (int64_t)P; ++jj) {
      const uint32_t j = (uint32_t)jj;
      uint32_t *my = inc + (size_t)j * chunk;
      uint32_t cnt = 0;
      while (cnt < chunk && pos_edge[j] < stream_first[j + 1]) {
        const uint32_t e = stream_edges[pos_edge[j]];
        if (pos_cl[j] >= ef[e + 1]) {  /* next root edge of this stream */
          pos_edge[j]++;
          if (pos_edge[j] < stream_first[j + 1]) pos_cl[j] = ef[stream_edges[pos_edge[j]]];
          continue;
        }
        const uint32_t *row = cl + pos_cl[j] * (uint64_t)k;
        uint32_t best = row[0];
        uint64_t bv = loads[best];
        for (uint32_t q = 0; q < cnt; ++q) bv += my[q] == best;
        for (int a = 1; a < k; ++a) {
          const uint32_t x = row[a];
          uint64_t xv = loads[x];
          for (uint32_t q = 0; q < cnt; ++q) xv += my[q] == x;
          if (xv < bv) {
            best = x;
            bv = xv;
          }
        }
        my[cnt++] = best;
        pos_cl[j]++;
      }
      ninc[j] = cnt;
      if (cnt) active = 1;
    }
    for (uint32_t j = 0; j < P; ++j) {
      const uint32_t *my = inc + (size_t)j * chunk;
      for (uint32_t q = 0; q < ninc[j]; ++q) loads[my[q]]++;
      ninc[j] = 0;
    }
  }
  free(pos_edge);
  free(pos_cl);
  free(inc);
  free(ninc);
}
