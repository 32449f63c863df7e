// kclpp_trim.cpp -- the k-clique core trim (kClistCoreTrim.c), A15-A18.
//
// Pipeline (main, kClistCoreTrim.c:707-775):
//   kcore        degree peel with the reference heap's tie order; vertices whose
//                running core value is below k-1 are dropped (:242-272)
//   relabel      survivors renumbered by peel rank, edges oriented high -> low
//                rank, input order kept (:274-294)
//   DAG          sorted out-CSR of the survivors (mkspecial, :306-331)
//   nck          k-clique degree of every survivor: the GPU count kernel on
//                that DAG (onepass, :394-416)
//   peel         EXACT: the reference's k-clique-degree heap peel with a local
//                recount around every popped vertex (kcliquecore/oneshortpass,
//                :577-666): the heap's pops are sequential by definition and
//                stay on the host, the recounts run on the GPU in speculative
//                batches of predicted pops (a pop commits only when it is the
//                predicted one, so the result is the reference's bit for bit);
//                EXACT_HOST: the same peel with every recount on the host, one
//                pop at a time (the check of EXACT);
//                FAST: GPU rounds that drop every vertex whose k-clique degree
//                is below the best density seen and recount, ending at the
//                rho-core for that density
//   output       trimmed edges in original ids and input order (:686-699)
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "kclpp_internal.h"

using namespace kclpp;

struct kclpp_trim_result {
  kclpp_trim_info info;
  std::vector<uint32_t> map;
  std::vector<uint64_t> nck;
  std::vector<uint32_t> order;
  std::vector<uint64_t> core_num;
  std::vector<uint32_t> trimmed;  // pairs, original ids
  kclpp_peel_stats peel{};
};

namespace {

inline uint32_t isect(const uint32_t *a, uint32_t na, const uint32_t *b, uint32_t nb, uint32_t *out) {
  uint32_t i = 0, j = 0, s = 0;
  while (i < na && j < nb) {
    if (a[i] < b[j]) ++i;
    else if (b[j] < a[i]) ++j;
    else { out[s++] = a[i]; ++i; ++j; }
  }
  return s;
}

// Clique recursion of kClistCoreTrim.c:368-391 over the sorted DAG.
struct Rec {
  uint32_t kmax, core;
  const uint64_t *cd;
  const uint32_t *adj;
  std::vector<uint32_t> merge, size, ck;
  uint64_t *nck;
  void run(uint32_t k) {
    const size_t t = (size_t)(k - 3) * core, t2 = t + core;
    if (size[k - 3] < kmax - k) return;
    if (k == kmax) {
      for (uint32_t i = 0; i < kmax - 1; ++i) nck[ck[i]] += size[k - 3];
      for (uint32_t i = 0; i < size[k - 3]; ++i) nck[merge[t + i]]++;
      return;
    }
    for (uint32_t i = 0; i < size[k - 3]; ++i) {
      const uint32_t x = merge[t + i];
      ck[k - 1] = x;
      size[k - 2] = isect(adj + cd[x], (uint32_t)(cd[x + 1] - cd[x]), &merge[t], size[k - 3], &merge[t2]);
      run(k + 1);
    }
  }
};

// The bookkeeping of kcliquecore (kClistCoreTrim.c:605-666) for one pop: the
// running core number, the peel order, the edge count, the heap decrements in
// the order of the popped vertex's adjacency (updateLLU per live neighbour)
// and the best suffix density.
struct PeelBook {
  uint32_t n2;
  uint64_t kmax;
  kclpp_trim_info &I;
  kclpp_trim_result &R;
  uint64_t c = 0, ncktot;
  uint32_t ecount;  // `unsigned e` in the reference
  uint32_t i = 0;   // pops committed
  std::vector<uint64_t> whendel;
  PeelBook(uint32_t n2_, int k, kclpp_trim_info &I_, kclpp_trim_result &R_, uint64_t tot, uint64_t e2)
      : n2(n2_), kmax((uint64_t)k), I(I_), R(R_), ncktot(tot), ecount((uint32_t)e2), whendel((size_t)n2_ + 1, 0) {
    I.ncktrim = tot;
    I.ckrho = (double)ncktot / (double)n2;
    I.size = n2;
    I.rho = (double)(2 * ecount) / (double)(n2 * (n2 - 1));
  }
  // u popped with degree v; A = its live neighbours (ascending), W = the
  // k-cliques through u and each of them among the live vertices.
  void commit(PeelHeap &h, uint32_t u, uint64_t v, const uint32_t *A, uint32_t na, const uint64_t *W) {
    if (v > c) c = v;
    R.order[i] = u;
    R.core_num[i] = c;
    uint64_t ncktot2 = 0;
    for (uint32_t q = 0; q < na; ++q) {
      ecount--;
      h.dec(A[q], W[q]);
      ncktot2 += W[q];
    }
    const uint32_t size_tmp = n2 - i - 1;
    whendel[size_tmp] = ncktot2 / (kmax - 1);  // every clique is seen by k - 1 neighbours
    ncktot -= whendel[size_tmp];
    const double ckrho_tmp = (double)ncktot / (double)size_tmp;
    if (ckrho_tmp > I.ckrho) {
      I.ckrho = ckrho_tmp;
      I.size = size_tmp;
      I.rho = (double)(2 * ecount) / (double)(size_tmp * (size_tmp - 1));
    }
    ++i;
  }
  // The last vertex, the trimmed set (the vertices alive before the first
  // deletion of degree >= ckrho) and its clique count.
  void finish(PeelHeap &h, std::vector<char> &alive) {
    I.ntrim = n2;  // the reference leaves ntrim unset when n2 == 1
    for (uint32_t j = n2 - 1; j >= 1; --j) {
      if ((double)whendel[j] >= I.ckrho) { I.ntrim = j + 1; break; }
      I.ncktrim -= whendel[j];
    }
    uint64_t v;
    R.order[i] = h.pop(&v);
    R.core_num[i] = c;
    I.ckcore = c;
    for (uint32_t q = n2 - 1; q != n2 - I.ntrim - 1; --q) alive[R.order[q]] = 1;
  }
};

// oneshortpass on the host (kClistCoreTrim.c:577-603): the k-cliques through
// u and each live neighbour A[q], from the DAG recursion; nck2 is an all-zero
// scratch vector of n2 entries and is left all zero.
void recount_host(Rec &rec, uint32_t u, const uint32_t *A, uint32_t na, uint64_t *nck2, uint64_t *W) {
  for (uint32_t q = 0; q < na; ++q) W[q] = 0;
  if (na <= rec.kmax - 2) return;
  rec.nck = nck2;
  rec.ck[0] = u;
  for (uint32_t q = 0; q < na; ++q) {
    const uint32_t w = A[q];
    rec.ck[1] = w;
    rec.size[0] = isect(A, na, rec.adj + rec.cd[w], (uint32_t)(rec.cd[w + 1] - rec.cd[w]), rec.merge.data());
    rec.run(3);
  }
  for (uint32_t q = 0; q < na; ++q) {
    W[q] = nck2[A[q]];
    nck2[A[q]] = 0;
  }
  nck2[u] = 0;
}

// A read-only view of a PeelHeap that can pop without changing it (the pops
// land in a stamped overlay): the next pops the heap would make if no degree
// changed, i.e. the prediction of a speculative batch.
struct HeapPeek {
  const PeelHeap &h;
  std::vector<uint32_t> st, ok;
  std::vector<uint64_t> ov;
  uint32_t gen = 0, n = 0;
  explicit HeapPeek(const PeelHeap &h_) : h(h_), st(h_.key.size(), 0), ok(h_.key.size()), ov(h_.key.size()) {}
  void reset() {
    if (++gen == 0) {
      std::fill(st.begin(), st.end(), 0);
      gen = 1;
    }
    n = h.n;
  }
  uint32_t K(uint32_t i) const { return st[i] == gen ? ok[i] : h.key[i]; }
  uint64_t V(uint32_t i) const { return st[i] == gen ? ov[i] : h.val[i]; }
  void set(uint32_t i, uint32_t k, uint64_t v) { st[i] = gen; ok[i] = k; ov[i] = v; }
  // PeelHeap::pop's sequence of moves, positions only.
  uint32_t pop() {
    const uint32_t k0 = K(0);
    --n;
    set(0, K(n), V(n));
    uint32_t i = 0;
    for (;;) {
      const uint32_t j1 = 2 * i + 1, j2 = j1 + 1;
      if (j1 >= n) break;
      const uint32_t j = (j2 < n && V(j2) < V(j1)) ? j2 : j1;
      if (V(j) < V(i)) {
        const uint32_t ki = K(i), kj = K(j);
        const uint64_t vi = V(i), vj = V(j);
        set(i, kj, vj);
        set(j, ki, vi);
        i = j;
      } else {
        break;
      }
    }
    return k0;
  }
};

}  // namespace

extern "C" {

// k = 2 (NormalGraphCoreTrim.c, TrimByCoreDecomp :41-110): the degree peel of
// SortByCore; the best edge density along it is max_rho, and vertices are
// dropped in peel order while the degree they had when peeled is below it.
// Host only: the 2-cliques are the edges.
static kclpp_status trim_k2(const kclpp_edge_list *el, kclpp_trim_result **out) {
  std::unique_ptr<kclpp_trim_result> R(new kclpp_trim_result());
  kclpp_trim_info &I = R->info;
  memset(&I, 0, sizeof I);
  const uint32_t n = el->n;
  const uint64_t e = el->e();
  const std::vector<uint32_t> &P = el->pairs;
  I.n = I.n2 = n;
  I.e = I.e2 = e;
  I.total = e;
  std::vector<uint32_t> order(n);
  std::vector<uint64_t> at_pop(n);
  core_peel_host(n, P, order.data(), at_pop.data());
  double max_rho = -1;
  uint64_t cnt = e, core = 0;
  R->core_num.resize(n);
  for (uint32_t i = 0; i < n; ++i) {
    if (max_rho < (double)cnt / (double)(n - i)) {
      max_rho = (double)cnt / (double)(n - i);
      I.size = n - i;
    }
    cnt -= at_pop[i];
    core = std::max(core, at_pop[i]);
    R->core_num[i] = core;
  }
  I.core = (uint32_t)core;
  I.ckcore = core;
  I.ckrho = I.rho = max_rho;
  std::vector<char> alive(n, 1);
  cnt = e;
  for (uint32_t i = 0; i < n; ++i) {
    if ((double)at_pop[i] < max_rho) {
      alive[order[i]] = 0;
      cnt -= at_pop[i];
    } else {
      I.ntrim = n - i;
      I.mtrim = I.ncktrim = cnt;
      break;
    }
  }
  R->map.resize(n);
  R->nck.assign(n, 0);
  for (uint32_t v = 0; v < n; ++v) R->map[v] = v;
  for (uint64_t i = 0; i < e; ++i) { R->nck[P[2 * i]]++; R->nck[P[2 * i + 1]]++; }
  R->order = order;
  for (uint64_t i = 0; i < e; ++i)
    if (alive[P[2 * i]] && alive[P[2 * i + 1]]) {
      R->trimmed.push_back(P[2 * i]);
      R->trimmed.push_back(P[2 * i + 1]);
    }
  *out = R.release();
  return KCLPP_OK;
}

kclpp_status kclpp_trim(kclpp_ctx *ctx, const kclpp_edge_list *el, int kmax, int mode, kclpp_trim_result **out) {
  if (!el || !out) return set_error(KCLPP_ERR_INVALID, "kclpp_trim: null argument");
  *out = nullptr;
  if (mode != KCLPP_TRIM_EXACT && mode != KCLPP_TRIM_FAST && mode != KCLPP_TRIM_EXACT_HOST)
    return set_error(KCLPP_ERR_INVALID, "unknown trim mode");
  if (kmax == 2) return trim_k2(el, out);
  if (!ctx) return set_error(KCLPP_ERR_INVALID, "kclpp_trim: null context (needed for k >= 3)");
  if (kmax < 3 || kmax > KCLPP_MAX_K)
    return set_error(KCLPP_ERR_UNSUPPORTED, "k = %d outside [2, %d]", kmax, KCLPP_MAX_K);
  std::unique_ptr<kclpp_trim_result> R(new kclpp_trim_result());
  kclpp_trim_info &I = R->info;
  memset(&I, 0, sizeof I);
  const uint32_t n = el->n;
  const uint64_t e = el->e();
  const std::vector<uint32_t> &P = el->pairs;
  I.n = n;
  I.e = e;
  // mkgraph (:198-220)
  std::vector<uint64_t> cd0((size_t)n + 1, 0);
  for (uint64_t i = 0; i < e; ++i) { cd0[P[2 * i] + 1]++; cd0[P[2 * i + 1] + 1]++; }
  for (uint32_t i = 1; i <= n; ++i) cd0[i] += cd0[i - 1];
  std::vector<uint32_t> adj0(2 * e);
  {
    std::vector<uint64_t> f(cd0.begin(), cd0.end() - 1);
    for (uint64_t i = 0; i < e; ++i) {
      adj0[f[P[2 * i]]++] = P[2 * i + 1];
      adj0[f[P[2 * i + 1]]++] = P[2 * i];
    }
  }
  // kcore (:242-272)
  std::vector<uint32_t> rank(n), map(n);
  uint32_t n2 = n;
  {
    PeelHeap h(n);
    for (uint32_t i = 0; i < n; ++i) h.push(i, cd0[i + 1] - cd0[i]);
    uint32_t r = 0, c = 0;
    const uint32_t kk = (uint32_t)kmax - 1;
    for (uint32_t i = 0; i < n; ++i) {
      uint64_t v;
      uint32_t key = h.pop(&v);
      if (v > c) c = (uint32_t)v;
      if (c < kk) { rank[key] = UINT32_MAX; n2--; }
      else { map[n2 - (++r)] = key; rank[key] = n2 - r; }
      for (uint64_t j = cd0[key]; j < cd0[key + 1]; ++j) h.dec(adj0[j], 1);
    }
    I.core = c;
  }
  I.n2 = n2;
  map.resize(n2);
  R->map = map;
  std::vector<uint32_t>().swap(adj0);
  // relabelnodes (:274-294)
  std::vector<uint32_t> E;
  E.reserve(2 * e);
  for (uint64_t i = 0; i < e; ++i) {
    uint32_t s = rank[P[2 * i]], t = rank[P[2 * i + 1]];
    if (s == UINT32_MAX || t == UINT32_MAX) continue;
    if (s < t) std::swap(s, t);
    if (s == t) return set_error(KCLPP_ERR_INVALID, "self loop in input; the graph must be simple");
    E.push_back(s);
    E.push_back(t);
  }
  const uint64_t e2 = E.size() / 2;
  I.e2 = e2;
  R->nck.assign(n2, 0);
  R->order.assign(n2, 0);
  R->core_num.assign(n2, 0);
  if (n2 == 0) {
    *out = R.release();
    return KCLPP_OK;
  }
  // mkspecial (:306-331)
  std::vector<uint64_t> cd((size_t)n2 + 1, 0);
  std::vector<uint32_t> adj(e2);
  {
    for (uint64_t i = 0; i < e2; ++i) cd[E[2 * i] + 1]++;
    for (uint32_t i = 1; i <= n2; ++i) cd[i] += cd[i - 1];
    std::vector<uint64_t> f(cd.begin(), cd.end() - 1);
    for (uint64_t i = 0; i < e2; ++i) adj[f[E[2 * i]]++] = E[2 * i + 1];
    for (uint32_t i = 0; i < n2; ++i) std::sort(adj.begin() + cd[i], adj.begin() + cd[i + 1]);
  }
  // onepass on the GPU (:394-416)
  uint64_t tot = 0;
  {
    kclpp_graph *g = nullptr;
    kclpp_status s = kclpp_graph_from_csr(ctx, n2, e2, cd.data(), adj.data(), &g);
    if (s != KCLPP_OK) return s;
    s = kclpp_count_cliques(ctx, g, kmax, R->nck.data(), &tot);
    kclpp_graph_free(g);
    if (s != KCLPP_OK) return s;
  }
  I.total = tot;
  // mkgraph2 (:547-573)
  std::vector<uint64_t> cu((size_t)n2 + 1, 0);
  std::vector<uint32_t> au(2 * e2);
  {
    for (uint64_t i = 0; i < e2; ++i) { cu[E[2 * i] + 1]++; cu[E[2 * i + 1] + 1]++; }
    for (uint32_t i = 1; i <= n2; ++i) cu[i] += cu[i - 1];
    std::vector<uint64_t> f(cu.begin(), cu.end() - 1);
    for (uint64_t i = 0; i < e2; ++i) {
      au[f[E[2 * i]]++] = E[2 * i + 1];
      au[f[E[2 * i + 1]]++] = E[2 * i];
    }
    for (uint32_t i = 0; i < n2; ++i) std::sort(au.begin() + cu[i], au.begin() + cu[i + 1]);
  }
  std::vector<char> alive(n2, 0);
  if (mode == KCLPP_TRIM_EXACT || mode == KCLPP_TRIM_EXACT_HOST) {
    // kcliquecore (:605-666): the reference's heap and its pops, one at a
    // time.  EXACT_HOST recounts each popped vertex on the host as the
    // reference does.  EXACT predicts the heap's next B pops (what it would
    // pop if no degree changed), recounts all of them at once on the GPU with
    // each one's live set as it would be at its pop, then commits pops while
    // the heap's actual minimum is the predicted vertex: a committed pop's
    // live set is then exactly the predicted one, so its counts are exact.
    // The first pop that differs ends the batch; its count is recomputed in
    // the next one.  B doubles while whole batches commit and shrinks to
    // what the last batch committed otherwise.
    const auto t_peel = std::chrono::steady_clock::now();
    PeelHeap h(n2);
    for (uint32_t i = 0; i < n2; ++i) h.push(i, R->nck[i]);
    PeelBook bk(n2, kmax, I, *R, tot, e2);
    Rec rec;
    rec.kmax = (uint32_t)kmax;
    rec.core = std::max<uint32_t>(I.core, 1);
    rec.cd = cd.data();
    rec.adj = adj.data();
    rec.merge.assign((size_t)(kmax - 2) * rec.core + 1, 0);
    rec.size.assign(kmax, 0);
    rec.ck.assign(kmax, 0);
    std::vector<uint64_t> nck2((size_t)n2 + 1, 0);
    kclpp_peel_stats &PS = R->peel;
    if (mode == KCLPP_TRIM_EXACT_HOST) {
      std::vector<uint32_t> live((size_t)n2 + 1);
      std::vector<uint64_t> W((size_t)n2 + 1);
      while (bk.i + 1 < n2) {
        uint64_t v;
        const uint32_t u = h.pop(&v);
        uint32_t na = 0;
        for (uint64_t j = cu[u]; j < cu[u + 1]; ++j)
          if (h.live(au[j])) live[na++] = au[j];
        recount_host(rec, u, live.data(), na, nck2.data(), W.data());
        bk.commit(h, u, v, live.data(), na, W.data());
        PS.host_roots += na > (uint32_t)kmax - 2;
      }
      PS.committed = PS.predicted = n2 ? n2 - 1 : 0;
      PS.batches = PS.committed;
    } else {
      kclpp_graph *gd = nullptr;
      kclpp_status st = kclpp_graph_from_csr(ctx, n2, e2, cd.data(), adj.data(), &gd);
      if (st != KCLPP_OK) return st;
      std::unique_ptr<kclpp_graph, void (*)(kclpp_graph *)> gd_own(gd, kclpp_graph_free);
      PeelRecount *P = nullptr;
      st = peel_recount_create(ctx, gd, kmax, &P);
      if (st != KCLPP_OK) return st;
      std::unique_ptr<PeelRecount, void (*)(PeelRecount *)> P_own(P, peel_recount_free);
      HeapPeek peek(h);
      std::vector<uint32_t> pred, mark((size_t)n2, 0), mpos((size_t)n2, 0), lcols;
      std::vector<uint64_t> loff, W;
      std::vector<uint8_t> gpu;
      uint32_t gen = 0;
      uint32_t B = 64;
      constexpr uint32_t kMaxBatch = 4096;
      while (bk.i + 1 < n2) {
        const uint32_t want = std::min<uint32_t>(B, n2 - 1 - bk.i);
        peek.reset();
        if (++gen == 0) {
          std::fill(mark.begin(), mark.end(), 0);
          gen = 1;
        }
        pred.resize(want);
        for (uint32_t j = 0; j < want; ++j) {
          pred[j] = peek.pop();
          mark[pred[j]] = gen;
          mpos[pred[j]] = j;
        }
        loff.assign((size_t)want + 1, 0);
        lcols.clear();
        gpu.assign(want, 0);
        for (uint32_t j = 0; j < want; ++j) {
          const uint32_t u = pred[j];
          for (uint64_t q = cu[u]; q < cu[u + 1]; ++q) {
            const uint32_t v = au[q];
            if (h.live(v) && !(mark[v] == gen && mpos[v] < j)) lcols.push_back(v);
          }
          loff[j + 1] = lcols.size();
          const uint64_t d = loff[j + 1] - loff[j];
          gpu[j] = d > (uint64_t)kmax - 2 && d <= KCLPP_MAX_OUTDEG;
        }
        W.assign(lcols.size(), 0);
        for (uint32_t j = 0; j < want; ++j) {
          const uint64_t d = loff[j + 1] - loff[j];
          if (d > KCLPP_MAX_OUTDEG) {  // beyond the GPU tiers: the host's recursion
            recount_host(rec, pred[j], lcols.data() + loff[j], (uint32_t)d, nck2.data(), W.data() + loff[j]);
            PS.host_roots++;
          }
        }
        st = peel_recount_run(P, want, loff.data(), lcols.data(), gpu.data(), W.data());
        if (st != KCLPP_OK) return st;
        uint32_t j = 0;
        for (; j < want && h.key[0] == pred[j]; ++j) {
          uint64_t v;
          const uint32_t u = h.pop(&v);
          bk.commit(h, u, v, lcols.data() + loff[j], (uint32_t)(loff[j + 1] - loff[j]), W.data() + loff[j]);
          PS.gpu_roots += gpu[j];
        }
        PS.batches++;
        PS.predicted += want;
        PS.committed += j;
        B = j == want ? std::min(2 * B, kMaxBatch) : std::max<uint32_t>(1, 2 * j);
      }
    }
    bk.finish(h, alive);
    PS.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_peel).count();
  } else {
    // FAST: density-threshold rounds on the GPU.
    std::vector<uint64_t> nck = R->nck;
    std::fill(alive.begin(), alive.end(), 1);
    uint32_t nl = n2;
    uint64_t total = tot, el_live = e2;
    I.ckrho = (double)total / (double)nl;
    I.size = nl;
    I.rho = (double)(2 * (uint32_t)el_live) / (double)(nl * (nl - 1));
    uint32_t removed_at = 0;
    for (int round = 0; round < 100000; ++round) {
      std::vector<uint32_t> drop;
      for (uint32_t v = 0; v < n2; ++v)
        if (alive[v] && (double)nck[v] < I.ckrho) drop.push_back(v);
      if (drop.empty()) break;
      for (uint32_t v : drop) { alive[v] = 0; R->order[removed_at++] = v; }
      nl -= (uint32_t)drop.size();
      // live sub-DAG with the same labels
      std::vector<uint64_t> lcd((size_t)n2 + 1, 0);
      std::vector<uint32_t> ladj;
      ladj.reserve(el_live);
      for (uint32_t s = 0; s < n2; ++s) {
        if (alive[s])
          for (uint64_t j = cd[s]; j < cd[s + 1]; ++j)
            if (alive[adj[j]]) ladj.push_back(adj[j]);
        lcd[s + 1] = ladj.size();
      }
      el_live = ladj.size();
      std::fill(nck.begin(), nck.end(), 0);
      total = 0;
      if (nl) {
        kclpp_graph *g = nullptr;
        kclpp_status s = kclpp_graph_from_csr(ctx, n2, el_live, lcd.data(), ladj.data(), &g);
        if (s != KCLPP_OK) return s;
        s = kclpp_count_cliques(ctx, g, kmax, nck.data(), &total);
        kclpp_graph_free(g);
        if (s != KCLPP_OK) return s;
        const double dens = (double)total / (double)nl;
        if (dens > I.ckrho) {
          I.ckrho = dens;
          I.size = nl;
          I.rho = (double)(2 * (uint32_t)el_live) / (double)(nl * (nl - 1));
        }
      }
    }
    for (uint32_t v = 0; v < n2; ++v)
      if (alive[v]) R->order[removed_at++] = v;
    I.ntrim = nl;
    I.ncktrim = total;
  }
  // printdensest trimmed graph (:686-699): input order, original ids.
  for (uint64_t i = 0; i < e2; ++i) {
    const uint32_t s = E[2 * i], t = E[2 * i + 1];
    if (alive[s] && alive[t]) {
      R->trimmed.push_back(map[s]);
      R->trimmed.push_back(map[t]);
    }
  }
  I.mtrim = R->trimmed.size() / 2;
  *out = R.release();
  return KCLPP_OK;
}

kclpp_status kclpp_trim_info_get(const kclpp_trim_result *t, kclpp_trim_info *info) {
  if (!t || !info) return set_error(KCLPP_ERR_INVALID, "null argument");
  *info = t->info;
  return KCLPP_OK;
}

kclpp_status kclpp_trim_copy(const kclpp_trim_result *t, uint32_t *map, uint64_t *nck, uint32_t *order,
                             uint64_t *core_num) {
  if (!t) return set_error(KCLPP_ERR_INVALID, "null argument");
  const size_t n2 = t->info.n2;
  if (map && n2) memcpy(map, t->map.data(), n2 * 4);
  if (nck && n2) memcpy(nck, t->nck.data(), n2 * 8);
  if (order && n2) memcpy(order, t->order.data(), n2 * 4);
  if (core_num && n2) memcpy(core_num, t->core_num.data(), n2 * 8);
  return KCLPP_OK;
}

kclpp_status kclpp_trim_peel_stats(const kclpp_trim_result *t, kclpp_peel_stats *st) {
  if (!t || !st) return set_error(KCLPP_ERR_INVALID, "null argument");
  *st = t->peel;
  return KCLPP_OK;
}

kclpp_status kclpp_trim_edges(const kclpp_trim_result *t, kclpp_edge_list **out) {
  if (!t || !out) return set_error(KCLPP_ERR_INVALID, "null argument");
  return kclpp_edge_list_create(t->trimmed.data(), t->trimmed.size() / 2, out);
}

void kclpp_trim_free(kclpp_trim_result *t) { delete t; }

}  // extern "C"
