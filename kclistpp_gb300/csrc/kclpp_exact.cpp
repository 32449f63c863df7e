// kclpp_exact.cpp -- the exact k-clique densest subgraph, by max-flow (host).
//
// The reference certifies with Boost's max-flow (MaxFlow.cpp, kCDensestMem.c),
// which is not part of this build.  This is the published construction for
// the k-clique densest subgraph (Goldberg's network, extended to k-cliques by
// Tsourakakis, "The K-clique Densest Subgraph Problem", WWW 2015), solved with
// Dinic's algorithm:
//
//   source -> v     capacity den * deg_k(v)      (deg_k: k-cliques through v)
//   v -> sink       capacity k * num             (alpha = num / den)
//   v -> psi        capacity den                 for every k-clique psi + {v}
//   psi -> u        capacity "infinite"          for every u in psi
//
// with one node psi per (k-1)-clique that extends to a k-clique.  The cut
// around the source alone costs den * k * |C_k|; a vertex set A whose density
// exceeds alpha gives a cheaper cut, so the maximum flow is below
// den * k * |C_k| exactly when some subgraph is denser than alpha, and the
// source side of a minimum cut is then such a set.  Starting from a known
// density and moving alpha to the density of that set until the flow
// saturates the source edges (Dinkelbach's iteration) ends at the optimum.
#include <algorithm>
#include <array>
#include <cstring>
#include <numeric>

#include "kclpp_internal.h"

using namespace kclpp;

namespace {

constexpr int kMaxKExact = 8;
constexpr uint64_t kMaxCliquesExact = 20000000;

// All k-cliques of a DAG (ids ascending inside each clique), by recursion on
// out-list intersections.
void list_cliques(const HostDag &D, int k, std::vector<uint32_t> &out, bool &too_many) {
  std::vector<std::vector<uint32_t>> cand(k);
  std::array<uint32_t, kMaxKExact> cur{};
  uint64_t count = 0;
  auto rec = [&](auto &&self, int level, const std::vector<uint32_t> &C) -> void {
    if (too_many) return;
    if (level == k) {
      std::array<uint32_t, kMaxKExact> c = cur;
      std::sort(c.begin(), c.begin() + k);
      out.insert(out.end(), c.begin(), c.begin() + k);
      if (++count > kMaxCliquesExact) too_many = true;
      return;
    }
    for (uint32_t u : C) {
      cur[level] = u;
      std::vector<uint32_t> &next = cand[level];
      next.clear();
      const uint32_t *a = D.cols.data() + D.off[u], *ae = D.cols.data() + D.off[u + 1];
      for (uint32_t x : C) {  // C ∩ N+(u): both ascending
        while (a < ae && *a < x) ++a;
        if (a < ae && *a == x) next.push_back(x);
      }
      std::vector<uint32_t> keep = next;  // the deeper levels reuse cand[level]
      self(self, level + 1, keep);
    }
  };
  for (uint32_t s = 0; s < D.n && !too_many; ++s) {
    cur[0] = s;
    std::vector<uint32_t> C(D.cols.begin() + (long)D.off[s], D.cols.begin() + (long)D.off[s + 1]);
    rec(rec, 1, C);
  }
}

struct Dinic {
  struct E {
    uint32_t to;
    int64_t cap;
  };
  std::vector<E> e;
  std::vector<std::vector<uint32_t>> g;
  std::vector<int> level;
  std::vector<size_t> it;
  explicit Dinic(size_t n) : g(n), level(n), it(n) {}
  void add(uint32_t a, uint32_t b, int64_t c) {
    g[a].push_back((uint32_t)e.size());
    e.push_back({b, c});
    g[b].push_back((uint32_t)e.size());
    e.push_back({a, 0});
  }
  bool bfs(uint32_t s, uint32_t t) {
    std::fill(level.begin(), level.end(), -1);
    std::vector<uint32_t> q{s};
    level[s] = 0;
    for (size_t h = 0; h < q.size(); ++h)
      for (uint32_t id : g[q[h]])
        if (e[id].cap > 0 && level[e[id].to] < 0) {
          level[e[id].to] = level[q[h]] + 1;
          q.push_back(e[id].to);
        }
    return level[t] >= 0;
  }
  // Iterative blocking-flow search (no recursion: paths can be long).
  int64_t push(uint32_t s, uint32_t t) {
    int64_t total = 0;
    std::vector<uint32_t> path;  // edge ids from s
    std::vector<uint32_t> nodes{s};
    while (true) {
      const uint32_t u = nodes.back();
      if (u == t) {
        int64_t f = INT64_MAX;
        for (uint32_t id : path) f = std::min(f, e[id].cap);
        for (uint32_t id : path) {
          e[id].cap -= f;
          e[id ^ 1].cap += f;
        }
        total += f;
        path.clear();
        nodes.assign(1, s);
        continue;
      }
      bool advanced = false;
      for (size_t &i = it[u]; i < g[u].size(); ++i) {
        const uint32_t id = g[u][i];
        if (e[id].cap > 0 && level[e[id].to] == level[u] + 1) {
          path.push_back(id);
          nodes.push_back(e[id].to);
          advanced = true;
          break;
        }
      }
      if (advanced) continue;
      if (u == s) break;  // no augmenting path left in this level graph
      level[u] = -1;      // dead end
      nodes.pop_back();
      path.pop_back();
      ++it[nodes.back()];
    }
    return total;
  }
  int64_t maxflow(uint32_t s, uint32_t t) {
    int64_t f = 0;
    while (bfs(s, t)) {
      std::fill(it.begin(), it.end(), 0);
      f += push(s, t);
    }
    return f;
  }
  // Nodes reachable from s in the residual graph (the source side of a minimum cut).
  std::vector<char> source_side(uint32_t s) const {
    std::vector<char> seen(g.size(), 0);
    std::vector<uint32_t> q{s};
    seen[s] = 1;
    for (size_t h = 0; h < q.size(); ++h)
      for (uint32_t id : g[q[h]])
        if (e[id].cap > 0 && !seen[e[id].to]) {
          seen[e[id].to] = 1;
          q.push_back(e[id].to);
        }
    return seen;
  }
};

uint64_t gcd64(uint64_t a, uint64_t b) {
  while (b) {
    const uint64_t t = a % b;
    a = b;
    b = t;
  }
  return a;
}

}  // namespace

extern "C" {

kclpp_status kclpp_densest_exact(const kclpp_edge_list *el, int k, kclpp_exact_info *info, uint8_t *members) {
  if (!el || !info) return set_error(KCLPP_ERR_INVALID, "kclpp_densest_exact: null argument");
  if (k < 2 || k > kMaxKExact) return set_error(KCLPP_ERR_UNSUPPORTED, "kclpp_densest_exact: k must be in [2, 8]");
  memset(info, 0, sizeof *info);
  const uint32_t n = el->n;
  std::vector<uint32_t> rank(n);
  core_order_host(n, el->pairs, rank.data());
  HostDag D;
  const kclpp_status st = make_dag_host(el->pairs, rank.data(), D);
  if (st != KCLPP_OK) return st;
  std::vector<uint32_t> cl;
  bool too_many = false;
  list_cliques(D, k, cl, too_many);
  if (too_many)
    return set_error(KCLPP_ERR_UNSUPPORTED, "kclpp_densest_exact: more than %llu k-cliques",
                     (unsigned long long)kMaxCliquesExact);
  const uint64_t nc = cl.size() / (size_t)k;
  info->cliques_total = nc;
  if (nc == 0) return KCLPP_OK;  // no k-clique: density 0
  // (k-1)-cliques psi: every clique minus one member, deduplicated.
  std::vector<uint64_t> order(nc * (uint64_t)k);
  std::iota(order.begin(), order.end(), 0);
  auto psi_less = [&](uint64_t a, uint64_t b) {  // a, b: clique * k + dropped member
    const uint32_t *ca = &cl[(a / k) * k], *cb = &cl[(b / k) * k];
    const int da = (int)(a % k), db = (int)(b % k);
    for (int i = 0, ia = 0, ib = 0; i < k - 1; ++i, ++ia, ++ib) {
      if (ia == da) ++ia;
      if (ib == db) ++ib;
      if (ca[ia] != cb[ib]) return ca[ia] < cb[ib];
    }
    return false;
  };
  std::sort(order.begin(), order.end(), psi_less);
  std::vector<uint32_t> psi_of(order.size());
  uint32_t npsi = 0;
  for (size_t i = 0; i < order.size(); ++i) {
    if (i > 0 && psi_less(order[i - 1], order[i])) ++npsi;
    psi_of[order[i]] = npsi;
  }
  ++npsi;
  std::vector<uint64_t> degk(n, 0);
  for (uint32_t v : cl) ++degk[v];
  // The density of a vertex set (as a fraction) and the start: all vertices
  // on some k-clique.
  auto density_of = [&](const std::vector<char> &in, uint64_t &num, uint64_t &den) {
    num = 0;
    den = 0;
    for (uint32_t v = 0; v < n; ++v) den += in[v] && degk[v] ? 1 : 0;
    for (uint64_t c = 0; c < nc; ++c) {
      bool all = true;
      for (int j = 0; j < k && all; ++j) all = in[cl[c * k + j]] != 0;
      num += all;
    }
  };
  std::vector<char> best(n, 0);
  for (uint32_t v = 0; v < n; ++v) best[v] = degk[v] > 0;
  uint64_t num = 0, den = 1;
  density_of(best, num, den);
  const uint32_t S = n + npsi, T = S + 1;
  for (int iter = 0; iter < 64; ++iter) {
    info->iterations = iter + 1;
    const uint64_t g = gcd64(num, den);
    const uint64_t a = num / g, b = den / g;
    Dinic F(T + 1);
    const int64_t inf = INT64_MAX / 4;
    for (uint32_t v = 0; v < n; ++v) {
      if (!degk[v]) continue;
      F.add(S, v, (int64_t)(b * degk[v]));
      F.add(v, T, (int64_t)((uint64_t)k * a));
    }
    // psi -> its members (once per psi), v -> psi (once per clique and member)
    std::vector<char> psi_done(npsi, 0);
    for (uint64_t r = 0; r < nc * (uint64_t)k; ++r) {
      const uint64_t c = r / k;
      const int drop = (int)(r % k);
      const uint32_t p = n + psi_of[r];
      F.add(cl[c * k + drop], p, (int64_t)b);
      if (!psi_done[psi_of[r]]) {
        psi_done[psi_of[r]] = 1;
        for (int j = 0; j < k; ++j)
          if (j != drop) F.add(p, cl[c * k + j], inf);
      }
    }
    const int64_t flow = F.maxflow(S, T);
    const int64_t full = (int64_t)(b * (uint64_t)k * nc);
    if (flow >= full) break;  // no subgraph denser than a / b
    std::vector<char> side = F.source_side(S);
    std::vector<char> in(n, 0);
    for (uint32_t v = 0; v < n; ++v) in[v] = side[v];
    uint64_t nn = 0, dd = 0;
    density_of(in, nn, dd);
    if (dd == 0 || nn * den <= num * dd) break;  // cannot happen for an exact flow
    num = nn;
    den = dd;
    best = in;
  }
  // num / den is the best set's clique count over its size, unreduced.
  info->cliques = num;
  info->size = (uint32_t)den;
  const uint64_t g = gcd64(num, den);
  info->num = num / g;
  info->den = den / g;
  info->density = (double)num / (double)den;
  if (members)
    for (uint32_t v = 0; v < n; ++v) members[v] = best[rank[v]] && degk[rank[v]] ? 1 : 0;
  return KCLPP_OK;
}

}  // extern "C"
