// kclpp_certify.cpp -- certifying the densest prefix exactly, driven by GPU passes.
//
// The reference's exact algorithm (kCDensestMem.c:478-530) takes the first
// block of the isotonic regression (PAVA, :329-364) of the prefix clique
// counts as the candidate S, checks that S is stable (:366-403: every clique
// reassigned to its lowest-ranked members leaves every member of S with more
// load than any vertex outside), then that no subset of S is denser (the
// Goldberg-type integrality test, :405-432), and falls back to a max-flow
// (:434-467).  It keeps every clique and its per-member weights in memory,
// which bounds it to small graphs.
//
// The same two conditions are restated here with per-vertex loads only, so
// that GPU passes produce them and nothing per clique is stored:
//   inside:  loads b_in from Seq passes on G[S] alone -- a feasible assignment
//            of the cliques inside S to their members.  A subset A of S with
//            j vertices and c cliques has c <= (sum of the j largest loads) /
//            T.  Densities are rationals: A is denser than S (m cliques, n
//            vertices) only if c >= floor(m j / n) + 1 = c_min(j).  So if for
//            every j either C(j, k) < c_min(j) or the top-j load sum is below
//            c_min(j) T, no subset of S is denser than S (integer arithmetic,
//            no tolerance).
//            The margin can be as small as 1 / (n j), which the loads reach only
//            after very many passes; where G[S] is small enough, the library's
//            max-flow (kclpp_densest_exact) decides it exactly instead, as the
//            reference falls back to its max-flow (:434-467).
//   outside: loads b_out from Seq passes on G in which the members of S start
//            at a value no clique can bring the others up to, so every clique
//            with a member outside S gives its unit outside S.  Any X = A u Y
//            with A in S and Y outside has cliques(X) <= cliques(A) +
//            sum_{y in Y} b_out(y); with the inside condition, if
//            max_{v not in S} b_out(v) <= m / n, density(X) <= m / n.
// Both together: S has the largest k-clique density of the graph, exactly m/n.
// The passes use shared loads (KCLPP_SEQ_SHARED): every pass gives each clique
// one unit, so the averaged loads are feasible assignments whatever the
// interleaving, and they converge in the fewest passes.
#include <algorithm>
#include <cstring>
#include <functional>
#include <memory>
#include <vector>

#include "kclpp_internal.h"

using namespace kclpp;

#define KCLPP_TRY_H(call)           \
  do {                              \
    const kclpp_status s_ = (call); \
    if (s_ != KCLPP_OK) return s_;  \
  } while (0)

namespace {

typedef unsigned __int128 u128;

// Largest G[S] (in k-cliques) handed to the host max-flow when the loads do
// not settle "inside" (kclpp_densest_exact's own limit is 2e7).
constexpr uint64_t kMaxFlowCliques = 20000000;

// C(j, k), saturated at 2^64.
u128 choose_capped(uint64_t j, int k) {
  if (j < (uint64_t)k) return 0;
  u128 c = 1;
  for (int i = 0; i < k; ++i) {
    c = c * (u128)(j - (uint64_t)i) / (u128)(i + 1);
    if (c > ((u128)1 << 64)) return (u128)1 << 64;
  }
  return c;
}

// CDF_Pava (kCDensestMem.c:335-351): blocks of the isotonic regression of
// the prefix counts with the reference's 0.999999 merge rule; returns the
// first block's size.
uint32_t pava_first_block(const std::vector<uint64_t> &tent) {
  const uint32_t n = (uint32_t)tent.size();
  if (!n) return 0;
  std::vector<uint32_t> nag(n);
  std::vector<double> val(n);
  nag[0] = 1;
  val[0] = (double)tent[0];
  uint32_t j = 0;
  for (uint32_t i = 1; i < n; ++i) {
    j += 1;
    val[j] = (double)tent[i];
    nag[j] = 1;
    while (j > 0 && val[j] >= val[j - 1] * 0.999999) {
      val[j - 1] = (nag[j] * val[j] + nag[j - 1] * val[j - 1]) / (nag[j] + nag[j - 1]);
      nag[j - 1] += nag[j];
      --j;
    }
  }
  return nag[0];
}

struct GraphFree {
  void operator()(kclpp_graph *g) const { kclpp_graph_free(g); }
};
struct ElFree {
  void operator()(kclpp_edge_list *e) const { kclpp_edge_list_free(e); }
};

}  // namespace

extern "C" {

kclpp_status kclpp_certify_densest(kclpp_ctx *ctx, const kclpp_graph *g, int k, const uint64_t *r,
                                   uint32_t max_passes, kclpp_certify_info *info, uint32_t *members) {
  if (!ctx || !g || !info) return set_error(KCLPP_ERR_INVALID, "kclpp_certify_densest: null argument");
  memset(info, 0, sizeof *info);
  if (k < 3 || k > KCLPP_MAX_K)
    return set_error(KCLPP_ERR_UNSUPPORTED, "certify: k = %d outside [3, %d]", k, KCLPP_MAX_K);
  uint32_t n = 0;
  uint64_t m_dag = 0;
  KCLPP_TRY_H(kclpp_graph_info(g, &n, &m_dag, nullptr));
  if (!n) return KCLPP_OK;
  if (!r) return set_error(KCLPP_ERR_INVALID, "kclpp_certify_densest: null r");
  // The candidate: the first PAVA block of the prefix counts in the order of r.
  std::vector<uint32_t> reordered(n), level(n);
  KCLPP_TRY_H(kclpp_sort_by_r_u64(ctx, n, r, reordered.data(), level.data()));
  std::vector<uint64_t> tent(n);
  KCLPP_TRY_H(kclpp_pava(ctx, g, k, level.data(), tent.data()));
  const uint32_t ns = pava_first_block(tent);
  uint64_t m = 0;
  for (uint32_t i = 0; i < ns; ++i) m += tent[i];
  info->n = ns;
  info->cliques = m;
  info->density = ns ? (double)m / (double)ns : 0.0;
  if (members)
    for (uint32_t i = 0; i < ns; ++i) members[i] = reordered[i];
  if (m == 0) return KCLPP_OK;
  // G[S], its vertices numbered by their place in S.
  std::vector<uint64_t> off((size_t)n + 1);
  std::vector<uint32_t> cols(m_dag);
  KCLPP_TRY_H(kclpp_graph_copy_csr(g, off.data(), cols.data()));
  std::vector<uint32_t> pos(n, UINT32_MAX);
  for (uint32_t i = 0; i < ns; ++i) pos[reordered[i]] = i;
  std::vector<uint32_t> pairs;
  for (uint32_t s = 0; s < n; ++s) {
    if (pos[s] == UINT32_MAX) continue;
    for (uint64_t e = off[s]; e < off[s + 1]; ++e)
      if (pos[cols[e]] != UINT32_MAX) {
        pairs.push_back(pos[s]);
        pairs.push_back(pos[cols[e]]);
      }
  }
  kclpp_edge_list *el_raw = nullptr;
  KCLPP_TRY_H(kclpp_edge_list_create(pairs.data(), pairs.size() / 2, &el_raw));
  std::unique_ptr<kclpp_edge_list, ElFree> el(el_raw);
  kclpp_graph *gs_raw = nullptr;
  KCLPP_TRY_H(kclpp_build_graph(ctx, el.get(), &gs_raw));
  std::unique_ptr<kclpp_graph, GraphFree> gs(gs_raw);
  uint32_t ns_graph = 0;
  KCLPP_TRY_H(kclpp_graph_info(gs.get(), &ns_graph, nullptr, nullptr));
  // Only the multiset of the inside loads matters (top-j sums), so G[S] may
  // number its vertices as its own core order does; vertices of S without an
  // edge inside S carry no load.
  std::vector<uint64_t> r_in(ns_graph, 0), r_out(n, 0), sorted(ns);
  const uint64_t kOut = 1ull << 62;  // far above any load a vertex outside S reaches
  for (uint32_t i = 0; i < ns; ++i) r_out[reordered[i]] = kOut;
  bool inside = false, outside = false;
  uint32_t T = 0;
  const uint32_t cap = std::max<uint32_t>(max_passes, 1);
  for (uint32_t target = 1; target <= cap; target = target > cap / 2 ? cap + 1 : 2 * target) {
    const uint32_t add = target - T;
    if (!inside && ns_graph)
      KCLPP_TRY_H(kclpp_seq_passes(ctx, gs.get(), k, add, KCLPP_SEQ_SHARED, r_in.data()));
    if (!outside) KCLPP_TRY_H(kclpp_seq_passes(ctx, g, k, add, KCLPP_SEQ_SHARED, r_out.data()));
    T = target;
    if (!inside) {
      std::fill(sorted.begin(), sorted.end(), 0);
      std::copy(r_in.begin(), r_in.end(), sorted.begin());
      std::sort(sorted.begin(), sorted.end(), std::greater<uint64_t>());
      bool ok = true;
      u128 top = 0;
      for (uint32_t j = 1; j <= ns && ok; ++j) {
        top += sorted[j - 1];
        const u128 cmin = (u128)m * j / ns + 1;
        if (choose_capped(j, k) < cmin) continue;  // too few vertices to be denser
        if (top >= cmin * (u128)T) ok = false;
      }
      if (ok) {
        inside = true;
        info->passes_inside = T;
      }
    }
    if (!outside) {
      uint64_t mx = 0;
      for (uint32_t v = 0; v < n; ++v)
        if (pos[v] == UINT32_MAX) mx = std::max(mx, r_out[v]);
      if ((u128)mx * ns <= (u128)T * m) {
        outside = true;
        info->passes_outside = T;
      }
    }
    if (inside && outside) break;
  }
  if (inside) info->inside_method = 1;
  // The loads decide "inside" only once they are nearly uniform on S (the
  // integrality margin can be 1 / (n j)); like the reference, which falls back
  // to a max-flow when its Goldberg test fails (kCDensestMem.c:434-467), G[S]
  // is then solved exactly where it is small enough: S's own density is the
  // optimum of G[S] exactly when no subset of S is denser.
  if (!inside && m <= kMaxFlowCliques) {
    kclpp_exact_info ex;
    const kclpp_status st = kclpp_densest_exact(el.get(), k, &ex, nullptr);
    if (st != KCLPP_OK && st != KCLPP_ERR_UNSUPPORTED) return st;
    if (st == KCLPP_OK && (u128)ex.num * ns == (u128)ex.den * m) {
      inside = true;
      info->inside_method = 2;
    }
  }
  info->inside = inside;
  info->outside = outside;
  info->certified = inside && outside;
  return KCLPP_OK;
}

}  // extern "C"
