// kclpp_order.cpp -- degeneracy order and DAG construction on the host (A2-A4).
//
// SortByCore (Graph.c:57-91) is a sequential min-degree peel whose tie order
// comes from the binary heap of BinaryHeap.c:6-90; the DAG orientation, and
// with it every clique's enumeration order and every Seq-kClist++ r value,
// depends on that order.  PeelHeap (kclpp_internal.h) performs the same swaps
// in the same sequence (an implementation of the same algorithm, not a copy),
// so the rank permutation is identical to the reference's.
#include <algorithm>
#include <cstring>

#include "kclpp_internal.h"

namespace kclpp {

// Undirected CSR of an edge list (both directions of every pair).
static void undirected_csr(uint32_t n, const std::vector<uint32_t> &pairs, std::vector<uint64_t> &cd,
                           std::vector<uint32_t> &adj) {
  const uint64_t e = pairs.size() / 2;
  cd.assign((size_t)n + 1, 0);
  for (uint64_t i = 0; i < e; ++i) { cd[pairs[2 * i] + 1]++; cd[pairs[2 * i + 1] + 1]++; }
  for (uint32_t i = 1; i <= n; ++i) cd[i] += cd[i - 1];
  adj.resize(2 * e);
  std::vector<uint64_t> fill(cd.begin(), cd.end() - 1);
  for (uint64_t i = 0; i < e; ++i) {
    uint32_t s = pairs[2 * i], t = pairs[2 * i + 1];
    adj[fill[s]++] = t;
    adj[fill[t]++] = s;
  }
}

void core_peel_host(uint32_t n, const std::vector<uint32_t> &pairs, uint32_t *order, uint64_t *degree_at_pop) {
  std::vector<uint64_t> cd;
  std::vector<uint32_t> adj;
  undirected_csr(n, pairs, cd, adj);
  PeelHeap h(n);
  for (uint32_t i = 0; i < n; ++i) h.push(i, cd[i + 1] - cd[i]);
  for (uint32_t i = 0; i < n; ++i) {
    uint64_t v = 0;
    const uint32_t k = h.pop(&v);
    order[i] = k;
    if (degree_at_pop) degree_at_pop[i] = v;
    for (uint64_t j = cd[k]; j < cd[k + 1]; ++j) h.dec(adj[j], 1);
  }
}

void core_order_host(uint32_t n, const std::vector<uint32_t> &pairs, uint32_t *rank) {
  std::vector<uint32_t> order(n);
  core_peel_host(n, pairs, order.data(), nullptr);
  for (uint32_t i = 0; i < n; ++i) rank[order[i]] = n - 1 - i;  // rank = n - (pops so far)
}

// KCLPP_ORDER_FAST: the bin-sort peel of Batagelj and Zaversnik ("An O(m)
// algorithm for cores decomposition of networks", 2003).  Vertices sit in an
// array sorted by their current degree, with the start of every degree's
// run; taking them in array order and moving each still-unpeeled neighbour of
// higher degree one run down is the min-degree peel in O(n + m).  Its ties
// fall differently from the binary heap's, so the permutation (and with it
// the DAG orientation and Seq-kClist++'s r) differs from SortByCore's; the
// core numbers, the degeneracy -- the DAG's largest out-degree -- and every
// clique count are the same.
void core_order_fast_host(uint32_t n, const std::vector<uint32_t> &pairs, uint32_t *rank) {
  std::vector<uint64_t> cd;
  std::vector<uint32_t> adj;
  undirected_csr(n, pairs, cd, adj);
  std::vector<uint32_t> deg(n), pos(n), vert(n);
  uint32_t md = 0;
  for (uint32_t v = 0; v < n; ++v) {
    deg[v] = (uint32_t)(cd[v + 1] - cd[v]);
    md = std::max(md, deg[v]);
  }
  std::vector<uint32_t> bin((size_t)md + 2, 0);  // bin[d]: start of the run of degree d
  for (uint32_t v = 0; v < n; ++v) bin[deg[v]]++;
  uint32_t start = 0;
  for (uint32_t d = 0; d <= md; ++d) {
    const uint32_t num = bin[d];
    bin[d] = start;
    start += num;
  }
  for (uint32_t v = 0; v < n; ++v) {
    pos[v] = bin[deg[v]]++;
    vert[pos[v]] = v;
  }
  for (uint32_t d = md; d > 0; --d) bin[d] = bin[d - 1];
  bin[0] = 0;
  for (uint32_t i = 0; i < n; ++i) {
    const uint32_t v = vert[i];
    for (uint64_t j = cd[v]; j < cd[v + 1]; ++j) {
      const uint32_t u = adj[j];
      if (deg[u] > deg[v]) {
        const uint32_t du = deg[u], pu = pos[u], pw = bin[du], w = vert[pw];
        if (u != w) {
          pos[u] = pw;
          vert[pu] = w;
          pos[w] = pu;
          vert[pw] = u;
        }
        bin[du]++;
        deg[u]--;
      }
    }
    rank[v] = n - 1 - i;
  }
}

kclpp_status make_dag_host(const std::vector<uint32_t> &pairs, const uint32_t *rank, HostDag &dag) {
  const uint64_t e = pairs.size() / 2;
  std::vector<uint64_t> keys(e);
  uint32_t n = 0;
  for (uint64_t i = 0; i < e; ++i) {
    uint32_t s = rank[pairs[2 * i]], t = rank[pairs[2 * i + 1]];
    if (s < t) std::swap(s, t);
    if (s == t) return set_error(KCLPP_ERR_INVALID, "edge %llu is a self loop (vertex %u); the graph must be simple",
                                 (unsigned long long)i, pairs[2 * i]);
    if (s + 1 > n) n = s + 1;
    keys[i] = ((uint64_t)s << 32) | t;
  }
  radix_sort_u64(keys);  // MakeGraph's qsort by (s, t), Graph.c:125
  for (uint64_t i = 1; i < e; ++i)
    if (keys[i] == keys[i - 1])
      return set_error(KCLPP_ERR_INVALID, "repeated edge in input; the graph must be simple");
  dag.n = n;
  dag.off.assign((size_t)n + 1, 0);
  dag.cols.resize(e);
  for (uint64_t i = 0; i < e; ++i) {
    dag.off[(keys[i] >> 32) + 1]++;
    dag.cols[i] = (uint32_t)keys[i];
  }
  uint32_t mx = 0;
  for (uint32_t i = 1; i <= n; ++i) {
    mx = std::max<uint32_t>(mx, (uint32_t)dag.off[i]);
    dag.off[i] += dag.off[i - 1];
  }
  dag.core = mx;
  return KCLPP_OK;
}

}  // namespace kclpp
