// kclpp_internal.h -- host-side types shared by the library's translation units.
#pragma once

#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "../../include/kclpp.h"

typedef struct CUstream_st *cudaStream_t;

struct kclpp_edge_list {
  uint32_t n = 0;               // max id + 1 (ReadEdgeList semantics)
  std::vector<uint32_t> pairs;  // s0 t0 s1 t1 ...
  uint64_t e() const { return pairs.size() / 2; }
};

namespace kclpp {

kclpp_status set_error(kclpp_status s, const char *fmt, ...);
void clear_error();

// Deterministic 64-bit generator (splitmix64); identical sequences on x86 and Arm.
struct SplitMix {
  uint64_t x;
  explicit SplitMix(uint64_t seed) : x(seed) {}
  inline uint64_t next() {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  inline double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  inline uint64_t below(uint64_t m) { return m ? next() % m : 0; }
};

// Stable LSD radix sort of 64-bit keys (16-bit digits, only the digits that vary).
void radix_sort_u64(std::vector<uint64_t> &keys);

// Indexed binary min-heap with the operation order of the reference's heaps
// (BinaryHeap.c:6-90 and the u64 heap of kClistCoreTrim.c:445-526): the same
// swaps in the same sequence, so ties pop in the reference's order.  The tie
// order defines the degeneracy order (hence the DAG and every Seq r) and the
// k-clique core peel's order, which is why it has to be the same algorithm.
struct PeelHeap {
  std::vector<uint32_t> pos;  // key -> position (UINT32_MAX once popped)
  std::vector<uint32_t> key;  // position -> key
  std::vector<uint64_t> val;  // position -> value
  uint32_t n = 0;
  explicit PeelHeap(uint32_t nmax) : pos(nmax, UINT32_MAX), key(nmax), val(nmax) {}
  inline void swap_at(uint32_t i, uint32_t j) {
    std::swap(pos[key[i]], pos[key[j]]);
    std::swap(key[i], key[j]);
    std::swap(val[i], val[j]);
  }
  inline void up(uint32_t i) {
    while (i > 0) {
      const uint32_t j = (i - 1) >> 1;
      if (val[j] > val[i]) { swap_at(i, j); i = j; }
      else break;
    }
  }
  inline void down() {
    uint32_t i = 0;
    for (;;) {
      const uint32_t j1 = 2 * i + 1, j2 = j1 + 1;
      if (j1 >= n) break;
      const uint32_t j = (j2 < n && val[j2] < val[j1]) ? j2 : j1;
      if (val[j] < val[i]) { swap_at(i, j); i = j; }
      else break;
    }
  }
  inline void push(uint32_t k, uint64_t v) {
    pos[k] = n;
    key[n] = k;
    val[n] = v;
    ++n;
    up(n - 1);
  }
  inline void dec(uint32_t k, uint64_t d) {
    const uint32_t i = pos[k];
    if (i != UINT32_MAX) { val[i] -= d; up(i); }
  }
  inline uint32_t pop(uint64_t *v) {
    const uint32_t k = key[0];
    if (v) *v = val[0];
    pos[k] = UINT32_MAX;
    --n;
    key[0] = key[n];
    val[0] = val[n];
    pos[key[0]] = 0;  // as the reference: re-points the last key even when n hits 0
    down();
    return k;
  }
  inline bool live(uint32_t k) const { return pos[k] != UINT32_MAX; }
};

// Host DAG in CSR form.
struct HostDag {
  uint32_t n = 0;
  uint32_t core = 0;              // max out-degree
  std::vector<uint64_t> off;      // n + 1
  std::vector<uint32_t> cols;     // m, ascending per row, cols < row
  uint64_t m() const { return cols.size(); }
};

// Context accessors for translation units other than the one defining kclpp_ctx.
cudaStream_t ctx_stream(kclpp_ctx *c);
int ctx_device(kclpp_ctx *c);
int ctx_sms(kclpp_ctx *c);
void ctx_count_launch(kclpp_ctx *c, int n);
uint32_t *ctx_err_word(kclpp_ctx *c);
// Reads (and clears) the device status word after synchronising the stream.
kclpp_status ctx_check_err(kclpp_ctx *c);
// Graph accessors for the same: the host DAG and its device copy.
const HostDag &graph_dag(const kclpp_graph *g);
const uint64_t *graph_dev_offsets(const kclpp_graph *g);
const uint32_t *graph_dev_cols(const kclpp_graph *g);
int graph_device(const kclpp_graph *g);

// Recounts of the k-clique core peel on the GPU (kclpp_peel.cu): for a batch
// of roots with explicit member lists (live neighbours, ascending), the
// k-cliques through each root and member, for the roots flagged in gpu[].
struct PeelRecount;
kclpp_status peel_recount_create(kclpp_ctx *c, const kclpp_graph *g, int k, PeelRecount **out);
kclpp_status peel_recount_run(PeelRecount *P, uint32_t nroots, const uint64_t *loff, const uint32_t *lcols,
                              const uint8_t *gpu, uint64_t *w);
void peel_recount_free(PeelRecount *P);

// SortByCore with the reference heap's tie order.
void core_order_host(uint32_t n, const std::vector<uint32_t> &pairs, uint32_t *rank);
// The same peel: vertices in pop order and the degree each had when popped
// (degree_at_pop may be null).
void core_peel_host(uint32_t n, const std::vector<uint32_t> &pairs, uint32_t *order, uint64_t *degree_at_pop);
// The same peel by bin sort, O(n + m), with its own tie order (KCLPP_ORDER_FAST).
void core_order_fast_host(uint32_t n, const std::vector<uint32_t> &pairs, uint32_t *rank);
// Relabel + sort + CSR; fails on self loops or repeated edges.
kclpp_status make_dag_host(const std::vector<uint32_t> &pairs, const uint32_t *rank, HostDag &dag);

}  // namespace kclpp
