// kclpp_internal.h -- host-side types shared by the library's translation units.
#pragma once

#include <cstdint>
#include <string>
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
// Graph accessors for the same: the host DAG and its device copy.
const HostDag &graph_dag(const kclpp_graph *g);
const uint64_t *graph_dev_offsets(const kclpp_graph *g);
const uint32_t *graph_dev_cols(const kclpp_graph *g);
int graph_device(const kclpp_graph *g);

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
