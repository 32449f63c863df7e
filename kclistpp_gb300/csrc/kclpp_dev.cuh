// kclpp_dev.cuh -- device-side types and warp primitives shared by the kernels.
//
// Work decomposition (all modes): one *root vertex* s at a time.  The k-cliques
// whose largest id is s are {s} ∪ K for the (k-1)-cliques K of G_s, the graph
// induced on the out-list N+(s) (kCDensestNoAtom.c:71-118 induces the same
// vertices per root edge; every root edge (s, t) has C(s, t) = N+(t) ∩ N+(s) =
// the row of t in G_s).  G_s is held as a bitmap adjacency matrix:
//   tier S  (d+(s) <= 64):       one warp per root, one 64-bit row per vertex,
//                                one lane per row / per root edge;
//   tier M  (64 < d+(s) <= 1024): one CTA per root, rows of W = ceil(d/32)
//                                32-bit words in shared memory, one lane per
//                                word, one warp per row / per root edge;
//   tier L  (1024 < d+(s) <= 2048): as tier M with two words per lane and the
//                                rows in a per-CTA global-memory slab.
// Roots are taken from a descending-work list by atomic counters (persistent
// CTAs); root edges / rows inside a root from a per-root global counter, which
// CTAs that have run out of roots join (work stealing).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace kclpp {
namespace dev {

#define KCL_FULL 0xffffffffu

// Error bits written to the context's device status word.
enum : uint32_t {
  ERR_OVERFLOW = 1u,     // a 32-bit stream counter would have wrapped
  ERR_DEGREE = 2u,       // a root's out-degree exceeds its tier's limit
};

enum Mode { MODE_COUNT = 0, MODE_ORDER = 1, MODE_SEQ = 2 };
enum KeyKind { KEY_SIM = 0, KEY_LEVEL = 1 };

struct PassArgs {
  const uint64_t *off;            // DAG out-CSR
  const uint32_t *cols;
  const uint32_t *roots;          // this tier's roots, descending work
  uint32_t num_roots;
  uint32_t dmax;                  // largest out-degree among them
  uint32_t *work;                 // root counter (zeroed before launch)
  uint32_t *task_next;            // tiers M, L: per-root sub-task counters (zeroed)
  uint32_t *active;               // tiers M, L: one slot per CTA, the root it holds (nullptr: no stealing)
  uint32_t *err;                  // status word
  int key_kind;                   // MODE_ORDER
  const double *rho;              // KEY_SIM
  const uint32_t *level;          // KEY_LEVEL
  unsigned long long *out;        // COUNT: nck; ORDER: per-vertex count; SEQ: r after the pass
  const unsigned long long *r_in; // SEQ: r at the start of the pass
  uint32_t *slab;                 // tier L: per-CTA row storage in global memory
  uint64_t slab_words;            // words per CTA in slab
  uint32_t deg_lo, deg_hi;        // id-order schedules: out-degree window of this launch
  unsigned long long *total;      // id-order schedules: sum of the roots' own clique counts
  // MODE_COUNT over explicit member lists (the k-clique core peel's recounts):
  // when list_off is set, root s is an index into list_off / list_cols, its
  // members are list_cols[list_off[s] .. list_off[s + 1]) (ascending ids, the
  // induced rows still built from the DAG off / cols), and the number of
  // k-cliques of {root} ∪ members through member i is stored at
  // pair_out[list_off[s] + i] instead of being added to out[].
  const uint64_t *list_off;
  const uint32_t *list_cols;
  unsigned long long *pair_out;
  // MODE_SEQ with shared loads (KCLPP_SEQ_SHARED): out is the one load vector
  // of the pass, read by every stream when it starts and added to in place
  // when it closes.
  int shared_loads;
};

// A root's member list: its DAG out-list, or its explicit list (peel recounts).
__device__ __forceinline__ void root_span(const PassArgs &a, uint32_t s, uint64_t &o, int &d,
                                          const uint32_t *&cols) {
  if (a.list_off) {
    o = a.list_off[s];
    d = (int)(a.list_off[s + 1] - o);
    cols = a.list_cols;
  } else {
    o = a.off[s];
    d = (int)(a.off[s + 1] - o);
    cols = a.cols;
  }
}

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(KCL_FULL, v, o);
  return v;
}

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(KCL_FULL, v, o);
    v = w < v ? w : v;
  }
  return v;
}

// Ordering key of a vertex for MODE_ORDER: the clique credits its smallest key.
//  KEY_SIM:   (rho bits, id) -- rho >= 0, so the IEEE bit pattern orders as the
//             value; ties go to the smaller id (kCDensestCmpSync.c:139-143).
//  KEY_LEVEL: larger level first (PAVA, kCDensestNoAtom.c:195-209).
__device__ __forceinline__ uint64_t vertex_key(const PassArgs &a, uint32_t v) {
  if (a.key_kind == KEY_SIM) return (uint64_t)__double_as_longlong(a.rho[v]);
  return (uint64_t)(0xFFFFFFFFu - a.level[v]);
}

// Lower bound of y in the ascending list[0, n).
__device__ __forceinline__ int lower_bound_u32(const uint32_t *list, int n, uint32_t y) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (list[mid] < y) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

}  // namespace dev

// Host-side launchers (one translation unit per mode).
struct TierLaunch {
  int tier;          // 0 = S, 1 = M, 2 = L
  const uint32_t *roots;
  uint32_t num_roots;
  uint32_t dmax;
  uint32_t *work;
  uint32_t *task_next;
  uint32_t *active;  // kActiveSlots slots (nullptr: no stealing)
  int num_sms;
  int max_grid;      // upper bound on CTAs (tier L: CTAs the row slab holds)
  int warps;         // tiers M / L: warps per CTA (0 = the most resident warps)
};
cudaError_t launch_count(int k, const TierLaunch &t, dev::PassArgs a, cudaStream_t st);
cudaError_t launch_order(int k, const TierLaunch &t, dev::PassArgs a, cudaStream_t st);
cudaError_t launch_seq(int k, const TierLaunch &t, dev::PassArgs a, cudaStream_t st);
// Threads per CTA.  Tier S: kWarpsS warps.  Tiers M / L are sized at launch
// (the schedule's width, or the one that keeps the most warps resident at the
// launch's out-degree bound): the Seq kernel's warps each run a root-edge
// stream with a per-warp delta array (8..kWarpsMSeqMax warps); the counting
// kernels' warps share one bitmap per CTA (8..kWarpsMMax warps).
constexpr int kWarpsS = 4;
constexpr int kWarpsM = 8;
constexpr int kWarpsMMax = 32;
constexpr int kWarpsMSeqMax = 24;
// Widest CTA of a tier M / L launch: the counting kernels at k = 5 stop at 24
// warps so that two CTAs fit the register file at their 42-register budget.
template <int MODE, int K>
constexpr int warps_m() { return MODE == dev::MODE_SEQ ? kWarpsMSeqMax : (K == 5 ? 24 : kWarpsMMax); }
// Tier bounds on a root's out-degree.  The Seq kernel keeps only the smallest
// roots on tier S (a lane runs a whole root-edge stream there, which is slow
// on dense roots); the counting kernels use tier S up to 64.
constexpr uint32_t kTierSMax = 64;
constexpr uint32_t kTierSMaxSeq = 16;
constexpr uint32_t kTierMMax = 1024;
constexpr uint32_t kTierLMax = 2048;
// Slots of a stealing launch's root registry (its grid is capped to this).
constexpr uint32_t kActiveSlots = 2048;

}  // namespace kclpp
