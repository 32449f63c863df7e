// kclpp_api.cu -- the C ABI: contexts, device graphs, passes, extraction, trim.
//
// Data layout in HBM, per graph: the DAG out-CSR (offsets u64[n+1], cols
// u32[m], ascending rows, cols < row), the source of every edge (u32[m], for
// the edge-parallel CountEdges), and the root schedule: every vertex with an
// out-edge, split into tiers by out-degree and sorted by descending estimated
// work inside each tier.  Per-pass vectors (r, counts, level) live in a
// workspace owned by the graph and reused across calls.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <numeric>

#include "kclpp_dev.cuh"
#include "kclpp_internal.h"

namespace kclpp {
const char *last_error_cstr();
}
using namespace kclpp;

#define KCL_CUDA(call)                                                                        \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      return set_error(e_ == cudaErrorMemoryAllocation ? KCLPP_ERR_NOMEM : KCLPP_ERR_CUDA,    \
                       "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);  \
  } while (0)

#define KCL_TRY(call)                      \
  do {                                     \
    kclpp_status s_ = (call);              \
    if (s_ != KCLPP_OK) return s_;         \
  } while (0)

struct PendingTime {
  int mode, tier;
  uint32_t dmax;
  cudaEvent_t a, b;
};

struct kclpp_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int num_sms = 1;
  uint32_t *d_err = nullptr;
  uint64_t launches = 0;
  bool profile = false;
  // Side streams for the concurrent launch of a pass's root groups, forked
  // from and joined back into `stream` with events.
  cudaStream_t side[4] = {};
  cudaEvent_t fork_ev = nullptr, join_ev[4] = {};
  std::vector<PendingTime> pending;
  std::vector<cudaEvent_t> event_pool;
};

static cudaEvent_t take_event(kclpp_ctx *c) {
  if (!c->event_pool.empty()) {
    cudaEvent_t e = c->event_pool.back();
    c->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  return e;
}

// Scheduler words of a pass: root counters of up to 5 launch groups, then one
// stealing registry (kActiveSlots words) per group.
constexpr size_t kWorkActive = 32;
constexpr size_t kWorkWords = kWorkActive + 5 * (size_t)kActiveSlots;

struct TierInfo {
  int tier;
  int bucket;  // 0..3: the M1, M2, M3 and L root groups (kclpp_schedule.seq_warps); -1: tier S
  uint32_t offset, count, dmax;
};

struct kclpp_graph {
  int device = 0;
  HostDag dag;
  // Schedule knobs (tier bounds, stealing); the autotuner may change them.
  kclpp_schedule sp = {kTierSMax, kTierSMaxSeq, 256, 512, 1, 0, 4, {0, 0, 0, 0}, 1, {0, 0, 0, 0}, 256, 512, 1};
  // KCLPP_SEQ_WAVES: one Seq schedule per wave (roots grouped by a fixed hash).
  std::vector<std::vector<TierInfo>> wave_tiers;
  std::vector<uint32_t> wave_base;
  uint64_t *d_off = nullptr;
  uint32_t *d_cols = nullptr;
  uint32_t *d_src = nullptr;
  uint32_t *d_roots = nullptr;
  // Two schedules over the same roots: [0] for the counting kernels (tier S up
  // to out-degree 64), [1] for the Seq kernel (tier S up to 16).
  std::vector<TierInfo> tiers[2];
  // Sharding (several devices splitting one pass): owner rank of every root.
  std::vector<uint32_t> owner;
  uint32_t shard_rank = 0, shard_world = 1;
  uint32_t sched_base[2] = {0, 0};
  uint32_t maxdeg = 0;
  // workspace
  unsigned long long *d_a = nullptr, *d_b = nullptr;
  double *d_rho = nullptr;
  uint32_t *d_level = nullptr;
  uint32_t *d_work = nullptr;   // [0,16): root counters per tier; from kWorkActive: the
                                // stealing registries, kActiveSlots words per tier
  uint32_t *d_task = nullptr;   // per-root sub-task counters (tiers M, L)
  uint32_t num_roots = 0;
  uint32_t task_cap = 0;
  unsigned long long *d_scalar = nullptr;
  uint32_t *d_slab = nullptr;
  uint64_t slab_words = 0;
  int slab_ctas = 0;
};

// ---------------------------------------------------------------------------
// small device helpers
namespace {

__global__ void k_sim_update(double *rho, const unsigned long long *cnt, uint32_t n, uint32_t t) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  // rho = (t * rho + 2.0 * rho_add) / (t + 2.0), each operation rounded
  // separately (kCDensestCmpSync.c:403); rho_add is an exact integer.
  const double td = __uint2double_rn(t);
  const double add = __ull2double_rn(cnt[i]);
  rho[i] = __ddiv_rn(__dadd_rn(__dmul_rn(td, rho[i]), __dmul_rn(2.0, add)), __dadd_rn(td, 2.0));
}

__global__ void k_scatter_level(unsigned long long *tent, const unsigned long long *cnt, const uint32_t *level,
                                uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) tent[level[i]] = cnt[i];
}

__global__ void k_count_edges(const uint32_t *src, const uint32_t *cols, uint64_t m, const uint32_t *level,
                              uint32_t nstar, unsigned long long *out) {
  unsigned long long c = 0;
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x)
    c += (level[src[e]] < nstar && level[cols[e]] < nstar);
  c = dev::warp_sum(c);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

inline int blocks_for(uint64_t n, int t = 256) { return (int)std::max<uint64_t>(1, (n + t - 1) / t); }

}  // namespace

// ---------------------------------------------------------------------------
static kclpp_status check_err(kclpp_ctx *c) {
  uint32_t e = 0;
  KCL_CUDA(cudaMemcpyAsync(&e, c->d_err, sizeof e, cudaMemcpyDeviceToHost, c->stream));
  KCL_CUDA(cudaStreamSynchronize(c->stream));
  if (e) {
    KCL_CUDA(cudaMemsetAsync(c->d_err, 0, sizeof(uint32_t), c->stream));
    if (e & dev::ERR_OVERFLOW) return set_error(KCLPP_ERR_OVERFLOW, "a per-stream 32-bit counter would have wrapped");
    if (e & dev::ERR_DEGREE) return set_error(KCLPP_ERR_UNSUPPORTED, "a root's out-degree exceeds its tier");
    return set_error(KCLPP_ERR_CUDA, "device status word 0x%x", e);
  }
  return KCLPP_OK;
}

static kclpp_status set_device(kclpp_ctx *c) {
  KCL_CUDA(cudaSetDevice(c->device));
  return KCLPP_OK;
}

template <typename T>
static kclpp_status dalloc(T **p, size_t count) {
  if (*p) return KCLPP_OK;
  KCL_CUDA(cudaMalloc((void **)p, std::max<size_t>(count, 1) * sizeof(T)));
  return KCLPP_OK;
}

// Root partition for sharded passes: roots by descending estimated work
// (out-degree squared), each to the rank with the least work so far (ties to
// the lower rank).  Deterministic, so every rank computes the same plan.
static void shard_plan_host(uint32_t n, const uint64_t *off, uint32_t world, uint32_t *owner) {
  std::vector<uint32_t> roots;
  for (uint32_t s = 0; s < n; ++s) {
    owner[s] = 0;
    if (off[s + 1] > off[s]) roots.push_back(s);
  }
  auto w = [&](uint32_t s) { const uint64_t d = off[s + 1] - off[s]; return d * d; };
  std::stable_sort(roots.begin(), roots.end(), [&](uint32_t a, uint32_t b) { return w(a) > w(b); });
  std::vector<uint64_t> load(world, 0);
  for (uint32_t s : roots) {
    uint32_t best = 0;
    for (uint32_t r = 1; r < world; ++r)
      if (load[r] < load[best]) best = r;
    owner[s] = best;
    load[best] += w(s);
  }
}

// Wave of a root for KCLPP_SEQ_WAVES: a fixed multiplicative hash, so roots of
// similar work spread over the waves.
static inline uint32_t wave_of(uint32_t s, uint32_t B) { return (uint32_t)(s * 2654435761u) % B; }

// Root schedules: tiers by out-degree, descending work (out-degree, then id)
// inside each tier; tier L first, then tier M from the largest roots down, so
// that the longest CTAs start first.
static kclpp_status build_schedule(kclpp_ctx *c, kclpp_graph *g) {
  const HostDag &D = g->dag;
  auto deg = [&](uint32_t s) { return (uint32_t)(D.off[s + 1] - D.off[s]); };
  auto by_work = [&](uint32_t a, uint32_t b) {
    const uint32_t da = deg(a), db = deg(b);
    return da != db ? da > db : a < b;
  };
  std::vector<uint32_t> all;
  bool any_l = false;
  uint32_t mx = 0;
  for (int sch = 0; sch < 2; ++sch) {
    const uint32_t smax = sch == 0 ? g->sp.tier_s_max : g->sp.tier_s_max_seq;
    const uint32_t split1 = sch == 0 ? g->sp.m_split1 : g->sp.seq_split1;
    const uint32_t split2 = sch == 0 ? g->sp.m_split2 : g->sp.seq_split2;
    std::vector<uint32_t> tS, tM1, tM2, tM3, tL;
    for (uint32_t s = 0; s < D.n; ++s) {
      const uint32_t d = deg(s);
      if (d == 0) continue;
      if (g->shard_world > 1 && g->owner[s] != g->shard_rank) continue;
      mx = std::max(mx, d);
      if (d <= smax) tS.push_back(s);
      else if (d <= split1) tM1.push_back(s);
      else if (d <= split2) tM2.push_back(s);
      else if (d <= kTierMMax) tM3.push_back(s);
      else tL.push_back(s);
    }
    any_l |= !tL.empty();
    g->sched_base[sch] = (uint32_t)all.size();
    g->tiers[sch].clear();
    auto add = [&](std::vector<uint32_t> &v, int tier, int bucket) {
      if (v.empty()) return;
      std::sort(v.begin(), v.end(), by_work);
      TierInfo t;
      t.tier = tier;
      t.bucket = bucket;
      t.offset = (uint32_t)all.size();
      t.count = (uint32_t)v.size();
      t.dmax = deg(v.front());
      all.insert(all.end(), v.begin(), v.end());
      g->tiers[sch].push_back(t);
    };
    add(tL, 2, 3);
    add(tM3, 1, 2);
    add(tM2, 1, 1);
    add(tM1, 1, 0);
    add(tS, 0, -1);
    if (sch == 0) g->num_roots = (uint32_t)all.size();
  }
  g->maxdeg = mx;
  // Waves: the Seq roots again, grouped by wave_of(s); each group tiered as the
  // Seq schedule is.
  g->wave_tiers.clear();
  g->wave_base.clear();
  const uint32_t B = std::max<uint32_t>(g->sp.seq_waves, 1);
  if (B > 1) {
    std::vector<std::vector<uint32_t>> grp(B);
    for (uint32_t s = 0; s < D.n; ++s) {
      if (deg(s) == 0) continue;
      if (g->shard_world > 1 && g->owner[s] != g->shard_rank) continue;
      grp[wave_of(s, B)].push_back(s);
    }
    for (uint32_t w = 0; w < B; ++w) {
      g->wave_base.push_back((uint32_t)all.size());
      std::vector<uint32_t> tS, tM1, tM2, tM3, tL;
      for (uint32_t s : grp[w]) {
        const uint32_t d = deg(s);
        if (d <= g->sp.tier_s_max_seq) tS.push_back(s);
        else if (d <= g->sp.seq_split1) tM1.push_back(s);
        else if (d <= g->sp.seq_split2) tM2.push_back(s);
        else if (d <= kTierMMax) tM3.push_back(s);
        else tL.push_back(s);
      }
      std::vector<TierInfo> tw;
      auto addw = [&](std::vector<uint32_t> &v, int tier, int bucket) {
        if (v.empty()) return;
        std::sort(v.begin(), v.end(), by_work);
        TierInfo t;
        t.tier = tier;
        t.bucket = bucket;
        t.offset = (uint32_t)all.size();
        t.count = (uint32_t)v.size();
        t.dmax = deg(v.front());
        all.insert(all.end(), v.begin(), v.end());
        tw.push_back(t);
      };
      addw(tL, 2, 3);
      addw(tM3, 1, 2);
      addw(tM2, 1, 1);
      addw(tM1, 1, 0);
      addw(tS, 0, -1);
      g->wave_tiers.push_back(tw);
    }
  }
  KCL_TRY(dalloc(&g->d_roots, all.size()));
  if (!all.empty())
    KCL_CUDA(cudaMemcpyAsync(g->d_roots, all.data(), all.size() * 4, cudaMemcpyHostToDevice, c->stream));
  KCL_TRY(dalloc(&g->d_work, kWorkWords));
  if (g->num_roots > g->task_cap) {  // the counters must cover every root of the schedule
    cudaFree(g->d_task);
    g->d_task = nullptr;
    g->task_cap = 0;
  }
  KCL_TRY(dalloc(&g->d_task, g->num_roots));
  g->task_cap = std::max(g->task_cap, std::max<uint32_t>(g->num_roots, 1));
  if (any_l) {
    g->slab_ctas = c->num_sms;
    const uint64_t W = (kTierLMax + 31) / 32;
    g->slab_words = (uint64_t)kTierLMax * W;
    KCL_TRY(dalloc(&g->d_slab, g->slab_words * g->slab_ctas));
  }
  return KCLPP_OK;
}

static kclpp_status upload_graph(kclpp_ctx *c, kclpp_graph *g) {
  const HostDag &D = g->dag;
  if (D.core > kTierLMax)
    return set_error(KCLPP_ERR_UNSUPPORTED, "max out-degree %u exceeds the supported %u", D.core, kTierLMax);
  KCL_TRY(dalloc(&g->d_off, (size_t)D.n + 1));
  KCL_TRY(dalloc(&g->d_cols, D.m()));
  KCL_TRY(dalloc(&g->d_src, D.m()));
  KCL_CUDA(cudaMemcpyAsync(g->d_off, D.off.data(), ((size_t)D.n + 1) * 8, cudaMemcpyHostToDevice, c->stream));
  if (D.m()) {
    KCL_CUDA(cudaMemcpyAsync(g->d_cols, D.cols.data(), D.m() * 4, cudaMemcpyHostToDevice, c->stream));
    std::vector<uint32_t> src(D.m());
    for (uint32_t s = 0; s < D.n; ++s)
      for (uint64_t e = D.off[s]; e < D.off[s + 1]; ++e) src[e] = s;
    KCL_CUDA(cudaMemcpyAsync(g->d_src, src.data(), D.m() * 4, cudaMemcpyHostToDevice, c->stream));
    KCL_CUDA(cudaStreamSynchronize(c->stream));
  }
  KCL_TRY(build_schedule(c, g));
  const size_t n1 = (size_t)D.n + 1;
  KCL_TRY(dalloc(&g->d_a, n1));
  KCL_TRY(dalloc(&g->d_b, n1));
  KCL_TRY(dalloc(&g->d_rho, n1));
  KCL_TRY(dalloc(&g->d_level, n1));
  KCL_TRY(dalloc(&g->d_scalar, 4));
  KCL_CUDA(cudaStreamSynchronize(c->stream));
  return KCLPP_OK;
}

static void free_graph_dev(kclpp_graph *g) {
  cudaFree(g->d_off); cudaFree(g->d_cols); cudaFree(g->d_src); cudaFree(g->d_roots);
  cudaFree(g->d_a); cudaFree(g->d_b); cudaFree(g->d_rho); cudaFree(g->d_level);
  cudaFree(g->d_work); cudaFree(g->d_task); cudaFree(g->d_scalar); cudaFree(g->d_slab);
}

// Where a pass runs: its stream and its scheduler counters.  Concurrent passes
// (the batch's k values) each need their own counters.
struct Exec {
  cudaStream_t st;
  uint32_t *work;  // kWorkWords words
  uint32_t *task;  // one per root
};

// Launch every tier of one mode.
static kclpp_status run_tiers(kclpp_ctx *c, kclpp_graph *g, int mode, int k, dev::PassArgs a,
                              const Exec *ex = nullptr, int wave = -1) {
  const int sch = mode == dev::MODE_SEQ ? 1 : 0;
  const bool wv = mode == dev::MODE_SEQ && wave >= 0;
  const std::vector<TierInfo> &tiers = wv ? g->wave_tiers[wave] : g->tiers[sch];
  const uint32_t base = wv ? g->wave_base[wave] : g->sched_base[sch];
  if (tiers.empty()) return KCLPP_OK;
  const Exec E = ex ? *ex : Exec{c->stream, g->d_work, g->d_task};
  KCL_CUDA(cudaMemsetAsync(E.work, 0, kWorkActive * sizeof(uint32_t), E.st));
  KCL_CUDA(cudaMemsetAsync(E.work + kWorkActive, 0xff, (kWorkWords - kWorkActive) * sizeof(uint32_t), E.st));
  KCL_CUDA(cudaMemsetAsync(E.task, 0, (size_t)g->num_roots * sizeof(uint32_t), E.st));
  a.off = g->d_off;
  a.cols = g->d_cols;
  a.err = c->d_err;
  a.slab = g->d_slab;
  a.slab_words = g->slab_words;
  // Root groups of one pass are independent (they read the pass-start vector
  // and add into the output), so they may run side by side: the later groups
  // fill the SMs that the first one's tail leaves idle.
  const int nside =
      (!ex && (mode == dev::MODE_SEQ ? g->sp.concurrent_tiers : g->sp.concurrent_count) && tiers.size() > 1)
          ? (int)std::min<size_t>(tiers.size() - 1, 4)
          : 0;
  if (nside) {
    KCL_CUDA(cudaEventRecord(c->fork_ev, E.st));
    for (int j = 0; j < nside; ++j) KCL_CUDA(cudaStreamWaitEvent(c->side[j], c->fork_ev, 0));
  }
  for (size_t i = 0; i < tiers.size(); ++i) {
    const TierInfo &t = tiers[i];
    const cudaStream_t ls = (nside && i > 0) ? c->side[(i - 1) % nside] : E.st;
    TierLaunch tl;
    tl.tier = t.tier;
    tl.roots = g->d_roots + t.offset;
    tl.num_roots = t.count;
    tl.dmax = t.dmax;
    tl.work = E.work + i;
    tl.task_next = E.task + (t.offset - base);
    // Work stealing pays off for the Seq chains (long, uneven root edges); the
    // counting kernels finish their roots quickly and by default do not steal.
    const bool steal = mode == dev::MODE_SEQ ? g->sp.steal_seq != 0 : g->sp.steal_count != 0;
    tl.active = steal ? E.work + kWorkActive + i * kActiveSlots : nullptr;
    tl.num_sms = c->num_sms;
    tl.max_grid = t.tier == 2 ? g->slab_ctas : 0;
    tl.warps = t.bucket < 0 ? 0 : (int)(mode == dev::MODE_SEQ ? g->sp.seq_warps[t.bucket] : g->sp.count_warps[t.bucket]);
    cudaError_t e = cudaSuccess;
    PendingTime pt{mode, t.tier, t.dmax, nullptr, nullptr};
    const bool prof = c->profile && !ex;
    if (prof) {
      pt.a = take_event(c);
      pt.b = take_event(c);
      if (pt.a) cudaEventRecord(pt.a, ls);
    }
    if (mode == dev::MODE_COUNT) e = launch_count(k, tl, a, ls);
    else if (mode == dev::MODE_ORDER) e = launch_order(k, tl, a, ls);
    else e = launch_seq(k, tl, a, ls);
    if (prof && pt.a && pt.b) {
      cudaEventRecord(pt.b, ls);
      c->pending.push_back(pt);
    }
    if (e != cudaSuccess) {
      // Join what the side streams already hold before reporting, so that the
      // caller's stream orders after every launch of this pass.
      for (int j = 0; j < nside; ++j) {
        cudaEventRecord(c->join_ev[j], c->side[j]);
        cudaStreamWaitEvent(E.st, c->join_ev[j], 0);
      }
      return set_error(KCLPP_ERR_CUDA, "kernel launch (mode %d, tier %d, k %d): %s", mode, t.tier, k,
                       cudaGetErrorString(e));
    }
    c->launches++;
  }
  for (int j = 0; j < nside; ++j) {
    KCL_CUDA(cudaEventRecord(c->join_ev[j], c->side[j]));
    KCL_CUDA(cudaStreamWaitEvent(E.st, c->join_ev[j], 0));
  }
  return KCLPP_OK;
}

// ---- device-resident passes (enqueue only) ---------------------------------
static bool valid_seq_mode(int m) {
  return m == KCLPP_SEQ_EDGE_STREAMS || m == KCLPP_SEQ_WAVES || m == KCLPP_SEQ_SHARED;
}

// One Seq pass from `in` into `out`.  KCLPP_SEQ_WAVES runs the waves in order,
// each wave's root-edge streams starting from r after the previous waves; it
// uses `in` as the second ping-pong buffer (its contents are not needed after
// the pass).
static kclpp_status seq_pass_dev(kclpp_ctx *c, kclpp_graph *g, int k, const unsigned long long *in,
                                 unsigned long long *out,
                                 int det_mode = KCLPP_SEQ_EDGE_STREAMS) {
  const uint32_t n = g->dag.n;
  if (det_mode == KCLPP_SEQ_WAVES && g->wave_tiers.size() > 1 && in != out) {
    unsigned long long *src = const_cast<unsigned long long *>(in), *dst = out;
    for (size_t w = 0; w < g->wave_tiers.size(); ++w) {
      KCL_CUDA(cudaMemcpyAsync(dst, src, (size_t)n * 8, cudaMemcpyDeviceToDevice, c->stream));
      dev::PassArgs a{};
      a.r_in = src;
      a.out = dst;
      KCL_TRY(run_tiers(c, g, dev::MODE_SEQ, k, a, nullptr, (int)w));
      std::swap(src, dst);
    }
    if (src != out) KCL_CUDA(cudaMemcpyAsync(out, src, (size_t)n * 8, cudaMemcpyDeviceToDevice, c->stream));
    return KCLPP_OK;
  }
  if (in != out) KCL_CUDA(cudaMemcpyAsync(out, in, (size_t)n * 8, cudaMemcpyDeviceToDevice, c->stream));
  dev::PassArgs a{};
  a.r_in = in;
  a.out = out;
  if (det_mode == KCLPP_SEQ_SHARED) {
    // One load vector, read and added to in place by every stream.
    a.r_in = out;
    a.shared_loads = 1;
  }
  return run_tiers(c, g, dev::MODE_SEQ, k, a);
}

static kclpp_status sim_counts_dev(kclpp_ctx *c, kclpp_graph *g, int k, const double *rho, unsigned long long *cnt) {
  KCL_CUDA(cudaMemsetAsync(cnt, 0, (size_t)g->dag.n * 8, c->stream));
  dev::PassArgs a{};
  a.key_kind = dev::KEY_SIM;
  a.rho = rho;
  a.out = cnt;
  return run_tiers(c, g, dev::MODE_ORDER, k, a);
}

static kclpp_status sim_pass_dev(kclpp_ctx *c, kclpp_graph *g, int k, uint32_t t, double *rho) {
  KCL_TRY(sim_counts_dev(c, g, k, rho, g->d_a));
  const uint32_t n = g->dag.n;
  if (n) {
    k_sim_update<<<blocks_for(n), 256, 0, c->stream>>>(rho, g->d_a, n, t);
    KCL_CUDA(cudaGetLastError());
    c->launches++;
  }
  return KCLPP_OK;
}

static kclpp_status pava_dev(kclpp_ctx *c, kclpp_graph *g, int k, const uint32_t *level_dev,
                             unsigned long long *tent_dev) {
  const uint32_t n = g->dag.n;
  KCL_CUDA(cudaMemsetAsync(g->d_a, 0, (size_t)n * 8, c->stream));
  dev::PassArgs a{};
  a.key_kind = dev::KEY_LEVEL;
  a.level = level_dev;
  a.out = g->d_a;
  KCL_TRY(run_tiers(c, g, dev::MODE_ORDER, k, a));
  if (n) {
    k_scatter_level<<<blocks_for(n), 256, 0, c->stream>>>(tent_dev, g->d_a, level_dev, n);
    KCL_CUDA(cudaGetLastError());
    c->launches++;
  }
  return KCLPP_OK;
}

static kclpp_status check_k(int k, int lo) {
  if (k < lo || k > KCLPP_MAX_K)
    return set_error(KCLPP_ERR_UNSUPPORTED, "k = %d outside the supported range [%d, %d]", k, lo, KCLPP_MAX_K);
  return KCLPP_OK;
}

// After kclpp_graph_shard(world > 1) the graph's root schedule holds this
// rank's roots only, so a whole-graph result would silently be partial: only
// the shard entry points (kclpp_seq_delta_dev, kclpp_sim_counts_dev) accept a
// sharded graph; kclpp_graph_shard(ctx, g, 0, 1) restores the full schedule.
static kclpp_status check_unsharded(const kclpp_graph *g, const char *fn) {
  if (g->shard_world > 1)
    return set_error(KCLPP_ERR_INVALID, "%s: the graph is sharded (rank %u of %u); only kclpp_seq_delta_dev and "
                     "kclpp_sim_counts_dev run on a shard", fn, g->shard_rank, g->shard_world);
  return KCLPP_OK;
}

// ---- host-side pieces of the extraction (A10, A12, A13) --------------------
struct KeyId {
  uint64_t key;
  uint32_t id;
};
static void sort_desc(uint32_t n, std::vector<KeyId> &v, uint32_t *reordered, uint32_t *level) {
  std::sort(v.begin(), v.end(), [](const KeyId &a, const KeyId &b) {
    return a.key != b.key ? a.key > b.key : a.id < b.id;
  });
  for (uint32_t i = 0; i < n; ++i) {
    if (reordered) reordered[i] = v[i].id;
    if (level) level[v[i].id] = i;
  }
}

extern "C" {

const char *kclpp_status_string(kclpp_status s) {
  switch (s) {
    case KCLPP_OK: return "ok";
    case KCLPP_ERR_INVALID: return "invalid argument";
    case KCLPP_ERR_IO: return "i/o error";
    case KCLPP_ERR_NOMEM: return "out of memory";
    case KCLPP_ERR_CUDA: return "cuda error";
    case KCLPP_ERR_UNSUPPORTED: return "unsupported";
    case KCLPP_ERR_OVERFLOW: return "counter overflow";
    case KCLPP_ERR_NODEVICE: return "no cuda device";
    default: return "unknown status";
  }
}
const char *kclpp_last_error(void) { return last_error_cstr(); }
const char *kclpp_version(void) { return "kclpp-gb300 0.1 (sm_103a)"; }

kclpp_status kclpp_create(int device, void *stream, kclpp_ctx **out) {
  if (!out) return set_error(KCLPP_ERR_INVALID, "kclpp_create: null out");
  *out = nullptr;
  int nd = 0;
  cudaError_t e = cudaGetDeviceCount(&nd);
  if (e != cudaSuccess || nd == 0) return set_error(KCLPP_ERR_NODEVICE, "no CUDA device (%s)", cudaGetErrorString(e));
  if (device < 0 || device >= nd) return set_error(KCLPP_ERR_INVALID, "device %d out of range", device);
  std::unique_ptr<kclpp_ctx> c(new kclpp_ctx());
  c->device = device;
  KCL_CUDA(cudaSetDevice(device));
  KCL_CUDA(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device));
  if (stream) {
    c->stream = (cudaStream_t)stream;
  } else {
    KCL_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    c->own_stream = true;
  }
  for (int i = 0; i < 4; ++i) {
    KCL_CUDA(cudaStreamCreateWithFlags(&c->side[i], cudaStreamNonBlocking));
    KCL_CUDA(cudaEventCreateWithFlags(&c->join_ev[i], cudaEventDisableTiming));
  }
  KCL_CUDA(cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming));
  KCL_CUDA(cudaMalloc((void **)&c->d_err, sizeof(uint32_t)));
  KCL_CUDA(cudaMemsetAsync(c->d_err, 0, sizeof(uint32_t), c->stream));
  KCL_CUDA(cudaStreamSynchronize(c->stream));
  *out = c.release();
  return KCLPP_OK;
}

kclpp_status kclpp_destroy(kclpp_ctx *c) {
  if (!c) return KCLPP_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (auto &p : c->pending) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
  for (auto e : c->event_pool) cudaEventDestroy(e);
  cudaFree(c->d_err);
  for (int i = 0; i < 4; ++i) {
    if (c->side[i]) cudaStreamDestroy(c->side[i]);
    if (c->join_ev[i]) cudaEventDestroy(c->join_ev[i]);
  }
  if (c->fork_ev) cudaEventDestroy(c->fork_ev);
  if (c->own_stream) cudaStreamDestroy(c->stream);
  delete c;
  return KCLPP_OK;
}

kclpp_status kclpp_synchronize(kclpp_ctx *c) {
  if (!c) return set_error(KCLPP_ERR_INVALID, "null context");
  KCL_TRY(set_device(c));
  return check_err(c);
}

uint64_t kclpp_launch_count(const kclpp_ctx *c) { return c ? c->launches : 0; }

kclpp_status kclpp_profile_enable(kclpp_ctx *c, int on) {
  if (!c) return set_error(KCLPP_ERR_INVALID, "null context");
  c->profile = on != 0;
  return KCLPP_OK;
}

kclpp_status kclpp_profile_read(kclpp_ctx *c, kclpp_kernel_time *out, int cap, int *count) {
  if (!c || (!out && cap > 0)) return set_error(KCLPP_ERR_INVALID, "null argument");
  KCL_TRY(set_device(c));
  KCL_CUDA(cudaStreamSynchronize(c->stream));
  std::vector<kclpp_kernel_time> agg;
  for (auto &p : c->pending) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p.a, p.b);
    auto it = std::find_if(agg.begin(), agg.end(), [&](const kclpp_kernel_time &x) {
      return x.mode == p.mode && x.tier == p.tier && x.dmax == p.dmax;
    });
    if (it == agg.end()) {
      agg.push_back({p.mode, p.tier, p.dmax, 0u, 0.0});
      it = agg.end() - 1;
    }
    it->launches++;
    it->ms += ms;
    c->event_pool.push_back(p.a);
    c->event_pool.push_back(p.b);
  }
  c->pending.clear();
  const int nw = std::min<int>(cap, (int)agg.size());
  for (int i = 0; i < nw; ++i) out[i] = agg[i];
  if (count) *count = (int)agg.size();
  return KCLPP_OK;
}

// ---- graphs -------------------------------------------------------------------
kclpp_status kclpp_core_order(const kclpp_edge_list *el, uint32_t *rank_out) {
  if (!el || !rank_out) return set_error(KCLPP_ERR_INVALID, "kclpp_core_order: null argument");
  core_order_host(el->n, el->pairs, rank_out);
  return KCLPP_OK;
}

static kclpp_status finish_graph(kclpp_ctx *c, kclpp_graph *gp, kclpp_graph **out) {
  std::unique_ptr<kclpp_graph> g(gp);
  g->device = c->device;
  kclpp_status s = upload_graph(c, g.get());
  if (s != KCLPP_OK) {
    free_graph_dev(g.get());
    return s;
  }
  *out = g.release();
  return KCLPP_OK;
}

kclpp_status kclpp_make_graph(kclpp_ctx *c, const kclpp_edge_list *el, const uint32_t *rank, kclpp_graph **out) {
  if (!c || !el || !rank || !out) return set_error(KCLPP_ERR_INVALID, "kclpp_make_graph: null argument");
  *out = nullptr;
  KCL_TRY(set_device(c));
  auto *g = new kclpp_graph();
  kclpp_status s = make_dag_host(el->pairs, rank, g->dag);
  if (s != KCLPP_OK) { delete g; return s; }
  return finish_graph(c, g, out);
}

kclpp_status kclpp_build_graph(kclpp_ctx *c, const kclpp_edge_list *el, kclpp_graph **out) {
  return kclpp_build_graph_mode(c, el, KCLPP_ORDER_EXACT, out);
}

kclpp_status kclpp_core_order_mode(const kclpp_edge_list *el, int mode, uint32_t *rank_out) {
  if (!el || !rank_out) return set_error(KCLPP_ERR_INVALID, "kclpp_core_order_mode: null argument");
  if (mode == KCLPP_ORDER_EXACT) core_order_host(el->n, el->pairs, rank_out);
  else if (mode == KCLPP_ORDER_FAST) core_order_fast_host(el->n, el->pairs, rank_out);
  else return set_error(KCLPP_ERR_INVALID, "unknown order mode %d", mode);
  return KCLPP_OK;
}

kclpp_status kclpp_build_graph_mode(kclpp_ctx *c, const kclpp_edge_list *el, int mode, kclpp_graph **out) {
  if (!c || !el || !out) return set_error(KCLPP_ERR_INVALID, "kclpp_build_graph: null argument");
  std::vector<uint32_t> rank(el->n);
  KCL_TRY(kclpp_core_order_mode(el, mode, rank.data()));
  return kclpp_make_graph(c, el, rank.data(), out);
}

kclpp_status kclpp_graph_from_csr(kclpp_ctx *c, uint32_t n, uint64_t m, const uint64_t *offsets,
                                  const uint32_t *cols, kclpp_graph **out) {
  if (!c || !offsets || (!cols && m) || !out) return set_error(KCLPP_ERR_INVALID, "kclpp_graph_from_csr: null argument");
  *out = nullptr;
  if (offsets[0] != 0 || offsets[n] != m) return set_error(KCLPP_ERR_INVALID, "offsets[0] must be 0 and offsets[n] = m");
  KCL_TRY(set_device(c));
  auto *g = new kclpp_graph();
  g->dag.n = n;
  g->dag.off.assign(offsets, offsets + n + 1);
  g->dag.cols.assign(cols, cols + m);
  uint32_t mx = 0;
  for (uint32_t s = 0; s < n; ++s) {
    if (offsets[s + 1] < offsets[s]) { delete g; return set_error(KCLPP_ERR_INVALID, "offsets not monotone at %u", s); }
    mx = std::max<uint32_t>(mx, (uint32_t)(offsets[s + 1] - offsets[s]));
    for (uint64_t e = offsets[s]; e < offsets[s + 1]; ++e) {
      if (cols[e] >= s || (e > offsets[s] && cols[e] <= cols[e - 1])) {
        delete g;
        return set_error(KCLPP_ERR_INVALID, "row %u is not strictly ascending below the source", s);
      }
    }
  }
  g->dag.core = mx;
  return finish_graph(c, g, out);
}

kclpp_status kclpp_graph_info(const kclpp_graph *g, uint32_t *n, uint64_t *m, uint32_t *core) {
  if (!g) return set_error(KCLPP_ERR_INVALID, "null graph");
  if (n) *n = g->dag.n;
  if (m) *m = g->dag.m();
  if (core) *core = g->dag.core;
  return KCLPP_OK;
}

kclpp_status kclpp_graph_copy_csr(const kclpp_graph *g, uint64_t *offsets, uint32_t *cols) {
  if (!g) return set_error(KCLPP_ERR_INVALID, "null graph");
  if (offsets) memcpy(offsets, g->dag.off.data(), g->dag.off.size() * 8);
  if (cols && g->dag.m()) memcpy(cols, g->dag.cols.data(), g->dag.m() * 4);
  return KCLPP_OK;
}

void kclpp_graph_free(kclpp_graph *g) {
  if (!g) return;
  cudaSetDevice(g->device);
  free_graph_dev(g);
  delete g;
}

// ---- counts ---------------------------------------------------------------------
kclpp_status kclpp_count_cliques(kclpp_ctx *c, const kclpp_graph *gc, int k, uint64_t *per_vertex, uint64_t *total) {
  if (!c || !gc) return set_error(KCLPP_ERR_INVALID, "null argument");
  KCL_TRY(check_unsharded(gc, "kclpp_count_cliques"));
  KCL_TRY(check_k(k, 3));
  KCL_TRY(set_device(c));
  kclpp_graph *g = const_cast<kclpp_graph *>(gc);
  const uint32_t n = g->dag.n;
  KCL_CUDA(cudaMemsetAsync(g->d_a, 0, (size_t)n * 8 + 8, c->stream));
  dev::PassArgs a{};
  a.out = g->d_a;
  KCL_TRY(run_tiers(c, g, dev::MODE_COUNT, k, a));
  KCL_TRY(check_err(c));
  std::vector<uint64_t> h(n);
  if (n) KCL_CUDA(cudaMemcpyAsync(h.data(), g->d_a, (size_t)n * 8, cudaMemcpyDeviceToHost, c->stream));
  KCL_CUDA(cudaStreamSynchronize(c->stream));
  unsigned __int128 sum = 0;
  for (uint64_t v : h) sum += v;
  if (per_vertex && n) memcpy(per_vertex, h.data(), (size_t)n * 8);
  if (total) *total = (uint64_t)(sum / (unsigned)k);
  return KCLPP_OK;
}

// ---- Seq --------------------------------------------------------------------------
static kclpp_status seq_passes_on(kclpp_ctx *c, kclpp_graph *g, int k, uint32_t passes, unsigned long long *r,
                                  int det_mode = KCLPP_SEQ_EDGE_STREAMS) {
  if (det_mode == KCLPP_SEQ_SHARED) {  // in place
    for (uint32_t p = 0; p < passes; ++p) KCL_TRY(seq_pass_dev(c, g, k, r, r, det_mode));
    return KCLPP_OK;
  }
  // Ping-pong between r and the workspace; end with the result in r.
  unsigned long long *in = r, *out = g->d_b;
  for (uint32_t p = 0; p < passes; ++p) {
    KCL_TRY(seq_pass_dev(c, g, k, in, out, det_mode));
    std::swap(in, out);
  }
  if (in != r) KCL_CUDA(cudaMemcpyAsync(r, in, (size_t)g->dag.n * 8, cudaMemcpyDeviceToDevice, c->stream));
  return KCLPP_OK;
}

kclpp_status kclpp_seq_passes_dev(kclpp_ctx *c, const kclpp_graph *gc, int k, uint32_t passes, int det_mode,
                                  uint64_t *r_dev) {
  if (!c || !gc || (!r_dev && gc->dag.n)) return set_error(KCLPP_ERR_INVALID, "null argument");
  KCL_TRY(check_unsharded(gc, "kclpp_seq_passes_dev"));
  KCL_TRY(check_k(k, 3));
  if (!valid_seq_mode(det_mode)) return set_error(KCLPP_ERR_INVALID, "unknown det_mode %d", det_mode);
  KCL_TRY(set_device(c));
  return seq_passes_on(c, const_cast<kclpp_graph *>(gc), k, passes, (unsigned long long *)r_dev, det_mode);
}

kclpp_status kclpp_seq_passes(kclpp_ctx *c, const kclpp_graph *gc, int k, uint32_t passes, int det_mode,
                              uint64_t *r) {
  if (!c || !gc || (!r && gc->dag.n)) return set_error(KCLPP_ERR_INVALID, "null argument");
  KCL_TRY(check_unsharded(gc, "kclpp_seq_passes"));
  KCL_TRY(check_k(k, 3));
  if (!valid_seq_mode(det_mode)) return set_error(KCLPP_ERR_INVALID, "unknown det_mode %d", det_mode);
  KCL_TRY(set_device(c));
  kclpp_graph *g = const_cast<kclpp_graph *>(gc);
  const size_t bytes = (size_t)g->dag.n * 8;
  if (!bytes) return KCLPP_OK;
  KCL_CUDA(cudaMemcpyAsync(g->d_a, r, bytes, cudaMemcpyHostToDevice, c->stream));
  KCL_TRY(seq_passes_on(c, g, k, passes, g->d_a, det_mode));
  KCL_CUDA(cudaMemcpyAsync(r, g->d_a, bytes, cudaMemcpyDeviceToHost, c->stream));
  return check_err(c);
}

kclpp_status kclpp_seq_passes_csr(kclpp_ctx *c, uint32_t n, uint64_t m, const uint64_t *offsets, const uint32_t *cols,
                                  int k, uint32_t passes, int det_mode, uint64_t *r) {
  kclpp_graph *g = nullptr;
  KCL_TRY(kclpp_graph_from_csr(c, n, m, offsets, cols, &g));
  kclpp_status s = kclpp_seq_passes(c, g, k, passes, det_mode, r);
  kclpp_graph_free(g);
  return s;
}

// ---- Sim --------------------------------------------------------------------------
kclpp_status kclpp_sim_counts(kclpp_ctx *c, const kclpp_graph *gc, int k, const double *rho, uint64_t *cnt) {
  if (!c || !gc || ((!rho || !cnt) && gc->dag.n)) return set_error(KCLPP_ERR_INVALID, "null argument");
  KCL_TRY(check_unsharded(gc, "kclpp_sim_counts"));
  KCL_TRY(check_k(k, 2));
  KCL_TRY(set_device(c));
  kclpp_graph *g = const_cast<kclpp_graph *>(gc);
  const size_t bytes = (size_t)g->dag.n * 8;
  if (!bytes) return KCLPP_OK;
  KCL_CUDA(cudaMemcpyAsync(g->d_rho, rho, bytes, cudaMemcpyHostToDevice, c->stream));
  KCL_TRY(sim_counts_dev(c, g, k, g->d_rho, g->d_a));
  KCL_CUDA(cudaMemcpyAsync(cnt, g->d_a, bytes, cudaMemcpyDeviceToHost, c->stream));
  return check_err(c);
}

kclpp_status kclpp_sim_passes_dev(kclpp_ctx *c, const kclpp_graph *gc, int k, uint32_t t_first, uint32_t passes,
                                  double *rho_dev) {
  if (!c || !gc || (!rho_dev && gc->dag.n)) return set_error(KCLPP_ERR_INVALID, "null argument");
  KCL_TRY(check_unsharded(gc, "kclpp_sim_passes_dev"));
  KCL_TRY(check_k(k, 2));
  if (t_first < 1) return set_error(KCLPP_ERR_INVALID, "t_first must be >= 1");
  KCL_TRY(set_device(c));
  kclpp_graph *g = const_cast<kclpp_graph *>(gc);
  for (uint32_t p = 0; p < passes; ++p) KCL_TRY(sim_pass_dev(c, g, k, t_first + p, rho_dev));
  return KCLPP_OK;
}

kclpp_status kclpp_sim_passes(kclpp_ctx *c, const kclpp_graph *gc, int k, uint32_t t_first, uint32_t passes,
                              double *rho) {
  if (!c || !gc || (!rho && gc->dag.n)) return set_error(KCLPP_ERR_INVALID, "null argument");
  KCL_TRY(check_unsharded(gc, "kclpp_sim_passes"));
  KCL_TRY(check_k(k, 2));
  if (t_first < 1) return set_error(KCLPP_ERR_INVALID, "t_first must be >= 1");
  KCL_TRY(set_device(c));
  kclpp_graph *g = const_cast<kclpp_graph *>(gc);
  const size_t bytes = (size_t)g->dag.n * 8;
  if (!bytes) return KCLPP_OK;
  KCL_CUDA(cudaMemcpyAsync(g->d_rho, rho, bytes, cudaMemcpyHostToDevice, c->stream));
  for (uint32_t p = 0; p < passes; ++p) KCL_TRY(sim_pass_dev(c, g, k, t_first + p, g->d_rho));
  KCL_CUDA(cudaMemcpyAsync(rho, g->d_rho, bytes, cudaMemcpyDeviceToHost, c->stream));
  return check_err(c);
}

kclpp_status kclpp_sim_passes_csr(kclpp_ctx *c, uint32_t n, uint64_t m, const uint64_t *offsets, const uint32_t *cols,
                                  int k, uint32_t t_first, uint32_t passes, double *rho) {
  kclpp_graph *g = nullptr;
  KCL_TRY(kclpp_graph_from_csr(c, n, m, offsets, cols, &g));
  kclpp_status s = kclpp_sim_passes(c, g, k, t_first, passes, rho);
  kclpp_graph_free(g);
  return s;
}

// ---- sharded passes (several devices splitting one pass) -----------------------------
kclpp_status kclpp_shard_plan(uint32_t n, const uint64_t *offsets, uint32_t world, uint32_t *owner) {
  if (!offsets || (!owner && n) || world == 0) return set_error(KCLPP_ERR_INVALID, "kclpp_shard_plan: bad argument");
  shard_plan_host(n, offsets, world, owner);
  return KCLPP_OK;
}

kclpp_status kclpp_graph_shard(kclpp_ctx *c, kclpp_graph *g, uint32_t rank, uint32_t world) {
  if (!c || !g || world == 0 || rank >= world) return set_error(KCLPP_ERR_INVALID, "kclpp_graph_shard: bad argument");
  KCL_TRY(set_device(c));
  g->owner.assign(g->dag.n, 0);
  if (world > 1) shard_plan_host(g->dag.n, g->dag.off.data(), world, g->owner.data());
  g->shard_rank = rank;
  g->shard_world = world;
  cudaFree(g->d_roots);
  g->d_roots = nullptr;
  KCL_TRY(build_schedule(c, g));
  KCL_CUDA(cudaStreamSynchronize(c->stream));
  return KCLPP_OK;
}

kclpp_status kclpp_seq_delta_dev(kclpp_ctx *c, const kclpp_graph *gc, int k, const uint64_t *r_dev, uint64_t *delta_dev) {
  if (!c || !gc || ((!r_dev || !delta_dev) && gc->dag.n)) return set_error(KCLPP_ERR_INVALID, "null argument");
  KCL_TRY(check_k(k, 3));
  KCL_TRY(set_device(c));
  kclpp_graph *g = const_cast<kclpp_graph *>(gc);
  if (!g->dag.n) return KCLPP_OK;
  KCL_CUDA(cudaMemsetAsync(delta_dev, 0, (size_t)g->dag.n * 8, c->stream));
  dev::PassArgs a{};
  a.r_in = (const unsigned long long *)r_dev;
  a.out = (unsigned long long *)delta_dev;
  return run_tiers(c, g, dev::MODE_SEQ, k, a);
}

kclpp_status kclpp_sim_counts_dev(kclpp_ctx *c, const kclpp_graph *gc, int k, const double *rho_dev, uint64_t *cnt_dev) {
  if (!c || !gc || ((!rho_dev || !cnt_dev) && gc->dag.n)) return set_error(KCLPP_ERR_INVALID, "null argument");
  KCL_TRY(check_k(k, 2));
  KCL_TRY(set_device(c));
  kclpp_graph *g = const_cast<kclpp_graph *>(gc);
  if (!g->dag.n) return KCLPP_OK;
  return sim_counts_dev(c, g, k, rho_dev, (unsigned long long *)cnt_dev);
}

kclpp_status kclpp_sim_update_dev(kclpp_ctx *c, uint32_t n, uint32_t t, double *rho_dev, const uint64_t *cnt_dev) {
  if (!c || ((!rho_dev || !cnt_dev) && n) || t < 1) return set_error(KCLPP_ERR_INVALID, "bad argument");
  KCL_TRY(set_device(c));
  if (!n) return KCLPP_OK;
  k_sim_update<<<blocks_for(n), 256, 0, c->stream>>>(rho_dev, (const unsigned long long *)cnt_dev, n, t);
  KCL_CUDA(cudaGetLastError());
  c->launches++;
  return KCLPP_OK;
}

// ---- schedule knobs and the autotuner ----------------------------------------------------
static kclpp_status check_schedule(const kclpp_schedule *sp) {
  for (int i = 0; i < 4; ++i) {
    const uint32_t w = sp->seq_warps[i];
    if (w != 0 && w != 2 && (w < 4 || w > (uint32_t)kWarpsMSeqMax || w % 4))
      return set_error(KCLPP_ERR_INVALID, "seq_warps entries must be 0 or one of 2, 4, 8, 12, 16, 20, 24");
    const uint32_t v = sp->count_warps[i];
    if (v != 0 && (v < 8 || v > (uint32_t)kWarpsMMax || v % 8))
      return set_error(KCLPP_ERR_INVALID, "count_warps entries must be 0 or one of 8, 16, 24, 32");
  }
  if (sp->seq_waves < 1 || sp->seq_waves > 1024)
    return set_error(KCLPP_ERR_INVALID, "seq_waves must be in [1, 1024]");
  if (sp->tier_s_max > kTierSMax || sp->tier_s_max_seq > kTierSMax || sp->m_split1 < sp->tier_s_max ||
      sp->m_split2 < sp->m_split1 || sp->m_split2 > kTierMMax || sp->seq_split1 < sp->tier_s_max_seq ||
      sp->seq_split2 < sp->seq_split1 || sp->seq_split2 > kTierMMax)
    return set_error(KCLPP_ERR_INVALID, "schedule bounds out of range (tier S <= %u <= split1 <= split2 <= %u)",
                     kTierSMax, kTierMMax);
  return KCLPP_OK;
}

kclpp_status kclpp_graph_get_schedule(const kclpp_graph *g, kclpp_schedule *sp) {
  if (!g || !sp) return set_error(KCLPP_ERR_INVALID, "null argument");
  *sp = g->sp;
  return KCLPP_OK;
}

kclpp_status kclpp_graph_set_schedule(kclpp_ctx *c, kclpp_graph *g, const kclpp_schedule *sp) {
  if (!c || !g || !sp) return set_error(KCLPP_ERR_INVALID, "null argument");
  KCL_TRY(check_schedule(sp));
  KCL_TRY(set_device(c));
  g->sp = *sp;
  cudaFree(g->d_roots);
  g->d_roots = nullptr;
  KCL_TRY(build_schedule(c, g));
  KCL_CUDA(cudaStreamSynchronize(c->stream));
  return KCLPP_OK;
}

// One pass of `mode`, timed with events on the context's stream: Seq from
// the vector one pass from zero leaves (the first pass, all ties, is not
// typical of a run), the counting kernels from a zero vector.
static kclpp_status time_pass(kclpp_ctx *c, kclpp_graph *g, int k, int mode, float *ms) {
  const size_t bytes = (size_t)g->dag.n * 8;
  cudaEvent_t e0 = take_event(c), e1 = take_event(c);
  if (!e0 || !e1) return set_error(KCLPP_ERR_CUDA, "event creation failed");
  for (int rep = 0; rep < 2; ++rep) {  // the first run warms caches and loads the kernel
    if (mode == dev::MODE_SEQ) {
      KCL_CUDA(cudaMemsetAsync(g->d_a, 0, bytes, c->stream));
      KCL_TRY(seq_pass_dev(c, g, k, g->d_a, g->d_b));
      KCL_CUDA(cudaEventRecord(e0, c->stream));
      KCL_TRY(seq_pass_dev(c, g, k, g->d_b, g->d_a));
    } else {
      KCL_CUDA(cudaMemsetAsync(g->d_rho, 0, bytes, c->stream));
      KCL_CUDA(cudaEventRecord(e0, c->stream));
      KCL_TRY(sim_counts_dev(c, g, k, g->d_rho, g->d_a));
    }
    KCL_CUDA(cudaEventRecord(e1, c->stream));
  }
  KCL_CUDA(cudaEventSynchronize(e1));
  KCL_CUDA(cudaEventElapsedTime(ms, e0, e1));
  c->event_pool.push_back(e0);
  c->event_pool.push_back(e1);
  return check_err(c);
}

// Per-launch times of one pass of `mode` (after a warm-up pass), in launch
// order: the per-launch events of the profiler, kept apart from the caller's.
static kclpp_status time_tiers(kclpp_ctx *c, kclpp_graph *g, int k, int mode, std::vector<float> &ms) {
  const size_t bytes = (size_t)g->dag.n * 8;
  std::vector<PendingTime> saved;
  saved.swap(c->pending);
  const bool was = c->profile;
  kclpp_status st = KCLPP_OK;
  for (int rep = 0; rep < 2 && st == KCLPP_OK; ++rep) {
    for (auto &p : c->pending) { c->event_pool.push_back(p.a); c->event_pool.push_back(p.b); }
    c->pending.clear();
    c->profile = rep == 1;
    if (mode == dev::MODE_SEQ) {
      // the timed pass (rep 1) starts from one pass's result, as in time_pass
      if (rep == 0 && cudaMemsetAsync(g->d_a, 0, bytes, c->stream) != cudaSuccess)
        st = set_error(KCLPP_ERR_CUDA, "memset failed");
      if (st == KCLPP_OK) st = rep == 0 ? seq_pass_dev(c, g, k, g->d_a, g->d_b) : seq_pass_dev(c, g, k, g->d_b, g->d_a);
    } else {
      if (cudaMemsetAsync(g->d_rho, 0, bytes, c->stream) != cudaSuccess) st = set_error(KCLPP_ERR_CUDA, "memset failed");
      if (st == KCLPP_OK) st = sim_counts_dev(c, g, k, g->d_rho, g->d_a);
    }
  }
  c->profile = was;
  if (st == KCLPP_OK && cudaStreamSynchronize(c->stream) != cudaSuccess) st = set_error(KCLPP_ERR_CUDA, "sync failed");
  ms.clear();
  for (auto &p : c->pending) {
    float t = 0.f;
    if (st == KCLPP_OK) cudaEventElapsedTime(&t, p.a, p.b);
    ms.push_back(t);
    c->event_pool.push_back(p.a);
    c->event_pool.push_back(p.b);
  }
  c->pending.swap(saved);
  if (st != KCLPP_OK) return st;
  return check_err(c);
}

kclpp_status kclpp_autotune(kclpp_ctx *c, kclpp_graph *g, int k, int kernel, kclpp_tune_result *out) {
  if (!c || !g || !out) return set_error(KCLPP_ERR_INVALID, "null argument");
  KCL_TRY(check_unsharded(g, "kclpp_autotune"));
  if (kernel != KCLPP_KERNEL_SEQ && kernel != KCLPP_KERNEL_ORDER)
    return set_error(KCLPP_ERR_INVALID, "autotune: kernel must be KCLPP_KERNEL_SEQ or KCLPP_KERNEL_ORDER");
  KCL_TRY(check_k(k, kernel == KCLPP_KERNEL_SEQ ? 3 : 2));
  KCL_TRY(set_device(c));
  memset(out, 0, sizeof *out);
  const int mode = kernel == KCLPP_KERNEL_SEQ ? dev::MODE_SEQ : dev::MODE_ORDER;
  const kclpp_schedule base = g->sp;
  std::vector<kclpp_schedule> cand;
  const uint32_t smax[3] = {8, 16, 32};
  const uint32_t smax_count[2] = {32, 64};
  const uint32_t splits[4][2] = {{256, 512}, {320, 640}, {384, 768}, {448, 896}};
  for (int sp = 0; sp < 4; ++sp)
    for (int st = 0; st < 2; ++st) {
      if (mode == dev::MODE_SEQ) {
        for (uint32_t sm : smax) {
          kclpp_schedule x = base;
          x.tier_s_max_seq = sm;
          x.seq_split1 = splits[sp][0];
          x.seq_split2 = splits[sp][1];
          x.steal_seq = st == 0;
          cand.push_back(x);
        }
      } else {
        for (uint32_t sm : smax_count) {
          kclpp_schedule x = base;
          x.tier_s_max = sm;
          x.m_split1 = splits[sp][0];
          x.m_split2 = splits[sp][1];
          x.steal_count = st;
          cand.push_back(x);
        }
      }
    }
  float best = 1e30f, def = 0.f;
  kclpp_schedule best_sp = base;
  {
    float ms = 0.f;
    KCL_TRY(time_pass(c, g, k, mode, &ms));
    def = ms;
    best = ms;
  }
  for (const kclpp_schedule &x : cand) {
    KCL_TRY(kclpp_graph_set_schedule(c, g, &x));
    float ms = 0.f;
    KCL_TRY(time_pass(c, g, k, mode, &ms));
    if (ms < best) { best = ms; best_sp = x; }
  }
  {
    // Warps per CTA, chosen per root group: the groups run as separate
    // launches, so each one's width is tuned on its own launch time.
    const bool sq = mode == dev::MODE_SEQ;
    const uint32_t seq_w[7] = {2, 4, 8, 12, 16, 20, 24}, cnt_w[4] = {8, 16, 24, 32};
    const uint32_t *widths = sq ? seq_w : cnt_w;
    const int nwid = sq ? 7 : 4;
    float bt[4] = {1e30f, 1e30f, 1e30f, 1e30f};
    kclpp_schedule tuned = best_sp;
    bool any = false;
    for (int wi = 0; wi < nwid; ++wi) {
      const uint32_t w = widths[wi];
      kclpp_schedule x = best_sp;
      (sq ? x.concurrent_tiers : x.concurrent_count) = 0;  // each group's own launch time
      for (int b = 0; b < 4; ++b) (sq ? x.seq_warps : x.count_warps)[b] = w;
      KCL_TRY(kclpp_graph_set_schedule(c, g, &x));
      std::vector<float> ms;
      KCL_TRY(time_tiers(c, g, k, mode, ms));
      const std::vector<TierInfo> &tiers = g->tiers[sq ? 1 : 0];
      for (size_t i = 0; i < tiers.size() && i < ms.size(); ++i) {
        const int b = tiers[i].bucket;
        if (b >= 0 && ms[i] < bt[b]) {
          bt[b] = ms[i];
          (sq ? tuned.seq_warps : tuned.count_warps)[b] = w;
          any = true;
        }
      }
    }
    if (any) {
      KCL_TRY(kclpp_graph_set_schedule(c, g, &tuned));
      float ms = 0.f;
      KCL_TRY(time_pass(c, g, k, mode, &ms));
      if (ms < best) { best = ms; best_sp = tuned; }
    }
  }
  {
    // Root groups side by side or one after another.
    kclpp_schedule x = best_sp;
    if (mode == dev::MODE_SEQ) x.concurrent_tiers = !best_sp.concurrent_tiers;
    else x.concurrent_count = !best_sp.concurrent_count;
    KCL_TRY(kclpp_graph_set_schedule(c, g, &x));
    float ms = 0.f;
    KCL_TRY(time_pass(c, g, k, mode, &ms));
    if (ms < best) { best = ms; best_sp = x; }
  }
  KCL_TRY(kclpp_graph_set_schedule(c, g, &best_sp));
  out->best = best_sp;
  out->best_ms = best;
  out->default_ms = def;
  out->candidates = (int)cand.size() + 2 + (mode == dev::MODE_SEQ ? 8 : 5);
  return KCLPP_OK;
}

// ---- batches: many graphs and several k values in one captured CUDA graph -----------------
}  // extern "C"

struct BatchBranch {
  int k = 0;
  cudaStream_t st = nullptr;
  cudaEvent_t join = nullptr;
  uint32_t *work = nullptr, *task = nullptr;
  unsigned long long *buf[2] = {nullptr, nullptr};  // Seq ping-pong, or Sim counts in buf[0]
  double *rho = nullptr;
  void *result = nullptr;  // device vector holding the branch's final r / rho
};

struct kclpp_batch {
  kclpp_graph *g = nullptr;
  std::vector<uint32_t> voff;  // per graph: first vertex in the union
  std::vector<BatchBranch> br;
  cudaEvent_t fork = nullptr;
  cudaGraphExec_t exec = nullptr;
  int exec_kernel = -1;
  std::vector<int> exec_ks;
  uint32_t exec_passes = 0;
  kclpp_schedule exec_sched{};  // the union graph's schedule when the graph was captured
};

static void batch_release(kclpp_batch *b) {
  for (auto &x : b->br) {
    if (x.st) cudaStreamDestroy(x.st);
    if (x.join) cudaEventDestroy(x.join);
    cudaFree(x.work); cudaFree(x.task); cudaFree(x.buf[0]); cudaFree(x.buf[1]); cudaFree(x.rho);
  }
  b->br.clear();
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
}

extern "C" {

kclpp_status kclpp_batch_create(kclpp_ctx *c, const kclpp_edge_list *const *els, uint32_t count, kclpp_batch **out) {
  if (!c || !out || (!els && count)) return set_error(KCLPP_ERR_INVALID, "null argument");
  *out = nullptr;
  KCL_TRY(set_device(c));
  auto *g = new kclpp_graph();
  std::vector<uint32_t> voff(1, 0);
  uint64_t m = 0;
  std::vector<HostDag> dags(count);
  for (uint32_t i = 0; i < count; ++i) {
    if (!els[i]) { delete g; return set_error(KCLPP_ERR_INVALID, "batch: null edge list %u", i); }
    std::vector<uint32_t> rank(els[i]->n);
    core_order_host(els[i]->n, els[i]->pairs, rank.data());
    kclpp_status s = make_dag_host(els[i]->pairs, rank.data(), dags[i]);
    if (s != KCLPP_OK) { delete g; return s; }
    if ((uint64_t)voff.back() + dags[i].n > UINT32_MAX) { delete g; return set_error(KCLPP_ERR_UNSUPPORTED, "batch: more than 2^32 vertices"); }
    voff.push_back(voff.back() + dags[i].n);
    m += dags[i].m();
  }
  // Disjoint union: graph i's vertices are shifted by voff[i]; every row stays
  // ascending and below its source, so the union is a DAG of the same kind.
  HostDag &U = g->dag;
  U.n = voff.back();
  U.off.assign((size_t)U.n + 1, 0);
  U.cols.resize(m);
  uint64_t at = 0;
  uint32_t core = 0;
  for (uint32_t i = 0; i < count; ++i) {
    const HostDag &D = dags[i];
    for (uint32_t s = 0; s < D.n; ++s) {
      U.off[voff[i] + s] = at;
      for (uint64_t e = D.off[s]; e < D.off[s + 1]; ++e) U.cols[at++] = D.cols[e] + voff[i];
    }
    core = std::max(core, D.core);
  }
  U.off[U.n] = at;
  U.core = core;
  kclpp_graph *gg = nullptr;
  KCL_TRY(finish_graph(c, g, &gg));
  auto *b = new kclpp_batch();
  b->g = gg;
  b->voff = std::move(voff);
  *out = b;
  return KCLPP_OK;
}

kclpp_status kclpp_batch_info(const kclpp_batch *b, uint32_t *graphs, uint32_t *total_n, uint64_t *total_m,
                              kclpp_graph **union_graph) {
  if (!b) return set_error(KCLPP_ERR_INVALID, "null batch");
  if (graphs) *graphs = (uint32_t)b->voff.size() - 1;
  if (total_n) *total_n = b->g->dag.n;
  if (total_m) *total_m = b->g->dag.m();
  if (union_graph) *union_graph = b->g;
  return KCLPP_OK;
}

kclpp_status kclpp_batch_vertex_offsets(const kclpp_batch *b, uint32_t *offsets) {
  if (!b || !offsets) return set_error(KCLPP_ERR_INVALID, "null argument");
  memcpy(offsets, b->voff.data(), b->voff.size() * 4);
  return KCLPP_OK;
}

// Record every branch's passes on its own stream (inside or outside a capture).
static kclpp_status batch_record(kclpp_ctx *c, kclpp_batch *b, int kernel, uint32_t passes) {
  kclpp_graph *g = b->g;
  const uint32_t n = g->dag.n;
  KCL_CUDA(cudaEventRecord(b->fork, c->stream));
  for (auto &x : b->br) {
    KCL_CUDA(cudaStreamWaitEvent(x.st, b->fork, 0));
    const Exec E{x.st, x.work, x.task};
    if (kernel == KCLPP_KERNEL_SEQ) {
      KCL_CUDA(cudaMemsetAsync(x.buf[0], 0, (size_t)n * 8, x.st));
      int cur = 0;
      for (uint32_t p = 0; p < passes; ++p) {
        KCL_CUDA(cudaMemcpyAsync(x.buf[cur ^ 1], x.buf[cur], (size_t)n * 8, cudaMemcpyDeviceToDevice, x.st));
        dev::PassArgs a{};
        a.r_in = x.buf[cur];
        a.out = x.buf[cur ^ 1];
        KCL_TRY(run_tiers(c, g, dev::MODE_SEQ, x.k, a, &E));
        cur ^= 1;
      }
      x.result = x.buf[cur];
    } else {
      KCL_CUDA(cudaMemsetAsync(x.rho, 0, (size_t)n * 8, x.st));
      for (uint32_t p = 0; p < passes; ++p) {
        KCL_CUDA(cudaMemsetAsync(x.buf[0], 0, (size_t)n * 8, x.st));
        dev::PassArgs a{};
        a.key_kind = dev::KEY_SIM;
        a.rho = x.rho;
        a.out = x.buf[0];
        KCL_TRY(run_tiers(c, g, dev::MODE_ORDER, x.k, a, &E));
        k_sim_update<<<blocks_for(n), 256, 0, x.st>>>(x.rho, x.buf[0], n, p + 1);
        KCL_CUDA(cudaGetLastError());
        c->launches++;
      }
      x.result = x.rho;
    }
    KCL_CUDA(cudaEventRecord(x.join, x.st));
    KCL_CUDA(cudaStreamWaitEvent(c->stream, x.join, 0));
  }
  return KCLPP_OK;
}

kclpp_status kclpp_batch_run(kclpp_ctx *c, kclpp_batch *b, int kernel, const int *ks, int nk, uint32_t passes,
                             void *out) {
  if (!c || !b || !ks || nk <= 0 || (!out && b->g->dag.n)) return set_error(KCLPP_ERR_INVALID, "null argument");
  if (kernel != KCLPP_KERNEL_SEQ && kernel != KCLPP_KERNEL_ORDER)
    return set_error(KCLPP_ERR_INVALID, "batch: kernel must be KCLPP_KERNEL_SEQ or KCLPP_KERNEL_ORDER (Sim)");
  for (int i = 0; i < nk; ++i) KCL_TRY(check_k(ks[i], kernel == KCLPP_KERNEL_SEQ ? 3 : 2));
  KCL_TRY(set_device(c));
  kclpp_graph *g = b->g;
  const uint32_t n = g->dag.n;
  if (!n) return KCLPP_OK;
  const std::vector<int> want(ks, ks + nk);
  // A schedule set on the union graph since the capture (kclpp_autotune,
  // kclpp_graph_set_schedule) changes the launches: capture again.
  const bool same = b->exec && b->exec_kernel == kernel && b->exec_ks == want && b->exec_passes == passes &&
                    memcmp(&b->exec_sched, &g->sp, sizeof g->sp) == 0;
  if (!same) {
    batch_release(b);
    if (!b->fork) KCL_CUDA(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    b->br.resize(nk);
    for (int i = 0; i < nk; ++i) {
      BatchBranch &x = b->br[i];
      x.k = ks[i];
      KCL_CUDA(cudaStreamCreateWithFlags(&x.st, cudaStreamNonBlocking));
      KCL_CUDA(cudaEventCreateWithFlags(&x.join, cudaEventDisableTiming));
      KCL_TRY(dalloc(&x.work, kWorkWords));
      KCL_TRY(dalloc(&x.task, std::max<uint32_t>(g->num_roots, 1)));
      KCL_TRY(dalloc(&x.buf[0], n));
      if (kernel == KCLPP_KERNEL_SEQ) KCL_TRY(dalloc(&x.buf[1], n));
      else KCL_TRY(dalloc(&x.rho, n));
    }
    // One run outside the capture settles the kernels' launch settings.
    KCL_TRY(batch_record(c, b, kernel, std::min<uint32_t>(passes, 1)));
    KCL_CUDA(cudaStreamSynchronize(c->stream));
    cudaGraph_t graph = nullptr;
    KCL_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed));
    kclpp_status rs = batch_record(c, b, kernel, passes);
    cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
    if (rs != KCLPP_OK) { if (graph) cudaGraphDestroy(graph); return rs; }
    if (ce != cudaSuccess) return set_error(KCLPP_ERR_CUDA, "batch capture: %s", cudaGetErrorString(ce));
    ce = cudaGraphInstantiate(&b->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) return set_error(KCLPP_ERR_CUDA, "batch instantiate: %s", cudaGetErrorString(ce));
    b->exec_kernel = kernel;
    b->exec_ks = want;
    b->exec_passes = passes;
    b->exec_sched = g->sp;
  }
  KCL_CUDA(cudaGraphLaunch(b->exec, c->stream));
  c->launches++;
  for (int i = 0; i < nk; ++i)
    KCL_CUDA(cudaMemcpyAsync((char *)out + (size_t)i * n * 8, b->br[i].result, (size_t)n * 8,
                             cudaMemcpyDeviceToHost, c->stream));
  return check_err(c);
}

void kclpp_batch_free(kclpp_batch *b) {
  if (!b) return;
  batch_release(b);
  if (b->fork) cudaEventDestroy(b->fork);
  kclpp_graph_free(b->g);
  delete b;
}

// ---- sort, PAVA, densest prefix ------------------------------------------------------
kclpp_status kclpp_sort_by_r_u64(kclpp_ctx *c, uint32_t n, const uint64_t *r, uint32_t *reordered, uint32_t *level) {
  (void)c;
  if (!r && n) return set_error(KCLPP_ERR_INVALID, "null r");
  std::vector<KeyId> v(n);
  for (uint32_t i = 0; i < n; ++i) v[i] = {r[i], i};
  sort_desc(n, v, reordered, level);
  return KCLPP_OK;
}

kclpp_status kclpp_sort_by_r_f64(kclpp_ctx *c, uint32_t n, const double *r, uint32_t *reordered, uint32_t *level) {
  (void)c;
  if (!r && n) return set_error(KCLPP_ERR_INVALID, "null r");
  std::vector<KeyId> v(n);
  for (uint32_t i = 0; i < n; ++i) v[i] = {(uint64_t)(unsigned long long)r[i], i};  // (unsigned long long)rho
  sort_desc(n, v, reordered, level);
  return KCLPP_OK;
}

kclpp_status kclpp_pava(kclpp_ctx *c, const kclpp_graph *gc, int k, const uint32_t *level, uint64_t *tentative) {
  if (!c || !gc || ((!level || !tentative) && gc->dag.n)) return set_error(KCLPP_ERR_INVALID, "null argument");
  KCL_TRY(check_unsharded(gc, "kclpp_pava"));
  KCL_TRY(check_k(k, 2));
  KCL_TRY(set_device(c));
  kclpp_graph *g = const_cast<kclpp_graph *>(gc);
  const uint32_t n = g->dag.n;
  if (!n) return KCLPP_OK;
  KCL_CUDA(cudaMemcpyAsync(g->d_level, level, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
  KCL_TRY(pava_dev(c, g, k, g->d_level, g->d_b));
  KCL_CUDA(cudaMemcpyAsync(tentative, g->d_b, (size_t)n * 8, cudaMemcpyDeviceToHost, c->stream));
  return check_err(c);
}

kclpp_status kclpp_count_edges(kclpp_ctx *c, const kclpp_graph *gc, uint32_t num_nodes, const uint32_t *nodes,
                               uint32_t *m_out) {
  if (!c || !gc || !m_out || (!nodes && num_nodes)) return set_error(KCLPP_ERR_INVALID, "null argument");
  KCL_TRY(set_device(c));
  kclpp_graph *g = const_cast<kclpp_graph *>(gc);
  const uint32_t n = g->dag.n;
  // level[v] = position among nodes (n for vertices not listed); CountEdges
  // then keeps the edges with both ends below num_nodes.
  std::vector<uint32_t> lv(n, UINT32_MAX);
  for (uint32_t i = 0; i < num_nodes; ++i) {
    if (nodes[i] >= n) return set_error(KCLPP_ERR_INVALID, "node id %u out of range", nodes[i]);
    lv[nodes[i]] = 0;
  }
  if (!n) { *m_out = 0; return KCLPP_OK; }
  KCL_CUDA(cudaMemcpyAsync(g->d_level, lv.data(), (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
  KCL_CUDA(cudaMemsetAsync(g->d_scalar, 0, 8, c->stream));
  const uint64_t m = g->dag.m();
  if (m) {
    k_count_edges<<<std::min(blocks_for(m), c->num_sms * 8), 256, 0, c->stream>>>(g->d_src, g->d_cols, m,
                                                                               g->d_level, 1u, g->d_scalar);
    KCL_CUDA(cudaGetLastError());
    c->launches++;
  }
  unsigned long long h = 0;
  KCL_CUDA(cudaMemcpyAsync(&h, g->d_scalar, 8, cudaMemcpyDeviceToHost, c->stream));
  KCL_TRY(check_err(c));
  *m_out = (uint32_t)h;
  return KCLPP_OK;
}

// Shared tail of both extractions: PAVA pass on the device, CountEdges.
static kclpp_status pava_and_edges(kclpp_ctx *c, kclpp_graph *g, int k, const std::vector<uint32_t> &level,
                                   std::vector<uint64_t> &tent) {
  const uint32_t n = g->dag.n;
  KCL_CUDA(cudaMemcpyAsync(g->d_level, level.data(), (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
  KCL_TRY(pava_dev(c, g, k, g->d_level, g->d_b));
  tent.resize(n);
  KCL_CUDA(cudaMemcpyAsync(tent.data(), g->d_b, (size_t)n * 8, cudaMemcpyDeviceToHost, c->stream));
  return check_err(c);
}

static kclpp_status edges_in_prefix(kclpp_ctx *c, kclpp_graph *g, uint32_t nstar, uint32_t *m_out) {
  KCL_CUDA(cudaMemsetAsync(g->d_scalar, 0, 8, c->stream));
  const uint64_t m = g->dag.m();
  if (m) {
    k_count_edges<<<std::min(blocks_for(m), c->num_sms * 8), 256, 0, c->stream>>>(g->d_src, g->d_cols, m,
                                                                               g->d_level, nstar, g->d_scalar);
    KCL_CUDA(cudaGetLastError());
    c->launches++;
  }
  unsigned long long h = 0;
  KCL_CUDA(cudaMemcpyAsync(&h, g->d_scalar, 8, cudaMemcpyDeviceToHost, c->stream));
  KCL_TRY(check_err(c));
  *m_out = (uint32_t)h;
  return KCLPP_OK;
}

extern "C++" {
// The upper bound of kCDensestNoAtom.c:352-369 (Seq) and kCDensestCmpSync.c:
// 365-381 (Sim): walk the vertices in load order, the running binomial
// C(i+1, k) against the prefix's load; next_load(i) adds the i-th vertex and
// returns the prefix load as the reference computes it (Seq: the integer sum
// divided by T; Sim: the FP64 sum), so the FP operations are the reference's.
template <typename NextLoad>
static double upper_bound_scan(uint32_t n, int k, NextLoad next_load) {
  double ub = 0, ip1ck = 1;
  for (uint32_t i = 0; i < n; ++i) {
    const double load = next_load(i);
    if (i + 1 == (uint32_t)k) ip1ck = 1;
    else if (i + 1 > (uint32_t)k) ip1ck = (ip1ck * (i + 1)) / (i + 1 - k);
    if (ip1ck < load) ub = ip1ck / (i + 1);
    else {
      if (ub < load / (i + 1)) ub = load / (i + 1);
      break;
    }
  }
  return ub;
}

// kCDensestNoAtom.c:342-349: the first strictly largest prefix density of the
// exact prefix clique counts (integer accumulator).
static void densest_prefix_u64(const std::vector<uint64_t> &tent, kclpp_densest_info *info) {
  double density = -1;
  unsigned long long sum = 0;
  for (uint32_t i = 0; i < (uint32_t)tent.size(); ++i) {
    sum += tent[i];
    if ((double)sum / (i + 1) > density) {
      density = (double)sum / (i + 1);
      info->n = i + 1;
      info->cliques = sum;
    }
  }
  info->density = density;
}
}  // extern "C++"

kclpp_status kclpp_extract_densest_seq(kclpp_ctx *c, const kclpp_graph *gc, int k, uint32_t T, const uint64_t *r,
                                       kclpp_densest_info *info, uint32_t *reordered_out) {
  if (!c || !gc || !info || (!r && gc->dag.n)) return set_error(KCLPP_ERR_INVALID, "null argument");
  KCL_TRY(check_unsharded(gc, "kclpp_extract_densest_seq"));
  KCL_TRY(check_k(k, 3));
  if (T < 1) return set_error(KCLPP_ERR_INVALID, "T must be >= 1");
  KCL_TRY(set_device(c));
  kclpp_graph *g = const_cast<kclpp_graph *>(gc);
  memset(info, 0, sizeof *info);
  const uint32_t n = g->dag.n;
  if (!n) return KCLPP_OK;
  std::vector<uint32_t> reordered(n), level(n);
  KCL_TRY(kclpp_sort_by_r_u64(c, n, r, reordered.data(), level.data()));
  std::vector<uint64_t> tent;
  KCL_TRY(pava_and_edges(c, g, k, level, tent));
  densest_prefix_u64(tent, info);
  KCL_TRY(edges_in_prefix(c, g, info->n, &info->m));
  unsigned long long sum = 0;
  info->ub = upper_bound_scan(n, k, [&](uint32_t i) {
    sum += r[reordered[i]];
    return (double)sum / T;
  });
  if (reordered_out) memcpy(reordered_out, reordered.data(), (size_t)n * 4);
  return KCLPP_OK;
}

kclpp_status kclpp_extract_densest_sim(kclpp_ctx *c, const kclpp_graph *gc, int k, const double *rho,
                                       kclpp_densest_info *info, uint32_t *reordered_out) {
  if (!c || !gc || !info || (!rho && gc->dag.n)) return set_error(KCLPP_ERR_INVALID, "null argument");
  KCL_TRY(check_unsharded(gc, "kclpp_extract_densest_sim"));
  KCL_TRY(check_k(k, 2));
  KCL_TRY(set_device(c));
  kclpp_graph *g = const_cast<kclpp_graph *>(gc);
  memset(info, 0, sizeof *info);
  const uint32_t n = g->dag.n;
  if (!n) return KCLPP_OK;
  std::vector<uint32_t> reordered(n), level(n);
  KCL_TRY(kclpp_sort_by_r_f64(c, n, rho, reordered.data(), level.data()));
  std::vector<uint64_t> tent;
  KCL_TRY(pava_and_edges(c, g, k, level, tent));
  // kCDensestCmpSync.c:354-361 (double accumulator)
  double density = -1, sum = 0;
  uint64_t isum = 0;
  for (uint32_t i = 0; i < n; ++i) {
    sum += (double)tent[i];
    isum += tent[i];
    if (sum / (i + 1) > density) {
      density = sum / (i + 1);
      info->n = i + 1;
      info->cliques = isum;
    }
  }
  info->density = density;
  KCL_TRY(edges_in_prefix(c, g, info->n, &info->m));
  sum = 0;
  info->ub = upper_bound_scan(n, k, [&](uint32_t i) {
    sum += rho[reordered[i]];
    return sum;
  });
  if (reordered_out) memcpy(reordered_out, reordered.data(), (size_t)n * 4);
  return KCLPP_OK;
}

// ---- whole runs ------------------------------------------------------------------------
kclpp_status kclpp_seq_main(kclpp_ctx *c, const kclpp_graph *gc, int k, uint32_t num_iter, int det_mode,
                            uint64_t *r_out, kclpp_densest_info *infos, int max_infos, int *n_infos) {
  if (!c || !gc) return set_error(KCLPP_ERR_INVALID, "null argument");
  KCL_TRY(check_unsharded(gc, "kclpp_seq_main"));
  KCL_TRY(check_k(k, 3));
  if (!valid_seq_mode(det_mode)) return set_error(KCLPP_ERR_INVALID, "unknown det_mode %d", det_mode);
  KCL_TRY(set_device(c));
  kclpp_graph *g = const_cast<kclpp_graph *>(gc);
  const uint32_t n = g->dag.n;
  std::vector<uint64_t> r(n, 0);
  int made = 0;
  unsigned long long *dr = nullptr;
  KCL_CUDA(cudaMalloc((void **)&dr, std::max<size_t>((size_t)n * 8, 8)));
  std::unique_ptr<unsigned long long, decltype(&cudaFree)> guard(dr, &cudaFree);
  if (n) KCL_CUDA(cudaMemsetAsync(dr, 0, (size_t)n * 8, c->stream));
  for (uint32_t T = 1, t = 1; T <= num_iter; T <<= 1) {
    if (T > t - 1) {
      KCL_TRY(seq_passes_on(c, g, k, T - (t - 1), dr, det_mode));
      t = T + 1;
    }
    if (n) KCL_CUDA(cudaMemcpyAsync(r.data(), dr, (size_t)n * 8, cudaMemcpyDeviceToHost, c->stream));
    KCL_TRY(check_err(c));
    kclpp_densest_info info;
    KCL_TRY(kclpp_extract_densest_seq(c, g, k, T, r.data(), &info, nullptr));
    if (infos && made < max_infos) infos[made] = info;
    ++made;
    if (T > (UINT32_MAX >> 1)) break;
  }
  if (r_out && n) memcpy(r_out, r.data(), (size_t)n * 8);
  if (n_infos) *n_infos = made;
  return KCLPP_OK;
}

kclpp_status kclpp_sim_main(kclpp_ctx *c, const kclpp_graph *gc, int k, uint32_t num_iter, double *rho_out,
                            kclpp_densest_info *infos, int max_infos, int *n_infos) {
  if (!c || !gc) return set_error(KCLPP_ERR_INVALID, "null argument");
  KCL_TRY(check_unsharded(gc, "kclpp_sim_main"));
  KCL_TRY(check_k(k, 2));
  KCL_TRY(set_device(c));
  kclpp_graph *g = const_cast<kclpp_graph *>(gc);
  const uint32_t n = g->dag.n;
  std::vector<double> rho(n, 0.0);
  int made = 0;
  if (n) KCL_CUDA(cudaMemsetAsync(g->d_rho, 0, (size_t)n * 8, c->stream));
  for (uint32_t T = 1, t = 1; T <= num_iter; T <<= 1) {
    for (; t <= T; ++t) KCL_TRY(sim_pass_dev(c, g, k, t, g->d_rho));
    if (n) KCL_CUDA(cudaMemcpyAsync(rho.data(), g->d_rho, (size_t)n * 8, cudaMemcpyDeviceToHost, c->stream));
    KCL_TRY(check_err(c));
    kclpp_densest_info info;
    KCL_TRY(kclpp_extract_densest_sim(c, g, k, rho.data(), &info, nullptr));
    if (infos && made < max_infos) infos[made] = info;
    ++made;
    if (T > (UINT32_MAX >> 1)) break;
  }
  if (rho_out && n) memcpy(rho_out, rho.data(), (size_t)n * 8);
  if (n_infos) *n_infos = made;
  return KCLPP_OK;
}

}  // extern "C"

// ---- context accessors for the other translation units ------------------------------------
namespace kclpp {
cudaStream_t ctx_stream(kclpp_ctx *c) { return c->stream; }
int ctx_device(kclpp_ctx *c) { return c->device; }
int ctx_sms(kclpp_ctx *c) { return c->num_sms; }
void ctx_count_launch(kclpp_ctx *c, int n) { c->launches += (uint64_t)n; }
uint32_t *ctx_err_word(kclpp_ctx *c) { return c->d_err; }
kclpp_status ctx_check_err(kclpp_ctx *c) { return check_err(c); }
const HostDag &graph_dag(const kclpp_graph *g) { return g->dag; }
const uint64_t *graph_dev_offsets(const kclpp_graph *g) { return g->d_off; }
const uint32_t *graph_dev_cols(const kclpp_graph *g) { return g->d_cols; }
int graph_device(const kclpp_graph *g) { return g->device; }
}  // namespace kclpp

// ---- learned warm start: graph-level pieces -------------------------------------------------
// Core numbers of the undirected graph behind a DAG (bucket peel, O(n + m)).
static void core_numbers_host(const HostDag &D, std::vector<uint32_t> &deg, std::vector<uint32_t> &core) {
  const uint32_t n = D.n;
  deg.assign(n, 0);
  for (uint32_t s = 0; s < n; ++s) {
    deg[s] += (uint32_t)(D.off[s + 1] - D.off[s]);
    for (uint64_t e = D.off[s]; e < D.off[s + 1]; ++e) deg[D.cols[e]]++;
  }
  std::vector<uint64_t> cu((size_t)n + 1, 0);
  for (uint32_t v = 0; v < n; ++v) cu[v + 1] = cu[v] + deg[v];
  std::vector<uint32_t> adj(cu[n]);
  {
    std::vector<uint64_t> f(cu.begin(), cu.end() - 1);
    for (uint32_t s = 0; s < n; ++s)
      for (uint64_t e = D.off[s]; e < D.off[s + 1]; ++e) {
        adj[f[s]++] = D.cols[e];
        adj[f[D.cols[e]]++] = s;
      }
  }
  uint32_t md = 0;
  for (uint32_t v = 0; v < n; ++v) md = std::max(md, deg[v]);
  std::vector<uint32_t> cur(deg), bin((size_t)md + 2, 0), pos(n), vert(n);
  for (uint32_t v = 0; v < n; ++v) bin[cur[v]]++;
  uint32_t start = 0;
  for (uint32_t d = 0; d <= md; ++d) { uint32_t c = bin[d]; bin[d] = start; start += c; }
  for (uint32_t v = 0; v < n; ++v) { pos[v] = bin[cur[v]]; vert[pos[v]] = v; bin[cur[v]]++; }
  for (uint32_t d = md + 1; d >= 1; --d) bin[d] = bin[d - 1];
  bin[0] = 0;
  for (uint32_t i = 0; i < n; ++i) {
    const uint32_t v = vert[i];
    for (uint64_t e = cu[v]; e < cu[v + 1]; ++e) {
      const uint32_t u = adj[e];
      if (cur[u] > cur[v]) {
        const uint32_t du = cur[u], pu = pos[u], pw = bin[du], w = vert[pw];
        if (u != w) { pos[u] = pw; vert[pu] = w; pos[w] = pu; vert[pw] = u; }
        bin[du]++;
        cur[u]--;
      }
    }
  }
  core.swap(cur);
}

extern "C" {

kclpp_status kclpp_warm_features(kclpp_ctx *c, const kclpp_graph *gc, float *X_dev) {
  if (!c || !gc || (!X_dev && gc->dag.n)) return set_error(KCLPP_ERR_INVALID, "null argument");
  KCL_TRY(check_unsharded(gc, "kclpp_warm_features"));
  KCL_TRY(set_device(c));
  kclpp_graph *g = const_cast<kclpp_graph *>(gc);
  const uint32_t n = g->dag.n;
  if (!n) return KCLPP_OK;
  std::vector<uint32_t> deg, core;
  core_numbers_host(g->dag, deg, core);
  uint32_t *d_deg = nullptr, *d_core = nullptr;
  KCL_CUDA(cudaMalloc((void **)&d_deg, (size_t)n * 4));
  std::unique_ptr<uint32_t, decltype(&cudaFree)> g1(d_deg, &cudaFree);
  KCL_CUDA(cudaMalloc((void **)&d_core, (size_t)n * 4));
  std::unique_ptr<uint32_t, decltype(&cudaFree)> g2(d_core, &cudaFree);
  KCL_CUDA(cudaMemcpyAsync(d_deg, deg.data(), (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
  KCL_CUDA(cudaMemcpyAsync(d_core, core.data(), (size_t)n * 4, cudaMemcpyHostToDevice, c->stream));
  // triangles and 4-cliques per vertex with the count kernels
  for (int k = 3; k <= 4; ++k) {
    unsigned long long *out = k == 3 ? g->d_a : g->d_b;
    KCL_CUDA(cudaMemsetAsync(out, 0, (size_t)n * 8, c->stream));
    dev::PassArgs a{};
    a.out = out;
    KCL_TRY(run_tiers(c, g, dev::MODE_COUNT, k, a));
  }
  KCL_TRY(kclpp_warm_features_dev(c, n, d_deg, d_core, (const uint64_t *)g->d_a, (const uint64_t *)g->d_b, X_dev));
  KCL_CUDA(cudaStreamSynchronize(c->stream));
  return check_err(c);
}

kclpp_status kclpp_warm_start_r(kclpp_ctx *c, const kclpp_graph *gc, const kclpp_warm_model *M, float t0,
                                uint64_t *r0_dev) {
  if (!c || !gc || !M || (!r0_dev && gc->dag.n)) return set_error(KCLPP_ERR_INVALID, "null argument");
  KCL_TRY(set_device(c));
  const uint32_t n = gc->dag.n;
  if (!n) return KCLPP_OK;
  float *X = nullptr, *Y = nullptr;
  KCL_CUDA(cudaMalloc((void **)&X, (size_t)n * 16));
  std::unique_ptr<float, decltype(&cudaFree)> g1(X, &cudaFree);
  KCL_CUDA(cudaMalloc((void **)&Y, (size_t)n * 4));
  std::unique_ptr<float, decltype(&cudaFree)> g2(Y, &cudaFree);
  KCL_TRY(kclpp_warm_features(c, gc, X));
  KCL_TRY(kclpp_warm_predict_dev(c, M, X, n, Y));
  KCL_TRY(kclpp_warm_r0_dev(c, Y, n, t0, r0_dev));
  KCL_CUDA(cudaStreamSynchronize(c->stream));
  return check_err(c);
}

kclpp_status kclpp_extract_densest_seq_warm(kclpp_ctx *c, const kclpp_graph *gc, int k, uint32_t T,
                                            const uint64_t *r, const uint64_t *r0, kclpp_densest_info *info) {
  if (!c || !gc || !info || ((!r || !r0) && gc->dag.n)) return set_error(KCLPP_ERR_INVALID, "null argument");
  KCL_TRY(check_unsharded(gc, "kclpp_extract_densest_seq_warm"));
  KCL_TRY(check_k(k, 3));
  if (T < 1) return set_error(KCLPP_ERR_INVALID, "T must be >= 1");
  KCL_TRY(set_device(c));
  kclpp_graph *g = const_cast<kclpp_graph *>(gc);
  memset(info, 0, sizeof *info);
  const uint32_t n = g->dag.n;
  if (!n) return KCLPP_OK;
  // Densest prefix in the order of r (warm start included): the same scan as
  // kCDensestNoAtom.c:341-349 on exact prefix clique counts.
  std::vector<uint32_t> reordered(n), level(n);
  KCL_TRY(kclpp_sort_by_r_u64(c, n, r, reordered.data(), level.data()));
  std::vector<uint64_t> tent;
  KCL_TRY(pava_and_edges(c, g, k, level, tent));
  densest_prefix_u64(tent, info);
  KCL_TRY(edges_in_prefix(c, g, info->n, &info->m));
  // Upper bound from the loads the T passes added: (r - r0) / T is a feasible
  // fractional assignment of the cliques (every pass gives each clique one
  // unit), and the bound of kCDensestNoAtom.c:352-369 needs the loads in
  // descending order of the loads themselves.
  std::vector<uint64_t> inc(n);
  for (uint32_t i = 0; i < n; ++i) inc[i] = r[i] - r0[i];
  std::sort(inc.begin(), inc.end(), std::greater<uint64_t>());
  unsigned long long sum = 0;
  info->ub = upper_bound_scan(n, k, [&](uint32_t i) {
    sum += inc[i];
    return (double)sum / T;
  });
  return KCLPP_OK;
}

}  // extern "C"
