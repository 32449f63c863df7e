// kclpp_sample.cu -- Seq-Sampling++ on the GPU (kCDensestSamplingKclistpp.c):
// the clique sample kept in device memory, the "++" passes over it, and the
// report (densest prefix of the sampled loads, exact count inside it, bound).
//
// Sampling kernel: one CTA per root vertex s (persistent CTAs, roots by
// decreasing out-degree from an atomic counter).  The CTA loads N+(s) and the
// members' keys, builds G_s as bitmap rows (row i = the members of N+(s) that
// are out-neighbours of the i-th one) in shared memory -- or, for out-degrees
// whose rows do not fit, in a per-CTA global slab -- and its threads take the
// root edges (s, t) from a shared counter and walk each edge's clique tree
// depth first, one 32-bit word of the candidate set at a time.  A clique is
// kept when its key sum passes the threshold (kclpp_sample.cuh); kept rows are
// appended at an atomic cursor.  The order of the rows is therefore arbitrary,
// and nothing downstream depends on it.
//
// "++" pass: W waves (a fixed byte per kept clique).  Wave w: every clique of
// the wave adds one to delta[argmin] (values as the earlier waves left them),
// then rho += delta over all vertices.  Integer adds commute, so the result
// is the same for every schedule.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>
#include <vector>

#include <cuda_runtime.h>

#include "kclpp_internal.h"
#include "kclpp_sample.cuh"

using namespace kclpp;

#define SCUDA(call)                                                                           \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      return set_error(e_ == cudaErrorMemoryAllocation ? KCLPP_ERR_NOMEM : KCLPP_ERR_CUDA,    \
                       "%s: %s", #call, cudaGetErrorString(e_));                               \
  } while (0)

#define STRY(call)                         \
  do {                                     \
    kclpp_status s_ = (call);              \
    if (s_ != KCLPP_OK) return s_;         \
  } while (0)

namespace {

constexpr int kSampleThreads = 512;
constexpr uint32_t kSmallRoots = 128;  // out-degree bound of the first launch group
constexpr int kPassThreads = 256;

struct SampleArgs {
  const uint64_t *off;
  const uint32_t *cols;
  const uint32_t *roots;  // this group's roots
  uint32_t num_roots;
  uint32_t dmax;          // largest out-degree in the group
  uint32_t ws;            // words per bitmap row
  uint32_t *work;         // root counter (zeroed)
  uint32_t *slab;         // rows in global memory (nullptr: in shared memory)
  uint64_t slab_words;    // per CTA
  uint64_t seed, threshold;
  int all;
  uint32_t waves;
  uint32_t *rows;         // kept cliques, K ids each
  uint8_t *wave;
  unsigned long long cap;
  unsigned long long *count;
};

template <int K>
struct DevEmit {
  const uint32_t *list;
  uint32_t s;
  uint32_t *rows;
  uint8_t *wave;
  unsigned long long cap;
  unsigned long long *count;
  uint64_t threshold;
  bool all;
  uint32_t waves;
  __device__ __forceinline__ void operator()(uint64_t h, const uint32_t *path, uint32_t v) const {
    if (!smp::kept(h, threshold, all)) return;
    const unsigned long long pos = atomicAdd(count, 1ull);
    if (pos >= cap) return;  // counted only: the host grows the buffer and samples again
    smp::write_row<K>(rows + pos * K, list, s, path, v);
    wave[pos] = (uint8_t)smp::wave_of(h, waves);
  }
};

// Shared memory: keys (dmax u64), list (dmax u32), then the rows unless the
// launch gives a slab.
template <int K>
__global__ void __launch_bounds__(kSampleThreads) k_sample(SampleArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint64_t *keys = reinterpret_cast<uint64_t *>(smem);
  uint32_t *list = reinterpret_cast<uint32_t *>(keys + a.dmax);
  uint32_t *rows = a.slab ? a.slab + (size_t)blockIdx.x * a.slab_words : list + a.dmax;
  __shared__ uint32_t s_root, s_edge;
  for (;;) {
    if (threadIdx.x == 0) {
      s_root = atomicAdd(a.work, 1u);
      s_edge = 0;
    }
    __syncthreads();
    const uint32_t ri = s_root;
    if (ri >= a.num_roots) break;
    const uint32_t s = a.roots[ri];
    const uint64_t o = a.off[s];
    const uint32_t d = (uint32_t)(a.off[s + 1] - o);  // K - 1 <= d <= dmax (host)
    for (uint32_t i = threadIdx.x; i < d; i += blockDim.x) {
      const uint32_t x = a.cols[o + i];
      list[i] = x;
      keys[i] = smp::vertex_key(a.seed, x);
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < d; i += blockDim.x)
      smp::build_row(i, list, a.off, a.cols, rows + (size_t)i * a.ws);
    __syncthreads();
    DevEmit<K> em{list, s, a.rows, a.wave, a.cap, a.count, a.threshold, a.all != 0, a.waves};
    const uint64_t hs = smp::vertex_key(a.seed, s);
    for (;;) {
      const uint32_t t = atomicAdd(&s_edge, 1u);
      if (t >= d) break;
      if (t + 2 < (uint32_t)K) continue;  // row t holds fewer than K - 2 candidates
      smp::edge_cliques<K>(t, hs, rows, a.ws, keys, em);
    }
    __syncthreads();  // the next root overwrites list, keys, rows and s_root
  }
}

__global__ void k_wave(const uint32_t *rows, const uint8_t *wave, uint64_t n_rows, int k, uint32_t w,
                       const uint32_t *rho, uint32_t *delta) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n_rows; i += stride) {
    if (wave[i] != w) continue;
    atomicAdd(&delta[smp::argmin_member(rows + i * (uint64_t)k, k, rho)], 1u);
  }
}

__global__ void k_apply(uint32_t n, uint32_t *rho, uint32_t *delta) {
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const uint32_t d = delta[v];
    if (d) {
      rho[v] += d;
      delta[v] = 0;
    }
  }
}

__global__ void k_push(const uint32_t *rows, uint64_t n_rows, int k, const uint32_t *rank, uint32_t *push) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n_rows; i += stride)
    atomicAdd(&push[smp::max_rank(rows + i * (uint64_t)k, k, rank)], 1u);
}

template <typename T>
cudaError_t dalloc(T **p, size_t count) {
  return cudaMalloc((void **)p, std::max<size_t>(count, 1) * sizeof(T));
}

// Bytes of shared memory a sampling CTA needs at out-degree bound d, with or
// without the rows.
size_t sample_smem(uint32_t d, bool rows) {
  const size_t ws = (d + 31) / 32;
  return (size_t)d * 12 + (rows ? ws * d * 4 : 0);
}

}  // namespace

struct kclpp_sampling {
  const kclpp_graph *g = nullptr;
  int device = 0;
  int k = 0;
  uint32_t n = 0;
  uint64_t target = 0, seed = 0, total = 0, sampled = 0, threshold = 0, cap = 0;
  double prob = 1.0;
  int all = 1;
  uint32_t waves = 1, passes = 0;
  uint32_t *d_rows = nullptr;
  uint8_t *d_wave = nullptr;
  uint32_t *d_rho = nullptr, *d_delta = nullptr, *d_rank = nullptr, *d_push = nullptr;
  ~kclpp_sampling() {
    cudaSetDevice(device);
    for (void *p : {(void *)d_rows, (void *)d_wave, (void *)d_rho, (void *)d_delta, (void *)d_rank, (void *)d_push})
      if (p) cudaFree(p);
  }
};

namespace {

template <int K>
kclpp_status launch_groups(kclpp_ctx *c, kclpp_sampling *S, const SampleArgs &base,
                           const std::vector<uint32_t> &roots_by_degree, const uint32_t *d_roots, uint32_t *d_work,
                           const HostDag &D) {
  cudaStream_t st = ctx_stream(c);
  const int sms = ctx_sms(c);
  int optin = 0;
  SCUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, S->device));
  const size_t limit = (size_t)optin - 256;  // room for the static counters
  auto fn = k_sample<K>;
  SCUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit));
  auto deg = [&](uint32_t v) { return (uint32_t)(D.off[v + 1] - D.off[v]); };
  // Groups of roots by out-degree: > the largest whose rows fit shared memory
  // (rows in a slab), then up to that bound, then up to kSmallRoots.
  uint32_t d_fit = smp::kMaxDegree;
  while (d_fit > 0 && sample_smem(d_fit, true) > limit) --d_fit;
  const uint32_t nr = (uint32_t)roots_by_degree.size();
  uint32_t b1 = 0;
  while (b1 < nr && deg(roots_by_degree[b1]) > d_fit) ++b1;
  uint32_t b2 = b1;
  while (b2 < nr && deg(roots_by_degree[b2]) > kSmallRoots) ++b2;
  const uint32_t bounds[4] = {0, b1, b2, nr};
  // The slab is freed on every return path (cudaFree waits for the kernels).
  struct Slab {
    uint32_t *p = nullptr;
    ~Slab() {
      if (p) cudaFree(p);
    }
  } slab;
  for (int grp = 0; grp < 3; ++grp) {
    const uint32_t lo = bounds[grp], hi = bounds[grp + 1];
    if (lo == hi) continue;
    SampleArgs a = base;
    a.roots = d_roots + lo;
    a.num_roots = hi - lo;
    a.dmax = deg(roots_by_degree[lo]);
    a.ws = (a.dmax + 31) / 32;
    a.work = d_work + grp;
    const bool in_smem = grp > 0;
    const size_t smem = sample_smem(a.dmax, in_smem);
    int per_sm = 0;
    SCUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kSampleThreads, smem));
    if (per_sm < 1) return set_error(KCLPP_ERR_UNSUPPORTED, "sampling kernel does not fit (%zu B shared)", smem);
    const uint32_t grid = std::min<uint32_t>((uint32_t)per_sm * (uint32_t)sms, a.num_roots);
    if (!in_smem) {
      a.slab_words = (uint64_t)a.dmax * a.ws;
      SCUDA(dalloc(&slab.p, (size_t)grid * a.slab_words));
      a.slab = slab.p;
    }
    fn<<<grid, kSampleThreads, smem, st>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(KCLPP_ERR_CUDA, "sampling kernel: %s", cudaGetErrorString(e));
    ctx_count_launch(c, 1);
  }
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return set_error(KCLPP_ERR_CUDA, "sampling kernel: %s", cudaGetErrorString(e));
  return KCLPP_OK;
}

kclpp_status launch_k(int k, kclpp_ctx *c, kclpp_sampling *S, const SampleArgs &a, const std::vector<uint32_t> &r,
                      const uint32_t *d_roots, uint32_t *d_work, const HostDag &D) {
  switch (k) {
    case 3: return launch_groups<3>(c, S, a, r, d_roots, d_work, D);
    case 4: return launch_groups<4>(c, S, a, r, d_roots, d_work, D);
    case 5: return launch_groups<5>(c, S, a, r, d_roots, d_work, D);
    case 6: return launch_groups<6>(c, S, a, r, d_roots, d_work, D);
    case 7: return launch_groups<7>(c, S, a, r, d_roots, d_work, D);
    case 8: return launch_groups<8>(c, S, a, r, d_roots, d_work, D);
    default: return set_error(KCLPP_ERR_UNSUPPORTED, "k = %d", k);
  }
}

// Runs the sampling kernel until the row buffer holds every kept clique (a
// second run, with the buffer sized to the first run's count, only when the
// first overflowed; the kept set does not change between runs).
kclpp_status sample(kclpp_ctx *c, kclpp_sampling *S) {
  const HostDag &D = graph_dag(S->g);
  const int k = S->k;
  std::vector<uint32_t> roots;
  for (uint32_t v = 0; v < D.n; ++v)
    if (D.off[v + 1] - D.off[v] >= (uint64_t)(k - 1)) roots.push_back(v);
  std::stable_sort(roots.begin(), roots.end(), [&](uint32_t a, uint32_t b) {
    return D.off[a + 1] - D.off[a] > D.off[b + 1] - D.off[b];
  });
  if (roots.empty() || S->total == 0) {
    S->sampled = 0;
    return KCLPP_OK;
  }
  cudaStream_t st = ctx_stream(c);
  uint32_t *d_roots = nullptr, *d_work = nullptr;
  unsigned long long *d_count = nullptr;
  auto release = [&]() {
    if (d_roots) cudaFree(d_roots);
    if (d_work) cudaFree(d_work);
    if (d_count) cudaFree(d_count);
  };
  kclpp_status status = KCLPP_OK;
  for (int attempt = 0; attempt < 2; ++attempt) {
    cudaError_t e = cudaSuccess;
    if (!d_roots) e = dalloc(&d_roots, roots.size());
    if (e == cudaSuccess && !d_work) e = dalloc(&d_work, 4);
    if (e == cudaSuccess && !d_count) e = dalloc(&d_count, 1);
    if (e == cudaSuccess && !S->d_rows) e = dalloc(&S->d_rows, (size_t)S->cap * k);
    if (e == cudaSuccess && !S->d_wave) e = dalloc(&S->d_wave, (size_t)S->cap);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_roots, roots.data(), roots.size() * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_work, 0, 16, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_count, 0, 8, st);
    if (e != cudaSuccess) {
      release();
      return set_error(e == cudaErrorMemoryAllocation ? KCLPP_ERR_NOMEM : KCLPP_ERR_CUDA, "sampling: %s",
                       cudaGetErrorString(e));
    }
    SampleArgs a{};
    a.off = graph_dev_offsets(S->g);
    a.cols = graph_dev_cols(S->g);
    a.seed = S->seed;
    a.threshold = S->threshold;
    a.all = S->all;
    a.waves = S->waves;
    a.rows = S->d_rows;
    a.wave = S->d_wave;
    a.cap = S->cap;
    a.count = d_count;
    status = launch_k(k, c, S, a, roots, d_roots, d_work, D);
    if (status != KCLPP_OK) break;
    unsigned long long got = 0;
    e = cudaMemcpyAsync(&got, d_count, 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      status = set_error(KCLPP_ERR_CUDA, "sampling: %s", cudaGetErrorString(e));
      break;
    }
    S->sampled = got;
    if (got <= S->cap) break;
    if (attempt == 1) {
      status = set_error(KCLPP_ERR_CUDA, "sampling: the kept set changed between runs");
      break;
    }
    cudaFree(S->d_rows);
    cudaFree(S->d_wave);
    S->d_rows = nullptr;
    S->d_wave = nullptr;
    S->cap = got;
  }
  release();
  return status;
}

kclpp_status check_ctx(kclpp_ctx *c, const kclpp_sampling *S) {
  if (!c || !S) return set_error(KCLPP_ERR_INVALID, "null argument");
  if (ctx_device(c) != S->device) return set_error(KCLPP_ERR_INVALID, "context and sampling on different devices");
  SCUDA(cudaSetDevice(S->device));
  return KCLPP_OK;
}

kclpp_status run_passes(kclpp_ctx *c, kclpp_sampling *S, uint32_t passes) {
  if (!passes || !S->sampled || !S->n) return KCLPP_OK;
  cudaStream_t st = ctx_stream(c);
  const int sms = ctx_sms(c);
  const uint32_t grid_rows =
      (uint32_t)std::min<uint64_t>((S->sampled + kPassThreads - 1) / kPassThreads, (uint64_t)sms * 8);
  const uint32_t grid_n = std::min<uint32_t>((S->n + kPassThreads - 1) / kPassThreads, (uint32_t)sms * 8);
  for (uint32_t p = 0; p < passes; ++p) {
    for (uint32_t w = 0; w < S->waves; ++w) {
      k_wave<<<grid_rows, kPassThreads, 0, st>>>(S->d_rows, S->d_wave, S->sampled, S->k, w, S->d_rho, S->d_delta);
      k_apply<<<grid_n, kPassThreads, 0, st>>>(S->n, S->d_rho, S->d_delta);
    }
    SCUDA(cudaGetLastError());
    ctx_count_launch(c, 2 * (int)S->waves);
  }
  SCUDA(cudaStreamSynchronize(st));
  return KCLPP_OK;
}

}  // namespace

extern "C" {

kclpp_status kclpp_sampling_create(kclpp_ctx *c, const kclpp_graph *g, int k, uint64_t target, uint64_t seed,
                                   uint32_t waves, kclpp_sampling **out) {
  if (!c || !g || !out) return set_error(KCLPP_ERR_INVALID, "null argument");
  *out = nullptr;
  if (k < 3 || k > KCLPP_MAX_K)
    return set_error(KCLPP_ERR_UNSUPPORTED, "k = %d outside the sampling range [3, %d]", k, KCLPP_MAX_K);
  if (target < 1 || target > 0x7fffffffull) return set_error(KCLPP_ERR_INVALID, "target outside [1, 2^31 - 1]");
  if (waves < 1 || waves > smp::kMaxWaves) return set_error(KCLPP_ERR_INVALID, "waves outside [1, 256]");
  if (ctx_device(c) != graph_device(g)) return set_error(KCLPP_ERR_INVALID, "context and graph on different devices");
  const HostDag &D = graph_dag(g);
  if (D.core > smp::kMaxDegree)
    return set_error(KCLPP_ERR_UNSUPPORTED, "out-degree %u exceeds %u", D.core, smp::kMaxDegree);
  std::unique_ptr<kclpp_sampling> S(new kclpp_sampling());
  S->g = g;
  S->device = ctx_device(c);
  S->k = k;
  S->n = D.n;
  S->target = target;
  S->seed = seed;
  S->waves = waves;
  SCUDA(cudaSetDevice(S->device));
  // The COUNT task (kCDensestSamplingKclistpp.c:153-157, 191-195), then p (:272).
  STRY(kclpp_count_cliques(c, g, k, nullptr, &S->total));
  S->all = target >= S->total;
  S->prob = S->all ? 1.0 : (double)target / (double)S->total;
  S->threshold = S->all ? 0 : (uint64_t)std::ldexp(S->prob, 64);
  // Room for the expected sample plus a margin well beyond its spread.
  S->cap = S->all ? S->total : std::min<uint64_t>(S->total, target + target / 8 + 4096);
  SCUDA(dalloc(&S->d_rho, S->n));
  SCUDA(dalloc(&S->d_delta, S->n));
  SCUDA(dalloc(&S->d_rank, S->n));
  SCUDA(dalloc(&S->d_push, S->n));
  cudaStream_t st = ctx_stream(c);
  SCUDA(cudaMemsetAsync(S->d_rho, 0, (size_t)std::max<uint32_t>(S->n, 1) * 4, st));
  SCUDA(cudaMemsetAsync(S->d_delta, 0, (size_t)std::max<uint32_t>(S->n, 1) * 4, st));
  STRY(sample(c, S.get()));
  *out = S.release();
  return KCLPP_OK;
}

void kclpp_sampling_free(kclpp_sampling *s) { delete s; }

kclpp_status kclpp_sampling_info_get(const kclpp_sampling *s, kclpp_sampling_info *info) {
  if (!s || !info) return set_error(KCLPP_ERR_INVALID, "null argument");
  info->cliques_total = s->total;
  info->sampled = s->sampled;
  info->prob = s->prob;
  info->threshold = s->threshold;
  info->all = s->all;
  info->waves = s->waves;
  info->passes = s->passes;
  return KCLPP_OK;
}

kclpp_status kclpp_sampling_cliques(kclpp_ctx *c, const kclpp_sampling *s, uint32_t *rows, uint8_t *waves) {
  STRY(check_ctx(c, s));
  const int k = s->k;
  const size_t S = (size_t)s->sampled;
  if (!S || (!rows && !waves)) return KCLPP_OK;
  std::vector<uint32_t> r(S * k);
  std::vector<uint8_t> w(S);
  cudaStream_t st = ctx_stream(c);
  SCUDA(cudaMemcpyAsync(r.data(), s->d_rows, r.size() * 4, cudaMemcpyDeviceToHost, st));
  SCUDA(cudaMemcpyAsync(w.data(), s->d_wave, S, cudaMemcpyDeviceToHost, st));
  SCUDA(cudaStreamSynchronize(st));
  std::vector<size_t> idx(S);
  std::iota(idx.begin(), idx.end(), (size_t)0);
  std::sort(idx.begin(), idx.end(), [&](size_t a, size_t b) {
    for (int j = k - 1; j >= 0; --j)
      if (r[a * k + j] != r[b * k + j]) return r[a * k + j] < r[b * k + j];
    return false;
  });
  for (size_t i = 0; i < S; ++i) {
    if (rows) memcpy(rows + i * k, &r[idx[i] * k], (size_t)k * 4);
    if (waves) waves[i] = w[idx[i]];
  }
  return KCLPP_OK;
}

kclpp_status kclpp_sampling_passes(kclpp_ctx *c, kclpp_sampling *s, uint32_t passes) {
  STRY(check_ctx(c, s));
  STRY(run_passes(c, s, passes));
  s->passes += passes;
  return KCLPP_OK;
}

kclpp_status kclpp_sampling_get_rho(kclpp_ctx *c, const kclpp_sampling *s, uint32_t *rho) {
  STRY(check_ctx(c, s));
  if (!s->n) return KCLPP_OK;
  if (!rho) return set_error(KCLPP_ERR_INVALID, "null argument");
  cudaStream_t st = ctx_stream(c);
  SCUDA(cudaMemcpyAsync(rho, s->d_rho, (size_t)s->n * 4, cudaMemcpyDeviceToHost, st));
  SCUDA(cudaStreamSynchronize(st));
  return KCLPP_OK;
}

kclpp_status kclpp_sampling_set_rho(kclpp_ctx *c, kclpp_sampling *s, const uint32_t *rho, uint32_t passes) {
  STRY(check_ctx(c, s));
  if (s->n && !rho) return set_error(KCLPP_ERR_INVALID, "null argument");
  cudaStream_t st = ctx_stream(c);
  if (s->n) SCUDA(cudaMemcpyAsync(s->d_rho, rho, (size_t)s->n * 4, cudaMemcpyHostToDevice, st));
  SCUDA(cudaStreamSynchronize(st));
  s->passes = passes;
  return KCLPP_OK;
}

kclpp_status kclpp_sampling_extract(kclpp_ctx *c, kclpp_sampling *s, uint32_t T, kclpp_sampling_report *rep,
                                    uint32_t *order) {
  STRY(check_ctx(c, s));
  if (!rep) return set_error(KCLPP_ERR_INVALID, "null argument");
  if (T < 1) return set_error(KCLPP_ERR_INVALID, "T must be at least 1");
  memset(rep, 0, sizeof *rep);
  rep->T = T;
  const uint32_t n = s->n;
  const int k = s->k;
  if (!n) return KCLPP_OK;
  cudaStream_t st = ctx_stream(c);
  std::vector<uint32_t> rho(n), ord(n), rank(n), push(n);
  SCUDA(cudaMemcpyAsync(rho.data(), s->d_rho, (size_t)n * 4, cudaMemcpyDeviceToHost, st));
  SCUDA(cudaStreamSynchronize(st));
  // Vertices by decreasing load, ties by ascending id (:367-373).
  std::iota(ord.begin(), ord.end(), 0u);
  std::stable_sort(ord.begin(), ord.end(), [&](uint32_t a, uint32_t b) { return rho[a] > rho[b]; });
  for (uint32_t i = 0; i < n; ++i) rank[ord[i]] = i;
  // Each kept clique to its last vertex in that order (:375-383), on the GPU.
  SCUDA(cudaMemcpyAsync(s->d_rank, rank.data(), (size_t)n * 4, cudaMemcpyHostToDevice, st));
  SCUDA(cudaMemsetAsync(s->d_push, 0, (size_t)n * 4, st));
  if (s->sampled) {
    const uint32_t grid =
        (uint32_t)std::min<uint64_t>((s->sampled + kPassThreads - 1) / kPassThreads, (uint64_t)ctx_sms(c) * 8);
    k_push<<<grid, kPassThreads, 0, st>>>(s->d_rows, s->sampled, k, s->d_rank, s->d_push);
    SCUDA(cudaGetLastError());
    ctx_count_launch(c, 1);
  }
  SCUDA(cudaMemcpyAsync(push.data(), s->d_push, (size_t)n * 4, cudaMemcpyDeviceToHost, st));
  SCUDA(cudaStreamSynchronize(st));
  // The densest prefix (:385-394): the first strictly best count / size.
  double best = -1;
  uint64_t cnt = 0;
  for (uint32_t i = 0; i < n; ++i) {
    cnt += push[i];
    const double dens = (double)cnt / (double)(i + 1);
    if (best < dens) {
      rep->n = i + 1;
      rep->m = cnt;
      best = dens;
    }
  }
  rep->density = best;
  // The bound from the loads (:400-417), in the reference's operation order.
  {
    uint64_t sum = 0;
    double ub = 0, ip1ck = 0;
    for (uint32_t i = 0; i < n; ++i) {
      sum += rho[ord[i]];
      if (i + 1 == (uint32_t)k) ip1ck = 1;
      else if (i + 1 > (uint32_t)k) ip1ck = (ip1ck * (double)(i + 1)) / (double)(i + 1 - k);
      const double avg = (double)sum / (double)T;
      if (ip1ck < avg) {
        ub = ip1ck / (double)(i + 1);
      } else {
        const double v = avg / (double)(i + 1);
        if (ub < v) ub = v;
        break;
      }
    }
    rep->ub = ub;
  }
  // The densest subgraph's exact clique count (MakeDensestSubgraphEdgeList and
  // the COUNT_IN_SUBGRAPH task, :420-435, :467-471): its edges, labelled by
  // their position in the order, through the library's own pipeline.
  const HostDag &D = graph_dag(s->g);
  std::vector<uint32_t> pairs;
  for (uint32_t a = 0; a < D.n; ++a) {
    if (rank[a] >= rep->n) continue;
    for (uint64_t e = D.off[a]; e < D.off[a + 1]; ++e) {
      const uint32_t b = D.cols[e];
      if (rank[b] >= rep->n) continue;
      pairs.push_back(rank[a]);
      pairs.push_back(rank[b]);
    }
  }
  rep->sub_e = pairs.size() / 2;
  if (rep->sub_e) {
    kclpp_edge_list *el = nullptr;
    kclpp_graph *sg = nullptr;
    kclpp_status st2 = kclpp_edge_list_create(pairs.data(), rep->sub_e, &el);
    if (st2 == KCLPP_OK) st2 = kclpp_build_graph(c, el, &sg);
    if (st2 == KCLPP_OK) st2 = kclpp_count_cliques(c, sg, k, nullptr, &rep->sub_cliques);
    uint32_t sn = 0, score = 0;
    uint64_t sm = 0;
    if (st2 == KCLPP_OK) st2 = kclpp_graph_info(sg, &sn, &sm, &score);
    kclpp_graph_free(sg);
    kclpp_edge_list_free(el);
    if (st2 != KCLPP_OK) return st2;
    rep->sub_n = sn;
    rep->sub_core = score;
  }
  // The report line's figures (:475-477), with the reference's unsigned n - 1.
  rep->edge_density = (double)rep->sub_e * 2.0 / (double)rep->sub_n / (double)(uint32_t)(rep->sub_n - 1u);
  rep->clique_density = (double)rep->sub_cliques / (double)rep->sub_n;
  rep->upper_bound = rep->ub / s->prob / (1 - std::sqrt(6 * std::log((double)n) / rep->ub));
  if (order) memcpy(order, ord.data(), (size_t)n * 4);
  return KCLPP_OK;
}

kclpp_status kclpp_sampling_main(kclpp_ctx *c, const kclpp_graph *g, int k, uint32_t num_iter, uint64_t target,
                                 uint64_t seed, uint32_t waves, kclpp_sampling_report *reps, int cap, int *count) {
  if (count) *count = 0;
  if (cap > 0 && !reps) return set_error(KCLPP_ERR_INVALID, "null argument");
  kclpp_sampling *s = nullptr;
  STRY(kclpp_sampling_create(c, g, k, target, seed, waves, &s));
  std::unique_ptr<kclpp_sampling> hold(s);
  int made = 0;
  for (uint64_t T = 1; T <= num_iter; T <<= 1) {
    STRY(kclpp_sampling_passes(c, s, (uint32_t)T - s->passes));
    if (made < cap) STRY(kclpp_sampling_extract(c, s, (uint32_t)T, &reps[made], nullptr));
    ++made;
  }
  if (count) *count = std::min(made, std::max(cap, 0));
  return KCLPP_OK;
}

}  // extern "C"
