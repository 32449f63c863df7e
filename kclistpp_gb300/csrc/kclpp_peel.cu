// kclpp_peel.cu -- the recounts of the k-clique core peel on the GPU.
//
// kcliquecore (kClistCoreTrim.c:605-666) pops the vertex u of smallest
// k-clique degree and, in oneshortpass (:577-603), counts for every neighbour
// v still in the heap the k-cliques {u, v, ...} among the vertices still in
// the heap; v's degree then drops by that count.  Here a batch of such
// recounts runs at once: root j of the batch is a popped (or predicted) vertex
// and its member list is its live neighbours, ascending.  The count kernels'
// explicit-list mode induces each root's member rows from the DAG and stores,
// per member, the number of (k-1)-cliques of the induced graph through it --
// exactly oneshortpass's nck2[v].
//
// Roots are launched in three groups by member count: tier S (<= 64, a warp
// per root), tier M (<= 1024, a CTA per root, rows in shared memory) and tier L
// (<= 2048, rows in a per-CTA global slab); tiers M and L steal, so that a
// batch of one large root still spreads over every SM.  Larger lists are left
// to the caller (the host's recursion).
#include <algorithm>
#include <cstring>
#include <vector>

#include "kclpp_dev.cuh"
#include "kclpp_internal.h"

namespace kclpp {

#define PCUDA(call)                                                                                        \
  do {                                                                                                     \
    cudaError_t e_ = (call);                                                                               \
    if (e_ != cudaSuccess)                                                                                 \
      return set_error(e_ == cudaErrorMemoryAllocation ? KCLPP_ERR_NOMEM : KCLPP_ERR_CUDA, "%s: %s (%s:%d)", \
                       #call, cudaGetErrorString(e_), __FILE__, __LINE__);                                 \
  } while (0)

namespace {
constexpr uint32_t kRegistryWords = kActiveSlots;  // one stealing registry per stealing group
constexpr uint32_t kPeelWorkHeader = 32;           // root counters of the groups

template <typename T>
cudaError_t grow_dev(T **p, size_t *cap, size_t need) {
  if (need <= *cap && *p) return cudaSuccess;
  cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  const size_t c = std::max<size_t>(need + need / 2, 1024);
  cudaError_t e = cudaMalloc((void **)p, c * sizeof(T));
  if (e == cudaSuccess) *cap = c;
  return e;
}
template <typename T>
cudaError_t grow_host(T **p, size_t *cap, size_t need) {
  if (need <= *cap && *p) return cudaSuccess;
  cudaFreeHost(*p);
  *p = nullptr;
  *cap = 0;
  const size_t c = std::max<size_t>(need + need / 2, 1024);
  cudaError_t e = cudaMallocHost((void **)p, c * sizeof(T));
  if (e == cudaSuccess) *cap = c;
  return e;
}
}  // namespace

struct PeelRecount {
  kclpp_ctx *ctx = nullptr;
  const kclpp_graph *g = nullptr;
  int k = 0;
  // device
  uint64_t *d_loff = nullptr;
  uint32_t *d_lcols = nullptr;
  unsigned long long *d_w = nullptr;
  uint32_t *d_roots = nullptr;
  uint32_t *d_task = nullptr;
  uint32_t *d_work = nullptr;
  uint32_t *d_slab = nullptr;
  size_t cap_loff = 0, cap_lcols = 0, cap_w = 0, cap_roots = 0, cap_task = 0;
  uint64_t slab_words = 0;
  int slab_ctas = 0;
  // pinned staging
  uint64_t *h_loff = nullptr;
  uint32_t *h_lcols = nullptr;
  unsigned long long *h_w = nullptr;
  uint32_t *h_roots = nullptr;
  size_t hcap_loff = 0, hcap_lcols = 0, hcap_w = 0, hcap_roots = 0;
};

kclpp_status peel_recount_create(kclpp_ctx *c, const kclpp_graph *g, int k, PeelRecount **out) {
  *out = nullptr;
  auto *P = new PeelRecount();
  P->ctx = c;
  P->g = g;
  P->k = k;
  cudaError_t e = cudaMalloc((void **)&P->d_work, (kPeelWorkHeader + 2 * kRegistryWords) * sizeof(uint32_t));
  if (e != cudaSuccess) {
    delete P;
    return set_error(KCLPP_ERR_NOMEM, "peel recount: %s", cudaGetErrorString(e));
  }
  *out = P;
  return KCLPP_OK;
}

void peel_recount_free(PeelRecount *P) {
  if (!P) return;
  cudaFree(P->d_loff); cudaFree(P->d_lcols); cudaFree(P->d_w); cudaFree(P->d_roots);
  cudaFree(P->d_task); cudaFree(P->d_work); cudaFree(P->d_slab);
  cudaFreeHost(P->h_loff); cudaFreeHost(P->h_lcols); cudaFreeHost(P->h_w); cudaFreeHost(P->h_roots);
  delete P;
}

// Counts for the roots j < nroots with gpu[j] set: w[loff[j] + i] = k-cliques
// through root j and its member i (lists in lcols, ascending, 2 .. 2048
// members).  Entries of the other roots are left as they are in w.
kclpp_status peel_recount_run(PeelRecount *P, uint32_t nroots, const uint64_t *loff, const uint32_t *lcols,
                              const uint8_t *gpu, uint64_t *w) {
  kclpp_ctx *c = P->ctx;
  const cudaStream_t st = ctx_stream(c);
  const uint64_t total = loff[nroots];
  // groups: L (1025..2048), M (65..1024), S (k-1..64), each by descending size
  std::vector<uint32_t> grp[3];
  for (uint32_t j = 0; j < nroots; ++j) {
    if (!gpu[j]) continue;
    const uint64_t d = loff[j + 1] - loff[j];
    if (d > kTierLMax) return set_error(KCLPP_ERR_INVALID, "peel recount: a list of %llu members", (unsigned long long)d);
    grp[d > kTierMMax ? 0 : (d > kTierSMax ? 1 : 2)].push_back(j);
  }
  size_t nr = 0;
  for (auto &v : grp) {
    std::stable_sort(v.begin(), v.end(), [&](uint32_t a, uint32_t b) {
      return loff[a + 1] - loff[a] > loff[b + 1] - loff[b];
    });
    nr += v.size();
  }
  if (nr == 0) return KCLPP_OK;
  PCUDA(grow_host(&P->h_loff, &P->hcap_loff, (size_t)nroots + 1));
  PCUDA(grow_host(&P->h_lcols, &P->hcap_lcols, (size_t)total));
  PCUDA(grow_host(&P->h_w, &P->hcap_w, (size_t)total));
  PCUDA(grow_host(&P->h_roots, &P->hcap_roots, nr));
  PCUDA(grow_dev(&P->d_loff, &P->cap_loff, (size_t)nroots + 1));
  PCUDA(grow_dev(&P->d_lcols, &P->cap_lcols, (size_t)total));
  PCUDA(grow_dev(&P->d_w, &P->cap_w, (size_t)total));
  PCUDA(grow_dev(&P->d_roots, &P->cap_roots, nr));
  PCUDA(grow_dev(&P->d_task, &P->cap_task, nr));
  if (!grp[0].empty() && !P->d_slab) {
    P->slab_ctas = ctx_sms(c);
    P->slab_words = (uint64_t)kTierLMax * ((kTierLMax + 31) / 32);
    PCUDA(cudaMalloc((void **)&P->d_slab, P->slab_words * P->slab_ctas * sizeof(uint32_t)));
  }
  memcpy(P->h_loff, loff, ((size_t)nroots + 1) * 8);
  memcpy(P->h_lcols, lcols, (size_t)total * 4);
  size_t at = 0;
  for (auto &v : grp) {
    memcpy(P->h_roots + at, v.data(), v.size() * 4);
    at += v.size();
  }
  PCUDA(cudaMemcpyAsync(P->d_loff, P->h_loff, ((size_t)nroots + 1) * 8, cudaMemcpyHostToDevice, st));
  PCUDA(cudaMemcpyAsync(P->d_lcols, P->h_lcols, (size_t)total * 4, cudaMemcpyHostToDevice, st));
  PCUDA(cudaMemcpyAsync(P->d_roots, P->h_roots, nr * 4, cudaMemcpyHostToDevice, st));
  PCUDA(cudaMemsetAsync(P->d_work, 0, kPeelWorkHeader * sizeof(uint32_t), st));
  PCUDA(cudaMemsetAsync(P->d_work + kPeelWorkHeader, 0xff, 2 * kRegistryWords * sizeof(uint32_t), st));
  PCUDA(cudaMemsetAsync(P->d_task, 0, nr * sizeof(uint32_t), st));
  dev::PassArgs a{};
  a.off = graph_dev_offsets(P->g);
  a.cols = graph_dev_cols(P->g);
  a.err = ctx_err_word(c);
  a.list_off = P->d_loff;
  a.list_cols = P->d_lcols;
  a.pair_out = P->d_w;
  a.slab = P->d_slab;
  a.slab_words = P->slab_words;
  at = 0;
  int launched = 0;
  for (int t = 0; t < 3; ++t) {
    const std::vector<uint32_t> &v = grp[t];
    if (v.empty()) continue;
    TierLaunch tl{};
    tl.tier = t == 0 ? 2 : (t == 1 ? 1 : 0);
    tl.roots = P->d_roots + at;
    tl.num_roots = (uint32_t)v.size();
    tl.dmax = (uint32_t)(loff[v.front() + 1] - loff[v.front()]);
    tl.work = P->d_work + t;
    tl.task_next = P->d_task + at;
    tl.active = t < 2 ? P->d_work + kPeelWorkHeader + (size_t)t * kRegistryWords : nullptr;
    tl.num_sms = ctx_sms(c);
    tl.max_grid = t == 0 ? P->slab_ctas : 0;
    tl.warps = 0;
    cudaError_t e = launch_count(P->k, tl, a, st);
    if (e != cudaSuccess) return set_error(KCLPP_ERR_CUDA, "peel recount launch: %s", cudaGetErrorString(e));
    ++launched;
    at += v.size();
  }
  ctx_count_launch(c, launched);
  PCUDA(cudaMemcpyAsync(P->h_w, P->d_w, (size_t)total * 8, cudaMemcpyDeviceToHost, st));
  const kclpp_status es = ctx_check_err(c);  // synchronises the stream
  if (es != KCLPP_OK) return es;
  for (auto &v : grp)
    for (uint32_t j : v) memcpy(w + loff[j], P->h_w + loff[j], (size_t)(loff[j + 1] - loff[j]) * 8);
  return KCLPP_OK;
}

}  // namespace kclpp
