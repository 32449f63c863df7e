// kclpp_warm.cu -- learned warm start for Seq-kClist++ (no reference counterpart).
//
// A small MLP predicts every vertex's "++" load (r / T after many passes) from
// four per-vertex features; the prediction, scaled by a virtual pass count T0,
// becomes the starting r of the passes.  Everything runs on the device with
// kernels written here:
//   features   log1p of [degree, core number, triangles, 4-cliques capped at
//              2^24]; the clique counts come from the library's count kernels
//   model      4 -> 64 (ReLU) -> 1, weights stored in bf16, every product and
//              sum in fp32; fp32 master weights for training
//   training   full-batch mean-squared error on log1p(load): forward and
//              backward with a warp per vertex (each lane owns two hidden
//              units and their gradients; one global fp32 atomic per parameter
//              per warp), then an Adam step
// The plain zero-start run stays the fallback and the yardstick: the warm start
// changes only where the passes start, and its upper bound is computed from
// the increments the passes add (a feasible load), never from the prediction.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "kclpp_dev.cuh"
#include "kclpp_internal.h"

namespace kclpp {
namespace warm {

constexpr int F = 4;     // features
constexpr int H = 64;    // hidden units
constexpr int NP = H * F + H + H + 1;  // parameters: W1, b1, W2, b2
constexpr int OFF_W1 = 0, OFF_B1 = H * F, OFF_W2 = H * F + H, OFF_B2 = H * F + 2 * H;

// Layout: a warp per vertex, lane l owns hidden units l and l + 32 (their
// W1 rows, b1 and W2 entries live in the lane's registers, converted once from
// bf16).  The output needs one warp sum per vertex.
struct LaneParams {
  float w1[2][F], b1[2], w2[2], b2;
};
__device__ __forceinline__ LaneParams lane_params(const __nv_bfloat16 *pb, int lane) {
  LaneParams P;
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int j = lane + 32 * q;
#pragma unroll
    for (int f = 0; f < F; ++f) P.w1[q][f] = __bfloat162float(pb[OFF_W1 + j * F + f]);
    P.b1[q] = __bfloat162float(pb[OFF_B1 + j]);
    P.w2[q] = __bfloat162float(pb[OFF_W2 + j]);
  }
  P.b2 = __bfloat162float(pb[OFF_B2]);
  return P;
}

__device__ __forceinline__ float forward_warp(const LaneParams &P, const float *x, float h[2]) {
  float part = 0.f;
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    float a = P.b1[q];
#pragma unroll
    for (int f = 0; f < F; ++f) a = __fmaf_rn(P.w1[q][f], x[f], a);
    h[q] = fmaxf(a, 0.f);
    part = __fmaf_rn(P.w2[q], h[q], part);
  }
  return dev::warp_sum(part) + P.b2;
}

__global__ void k_predict(const __nv_bfloat16 *pb, const float *X, uint32_t n, float *Y) {
  const int lane = threadIdx.x & 31;
  const LaneParams P = lane_params(pb, lane);
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
    float x[F], h[2];
#pragma unroll
    for (int f = 0; f < F; ++f) x[f] = X[(size_t)i * F + f];
    const float y = forward_warp(P, x, h);
    if (lane == 0) Y[i] = y;
  }
}

// Gradients of L = (1/n) sum (y_hat - y)^2 with respect to the parameters, and L.
__global__ void k_grad(const __nv_bfloat16 *pb, const float *X, const float *Y, uint32_t n, float inv_n,
                       float *grad, float *loss) {
  const int lane = threadIdx.x & 31;
  const LaneParams P = lane_params(pb, lane);
  float gw1[2][F] = {}, gb1[2] = {}, gw2[2] = {}, gb2 = 0.f, l = 0.f;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
    float x[F], h[2];
#pragma unroll
    for (int f = 0; f < F; ++f) x[f] = X[(size_t)i * F + f];
    const float e = forward_warp(P, x, h) - Y[i];
    l = __fmaf_rn(e, e, l);
    const float dy = 2.f * e * inv_n;
    gb2 += dy;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      gw2[q] = __fmaf_rn(dy, h[q], gw2[q]);
      if (h[q] > 0.f) {
        const float dh = dy * P.w2[q];
        gb1[q] += dh;
#pragma unroll
        for (int f = 0; f < F; ++f) gw1[q][f] = __fmaf_rn(dh, x[f], gw1[q][f]);
      }
    }
  }
  // Lane-owned gradients go straight to global memory (one atomic per
  // parameter per warp); b2 and the loss are warp-uniform.
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    const int j = lane + 32 * q;
#pragma unroll
    for (int f = 0; f < F; ++f)
      if (gw1[q][f] != 0.f) atomicAdd(&grad[OFF_W1 + j * F + f], gw1[q][f]);
    if (gb1[q] != 0.f) atomicAdd(&grad[OFF_B1 + j], gb1[q]);
    if (gw2[q] != 0.f) atomicAdd(&grad[OFF_W2 + j], gw2[q]);
  }
  if (lane == 0) {
    if (gb2 != 0.f) atomicAdd(&grad[OFF_B2], gb2);
    if (l != 0.f) atomicAdd(loss, l * inv_n);
  }
}

// Adam on the fp32 master weights; refreshes the bf16 copies.
__global__ void k_adam(float *w, float *m, float *v, const float *g, __nv_bfloat16 *pb, float lr, float b1,
                       float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NP) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float upd = lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  w[i] -= upd;
  pb[i] = __float2bfloat16_rn(w[i]);
}

__global__ void k_to_bf16(const float *w, __nv_bfloat16 *pb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < NP) pb[i] = __float2bfloat16_rn(w[i]);
}

// features: [log1p(deg), log1p(core), log1p(tri), log1p(min(k4, 2^24))]
__global__ void k_features(const uint32_t *deg, const uint32_t *core, const unsigned long long *tri,
                           const unsigned long long *k4, uint32_t n, float *X) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned long long cap = 1ull << 24;
  X[(size_t)i * F + 0] = log1pf((float)deg[i]);
  X[(size_t)i * F + 1] = log1pf((float)core[i]);
  X[(size_t)i * F + 2] = log1pf((float)tri[i]);
  X[(size_t)i * F + 3] = log1pf((float)(k4[i] < cap ? k4[i] : cap));
}

// r0 = round(T0 * expm1(prediction)), never negative.
__global__ void k_warm_r(const float *Y, uint32_t n, float t0, unsigned long long *r0) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float load = expm1f(Y[i]);
  if (!(load > 0.f)) load = 0.f;
  r0[i] = (unsigned long long)llrintf(fminf(load * t0, 1e18f));
}

}  // namespace warm
}  // namespace kclpp

using namespace kclpp;
using namespace kclpp::warm;

struct kclpp_warm_model {
  int device = 0;
  float *w = nullptr, *m = nullptr, *v = nullptr, *g = nullptr, *loss = nullptr;
  __nv_bfloat16 *pb = nullptr;
  int step = 0;
};

#define WCUDA(call)                                                                           \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      return set_error(e_ == cudaErrorMemoryAllocation ? KCLPP_ERR_NOMEM : KCLPP_ERR_CUDA,    \
                       "%s: %s", #call, cudaGetErrorString(e_));                               \
  } while (0)

extern "C" {

kclpp_status kclpp_warm_create(kclpp_ctx *c, uint64_t seed, kclpp_warm_model **out) {
  if (!c || !out) return set_error(KCLPP_ERR_INVALID, "null argument");
  *out = nullptr;
  std::unique_ptr<kclpp_warm_model> M(new kclpp_warm_model());
  M->device = ctx_device(c);
  WCUDA(cudaSetDevice(M->device));
  for (float **p : {&M->w, &M->m, &M->v, &M->g}) WCUDA(cudaMalloc((void **)p, NP * sizeof(float)));
  WCUDA(cudaMalloc((void **)&M->loss, sizeof(float)));
  WCUDA(cudaMalloc((void **)&M->pb, NP * sizeof(__nv_bfloat16)));
  // He-style initialisation from a seeded generator (host, deterministic).
  SplitMix r(seed ^ 0x5eedull);
  std::vector<float> h(NP, 0.f);
  for (int j = 0; j < H * F; ++j) h[OFF_W1 + j] = (float)((r.uniform() * 2 - 1) * std::sqrt(6.0 / F));
  for (int j = 0; j < H; ++j) h[OFF_B1 + j] = 0.01f;
  for (int j = 0; j < H; ++j) h[OFF_W2 + j] = (float)((r.uniform() * 2 - 1) * std::sqrt(6.0 / H));
  h[OFF_B2] = 0.f;
  cudaStream_t st = ctx_stream(c);
  WCUDA(cudaMemcpyAsync(M->w, h.data(), NP * sizeof(float), cudaMemcpyHostToDevice, st));
  WCUDA(cudaMemsetAsync(M->m, 0, NP * sizeof(float), st));
  WCUDA(cudaMemsetAsync(M->v, 0, NP * sizeof(float), st));
  k_to_bf16<<<1, 512, 0, st>>>(M->w, M->pb);
  WCUDA(cudaGetLastError());
  ctx_count_launch(c, 1);
  WCUDA(cudaStreamSynchronize(st));
  *out = M.release();
  return KCLPP_OK;
}

void kclpp_warm_free(kclpp_warm_model *M) {
  if (!M) return;
  cudaSetDevice(M->device);
  cudaFree(M->w); cudaFree(M->m); cudaFree(M->v); cudaFree(M->g); cudaFree(M->loss); cudaFree(M->pb);
  delete M;
}

kclpp_status kclpp_warm_get_params(const kclpp_warm_model *M, float *params) {
  if (!M || !params) return set_error(KCLPP_ERR_INVALID, "null argument");
  WCUDA(cudaMemcpy(params, M->w, NP * sizeof(float), cudaMemcpyDeviceToHost));
  return KCLPP_OK;
}

kclpp_status kclpp_warm_set_params(kclpp_ctx *c, kclpp_warm_model *M, const float *params) {
  if (!c || !M || !params) return set_error(KCLPP_ERR_INVALID, "null argument");
  cudaStream_t st = ctx_stream(c);
  WCUDA(cudaMemcpyAsync(M->w, params, NP * sizeof(float), cudaMemcpyHostToDevice, st));
  k_to_bf16<<<1, 512, 0, st>>>(M->w, M->pb);
  WCUDA(cudaGetLastError());
  ctx_count_launch(c, 1);
  WCUDA(cudaStreamSynchronize(st));
  return KCLPP_OK;
}

// Warp-per-vertex kernels: 8 warps per CTA, at most 8 CTAs per SM.
static int grid_for(kclpp_ctx *c, uint32_t n) {
  const int per = (int)std::min<uint64_t>((n + 7) / 8, (uint64_t)ctx_sms(c) * 8);
  return std::max(per, 1);
}

kclpp_status kclpp_warm_predict_dev(kclpp_ctx *c, const kclpp_warm_model *M, const float *X_dev, uint32_t n,
                                    float *Y_dev) {
  if (!c || !M || ((!X_dev || !Y_dev) && n)) return set_error(KCLPP_ERR_INVALID, "null argument");
  if (!n) return KCLPP_OK;
  k_predict<<<grid_for(c, n), 256, 0, ctx_stream(c)>>>(M->pb, X_dev, n, Y_dev);
  WCUDA(cudaGetLastError());
  ctx_count_launch(c, 1);
  return KCLPP_OK;
}

kclpp_status kclpp_warm_grad_dev(kclpp_ctx *c, kclpp_warm_model *M, const float *X_dev, const float *Y_dev,
                                 uint32_t n, float *grad_host, float *loss_host) {
  if (!c || !M || ((!X_dev || !Y_dev) && n) || n == 0) return set_error(KCLPP_ERR_INVALID, "bad argument");
  cudaStream_t st = ctx_stream(c);
  WCUDA(cudaMemsetAsync(M->g, 0, NP * sizeof(float), st));
  WCUDA(cudaMemsetAsync(M->loss, 0, sizeof(float), st));
  k_grad<<<grid_for(c, n), 256, 0, st>>>(M->pb, X_dev, Y_dev, n, 1.f / (float)n, M->g, M->loss);
  WCUDA(cudaGetLastError());
  ctx_count_launch(c, 1);
  if (grad_host) WCUDA(cudaMemcpyAsync(grad_host, M->g, NP * sizeof(float), cudaMemcpyDeviceToHost, st));
  if (loss_host) WCUDA(cudaMemcpyAsync(loss_host, M->loss, sizeof(float), cudaMemcpyDeviceToHost, st));
  WCUDA(cudaStreamSynchronize(st));
  return KCLPP_OK;
}

kclpp_status kclpp_warm_train(kclpp_ctx *c, kclpp_warm_model *M, const float *X_dev, const float *Y_dev, uint32_t n,
                              uint32_t steps, float lr, float *loss_host) {
  if (!c || !M || ((!X_dev || !Y_dev) && n) || n == 0) return set_error(KCLPP_ERR_INVALID, "bad argument");
  cudaStream_t st = ctx_stream(c);
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (uint32_t s = 0; s < steps; ++s) {
    WCUDA(cudaMemsetAsync(M->g, 0, NP * sizeof(float), st));
    WCUDA(cudaMemsetAsync(M->loss, 0, sizeof(float), st));
    k_grad<<<grid_for(c, n), 256, 0, st>>>(M->pb, X_dev, Y_dev, n, 1.f / (float)n, M->g, M->loss);
    M->step++;
    const float c1 = 1.f - std::pow(b1, (float)M->step), c2 = 1.f - std::pow(b2, (float)M->step);
    k_adam<<<1, 512, 0, st>>>(M->w, M->m, M->v, M->g, M->pb, lr, b1, b2, eps, c1, c2);
    WCUDA(cudaGetLastError());
    ctx_count_launch(c, 2);
  }
  if (loss_host) {
    // loss of the final parameters
    WCUDA(cudaMemsetAsync(M->g, 0, NP * sizeof(float), st));
    WCUDA(cudaMemsetAsync(M->loss, 0, sizeof(float), st));
    k_grad<<<grid_for(c, n), 256, 0, st>>>(M->pb, X_dev, Y_dev, n, 1.f / (float)n, M->g, M->loss);
    WCUDA(cudaGetLastError());
    ctx_count_launch(c, 1);
    WCUDA(cudaMemcpyAsync(loss_host, M->loss, sizeof(float), cudaMemcpyDeviceToHost, st));
  }
  WCUDA(cudaStreamSynchronize(st));
  return KCLPP_OK;
}

kclpp_status kclpp_warm_features_dev(kclpp_ctx *c, uint32_t n, const uint32_t *deg_dev, const uint32_t *core_dev,
                                     const uint64_t *tri_dev, const uint64_t *k4_dev, float *X_dev) {
  if (!c || ((!deg_dev || !core_dev || !tri_dev || !k4_dev || !X_dev) && n))
    return set_error(KCLPP_ERR_INVALID, "null argument");
  if (!n) return KCLPP_OK;
  k_features<<<(n + 255) / 256, 256, 0, ctx_stream(c)>>>(
      deg_dev, core_dev, (const unsigned long long *)tri_dev, (const unsigned long long *)k4_dev, n, X_dev);
  WCUDA(cudaGetLastError());
  ctx_count_launch(c, 1);
  return KCLPP_OK;
}

kclpp_status kclpp_warm_r0_dev(kclpp_ctx *c, const float *Y_dev, uint32_t n, float t0, uint64_t *r0_dev) {
  if (!c || ((!Y_dev || !r0_dev) && n)) return set_error(KCLPP_ERR_INVALID, "null argument");
  if (!n) return KCLPP_OK;
  k_warm_r<<<(n + 255) / 256, 256, 0, ctx_stream(c)>>>(Y_dev, n, t0, (unsigned long long *)r0_dev);
  WCUDA(cudaGetLastError());
  ctx_count_launch(c, 1);
  return KCLPP_OK;
}

}  // extern "C"
