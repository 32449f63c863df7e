// kclpp_k_count.cu -- instantiates the MODE_COUNT clique kernels (one translation
// unit per mode so that the library builds in parallel), and the k-clique
// degree entry point that allocates nothing.
#include <cstring>
#include <mutex>

#include "kclpp_internal.h"
#include "kclpp_kernels.cuh"

namespace kclpp {
cudaError_t launch_count(int k, const TierLaunch &t, dev::PassArgs a, cudaStream_t st) {
  return launch_mode<dev::MODE_COUNT>(k, t, a, st);
}

// ---------------------------------------------------------------------------
// k-clique degrees without any allocation.
//
// Some callers cannot allocate device memory at the point where they need
// clique degrees: code running inside a memory pool or arena that owns all of
// the device's memory, callers that must not take the allocator's locks or
// implicit synchronisation in the middle of their own pipeline, or plug-in
// hosts that hand the library only the buffers it may touch.  For them the
// scheduler's working memory -- per-launch root counters, the steal cursor,
// one sub-task counter per vertex, the status word and the clique total --
// lives in a statically sized device array that the library carries in its
// image, so the call needs nothing beyond the caller's inputs and outputs.
//
// Limits: at most kNoAllocMaxVertices vertices (the array holds one counter per
// vertex: 8 MiB plus 256 bytes, resident on every device that loads the
// library until the process exits) and out-degree at most 1024 (the larger
// roots' bitmap rows need a global slab, which would be another allocation).
//
// The array is shared by every call on a device: the call clears the part it
// uses before launching, and two calls whose kernels overlap on the GPU (for
// instance on two streams at once) race on it.  The first call on each device
// looks up the array's device address (cudaGetSymbolAddress, with that device
// current).  No call may be made while a stream is being captured: the call
// ends with a read-back of its status and a synchronisation, so it returns
// KCLPP_ERR_INVALID when the stream reports a capture in progress.
constexpr uint32_t kNoAllocMaxVertices = 1u << 21;
constexpr uint32_t kNoAllocHeader = 64;  // words before the per-vertex counters

static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocHeader + kNoAllocMaxVertices];

namespace {
std::mutex g_scratch_mu;
uint32_t *g_scratch_addr[64] = {};  // per device
}  // namespace

// The id-order (IDENT) instantiations of the count kernels: tier S over the
// vertices of out-degree 1..64, tier M over the rest (rows in shared memory).
template <int K>
static cudaError_t noalloc_tier(int tier, dev::PassArgs a, int sms, cudaStream_t st) {
  using namespace dev;
  int per_sm = 1;
  if (tier == 0) {
    static LaunchCache lc;
    const size_t sm = sizeof(SmemS<MODE_COUNT>) * kWarpsS;
    auto fn = tier_s_kernel<MODE_COUNT, K, true>;
    cudaError_t e = prepare(fn, lc, kWarpsS * 32, sm, &per_sm);
    if (e != cudaSuccess) return e;
    fn<<<per_sm * sms, kWarpsS * 32, sm, st>>>(a);
    return cudaGetLastError();
  }
  static LaunchCache lc;
  constexpr int NW = kWarpsM;
  const size_t sm = layout_m(MODE_COUNT, K, a.dmax, NW, true).total;
  auto fn = tier_m_kernel<MODE_COUNT, K, 1, true, true>;
  cudaError_t e = prepare(fn, lc, NW * 32, sm, &per_sm);
  if (e != cudaSuccess) return e;
  fn<<<per_sm * sms, NW * 32, sm, st>>>(a);
  return cudaGetLastError();
}

static cudaError_t launch_noalloc_count(int k, int tier, dev::PassArgs a, int sms, cudaStream_t st) {
  switch (k) {
    case 3: return noalloc_tier<3>(tier, a, sms, st);
    case 4: return noalloc_tier<4>(tier, a, sms, st);
    case 5: return noalloc_tier<5>(tier, a, sms, st);
    case 6: return noalloc_tier<6>(tier, a, sms, st);
    case 7: return noalloc_tier<7>(tier, a, sms, st);
    case 8: return noalloc_tier<8>(tier, a, sms, st);
    default: return cudaErrorInvalidValue;
  }
}

static cudaError_t scratch_address(int device, uint32_t **out) {
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (device < 0 || device >= 64) return cudaErrorInvalidDevice;
  if (!g_scratch_addr[device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[device] = static_cast<uint32_t *>(p);
  }
  *out = g_scratch_addr[device];
  return cudaSuccess;
}

}  // namespace kclpp

extern "C" kclpp_status kclpp_count_cliques_noalloc(void *stream, uint32_t n, uint64_t m, const uint64_t *offsets,
                                                    const uint32_t *cols, int k, uint64_t *nck, uint64_t *total) {
  using namespace kclpp;
  if (!offsets || (!cols && m) || (!nck && n))
    return set_error(KCLPP_ERR_INVALID, "kclpp_count_cliques_noalloc: null argument");
  if (k < 3 || k > KCLPP_MAX_K)
    return set_error(KCLPP_ERR_UNSUPPORTED, "k = %d outside the supported range [3, %d]", k, KCLPP_MAX_K);
  if (n > kNoAllocMaxVertices)
    return set_error(KCLPP_ERR_UNSUPPORTED,
                     "kclpp_count_cliques_noalloc: %u vertices exceed its limit of %u (use kclpp_count_cliques)", n,
                     kNoAllocMaxVertices);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // The call reads its status back and synchronises, neither of which a
  // stream capture allows: refuse instead of invalidating the capture.
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone)
    return set_error(KCLPP_ERR_INVALID, "kclpp_count_cliques_noalloc: called while a stream capture is in progress");
  int device = 0, sms = 1;
  uint32_t *scr = nullptr;
  cudaError_t e = cudaGetDevice(&device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = scratch_address(device, &scr);
  // Clear the counters this call uses and the output.
  if (e == cudaSuccess) e = cudaMemsetAsync(scr, 0, (kNoAllocHeader + (size_t)n) * sizeof(uint32_t), st);
  if (e == cudaSuccess && n) e = cudaMemsetAsync(nck, 0, (size_t)n * sizeof(uint64_t), st);
  if (e != cudaSuccess) return set_error(KCLPP_ERR_CUDA, "kclpp_count_cliques_noalloc: %s", cudaGetErrorString(e));
  if (n) {
    dev::PassArgs a{};
    a.off = offsets;
    a.cols = cols;
    a.err = scr + 3;
    a.out = reinterpret_cast<unsigned long long *>(nck);
    a.total = reinterpret_cast<unsigned long long *>(scr + 4);
    a.num_roots = n;
    a.task_next = scr + kNoAllocHeader;
    // Tier S: one warp per vertex of out-degree 1..64.
    {
      dev::PassArgs s = a;
      s.work = scr + 0;
      s.dmax = dev::kSMaxD;
      s.deg_lo = 1;
      s.deg_hi = dev::kSMaxD;
      e = launch_noalloc_count(k, 0, s, sms, st);
    }
    // Tier M: one CTA per vertex of out-degree 65..1024 (larger ones set the
    // status word and are reported below).
    if (e == cudaSuccess) {
      dev::PassArgs s = a;
      s.work = scr + 1;
      s.active = nullptr;  // no stealing: the registry would need one slot per CTA
      s.dmax = kTierMMax;
      s.deg_lo = dev::kSMaxD + 1;
      s.deg_hi = UINT32_MAX;
      e = launch_noalloc_count(k, 1, s, sms, st);
    }
    if (e != cudaSuccess) return set_error(KCLPP_ERR_CUDA, "kclpp_count_cliques_noalloc: launch: %s", cudaGetErrorString(e));
  }
  uint32_t head[6] = {0, 0, 0, 0, 0, 0};
  e = cudaMemcpyAsync(head, scr, sizeof head, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return set_error(KCLPP_ERR_CUDA, "kclpp_count_cliques_noalloc: %s", cudaGetErrorString(e));
  if (head[3] & dev::ERR_DEGREE)
    return set_error(KCLPP_ERR_UNSUPPORTED, "kclpp_count_cliques_noalloc: an out-degree exceeds %u", kTierMMax);
  if (head[3]) return set_error(KCLPP_ERR_CUDA, "kclpp_count_cliques_noalloc: device status 0x%x", head[3]);
  if (total) {
    uint64_t t = 0;
    memcpy(&t, &head[4], sizeof t);
    *total = t;
  }
  return KCLPP_OK;
}
