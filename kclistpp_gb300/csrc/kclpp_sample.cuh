// kclpp_sample.cuh -- Seq-Sampling++ (kCDensestSamplingKclistpp.c): the parts
// of the sampling kernels that are plain per-thread code, written once for
// the device and the host so that the host build can check them against the
// oracle without a GPU.
//
// The reference keeps each k-clique with probability p = target / (number of
// k-cliques), capped at 1 (kCDensestSamplingKclistpp.c:160-198 and 289), by
// calling rand() once per clique in enumeration order: the sample depends on
// the thread schedule and on the time of day (srand(time(NULL)), :492).  Here
// the choice is a function of the clique itself, a counter-based draw in the
// sense of the Random123 generators: every vertex has a 64-bit key
// key(v) = mix64(seed + (v + 1) * 0x9E3779B97F4A7C15), a clique Q has the key
// sum H(Q) = sum of its members' keys (mod 2^64), and Q is kept iff
// mix64(H(Q)) < threshold = floor(p * 2^64) (every clique when p = 1).  mix64
// is SplitMix64's output function (Steele, Lea and Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014).  The sample is then the same
// for every schedule, on every device, and the order in which the cliques are
// found does not matter.  The same sum gives each kept clique its wave in the
// "++" passes: wave(Q) = ((mix64(H(Q) ^ kWaveSalt) >> 32) * W) >> 32.
#pragma once

#include <cstddef>
#include <cstdint>

#if defined(__CUDACC__)
#define KCLPP_HD __host__ __device__ __forceinline__
#else
#define KCLPP_HD inline
#endif

namespace kclpp {
namespace smp {

constexpr uint64_t kGamma = 0x9E3779B97F4A7C15ull;
constexpr uint64_t kWaveSalt = 0xD1B54A32D192ED03ull;
constexpr int kMaxWords = 64;          // rows of up to 2048 candidates
constexpr uint32_t kMaxDegree = 2048;  // out-degree bound of the sampling kernels
constexpr uint32_t kMaxWaves = 256;    // waves are stored as one byte per clique

KCLPP_HD uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
KCLPP_HD uint64_t vertex_key(uint64_t seed, uint32_t v) { return mix64(seed + ((uint64_t)v + 1ull) * kGamma); }
KCLPP_HD bool kept(uint64_t h, uint64_t threshold, bool all) { return all || mix64(h) < threshold; }
KCLPP_HD uint32_t wave_of(uint64_t h, uint32_t waves) {
  return (uint32_t)(((mix64(h ^ kWaveSalt) >> 32) * (uint64_t)waves) >> 32);
}

KCLPP_HD int lowest_bit(uint32_t x) {
#if defined(__CUDA_ARCH__)
  return __ffs((int)x) - 1;
#else
  return __builtin_ctz(x);
#endif
}

// Row i of a root's bitmap: the positions j < i of the root's out-list
// (list, ascending global ids) whose vertex is an out-neighbour of list[i].
// N+(list[i]) is ascending and lies below list[i], so one merge over
// list[0, i) finds them.  Writes words [0, (i >> 5) + 1) of row.
KCLPP_HD void build_row(uint32_t i, const uint32_t *list, const uint64_t *off, const uint32_t *cols, uint32_t *row) {
  const uint32_t nw = (i >> 5) + 1;
  for (uint32_t w = 0; w < nw; ++w) row[w] = 0;
  const uint32_t x = list[i];
  uint32_t j = 0;
  for (uint64_t e = off[x], end = off[x + 1]; e < end && j < i; ++e) {
    const uint32_t y = cols[e];
    while (j < i && list[j] < y) ++j;
    if (j < i && list[j] == y) row[j >> 5] |= 1u << (j & 31);
  }
}

// The cliques that extend a prefix of a root's clique tree.  P holds the
// prefix's common candidates (bits of local ids in words [0, nw)), h the sum
// of the prefix's keys and path[0, K - 1 - L) its members after the root
// (path[0] = the root edge's head).  L members remain to be chosen; at the
// last one every candidate v closes a k-clique, passed to emit(H, path, v).
// Every member of P lies below the prefix's last member, and row u only has
// bits below u, so the intersection with row u needs words [0, (u >> 5) + 1).
template <int K, int L, typename Emit>
KCLPP_HD void cliques_below(const uint32_t *P, uint32_t nw, uint64_t h, uint32_t *path, const uint32_t *rows,
                            uint32_t ws, const uint64_t *keys, Emit &emit) {
  if constexpr (L == 1) {
    for (uint32_t w = 0; w < nw; ++w) {
      uint32_t bits = P[w];
      while (bits) {
        const uint32_t v = 32u * w + (uint32_t)lowest_bit(bits);
        bits &= bits - 1;
        emit(h + keys[v], path, v);
      }
    }
  } else {
    uint32_t Q[kMaxWords];
    for (uint32_t w = 0; w < nw; ++w) {
      uint32_t bits = P[w];
      while (bits) {
        const uint32_t u = 32u * w + (uint32_t)lowest_bit(bits);
        bits &= bits - 1;
        const uint32_t *ru = rows + (size_t)u * ws;
        const uint32_t nq = (u >> 5) + 1;
        uint32_t any = 0;
        for (uint32_t j = 0; j < nq; ++j) {
          Q[j] = P[j] & ru[j];
          any |= Q[j];
        }
        if (!any) continue;
        path[K - 1 - L] = u;
        cliques_below<K, L - 1>(Q, nq, h + keys[u], path, rows, ws, keys, emit);
      }
    }
  }
}

// Every k-clique whose two largest members are the root s (key sum hs) and
// its out-neighbour at local position t.
template <int K, typename Emit>
KCLPP_HD void edge_cliques(uint32_t t, uint64_t hs, const uint32_t *rows, uint32_t ws, const uint64_t *keys,
                           Emit &emit) {
  uint32_t path[K];
  path[0] = t;
  cliques_below<K, K - 2>(rows + (size_t)t * ws, (t >> 5) + 1, hs + keys[t], path, rows, ws, keys, emit);
}

// A kept clique's row: its members' global ids in ascending order (the
// reference's ck[] rows, kCDensestSamplingKclistpp.c:166-169: cknodes[0] is
// the deepest member).  path holds local ids, path[0] the largest after s.
template <int K>
KCLPP_HD void write_row(uint32_t *row, const uint32_t *list, uint32_t s, const uint32_t *path, uint32_t v) {
  row[0] = list[v];
  for (int i = 1; i <= K - 2; ++i) row[i] = list[path[K - 2 - i]];
  row[K - 1] = s;
}

// The member of a stored clique that takes its unit in a "++" pass: the
// smallest value, ties to the earliest member of the row, i.e. the smallest
// id (InMemoryFrankWolfe, kCDensestSamplingKclistpp.c:356-360).
KCLPP_HD uint32_t argmin_member(const uint32_t *row, int k, const uint32_t *rho) {
  uint32_t g = row[0], gv = rho[g];
  for (int j = 1; j < k; ++j) {
    const uint32_t v = row[j], vv = rho[v];
    if (vv < gv) {
      g = v;
      gv = vv;
    }
  }
  return g;
}

// The position of a stored clique's last vertex in the order by decreasing
// value (ExtractDensest, kCDensestSamplingKclistpp.c:380-386).
KCLPP_HD uint32_t max_rank(const uint32_t *row, int k, const uint32_t *rank) {
  uint32_t r = rank[row[0]];
  for (int j = 1; j < k; ++j) {
    const uint32_t q = rank[row[j]];
    r = q > r ? q : r;
  }
  return r;
}

}  // namespace smp
}  // namespace kclpp
