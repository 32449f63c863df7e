// kclpp_kernels.cuh -- the clique kernels (included by one translation unit per mode).
//
// Three modes share one root-vertex skeleton (build G_s as bitmaps, then work
// per row / per root edge):
//
//  MODE_COUNT  k-clique degree of every vertex (onepass/recursion,
//              kClistCoreTrim.c:368-416).  Rows are the symmetric adjacency S
//              of G_s; the (k-1)-cliques of G_s through x number the
//              (k-2)-cliques of S[x], counted with the id orientation
//              A[y] = S[y] ∩ {ids below y}, popcount at the last level.
//
//  MODE_ORDER  cliques credited to their smallest-key member (Sim-kClist++'s
//              rho_add, kCDensestCmpSync.c:138-146; PAVA's largest level,
//              kCDensestNoAtom.c:191-213).  G_s is relabelled by key rank and
//              oriented upward: the cliques whose smallest member in G_s is p
//              number the (k-2)-cliques of Up[p]; p takes them if its key is
//              below s's, otherwise s does.  Pure popcount counting: no clique
//              is visited one by one.
//
//  MODE_SEQ    Seq-kClist++'s in-place "++" chain (kCDensestNoAtom.c:155-268),
//              one independent stream per root edge (s, t) starting from the
//              pass-start r.  Cliques are visited in the reference's order
//              (ascending ids at every level); the argmin prefix is cached as a
//              vertex and its value re-read at every comparison, exactly as the
//              reference does.  At the last level the chain
//                  for v in V ascending: if cur[v] < cur[g] then cur[v]++ else cur[g]++
//              runs 32 candidates at a time (tiers M, L): a candidate fails
//              (credits g) iff cur[v] >= c0 + (failures before it); the failure
//              mask is the unique fixed point of that rule and is found by
//              iterating ballots (lane i is final after i+1 rounds, so the loop
//              is bounded by 33 rounds).
//
// Set iteration always walks a copy of the set (`it`) and intersects with the
// unmodified set, because the child set of u is P ∩ N+(u) over all of P.
#pragma once

#include <mutex>
#include <utility>
#include <vector>

#include "kclpp_dev.cuh"

namespace kclpp {
namespace dev {

// ========================================================================
// Tier S: one warp per root, d <= 64, 64-bit rows, one lane per row / edge.
constexpr int kSMaxD = 64;
constexpr int kSDl = kSMaxD + 1;  // per-lane delta stride

template <int MODE>
struct SmemS {
  uint32_t list[kSMaxD];
  unsigned long long rows[kSMaxD];
  unsigned long long base[kSMaxD + 1];  // SEQ: pass-start r; ORDER: keys
  unsigned long long acc[kSMaxD + 1];   // SEQ: per-root increments
  uint8_t rank[kSMaxD];
  uint8_t inv[kSMaxD];
  uint32_t dl[MODE == MODE_SEQ ? 32 * kSDl : 1];  // SEQ: per-lane stream deltas
};

__device__ __forceinline__ unsigned long long below64(int y) {
  return y == 0 ? 0ull : ((1ull << y) - 1ull);
}

// Number of R-cliques inside P.  Orientation rows[y], restricted to ids below
// y when BELOW (symmetric rows), used as is otherwise (upward rows).
template <int R, bool BELOW>
__device__ __forceinline__ uint64_t cnt64(unsigned long long P, const unsigned long long *rows) {
  if constexpr (R == 0) {
    return 1;
  } else if constexpr (R == 1) {
    return (uint64_t)__popcll(P);
  } else {
    uint64_t c = 0;
    unsigned long long it = P;
    while (it) {
      const int y = __ffsll((long long)it) - 1;
      it &= it - 1;
      unsigned long long A = rows[y];
      if (BELOW) A &= below64(y);
      c += cnt64<R - 1, BELOW>(P & A, rows);
    }
    return c;
  }
}

// Seq chain inside one lane (tier S).  L = levels left (k-2 at the top).
// Returns the number of cliques visited.
template <int L>
__device__ __forceinline__ uint32_t seq64(unsigned long long P, int g, const unsigned long long *rows,
                                          const unsigned long long *base, uint32_t *dl) {
  if constexpr (L == 1) {
    // clique_size == 3 branch, kCDensestNoAtom.c:162-171
    uint32_t c = 0;
    unsigned long long it = P;
    while (it) {
      const int u = __ffsll((long long)it) - 1;
      it &= it - 1;
      const int g2 = (base[u] + dl[u]) < (base[g] + dl[g]) ? u : g;
      dl[g2]++;
      ++c;
    }
    return c;
  } else if constexpr (L == 2) {
    // l == 2 branch, kCDensestNoAtom.c:173-188
    uint32_t c = 0;
    unsigned long long it = P;
    while (it) {
      const int u = __ffsll((long long)it) - 1;
      it &= it - 1;
      const int g2 = (base[u] + dl[u]) < (base[g] + dl[g]) ? u : g;
      unsigned long long V = P & rows[u];
      while (V) {
        const int v = __ffsll((long long)V) - 1;
        V &= V - 1;
        const int g3 = (base[v] + dl[v]) < (base[g2] + dl[g2]) ? v : g2;
        dl[g3]++;
        ++c;
      }
    }
    return c;
  } else {
    // general level, kCDensestNoAtom.c:218-267
    if (__popcll(P) < L) return 0;
    uint32_t c = 0;
    unsigned long long it = P;
    while (it) {
      const int u = __ffsll((long long)it) - 1;
      it &= it - 1;
      const int g2 = (base[u] + dl[u]) < (base[g] + dl[g]) ? u : g;
      c += seq64<L - 1>(P & rows[u], g2, rows, base, dl);
    }
    return c;
  }
}

// IDENT = true: the schedule is every vertex in id order (no root list), a
// vertex being a root of this launch when its out-degree lies in
// [a.deg_lo, a.deg_hi]; the roots' own clique counts are also summed into
// *a.total.  Used by the entry point that allocates nothing.
template <int MODE, int K, bool IDENT = false>
__global__ void __launch_bounds__(kWarpsS * 32) tier_s_kernel(PassArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using SM = SmemS<MODE>;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  SM &sm = reinterpret_cast<SM *>(smem_raw)[wid];
  if constexpr (MODE == MODE_SEQ) {
    for (int i = lane; i <= kSMaxD; i += 32) sm.acc[i] = 0;
    for (int i = 0; i < kSDl; ++i) sm.dl[lane * kSDl + i] = 0;
  }
  __syncwarp();
  for (;;) {
    uint32_t idx = 0;
    if (lane == 0) idx = atomicAdd(a.work, 1u);
    idx = __shfl_sync(KCL_FULL, idx, 0);
    if (idx >= a.num_roots) break;
    const uint32_t s = IDENT ? idx : a.roots[idx];
    uint64_t o;
    int d;
    const uint32_t *lcols;
    root_span(a, s, o, d, lcols);
    if constexpr (IDENT) {
      if ((uint32_t)d < a.deg_lo || (uint32_t)d > a.deg_hi) continue;
    }
    if (d > kSMaxD) {
      if (lane == 0) atomicOr(a.err, ERR_DEGREE);
      continue;
    }
    if (d < K - 1 || d == 0) continue;
    for (int i = lane; i < d; i += 32) sm.list[i] = lcols[o + i];
    int tau = 0;
    if constexpr (MODE == MODE_ORDER) {
      for (int i = lane; i < d; i += 32) sm.base[i] = vertex_key(a, sm.list[i]);
      const uint64_t ks = vertex_key(a, s);
      __syncwarp();
      int t = 0;
      for (int i = lane; i < d; i += 32) {
        const uint64_t ki = sm.base[i];
        int r = 0;
        for (int j = 0; j < d; ++j) {
          const uint64_t kj = sm.base[j];
          r += (kj < ki) || (kj == ki && j < i);
        }
        sm.rank[i] = (uint8_t)r;
        sm.inv[r] = (uint8_t)i;
        t += (ki <= ks);  // (key_i, i) < (key_s, d): s has the largest id
      }
      tau = warp_sum(t);
    }
    if constexpr (MODE == MODE_SEQ) {
      // Shared loads: the root's values as the load vector holds them now.
      if (a.shared_loads) {
        for (int i = lane; i < d; i += 32) sm.base[i] = __ldcg(a.out + sm.list[i]);
        if (lane == 0) sm.base[d] = __ldcg(a.out + s);
      } else {
        for (int i = lane; i < d; i += 32) sm.base[i] = a.r_in[sm.list[i]];
        if (lane == 0) sm.base[d] = a.r_in[s];
      }
    }
    for (int i = lane; i < kSMaxD; i += 32) sm.rows[i] = 0;
    __syncwarp();
    if (K >= 3) {
      // Row i: out-neighbours of list[i] inside N+(s), by merging the two
      // ascending lists (MakeSubgraph's induced adjacency, :104-113).
      for (int i = lane; i < d; i += 32) {
        const uint32_t x = sm.list[i];
        const uint64_t xe = a.off[x + 1];
        unsigned long long row = 0;
        int j = 0;
        for (uint64_t e = a.off[x]; e < xe && j < i; ++e) {
          const uint32_t y = a.cols[e];
          while (j < i && sm.list[j] < y) ++j;
          if (j < i && sm.list[j] == y) row |= 1ull << j;
        }
        if constexpr (MODE == MODE_SEQ) {
          sm.rows[i] = row;
        } else if constexpr (MODE == MODE_COUNT) {
          atomicOr(&sm.rows[i], row);
          unsigned long long it = row;
          while (it) {
            const int j2 = __ffsll((long long)it) - 1;
            it &= it - 1;
            atomicOr(&sm.rows[j2], 1ull << i);
          }
        } else {
          const int ri = sm.rank[i];
          unsigned long long it = row;
          while (it) {
            const int j2 = __ffsll((long long)it) - 1;
            it &= it - 1;
            const int rj = sm.rank[j2];
            const int lo = ri < rj ? ri : rj, hi = ri < rj ? rj : ri;
            atomicOr(&sm.rows[lo], 1ull << hi);
          }
        }
      }
      __syncwarp();
    }
    if constexpr (MODE == MODE_SEQ) {
      uint32_t *dl = &sm.dl[lane * kSDl];
      for (int j = lane; j < d; j += 32) {
        const unsigned long long C = sm.rows[j];
        if (!C) continue;
        const int g0 = sm.base[j] < sm.base[d] ? j : d;  // kCDensestNoAtom.c:287
        seq64<K - 2>(C, g0, sm.rows, sm.base, dl);
        // Close the stream: its increments fell on {s, t} ∪ C (shared loads:
        // straight to the load vector).
        auto close = [&](int i) {
          if (!dl[i]) return;
          if (a.shared_loads) atomicAdd(a.out + (i < d ? sm.list[i] : s), (unsigned long long)dl[i]);
          else atomicAdd(&sm.acc[i], (unsigned long long)dl[i]);
          dl[i] = 0;
        };
        unsigned long long it = C;
        while (it) {
          const int i = __ffsll((long long)it) - 1;
          it &= it - 1;
          close(i);
        }
        close(j);
        close(d);
      }
      __syncwarp();
      for (int i = lane; i <= d; i += 32) {
        const unsigned long long v = sm.acc[i];
        if (v) {
          atomicAdd(&a.out[i < d ? sm.list[i] : s], v);
          sm.acc[i] = 0;
        }
      }
    } else if constexpr (MODE == MODE_ORDER) {
      uint64_t ssum = 0;
      for (int p = lane; p < d; p += 32) {
        const uint64_t c = cnt64<K - 2, false>(sm.rows[p], sm.rows);
        if (p < tau) {
          if (c) atomicAdd(&a.out[sm.list[sm.inv[p]]], (unsigned long long)c);
        } else {
          ssum += c;
        }
      }
      ssum = warp_sum(ssum);
      if (lane == 0 && ssum) atomicAdd(&a.out[s], (unsigned long long)ssum);
    } else {
      uint64_t tot = 0;
      for (int x = lane; x < d; x += 32) {
        const uint64_t c = cnt64<K - 2, true>(sm.rows[x], sm.rows);
        if (a.list_off) a.pair_out[o + x] = (unsigned long long)c;
        else if (c) atomicAdd(&a.out[sm.list[x]], (unsigned long long)c);
        tot += c;
      }
      tot = warp_sum(tot);
      if (lane == 0 && tot && !a.list_off) {
        atomicAdd(&a.out[s], (unsigned long long)(tot / (K - 1)));
        if constexpr (IDENT) atomicAdd(a.total, (unsigned long long)(tot / (K - 1)));
      }
    }
    __syncwarp();
  }
}

// ========================================================================
// Tiers M and L: one CTA per root, rows of W 32-bit words, lane w holds word
// w (tier M, W <= 32) or words w and w + 32 (tier L, W <= 64).
template <int WPL>
struct Bits {
  uint32_t w[WPL];
};

// Seq rows hold only the ids below their own (N+(x) lies below x): row i
// keeps (i >> 5) + 1 words, packed one after another from word tri_off(i),
// which halves the bitmap and leaves shared memory for more stream warps.
__host__ __device__ __forceinline__ uint32_t tri_off(uint32_t i) {
  const uint32_t a = i >> 5, b = i & 31;
  return i + a * (16u * a + b - 16u * (a > 0));
}
template <int WPL, bool TRI = false>
__device__ __forceinline__ Bits<WPL> load_row(const uint32_t *rows, int r, int W, int lane) {
  Bits<WPL> b;
  const size_t o = TRI ? (size_t)tri_off((uint32_t)r) : (size_t)r * W;
  const int n = TRI ? (r >> 5) + 1 : W;
#pragma unroll
  for (int q = 0; q < WPL; ++q) {
    const int w = lane + 32 * q;
    b.w[q] = w < n ? rows[o + w] : 0u;
  }
  return b;
}
template <int WPL>
__device__ __forceinline__ Bits<WPL> band(const Bits<WPL> &a, const Bits<WPL> &b) {
  Bits<WPL> c;
#pragma unroll
  for (int q = 0; q < WPL; ++q) c.w[q] = a.w[q] & b.w[q];
  return c;
}
template <int WPL>
__device__ __forceinline__ int popc_lane(const Bits<WPL> &a) {
  int c = 0;
#pragma unroll
  for (int q = 0; q < WPL; ++q) c += __popc(a.w[q]);
  return c;
}
template <int WPL>
__device__ __forceinline__ bool any_bits(const Bits<WPL> &a) {
  uint32_t o = 0;
#pragma unroll
  for (int q = 0; q < WPL; ++q) o |= a.w[q];
  return __any_sync(KCL_FULL, o != 0);
}
// Mask of the ids below y for this lane's words.
template <int WPL>
__device__ __forceinline__ Bits<WPL> below_mask(int y, int lane) {
  Bits<WPL> b;
#pragma unroll
  for (int q = 0; q < WPL; ++q) {
    const int w = lane + 32 * q;
    const int yw = y >> 5;
    b.w[q] = w < yw ? 0xffffffffu : (w == yw ? ((1u << (y & 31)) - 1u) : 0u);
  }
  return b;
}

// Visit the members of a distributed set in ascending order (uniform across
// the warp).  F(u) is called by all lanes.
template <int WPL, typename F>
__device__ __forceinline__ void for_each_bit(const Bits<WPL> &P, F &&f) {
#pragma unroll
  for (int q = 0; q < WPL; ++q) {
    uint32_t m = __ballot_sync(KCL_FULL, P.w[q] != 0);
    while (m) {
      const int L = __ffs(m) - 1;
      m &= m - 1;
      uint32_t wb = __shfl_sync(KCL_FULL, P.w[q], L);
      while (wb) {
        const int b = __ffs(wb) - 1;
        wb &= wb - 1;
        f((L + 32 * q) * 32 + b);
      }
    }
  }
}

// Per-lane partial count of R-cliques inside P.
template <int R, bool BELOW, int WPL>
__device__ __forceinline__ uint64_t cnt_warp(const Bits<WPL> &P, const uint32_t *rows, int W, int lane) {
  if constexpr (R == 0) {
    return lane == 0 ? 1u : 0u;
  } else if constexpr (R == 1) {
    return (uint64_t)popc_lane(P);
  } else {
    uint64_t c = 0;
    for_each_bit<WPL>(P, [&](int y) {
      Bits<WPL> A = load_row<WPL>(rows, y, W, lane);
      if (BELOW) A = band(A, below_mask<WPL>(y, lane));
      c += cnt_warp<R - 1, BELOW, WPL>(band(P, A), rows, W, lane);
    });
    return c;
  }
}

// Edges of G_s inside P, each once, as per-lane partial sums (the k = 4 count,
// (k-2)-cliques = edges): the counting rows are symmetric and each member y
// counts its neighbours below it (BELOW), the Order rows are oriented upward
// and y counts its whole row.  P's members are compacted and a lane takes one
// member at a time, walking only the words its row can occupy -- instead of
// a warp per member over all W words (cnt_warp), which leaves the lanes past
// W idle and re-reads the empty half of every row.  scratch: 32 words for P,
// then the member list (u16).
template <bool BELOW>
__device__ __forceinline__ uint32_t edges_in(const Bits<1> &P, const uint32_t *rows, int W, int lane,
                                             uint32_t *scratch) {
  uint16_t *members = reinterpret_cast<uint16_t *>(scratch + 32);
  if (lane < W) scratch[lane] = P.w[0];
  const uint32_t lt = lanemask_lt();
  uint32_t total = 0;
  uint32_t nz = __ballot_sync(KCL_FULL, P.w[0] != 0);
  while (nz) {
    const int L = __ffs(nz) - 1;
    nz &= nz - 1;
    const uint32_t word = __shfl_sync(KCL_FULL, P.w[0], L);
    if ((word >> lane) & 1u) members[total + __popc(word & lt)] = (uint16_t)((L << 5) | lane);
    total += (uint32_t)__popc(word);
  }
  __syncwarp();
  uint32_t c = 0;
  for (uint32_t i = lane; i < total; i += 32) {
    const int y = members[i];
    const uint32_t *ry = rows + (size_t)y * W;
    if constexpr (BELOW) {
      const int hi = y >> 5;
      for (int w = 0; w < hi; ++w) c += __popc(scratch[w] & ry[w]);
      c += __popc(scratch[hi] & ry[hi] & ((1u << (y & 31)) - 1u));
    } else {
      for (int w = y >> 5; w < W; ++w) c += __popc(scratch[w] & ry[w]);
    }
  }
  __syncwarp();  // the next row reuses the scratch
  return c;
}

// Triangles of G_s inside P, each once, as per-lane partial sums (the k = 5
// count): a lane per member y of P walks the members z of P ∩ row(y) (below y
// with BELOW) and adds |P ∩ row(y) ∩ row(z)| over the words those rows can
// occupy.  scratch as in edges_in.
template <bool BELOW>
__device__ __forceinline__ uint32_t triangles_in(const Bits<1> &P, const uint32_t *rows, int W, int lane,
                                                 uint32_t *scratch) {
  uint16_t *members = reinterpret_cast<uint16_t *>(scratch + 32);
  if (lane < W) scratch[lane] = P.w[0];
  const uint32_t lt = lanemask_lt();
  uint32_t total = 0;
  uint32_t nz = __ballot_sync(KCL_FULL, P.w[0] != 0);
  while (nz) {
    const int L = __ffs(nz) - 1;
    nz &= nz - 1;
    const uint32_t word = __shfl_sync(KCL_FULL, P.w[0], L);
    if ((word >> lane) & 1u) members[total + __popc(word & lt)] = (uint16_t)((L << 5) | lane);
    total += (uint32_t)__popc(word);
  }
  __syncwarp();
  uint32_t c = 0;
  for (uint32_t i = lane; i < total; i += 32) {
    const int y = members[i];
    const uint32_t *ry = rows + (size_t)y * W;
    const int lo_w = BELOW ? 0 : (y >> 5), hi_w = BELOW ? (y >> 5) : W - 1;
    for (int w = lo_w; w <= hi_w; ++w) {
      uint32_t q = scratch[w] & ry[w];
      if (BELOW && w == (y >> 5)) q &= (1u << (y & 31)) - 1u;
      while (q) {
        const int b = __ffs(q) - 1;
        q &= q - 1;
        const int z = (w << 5) | b;
        const uint32_t *rz = rows + (size_t)z * W;
        if constexpr (BELOW) {
          const int zh = z >> 5;
          for (int w2 = 0; w2 < zh; ++w2) c += __popc(scratch[w2] & ry[w2] & rz[w2]);
          c += __popc(scratch[zh] & ry[zh] & rz[zh] & ((1u << (z & 31)) - 1u));
        } else {
          for (int w2 = z >> 5; w2 < W; ++w2) c += __popc(scratch[w2] & ry[w2] & rz[w2]);
        }
      }
    }
  }
  __syncwarp();  // the next row reuses the scratch
  return c;
}

// Shared-memory layout of a tier M / L CTA (dmax = largest out-degree the
// launch allows, NW warps).  Tier L keeps `rows` in a global slab instead.
struct LayoutM {
  size_t list, rows, base, acc, rank, inv, dl, cbuf, total;
};
// Per-warp scratch of the k = 4 counting path (edges_in): P's words and its
// members, compacted.
__host__ __device__ inline size_t cbuf_words(uint32_t dmax) { return 32 + (dmax + 1) / 2; }
__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }
__host__ __device__ inline LayoutM layout_m(int mode, int k, uint32_t dmax, int nw, bool rows_in_smem) {
  LayoutM L;
  const size_t W = (dmax + 31) / 32;
  size_t at = 0;
  L.list = at; at = align16(at + (size_t)dmax * 4);
  L.rows = at;
  if (rows_in_smem) at = align16(at + (mode == MODE_SEQ ? (size_t)tri_off(dmax) : (size_t)dmax * W) * 4);
  L.base = at; if (mode != MODE_COUNT) at = align16(at + (size_t)(dmax + 1) * 8);
  L.acc = at; if (mode == MODE_SEQ) at = align16(at + (size_t)(dmax + 1) * 8);
  L.rank = at; if (mode == MODE_ORDER) at = align16(at + (size_t)dmax * 2);
  L.inv = at; if (mode == MODE_ORDER) at = align16(at + (size_t)dmax * 2);
  L.dl = at; if (mode == MODE_SEQ) at = align16(at + (size_t)nw * (dmax + 1) * 4);
  L.cbuf = at;
  if (mode != MODE_SEQ && (k == 4 || k == 5) && rows_in_smem) at = align16(at + (size_t)nw * cbuf_words(dmax) * 4);
  L.total = at;
  return L;
}

// Current values of a root-edge stream's vertices (pass-start r plus the
// stream's own increments), in one of two forms:
//  * Vals32: one u32 per vertex, offset from the smallest pass-start value of
//    the stream (off) and capped at cap, when every value the stream can reach
//    stays below 2^31 (see seq_stream);
//  * Vals64: the pass-start u64 plus a u32 delta per vertex.
// Vertex x's word is only ever read and written by lane x & 31 (the chain,
// the argmin write-backs, the stream's setup and close), so the chains need
// no warp barrier.
struct Vals32 {
  using T = uint32_t;
  uint32_t *cur;
  __device__ __forceinline__ T get(int v, uint32_t &raw) const { raw = cur[v]; return raw; }
  __device__ __forceinline__ void bump(int v, uint32_t raw, uint32_t *) const { cur[v] = raw + 1u; }
  __device__ __forceinline__ void add(int v, T delta, uint32_t *) const { cur[v] += delta; }
};
template <bool OVF>
struct Vals64 {
  using T = unsigned long long;
  const unsigned long long *base;
  uint32_t *dl;
  __device__ __forceinline__ T get(int v, uint32_t &raw) const { raw = dl[v]; return base[v] + raw; }
  __device__ __forceinline__ void bump(int v, uint32_t raw, uint32_t *err) const {
    if (OVF && raw == 0xffffffffu) atomicOr(err, ERR_OVERFLOW);
    dl[v] = raw + 1u;
  }
  __device__ __forceinline__ void add(int v, T delta, uint32_t *err) const {
    const unsigned long long nd = (unsigned long long)dl[v] + delta;
    if (OVF && nd > 0xffffffffull) atomicOr(err, ERR_OVERFLOW);
    dl[v] = (uint32_t)nd;
  }
};

// Shared loads (KCLPP_SEQ_SHARED): a vertex's current value is the CTA's copy
// of the pass's one load vector -- 32 bits, relative to the smallest value
// of the root's vertices when the root started, capped at kSharedCap --
// refreshed from the vector when a stream starts and raised by the CTA's
// closing streams, plus this stream's own increments (a u32 per vertex, owned
// by lane v & 31 as in Vals64).  Other warps refresh and close concurrently,
// so a read is a recent snapshot, and a capped value hides how far above the
// others it is: the values steer which member gets a unit, never whether a
// unit is given.
constexpr uint32_t kSharedCap = 1u << 29;
struct ValsShared {
  using T = uint32_t;
  const uint32_t *cur;
  uint32_t *dl;
  __device__ __forceinline__ T get(int v, uint32_t &raw) const {
    raw = dl[v];
    return *(const volatile uint32_t *)(cur + v) + raw;
  }
  __device__ __forceinline__ void bump(int v, uint32_t raw, uint32_t *err) const {
    if (raw == 0xffffffffu) atomicOr(err, ERR_OVERFLOW);
    dl[v] = raw + 1u;
  }
  __device__ __forceinline__ void add(int v, T delta, uint32_t *err) const {
    const unsigned long long nd = (unsigned long long)dl[v] + delta;
    if (nd > 0xffffffffull) atomicOr(err, ERR_OVERFLOW);
    dl[v] = (uint32_t)nd;
  }
};

// Distance from the prefix value c to a candidate's value, as the chain's
// fixed point uses it: -1 below c, else the difference clamped to 2^31 - 1
// (a plain 32-bit difference for Vals32, whose values all lie below 2^31).
template <typename T>
__device__ __forceinline__ int distance(T av, T c) {
  if constexpr (sizeof(T) == 4) {
    return (int)(av - c);
  } else {
    if (av < c) return -1;
    const T dd = av - c;
    return dd > 0x7fffffffull ? 0x7fffffff : (int)dd;
  }
}

// The fixed point of one 32-candidate word of the chain: lane b stands for
// candidate b of the word (valid when its bit is set), rel its distance to
// the prefix value c at the word's start.  Candidate i falls to the prefix
// iff rel_i >= the number of earlier candidates of the word that fell to it
// (kCDensestNoAtom.c:162-171 and 180-186, resolved by ballots).  Returns the
// mask of the candidates that fall.
__device__ __forceinline__ uint32_t word_fixed_point(int rel, uint32_t lt) {
  // Start from "every candidate at or above c falls": once the loads have
  // spread, that guess is already exact and one vote confirms it; ties (the
  // first pass) take a few more rounds.  When no candidate is at or above c,
  // every one takes its clique and the guess is the fixed point already.
  uint32_t m = __ballot_sync(KCL_FULL, rel >= 0);
  if (m) {
    uint32_t m2 = __ballot_sync(KCL_FULL, rel >= __popc(m & lt));
    if (m2 != m) {
      m = m2;
      for (int r = 0; r < 32; ++r) {
        m2 = __ballot_sync(KCL_FULL, rel >= __popc(m & lt));
        if (m2 == m) break;
        m = m2;
      }
    }
  }
  return m;
}

// The Seq chain over V (the last level), one 32-bit word of V at a time: lane
// b stands for candidate 32 * word + b.  c is the current value of the prefix
// argmin (kCDensestNoAtom.c:162-171 and 180-186: each clique goes to the
// candidate w when r[w] < c, strict, else to the prefix argmin, whose value
// then grows by one).  Returns the prefix argmin's new value.
template <int WPL, typename VA>
__device__ __forceinline__ typename VA::T chain_words(const Bits<WPL> &V, typename VA::T c, const VA &va, int lane,
                                                      uint32_t *err) {
  using T = typename VA::T;
  const uint32_t lt = lanemask_lt();
#pragma unroll
  for (int q = 0; q < WPL; ++q) {
    uint32_t nz = __ballot_sync(KCL_FULL, V.w[q] != 0);
    while (nz) {
      const int L = __ffs(nz) - 1;
      nz &= nz - 1;
      const uint32_t word = __shfl_sync(KCL_FULL, V.w[q], L);
      const bool valid = (word >> lane) & 1u;
      const int v = ((L + 32 * q) << 5) | lane;
      int rel = -1;
      uint32_t raw = 0;
      if (valid) rel = distance<T>(va.get(v, raw), c);
      const uint32_t m = word_fixed_point(rel, lt);
      if (valid && !((m >> lane) & 1u)) va.bump(v, raw, err);
      c += (T)__popc(m);
    }
  }
  return c;
}

// The same chain over V of one word per lane (lane w holds word w of V) with
// 32-bit values, skipping the words that fall whole.  lo (lane w): the
// smallest value the stream started with among C's members in word w.
// Values only grow, and the prefix value at any candidate of V is at most c
// plus the number of candidates before it (< tot), so every candidate of a
// word with lo >= c + tot - 1 falls to the prefix: only the other words run
// their fixed point, in order, each from its exact prefix value c + (the
// candidates of V before it) - (those of them that took their clique).
template <typename VA>
__device__ __forceinline__ uint32_t chain_word1(uint32_t q, uint32_t c, const VA &va, uint32_t lo, int lane,
                                                uint32_t *err) {
  const uint32_t pop = (uint32_t)__popc(q);
  const uint32_t tot = __reduce_add_sync(KCL_FULL, pop);
  if (!tot) return c;
  uint32_t bad = __ballot_sync(KCL_FULL, pop != 0u && lo < c + tot - 1u);
  if (!bad) return c + tot;
  const uint32_t lt = lanemask_lt();
  uint32_t taken = 0;
  do {
    const int L = __ffs(bad) - 1;
    bad &= bad - 1;
    const uint32_t before = __reduce_add_sync(KCL_FULL, lane < L ? pop : 0u);
    const uint32_t cL = c + before - taken;
    const uint32_t word = __shfl_sync(KCL_FULL, q, L);
    const bool valid = (word >> lane) & 1u;
    const int v = (L << 5) | lane;
    int rel = -1;
    uint32_t raw = 0;
    if (valid) rel = (int)(va.get(v, raw) - cL);
    const uint32_t m = word_fixed_point(rel, lt);
    if (valid && !((m >> lane) & 1u)) va.bump(v, raw, err);
    taken += (uint32_t)(__popc(word) - __popc(m));
  } while (bad);
  return c + tot - taken;
}

// Current value of vertex x, read by the lane that owns it and broadcast.
template <typename VA>
__device__ __forceinline__ typename VA::T value_of(int x, const VA &va, int lane) {
  typename VA::T v = 0;
  uint32_t raw;
  if ((x & 31) == lane) v = va.get(x, raw);
  return __shfl_sync(KCL_FULL, v, x & 31);
}

// Level L of a root-edge stream over candidates P with prefix argmin g of
// current value cg (kCDensestNoAtom.c:173-188 for L = 2, 237-259 above).
// Returns g's new value; the argmin of a deeper prefix, when it is u, is
// written back by u's lane.  SKIP (one word per lane, 32-bit values): the
// last level runs chain_word1 with lo, the per-word lower bounds.
template <int L, int WPL, typename VA, bool SKIP>
__device__ __forceinline__ typename VA::T seq_rec(const Bits<WPL> &P, typename VA::T cg, const uint32_t *rows,
                                                  const VA &va, typename VA::T lo, int lane, uint32_t *err) {
  using T = typename VA::T;
  if constexpr (L == 1) {
    if constexpr (SKIP) {
      static_assert(WPL == 1 && sizeof(T) == 4, "the word skip needs one word per lane and 32-bit values");
      return chain_word1<VA>(P.w[0], cg, va, lo, lane, err);
    } else {
      return chain_words<WPL, VA>(P, cg, va, lane, err);
    }
  } else if constexpr (WPL == 1) {
    if constexpr (L >= 3) {
      const uint32_t pc = __reduce_add_sync(KCL_FULL, (uint32_t)__popc(P.w[0]));  // kCDensestNoAtom.c:218
      if (pc < (uint32_t)L) return cg;
    }
    // The members u of P in ascending order, word a of P at a time.  Row u =
    // 32 a + b keeps a + 1 words, packed from tri_off(32 a) = 16 a (a + 1)
    // with a stride of a + 1 words between the rows of word a.
    uint32_t nzw = __ballot_sync(KCL_FULL, P.w[0] != 0);
    while (nzw) {
      const int a = __ffs(nzw) - 1;
      nzw &= nzw - 1;
      uint32_t wb = __shfl_sync(KCL_FULL, P.w[0], a);
      const uint32_t stride = (uint32_t)a + 1u;
      const uint32_t *row0 = rows + 16u * (uint32_t)a * stride + (uint32_t)lane;
      const bool in_row = lane <= a;
      while (wb) {
        const int b = __ffs(wb) - 1;
        wb &= wb - 1;
        const int u = (a << 5) | b;
        // u's value: its word is written by lane b only; the warp barrier
        // orders those writes before every lane's read.
        __syncwarp();
        uint32_t raw;
        const T vu = va.get(u, raw);
        const bool take = vu < cg;  // strict: ties stay with the earlier argmin
        Bits<1> Q;
        Q.w[0] = in_row ? (P.w[0] & row0[(uint32_t)b * stride]) : 0u;
        const T c0 = take ? vu : cg;
        const T c1 = seq_rec<L - 1, 1, VA, SKIP>(Q, c0, rows, va, lo, lane, err);
        if (take) {
          if (lane == b) va.add(u, c1 - c0, err);
        } else {
          cg = c1;
        }
      }
    }
    return cg;
  } else {
    if constexpr (L >= 3) {
      const int pc = warp_sum(popc_lane(P));  // kCDensestNoAtom.c:218
      if (pc < L) return cg;
    }
    for_each_bit<WPL>(P, [&](int u) {
      const T vu = value_of<VA>(u, va, lane);
      const bool take = vu < cg;  // strict: ties stay with the earlier argmin
      const Bits<WPL> Q = band(P, load_row<WPL, true>(rows, u, 0, lane));
      const T c0 = take ? vu : cg;
      const T c1 = seq_rec<L - 1, WPL, VA, SKIP>(Q, c0, rows, va, lo, lane, err);
      if (take) {
        if (lane == (u & 31)) va.add(u, c1 - c0, err);
      } else {
        cg = c1;
      }
    });
    return cg;
  }
}

// Apply f(i) on the lane owning each member i of C (lane i & 31).
template <int WPL, typename F>
__device__ __forceinline__ void for_members(const Bits<WPL> &C, int lane, F &&f) {
#pragma unroll
  for (int qq = 0; qq < WPL; ++qq) {
    uint32_t nz = __ballot_sync(KCL_FULL, C.w[qq] != 0);
    while (nz) {
      const int L = __ffs(nz) - 1;
      nz &= nz - 1;
      const uint32_t word = __shfl_sync(KCL_FULL, C.w[qq], L);
      if ((word >> lane) & 1u) f(((L + 32 * qq) << 5) | lane);
    }
  }
}

// Every root-edge stream of the current root, the warp taking streams from
// the root's shared counter (largest candidate sets first); increments go to
// the CTA's acc[] (kCDensestNoAtom.c:270-295 per root edge).
//
// A stream's values fit the 32-bit form when, with off = the smallest
// pass-start value among {s, t} and C and cap = (the edge argmin's value
// - off) + the most increments one vertex can take in the stream + 64, cap
// stays below 2^31: values above cap are stored as cap, which changes no
// comparison -- the prefix value never exceeds cap - 64, so such a candidate
// falls to the prefix whatever came before it (its distance is >= 64 > 31),
// and it never becomes the prefix argmin.
template <int K, int WPL>
__device__ __forceinline__ void seq_streams(uint32_t *next, int d, const uint32_t *rows,
                                            const unsigned long long *base, uint32_t *cur,
                                            unsigned long long *acc, int lane, uint32_t *err) {
  for (;;) {
    int q = 0;
    if (lane == 0) q = (int)atomicAdd(next, 1u);
    q = __shfl_sync(KCL_FULL, q, 0);
    if (q >= d) break;
    const int j = d - 1 - q;
    const Bits<WPL> C = load_row<WPL, true>(rows, j, 0, lane);
    if (!any_bits<WPL>(C)) continue;
    const int g0 = base[j] < base[d] ? j : d;  // kCDensestNoAtom.c:287
    bool r32 = false;
    unsigned long long off = 0, cap = 0;
    if constexpr (K <= 5) {
      unsigned long long lo = base[g0];
      int nc = 0;
      for_members<WPL>(C, lane, [&](int i) {
        const unsigned long long b = base[i];
        lo = b < lo ? b : lo;
        ++nc;
      });
      lo = warp_min_u64(lo);
      nc = warp_sum(nc);
      unsigned long long bound = 1;  // C(nc, K - 2) >= the increments of one vertex
      for (int i = 0; i < K - 2; ++i) bound = bound * (unsigned long long)(nc - i) / (unsigned long long)(i + 1);
      off = lo;
      cap = (base[g0] - lo) + bound + 64;
      r32 = cap < 0x7fffffffull;
    }
    if (r32) {
      // Stored values, and per word of C the smallest of them (lane = word).
      uint32_t lo = 0xffffffffu;
#pragma unroll
      for (int qq = 0; qq < WPL; ++qq) {
        uint32_t nz = __ballot_sync(KCL_FULL, C.w[qq] != 0);
        while (nz) {
          const int L = __ffs(nz) - 1;
          nz &= nz - 1;
          const uint32_t word = __shfl_sync(KCL_FULL, C.w[qq], L);
          uint32_t val = 0xffffffffu;
          if ((word >> lane) & 1u) {
            const int i = ((L + 32 * qq) << 5) | lane;
            const unsigned long long rel = base[i] - off;
            val = (uint32_t)(rel < cap ? rel : cap);
            cur[i] = val;
          }
          val = __reduce_min_sync(KCL_FULL, val);
          if (qq == 0 && lane == L) lo = val;
        }
      }
      const Vals32 va{cur};
      const uint32_t c0 = (uint32_t)(base[g0] - off);
      const uint32_t c1 = seq_rec<K - 2, WPL, Vals32, (WPL == 1)>(C, c0, rows, va, lo, lane, err);
      for_members<WPL>(C, lane, [&](int i) {
        const unsigned long long rel = base[i] - off;
        const uint32_t delta = cur[i] - (uint32_t)(rel < cap ? rel : cap);
        if (delta) atomicAdd(&acc[i], (unsigned long long)delta);
      });
      if (lane == 0 && c1 != c0) atomicAdd(&acc[g0], (unsigned long long)(c1 - c0));
    } else {
      for_members<WPL>(C, lane, [&](int i) { cur[i] = 0; });
      const Vals64<(K >= 6)> va{base, cur};
      const unsigned long long c0 = base[g0];
      const unsigned long long c1 = seq_rec<K - 2, WPL, Vals64<(K >= 6)>, false>(C, c0, rows, va, 0u, lane, err);
      for_members<WPL>(C, lane, [&](int i) {
        const uint32_t delta = cur[i];
        if (delta) atomicAdd(&acc[i], (unsigned long long)delta);
      });
      if (lane == 0 && c1 != c0) atomicAdd(&acc[g0], c1 - c0);
    }
  }
}

// KCLPP_SEQ_SHARED: every root-edge stream of the current root against the
// pass's one load vector r (updated in place).  When a stream starts, the
// CTA's copy of its vertices' values is raised to r's (relative to off, the
// root's smallest value when it started); the chain is the reference's
// (kCDensestNoAtom.c:155-268) on the copy plus the stream's own increments;
// when it closes, its increments go to the copy (seen at once by the CTA's
// other streams) and, by atomic adds, to r (seen by every stream that starts
// later).  Every clique still gives exactly one unit to one of its members,
// so r / T stays a feasible load whatever the interleaving; which member
// gets it depends on the timing of the other streams (not deterministic).
// The vector is read and added to once per stream and vertex, not per
// clique: the whole GPU reading a few kilobytes of L2 at every candidate
// serialises on the few L2 slices that hold them.
template <int K, int WPL>
__device__ __forceinline__ void seq_streams_shared(uint32_t *next, int d, const uint32_t *rows, const uint32_t *list,
                                                   uint32_t s, unsigned long long *r, unsigned long long off,
                                                   uint32_t *cur, uint32_t *dl, int lane, uint32_t *err) {
  const ValsShared va{cur, dl};
  auto id = [&](int i) { return i < d ? list[i] : s; };
  auto refresh = [&](int i) {
    const unsigned long long v = __ldcg(r + id(i)) - off;
    atomicMax(cur + i, v < kSharedCap ? (uint32_t)v : kSharedCap);
  };
  auto close = [&](int i, uint32_t x) {
    atomicAdd(cur + i, x);
    atomicAdd(r + id(i), (unsigned long long)x);
  };
  for (;;) {
    int q = 0;
    if (lane == 0) q = (int)atomicAdd(next, 1u);
    q = __shfl_sync(KCL_FULL, q, 0);
    if (q >= d) break;
    const int j = d - 1 - q;
    const Bits<WPL> C = load_row<WPL, true>(rows, j, 0, lane);
    if (!any_bits<WPL>(C)) continue;
    // Refresh the members' values and take, per word of C (lane = word), the
    // smallest of them: values only grow while the stream runs, so a word
    // whose candidates all start at or above the prefix's reach falls to the
    // prefix whole (the chain's skip).
    uint32_t lo = 0xffffffffu;
#pragma unroll
    for (int qq = 0; qq < WPL; ++qq) {
      uint32_t nz = __ballot_sync(KCL_FULL, C.w[qq] != 0);
      while (nz) {
        const int L = __ffs(nz) - 1;
        nz &= nz - 1;
        const uint32_t word = __shfl_sync(KCL_FULL, C.w[qq], L);
        uint32_t val = 0xffffffffu;
        if ((word >> lane) & 1u) {
          const int i = ((L + 32 * qq) << 5) | lane;
          refresh(i);
          dl[i] = 0;
          val = *(volatile uint32_t *)(cur + i);
        }
        val = __reduce_min_sync(KCL_FULL, val);
        if (qq == 0 && lane == L) lo = val;
      }
    }
    uint32_t vj = 0, vd = 0;
    if (lane == 0) {
      refresh(j);
      refresh(d);
      vj = *(volatile uint32_t *)(cur + j);
      vd = *(volatile uint32_t *)(cur + d);
    }
    __syncwarp();
    const int g0 = __shfl_sync(KCL_FULL, vj < vd ? j : d, 0);  // kCDensestNoAtom.c:287
    const uint32_t c0 = __shfl_sync(KCL_FULL, vj < vd ? vj : vd, 0);
    const uint32_t c1 = seq_rec<K - 2, WPL, ValsShared, (WPL == 1)>(C, c0, rows, va, lo, lane, err);
    for_members<WPL>(C, lane, [&](int i) {
      const uint32_t x = dl[i];
      if (x) close(i, x);
    });
    if (lane == 0 && c1 != c0) close(g0, c1 - c0);
  }
}

// Work stealing: once the root list is exhausted, an idle CTA joins a root
// whose sub-tasks (root edges or rows) are not all taken, rebuilds that root's
// G_s and takes sub-tasks from the same global counter.  Every CTA publishes
// the root it holds in its slot of a.active, so a thief looks at the roots in
// progress only (one slot per CTA, scanned by one warp) and joins the one with
// the most sub-tasks left.  Returns UINT32_MAX when none has kMinSteal left.
constexpr uint32_t kMinSteal = 2;
template <bool IDENT>
__device__ __forceinline__ uint32_t find_victim(const PassArgs &a, int need, int lane) {
  uint32_t best = 0, best_idx = UINT32_MAX;  // best = sub-tasks left (0: none)
  for (uint32_t b = lane; b < gridDim.x; b += 32) {
    const uint32_t idx = *(volatile uint32_t *)(a.active + b);
    if (idx >= a.num_roots) continue;
    const uint32_t s = IDENT ? idx : a.roots[idx];
    const uint32_t d = a.list_off ? (uint32_t)(a.list_off[s + 1] - a.list_off[s]) : (uint32_t)(a.off[s + 1] - a.off[s]);
    const uint32_t taken = *(volatile uint32_t *)(a.task_next + idx);
    const bool in_window = !IDENT || (d >= a.deg_lo && d <= a.deg_hi && d <= a.dmax);
    if (in_window && (int)d >= need && taken + kMinSteal <= d && d - taken > best) {
      best = d - taken;
      best_idx = idx;
    }
  }
  const uint32_t top = __reduce_max_sync(KCL_FULL, best);
  if (top == 0) return UINT32_MAX;
  const uint32_t who = __ballot_sync(KCL_FULL, best == top);
  return __shfl_sync(KCL_FULL, best_idx, __ffs(who) - 1);
}

// Register budget of a tier M / L kernel, as CTAs of the widest launch that
// must fit one SM: two for the shallow recursions (the Seq kernel then keeps
// <= 42 registers a thread at k = 3, 4; the counting kernels <= 32 at k <= 4
// and <= 42 at k = 5 with 24-warp CTAs), one for the deeper ones, which would
// otherwise spill.
template <int MODE, int K>
constexpr int min_ctas_m() { return K <= (MODE == MODE_SEQ ? 4 : 5) ? 2 : 1; }

template <int MODE, int K, int WPL, bool ROWS_IN_SMEM, bool IDENT = false>
__global__ void __launch_bounds__(warps_m<MODE, K>() * 32, min_ctas_m<MODE, K>()) tier_m_kernel(PassArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int NW = (int)(blockDim.x >> 5);
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int dmax = (int)a.dmax;
  const LayoutM lay = layout_m(MODE, K, a.dmax, NW, ROWS_IN_SMEM);
  uint32_t *list = reinterpret_cast<uint32_t *>(smem_raw + lay.list);
  uint32_t *rows = ROWS_IN_SMEM ? reinterpret_cast<uint32_t *>(smem_raw + lay.rows)
                                : a.slab + (size_t)blockIdx.x * a.slab_words;
  unsigned long long *base = reinterpret_cast<unsigned long long *>(smem_raw + lay.base);
  unsigned long long *acc = reinterpret_cast<unsigned long long *>(smem_raw + lay.acc);
  uint16_t *rank = reinterpret_cast<uint16_t *>(smem_raw + lay.rank);
  uint16_t *inv = reinterpret_cast<uint16_t *>(smem_raw + lay.inv);
  uint32_t *dl = reinterpret_cast<uint32_t *>(smem_raw + lay.dl) + (size_t)wid * (dmax + 1);
  uint32_t *cbuf = reinterpret_cast<uint32_t *>(smem_raw + lay.cbuf) + (size_t)wid * cbuf_words(a.dmax);

  __shared__ uint32_t s_idx;
  __shared__ int s_tau;
  __shared__ unsigned long long s_sum;
  __shared__ unsigned long long s_off;  // shared-load Seq: the root's smallest value

  if constexpr (MODE == MODE_SEQ) {
    for (int i = tid; i <= dmax; i += NW * 32) acc[i] = 0;
    for (int i = lane; i <= dmax; i += 32) dl[i] = 0;
  }
  bool stealing = false;  // warp 0's view (uniform across its lanes)
  __syncthreads();
  for (;;) {
    if (wid == 0) {
      uint32_t idx = UINT32_MAX;
      if (!stealing) {
        if (lane == 0) idx = atomicAdd(a.work, 1u);
        idx = __shfl_sync(KCL_FULL, idx, 0);
        if (idx >= a.num_roots) stealing = true;
      }
      if (stealing) idx = a.active ? find_victim<IDENT>(a, K - 1, lane) : UINT32_MAX;
      if (lane == 0) {
        s_idx = idx;
        s_tau = 0;
        s_sum = 0;
        s_off = ~0ull;
        if (a.active && idx != UINT32_MAX) a.active[blockIdx.x] = idx;  // visible to thieves
      }
    }
    __syncthreads();
    const uint32_t idx = s_idx;
    if (idx == UINT32_MAX) break;
    uint32_t *next = a.task_next + idx;  // root's sub-task counter, shared by every CTA on it
    const uint32_t s = IDENT ? idx : a.roots[idx];
    uint64_t o;
    int d;
    const uint32_t *lcols;
    if constexpr (MODE == MODE_COUNT) {
      root_span(a, s, o, d, lcols);
    } else {
      o = a.off[s];
      d = (int)(a.off[s + 1] - o);
      lcols = a.cols;
    }
    if constexpr (IDENT) {
      if ((uint32_t)d < a.deg_lo || (uint32_t)d > a.deg_hi) {
        __syncthreads();
        continue;
      }
    }
    if (d > dmax || d > 32 * 32 * WPL) {
      if (tid == 0) { atomicOr(a.err, ERR_DEGREE); atomicMax(next, (uint32_t)d); }
      __syncthreads();
      continue;
    }
    if (d < K - 1 || d == 0) {
      __syncthreads();
      continue;
    }
    const int W = (d + 31) >> 5;
    const int row_words = MODE == MODE_SEQ ? (int)tri_off((uint32_t)d) : d * W;
    for (int i = tid; i < d; i += NW * 32) list[i] = lcols[o + i];
    for (int i = tid; i < row_words; i += NW * 32) rows[i] = 0;
    if constexpr (MODE == MODE_ORDER) {
      for (int i = tid; i < d; i += NW * 32) base[i] = vertex_key(a, a.cols[o + i]);
      if (tid == 0) base[d] = vertex_key(a, s);
    }
    if constexpr (MODE == MODE_SEQ) {
      if (a.shared_loads) {
        // The load vector as it is now (from L2: other SMs add to it), as 32-bit
        // values relative to its smallest entry among the root's vertices, in
        // the acc array (which this mode does not otherwise use).
        uint32_t *cur = reinterpret_cast<uint32_t *>(acc);
        unsigned long long mn = ~0ull;
        for (int i = tid; i <= d; i += NW * 32) {
          base[i] = __ldcg(a.out + (i < d ? a.cols[o + i] : s));
          mn = base[i] < mn ? base[i] : mn;
        }
        mn = warp_min_u64(mn);
        if (lane == 0) atomicMin(&s_off, mn);
        __syncthreads();
        const unsigned long long off = s_off;
        for (int i = tid; i <= d; i += NW * 32) {
          const unsigned long long v = base[i] - off;
          cur[i] = v < kSharedCap ? (uint32_t)v : kSharedCap;
        }
      } else {
        for (int i = tid; i < d; i += NW * 32) base[i] = a.r_in[a.cols[o + i]];
        if (tid == 0) base[d] = a.r_in[s];
      }
    }
    __syncthreads();
    if constexpr (MODE == MODE_ORDER) {
      const unsigned long long ks = base[d];
      int t = 0;
      for (int i = tid; i < d; i += NW * 32) {
        const unsigned long long ki = base[i];
        int r = 0;
        for (int j = 0; j < d; ++j) {
          const unsigned long long kj = base[j];
          r += (kj < ki) || (kj == ki && j < i);
        }
        rank[i] = (uint16_t)r;
        inv[r] = (uint16_t)i;
        t += (ki <= ks);
      }
      t = warp_sum(t);
      if (lane == 0 && t) atomicAdd(&s_tau, t);
      __syncthreads();
    }
    if (K >= 3) {
      // Row i: N+(list[i]) ∩ N+(s) (MakeSubgraph's induced adjacency,
      // kCDensestNoAtom.c:104-113), one warp per row, a lane per out-neighbour.
      for (int i = wid; i < d; i += NW) {
        if (i == 0) continue;
        const uint32_t x = list[i];
        const uint32_t top = list[i - 1];
        const uint64_t xe = a.off[x + 1];
        for (uint64_t e = a.off[x] + lane; e < xe; e += 32) {
          const uint32_t y = a.cols[e];
          if (y > top) break;  // ascending: no later neighbour is in list[0, i)
          const int j = lower_bound_u32(list, i, y);
          if (list[j] != y) continue;
          if constexpr (MODE == MODE_SEQ) {
            atomicOr(&rows[(size_t)tri_off((uint32_t)i) + (j >> 5)], 1u << (j & 31));
          } else if constexpr (MODE == MODE_COUNT) {
            atomicOr(&rows[(size_t)i * W + (j >> 5)], 1u << (j & 31));
            atomicOr(&rows[(size_t)j * W + (i >> 5)], 1u << (i & 31));
          } else {
            const int ri = rank[i], rj = rank[j];
            const int lo = ri < rj ? ri : rj, hi = ri < rj ? rj : ri;
            atomicOr(&rows[(size_t)lo * W + (hi >> 5)], 1u << (hi & 31));
          }
        }
      }
      __syncthreads();
    }
    if constexpr (MODE == MODE_SEQ) {
      if (a.shared_loads)
        seq_streams_shared<K, WPL>(next, d, rows, list, s, a.out, s_off, reinterpret_cast<uint32_t *>(acc), dl,
                                   lane, a.err);
      else
        seq_streams<K, WPL>(next, d, rows, base, dl, acc, lane, a.err);
      __syncthreads();
      for (int i = tid; i <= d; i += NW * 32) {
        const unsigned long long v = acc[i];
        if (v) {
          // shared loads: already in the load vector, stream by stream
          if (!a.shared_loads) atomicAdd(&a.out[i < d ? list[i] : s], v);
          acc[i] = 0;
        }
      }
    } else {
      const int tau = (MODE == MODE_ORDER) ? s_tau : 0;
      unsigned long long mine = 0;
      for (;;) {
        int p = 0;
        if (lane == 0) p = (int)atomicAdd(next, 1u);
        p = __shfl_sync(KCL_FULL, p, 0);
        if (p >= d) break;
        const Bits<WPL> P = load_row<WPL>(rows, p, W, lane);
        uint64_t c = 0;
        uint64_t c_low = 0;
        if constexpr (K == 4 && WPL == 1 && ROWS_IN_SMEM) {
          c = warp_sum((uint64_t)edges_in<MODE == MODE_COUNT>(P, rows, W, lane, cbuf));
          if constexpr (MODE == MODE_COUNT)
            c_low = warp_sum((uint64_t)edges_in<true>(band(P, below_mask<WPL>(p, lane)), rows, W, lane, cbuf));
        } else if constexpr (K == 5 && WPL == 1 && ROWS_IN_SMEM) {
          c = warp_sum((uint64_t)triangles_in<MODE == MODE_COUNT>(P, rows, W, lane, cbuf));
          if constexpr (MODE == MODE_COUNT)
            c_low = warp_sum((uint64_t)triangles_in<true>(band(P, below_mask<WPL>(p, lane)), rows, W, lane, cbuf));
        } else {
          c = warp_sum(cnt_warp<K - 2, MODE == MODE_COUNT, WPL>(P, rows, W, lane));
          if constexpr (MODE == MODE_COUNT) {
            // s's own share: the (k-1)-cliques of G_s whose largest member is p,
            // i.e. the (k-2)-cliques among p's neighbours below it.  Summing
            // these (instead of dividing the row total by k-1) stays exact when
            // several CTAs split one root.
            c_low = warp_sum(cnt_warp<K - 2, true, WPL>(band(P, below_mask<WPL>(p, lane)), rows, W, lane));
          }
        }
        if (lane == 0) {
          if (MODE == MODE_COUNT) {
            if (a.list_off) a.pair_out[o + p] = (unsigned long long)c;
            else if (c) atomicAdd(&a.out[list[p]], (unsigned long long)c);
            mine += c_low;
          } else if (p < tau) {
            if (c) atomicAdd(&a.out[list[inv[p]]], (unsigned long long)c);
          } else {
            mine += c;
          }
        }
      }
      if (lane == 0 && mine) atomicAdd(&s_sum, mine);
      __syncthreads();
      if (tid == 0 && s_sum && !(MODE == MODE_COUNT && a.list_off)) {
        atomicAdd(&a.out[s], s_sum);
        if constexpr (IDENT && MODE == MODE_COUNT) atomicAdd(a.total, s_sum);
      }
    }
    if (tid == 0 && a.active) a.active[blockIdx.x] = UINT32_MAX;
    __syncthreads();
  }
}

}  // namespace dev

// Per-kernel launch settings, computed once per (device, kernel, dynamic
// shared memory size): the opt-in shared-memory attribute (a per-device
// setting: cudaFuncSetAttribute applies to the current device only) and the
// number of CTAs one SM holds.  Launches then cost no runtime queries.
constexpr int kMaxDevices = 64;
struct LaunchCache {
  std::mutex mu;
  int attr_bytes[kMaxDevices];
  size_t occ_smem[64];  // fixed storage: launching never touches the heap
  int occ_dev[64];
  int occ_threads[64];
  int occ_ctas[64];
  int nocc = 0;
  // Seq tiers M / L: chosen warps per CTA by (device, out-degree bound, requested width).
  uint32_t nw_dmax[32];
  int nw_dev[32], nw_req[32], nw_val[32];
  int nnw = 0;
  LaunchCache() {
    for (int i = 0; i < kMaxDevices; ++i) attr_bytes[i] = -1;
  }
};

static inline int current_device() {
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= kMaxDevices) d = 0;
  return d;
}

template <typename Fn>
static cudaError_t prepare(Fn fn, LaunchCache &lc, int threads, size_t smem, int *per_sm) {
  const int dev = current_device();
  std::lock_guard<std::mutex> g(lc.mu);
  if ((int)smem > lc.attr_bytes[dev]) {
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    lc.attr_bytes[dev] = (int)smem;
  }
  for (int i = 0; i < lc.nocc; ++i)
    if (lc.occ_dev[i] == dev && lc.occ_smem[i] == smem && lc.occ_threads[i] == threads) {
      *per_sm = lc.occ_ctas[i];
      return cudaSuccess;
    }
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, threads, smem) != cudaSuccess || nb < 1) nb = 1;
  if (lc.nocc < 64) {
    lc.occ_dev[lc.nocc] = dev;
    lc.occ_smem[lc.nocc] = smem;
    lc.occ_threads[lc.nocc] = threads;
    lc.occ_ctas[lc.nocc] = nb;
    ++lc.nocc;
  }
  *per_sm = nb;
  return cudaSuccess;
}

// Warps per CTA of a tier M / L launch: `req` when nonzero, else the width
// that keeps the most warps resident per SM at this out-degree bound (ties:
// the narrower, i.e. more CTAs).  Seq: 8..24 in steps of 4, and on request 2
// or 4 (many small CTAs for groups of small roots, where a root has few root
// edges to share out); the counting kernels: 8..32 in steps of 8.
template <int MODE, int K, typename Fn>
static cudaError_t pick_warps(Fn fn, LaunchCache &lc, uint32_t dmax, bool rows_in_smem, int req, int *nw) {
  using namespace dev;
  constexpr int hi = warps_m<MODE, K>(), step = MODE == MODE_SEQ ? 4 : 8;
  const int lo = (MODE == MODE_SEQ && (req == 2 || req == 4)) ? req : 8;
  const int dev = current_device();
  {
    std::lock_guard<std::mutex> g(lc.mu);
    for (int i = 0; i < lc.nnw; ++i)
      if (lc.nw_dev[i] == dev && lc.nw_dmax[i] == dmax && lc.nw_req[i] == req) {
        *nw = lc.nw_val[i];
        return cudaSuccess;
      }
  }
  int best = 0, best_warps = -1;
  for (int w = lo; w <= hi; w = w < 8 ? w * 2 : w + step) {
    if (req > 0 && w != req) continue;
    const size_t sm = layout_m(MODE, K, dmax, w, rows_in_smem).total;
    if (sm > 227 * 1024) continue;
    int per_sm = 0;
    cudaError_t e = prepare(fn, lc, w * 32, sm, &per_sm);
    if (e != cudaSuccess) return e;
    if (per_sm * w > best_warps) { best_warps = per_sm * w; best = w; }
  }
  if (best == 0) best = req > hi ? hi : lo;  // a width this launch cannot take: the nearest one
  std::lock_guard<std::mutex> g(lc.mu);
  if (lc.nnw < 32) {
    lc.nw_dev[lc.nnw] = dev;
    lc.nw_dmax[lc.nnw] = dmax;
    lc.nw_req[lc.nnw] = req;
    lc.nw_val[lc.nnw] = best;
    ++lc.nnw;
  }
  *nw = best;
  return cudaSuccess;
}

// Persistent grid: as many CTAs as are resident at once.  Tier S needs no
// more warps than roots; tiers M and L keep every resident CTA, because a CTA
// without a root of its own steals sub-tasks from the unfinished roots.
static int persistent_grid(int per_sm, const TierLaunch &t, int roots_per_cta, bool steals) {
  long long g = (long long)per_sm * t.num_sms;
  if (!steals) {
    const long long need = ((long long)t.num_roots + roots_per_cta - 1) / roots_per_cta;
    if (need < g) g = need;
  }
  if (t.max_grid > 0 && g > t.max_grid) g = t.max_grid;
  if (steals && g > (long long)kActiveSlots) g = kActiveSlots;  // one registry slot per CTA
  return (int)(g < 1 ? 1 : g);
}

template <int MODE, int K>
cudaError_t launch_tier(const TierLaunch &t, dev::PassArgs a, cudaStream_t st) {
  using namespace dev;
  a.roots = t.roots;
  a.num_roots = t.num_roots;
  a.dmax = t.dmax;
  a.work = t.work;
  a.task_next = t.task_next;
  a.active = t.active;
  if (t.num_roots == 0) return cudaSuccess;
  int per_sm = 1;
  if (t.tier == 0) {
    static LaunchCache lc;
    const size_t sm = sizeof(SmemS<MODE>) * kWarpsS;
    auto fn = tier_s_kernel<MODE, K>;
    cudaError_t e = prepare(fn, lc, kWarpsS * 32, sm, &per_sm);
    if (e != cudaSuccess) return e;
    fn<<<persistent_grid(per_sm, t, kWarpsS, false), kWarpsS * 32, sm, st>>>(a);
    return cudaGetLastError();
  }
  if (t.tier == 1) {
    static LaunchCache lc;
    auto fn = tier_m_kernel<MODE, K, 1, true>;
    int nw = kWarpsM;
    cudaError_t e = pick_warps<MODE, K>(fn, lc, t.dmax, true, t.warps, &nw);
    if (e != cudaSuccess) return e;
    const size_t sm = layout_m(MODE, K, t.dmax, nw, true).total;
    e = prepare(fn, lc, nw * 32, sm, &per_sm);
    if (e != cudaSuccess) return e;
    fn<<<persistent_grid(per_sm, t, 1, t.active != nullptr), nw * 32, sm, st>>>(a);
    return cudaGetLastError();
  }
  static LaunchCache lc;
  auto fn = tier_m_kernel<MODE, K, 2, false>;
  int nw = kWarpsM;
  cudaError_t e = pick_warps<MODE, K>(fn, lc, t.dmax, false, t.warps, &nw);
  if (e != cudaSuccess) return e;
  const size_t sm = layout_m(MODE, K, t.dmax, nw, false).total;
  e = prepare(fn, lc, nw * 32, sm, &per_sm);
  if (e != cudaSuccess) return e;
  fn<<<persistent_grid(per_sm, t, 1, t.active != nullptr), nw * 32, sm, st>>>(a);
  return cudaGetLastError();
}

template <int MODE>
cudaError_t launch_mode(int k, const TierLaunch &t, dev::PassArgs a, cudaStream_t st) {
  switch (k) {
    case 2: if constexpr (MODE == dev::MODE_ORDER) return launch_tier<MODE, 2>(t, a, st); else break;
    case 3: return launch_tier<MODE, 3>(t, a, st);
    case 4: return launch_tier<MODE, 4>(t, a, st);
    case 5: return launch_tier<MODE, 5>(t, a, st);
    case 6: return launch_tier<MODE, 6>(t, a, st);
    case 7: return launch_tier<MODE, 7>(t, a, st);
    case 8: return launch_tier<MODE, 8>(t, a, st);
    default: break;
  }
  return cudaErrorInvalidValue;
}

}  // namespace kclpp
