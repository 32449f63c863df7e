// sample_emul.cpp -- host build of the sampling kernels' per-thread code
// (kclistpp_gb300/csrc/kclpp_sample.cuh), for tests without a GPU.
//
// Runs what one CTA of the sampling kernel runs for every root -- the out-list
// and keys, the bitmap rows, then every root edge's clique tree -- with the
// same functions, the same row stride and the same kept-row writer, one root
// at a time.  The "++" wave pass and the max-rank push use the kernels'
// per-clique functions.  Compiled by tests/test_sampling_host.py.
#include <algorithm>
#include <cstdint>
#include <vector>

#include "../kclistpp_gb300/csrc/kclpp_sample.cuh"

using namespace kclpp;

namespace {

template <int K>
struct HostEmit {
  const uint32_t *list;
  uint32_t s;
  uint32_t *rows;
  uint8_t *wave;
  uint64_t cap;
  uint64_t *count;
  uint64_t threshold;
  bool all;
  uint32_t waves;
  void operator()(uint64_t h, const uint32_t *path, uint32_t v) const {
    if (!smp::kept(h, threshold, all)) return;
    const uint64_t pos = (*count)++;
    if (pos >= cap) return;
    smp::write_row<K>(rows + pos * K, list, s, path, v);
    wave[pos] = (uint8_t)smp::wave_of(h, waves);
  }
};

template <int K>
uint64_t sample_k(uint32_t n, const uint64_t *off, const uint32_t *cols, uint32_t dmax, uint64_t seed,
                  uint64_t threshold, int all, uint32_t waves, uint32_t *rows, uint8_t *wave, uint64_t cap) {
  const uint32_t ws = (dmax + 31) / 32;
  std::vector<uint64_t> keys(dmax + 1);
  std::vector<uint32_t> list(dmax + 1), bits((size_t)(dmax + 1) * ws);
  uint64_t count = 0;
  for (uint32_t s = 0; s < n; ++s) {
    const uint32_t d = (uint32_t)(off[s + 1] - off[s]);
    if (d < (uint32_t)(K - 1)) continue;
    for (uint32_t i = 0; i < d; ++i) {
      list[i] = cols[off[s] + i];
      keys[i] = smp::vertex_key(seed, list[i]);
    }
    // Fill the rows with a pattern first: the walk must read only the words
    // build_row writes.
    std::fill(bits.begin(), bits.end(), 0xA5A5A5A5u);
    for (uint32_t i = 0; i < d; ++i) smp::build_row(i, list.data(), off, cols, bits.data() + (size_t)i * ws);
    HostEmit<K> em{list.data(), s, rows, wave, cap, &count, threshold, all != 0, waves};
    const uint64_t hs = smp::vertex_key(seed, s);
    for (uint32_t t = K - 2; t < d; ++t) smp::edge_cliques<K>(t, hs, bits.data(), ws, keys.data(), em);
  }
  return count;
}

}  // namespace

extern "C" {

uint64_t emul_sample(uint32_t n, const uint64_t *off, const uint32_t *cols, int k, uint32_t dmax, uint64_t seed,
                     uint64_t threshold, int all, uint32_t waves, uint32_t *rows, uint8_t *wave, uint64_t cap) {
  switch (k) {
    case 3: return sample_k<3>(n, off, cols, dmax, seed, threshold, all, waves, rows, wave, cap);
    case 4: return sample_k<4>(n, off, cols, dmax, seed, threshold, all, waves, rows, wave, cap);
    case 5: return sample_k<5>(n, off, cols, dmax, seed, threshold, all, waves, rows, wave, cap);
    case 6: return sample_k<6>(n, off, cols, dmax, seed, threshold, all, waves, rows, wave, cap);
    case 7: return sample_k<7>(n, off, cols, dmax, seed, threshold, all, waves, rows, wave, cap);
    case 8: return sample_k<8>(n, off, cols, dmax, seed, threshold, all, waves, rows, wave, cap);
    default: return 0;
  }
}

// One wave pass as the two kernels run it: per wave, every clique of the wave
// credits its argmin against the values before the wave, then the credits are
// added.
void emul_pass(uint32_t n, int k, uint64_t S, const uint32_t *rows, const uint8_t *wave, uint32_t waves,
               uint32_t *rho) {
  std::vector<uint32_t> delta(n, 0);
  for (uint32_t w = 0; w < waves; ++w) {
    for (uint64_t i = 0; i < S; ++i)
      if (wave[i] == w) ++delta[smp::argmin_member(rows + i * (uint64_t)k, k, rho)];
    for (uint32_t v = 0; v < n; ++v) {
      rho[v] += delta[v];
      delta[v] = 0;
    }
  }
}

void emul_push(int k, uint64_t S, const uint32_t *rows, const uint32_t *rank, uint32_t *push) {
  for (uint64_t i = 0; i < S; ++i) ++push[smp::max_rank(rows + i * (uint64_t)k, k, rank)];
}

}  // extern "C"
