// kclpp_gen.cpp -- edge-list I/O and seeded synthetic graph generators.
//
// Input side of the path: ReadEdgeList (Graph.c:34-53) and the seeded graphs
// that stand in for the paper's datasets (Chung-Lu, RMAT, Erdos-Renyi, planted
// dense communities).  All arithmetic is plain IEEE double with no fused
// multiply-add (the library is built with -ffp-contract=off), so a seed gives
// the same graph on x86 and Arm hosts.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <thread>
#include <vector>

#include "kclpp_internal.h"

namespace kclpp {

static thread_local std::string g_last_error;

kclpp_status set_error(kclpp_status s, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return s;
}
void clear_error() { g_last_error.clear(); }
const char *last_error_cstr() { return g_last_error.c_str(); }

void radix_sort_u64(std::vector<uint64_t> &keys) {
  const size_t n = keys.size();
  if (n < 2) return;
  uint64_t orv = 0, andv = ~0ull;
  for (uint64_t k : keys) { orv |= k; andv &= k; }
  const uint64_t vary = orv ^ andv;
  std::vector<uint64_t> tmp(n);
  std::vector<size_t> cnt(1 << 16);
  for (int shift = 0; shift < 64; shift += 16) {
    if (((vary >> shift) & 0xFFFFull) == 0) continue;
    std::fill(cnt.begin(), cnt.end(), 0);
    for (uint64_t k : keys) cnt[(k >> shift) & 0xFFFF]++;
    size_t sum = 0;
    for (auto &c : cnt) { size_t t = c; c = sum; sum += t; }
    for (uint64_t k : keys) tmp[cnt[(k >> shift) & 0xFFFF]++] = k;
    keys.swap(tmp);
  }
}

// Vose alias table for O(1) weighted sampling.
struct Alias {
  std::vector<double> prob;
  std::vector<uint32_t> alias;
  explicit Alias(const std::vector<double> &w) {
    const size_t n = w.size();
    prob.assign(n, 0.0);
    alias.assign(n, 0);
    double total = 0;
    for (double x : w) total += x;
    std::vector<double> p(n);
    std::vector<uint32_t> small, large;
    for (size_t i = 0; i < n; ++i) {
      p[i] = w[i] * (double)n / total;
      (p[i] < 1.0 ? small : large).push_back((uint32_t)i);
    }
    while (!small.empty() && !large.empty()) {
      uint32_t s = small.back(); small.pop_back();
      uint32_t l = large.back(); large.pop_back();
      prob[s] = p[s];
      alias[s] = l;
      p[l] = (p[l] + p[s]) - 1.0;
      (p[l] < 1.0 ? small : large).push_back(l);
    }
    for (uint32_t l : large) prob[l] = 1.0;
    for (uint32_t s : small) prob[s] = 1.0;
  }
  inline uint32_t draw(SplitMix &r) const {
    uint32_t i = (uint32_t)r.below(prob.size());
    return r.uniform() < prob[i] ? i : alias[i];
  }
};

// Canonicalise: (min, max), no self loops, sorted, deduplicated.
static void finish(std::vector<uint64_t> &keys, uint32_t n, kclpp_edge_list *el) {
  radix_sort_u64(keys);
  keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
  el->pairs.resize(keys.size() * 2);
  uint32_t mx = 0;
  for (size_t i = 0; i < keys.size(); ++i) {
    uint32_t u = (uint32_t)(keys[i] >> 32), v = (uint32_t)keys[i];
    el->pairs[2 * i] = u;
    el->pairs[2 * i + 1] = v;
    mx = std::max(mx, std::max(u, v));
  }
  el->n = keys.empty() ? 1 : mx + 1;
  (void)n;
}

static inline uint64_t pack(uint32_t u, uint32_t v) {
  if (u > v) std::swap(u, v);
  return ((uint64_t)u << 32) | v;
}

static std::vector<uint32_t> permutation(uint32_t n, SplitMix &r) {
  std::vector<uint32_t> p(n);
  std::iota(p.begin(), p.end(), 0u);
  for (uint32_t i = n; i > 1; --i) std::swap(p[i - 1], p[r.below(i)]);
  return p;
}

static void chung_lu_keys(uint32_t n, double avg, double gamma, SplitMix &r,
                          const std::vector<uint32_t> &perm, std::vector<uint64_t> &keys) {
  std::vector<double> w(n);
  const double ex = -1.0 / (gamma - 1.0);
  for (uint32_t i = 0; i < n; ++i) w[i] = std::pow((double)(i + 1), ex);
  Alias al(w);
  const uint64_t samples = (uint64_t)std::llround((double)n * avg / 2.0);
  keys.reserve(keys.size() + samples);
  for (uint64_t i = 0; i < samples; ++i) {
    uint32_t u = al.draw(r), v = al.draw(r);
    if (u == v) continue;
    keys.push_back(pack(perm[u], perm[v]));
  }
}

}  // namespace kclpp

using namespace kclpp;

extern "C" {

static bool planted_ok(const kclpp_gen_params *p) {
  return p->comm_min >= 2 && p->comm_max >= p->comm_min && p->p_in > 0 && p->p_in <= 1.0;
}

// Planted G(n_c, p_in) communities: disjoint slices of a fresh permutation,
// sizes log-uniform in [comm_min, comm_max]; stops at the first that no longer fits.
static void plant(uint32_t n, const kclpp_gen_params *p, SplitMix &rng, std::vector<uint64_t> &keys) {
  auto members = permutation(n, rng);
  uint64_t at = 0;
  const double lmin = std::log((double)p->comm_min), lmax = std::log((double)p->comm_max);
  for (uint32_t c = 0; c < p->communities; ++c) {
    uint32_t sz = (uint32_t)std::llround(std::exp(lmin + (lmax - lmin) * rng.uniform()));
    if (at + sz > n) break;
    for (uint32_t i = 0; i < sz; ++i)
      for (uint32_t j = i + 1; j < sz; ++j)
        if (rng.uniform() < p->p_in) keys.push_back(pack(members[at + i], members[at + j]));
    at += sz;
  }
}

kclpp_status kclpp_generate(const kclpp_gen_params *p, kclpp_edge_list **out) {
  if (!p || !out) return set_error(KCLPP_ERR_INVALID, "kclpp_generate: null argument");
  *out = nullptr;
  SplitMix rng(p->seed * 0x2545F4914F6CDD1Dull + 0x1234567ull);
  std::vector<uint64_t> keys;
  uint32_t n = p->n;
  try {
    switch (p->kind) {
      case KCLPP_GEN_CHUNG_LU: {
        if (n < 2 || !(p->avg_degree > 0) || !(p->gamma > 1.0))
          return set_error(KCLPP_ERR_INVALID, "chung-lu: need n >= 2, avg_degree > 0, gamma > 1");
        auto perm = permutation(n, rng);
        chung_lu_keys(n, p->avg_degree, p->gamma, rng, perm, keys);
        break;
      }
      case KCLPP_GEN_ER: {
        if (n < 2 || !(p->avg_degree > 0))
          return set_error(KCLPP_ERR_INVALID, "er: need n >= 2, avg_degree > 0");
        const uint64_t samples = (uint64_t)std::llround((double)n * p->avg_degree / 2.0);
        keys.reserve(samples);
        for (uint64_t i = 0; i < samples; ++i) {
          uint32_t u = (uint32_t)rng.below(n), v = (uint32_t)rng.below(n);
          if (u != v) keys.push_back(pack(u, v));
        }
        break;
      }
      case KCLPP_GEN_RMAT:
      case KCLPP_GEN_RMAT_PLANTED: {
        if (p->scale < 1 || p->scale > 31 || p->edge_factor < 1)
          return set_error(KCLPP_ERR_INVALID, "rmat: need 1 <= scale <= 31, edge_factor >= 1");
        if (p->kind == KCLPP_GEN_RMAT_PLANTED && !planted_ok(p))
          return set_error(KCLPP_ERR_INVALID, "rmat-planted: bad community parameters");
        const double a = p->a, ab = p->a + p->b, abc = p->a + p->b + p->c;
        if (!(a >= 0 && ab >= a && abc >= ab && abc <= 1.0))
          return set_error(KCLPP_ERR_INVALID, "rmat: bad quadrant probabilities");
        n = 1u << p->scale;
        const uint64_t samples = (uint64_t)p->edge_factor << p->scale;
        keys.reserve(samples);
        for (uint64_t i = 0; i < samples; ++i) {
          uint32_t u = 0, v = 0;
          for (uint32_t l = 0; l < p->scale; ++l) {
            double x = rng.uniform();
            uint32_t bu = 0, bv = 0;
            if (x < a) { }
            else if (x < ab) bv = 1;
            else if (x < abc) bu = 1;
            else { bu = 1; bv = 1; }
            u = (u << 1) | bu;
            v = (v << 1) | bv;
          }
          if (u != v) keys.push_back(pack(u, v));
        }
        // Scramble ids so that id order carries no degree information.
        auto perm = permutation(n, rng);
        for (auto &k : keys) k = pack(perm[(uint32_t)(k >> 32)], perm[(uint32_t)k]);
        if (p->kind == KCLPP_GEN_RMAT_PLANTED) plant(n, p, rng, keys);
        break;
      }
      case KCLPP_GEN_PLANTED: {
        if (n < 2 || !(p->avg_degree > 0) || !(p->gamma > 1.0) || !planted_ok(p))
          return set_error(KCLPP_ERR_INVALID, "planted: bad parameters");
        auto perm = permutation(n, rng);
        chung_lu_keys(n, p->avg_degree, p->gamma, rng, perm, keys);
        plant(n, p, rng, keys);
        break;
      }
      default:
        return set_error(KCLPP_ERR_INVALID, "kclpp_generate: unknown kind %d", p->kind);
    }
    auto *el = new kclpp_edge_list();
    finish(keys, n, el);
    *out = el;
  } catch (const std::bad_alloc &) {
    return set_error(KCLPP_ERR_NOMEM, "kclpp_generate: out of host memory");
  }
  return KCLPP_OK;
}

// Edge-list text parsing (ReadEdgeList, Graph.c:34-53: fscanf("%u %u") until it
// fails): whitespace-separated decimal numbers, read in pairs; reading stops
// at the first character that is neither a digit nor whitespace, or at a
// number above 2^32 - 1.  A number that such a character ends, and a last
// unpaired number, are dropped; a number that the end of the file ends counts.
namespace {

inline bool is_space(char c) { return c == ' ' || c == '\n' || c == '\t' || c == '\r'; }

// Numbers of buf[lo, hi) (hi is a whitespace position or the end of the
// file).  Returns false if the chunk holds a stop (bad character or
// overflow); the numbers before the stop are kept.
bool scan_chunk(const char *buf, size_t lo, size_t hi, std::vector<uint32_t> &out) {
  uint64_t cur = 0;
  bool innum = false;
  for (size_t i = lo; i < hi; ++i) {
    const char c = buf[i];
    if (c >= '0' && c <= '9') {
      cur = cur * 10 + (uint64_t)(c - '0');
      if (cur > 0xFFFFFFFFull) return false;
      innum = true;
    } else if (is_space(c)) {
      if (innum) out.push_back((uint32_t)cur);
      cur = 0;
      innum = false;
    } else {
      return false;
    }
  }
  // hi is whitespace (the next chunk starts there) or the end of the file
  if (innum) out.push_back((uint32_t)cur);
  return true;
}

}  // namespace

kclpp_status kclpp_read_edge_list_mt(const char *path, int threads, kclpp_edge_list **out) {
  if (!path || !out) return set_error(KCLPP_ERR_INVALID, "kclpp_read_edge_list: null argument");
  *out = nullptr;
  FILE *f = fopen(path, "rb");
  if (!f) return set_error(KCLPP_ERR_IO, "cannot open %s", path);
  std::vector<char> buf;
  long len = -1;
  if (fseek(f, 0, SEEK_END) == 0) {
    len = ftell(f);
    fseek(f, 0, SEEK_SET);
  }
  if (len > 0) {  // one read into a buffer of the file's size, then whatever follows
    buf.resize((size_t)len);
    buf.resize(fread(buf.data(), 1, buf.size(), f));
  }
  {
    std::vector<char> chunk(1 << 20);
    size_t got;
    while ((got = fread(chunk.data(), 1, chunk.size(), f)) > 0) buf.insert(buf.end(), chunk.data(), chunk.data() + got);
  }
  fclose(f);
  const size_t size = buf.size();
  if (threads <= 0) {
    const unsigned hc = std::thread::hardware_concurrency();
    threads = size < (8u << 20) ? 1 : (int)std::min<unsigned>(hc ? hc : 1, 16);
  }
  // Chunk starts at whitespace positions, so that no number spans two chunks.
  std::vector<size_t> cut{0};
  for (int t = 1; t < threads; ++t) {
    size_t p = std::max(cut.back(), size * (size_t)t / (size_t)threads);
    while (p < size && !is_space(buf[p])) ++p;
    if (p >= size) break;
    if (p > cut.back()) cut.push_back(p);
  }
  cut.push_back(size);
  const size_t nc = cut.size() - 1;
  std::vector<std::vector<uint32_t>> nums(nc);
  std::vector<char> clean(nc, 1);
  auto scan = [&](size_t c) {
    nums[c].reserve((cut[c + 1] - cut[c]) / 6 + 16);
    clean[c] = scan_chunk(buf.data(), cut[c], cut[c + 1], nums[c]);
  };
  if (nc == 1) {
    scan(0);
  } else {
    std::vector<std::thread> pool;
    for (size_t c = 0; c < nc; ++c) pool.emplace_back(scan, c);
    for (auto &th : pool) th.join();
  }
  // The numbers up to the first stop, paired in order.
  size_t used = nc, total = 0;
  for (size_t c = 0; c < nc; ++c) {
    total += nums[c].size();
    if (!clean[c]) { used = c + 1; break; }
  }
  const size_t np = total / 2;
  auto *el = new kclpp_edge_list();
  el->pairs.resize(2 * np);
  std::vector<size_t> at(used + 1, 0);
  for (size_t c = 0; c < used; ++c) at[c + 1] = std::min(at[c] + nums[c].size(), 2 * np);
  std::vector<uint32_t> mxs(used, 0);
  auto place = [&](size_t c) {
    const size_t take = at[c + 1] - at[c];
    uint32_t m = 0;
    for (size_t i = 0; i < take; ++i) {
      const uint32_t v = nums[c][i];
      el->pairs[at[c] + i] = v;
      m = v > m ? v : m;
    }
    mxs[c] = m;
  };
  if (used == 1) {
    place(0);
  } else {
    std::vector<std::thread> pool;
    for (size_t c = 0; c < used; ++c) pool.emplace_back(place, c);
    for (auto &th : pool) th.join();
  }
  uint32_t mx = 0;
  for (uint32_t m : mxs) mx = std::max(mx, m);
  el->n = np ? mx + 1 : 1;
  *out = el;
  return KCLPP_OK;
}

kclpp_status kclpp_read_edge_list(const char *path, kclpp_edge_list **out) {
  return kclpp_read_edge_list_mt(path, 0, out);
}

kclpp_status kclpp_edge_list_create(const uint32_t *pairs, uint64_t e, kclpp_edge_list **out) {
  if (!out || (!pairs && e)) return set_error(KCLPP_ERR_INVALID, "kclpp_edge_list_create: null argument");
  auto *el = new kclpp_edge_list();
  el->pairs.assign(pairs, pairs + 2 * e);
  uint32_t mx = 0;
  for (uint32_t v : el->pairs) mx = std::max(mx, v);
  el->n = mx + 1;
  *out = el;
  return KCLPP_OK;
}

kclpp_status kclpp_edge_list_info(const kclpp_edge_list *el, uint32_t *n, uint64_t *e) {
  if (!el) return set_error(KCLPP_ERR_INVALID, "null edge list");
  if (n) *n = el->n;
  if (e) *e = el->e();
  return KCLPP_OK;
}

kclpp_status kclpp_edge_list_copy(const kclpp_edge_list *el, uint32_t *pairs_out) {
  if (!el || !pairs_out) return set_error(KCLPP_ERR_INVALID, "null argument");
  if (!el->pairs.empty()) memcpy(pairs_out, el->pairs.data(), el->pairs.size() * sizeof(uint32_t));
  return KCLPP_OK;
}

kclpp_status kclpp_write_edge_list(const kclpp_edge_list *el, const char *path) {
  if (!el || !path) return set_error(KCLPP_ERR_INVALID, "null argument");
  FILE *f = fopen(path, "w");
  if (!f) return set_error(KCLPP_ERR_IO, "cannot open %s for writing", path);
  std::vector<char> buf;
  buf.reserve(1 << 22);
  char tmp[32];
  for (uint64_t i = 0; i < el->e(); ++i) {
    int len = snprintf(tmp, sizeof tmp, "%u %u\n", el->pairs[2 * i], el->pairs[2 * i + 1]);
    buf.insert(buf.end(), tmp, tmp + len);
    if (buf.size() > (1 << 22) - 64) { fwrite(buf.data(), 1, buf.size(), f); buf.clear(); }
  }
  if (!buf.empty()) fwrite(buf.data(), 1, buf.size(), f);
  int rc = fclose(f);
  return rc == 0 ? KCLPP_OK : set_error(KCLPP_ERR_IO, "write failed: %s", path);
}

void kclpp_edge_list_free(kclpp_edge_list *el) { delete el; }

}  // extern "C"
