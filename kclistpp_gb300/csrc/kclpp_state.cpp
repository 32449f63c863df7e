// kclpp_state.cpp -- checkpoints of a run: the r (Seq) or rho (Sim) vector with
// the passes done, k and a hash of the DAG, so that a run resumes where it
// stopped (the reference only has a commented-out dump of r,
// kCDensestNoAtom.c:398-401); binary edge lists; tuned schedules.  Host only.
//
// File layout (little-endian): "KCLPPST1", u32 kind, u32 k, u32 passes, u32 n,
// u64 graph hash, n x 8 bytes of the vector, u64 checksum (FNV-1a of every
// byte before it).
#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>

#include "kclpp_internal.h"

using namespace kclpp;

namespace {

constexpr char kMagic[8] = {'K', 'C', 'L', 'P', 'P', 'S', 'T', '1'};
constexpr size_t kHeader = 8 + 4 * 4 + 8;

uint64_t fnv1a(const unsigned char *p, size_t n, uint64_t h = 0xcbf29ce484222325ull) {
  for (size_t i = 0; i < n; ++i) {
    h ^= p[i];
    h *= 0x100000001b3ull;
  }
  return h;
}

void put32(unsigned char *p, uint32_t v) {
  for (int i = 0; i < 4; ++i) p[i] = (unsigned char)(v >> (8 * i));
}
void put64(unsigned char *p, uint64_t v) {
  for (int i = 0; i < 8; ++i) p[i] = (unsigned char)(v >> (8 * i));
}
uint32_t get32(const unsigned char *p) {
  uint32_t v = 0;
  for (int i = 0; i < 4; ++i) v |= (uint32_t)p[i] << (8 * i);
  return v;
}
uint64_t get64(const unsigned char *p) {
  uint64_t v = 0;
  for (int i = 0; i < 8; ++i) v |= (uint64_t)p[i] << (8 * i);
  return v;
}

}  // namespace

extern "C" {

kclpp_status kclpp_save_state(const char *path, const kclpp_state_info *info, const void *vec) {
  if (!path || !info || (!vec && info->n)) return set_error(KCLPP_ERR_INVALID, "kclpp_save_state: null argument");
  if (info->kind != KCLPP_KERNEL_SEQ && info->kind != KCLPP_KERNEL_ORDER)
    return set_error(KCLPP_ERR_INVALID, "kclpp_save_state: kind must be KCLPP_KERNEL_SEQ or KCLPP_KERNEL_ORDER");
  std::vector<unsigned char> buf(kHeader + (size_t)info->n * 8 + 8);
  memcpy(buf.data(), kMagic, 8);
  put32(&buf[8], (uint32_t)info->kind);
  put32(&buf[12], (uint32_t)info->k);
  put32(&buf[16], info->passes);
  put32(&buf[20], info->n);
  put64(&buf[24], info->graph_hash);
  const unsigned char *src = static_cast<const unsigned char *>(vec);
  for (uint32_t i = 0; i < info->n; ++i) {
    uint64_t v;
    memcpy(&v, src + (size_t)i * 8, 8);  // u64 or the f64 bit pattern
    put64(&buf[kHeader + (size_t)i * 8], v);
  }
  put64(&buf[buf.size() - 8], fnv1a(buf.data(), buf.size() - 8));
  FILE *f = fopen(path, "wb");
  if (!f) return set_error(KCLPP_ERR_IO, "cannot open %s for writing", path);
  const size_t w = fwrite(buf.data(), 1, buf.size(), f);
  const int rc = fclose(f);
  if (w != buf.size() || rc != 0) return set_error(KCLPP_ERR_IO, "write failed: %s", path);
  return KCLPP_OK;
}

kclpp_status kclpp_load_state(const char *path, kclpp_state_info *info, void *vec, uint32_t cap) {
  if (!path || !info) return set_error(KCLPP_ERR_INVALID, "kclpp_load_state: null argument");
  FILE *f = fopen(path, "rb");
  if (!f) return set_error(KCLPP_ERR_IO, "cannot open %s", path);
  std::vector<unsigned char> buf;
  unsigned char chunk[1 << 16];
  size_t got;
  while ((got = fread(chunk, 1, sizeof chunk, f)) > 0) buf.insert(buf.end(), chunk, chunk + got);
  fclose(f);
  if (buf.size() < kHeader + 8 || memcmp(buf.data(), kMagic, 8) != 0)
    return set_error(KCLPP_ERR_IO, "%s is not a kclpp checkpoint", path);
  const uint32_t n = get32(&buf[20]);
  if (buf.size() != kHeader + (size_t)n * 8 + 8) return set_error(KCLPP_ERR_IO, "%s: truncated checkpoint", path);
  if (get64(&buf[buf.size() - 8]) != fnv1a(buf.data(), buf.size() - 8))
    return set_error(KCLPP_ERR_IO, "%s: checksum mismatch", path);
  info->kind = (int)get32(&buf[8]);
  info->k = (int)get32(&buf[12]);
  info->passes = get32(&buf[16]);
  info->n = n;
  info->graph_hash = get64(&buf[24]);
  if (vec) {
    if (cap < n) return set_error(KCLPP_ERR_INVALID, "kclpp_load_state: the vector holds %u entries, %u needed", cap, n);
    unsigned char *dst = static_cast<unsigned char *>(vec);
    for (uint32_t i = 0; i < n; ++i) {
      const uint64_t v = get64(&buf[kHeader + (size_t)i * 8]);
      memcpy(dst + (size_t)i * 8, &v, 8);
    }
  }
  return KCLPP_OK;
}

// Binary edge lists: "KCLPPEL1", u32 n, u64 e, 2e x u32 pairs, u64 checksum
// (FNV-1a of every byte before it).  A cache of a parsed text file.
kclpp_status kclpp_write_edge_list_bin(const kclpp_edge_list *el, const char *path) {
  if (!el || !path) return set_error(KCLPP_ERR_INVALID, "kclpp_write_edge_list_bin: null argument");
  const uint64_t e = el->e();
  std::vector<unsigned char> buf(8 + 4 + 8 + (size_t)e * 8 + 8);
  memcpy(buf.data(), "KCLPPEL1", 8);
  put32(&buf[8], el->n);
  put64(&buf[12], e);
  for (size_t i = 0; i < el->pairs.size(); ++i) put32(&buf[20 + 4 * i], el->pairs[i]);
  put64(&buf[buf.size() - 8], fnv1a(buf.data(), buf.size() - 8));
  FILE *f = fopen(path, "wb");
  if (!f) return set_error(KCLPP_ERR_IO, "cannot open %s for writing", path);
  const size_t w = fwrite(buf.data(), 1, buf.size(), f);
  const int rc = fclose(f);
  if (w != buf.size() || rc != 0) return set_error(KCLPP_ERR_IO, "write failed: %s", path);
  return KCLPP_OK;
}

kclpp_status kclpp_read_edge_list_bin(const char *path, kclpp_edge_list **out) {
  if (!path || !out) return set_error(KCLPP_ERR_INVALID, "kclpp_read_edge_list_bin: null argument");
  *out = nullptr;
  FILE *f = fopen(path, "rb");
  if (!f) return set_error(KCLPP_ERR_IO, "cannot open %s", path);
  std::vector<unsigned char> buf;
  unsigned char chunk[1 << 16];
  size_t got;
  while ((got = fread(chunk, 1, sizeof chunk, f)) > 0) buf.insert(buf.end(), chunk, chunk + got);
  fclose(f);
  if (buf.size() < 28 || memcmp(buf.data(), "KCLPPEL1", 8) != 0)
    return set_error(KCLPP_ERR_IO, "%s is not a binary kclpp edge list", path);
  const uint64_t e = get64(&buf[12]);
  if (e > (buf.size() - 28) / 8 || buf.size() != 28 + (size_t)e * 8)
    return set_error(KCLPP_ERR_IO, "%s: truncated edge list", path);
  if (get64(&buf[buf.size() - 8]) != fnv1a(buf.data(), buf.size() - 8))
    return set_error(KCLPP_ERR_IO, "%s: checksum mismatch", path);
  const uint32_t n = get32(&buf[8]);
  std::unique_ptr<kclpp_edge_list> el(new kclpp_edge_list());
  el->n = n;
  el->pairs.resize((size_t)e * 2);
  // The checksum only catches accidental damage: a file written with a wrong
  // n passes it, and every later stage indexes arrays of n entries by these
  // ids, so each id is checked against n.
  for (size_t i = 0; i < el->pairs.size(); ++i) {
    const uint32_t v = get32(&buf[20 + 4 * i]);
    if (v >= n) return set_error(KCLPP_ERR_IO, "%s: vertex id %u is not below the stored n = %u", path, v, n);
    el->pairs[i] = v;
  }
  *out = el.release();
  return KCLPP_OK;
}

// Schedule cache: "KCLPPSC1", u64 graph hash, u32 k, u32 kernel, the 19
// 32-bit fields of kclpp_schedule in declaration order, u64 checksum (FNV-1a
// of every byte before it).
namespace {
constexpr size_t kSchedFields = 19;
constexpr size_t kSchedBytes = 8 + 8 + 4 + 4 + kSchedFields * 4 + 8;

void schedule_fields(const kclpp_schedule &sp, uint32_t *v) {
  size_t i = 0;
  v[i++] = sp.tier_s_max;
  v[i++] = sp.tier_s_max_seq;
  v[i++] = sp.m_split1;
  v[i++] = sp.m_split2;
  v[i++] = (uint32_t)sp.steal_seq;
  v[i++] = (uint32_t)sp.steal_count;
  v[i++] = sp.seq_waves;
  for (int j = 0; j < 4; ++j) v[i++] = sp.seq_warps[j];
  v[i++] = (uint32_t)sp.concurrent_tiers;
  for (int j = 0; j < 4; ++j) v[i++] = sp.count_warps[j];
  v[i++] = sp.seq_split1;
  v[i++] = sp.seq_split2;
  v[i++] = (uint32_t)sp.concurrent_count;
}

void schedule_from(const uint32_t *v, kclpp_schedule &sp) {
  size_t i = 0;
  sp.tier_s_max = v[i++];
  sp.tier_s_max_seq = v[i++];
  sp.m_split1 = v[i++];
  sp.m_split2 = v[i++];
  sp.steal_seq = (int)v[i++];
  sp.steal_count = (int)v[i++];
  sp.seq_waves = v[i++];
  for (int j = 0; j < 4; ++j) sp.seq_warps[j] = v[i++];
  sp.concurrent_tiers = (int)v[i++];
  for (int j = 0; j < 4; ++j) sp.count_warps[j] = v[i++];
  sp.seq_split1 = v[i++];
  sp.seq_split2 = v[i++];
  sp.concurrent_count = (int)v[i++];
}
}  // namespace

kclpp_status kclpp_schedule_save(const char *path, uint64_t graph_hash, int k, int kernel, const kclpp_schedule *sp) {
  if (!path || !sp) return set_error(KCLPP_ERR_INVALID, "kclpp_schedule_save: null argument");
  unsigned char buf[kSchedBytes];
  memcpy(buf, "KCLPPSC1", 8);
  put64(&buf[8], graph_hash);
  put32(&buf[16], (uint32_t)k);
  put32(&buf[20], (uint32_t)kernel);
  uint32_t v[kSchedFields];
  schedule_fields(*sp, v);
  for (size_t i = 0; i < kSchedFields; ++i) put32(&buf[24 + 4 * i], v[i]);
  put64(&buf[kSchedBytes - 8], fnv1a(buf, kSchedBytes - 8));
  FILE *f = fopen(path, "wb");
  if (!f) return set_error(KCLPP_ERR_IO, "cannot open %s for writing", path);
  const size_t w = fwrite(buf, 1, kSchedBytes, f);
  const int rc = fclose(f);
  if (w != kSchedBytes || rc != 0) return set_error(KCLPP_ERR_IO, "write failed: %s", path);
  return KCLPP_OK;
}

kclpp_status kclpp_schedule_load(const char *path, uint64_t graph_hash, int k, int kernel, kclpp_schedule *sp) {
  if (!path || !sp) return set_error(KCLPP_ERR_INVALID, "kclpp_schedule_load: null argument");
  FILE *f = fopen(path, "rb");
  if (!f) return set_error(KCLPP_ERR_IO, "cannot open %s", path);
  unsigned char buf[kSchedBytes + 1];
  const size_t got = fread(buf, 1, sizeof buf, f);
  fclose(f);
  if (got != kSchedBytes || memcmp(buf, "KCLPPSC1", 8) != 0)
    return set_error(KCLPP_ERR_IO, "%s is not a kclpp schedule", path);
  if (get64(&buf[kSchedBytes - 8]) != fnv1a(buf, kSchedBytes - 8))
    return set_error(KCLPP_ERR_IO, "%s: checksum mismatch", path);
  if (get64(&buf[8]) != graph_hash || (int)get32(&buf[16]) != k || (int)get32(&buf[20]) != kernel)
    return set_error(KCLPP_ERR_INVALID, "%s was tuned for another graph, k or kernel", path);
  uint32_t v[kSchedFields];
  for (size_t i = 0; i < kSchedFields; ++i) v[i] = get32(&buf[24 + 4 * i]);
  schedule_from(v, *sp);
  return KCLPP_OK;
}

kclpp_status kclpp_edge_list_hash(const kclpp_edge_list *el, uint64_t *hash) {
  if (!el || !hash) return set_error(KCLPP_ERR_INVALID, "kclpp_edge_list_hash: null argument");
  std::vector<unsigned char> b(8 + el->pairs.size() * 4);
  put64(b.data(), el->n);
  for (size_t i = 0; i < el->pairs.size(); ++i) put32(&b[8 + 4 * i], el->pairs[i]);
  *hash = fnv1a(b.data(), b.size());
  return KCLPP_OK;
}

}  // extern "C"
