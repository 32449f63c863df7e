/* seq_chain_emul.c -- the tier M Seq kernel's algorithm (MODE_SEQ, one 32-bit
 * word per lane, per-root-edge streams) restated on the host, lane by lane,
 * so that its exactness can be checked on the CPU against the oracle's pass
 * (tests/test_seq_chain_host.py).  Test infrastructure: it is not the kernel
 * code, it restates what the kernel does -- the per-root induced bitmap rows,
 * a stream per root edge from the pass-start loads, the 32-bit relative
 * values with their cap, the per-word lower bounds lo, the word skip against
 * c + |V| - 1, and the per-word ballot fixed point from the exact prefix value
 * c + (candidates of V before the word) - (those that took their clique).
 *
 *   seq_chain_emul <off.bin u64[n+1]> <cols.bin u32[m]> <r.bin u64[n]> <k> <out.bin u64[n]>
 *
 * Prints "streams <s> skipped <w> processed <p>" (chains decided by the skip
 * test alone, words run through the fixed point). */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned long long u64;

static void *load(const char *path, size_t *bytes) {
  FILE *f = fopen(path, "rb");
  if (!f) { perror(path); exit(2); }
  fseek(f, 0, SEEK_END);
  *bytes = (size_t)ftell(f);
  fseek(f, 0, SEEK_SET);
  void *b = malloc(*bytes ? *bytes : 1);
  if (*bytes && fread(b, 1, *bytes, f) != *bytes) { perror(path); exit(2); }
  fclose(f);
  return b;
}

enum { MAXW = 32, MAXD = 32 * MAXW };

/* Per root. */
static uint32_t W;                /* words per row */
static uint32_t rows[MAXD][MAXW]; /* row i: local ids j < i adjacent to i */
static uint32_t cur[MAXD + 1];    /* a stream's 32-bit values */
static uint32_t lo[MAXW];         /* per word of C: least starting value */
static u64 n_skipped, n_processed, n_streams;

static int popc(uint32_t x) { return __builtin_popcount(x); }

/* One word's fixed point: candidate b falls iff rel[b] >= the number of
 * earlier candidates of the word that fell. */
static uint32_t fixed_point(const int rel[32]) {
  uint32_t m = 0;
  for (int b = 0; b < 32; ++b) if (rel[b] >= 0) m |= 1u << b;
  for (int round = 0; round < 33; ++round) {
    uint32_t m2 = 0;
    for (int b = 0; b < 32; ++b) if (rel[b] >= popc(m & ((1u << b) - 1u))) m2 |= 1u << b;
    if (m2 == m) break;
    m = m2;
  }
  return m;
}

/* The last level over V (one word per lane). */
static uint32_t chain_word1(const uint32_t *V, uint32_t c) {
  uint32_t pop[MAXW], tot = 0;
  for (uint32_t w = 0; w < W; ++w) { pop[w] = (uint32_t)popc(V[w]); tot += pop[w]; }
  if (!tot) return c;
  uint32_t bad = 0;
  for (uint32_t w = 0; w < W; ++w)
    if (pop[w] && lo[w] < c + tot - 1u) bad |= 1u << w;
  if (!bad) { ++n_skipped; return c + tot; }
  uint32_t taken = 0;
  while (bad) {
    const int L = __builtin_ctz(bad);
    bad &= bad - 1;
    uint32_t before = 0;
    for (int w = 0; w < L; ++w) before += pop[w];
    const uint32_t cL = c + before - taken;
    const uint32_t word = V[L];
    int rel[32];
    for (int b = 0; b < 32; ++b) rel[b] = (word >> b & 1u) ? (int)(cur[32 * L + b] - cL) : -1;
    const uint32_t m = fixed_point(rel);
    const uint32_t tk = word & ~m;
    for (int b = 0; b < 32; ++b) if (tk >> b & 1u) cur[32 * L + b] += 1u;
    taken += (uint32_t)popc(tk);
    ++n_processed;
  }
  return c + tot - taken;
}

/* Level L over candidates P with prefix value cg; returns the new value. */
static uint32_t seq_rec(int L, const uint32_t *P, uint32_t cg) {
  if (L == 1) return chain_word1(P, cg);
  if (L >= 3) {
    int pc = 0;
    for (uint32_t w = 0; w < W; ++w) pc += popc(P[w]);
    if (pc < L) return cg;
  }
  for (uint32_t a = 0; a < W; ++a) {
    for (uint32_t wb = P[a]; wb; wb &= wb - 1) {
      const uint32_t u = 32 * a + (uint32_t)__builtin_ctz(wb);
      const uint32_t vu = cur[u];
      const int take = vu < cg; /* strict: ties stay with the earlier argmin */
      uint32_t Q[MAXW];
      for (uint32_t w = 0; w < W; ++w) Q[w] = P[w] & rows[u][w];
      const uint32_t c0 = take ? vu : cg;
      const uint32_t c1 = seq_rec(L - 1, Q, c0);
      if (take) cur[u] += c1 - c0;
      else cg = c1;
    }
  }
  return cg;
}

/* The same stream with 64-bit values and no skip (the kernel's other path). */
static u64 cur64[MAXD + 1];
static u64 seq_rec64(int L, const uint32_t *P, u64 cg) {
  if (L >= 3) {
    int pc = 0;
    for (uint32_t w = 0; w < W; ++w) pc += popc(P[w]);
    if (pc < L) return cg;
  }
  for (uint32_t a = 0; a < W; ++a) {
    for (uint32_t wb = P[a]; wb; wb &= wb - 1) {
      const uint32_t u = 32 * a + (uint32_t)__builtin_ctz(wb);
      if (L == 1) {
        if (cur64[u] < cg) cur64[u] += 1; else cg += 1;
        continue;
      }
      const u64 vu = cur64[u];
      const int take = vu < cg;
      uint32_t Q[MAXW];
      for (uint32_t w = 0; w < W; ++w) Q[w] = P[w] & rows[u][w];
      const u64 c0 = take ? vu : cg;
      const u64 c1 = seq_rec64(L - 1, Q, c0);
      if (take) cur64[u] += c1 - c0;
      else cg = c1;
    }
  }
  return cg;
}

int main(int argc, char **argv) {
  if (argc != 6) { fprintf(stderr, "usage: off cols r k out\n"); return 2; }
  size_t b;
  const u64 *off = load(argv[1], &b);
  const uint32_t n = (uint32_t)(b / 8 - 1);
  const uint32_t *cols = load(argv[2], &b);
  const u64 *r = load(argv[3], &b);
  const int k = atoi(argv[4]);
  u64 *acc = calloc(n ? n : 1, sizeof(u64));
  int *loc = malloc(sizeof(int) * (n ? n : 1));
  for (uint32_t i = 0; i < n; ++i) loc[i] = -1;
  for (uint32_t s = 0; s < n; ++s) {
    const uint32_t d = (uint32_t)(off[s + 1] - off[s]);
    if (d < (uint32_t)(k - 1)) continue;
    if (d > MAXD) { fprintf(stderr, "out-degree %u above %d\n", d, MAXD); return 3; }
    const uint32_t *list = cols + off[s];
    for (uint32_t i = 1; i < d; ++i)
      if (list[i - 1] >= list[i]) { fprintf(stderr, "unsorted out-list\n"); return 3; }
    W = (d + 31) / 32;
    for (uint32_t i = 0; i < d; ++i) loc[list[i]] = (int)i;
    for (uint32_t i = 0; i < d; ++i) {
      memset(rows[i], 0, sizeof rows[i]);
      const uint32_t x = list[i];
      for (u64 e = off[x]; e < off[x + 1]; ++e) {
        const int j = loc[cols[e]];
        if (j >= 0) rows[i][j >> 5] |= 1u << (j & 31);
      }
    }
    for (uint32_t j = 0; j < d; ++j) {
      const uint32_t *C = rows[j];
      int nc = 0;
      for (uint32_t w = 0; w < W; ++w) nc += popc(C[w]);
      if (!nc) continue;
      ++n_streams;
      const uint32_t t = list[j];
      const int g_is_t = r[t] < r[s];
      const u64 bg = g_is_t ? r[t] : r[s];
      /* 32-bit values relative to the smallest starting value of {s, t} and C,
         capped where no comparison can change (k <= 5, as the kernel). */
      u64 lo64 = bg;
      for (uint32_t w = 0; w < W; ++w)
        for (uint32_t wb = C[w]; wb; wb &= wb - 1) {
          const u64 x = r[list[32 * w + __builtin_ctz(wb)]];
          if (x < lo64) lo64 = x;
        }
      u64 bound = 1;
      for (int i = 0; i < k - 2; ++i) bound = bound * (u64)(nc - i) / (u64)(i + 1);
      const u64 cap = (bg - lo64) + bound + 64;
      if (k <= 5 && cap < 0x7fffffffull) {
        for (uint32_t w = 0; w < MAXW; ++w) lo[w] = 0xffffffffu;
        for (uint32_t w = 0; w < W; ++w)
          for (uint32_t wb = C[w]; wb; wb &= wb - 1) {
            const uint32_t i = 32 * w + (uint32_t)__builtin_ctz(wb);
            const u64 rel = r[list[i]] - lo64;
            cur[i] = (uint32_t)(rel < cap ? rel : cap);
            if (cur[i] < lo[w]) lo[w] = cur[i];
          }
        const uint32_t c0 = (uint32_t)(bg - lo64);
        const uint32_t c1 = seq_rec(k - 2, C, c0);
        for (uint32_t w = 0; w < W; ++w)
          for (uint32_t wb = C[w]; wb; wb &= wb - 1) {
            const uint32_t i = 32 * w + (uint32_t)__builtin_ctz(wb);
            const u64 rel = r[list[i]] - lo64;
            acc[list[i]] += (u64)(cur[i] - (uint32_t)(rel < cap ? rel : cap));
          }
        acc[g_is_t ? t : s] += (u64)(c1 - c0);
      } else {
        for (uint32_t w = 0; w < W; ++w)
          for (uint32_t wb = C[w]; wb; wb &= wb - 1) {
            const uint32_t i = 32 * w + (uint32_t)__builtin_ctz(wb);
            cur64[i] = r[list[i]];
          }
        const u64 c1 = seq_rec64(k - 2, C, bg);
        for (uint32_t w = 0; w < W; ++w)
          for (uint32_t wb = C[w]; wb; wb &= wb - 1) {
            const uint32_t i = 32 * w + (uint32_t)__builtin_ctz(wb);
            acc[list[i]] += cur64[i] - r[list[i]];
          }
        acc[g_is_t ? t : s] += c1 - bg;
      }
    }
    for (uint32_t i = 0; i < d; ++i) loc[list[i]] = -1;
  }
  FILE *f = fopen(argv[5], "wb");
  if (!f) { perror(argv[5]); return 2; }
  for (uint32_t i = 0; i < n; ++i) {
    const u64 v = r[i] + acc[i];
    fwrite(&v, 8, 1, f);
  }
  fclose(f);
  printf("streams %llu skipped %llu processed %llu\n", n_streams, n_skipped, n_processed);
  return 0;
}
