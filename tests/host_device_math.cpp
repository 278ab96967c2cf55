// Host build of the searches' warp-free index math (csrc/grand_device.cuh)
// checked against plain combinatorics: binomials, colex unranking (closed forms
// and the table search), colex successors, lexicographic ranks, the FP32 cost
// key, and whole run tiles (lane by lane) against a brute-force search in
// upstream's lexicographic order, first-hit and ML.  Warp collectives are
// stubbed: the functions checked here use none.  Prints "ok" or the first
// mismatch (exit 1).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

struct LaneIndex {
  unsigned x, y, z;
};
static LaneIndex threadIdx;
[[noreturn]] static void warp_stub() {
  fprintf(stderr, "a warp collective was called in the host build\n");
  abort();
}
static inline unsigned __ballot_sync(unsigned, int) { warp_stub(); }
template <class T>
static inline T __shfl_xor_sync(unsigned, T, int) {
  warp_stub();
}
template <class T>
static inline T __shfl_sync(unsigned, T, int) {
  warp_stub();
}
static inline unsigned __reduce_min_sync(unsigned, unsigned) { warp_stub(); }
static inline unsigned __reduce_max_sync(unsigned, unsigned) { warp_stub(); }
static inline int __clz(unsigned x) { return x ? __builtin_clz(x) : 32; }
static inline int __ffs(unsigned x) { return __builtin_ffs((int)x); }
static inline int __popc(unsigned x) { return __builtin_popcount(x); }
static inline float __fadd_rn(float a, float b) { return a + b; }
static inline unsigned __float_as_uint(float f) {
  unsigned u;
  memcpy(&u, &f, 4);
  return u;
}
static inline float __uint_as_float(unsigned u) {
  float f;
  memcpy(&f, &u, 4);
  return f;
}
static inline unsigned __vimin3_u32(unsigned a, unsigned b, unsigned c) {
  return std::min(a, std::min(b, c));
}
template <class T>
static inline T __ldg(const T *p) {
  return *p;
}
static inline unsigned min(unsigned a, unsigned b) { return a < b ? a : b; }
static inline int min(int a, int b) { return a < b ? a : b; }

#include "grand_device.cuh"
#include "grand_solo.h"

using namespace grand;

static unsigned long long C(int n, int k) {
  if (k < 0 || n < k) return 0;
  unsigned long long r = 1;
  for (int i = 1; i <= k; ++i) r = r * (unsigned long long)(n - k + i) / (unsigned long long)i;
  return r;
}

#define CHECK(cond, ...)              \
  do {                                \
    if (!(cond)) {                    \
      fprintf(stderr, __VA_ARGS__);   \
      fprintf(stderr, "\n");          \
      return 1;                       \
    }                                 \
  } while (0)

// colex rank of an ascending k-subset: sum of C(x_i, i + 1)
static unsigned long long colex_rank(const int *x, int k) {
  unsigned long long r = 0;
  for (int i = 0; i < k; ++i) r += C(x[i], i + 1);
  return r;
}

// Every run tile of a weight block, lane by lane: the lowest global index
// (first-hit) and the lowest {cost key, rank} (ML) over all lanes.
template <int KK>
static void all_run_tiles(const SegView &sv, const unsigned long long *t, const uint32_t *sw,
                          bool ml, unsigned long long &g, uint32_t &o, unsigned long long &rr) {
  for (int c = sv.w - 2; c <= sv.tam - 2; ++c) {
    const unsigned long long nt = run_tiles(t, c, sv.w, KK);
    for (unsigned long long q = 0; q < nt; ++q)
      for (unsigned lane = 0; lane < 32; ++lane) {
        threadIdx.x = lane;
        LaneBest lb;
        lb.reset();
        if (ml) eval_run_tile<KK, true>(sv, t, sw, c, q * 32ull * KK, lb);
        else eval_run_tile<KK, false>(sv, t, sw, c, q * 32ull * KK, lb);
        g = std::min(g, lb.g);
        if (lb.o < o || (lb.o == o && lb.r < rr)) {
          o = lb.o;
          rr = lb.r;
        }
      }
  }
}

int main() {
  std::vector<unsigned long long> t((size_t)(kMaxTam + 1) * (kMaxW + 1));
  for (int n = 0; n <= kMaxTam; ++n)
    for (int k = 0; k <= kMaxW; ++k) t[(size_t)n * (kMaxW + 1) + k] = C(n, k);

  // binomials: the multiplicative formula equals the table everywhere it is used
  for (int n = 0; n <= kMaxTam; ++n)
    for (int k = 0; k <= kMaxW; ++k)
      CHECK(binom(n, k) == C(n, k), "binom(%d,%d)", n, k);

  // colex unranking: closed forms (kk <= 3) and the table search agree with the
  // rank, and the successor steps rank r to rank r + 1
  std::mt19937_64 rng(20261203);
  for (int kk = 1; kk <= 5; ++kk) {
    const int cmax = kk == 1 ? 2048 : (kk == 2 ? 400 : (kk == 3 ? 120 : 40));
    for (int c = kk; c <= cmax; ++c) {
      const unsigned long long n = C(c, kk);
      const bool all = n <= 20000;
      const int samples = all ? (int)n : 2000;
      for (int s = 0; s < samples; ++s) {
        const unsigned long long r = all ? (unsigned long long)s : rng() % n;
        int y[5] = {0, 1, 2, 3, 4};
        sub_unrank(t.data(), r, kk, c, y);
        for (int i = 0; i < kk; ++i)
          CHECK(y[i] >= i && y[i] < c && (i == 0 || y[i] > y[i - 1]), "unrank range kk=%d c=%d r=%llu",
                kk, c, r);
        CHECK(colex_rank(y, kk) == r, "unrank kk=%d c=%d r=%llu", kk, c, r);
        if (r + 1 < n) {
          int z[5];
          memcpy(z, y, sizeof(z));
          sub_next(z, kk, c);
          CHECK(colex_rank(z, kk) == r + 1, "successor kk=%d c=%d r=%llu", kk, c, r);
        }
      }
    }
  }
  // large ranks of the closed forms (active sets up to the limit)
  for (int s = 0; s < 200000; ++s) {
    const int kk = 2 + (int)(rng() % 2);
    const int c = kk + (int)(rng() % (kMaxTam - kk));
    const unsigned long long r = rng() % C(c, kk);
    int y[5] = {0, 1, 2, 3, 4};
    sub_unrank(t.data(), r, kk, c, y);
    CHECK(colex_rank(y, kk) == r && y[kk - 1] < c, "large unrank kk=%d c=%d r=%llu", kk, c, r);
  }

  // lexicographic rank of (prefix, last index) against enumeration order
  for (int n = 1; n <= 12; ++n)
    for (int w = 2; w <= std::min(n, kMaxW); ++w) {
      std::vector<int> x(w);
      for (int i = 0; i < w; ++i) x[i] = i;
      for (unsigned long long r = 0;; ++r) {
        int p[5] = {0, 0, 0, 0, 0};
        for (int i = 0; i < w - 1; ++i) p[i] = x[i];
        CHECK(lex_rank(t.data(), n, w, p, w - 1, x[w - 1]) == r, "lex_rank n=%d w=%d r=%llu", n, w, r);
        int i = w - 1;
        while (i >= 0 && x[i] == n - w + i) --i;
        if (i < 0) break;
        ++x[i];
        for (int j = i + 1; j < w; ++j) x[j] = x[j - 1] + 1;
      }
    }

  // the FP32 cost key keeps the order of non-negative costs and inverts exactly
  for (int s = 0; s < 200000; ++s) {
    const float a = (float)(rng() % 100000) * 0.013f, b = (float)(rng() % 100000) * 0.013f;
    CHECK((cost_key(a) < cost_key(b)) == (a < b), "cost_key order %g %g", a, b);
    CHECK(key_cost(cost_key(a)) == a, "key_cost %g", a);
  }

  // whole run tiles, lane by lane, against brute force
  int cases = 0, matched = 0;
  for (int trial = 0; trial < 300; ++trial) {
    const int tam = 4 + (int)(rng() % 40);
    const int w = 3 + (int)(rng() % 4);  // 3..6
    if (w > tam || C(tam, w) > 2000000ull) continue;
    const int R = 6 + (int)(rng() % 58), nw = (R + 31) / 32, nwp = nw == 1 ? 1 : 2;
    std::vector<uint32_t> cols((size_t)tam * nwp, 0u), hc(tam), sw(32, 0u);
    for (int c = 0; c < tam; ++c)
      for (int r = 0; r < R; ++r)
        if (rng() & 1) cols[(size_t)c * nwp + r / 32] |= 1u << (r % 32);
    if (rng() % 3 == 0) {  // a duplicate column
      const int a = (int)(rng() % tam), b = (int)(rng() % tam);
      for (int i = 0; i < nwp; ++i) cols[(size_t)a * nwp + i] = cols[(size_t)b * nwp + i];
    }
    if (rng() % 4) {
      std::vector<int> pick(tam);
      for (int i = 0; i < tam; ++i) pick[i] = i;
      std::shuffle(pick.begin(), pick.end(), rng);
      for (int e = 0; e < w; ++e)
        for (int i = 0; i < nw; ++i) sw[i] ^= cols[(size_t)pick[e] * nwp + i];
    } else {
      for (int i = 0; i < nw; ++i) sw[i] = (uint32_t)rng();
      if (R % 32) sw[nw - 1] &= (1u << (R % 32)) - 1u;
    }
    auto sketch = [&](const uint32_t *v) {
      uint32_t h = 0;
      for (int r = 0; r < R; ++r)
        if ((v[r / 32] >> (r % 32)) & 1u) h ^= row_hash(r);
      return h;
    };
    for (int c = 0; c < tam; ++c) hc[c] = sketch(&cols[(size_t)c * nwp]);
    std::vector<float> llr(tam);
    for (auto &v : llr) v = (float)(1 + rng() % 6) * 0.25f;
    // run tiles of 4 prefixes per lane (the light path's width) or 8
    const int KK = (rng() & 1) ? 8 : 4;
    const SegView sv{hc.data(), cols.data(), llr.data(), sketch(sw.data()), tam, w, KK,
                     nwp, nw, C(tam - 1, w - 1), 1000ull};
    for (int ml = 0; ml < 2; ++ml) {
      unsigned long long g = kNone, rr = kNone;
      uint32_t o = 0xffffffffu;
      if (KK == 8) all_run_tiles<8>(sv, t.data(), sw.data(), ml != 0, g, o, rr);
      else all_run_tiles<4>(sv, t.data(), sw.data(), ml != 0, g, o, rr);
      unsigned long long bg = kNone, br = kNone;
      uint32_t bo = 0xffffffffu;
      std::vector<int> x(w);
      for (int i = 0; i < w; ++i) x[i] = i;
      for (unsigned long long r = 0;; ++r) {
        bool eq = true;
        for (int i = 0; i < nw && eq; ++i) {
          uint32_t z = sw[i];
          for (int e = 0; e < w; ++e) z ^= cols[(size_t)x[e] * nwp + i];
          eq = z == 0u;
        }
        if (eq) {
          if (bg == kNone) bg = sv.base + r;
          float cst = 0.0f;
          for (int e = 0; e < w; ++e) cst = cst + llr[x[e]];
          const uint32_t k2 = cost_key(cst);
          if (k2 < bo || (k2 == bo && r < br)) {
            bo = k2;
            br = r;
          }
        }
        int i = w - 1;
        while (i >= 0 && x[i] == tam - w + i) --i;
        if (i < 0) break;
        ++x[i];
        for (int j = i + 1; j < w; ++j) x[j] = x[j - 1] + 1;
      }
      if (!ml) CHECK(g == bg, "run tiles first-hit tam=%d w=%d: %llu vs %llu", tam, w, g, bg);
      else CHECK(o == bo && rr == br, "run tiles ML tam=%d w=%d", tam, w);
      matched += ml ? 0 : (bg != kNone);
      ++cases;
    }
  }
  CHECK(cases >= 200 && matched >= 50, "too few run-tile cases: %d (%d matched)", cases, matched);
  printf("ok %d run-tile cases\n", cases);

  // solo-column table: exactly the nonzero columns that contain no other nonzero
  // column (duplicates and zero columns excluded), each found by its sketch
  int solo_codes = 0, solo_seen = 0;
  for (int trial = 0; trial < 60; ++trial) {
    const int R = 3 + (int)(rng() % 120), m = 1 + (int)(rng() % 200);
    const int nw = (R + 31) / 32, nwp = nw <= 2 ? nw : (nw <= 4 ? 4 : 8);
    std::vector<uint32_t> cols((size_t)m * nwp, 0u), hcol(m, 0u);
    const int dens = 2 + (int)(rng() % 12);
    for (int c = 0; c < m; ++c) {
      if (rng() % 25 == 0) continue;  // a zero column
      for (int r = 0; r < R; ++r)
        if (rng() % dens == 0) cols[(size_t)c * nwp + r / 32] |= 1u << (r % 32);
    }
    for (int k = 0; k < 3 && m > 2; ++k) {  // duplicates and a column inside another
      const int a = (int)(rng() % m), b = (int)(rng() % m);
      if (k < 2) {
        for (int i = 0; i < nwp; ++i) cols[(size_t)a * nwp + i] = cols[(size_t)b * nwp + i];
      } else {
        for (int i = 0; i < nwp; ++i)
          cols[(size_t)a * nwp + i] = cols[(size_t)b * nwp + i] & (uint32_t)rng();
      }
    }
    for (int c = 0; c < m; ++c)
      for (int r = 0; r < R; ++r)
        if ((cols[(size_t)c * nwp + r / 32] >> (r % 32)) & 1u) hcol[c] ^= row_hash(r);
    const SoloTable t = build_solo_table(cols, nwp, nw, m, hcol);
    auto nonzero = [&](int c) {
      for (int i = 0; i < nw; ++i)
        if (cols[(size_t)c * nwp + i]) return true;
      return false;
    };
    auto inside = [&](int a, int b) {  // a's rows within b's
      for (int i = 0; i < nw; ++i)
        if (cols[(size_t)a * nwp + i] & ~cols[(size_t)b * nwp + i]) return false;
      return true;
    };
    for (int c = 0; c < m; ++c) {
      bool solo = nonzero(c);
      for (int o = 0; o < m && solo; ++o)
        if (o != c && nonzero(o) && inside(o, c)) solo = false;
      bool found = false;
      uint32_t i = hcol[c] & t.mask;
      for (uint32_t probe = 0; probe <= t.mask && t.cols[i] >= 0; ++probe, i = (i + 1) & t.mask)
        found = found || (t.cols[i] == c && t.keys[i] == hcol[c]);
      CHECK(found == solo, "solo table R=%d m=%d column %d: table %d, brute force %d", R, m, c,
            (int)found, (int)solo);
      solo_seen += solo;
    }
    ++solo_codes;
  }
  CHECK(solo_seen > 500, "too few solo columns: %d", solo_seen);
  printf("ok solo tables of %d codes (%d solo columns)\n", solo_codes, solo_seen);
  return 0;
}
