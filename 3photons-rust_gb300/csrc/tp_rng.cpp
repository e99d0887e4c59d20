// tp_rng.cpp — host-side jump-ahead algebra (see tp_rng.h).
#include "tp_rng.h"

#include <cstring>
#include <mutex>

namespace tp {

// ---------------------------------------------------------------------------
// xoshiro256+
// ---------------------------------------------------------------------------
void xoshiro_seed(uint64_t seed, uint64_t s[4]) {
  // SplitMix64 (Vigna), the expansion rand_xoshiro applies in seed_from_u64
  uint64_t x = seed;
  for (int i = 0; i < 4; ++i) {
    x += 0x9e3779b97f4a7c15ull;
    uint64_t z = x;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    s[i] = z ^ (z >> 31);
  }
}

uint64_t xoshiro_next(uint64_t s[4]) {
  const uint64_t result = s[0] + s[3];
  const uint64_t t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = (s[3] << 45) | (s[3] >> 19);
  return result;
}

namespace {

// Berlekamp-Massey over GF(2) on 512 bits of one state coordinate.
void derive_charpoly(uint64_t P[5]) {
  const int N = 512;
  uint8_t seq[N];
  uint64_t s[4];
  xoshiro_seed(0x5eed5eedull, s);
  for (int k = 0; k < N; ++k) {
    seq[k] = (uint8_t)(s[0] & 1);
    xoshiro_next(s);
  }
  // connection polynomial C(x) = 1 + c1 x + ... + cL x^L, as bit arrays
  uint8_t C[N + 1] = {0}, B[N + 1] = {0}, T[N + 1];
  C[0] = B[0] = 1;
  int L = 0, m = 1;
  for (int n = 0; n < N; ++n) {
    uint8_t d = seq[n];
    for (int i = 1; i <= L; ++i) d ^= (uint8_t)(C[i] & seq[n - i]);
    if (d == 0) {
      ++m;
    } else if (2 * L <= n) {
      std::memcpy(T, C, sizeof T);
      for (int i = 0; i + m <= N; ++i) C[i + m] ^= B[i];
      L = n + 1 - L;
      std::memcpy(B, T, sizeof B);
      m = 1;
    } else {
      for (int i = 0; i + m <= N; ++i) C[i + m] ^= B[i];
      ++m;
    }
  }
  // characteristic polynomial P(x) = x^L C(1/x): coefficient of x^(L-i) is c_i
  std::memset(P, 0, 5 * sizeof(uint64_t));
  for (int i = 0; i <= L; ++i)
    if (C[i]) {
      const int e = L - i;
      P[e >> 6] |= 1ull << (e & 63);
    }
}

}  // namespace

const uint64_t* xoshiro_charpoly() {
  static uint64_t P[5];
  static std::once_flag once;
  std::call_once(once, [] { derive_charpoly(P); });
  return P;
}

Gf2Poly gf2_mulmod(const Gf2Poly& a, const Gf2Poly& b) {
  const uint64_t* P = xoshiro_charpoly();
  uint64_t r[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = 0; i < 256; ++i) {
    if (!((b.w[i >> 6] >> (i & 63)) & 1)) continue;
    const int ws = i >> 6, bs = i & 63;
    for (int w = 0; w < 4; ++w) {
      r[w + ws] ^= a.w[w] << bs;
      if (bs) r[w + ws + 1] ^= a.w[w] >> (64 - bs);
    }
  }
  for (int i = 510; i >= 256; --i) {
    if (!((r[i >> 6] >> (i & 63)) & 1)) continue;
    const int sh = i - 256, ws = sh >> 6, bs = sh & 63;
    for (int w = 0; w < 5; ++w) {
      if (w + ws < 8) r[w + ws] ^= P[w] << bs;
      if (bs && w + ws + 1 < 8) r[w + ws + 1] ^= P[w] >> (64 - bs);
    }
  }
  Gf2Poly out;
  for (int w = 0; w < 4; ++w) out.w[w] = r[w];
  return out;
}

Gf2Poly gf2_xpow2k(unsigned k) {
  Gf2Poly x{{2, 0, 0, 0}};
  for (unsigned i = 0; i < k; ++i) x = gf2_mulmod(x, x);
  return x;
}

Gf2Poly gf2_xpow(uint64_t n) {
  Gf2Poly r{{1, 0, 0, 0}}, base{{2, 0, 0, 0}};
  while (n) {
    if (n & 1) r = gf2_mulmod(r, base);
    n >>= 1;
    if (n) base = gf2_mulmod(base, base);
  }
  return r;
}

void xoshiro_apply(const Gf2Poly& j, uint64_t s[4]) {
  uint64_t acc[4] = {0, 0, 0, 0};
  for (int i = 0; i < 256; ++i) {
    if ((j.w[i >> 6] >> (i & 63)) & 1)
      for (int w = 0; w < 4; ++w) acc[w] ^= s[w];
    xoshiro_next(s);
  }
  for (int w = 0; w < 4; ++w) s[w] = acc[w];
}

// ---------------------------------------------------------------------------
// ranf
// ---------------------------------------------------------------------------
RanfPoly ranf_mulmod(const RanfPoly& a, const RanfPoly& b) {
  uint64_t r[109];
  for (int k = 0; k < 109; ++k) r[k] = 0;
  for (int i = 0; i < 55; ++i) {
    if (!a.c[i]) continue;
    for (int j = 0; j < 55; ++j) r[i + j] = (r[i + j] + (uint64_t)a.c[i] * b.c[j]) % kRanfMod;
  }
  // x^55 = 1 - x^31
  for (int k = 108; k >= 55; --k) {
    const uint64_t c = r[k];
    if (!c) continue;
    r[k - 55] = (r[k - 55] + c) % kRanfMod;
    r[k - 24] = (r[k - 24] + kRanfMod - c) % kRanfMod;
    r[k] = 0;
  }
  RanfPoly out;
  for (int k = 0; k < 55; ++k) out.c[k] = (uint32_t)r[k];
  return out;
}

RanfPoly ranf_xpow(uint64_t n) {
  RanfPoly r{}, base{};
  r.c[0] = 1;
  base.c[1] = 1;
  while (n) {
    if (n & 1) r = ranf_mulmod(r, base);
    n >>= 1;
    if (n) base = ranf_mulmod(base, base);
  }
  return r;
}

namespace {
inline int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
inline int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
}  // namespace

void ranf_reset(int32_t n[55]) {
  // slot i (1-based) lives at n[i-1]
  for (int i = 1; i < 25; ++i) {
    n[i - 1] = wsub(n[i - 1], n[i + 30]);
    if (n[i - 1] < 0) n[i - 1] = wadd(n[i - 1], (int32_t)kRanfMod);
  }
  for (int i = 25; i < 56; ++i) {
    n[i - 1] = wsub(n[i - 1], n[i - 25]);
    if (n[i - 1] < 0) n[i - 1] = wadd(n[i - 1], (int32_t)kRanfMod);
  }
}

void ranf_seeded(int32_t seed, int32_t out[55]) {
  int32_t n[56] = {0};
  n[55] = seed;
  int32_t j = seed, k = 1;
  for (int i = 1; i < 55; ++i) {
    const int ii = (21 * i) % 55;
    n[ii] = k;
    k = wsub(j, k);
    if (k < 0) k = wadd(k, (int32_t)kRanfMod);
    j = n[ii];
  }
  for (int i = 0; i < 55; ++i) out[i] = n[i + 1];
  for (int r = 0; r < 10; ++r) ranf_reset(out);
}

bool ranf_canonical(const int32_t n[55]) {
  for (int i = 0; i < 55; ++i)
    if (n[i] < 0 || n[i] >= (int32_t)kRanfMod) return false;
  return true;
}

void ranf_apply(const RanfPoly& q, const int32_t window[110], int32_t out[55]) {
  for (int i = 0; i < 55; ++i) {
    uint64_t acc = 0;
    for (int m = 0; m < 55; ++m) acc = (acc + (uint64_t)q.c[m] * (uint32_t)window[i + m]) % kRanfMod;
    out[i] = (int32_t)acc;
  }
}

}  // namespace tp
