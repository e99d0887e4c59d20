// tp_rng.h — jump-ahead algebra for the reference's two random streams.
//
// Both generators are linear recurrences, so advancing a state by n draws
// is multiplication by x^n in the polynomial ring of the recurrence:
//
//  * xoshiro256+ (src/random/standard.rs; Blackman & Vigna) updates its
//    256-bit state by a GF(2)-linear map T. Its characteristic polynomial
//    P (degree 256) is recovered here by Berlekamp-Massey from the
//    generator's own output bits; then T^n s = sum_i j_i T^i s where
//    x^n mod P = sum_i j_i x^i. No published jump constant is used: the
//    2^128 jump of RandomGenerator::jump (standard.rs:53-55) is x^(2^128).
//
//  * Knuth's ranf (src/random/ranf.rs) produces, reset after reset, the
//    sequence X[k] = X[k-55] - X[k-24] mod 1e9 (ranf.rs:106-119), whose
//    characteristic polynomial is x^55 + x^31 - 1. Block r of 55 values
//    (the state after r resets beyond the 10 warm-up ones) is obtained from
//    blocks 0 and 1 by the coefficients of x^(55 r) mod that polynomial.
//    This holds while every state value lies in [0, 1e9), which the seeded
//    initialisation guarantees for seeds in [0, 1e9).
#ifndef TP_RNG_H
#define TP_RNG_H

#include <cstdint>

namespace tp {

// ---------------- xoshiro256+ ----------------
struct Gf2Poly {  // coefficients of x^0..x^255, bit i of w[i/64]
  uint64_t w[4];
};

void xoshiro_seed(uint64_t seed, uint64_t s[4]);   // SplitMix64 expansion
uint64_t xoshiro_next(uint64_t s[4]);             // one draw (raw u64)
const uint64_t* xoshiro_charpoly();               // 5 words, bit 256 set
Gf2Poly gf2_mulmod(const Gf2Poly& a, const Gf2Poly& b);
Gf2Poly gf2_xpow(uint64_t n);                     // x^n mod P
Gf2Poly gf2_xpow2k(unsigned k);                   // x^(2^k) mod P
void xoshiro_apply(const Gf2Poly& j, uint64_t s[4]);  // s <- j(T) s

// ---------------- ranf ----------------
constexpr uint32_t kRanfMod = 1000000000u;
struct RanfPoly {  // coefficients of x^0..x^54 modulo 1e9
  uint32_t c[55];
};

RanfPoly ranf_mulmod(const RanfPoly& a, const RanfPoly& b);
RanfPoly ranf_xpow(uint64_t n);  // x^n mod (x^55 + x^31 - 1)
// ranf state right after seeded_new: slots 1..55 in out[0..55)
void ranf_seeded(int32_t seed, int32_t out[55]);
void ranf_reset(int32_t n[55]);  // one reset, slots 1..55 in n[0..55)
bool ranf_canonical(const int32_t n[55]);
// out = block `window-block + r` given window = blocks (0, 1) (110 values)
// and q = x^(55 r) mod P
void ranf_apply(const RanfPoly& q, const int32_t window[110], int32_t out[55]);

}  // namespace tp

#endif
