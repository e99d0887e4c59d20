// tp_oracle.cpp — CPU restatement of 3photons-rust, used ONLY as test
// infrastructure: the checker of the GPU library's results, the CPU baseline
// timed by bench.py, and the generator of parity fixtures. Nothing in the
// product links, loads or calls this file.
//
// Build: g++ -O2 -ffp-contract=off (Rust never contracts a*b+c into an FMA,
// and x86-64 Rust code has no FMA at all). Every operation below follows the
// reference's operation order, including the order fixed by the third-party
// crates the reference calls:
//   nalgebra 0.32.3  column_sum / dot / norm_squared / gemv / cross;
//   num-complex 0.4.4  Mul, Div, powi, conj, norm_sqr;
//   rand 0.8.5 + rand_xoshiro 0.6.0  SplitMix64 seeding, xoshiro256+,
//     (next_u64 >> 11) * 2^-53 uniforms, the 2^128 jump;
//   LLVM powi lowering (square-and-multiply; constant operands are folded
//     with the host pow()).
// Parity pins: reference/res.data-features_* and reference/stdout.log-features_*
// (N = 1e7 at `valeurs`), checked byte-for-byte by tests/test_oracle_golden.py.
#include "tp_oracle.h"

#include <atomic>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

namespace {

constexpr double kPi = 3.14159265358979323846264338327950288;
constexpr double kFracPi2 = 1.57079632679489661923132169163975144;
constexpr double kSqrt2 = 1.41421356237309504880168872420969808;
constexpr double kMinPositive = 2.2250738585072014e-308;  // f64::MIN_POSITIVE
constexpr int kBatch = TP_BATCH_SIZE;

// LLVM lowers powi(x, n) with a constant n to square-and-multiply, the same
// sequence as compiler-rt's __powidf2.
double powi(double a, int b) {
  const bool recip = b < 0;
  if (recip) b = -b;
  double r = 1.0;
  for (;;) {
    if (b & 1) r *= a;
    b /= 2;
    if (b == 0) break;
    a *= a;
  }
  return recip ? 1.0 / r : r;
}

// ---------------------------------------------------------------------------
// RNG 1: Knuth's ranf (src/random/ranf.rs). i32 arithmetic wraps, as the
// reference's release build does.
// ---------------------------------------------------------------------------
inline int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
inline int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
constexpr int32_t kModulo = 1000000000;

struct Ranf {
  int32_t seed;
  int32_t n[56];
  int index;

  // RanfGenerator::reset (ranf.rs:106-119)
  void reset() {
    for (int i = 1; i < 25; ++i) {
      n[i] = wsub(n[i], n[i + 31]);
      if (n[i] < 0) n[i] = wadd(n[i], kModulo);
    }
    for (int i = 25; i < 56; ++i) {
      n[i] = wsub(n[i], n[i - 24]);
      if (n[i] < 0) n[i] = wadd(n[i], kModulo);
    }
  }
  // RanfGenerator::seeded_new (ranf.rs:36-66)
  void init(int32_t s) {
    seed = s;
    std::memset(n, 0, sizeof n);
    index = 55;
    n[55] = s;
    int32_t j = s, k = 1;
    for (int i = 1; i < 55; ++i) {
      int ii = (21 * i) % 55;
      n[ii] = k;
      k = wsub(j, k);
      if (k < 0) k = wadd(k, kModulo);
      j = n[ii];
    }
    for (int r = 0; r < 10; ++r) reset();
  }
  // random_array::<1> (ranf.rs:78-102)
  double random() {
    if (index < 1) {
      reset();
      index = 55;
    }
    index -= 1;
    return (double)n[index + 1] * 1e-9;
  }
  // random_array::<N> (ranf.rs:78-102), N <= 55
  void random_array(int N, double* out) {
    if (index < N) {
      reset();
      index = 55;
    }
    index -= N;
    for (int i = 0; i < N; ++i) out[i] = (double)n[index + 1 + i] * 1e-9;
  }
  // jump (ranf.rs:137-140)
  void jump() { init(wadd(seed, 123456)); }
};

// ---------------------------------------------------------------------------
// RNG 2: xoshiro256+ (Blackman & Vigna), seeded by SplitMix64 (Vigna), as
// rand_xoshiro 0.6.0's Xoshiro256Plus::seed_from_u64 does; uniforms as
// rand 0.8.5's Standard f64 (src/random/standard.rs:21-35).
// ---------------------------------------------------------------------------
struct Xoshiro {
  uint64_t s[4];

  static uint64_t splitmix_next(uint64_t& x) {
    x += 0x9e3779b97f4a7c15ull;
    uint64_t z = x;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
  }
  void init(uint64_t seed) {
    uint64_t x = seed;
    for (int i = 0; i < 4; ++i) s[i] = splitmix_next(x);
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next_u64() {
    const uint64_t result = s[0] + s[3];
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return result;
  }
  double random() { return (double)(next_u64() >> 11) * (1.0 / 9007199254740992.0); }
  void random_array(int N, double* out) {
    for (int i = 0; i < N; ++i) out[i] = random();
  }
  // The 2^128-draw jump, computed here independently of any published
  // constant: the 256x256 GF(2) matrix of one step is squared 128 times.
  void jump();
};

// 256x256 GF(2) matrix stored by columns: col[j] = M e_j (4 words each).
struct Gf2Mat {
  uint64_t col[256][4];
  void apply(const uint64_t in[4], uint64_t out[4]) const {
    uint64_t r[4] = {0, 0, 0, 0};
    for (int j = 0; j < 256; ++j)
      if ((in[j >> 6] >> (j & 63)) & 1)
        for (int w = 0; w < 4; ++w) r[w] ^= col[j][w];
    for (int w = 0; w < 4; ++w) out[w] = r[w];
  }
};

const Gf2Mat& xoshiro_jump128_matrix() {
  static Gf2Mat* m = [] {
    Gf2Mat* a = new Gf2Mat;
    for (int j = 0; j < 256; ++j) {  // one step applied to e_j
      Xoshiro x;
      for (int w = 0; w < 4; ++w) x.s[w] = 0;
      x.s[j >> 6] = 1ull << (j & 63);
      x.next_u64();
      for (int w = 0; w < 4; ++w) a->col[j][w] = x.s[w];
    }
    Gf2Mat* b = new Gf2Mat;
    for (int sq = 0; sq < 128; ++sq) {  // a <- a*a
      for (int j = 0; j < 256; ++j) a->apply(a->col[j], b->col[j]);
      std::swap(a, b);
    }
    delete b;
    return a;
  }();
  return *m;
}

void Xoshiro::jump() {
  uint64_t out[4];
  xoshiro_jump128_matrix().apply(s, out);
  for (int w = 0; w < 4; ++w) s[w] = out[w];
}

// Generic RNG holder
struct Rng {
  int kind;
  Ranf ranf;
  Xoshiro xo;
  void init(int k, uint64_t seed) {
    kind = k;
    if (kind == TP_RNG_RANF)
      ranf.init((int32_t)(uint32_t)seed);
    else
      xo.init(seed);
  }
  double random() { return kind == TP_RNG_RANF ? ranf.random() : xo.random(); }
  void random_array(int N, double* out) {
    if (kind == TP_RNG_RANF)
      ranf.random_array(N, out);
    else
      xo.random_array(N, out);
  }
  void jump() {
    if (kind == TP_RNG_RANF)
      ranf.jump();
    else
      xo.jump();
  }
};

// ---------------------------------------------------------------------------
// Complex arithmetic with num-complex 0.4 operation order
// ---------------------------------------------------------------------------
struct C {
  double re, im;
};
inline C cmul(C a, C b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
inline C cdiv(C a, C b) {
  const double ns = b.re * b.re + b.im * b.im;
  const double re = a.re * b.re + a.im * b.im;
  const double im = a.im * b.re - a.re * b.im;
  return {re / ns, im / ns};
}
inline C cadd(C a, C b) { return {a.re + b.re, a.im + b.im}; }
inline C rmul(double f, C z) { return {f * z.re, f * z.im}; }  // f64 * Complex
inline C mulr(C z, double f) { return {z.re * f, z.im * f}; }  // Complex * f64
inline C conj(C z) { return {z.re, -z.im}; }
inline C csq(C z) { return cmul(z, z); }  // powi(2)
inline double norm_sqr(C z) { return z.re * z.re + z.im * z.im; }

// ---------------------------------------------------------------------------
// Per-run constants
// ---------------------------------------------------------------------------
struct Consts {
  double e_total, ev_weight;
  double g_a, g_beta_p, g_beta_m;
  double sigma_contribs[5];
  double fact_com, norm_weight, propagator, delta;
};

// EventGenerator::new (evgen.rs:40-77): z_n and ln(weight)
double event_weight(double e_total) {
  double z_n = (3.0 - 1.0) * std::log(kFracPi2);
  for (int k = 2; k < 3; ++k) z_n -= 2.0 * std::log((double)(k - 1));
  z_n = z_n - std::log(3.0 - 1.0);
  const double ln_weight = (2.0 * 3.0 - 4.0) * std::log(e_total) + z_n;
  return std::exp(ln_weight);
}

Consts make_consts(const tp_config& cfg) {
  Consts k{};
  k.e_total = cfg.e_total;
  k.ev_weight = event_weight(cfg.e_total);
  // Couplings::new (coupling.rs:23-33)
  const double e2 = (4.0 * kPi) * cfg.alpha;
  const double e2_z = (4.0 * kPi) * cfg.alpha_z;
  const double cos2w = 1.0 - cfg.sin2_weinberg;
  const double g_beta = -std::sqrt(e2_z / ((4.0 * cos2w) * cfg.sin2_weinberg)) / powi(cfg.m_z0, 4);
  k.g_a = -powi(std::sqrt(e2), 3);
  k.g_beta_p = g_beta;
  k.g_beta_m = g_beta;
  // ResultsAccumulator::new (resacc.rs:59-117)
  const double fact_com = (1.0 / 6.0) * cfg.gev2_to_picobarn;
  const double relat_width = cfg.g_z0 / cfg.m_z0;
  const double p_aa = 2.0;
  const double p_ab = 1.0 - 4.0 * cfg.sin2_weinberg;
  const double p_bb = p_ab + 8.0 * powi(cfg.sin2_weinberg, 2);
  const double c_aa = fact_com * p_aa;
  const double c_ab = fact_com * p_ab / powi(cfg.m_z0, 2);
  const double c_bb = fact_com * p_bb / powi(cfg.m_z0, 4);
  const double dzeta = powi(cfg.e_total / cfg.m_z0, 2);
  const double delta = (dzeta - 1.0) / relat_width;
  const double propagator = 1.0 / (1.0 + powi(delta, 2));
  const double n_ev = (double)cfg.num_events;
  // (2 PI)^(4 - 3*3) has constant operands: folded with the host pow()
  const double norm = std::pow(2.0 * kPi, -5.0) / n_ev;
  const double norm_weight = k.ev_weight * norm;
  const double com = norm_weight / 4.0;
  const double aa = com * c_aa;
  const double bb = com * c_bb * propagator / powi(relat_width, 2);
  const double ab = com * c_ab * 2.0 * cfg.beta_plus * propagator / relat_width;
  k.sigma_contribs[0] = aa;
  k.sigma_contribs[1] = bb * powi(cfg.beta_plus, 2);
  k.sigma_contribs[2] = bb * powi(cfg.beta_minus, 2);
  k.sigma_contribs[3] = ab * delta;
  k.sigma_contribs[4] = -ab;
  k.fact_com = fact_com;
  k.norm_weight = norm_weight;
  k.propagator = propagator;
  k.delta = delta;
  return k;
}

// ---------------------------------------------------------------------------
// Event generation (evgen.rs:89-207) — p[particle][X,Y,Z,E]
// ---------------------------------------------------------------------------
struct Event {
  double p[5][4];
};

// generate_raw, default mode (evgen.rs:174-207). q[photon][coord].
void generate_raw_default(Rng& rng, double q[3][4], double* uniforms) {
  double cos_theta[3], phi[3], exp_min_e[3];
  int u = 0;
  for (int par = 0; par < 3; ++par) {  // from_fn walks column-major
    const double r0 = rng.random();
    cos_theta[par] = 2.0 * r0 - 1.0;
    const double r1 = rng.random();
    phi[par] = (2.0 * kPi) * r1;
    const double r2 = rng.random();
    const double r3 = rng.random();
    exp_min_e[par] = r2 * r3;
    if (uniforms) {
      uniforms[u++] = r0;
      uniforms[u++] = r1;
      uniforms[u++] = r2;
      uniforms[u++] = r3;
    }
  }
  for (int par = 0; par < 3; ++par) {
    const double cos_phi = std::cos(phi[par]);
    const double sin_phi = std::sin(phi[par]);
    const double sin_theta = std::sqrt(1.0 - powi(cos_theta[par], 2));
    const double energy = -std::log(exp_min_e[par] + kMinPositive);
    q[par][0] = energy * (sin_theta * sin_phi);
    q[par][1] = energy * (sin_theta * cos_phi);
    q[par][2] = energy * cos_theta[par];
    q[par][3] = energy * 1.0;
  }
}

// generate_raw, faster-evgen mode (evgen.rs:143-173, 221-249)
void generate_raw_faster(Rng& rng, double q[3][4]) {
  double params[9];
  rng.random_array(9, params);  // from_column_slice: column c = params[3c..3c+3]
  double cos_theta[3], exp_min_e[3];
  for (int p = 0; p < 3; ++p) {
    cos_theta[p] = 2.0 * params[p] - 1.0;
    exp_min_e[p] = params[3 + p] * params[6 + p];
  }
  // random_unit_2d_outgoing
  double v[6];
  rng.random_array(6, v);
  double pts[3][2], r2[3];
  for (int p = 0; p < 3; ++p) {  // from_iterator fills column-major
    pts[p][0] = 2.0 * v[p] - 1.0;
    pts[p][1] = 2.0 * v[3 + p] - 1.0;
    r2[p] = (0.0 + pts[p][0] * pts[p][0]) + pts[p][1] * pts[p][1];
  }
  const double min_pos2 = kMinPositive * kMinPositive;
  for (int p = 0; p < 3; ++p) {
    while (r2[p] > 1.0 || r2[p] < min_pos2) {
      double w[2];
      rng.random_array(2, w);
      pts[p][0] = 2.0 * w[0] - 1.0;
      pts[p][1] = 2.0 * w[1] - 1.0;
      r2[p] = 0.0 + (pts[p][0] * pts[p][0] + pts[p][1] * pts[p][1]);
    }
  }
  double sc[3][2];
  for (int p = 0; p < 3; ++p) {
    const double nrm = 1.0 / std::sqrt(r2[p]);
    sc[p][0] = pts[p][0] * nrm;
    sc[p][1] = pts[p][1] * nrm;
  }
  for (int p = 0; p < 3; ++p) {
    const double sin_theta = std::sqrt(1.0 - powi(cos_theta[p], 2));
    const double energy = -std::log(exp_min_e[p] + kMinPositive);
    q[p][0] = energy * (sin_theta * sc[p][0]);
    q[p][1] = energy * (sin_theta * sc[p][1]);
    q[p][2] = energy * cos_theta[p];
    q[p][3] = energy * 1.0;
  }
}

// EventGenerator::generate (evgen.rs:89-132)
void generate(const Consts& k, Rng& rng, int flags, Event& ev, double* uniforms) {
  double q[3][4];
  if (flags & TPO_MODE_FASTER_EVGEN)
    generate_raw_faster(rng, q);
  else
    generate_raw_default(rng, q, uniforms);

  double r[4];  // column_sum: zeros + q0 + q1 + q2
  for (int c = 0; c < 4; ++c) r[c] = ((0.0 + q[0][c]) + q[1][c]) + q[2][c];
  const double r_xyz_n2 = 0.0 + ((r[0] * r[0] + r[1] * r[1]) + r[2] * r[2]);
  const double r_norm_2 = r[3] * r[3] - r_xyz_n2;
  const double alpha = k.e_total / r_norm_2;
  const double r_norm = std::sqrt(r_norm_2);
  const double beta = 1.0 / (r_norm + r[3]);

  double p_e[3], p_xyz[3][3];
  for (int p = 0; p < 3; ++p) {
    // gemv: y = r_x*q_x, then y = r_y*q_y + 1*y, then y = r_z*q_z + 1*y
    double rq = r[0] * q[p][0];
    rq = r[1] * q[p][1] + 1.0 * rq;
    rq = r[2] * q[p][2] + 1.0 * rq;
    p_e[p] = alpha * (r[3] * q[p][3] - rq);
    const double b_rq_e = beta * rq - q[p][3];
    for (int c = 0; c < 3; ++c) p_xyz[p][c] = alpha * (r_norm * q[p][c] + b_rq_e * r[c]);
  }
  if (!(flags & TP_MODE_NO_PHOTON_SORTING)) {
    for (int a = 0; a < 2; ++a)
      for (int b = a + 1; b < 3; ++b)
        if (p_e[b] > p_e[a]) {
          std::swap(p_e[a], p_e[b]);
          for (int c = 0; c < 3; ++c) std::swap(p_xyz[a][c], p_xyz[b][c]);
        }
  }
  const double h = k.e_total / 2.0;
  ev.p[0][0] = -k.e_total / 2.0;
  ev.p[0][1] = 0.0;
  ev.p[0][2] = 0.0;
  ev.p[0][3] = h;
  ev.p[1][0] = h;
  ev.p[1][1] = 0.0;
  ev.p[1][2] = 0.0;
  ev.p[1][3] = h;
  for (int p = 0; p < 3; ++p) {
    for (int c = 0; c < 3; ++c) ev.p[2 + p][c] = p_xyz[p][c];
    ev.p[2 + p][3] = p_e[p];
  }
}

// EventCut::keep (evcut.rs:42-96); returns 0 if kept, else the failing cut
int cut(const tp_config& cfg, int flags, const Event& ev) {
  double min_e;
  if (flags & TP_MODE_NO_PHOTON_SORTING) {
    min_e = ev.p[2][3];
    for (int p = 1; p < 3; ++p) min_e = (min_e < ev.p[2 + p][3]) ? min_e : ev.p[2 + p][3];
  } else {
    min_e = ev.p[4][3];
  }
  if (min_e < cfg.e_min) return 1;
  const double* el = ev.p[0];
  double nums[3], dens[3];
  for (int p = 0; p < 3; ++p) {
    const double* q = ev.p[2 + p];
    double y = el[0] * q[0];  // gemv with x = el.xyz
    y = el[1] * q[1] + 1.0 * y;
    y = el[2] * q[2] + 1.0 * y;
    nums[p] = y;
    dens[p] = q[3] * el[3];
  }
  for (int p = 0; p < 3; ++p)
    if (std::fabs(nums[p]) > cfg.beam_photons_cut * dens[p]) return 2;
  for (int a = 0; a < 2; ++a)
    for (int b = a + 1; b < 3; ++b) {
      const double* pa = ev.p[2 + a];
      const double* pb = ev.p[2 + b];
      const double num = (pa[0] * pb[0] + pa[1] * pb[1]) + pa[2] * pb[2];
      const double den = pa[3] * pb[3];
      if (num > cfg.photon_photon_cut * den) return 3;
    }
  const double* a = ev.p[2];
  const double* b = ev.p[3];
  const double n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
  const double num = (el[0] * n[0] + el[1] * n[1]) + el[2] * n[2];
  const double nn = 0.0 + ((n[0] * n[0] + n[1] * n[1]) + n[2] * n[2]);
  const double den = el[3] * std::sqrt(nn);
  if (std::fabs(num) < cfg.beam_photon_plane_cut * den) return 4;
  return 0;
}

// SpinorProducts (spinor.rs:31-162) + MEsContributions (matelems.rs:53-86)
void m2_sums(const Consts& k, const Event& ev, double out[5]) {
  double xx[5];
  C fx[5];
  for (int i = 0; i < 5; ++i) {
    xx[i] = std::sqrt(ev.p[i][3] + ev.p[i][2]);
    if (xx[i] > kMinPositive)
      fx[i] = {ev.p[i][0] / xx[i], ev.p[i][1] / xx[i]};
    else
      fx[i] = {std::sqrt(2.0 * ev.p[i][3]), 0.0};
  }
  C sx[5][5];
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) {
      const C a = mulr(fx[i], xx[j]);
      const C b = mulr(fx[j], xx[i]);
      sx[i][j] = {a.re - b.re, a.im - b.im};
    }
  auto s = [&](int i, int j) { return sx[i][j]; };
  auto t = [&](int i, int j) {
    const C c = conj(sx[i][j]);
    return C{-c.re, -c.im};
  };
  const double nr8 = -(2.0 * kSqrt2);
  auto a_ppm = [&](int k1, int k2, int k3) {
    const C num = cmul(rmul(nr8, s(0, 1)), csq(s(0, k3)));
    const C den = cmul(cmul(cmul(s(0, k1), s(0, k2)), s(1, k1)), s(1, k2));
    return cdiv(num, den);
  };
  auto a_pmm = [&](int k1, int k2, int k3) {
    const C num = cmul(rmul(nr8, t(0, 1)), csq(t(1, k1)));
    const C den = cmul(cmul(cmul(t(1, k2), t(1, k3)), t(0, k2)), t(0, k3));
    return cdiv(num, den);
  };
  auto bp_ppm = [&](int k1, int k2, int k3) {
    return cmul(rmul(nr8, t(0, 1)), csq(cmul(t(k1, k2), s(k3, 0))));
  };
  auto bp_pmm = [&](int k1, int k2, int k3) {
    return cmul(rmul(nr8, s(0, 1)), csq(cmul(t(k1, 1), s(k2, k3))));
  };
  auto bm_ppp = [&](int k1, int k2, int k3) {
    const C sum = cadd(cadd(csq(cmul(t(k1, k2), t(k3, 1))), csq(cmul(t(k1, k3), t(k2, 1)))),
                       csq(cmul(t(k2, k3), t(k1, 1))));
    return cmul(rmul(nr8, s(0, 1)), sum);
  };
  auto bm_mmm = [&](int k1, int k2, int k3) {
    const C sum = cadd(cadd(csq(cmul(s(k1, 0), s(k2, k3))), csq(cmul(s(k2, 0), s(k1, k3)))),
                       csq(cmul(s(k3, 0), s(k1, k2))));
    return cmul(rmul(nr8, t(0, 1)), sum);
  };
  const C zero{0.0, 0.0};
  // helicities MMM, MMP, MPM, MPP, PMM, PMP, PPM, PPP (spinor.rs:72-116)
  const C a[8] = {zero, a_pmm(4, 2, 3), a_pmm(3, 2, 4), a_ppm(3, 4, 2),
                  a_pmm(2, 3, 4), a_ppm(2, 4, 3), a_ppm(2, 3, 4), zero};
  const C bp[8] = {zero, bp_pmm(4, 2, 3), bp_pmm(3, 2, 4), bp_ppm(3, 4, 2),
                   bp_pmm(2, 3, 4), bp_ppm(2, 4, 3), bp_ppm(2, 3, 4), zero};
  const C bm[8] = {bm_mmm(2, 3, 4), zero, zero, zero, zero, zero, zero, bm_ppp(2, 3, 4)};
  double m2[5][8];
  for (int h = 0; h < 8; ++h) {
    const C aa = mulr(a[h], k.g_a);
    const C bpp = mulr(bp[h], k.g_beta_p);
    const C bmm = mulr(bm[h], k.g_beta_m);
    const C mixed = cmul(rmul(2.0, aa), conj(bpp));
    m2[0][h] = norm_sqr(aa);
    m2[1][h] = norm_sqr(bpp);
    m2[2][h] = norm_sqr(bmm);
    m2[3][h] = mixed.re;
    m2[4][h] = mixed.im;
  }
  for (int c = 0; c < 5; ++c) {
    double acc = 0.0;
    for (int h = 0; h < 8; ++h) acc = acc + m2[c][h];
    out[c] = acc;
  }
}

struct Acc {
  uint64_t selected = 0;
  double spm2[5] = {0, 0, 0, 0, 0};
  double vars[5] = {0, 0, 0, 0, 0};
  double sigma = 0, variance = 0;
};

// ResultsAccumulator::integrate (resacc.rs:121-129)
void integrate(Acc& acc, const Consts& k, const double m[5]) {
  acc.selected += 1;
  for (int c = 0; c < 5; ++c) acc.spm2[c] += m[c];
  for (int c = 0; c < 5; ++c) acc.vars[c] += powi(m[c], 2);
  double w = 0.0;  // 5-vector dot: nalgebra's generic loop, summed in order
  for (int c = 0; c < 5; ++c) w += m[c] * k.sigma_contribs[c];
  acc.sigma += w;
  acc.variance += powi(w, 2);
}

// The per-batch closure (main.rs:103-128)
void simulate_batch(const tp_config& cfg, const Consts& k, int flags, Rng& rng, uint64_t n, Acc& acc) {
  Event ev;
  for (uint64_t i = 0; i < n; ++i) {
    generate(k, rng, flags, ev, nullptr);
    if (cut(cfg, flags, ev) == 0) {
      double m[5];
      m2_sums(k, ev, m);
      integrate(acc, k, m);
    }
  }
}

// Advances an RNG over one batch without the physics
// (EventGenerator::simulate_event_batch, evgen.rs:257-267)
void skip_batch(Rng& rng, int flags, uint64_t n) {
  if (flags & TPO_MODE_FASTER_EVGEN) {
    double q[3][4];
    for (uint64_t i = 0; i < n; ++i) generate_raw_faster(rng, q);
  } else {
    for (uint64_t i = 0; i < 12 * n; ++i) rng.random();
  }
}

// ---------------------------------------------------------------------------
// Positioning a stream far ahead by powers of its transition matrix, so that
// batches deep inside a 1e9- or 1e10-event run can be checked without
// stepping every draw before them. (The product jumps with characteristic
// polynomials; this is an independent method.)
// ---------------------------------------------------------------------------
// xoshiro256+: the state after d steps is M^d s, M the GF(2) step matrix.
void xoshiro_advance(Xoshiro& x, uint64_t d) {
  static const Gf2Mat* step = [] {
    Gf2Mat* m = new Gf2Mat;
    for (int j = 0; j < 256; ++j) {
      Xoshiro e;
      for (int w = 0; w < 4; ++w) e.s[w] = 0;
      e.s[j >> 6] = 1ull << (j & 63);
      e.next_u64();
      for (int w = 0; w < 4; ++w) m->col[j][w] = e.s[w];
    }
    return m;
  }();
  Gf2Mat* a = new Gf2Mat(*step);
  Gf2Mat* b = new Gf2Mat;
  while (d) {
    if (d & 1) {
      uint64_t out[4];
      a->apply(x.s, out);
      for (int w = 0; w < 4; ++w) x.s[w] = out[w];
    }
    d >>= 1;
    if (d) {  // a <- a * a
      for (int j = 0; j < 256; ++j) a->apply(a->col[j], b->col[j]);
      std::swap(a, b);
    }
  }
  delete a;
  delete b;
}

// ranf: one reset maps the 55 slots linearly over Z/1e9 (for states in
// [0, 1e9), where `v < 0 ? v + 1e9 : v` is v mod 1e9): block r = T^r block 0.
struct RanfMat {
  uint64_t m[55][55];  // m[i][j]: slot i + 1 from slot j + 1
};

void ranf_mat_mul(const RanfMat& A, const RanfMat& B, RanfMat& C) {
  for (int i = 0; i < 55; ++i)
    for (int j = 0; j < 55; ++j) {
      uint64_t acc = 0;
      for (int k = 0; k < 55; ++k) {
        acc += A.m[i][k] * B.m[k][j];
        if ((k & 15) == 15) acc %= (uint64_t)kModulo;
      }
      C.m[i][j] = acc % (uint64_t)kModulo;
    }
}

bool ranf_advance(Ranf& r, uint64_t d) {
  for (int s = 1; s < 56; ++s)
    if (r.n[s] < 0 || r.n[s] >= kModulo) return false;
  const uint64_t total = (uint64_t)(55 - r.index) + d;  // draws from the start of the current block
  uint64_t blocks = total / 55;
  RanfMat* a = new RanfMat;
  for (int j = 0; j < 55; ++j) {  // column j: one reset of the unit vector e_j
    int64_t v[56] = {0};
    v[j + 1] = 1;
    for (int i = 1; i < 25; ++i) v[i] = ((v[i] - v[i + 31]) % kModulo + kModulo) % kModulo;
    for (int i = 25; i < 56; ++i) v[i] = ((v[i] - v[i - 24]) % kModulo + kModulo) % kModulo;
    for (int i = 0; i < 55; ++i) a->m[i][j] = (uint64_t)v[i + 1];
  }
  RanfMat* t = new RanfMat;
  while (blocks) {
    if (blocks & 1) {
      uint64_t out[55];
      for (int i = 0; i < 55; ++i) {
        uint64_t acc = 0;
        for (int k = 0; k < 55; ++k) {
          acc += a->m[i][k] * (uint64_t)r.n[k + 1];
          if ((k & 15) == 15) acc %= (uint64_t)kModulo;
        }
        out[i] = acc % (uint64_t)kModulo;
      }
      for (int i = 0; i < 55; ++i) r.n[i + 1] = (int32_t)out[i];
    }
    blocks >>= 1;
    if (blocks) {
      ranf_mat_mul(*a, *a, *t);
      std::swap(a, t);
    }
  }
  delete a;
  delete t;
  r.index = (int)(55 - total % 55);
  return true;
}

uint64_t batch_size(const tp_config& cfg, uint64_t b) {
  const uint64_t lo = b * kBatch;
  if (lo >= cfg.num_events) return 0;
  const uint64_t hi = lo + kBatch;
  return (hi > cfg.num_events ? cfg.num_events : hi) - lo;
}

bool cfg_ok(const tp_config* cfg) {
  return cfg && cfg->num_events > 0 && std::isfinite(cfg->e_total) && cfg->e_total > 0;
}

// ---------------------------------------------------------------------------
// Rust float formatting
// ---------------------------------------------------------------------------
// Rust hides the sign of zero in the goldens' toolchain; NaN prints "NaN".
std::string rust_fixed(double x, int prec) {
  if (std::isnan(x)) return "NaN";
  if (std::isinf(x)) return x > 0 ? "inf" : "-inf";
  if (x == 0.0) x = 0.0;
  char buf[512];
  std::snprintf(buf, sizeof buf, "%.*f", prec, x);
  return buf;
}
std::string rust_exp(double x, int prec) {
  if (std::isnan(x)) return "NaN";
  if (std::isinf(x)) return x > 0 ? "inf" : "-inf";
  if (x == 0.0) x = 0.0;
  char buf[512];
  std::snprintf(buf, sizeof buf, "%.*e", prec, x);
  std::string s(buf);
  const size_t e = s.find('e');
  const int ex = std::atoi(s.c_str() + e + 1);
  return s.substr(0, e) + "e" + std::to_string(ex);
}
// Display {} for f64: shortest round-trip digits, positional notation
std::string rust_display(double x) {
  if (std::isnan(x)) return "NaN";
  if (std::isinf(x)) return x > 0 ? "inf" : "-inf";
  if (x == 0.0) return "0";
  char buf[512];
  auto r = std::to_chars(buf, buf + sizeof buf, x, std::chars_format::fixed);
  return std::string(buf, r.ptr);
}
std::string pad_left(const std::string& s, size_t w) {
  return s.size() >= w ? s : std::string(w - s.size(), ' ') + s;
}
std::string pad_right(const std::string& s, size_t w) {
  return s.size() >= w ? s : s + std::string(w - s.size(), ' ');
}

// write_engineering (output.rs:230-269) with SIG_DIGITS = 14
std::string engineering(double x) {
  const int sig_digits = 14;
  long precision = sig_digits - 1;
  if (x == 0.0) return "0";
  const double log_x = std::log10(std::fabs(x));
  if (log_x >= -3.0 && log_x <= (double)sig_digits) {
    precision = precision - (long)std::trunc(log_x);
    if (log_x < 0.0) precision += 1;
    std::string s = rust_fixed(x, (int)precision);
    if (s.find('.') != std::string::npos) {
      while (!s.empty() && s.back() == '0') s.pop_back();
      while (!s.empty() && s.back() == '.') s.pop_back();
    }
    return s;
  }
  return rust_exp(x, (int)precision);
}

std::string kv(const char* key, const std::string& val) {
  return " " + pad_right(key, 31) + ": " + val + "\n";
}

}  // namespace

// ===========================================================================
// C ABI of the oracle
// ===========================================================================
extern "C" {

int tpo_config_load(const char* path, tp_config* out, char* echo, size_t echo_len) {
  std::ifstream f(path);
  if (!f || !out) return TP_ERR_IO;
  std::vector<std::string> items;
  std::string line;
  while (std::getline(f, line)) {
    std::istringstream ls(line);
    std::string tok;
    if (ls >> tok) items.push_back(tok);
  }
  if (items.size() < 18) return TP_ERR_INVALID;
  auto pf = [&](int i, double& d) {
    char* end = nullptr;
    d = std::strtod(items[i].c_str(), &end);
    return end && *end == 0;
  };
  auto pb = [&](int i, int32_t& b) {
    std::string s = items[i];
    for (auto& c : s) c = (char)std::tolower((unsigned char)c);
    if (s == ".true." || s == "true") b = 1;
    else if (s == ".false." || s == "false") b = 0;
    else return false;
    return true;
  };
  tp_config c{};
  {
    char* end = nullptr;
    if (items[0].empty() || items[0][0] == '-') return TP_ERR_INVALID;
    c.num_events = std::strtoull(items[0].c_str(), &end, 10);
    if (!end || *end) return TP_ERR_INVALID;
  }
  double* dst[14] = {&c.e_total, &c.beam_photons_cut, &c.photon_photon_cut, &c.e_min,
                     &c.beam_photon_plane_cut, &c.alpha, &c.alpha_z, &c.gev2_to_picobarn,
                     &c.m_z0, &c.g_z0, &c.sin2_weinberg, &c.branching_ep_em,
                     &c.beta_plus, &c.beta_minus};
  for (int i = 0; i < 14; ++i)
    if (!pf(1 + i, *dst[i])) return TP_ERR_INVALID;
  {
    char* end = nullptr;
    long nb = std::strtol(items[15].c_str(), &end, 10);
    if (!end || *end) return TP_ERR_INVALID;
    c.num_bins = (int32_t)nb;
  }
  if (!pb(16, c.impr) || !pb(17, c.plot)) return TP_ERR_INVALID;
  if (echo && echo_len) {
    std::string s;
    s += "ITOT           : " + std::to_string(c.num_events) + "\n";
    s += "ETOT           : " + rust_display(c.e_total) + "\n";
    s += "oCutpar.ACUT   : " + rust_display(c.beam_photons_cut) + "\n";
    s += "oCutpar.BCUT   : " + rust_display(c.photon_photon_cut) + "\n";
    s += "oCutpar.EMIN   : " + rust_display(c.e_min) + "\n";
    s += "oCutpar.SINCUT : " + rust_display(c.beam_photon_plane_cut) + "\n";
    s += "ALPHA          : " + rust_display(c.alpha) + "\n";
    s += "ALPHAZ         : " + rust_display(c.alpha_z) + "\n";
    s += "CONVERS        : " + rust_display(c.gev2_to_picobarn) + "\n";
    s += "oParam.MZ0     : " + rust_display(c.m_z0) + "\n";
    s += "oParam.GZ0     : " + rust_display(c.g_z0) + "\n";
    s += "SIN2W          : " + rust_display(c.sin2_weinberg) + "\n";
    s += "BREPEM         : " + rust_display(c.branching_ep_em) + "\n";
    s += "BETAPLUS       : " + rust_display(c.beta_plus) + "\n";
    s += "BETAMOINS      : " + rust_display(c.beta_minus) + "\n";
    s += "NBIN           : " + std::to_string(c.num_bins) + "\n";
    s += std::string("oParam.IMPR    : ") + (c.impr ? "true" : "false") + "\n";
    s += std::string("PLOT           : ") + (c.plot ? "true" : "false") + "\n";
    std::snprintf(echo, echo_len, "%s", s.c_str());
  }
  *out = c;
  if (c.num_events == 0 || c.plot || c.impr) return TP_ERR_INVALID;
  return TP_OK;
}

double tpo_event_weight(double e_total) { return event_weight(e_total); }

void tpo_couplings(const tp_config* cfg, double out[3]) {
  Consts k = make_consts(*cfg);
  out[0] = k.g_a;
  out[1] = k.g_beta_p;
  out[2] = k.g_beta_m;
}

void tpo_sigma_contribs(const tp_config* cfg, double out[5]) {
  Consts k = make_consts(*cfg);
  for (int i = 0; i < 5; ++i) out[i] = k.sigma_contribs[i];
}

// Raw uniforms of a stream: draws [skip, skip + n) of one stream, or of
// batch `jumps` when the per-batch jump is requested (jumps > 0 applies
// RandomGenerator::jump that many times first).
int tpo_draws(int rng_kind, uint64_t seed, uint64_t jumps, uint64_t skip, uint64_t n, double* out) {
  Rng rng;
  rng.init(rng_kind & TP_RNG_KIND_MASK, seed);
  for (uint64_t j = 0; j < jumps; ++j) rng.jump();
  for (uint64_t i = 0; i < skip; ++i) rng.random();
  for (uint64_t i = 0; i < n; ++i) out[i] = rng.random();
  return TP_OK;
}

// Raw xoshiro256+ state after seeding and `jumps` 2^128 jumps
void tpo_xoshiro_state(uint64_t seed, uint64_t jumps, uint64_t state[4]) {
  Xoshiro x;
  x.init(seed);
  for (uint64_t j = 0; j < jumps; ++j) x.jump();
  for (int w = 0; w < 4; ++w) state[w] = x.s[w];
}

// Applies the 2^128 jump to an arbitrary xoshiro256 state
void tpo_xoshiro_jump128(uint64_t state[4]) {
  Xoshiro x;
  for (int w = 0; w < 4; ++w) x.s[w] = state[w];
  x.jump();
  for (int w = 0; w < 4; ++w) state[w] = x.s[w];
}

// Ranf state (slots 1..55 in out[0..55), out[55] = index) after `resets`
// extra resets following seeded_new
void tpo_ranf_state(int32_t seed, uint64_t resets, int32_t out[56]) {
  Ranf r;
  r.init(seed);
  for (uint64_t i = 0; i < resets; ++i) r.reset();
  for (int i = 0; i < 55; ++i) out[i] = r.n[i + 1];
  out[55] = r.index;
}

// Events [first_event, first_event + n) of a run, recomputed one by one.
int tpo_dump_events(const tp_config* cfg, int rng_kind, uint64_t seed, uint64_t first_event, uint64_t n,
                    tp_event_dump* out) {
  if (!cfg_ok(cfg) || !out) return TP_ERR_INVALID;
  const int flags = rng_kind & ~TP_RNG_KIND_MASK;
  if (flags & TPO_MODE_FASTER_EVGEN) return TP_ERR_UNSUPPORTED;
  const Consts k = make_consts(*cfg);
  Rng rng, sched;  // sched: the scheduler's copy, jumped once per batch
  rng.init(rng_kind & TP_RNG_KIND_MASK, seed);
  uint64_t e = 0;
  if (flags & TP_MODE_JUMP_PER_BATCH) {
    const uint64_t b = first_event / kBatch;
    for (uint64_t j = 0; j < b; ++j) rng.jump();
    sched = rng;
    e = b * kBatch;
  }
  for (; e < first_event; ++e)
    for (int i = 0; i < 12; ++i) rng.random();
  Event ev;
  for (uint64_t i = 0; i < n; ++i, ++e) {
    if ((flags & TP_MODE_JUMP_PER_BATCH) && e % kBatch == 0 && i > 0) {
      sched.jump();
      rng = sched;
    }
    tp_event_dump& d = out[i];
    std::memset(&d, 0, sizeof d);
    generate(k, rng, flags, ev, d.uniforms);
    for (int p = 0; p < 3; ++p)
      for (int c = 0; c < 4; ++c) d.p_out[p][c] = ev.p[2 + p][c];
    d.cut = cut(*cfg, flags, ev);
    if (d.cut == 0) m2_sums(k, ev, d.m2_sums);
  }
  return TP_OK;
}

// MEsContributions::m2_sums of given photon momenta ([photon][X,Y,Z,E])
void tpo_m2_sums_of(const tp_config* cfg, const double* p_out, double out[5]) {
  const Consts k = make_consts(*cfg);
  Event ev;
  const double h = cfg->e_total / 2.0;
  const double beams[2][4] = {{-cfg->e_total / 2.0, 0.0, 0.0, h}, {h, 0.0, 0.0, h}};
  for (int c = 0; c < 4; ++c) {
    ev.p[0][c] = beams[0][c];
    ev.p[1][c] = beams[1][c];
  }
  for (int p = 0; p < 3; ++p)
    for (int c = 0; c < 4; ++c) ev.p[2 + p][c] = p_out[4 * p + c];
  m2_sums(k, ev, out);
}

// Per-batch accumulators of batches [first_batch, first_batch + n_batches),
// computed the way the reference's schedulers do: one stream consumed in
// event order (skipping to first_batch by stepping), or one jumped stream per
// batch. threads > 1 runs batches in parallel (batch start states are
// prepared first by the stepping / jumping the reference's scheduler does).
// The batches of a run whose stream starts from `seed` jumped `jumps`
// times by RandomGenerator::jump (xoshiro: 2^128 draws, standard.rs:53-55;
// ranf: reseeded with seed + 123456 per jump, ranf.rs:137-140). jumps = 0 is
// the reference's run; jumps = p is one stream per parameter point p.
static int run_batches_from(const tp_config* cfg, int rng_kind, uint64_t seed, uint64_t jumps, uint64_t first_batch,
                            uint64_t n_batches, tp_batch_soa* out, int threads) {
  if (!cfg_ok(cfg) || !out) return TP_ERR_INVALID;
  const int flags = rng_kind & ~TP_RNG_KIND_MASK;
  const int kind = rng_kind & TP_RNG_KIND_MASK;
  if (kind != TP_RNG_RANF && kind != TP_RNG_XOSHIRO256P) return TP_ERR_INVALID;
  const Consts k = make_consts(*cfg);
  Rng rng;
  rng.init(kind, seed);
  for (uint64_t j = 0; j < jumps; ++j) rng.jump();
  // position the stream at first_batch: one-stream default-mode runs by a
  // matrix power (12 draws per event), the others batch by batch
  uint64_t skipped = 0;
  if (!(flags & (TP_MODE_JUMP_PER_BATCH | TPO_MODE_FASTER_EVGEN)) && first_batch > 0) {
    const uint64_t events = first_batch * (uint64_t)kBatch < cfg->num_events ? first_batch * (uint64_t)kBatch
                                                                               : cfg->num_events;
    if (kind == TP_RNG_XOSHIRO256P) {
      xoshiro_advance(rng.xo, 12 * events);
      skipped = first_batch;
    } else if (ranf_advance(rng.ranf, 12 * events)) {
      skipped = first_batch;
    }
  }
  for (uint64_t b = skipped; b < first_batch; ++b) {
    if (flags & TP_MODE_JUMP_PER_BATCH)
      rng.jump();
    else
      skip_batch(rng, flags, batch_size(*cfg, b));
  }
  auto store = [&](uint64_t i, const Acc& a) {
    out->selected[i] = a.selected;
    for (int c = 0; c < 5; ++c) {
      out->spm2[c * n_batches + i] = a.spm2[c];
      out->vars[c * n_batches + i] = a.vars[c];
    }
    out->sigma[i] = a.sigma;
    out->variance[i] = a.variance;
  };
  if (threads <= 1) {
    for (uint64_t i = 0; i < n_batches; ++i) {
      const uint64_t b = first_batch + i;
      Acc a;
      Rng r = rng;
      simulate_batch(*cfg, k, flags, r, batch_size(*cfg, b), a);
      store(i, a);
      if (flags & TP_MODE_JUMP_PER_BATCH)
        rng.jump();
      else
        rng = r;
    }
    return TP_OK;
  }
  std::vector<Rng> starts(n_batches);
  for (uint64_t i = 0; i < n_batches; ++i) {
    starts[i] = rng;
    if (flags & TP_MODE_JUMP_PER_BATCH)
      rng.jump();
    else
      skip_batch(rng, flags, batch_size(*cfg, first_batch + i));
  }
  std::atomic<uint64_t> next{0};
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t)
    pool.emplace_back([&] {
      for (;;) {
        const uint64_t i = next.fetch_add(1);
        if (i >= n_batches) break;
        Acc a;
        Rng r = starts[i];
        simulate_batch(*cfg, k, flags, r, batch_size(*cfg, first_batch + i), a);
        store(i, a);
      }
    });
  for (auto& th : pool) th.join();
  return TP_OK;
}

int tpo_run_batches(const tp_config* cfg, int rng_kind, uint64_t seed, uint64_t first_batch, uint64_t n_batches,
                    tp_batch_soa* out, int threads) {
  return run_batches_from(cfg, rng_kind, seed, 0, first_batch, n_batches, out, threads);
}

int tpo_run_batches_jumped(const tp_config* cfg, int rng_kind, uint64_t seed, uint64_t jumps, uint64_t first_batch,
                           uint64_t n_batches, tp_batch_soa* out, int threads) {
  return run_batches_from(cfg, rng_kind, seed, jumps, first_batch, n_batches, out, threads);
}

// Per-bin sums of the kept events of batches [first_batch, first_batch + n):
// out[bin][0..4] = m2_sums, [5] = events, [6] = sum w, [7] = sum w^2, with
// w = m2_sums . sigma_contribs (resacc.rs:126). Bin: ix * ny + iy with x =
// E of the most energetic photon, y = -p_x / E of it (cosine to the e-).
int tpo_binned(const tp_config* cfg, int rng_kind, uint64_t seed, uint64_t first_batch, uint64_t n_batches, int nx,
               int ny, double xlo, double xhi, double ylo, double yhi, double* out) {
  if (!cfg_ok(cfg) || !out || nx < 1 || ny < 1) return TP_ERR_INVALID;
  const int flags = rng_kind & ~TP_RNG_KIND_MASK;
  const Consts k = make_consts(*cfg);
  const double xinv = nx / (xhi - xlo), yinv = ny / (yhi - ylo);
  for (int i = 0; i < nx * ny * 8; ++i) out[i] = 0.0;
  Rng rng, sched;
  rng.init(rng_kind & TP_RNG_KIND_MASK, seed);
  sched = rng;
  for (uint64_t b = 0; b < first_batch; ++b) {
    if (flags & TP_MODE_JUMP_PER_BATCH) {
      sched.jump();
      rng = sched;
    } else {
      skip_batch(rng, flags, batch_size(*cfg, b));
    }
  }
  Event ev;
  for (uint64_t i = 0; i < n_batches; ++i) {
    const uint64_t n = batch_size(*cfg, first_batch + i);
    for (uint64_t e = 0; e < n; ++e) {
      generate(k, rng, flags, ev, nullptr);
      if (cut(*cfg, flags, ev) != 0) continue;
      double m[5];
      m2_sums(k, ev, m);
      int l = 0;
      if (ev.p[3][3] > ev.p[2 + l][3]) l = 1;
      if (ev.p[4][3] > ev.p[2 + l][3]) l = 2;
      const double en = ev.p[2 + l][3], c = -ev.p[2 + l][0] / en;
      int ix = (int)std::floor((en - xlo) * xinv), iy = (int)std::floor((c - ylo) * yinv);
      ix = ix < 0 ? 0 : (ix >= nx ? nx - 1 : ix);
      iy = iy < 0 ? 0 : (iy >= ny ? ny - 1 : iy);
      double* o = out + 8 * (ix * ny + iy);
      double w = 0.0;
      for (int cc = 0; cc < 5; ++cc) {
        o[cc] += m[cc];
        w += m[cc] * k.sigma_contribs[cc];
      }
      o[5] += 1.0;
      o[6] += w;
      o[7] += w * w;
    }
    if (flags & TP_MODE_JUMP_PER_BATCH) {
      sched.jump();
      rng = sched;
    }
  }
  return TP_OK;
}

// ResultsAccumulator::merge in batch order + finalize (resacc.rs:133-223)
int tpo_merge_finalize(const tp_config* cfg, const tp_batch_soa* b, uint64_t n, tp_final_results* res) {
  if (!cfg_ok(cfg) || !b || !res || n == 0) return TP_ERR_INVALID;
  const Consts k = make_consts(*cfg);
  Acc acc;
  for (uint64_t i = 0; i < n; ++i) {
    acc.selected += b->selected[i];
    for (int c = 0; c < 5; ++c) acc.spm2[c] += b->spm2[c * n + i];
    for (int c = 0; c < 5; ++c) acc.vars[c] += b->vars[c * n + i];
    acc.sigma += b->sigma[i];
    acc.variance += b->variance[i];
  }
  const double n_ev = (double)cfg->num_events;
  double vars[5];
  for (int c = 0; c < 5; ++c) {
    double v = (acc.vars[c] - powi(acc.spm2[c], 2) / n_ev) / (n_ev - 1.0);
    v = std::sqrt(v / n_ev) / std::fabs(acc.spm2[c] / n_ev);
    vars[c] = v;
  }
  double spm2[2][5];
  for (int s = 0; s < 2; ++s)
    for (int c = 0; c < 5; ++c) {
      spm2[s][c] = acc.spm2[c];
      res->vars[s][c] = vars[c];
    }
  const double polar_p = -2.0 * cfg->sin2_weinberg;
  const double polar_m = 1.0 + polar_p;
  const double polars[2] = {polar_m, polar_p};
  for (int c = 1; c < 5; ++c)
    for (int s = 0; s < 2; ++s) spm2[s][c] *= polars[s];
  for (int c = 1; c < 3; ++c)
    for (int s = 0; s < 2; ++s) spm2[s][c] *= polars[s];
  const double flux = 1.0 / (2.0 * powi(cfg->e_total, 2));
  const double f = k.fact_com * flux * k.norm_weight;
  for (int s = 0; s < 2; ++s)
    for (int c = 0; c < 5; ++c) spm2[s][c] *= f;
  const double gm_z0 = cfg->g_z0 * cfg->m_z0;
  const double pg = k.propagator / gm_z0;
  for (int c = 1; c < 5; ++c)
    for (int s = 0; s < 2; ++s) spm2[s][c] *= pg;
  for (int c = 1; c < 3; ++c)
    for (int s = 0; s < 2; ++s) spm2[s][c] /= gm_z0;
  for (int s = 0; s < 2; ++s) spm2[s][3] *= k.delta;
  auto colsum = [&](int c) { return (0.0 + spm2[0][c]) + spm2[1][c]; };
  auto inc_num = [&](int c) {
    const double a = spm2[0][c] * res->vars[0][c];
    const double b2 = spm2[1][c] * res->vars[1][c];
    return std::sqrt(0.0 + (a * a + b2 * b2));
  };
  res->beta_min = std::sqrt(colsum(0) / colsum(1));
  const double ss_denom = colsum(0);
  const double ss_norm = 1.0 / (2.0 * std::sqrt(ss_denom));
  res->ss_p = colsum(1) * ss_norm;
  res->ss_m = colsum(2) * ss_norm;
  const double inc_common = inc_num(0) / (2.0 * std::fabs(ss_denom));
  res->inc_ss_p = inc_num(1) / std::fabs(colsum(1)) + inc_common;
  res->inc_ss_m = inc_num(2) / std::fabs(colsum(2)) + inc_common;
  const double variance = (acc.variance - powi(acc.sigma, 2) / n_ev) / (n_ev - 1.0);
  res->prec = std::sqrt(variance / n_ev) / std::fabs(acc.sigma / n_ev);
  res->sigma = acc.sigma * flux;
  res->variance = variance;
  res->selected_events = acc.selected;
  for (int s = 0; s < 2; ++s)
    for (int c = 0; c < 5; ++c) res->spm2[s][c] = spm2[s][c];
  return TP_OK;
}

// res.data text (output.rs:62-142)
int tpo_format_res_data(const tp_config* cfg, const tp_final_results* r, char* buf, size_t len) {
  std::string s;
  s += kv("Nombre d'evenements", std::to_string(cfg->num_events));
  s += kv("... apres coupure", std::to_string(r->selected_events));
  s += kv("energie dans le CdM      (GeV)", engineering(cfg->e_total));
  s += kv("coupure / cos(photon,faisceau)", engineering(cfg->beam_photons_cut));
  s += kv("coupure / cos(photon,photon)", engineering(cfg->photon_photon_cut));
  s += kv("coupure / sin(normale,faisceau)", engineering(cfg->beam_photon_plane_cut));
  s += kv("coupure sur l'energie    (GeV)", engineering(cfg->e_min));
  s += kv("1/(constante de structure fine)", engineering(1.0 / cfg->alpha));
  s += kv("1/(structure fine au pic)", engineering(1.0 / cfg->alpha_z));
  s += kv("facteur de conversion GeV-2/pb", engineering(cfg->gev2_to_picobarn));
  s += kv("Masse du Z0              (GeV)", engineering(cfg->m_z0));
  s += kv("Largeur du Z0            (GeV)", engineering(cfg->g_z0));
  s += kv("Sinus^2 Theta Weinberg", engineering(cfg->sin2_weinberg));
  s += kv("Taux de branchement Z--->e+e-", engineering(cfg->branching_ep_em));
  s += kv("Beta plus", engineering(cfg->beta_plus));
  s += kv("Beta moins", engineering(cfg->beta_minus));
  s += " ---------------------------------------------\n";
  s += kv("Section Efficace          (pb)", engineering(r->sigma));
  s += kv("Ecart-Type                (pb)", engineering(r->sigma * r->prec));
  s += kv("Precision Relative", engineering(r->prec));
  s += " ---------------------------------------------\n";
  s += kv("Beta minimum", engineering(r->beta_min));
  s += kv("Stat. Significance  B+(pb-1/2)", engineering(r->ss_p));
  s += kv("Incert. Stat. Sign. B+(pb-1/2)", engineering(r->ss_p * r->inc_ss_p));
  s += kv("Stat. Significance  B-(pb-1/2)", engineering(r->ss_m));
  s += kv("Incert. Stat. Sign. B-(pb-1/2)", engineering(r->ss_m * r->inc_ss_m));
  s += "\n";
  const int decs = 7, width = decs + 8;
  for (int sp = 0; sp < 2; ++sp) {
    for (int c = 0; c < 5; ++c) {
      s += pad_left(std::to_string(sp + 1), 3) + pad_left(std::to_string(c + 1), 3);
      s += pad_left(rust_exp(r->spm2[sp][c], decs), width);
      s += pad_left(rust_exp(std::fabs(r->spm2[sp][c]) * r->vars[sp][c], decs), width);
      s += pad_left(rust_exp(r->vars[sp][c], decs), width);
      s += "\n";
    }
    s += "\n";
  }
  for (int c = 0; c < 5; ++c) {
    const double tmp1 = (0.0 + r->spm2[0][c]) + r->spm2[1][c];
    const double a = r->spm2[0][c] * r->vars[0][c];
    const double b = r->spm2[1][c] * r->vars[1][c];
    const double tmp2 = std::sqrt(0.0 + (a * a + b * b));
    s += "   " + pad_left(std::to_string(c + 1), 3);
    s += pad_left(rust_exp(tmp1 / 4.0, decs), width);
    s += pad_left(rust_exp(tmp2 / 4.0, decs), width);
    s += pad_left(rust_exp(tmp2 / std::fabs(tmp1), decs), width);
    s += "\n";
  }
  if (buf && len) std::snprintf(buf, len, "%s", s.c_str());
  return (int)s.size();
}

// stdout of the run after the config echo: "IBegin", eric, fawzi
// (evgen.rs:47, resfin.rs:66-194)
int tpo_format_report(const tp_config* cfg, const tp_final_results* r, char* buf, size_t len) {
  std::string s = "IBegin\n";
  const auto& m = r->spm2;
  auto line = [&](const std::string& l) { s += l + "\n"; };
  // eric
  const double mu_th = cfg->branching_ep_em * cfg->gev2_to_picobarn /
                       ((8.0 * 9.0 * 5.0 * std::pow(kPi, 2.0)) * cfg->m_z0 * cfg->g_z0);
  double sigma0[2], alpha0[2], beta0[2], lambda0[2], mu0[2];
  for (int sp = 0; sp < 2; ++sp) {
    sigma0[sp] = m[sp][0] / 2.0;
    alpha0[sp] = m[sp][4] / 2.0;
    beta0[sp] = -m[sp][3] / 2.0;
    lambda0[sp] = (m[sp][2] - m[sp][1]) / 2.0;
    mu0[sp] = (m[sp][2] + m[sp][1]) / 2.0;
  }
  const double mu_num = ((((0.0 + m[0][1]) + m[1][1]) + m[0][2]) + m[1][2]) / 4.0;
  line("");
  line("       :        -          +");
  line("sigma0  : " + rust_fixed(sigma0[0], 6) + " | " + rust_fixed(sigma0[1], 6));
  line("alpha0  : " + rust_exp(alpha0[0], 5) + " | " + rust_exp(alpha0[1], 4));
  line("beta0   : " + rust_display(beta0[0]) + " | " + rust_display(beta0[1]));
  line("lambda0 : " + rust_fixed(lambda0[0], 4) + " | " + rust_fixed(lambda0[1], 4));
  line("mu0     : " + rust_fixed(mu0[0], 4) + " | " + rust_fixed(mu0[1], 5));
  line("mu/lamb : " + rust_fixed(mu0[0] / lambda0[0], 5) + " | " + rust_fixed(mu0[1] / lambda0[1], 5));
  line("mu (num): " + rust_fixed(mu_num, 4));
  line("rapport : " + rust_fixed(mu_num / mu_th, 6));
  line("mu (th) : " + rust_fixed(mu_th, 4));
  // fawzi
  const double mre = cfg->m_z0 / cfg->e_total;
  const double gre = cfg->g_z0 * cfg->m_z0 / powi(cfg->e_total, 2);
  const double x = 1.0 - powi(mre, 2);
  const double sd = powi(x, 2) + powi(gre, 2);
  const C sdz{x / sd, -gre / sd};
  const double del = (1.0 - cfg->photon_photon_cut) / 2.0;
  const double eps = 2.0 * cfg->e_min / cfg->e_total;
  const double bra = cfg->m_z0 / (3.0 * 6.0 * std::pow(kPi, 3.0) * 16.0 * 120.0);
  const double sig = 12.0 * kPi / powi(cfg->m_z0, 2) * cfg->branching_ep_em * cfg->g_z0 * bra /
                     powi(cfg->e_total, 2) * powi(cfg->e_total / cfg->m_z0, 8) * norm_sqr(sdz) *
                     cfg->gev2_to_picobarn;
  const double eps_4 = powi(eps, 4);
  const double del_2 = powi(del, 2);
  const double del_3 = powi(del, 3);
  const double f1 = 1.0 - 15.0 * eps_4 - 9.0 / 7.0 * (1.0 - 70.0 * eps_4) * del_2 +
                    6.0 / 7.0 * (1.0 + 70.0 * eps_4) * del_3;
  const double g1 = 1.0 - 30.0 * eps_4 - 9.0 / 7.0 * (1.0 - 70.0 * eps_4) * del - 90.0 * eps_4 * del_2 -
                    1.0 / 7.0 * (1.0 - 420.0 * eps_4) * del_3;
  const double g2 = 1.0 - 25.0 * eps_4 - 6.0 / 7.0 * (1.0 - 70.0 * eps_4) * del -
                    3.0 / 7.0 * (1.0 + 210.0 * eps_4) * del_2 - 8.0 / 21.0 * (1.0 - 52.5 * eps_4) * del_3;
  const double g3 = 1.0 - 195.0 / 11.0 * eps_4 - 18.0 / 77.0 * (1.0 - 7.0 * eps_4) * del -
                    9.0 / 11.0 * (9.0 / 7.0 - 70.0 * eps_4) * del_2 -
                    8.0 / 11.0 * (1.0 - 105.0 / 11.0 * eps_4) * del_3;
  const double sc3 = powi(cfg->beam_photon_plane_cut, 3);
  const double ff = f1 * (1.0 - sc3);
  const double gg = g1 - 27.0 / 16.0 * g2 * cfg->beam_photon_plane_cut + 11.0 / 16.0 * g3 * sc3;
  const double sig_p = sig * (ff + 2.0 * gg);
  const double sig_m = sig_p + 2.0 * sig * gg;
  const double mc_p = ((0.0 + m[0][1]) + m[1][1]) / 4.0;
  const double mc_m = ((0.0 + m[0][2]) + m[1][2]) / 4.0;
  auto incr = [&](int c) {
    const double a = m[0][c] * r->vars[0][c];
    const double b = m[1][c] * r->vars[1][c];
    return std::sqrt(0.0 + (a * a + b * b)) / std::fabs((0.0 + m[0][c]) + m[1][c]);
  };
  const double incr_p = incr(1), incr_m = incr(2);
  line("");
  line("s (pb) :   Sig_cut_Th    Sig_Th      Rapport");
  line("       :   Sig_Num");
  line("       :   Ecart_relatif  Incertitude");
  line("");
  line("s+(pb) : " + rust_fixed(sig_p, 5) + " | " + rust_fixed(sig * 3.0, 5) + " | " +
       rust_fixed(sig_p / (3.0 * sig), 6));
  line("       : " + rust_fixed(mc_p, 5));
  line("       : " + rust_fixed(mc_p / sig_p - 1.0, 6) + " | " + rust_fixed(incr_p, 8) + " | " +
       rust_fixed((mc_p / sig_p - 1.0) / incr_p, 2));
  line("");
  line("s-(pb) : " + rust_fixed(sig_m, 5) + " | " + rust_fixed(sig * 5.0, 4) + " | " +
       rust_fixed(sig_m / (5.0 * sig), 6));
  line("       : " + rust_fixed(mc_m, 5));
  line("       : " + rust_fixed(mc_m / sig_m - 1.0, 6) + " | " + rust_fixed(incr_m, 9) + " | " +
       rust_fixed((mc_m / sig_m - 1.0) / incr_m, 2));
  line("");
  if (buf && len) std::snprintf(buf, len, "%s", s.c_str());
  return (int)s.size();
}

}  // extern "C"
