// tp_math.h — FP64 natural logarithm for the event kernels.
//
// Table-driven method (P. T. P. Tang, "Table-driven implementation of the
// logarithm function in IEEE floating-point arithmetic", ACM TOMS 16, 1990):
// x = 2^k m, m in [1, 2); with j the top 7 mantissa bits, r_j ~ 1/c_j
// (12 significant bits) and t = m r_j - 1 (one FMA, |t| < 2^-8 + 2^-12),
//   log x = k ln2 + (-log r_j) + log1p(t),
// k ln2 and -log r_j carried as hi + lo (hi parts add exactly), log1p(t) by
// its Taylor series to t^8. Near x = 1 (|x - 1| < 1/64) the series of
// log1p(x - 1) to degree 11 is used instead, so that no cancellation
// occurs. The table (tp_log_table.h) is generated by gen_log_table.py with
// arbitrary-precision decimal arithmetic. Arguments that are not positive
// finite normal numbers fall back to the CUDA log.
//
// Cost: ~17 FP64 operations against ~30 DFMA-equivalents for CUDA's log on
// GB300, whose FP64 pipe is narrow. Accuracy: tested against glibc's log
// (tests/test_math.py): faithful rounding everywhere, equal results in the
// vast majority of cases.
#ifndef TP_MATH_H
#define TP_MATH_H

#include <cmath>
#include <cstdint>
#include <cstring>

#include "tp_log_table.h"

#ifdef __CUDACC__
#define TP_HD __host__ __device__ __forceinline__
#else
#define TP_HD inline
#endif

namespace tp {

TP_HD uint64_t dbits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return u;
#endif
}

TP_HD double bitsd(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  std::memcpy(&x, &u, 8);
  return x;
#endif
}

#ifdef __CUDACC__
// device copy of the table (3 KiB, one per translation unit that includes
// this header; read through the read-only cache)
static __device__ const double kTpLogTableDev[128][3] = TP_LOG_TABLE_INIT;
#endif
#ifdef __CUDA_ARCH__
#define TP_LOG_T(j, c) (__ldg(&kTpLogTableDev[(j)][(c)]))
#else
#define TP_LOG_T(j, c) (kTpLogTable[(j)][(c)])
#endif

TP_HD double tp_fma(double a, double b, double c) {
#ifdef __CUDA_ARCH__
  return __fma_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}

TP_HD double tp_log_fallback(double x) {
#ifdef __CUDA_ARCH__
  return ::log(x);
#else
  return std::log(x);
#endif
}

TP_HD double tp_log(double x) {
  const uint64_t u = dbits(x);
  const uint64_t ex = u >> 52;  // sign + exponent
  if (ex == 0 || ex >= 0x7FF) return tp_log_fallback(x);  // <= 0, subnormal, inf, NaN
  const double f = x - 1.0;
  if (f > -0.015625 && f < 0.015625) {
    // log1p(f) = f - f^2/2 + f^3/3 - ... to f^11 (|f| < 2^-6)
    double q = 1.0 / 11.0;
    q = tp_fma(q, f, -1.0 / 10.0);
    q = tp_fma(q, f, 1.0 / 9.0);
    q = tp_fma(q, f, -1.0 / 8.0);
    q = tp_fma(q, f, 1.0 / 7.0);
    q = tp_fma(q, f, -1.0 / 6.0);
    q = tp_fma(q, f, 1.0 / 5.0);
    q = tp_fma(q, f, -1.0 / 4.0);
    q = tp_fma(q, f, 1.0 / 3.0);
    q = tp_fma(q, f, -0.5);
    return tp_fma(f * f, q, f);
  }
  const int k = (int)ex - 1023;
  const uint64_t mb = u & 0x000FFFFFFFFFFFFFull;
  const int j = (int)(mb >> 45);
  const double m = bitsd(mb | 0x3FF0000000000000ull);
  const double t = tp_fma(m, TP_LOG_T(j, 0), -1.0);
  // log1p(t) - t = t^2 (-1/2 + t/3 - t^2/4 + ... - t^6/8)
  double q = -1.0 / 8.0;
  q = tp_fma(q, t, 1.0 / 7.0);
  q = tp_fma(q, t, -1.0 / 6.0);
  q = tp_fma(q, t, 1.0 / 5.0);
  q = tp_fma(q, t, -1.0 / 4.0);
  q = tp_fma(q, t, 1.0 / 3.0);
  q = tp_fma(q, t, -0.5);
  const double kd = (double)k;
  const double hi = tp_fma(kd, TP_LN2_HI, TP_LOG_T(j, 1));  // exact
  const double lo = tp_fma(kd, TP_LN2_LO, TP_LOG_T(j, 2));
  return hi + (t + tp_fma(t * t, q, lo));
}

}  // namespace tp

#endif
