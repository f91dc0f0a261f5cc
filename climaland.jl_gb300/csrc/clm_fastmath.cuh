// Table-driven FP64 exp and log for the column kernels.
//
// GB300 runs FP64 at a small fraction of its FP32 rate, and the soil physics
// spends most of its FP64 instructions in exp and log (every van Genuchten
// power is exp(b log a)). These follow Tang's published table-driven methods
// (ACM TOMS 15(2) 1989 for exp, 16(4) 1990 for log) with 64-entry tables
// (clm_fastmath_tables.h, generated by gen_fastmath_tables.py) and Taylor
// polynomials, and cost about 10 (exp) and 14 (log) FP64 operations. Errors
// are below about 1 ulp in the ranges the physics uses; arguments outside the
// fast ranges (non-finite, non-positive or subnormal for log, |x| > 700 for
// exp) go to the CUDA math library.
//
// The same code compiles for the host, so a CPU harness can replay the
// kernels bit for bit apart from FMA contraction.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#include "clm_fastmath_tables.h"

#ifndef CLM_HD
#define CLM_HD __host__ __device__ __forceinline__
#endif

namespace clm {
namespace fm {

// Where the tables live: shared memory on the device (copied once per CTA),
// the static arrays on the host.
struct Tables {
  const double* exp2j;
  const double* invc;
  const double* logc_hi;
  const double* logc_lo;
  const float* ff;  // 2^(j/64) as float pairs (hi[64], lo[64]) for clm_ff.cuh
};

// Staged size in doubles: the FP64 tables, then 128 floats of pairs.
constexpr int kStageDoubles = TABLE_SIZE + 64;

static const double kTableHost[TABLE_SIZE] = CLM_FM_TABLE_INIT;

inline Tables host_tables() {
  static float pairs[128];
  static bool filled = false;
  if (!filled) {
    for (int j = 0; j < 64; ++j) {
      const float hi = (float)kTableHost[j];
      pairs[j] = hi;
      pairs[64 + j] = (float)(kTableHost[j] - (double)hi);
    }
    filled = true;
  }
  return Tables{kTableHost, kTableHost + 64, kTableHost + 128, kTableHost + 192, pairs};
}

#ifdef __CUDACC__
static __constant__ double kTableConst[TABLE_SIZE] = CLM_FM_TABLE_INIT;

// Copy the tables into shared memory (stage_doubles<kPairs>() doubles at
// `sm`); the caller synchronises the block before use. Lanes look up
// data-dependent entries, which shared memory serves without the
// serialisation that divergent constant-memory reads incur. kPairs: also the
// float pairs of the double-float code (mixed path only).
template <bool kPairs>
__host__ __device__ constexpr int stage_doubles() { return kPairs ? kStageDoubles : TABLE_SIZE; }

template <bool kPairs = false>
__device__ __forceinline__ Tables stage_tables(double* sm) {
  for (int i = threadIdx.x; i < TABLE_SIZE; i += blockDim.x) sm[i] = kTableConst[i];
  float* pairs = nullptr;
  if (kPairs) {
    pairs = reinterpret_cast<float*>(sm + TABLE_SIZE);
    for (int j = threadIdx.x; j < 64; j += blockDim.x) {
      const float hi = (float)kTableConst[j];
      pairs[j] = hi;
      pairs[64 + j] = (float)(kTableConst[j] - (double)hi);
    }
  }
  return Tables{sm, sm + 64, sm + 128, sm + 192, pairs};
}
#endif

CLM_HD int64_t bits_of(double x) {
#ifdef __CUDA_ARCH__
  return __double_as_longlong(x);
#else
  int64_t b;
  std::memcpy(&b, &x, sizeof b);
  return b;
#endif
}

CLM_HD double from_bits(int64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double(b);
#else
  double x;
  std::memcpy(&x, &b, sizeof x);
  return x;
#endif
}

// exp(x): x = (64 k' + j) ln2/64 + r, |r| <= ln2/128;
// exp(x) = 2^k' 2^(j/64) (1 + expm1(r)), expm1 by its degree-5 Taylor
// polynomial (truncation < 4e-17).
// Range checks compare the bit patterns as integers (the FP64 pipe is the
// scarce one): |x| <= 700 <=> (bits & ~sign) <= bits(700), NaN included in
// the slow path since its magnitude bits exceed those of any finite value.
constexpr int64_t kBits700 = 0x4085E00000000000LL;  // 700.0

CLM_HD double exp(const Tables& T, double x) {
  if ((bits_of(x) & 0x7FFFFFFFFFFFFFFFLL) > kBits700) return ::exp(x);
  const double shifter = 6755399441055744.0;  // 1.5 * 2^52: round to integer
  const double kd = fma(x, INV_LNN, shifter);
  const int64_t k = bits_of(kd) - bits_of(shifter);
  const double kf = kd - shifter;
  double r = fma(-kf, LNN_HI, x);
  r = fma(-kf, LNN_LO, r);
  const int j = (int)(k & 63);
  const int64_t m = k >> 6;
  double q = fma(r, 1.0 / 120.0, 1.0 / 24.0);
  q = fma(q, r, 1.0 / 6.0);
  q = fma(q, r, 0.5);
  const double p = fma(r * r, q, r);  // expm1(r)
  const double t = T.exp2j[j];
  const double y = fma(t, p, t);
  return from_bits(bits_of(y) + m * 4503599627370496LL);  // + m * 2^52
}

// log(x): x = 2^e m, m in [1, 2), j = top six fraction bits of m,
// r = m / c_j - 1 (one fma, |r| <= 1/64), log(x) = e ln2 + log(c_j) +
// log1p(r), log1p by its degree-9 Taylor polynomial (truncation < 1e-19).
CLM_HD double log(const Tables& T, double x) {
  int64_t b = bits_of(x);
  // positive normal finite only: bits in [0x0010000000000000, 0x7FF0000000000000)
  if ((uint64_t)(b - 0x0010000000000000LL) >= (uint64_t)0x7FE0000000000000LL) return ::log(x);
  int e = (int)((b >> 52) & 0x7FF) - 1023;
  const int j = (int)((b >> 46) & 63);
  const double mant = from_bits((b & 0x000FFFFFFFFFFFFFLL) | 0x3FF0000000000000LL);
  e += (j >= 32) ? 1 : 0;
  const double r = fma(mant, T.invc[j], -1.0);
  double q = fma(r, 1.0 / 9.0, -1.0 / 8.0);
  q = fma(q, r, 1.0 / 7.0);
  q = fma(q, r, -1.0 / 6.0);
  q = fma(q, r, 1.0 / 5.0);
  q = fma(q, r, -1.0 / 4.0);
  q = fma(q, r, 1.0 / 3.0);
  q = fma(q, r, -0.5);
  const double l1p = fma(r * r, q, r);
  const double ed = (double)e;
  const double lo = fma(ed, LN2_LO, T.logc_lo[j]) + l1p;
  const double hi = fma(ed, LN2_HI, T.logc_hi[j]);
  return hi + lo;
}

// a^b = exp(b log a) for a > 0 (the van Genuchten powers).
CLM_HD double pow_pos(const Tables& T, double a, double b) { return exp(T, b * log(T, a)); }

// 1/x by Newton-Raphson iteration r <- r + r (1 - x r) from a
// single-precision seed (each step squares the relative error: 2^-22 ->
// 2^-44 -> below 2^-53 before the final rounding; the residual 1 - x r is
// exact in one FMA). Within one ulp of the correctly rounded quotient, for
// four FP64 FMAs; the seed comes from integer re-biasing of x's exponent and
// top significand bits (no conversion instruction) and a float reciprocal.
// |x| outside [2^-120, 2^120], zero, infinities and NaN: the IEEE division.
CLM_HD float rcp_seed(float x) {
#ifdef __CUDA_ARCH__
  return __fdividef(1.0f, x);
#else
  return 1.0f / x;
#endif
}

CLM_HD double rcp(double x) {
  const int64_t b = bits_of(x);
  const int e = (int)((b >> 52) & 0x7FF);
  if (e < 1023 - 120 || e > 1023 + 120) return 1.0 / x;
  // x as a float with its significand truncated to 24 bits
  const uint32_t fb = (uint32_t)((uint64_t)b >> 32 & 0x80000000u) |
                      ((uint32_t)(e - 1023 + 127) << 23) | (uint32_t)((b >> 29) & 0x7FFFFF);
  float xf;
  std::memcpy(&xf, &fb, sizeof xf);
  const float rf = rcp_seed(xf);
  uint32_t rb;
  std::memcpy(&rb, &rf, sizeof rb);
  // the float seed widened to double (normal: |1/x| within [2^-121, 2^121])
  const int64_t db = ((int64_t)(rb & 0x80000000u) << 32) |
                     ((int64_t)(((rb >> 23) & 0xFF) - 127 + 1023) << 52) |
                     ((int64_t)(rb & 0x7FFFFF) << 29);
  double r = from_bits(db);
  double t = fma(-x, r, 1.0);
  r = fma(r, t, r);
  t = fma(-x, r, 1.0);
  return fma(r, t, r);
}

}  // namespace fm
}  // namespace clm
