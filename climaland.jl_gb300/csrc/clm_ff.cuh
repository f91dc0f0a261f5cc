// Double-float ("ff") arithmetic on the FP32 pipe for the mixed path.
//
// GB300 issues FP32 at many times its FP64 rate. The mixed path evaluates the
// transcendental soil closures (van Genuchten powers, hydraulic and thermal
// conductivity, temperature) on unevaluated pairs hi + lo of floats, which
// carry about 48 significant bits (relative error near 2^-44 after a few
// operations); IEEE FP64 stays for the Newton residual assembly, the state
// increments, the phase partition and the budgets.
//
// Algorithms (published; written here from their descriptions):
//   two_sum            Knuth, TAOCP vol. 2, 4.2.2 (6 flops, any order)
//   fast_two_sum       Dekker 1971 (|a| >= |b|)
//   two_prod           with a fused multiply-add (exact product error)
//   add, mul, div      Joldes, Muller, Popescu, "Tight and rigorous error
//                      bounds for basic building blocks of double-word
//                      arithmetic", ACM TOMS 44(2) 2017: AccurateDWPlusDW,
//                      DWTimesDW (FMA variant), DWDivDW
//   exp                table-driven (2^(j/64), Tang 1989) with a short
//                      polynomial on a double-word reduced argument
//   log                one Newton step y + x e^(-y) - 1 from the float log
// Every routine compiles for host and device, so the CPU tests check the
// same code; host builds must not contract a*b+c (-ffp-contract=off).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifndef CLM_HD
#define CLM_HD __host__ __device__ __forceinline__
#endif

namespace clm {
namespace ff {

struct F2 {
  float hi, lo;
};

CLM_HD uint32_t fbits(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  uint32_t b;
  std::memcpy(&b, &x, sizeof b);
  return b;
#endif
}

CLM_HD float ffrom(uint32_t b) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float x;
  std::memcpy(&x, &b, sizeof x);
  return x;
#endif
}

CLM_HD uint64_t dbits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  std::memcpy(&b, &x, sizeof b);
  return b;
#endif
}

CLM_HD double dfrom(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double x;
  std::memcpy(&x, &b, sizeof x);
  return x;
#endif
}

// ---- conversion-free helpers ------------------------------------------------
// Float <-> integer conversions and rounding instructions share the FP64
// pipe on GB300; these use FP32 and integer arithmetic instead.
constexpr float kShift = 12582912.0f;  // 1.5 * 2^23

// nearest integer of x (|x| < 2^22), as a float and as an int
CLM_HD float round_f(float x, int& k) {
  const float s = x + kShift;
  k = (int)(fbits(s) - fbits(kShift));
  return s - kShift;
}

// (float)k for |k| < 2^22
CLM_HD float int_to_float(int k) { return ffrom(fbits(kShift) + (uint32_t)k) - kShift; }

// (float)r, correctly rounded, for r < 2^29: two exact 23-bit halves, one rounding
CLM_HD float u29_to_float(uint32_t r) {
  const float lo = ffrom(0x4B000000u | (r & 0x7FFFFFu)) - 8388608.0f;
  const float hi = ffrom(0x4B000000u | (r >> 23)) - 8388608.0f;
  return fmaf(hi, 8388608.0f, lo);
}

// first approximations (multi-function unit on the device)
CLM_HD float log_approx(float x) {
#ifdef __CUDA_ARCH__
  return __logf(x);
#else
  return std::log(x);
#endif
}

CLM_HD float exp_approx(float x) {
#ifdef __CUDA_ARCH__
  return __expf(x);
#else
  return std::exp(x);
#endif
}

// a / b with the multi-function unit's reciprocal on the device (within 2
// ulps for |b| below 2^126; IEEE division on the host). The double-float
// division below recovers its error in the remainder term.
CLM_HD float fast_div(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fdividef(a, b);
#else
  return a / b;
#endif
}

// ---- error-free transformations -------------------------------------------
CLM_HD F2 two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return F2{s, e};
}

CLM_HD F2 fast_two_sum(float a, float b) {
  const float s = a + b;
  const float e = b - (s - a);
  return F2{s, e};
}

CLM_HD F2 two_prod(float a, float b) {
  const float p = a * b;
  const float e = fmaf(a, b, -p);
  return F2{p, e};
}

// ---- double-word operations ---------------------------------------------------
CLM_HD F2 make(float x) { return F2{x, 0.0f}; }
CLM_HD F2 neg(F2 x) { return F2{-x.hi, -x.lo}; }

// AccurateDWPlusDW (relative error <= 3u^2 + 13u^3, u = 2^-24)
CLM_HD F2 add(F2 x, F2 y) {
  F2 s = two_sum(x.hi, y.hi);
  const F2 t = two_sum(x.lo, y.lo);
  float c = s.lo + t.hi;
  const F2 v = fast_two_sum(s.hi, c);
  const float w = t.lo + v.lo;
  return fast_two_sum(v.hi, w);
}

CLM_HD F2 sub(F2 x, F2 y) { return add(x, neg(y)); }

// SloppyDWPlusDW (Joldes, Muller, Popescu, Algorithm 5): relative error of
// order 2^-46 when the operands cannot cancel (same signs, or |y| much
// smaller than |x|; every caller states which), so the accurate variant's
// second two_sum is not needed.
CLM_HD F2 add_small(F2 x, F2 y) {
  const F2 s = two_sum(x.hi, y.hi);
  const float v = x.lo + y.lo;
  const float w = s.lo + v;
  return fast_two_sum(s.hi, w);
}

// DWPlusFP (relative error <= 2u^2)
CLM_HD F2 add_f(F2 x, float y) {
  const F2 s = two_sum(x.hi, y);
  const float v = x.lo + s.lo;
  return fast_two_sum(s.hi, v);
}

// DWTimesDW with FMA (relative error <= 4u^2)
CLM_HD F2 mul(F2 x, F2 y) {
  const F2 c = two_prod(x.hi, y.hi);
  float tl = x.hi * y.lo;
  tl = fmaf(x.lo, y.hi, tl);
  const float cl = c.lo + tl;
  return fast_two_sum(c.hi, cl);
}

// DWTimesFP with FMA (relative error <= 2u^2)
CLM_HD F2 mul_f(F2 x, float y) {
  const F2 c = two_prod(x.hi, y);
  const float cl = fmaf(x.lo, y, c.lo);
  return fast_two_sum(c.hi, cl);
}

// DWDivDW (relative error <= 15u^2 + 56u^3)
// The quotient estimate th need not be correctly rounded: the remainder
// x - th y is exact (two_prod, and Sterbenz for the subtraction of the high
// words) and its quotient tl corrects th to the pair's precision.
CLM_HD F2 div(F2 x, F2 y) {
  const float th = fast_div(x.hi, y.hi);
  const F2 r = mul_f(y, th);
  const float ph = x.hi - r.hi;
  const float dl = x.lo - r.lo;
  const float d = ph + dl;
  const float tl = fast_div(d, y.hi);
  return fast_two_sum(th, tl);
}

// ---- conversions ----------------------------------------------------------------
// double -> hi + lo by splitting the significand with integer operations (no
// FP64 instruction): hi keeps the leading 24 bits, lo the next 24 (rounded),
// then renormalised. For |d| in [2^-70, 2^100] (both parts stay normal);
// outside that range (and for 0, non-finite) through float conversions.
CLM_HD F2 from_double(double d) {
  const uint64_t b = dbits(d);
  const int e = (int)((b >> 52) & 0x7FF);
  if (e < 1023 - 70 || e > 1023 + 100) {
    const float hi = (float)d;
    return F2{hi, (float)(d - (double)hi)};
  }
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  const uint64_t m = b & 0x000FFFFFFFFFFFFFull;
  // hi: exponent e, top 23 fraction bits (truncated)
  const uint32_t hib = sign | ((uint32_t)(e - 1023 + 127) << 23) | (uint32_t)(m >> 29);
  const float hi = ffrom(hib);
  // lo: the remaining 29 fraction bits, value rem * 2^(e - 1023 - 52)
  const uint32_t rem = (uint32_t)(m & 0x1FFFFFFFu);
  const float scale = ffrom((uint32_t)(e - 1023 - 52 + 127) << 23);  // 2^(e-1075), normal
  const float lo = u29_to_float(rem) * scale;  // rem rounded to 24 bits
  return fast_two_sum(hi, sign ? -lo : lo);
}

// float -> double by re-biasing the exponent (normal floats; zero, subnormal
// and non-finite values through the conversion instruction).
CLM_HD double widen(float x) {
  const uint32_t b = fbits(x);
  const uint32_t e = (b >> 23) & 0xFF;
  if (e == 0 || e == 0xFF) return (double)x;
  const uint64_t s = (uint64_t)(b & 0x80000000u) << 32;
  return dfrom(s | ((uint64_t)(e - 127 + 1023) << 52) | ((uint64_t)(b & 0x7FFFFFu) << 29));
}

// hi + lo -> double: both are exact in double; one FP64 addition.
CLM_HD double to_double(F2 x) { return widen(x.hi) + widen(x.lo); }

// float -> double with integer operations only and no branch: exact for
// normal floats; zero and subnormal floats give a signed zero; infinities
// and NaN keep their class. For the mixed path's float increments and
// right-hand sides, which are never subnormal in magnitude that matters.
CLM_HD double widen_fast(float x) {
  const uint32_t b = fbits(x);
  const uint32_t e = (b >> 23) & 0xFF;
  const uint64_t sign = (uint64_t)(b & 0x80000000u) << 32;
  const uint64_t mant = (uint64_t)(b & 0x7FFFFFu) << 29;
  uint64_t r = sign | ((uint64_t)(e + 896) << 52) | mant;
  r = (e == 0) ? sign : r;
  r = (e == 0xFF) ? (sign | 0x7FF0000000000000ull | mant) : r;
  return dfrom(r);
}

// double -> float by truncating the significand (relative error below
// 2^-23), integer operations only: the mixed path's float Jacobian entries
// and right-hand sides. Magnitudes below the float normal range give a
// signed zero; above it, and infinities, an infinity; NaN stays NaN.
CLM_HD float narrow_trunc(double d) {
  const uint64_t b = dbits(d);
  const uint32_t h = (uint32_t)(b >> 32);
  const uint32_t sign = h & 0x80000000u;
  const int E = (int)((h >> 20) & 0x7FF);
  const int e = E - 896;  // float biased exponent
  const uint32_t mant = (uint32_t)(b >> 29) & 0x7FFFFFu;
  uint32_t r = sign | ((uint32_t)e << 23) | mant;
  r = (e <= 0) ? sign : r;
  const bool nan = E == 0x7FF && (b & 0x000FFFFFFFFFFFFFull) != 0;
  r = (e >= 255) ? (sign | 0x7F800000u | (nan ? 0x400000u : 0u)) : r;
  return ffrom(r);
}

// ---- tables -----------------------------------------------------------------------
// 2^(j/64), j = 0..63, as double-float pairs (hi[64] then lo[64]).
struct Tables {
  const float* t;  // 128 floats
};

// ---- exp and log ------------------------------------------------------------------
// Argument range of exp at full double-float precision: [kExpMin, kExpMax]
// (the result's lo word stays normal; 2^k stays normal).
constexpr float kExpMin = -65.0f;
constexpr float kExpMax = 80.0f;

// exp(x) for x.hi in [kExpMin, kExpMax] (the caller checks). x = k ln2/64 + r,
// |r| <= ln2/128, with ln2/64 split as C1 (11 bits: k C1 is exact for
// |k| < 2^13) + C2 (24 bits) + C3; e^r - 1 = r + r^2 (1/2 + r c(r)), c(r) =
// 1/6 + r/24 + r^2/120 in float (its error enters below 2^-48).
template <bool kLo>
CLM_HD F2 exp_impl(const Tables& T, F2 x) {
  const float kInvL = 92.33248138427734f;          // 64 / ln2
  const float C1 = 0.010833740234375f;             // ln2/64 to 11 significant bits
  const float C2 = -3.3155381515825866e-06f;       // ln2/64 - C1 to 24 bits
  const float C3 = 2.572804640231345e-14f;         // remainder
  int k;
  const float kf = round_f(x.hi * kInvL, k);
  const float t = fmaf(-kf, C1, x.hi);  // exact
  const F2 p = two_prod(kf, C2);
  F2 r = two_sum(t, -p.hi);  // exact
  if (kLo) r = add_f(r, x.lo);  // x.lo kept to the last bit
  r = fast_two_sum(r.hi, r.lo - (p.lo + kf * C3));
  const int j = k & 63;
  const int m = (k - j) / 64;
  const float c = fmaf(fmaf(r.hi, 1.0f / 120.0f, 1.0f / 24.0f), r.hi, 1.0f / 6.0f);
  const F2 s = two_sum(0.5f, r.hi * c);
  const F2 q = mul(mul(r, r), s);
  const F2 em1 = add_small(r, q);  // e^r - 1 (|q| <= |r| |r| / 2, |r| <= ln2/128)
  const F2 tj = F2{T.t[j], T.t[64 + j]};
  const F2 y = add_small(tj, mul(tj, em1));  // tj >= 1, |tj em1| <= 2 |em1|
  const float sc = ffrom((uint32_t)(m + 127) << 23);  // 2^m
  return F2{y.hi * sc, y.lo * sc};
}

CLM_HD F2 exp(const Tables& T, F2 x) { return exp_impl<true>(T, x); }

// exp of a single float (the reduction skips the low word)
CLM_HD F2 exp1(const Tables& T, float x) { return exp_impl<false>(T, make(x)); }

// log(x) for x > 0 (normal float hi): x = 2^k xm with xm in [1, 2) (exact
// scaling), y0 = log_approx(xm.hi) (absolute error below 2^-21), t =
// xm e^(-y0) - 1 (|t| < 1e-6, exp argument within +-0.7), log x = k ln2 +
// y0 + t - t^2/2 (+ O(t^3) < 1e-18); ln2 split as L1 (16 bits: k L1 exact
// for |k| < 2^8) + L2 + L3.
CLM_HD F2 log(const Tables& T, F2 x) {
  const float L1 = 0.693145751953125f;
  const float L2 = 1.428606765330187e-06f;
  const float L3 = 5.497923148104107e-14f;
  const int k = (int)((fbits(x.hi) >> 23) & 0xFF) - 127;
  const float sc = ffrom((uint32_t)(127 - k) << 23);  // 2^-k
  const F2 xm = F2{x.hi * sc, x.lo * sc};
  const float y0 = log_approx(xm.hi);
  const F2 e = exp1(T, -y0);
  const F2 t = add_f(mul(xm, e), -1.0f);
  const float kf = int_to_float(k);
  F2 y = add(two_sum(kf * L1, y0), t);  // k L1 exact
  y = add(y, two_prod(kf, L2));
  return add_f(y, fmaf(kf, L3, -0.5f * t.hi * t.hi));
}

// ---- table staging -------------------------------------------------------------------
// From the FP64 table of 2^(j/64): hi = float(v), lo = float(v - hi).
CLM_HD void fill_table(const double* exp2j, float* out) {
  for (int j = 0; j < 64; ++j) {
    const float hi = (float)exp2j[j];
    out[j] = hi;
    out[64 + j] = (float)(exp2j[j] - (double)hi);
  }
}

}  // namespace ff
}  // namespace clm
