// Accuracy of the double-float routines (climaland.jl_gb300/csrc/clm_ff.cuh)
// against FP64, on seeded random arguments over the ranges the soil closures
// use. Prints one line per routine: name, worst relative error, count.
#define CLM_HD inline
#include <cmath>
#include <cstdio>
#include <random>

#include "clm_ff.cuh"

using namespace clm::ff;

static double rel(double got, double want) {
  return std::fabs(got - want) / std::fmax(std::fabs(want), 1e-300);
}

int main() {
  double tab[64];
  for (int j = 0; j < 64; ++j) tab[j] = std::exp2(j / 64.0);
  float t2[128];
  fill_table(tab, t2);
  const Tables T{t2};
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  const int N = 400000;
  double e_rt = 0, e_add = 0, e_mul = 0, e_div = 0, e_exp = 0, e_log = 0, e_logabs = 0;
  for (int i = 0; i < N; ++i) {
    // operands and results inside the normal float range
    const double a = std::exp((U(rng) - 0.5) * 60.0) * (U(rng) < 0.5 ? -1 : 1);
    const double b = std::exp((U(rng) - 0.5) * 60.0);
    const F2 fa = from_double(a), fb = from_double(b);
    const double da = to_double(fa), db = to_double(fb);
    e_rt = std::fmax(e_rt, rel(da, a));
    e_add = std::fmax(e_add, rel(to_double(add(fa, fb)), da + db) * std::fabs(da + db) /
                                 std::fmax(std::fabs(da), std::fabs(db)));
    e_mul = std::fmax(e_mul, rel(to_double(mul(fa, fb)), da * db));
    e_div = std::fmax(e_div, rel(to_double(div(fa, fb)), da / db));
    const double x = -65.0 + U(rng) * 145.0;  // [kExpMin, kExpMax]
    const F2 fx = from_double(x);
    e_exp = std::fmax(e_exp, rel(to_double(exp(T, fx)), std::exp(to_double(fx))));
    const double y = std::exp((U(rng) - 0.5) * 2.0 * 80.0);
    const F2 fy = from_double(y);
    const double ly = std::log(to_double(fy));
    const double gl = to_double(log(T, fy));
    e_log = std::fmax(e_log, rel(gl, ly));
    e_logabs = std::fmax(e_logabs, std::fabs(gl - ly) / std::fmax(1.0, std::fabs(ly)));
  }
  std::printf("roundtrip %.3e %d\n", e_rt, N);
  std::printf("add %.3e %d\n", e_add, N);
  std::printf("mul %.3e %d\n", e_mul, N);
  std::printf("div %.3e %d\n", e_div, N);
  std::printf("exp %.3e %d\n", e_exp, N);
  std::printf("log %.3e %d\n", e_log, N);
  std::printf("log_abs %.3e %d\n", e_logabs, N);
  return 0;
}
