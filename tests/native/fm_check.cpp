// Accuracy of the FP64 fast math of the column kernels
// (climaland.jl_gb300/csrc/clm_fastmath.cuh) against the host's libm and
// IEEE division, on seeded random arguments over the ranges the soil
// closures use. Prints one line per routine: name, worst error in ulps of
// the reference result.
#define CLM_HD inline
#include <cmath>
#include <cstdio>
#include <random>

#include "clm_fastmath.cuh"

using namespace clm;

static double ulps(double got, double want) {
  const double u = std::nextafter(std::fabs(want), INFINITY) - std::fabs(want);
  return std::fabs(got - want) / u;
}

int main() {
  const fm::Tables T = fm::host_tables();
  std::mt19937_64 rng(2024);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  const int N = 400000;
  double e_exp = 0, e_log = 0, e_rcp = 0, e_rcp_wide = 0;
  for (int i = 0; i < N; ++i) {
    const double x = (U(rng) - 0.5) * 1400.0;  // |x| <= 700
    e_exp = std::fmax(e_exp, ulps(fm::exp(T, x), std::exp(x)));
    const double y = std::exp((U(rng) - 0.5) * 1380.0);  // normal positives
    const double ly = std::log(y);
    if (std::fabs(ly) > 1e-3) e_log = std::fmax(e_log, ulps(fm::log(T, y), ly));
    const double z = std::exp((U(rng) - 0.5) * 160.0) * (U(rng) < 0.5 ? -1.0 : 1.0);  // |z| in [e^-80, e^80]
    e_rcp = std::fmax(e_rcp, ulps(fm::rcp(z), 1.0 / z));
    const double zw = std::exp((U(rng) - 0.5) * 1300.0);  // including the division fallback
    e_rcp_wide = std::fmax(e_rcp_wide, ulps(fm::rcp(zw), 1.0 / zw));
  }
  std::printf("exp %.6g\nlog %.6g\nrcp %.6g\nrcp_wide %.6g\n", e_exp, e_log, e_rcp, e_rcp_wide);
  // special values go through the division
  const bool special = std::isinf(fm::rcp(0.0)) && fm::rcp(INFINITY) == 0.0 && std::isnan(fm::rcp(NAN)) &&
                       fm::rcp(-2.0) == -0.5 && fm::rcp(1.0) == 1.0;
  std::printf("rcp_special %d\n", special ? 0 : 1);
  return 0;
}
