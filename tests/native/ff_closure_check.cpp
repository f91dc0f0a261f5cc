// The mixed path's double-float pressure head and its derivative
// (clm_physics_ff.cuh: psi_dpsi_ff, van Genuchten and Brooks-Corey) against
// the FP64 closure (clm_physics.cuh: psi_dpsi) on seeded random columns and
// states, unsaturated and saturated (S > 1: psi = (v - nu_eff) / S_s).
// Prints, per closure and branch: worst error of psi relative to
// max(|psi|, 1 m), worst relative error of dpsi (float), the points
// evaluated in double-float, and the points handed back to FP64.
#define CLM_HD inline
#define __device__
#define __forceinline__ inline
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <random>
using std::isfinite;
inline double rsqrt(double x) { return 1.0 / std::sqrt(x); }

#include "clm_column.cuh"

using namespace clm;

template <class CM, class ColF>
void check(const char* name, const Tables& Tb, std::mt19937_64& rng, CM (*make)(std::mt19937_64&),
           ColF (*make_f)(double, double, const CM&)) {
  std::uniform_real_distribution<double> U(0.0, 1.0);
  const ff::Tables FT{Tb.ff};
  double e_psi[2] = {0, 0}, e_d[2] = {0, 0};
  int n_ff[2] = {0, 0}, n_back[2] = {0, 0};
  for (int i = 0; i < 200000; ++i) {
    const CM g = make(rng);
    const double nu = 0.35 + 0.2 * U(rng), theta_r = 0.02 + 0.08 * U(rng);
    const double S_s = std::pow(10.0, -4.0 + 2.0 * U(rng));
    const double ti = U(rng) < 0.3 ? 0.1 * U(rng) : 0.0;
    const double nu_eff = nu - ti;
    // vartheta from just above theta_r to 20 % above nu_eff; one point in
    // five very dry (theta_r + 1e-12 .. 1e-4: S^(-1/m) beyond e^80 for small m)
    const double v = U(rng) < 0.2 ? theta_r + std::pow(10.0, -12.0 + 8.0 * U(rng))
                                  : theta_r + 1e-6 + (1.2 * nu_eff - theta_r) * U(rng);
    const int sat = v > nu_eff ? 1 : 0;
    // the FP64 closure at the inputs as the double-float pairs hold them
    // (about 48 significant bits): the comparison measures the closure's
    // arithmetic, not the rounding of its inputs
    const ColF cf = make_f(nu, theta_r, g);
    const ff::F2 nu_f = ff::sub(cf.nu, ff::from_double(ti)), v_f = ff::from_double(v);
    double psi, d;
    psi_dpsi<true>(Tb, g, ff::to_double(nu_f), ff::to_double(v_f), ff::to_double(cf.theta_r), S_s, psi, d);
    double psi_f;
    float d_f;
    if (!psi_dpsi_ff(FT, cf, nu_f, v_f, 1.0 / S_s, psi_f, d_f)) {
      ++n_back[sat];
      continue;
    }
    ++n_ff[sat];
    // relative to max(|psi|, 1 m): near saturation psi is small and its
    // relative error is the cancellation in S^(-1/m) - 1, in FP64 as well
    e_psi[sat] = std::fmax(e_psi[sat], std::fabs(psi_f - psi) / std::fmax(std::fabs(psi), 1.0));
    // dpsi in float: compared where the FP64 value is inside the float range
    // (beyond it, the FP64 closure's value rounds to infinity as well)
    if (std::fabs(d) < 1e38) e_d[sat] = std::fmax(e_d[sat], std::fabs((double)d_f - d) / std::fabs(d));
  }
  for (int b = 0; b < 2; ++b)
    std::printf("%s_%s %.3e %.3e %d %d\n", name, b ? "saturated" : "unsaturated", e_psi[b], e_d[b], n_ff[b],
                n_back[b]);
}

static VG rand_vg(std::mt19937_64& r) {
  std::uniform_real_distribution<double> U(0.0, 1.0);
  return make_vg(0.5 + 4.5 * U(r), 1.2 + 1.3 * U(r));
}
static BC rand_bc(std::mt19937_64& r) {
  std::uniform_real_distribution<double> U(0.0, 1.0);
  return make_bc(-(0.05 + 0.5 * U(r)), 0.1 + 0.4 * U(r));
}

int main() {
  const Tables Tb = fm::host_tables();
  std::mt19937_64 rng(2024);
  check<VG, ColFF>("vg", Tb, rng, rand_vg, make_col_ff);
  check<BC, ColFFBC>("bc", Tb, rng, rand_bc, make_col_ff);
  return 0;
}
