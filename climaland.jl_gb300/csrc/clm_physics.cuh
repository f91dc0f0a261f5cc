// Pointwise soil physics (host and device).
//
// Same mathematics as the reference closures
//   src/standalone/Soil/soil_hydrology_parameterizations.jl (a2-a9)
//   src/standalone/Soil/soil_heat_parameterizations.jl      (a11-a15)
// rearranged for a GPU with a narrow FP64 pipe: every power a^b is
// exp(b log a) with the table-driven exp/log of clm_fastmath.cuh, and the
// logs and exponentials that psi, dpsi/dvartheta and K have in common are
// computed once per point. Where the reference rounds an intermediate (for
// example 1 - S^(1/m) before raising it to m) the same intermediate is
// rounded here, so cancellation behaves the same way in both.
#pragma once

#include <cstdint>

#include "../../include/climaland_cuda.h"
#include "clm_fastmath.cuh"

#ifndef CLM_HD
#define CLM_HD __host__ __device__ __forceinline__
#endif

namespace clm {

constexpr double kSqrtEps = 1.4901161193847656e-08;  // sqrt(eps(Float64))
constexpr double kEps = 2.220446049250313e-16;       // eps(Float64)
constexpr double kLn10 = 2.302585092994045684;

using fm::Tables;

// Physical constants, derived once per handle (LandParameters fields).
struct Earth {
  double rho_l, rho_i, T_0, T_freeze, LH_f0, grav;
  double rhocp_l, rhocp_i;      // cp_l rho_l, cp_i rho_i
  double rho_i_over_rho_l;      // for theta_tot and budgets
  double rho_l_over_rho_i;      // ice tendency factor
  double rho_i_LH_f0;           // latent energy per unit ice fraction
  double grav_over_LH_f0;       // Tf_depressed exponent
  double LH_f0_over_grav;       // psi_T prefactor
  double inv_T_freeze;          // 1 / T_freeze
};

inline Earth make_earth(const clm_earth_params& e) {
  Earth E;
  E.rho_l = e.rho_l;
  E.rho_i = e.rho_i;
  E.T_0 = e.T_0;
  E.T_freeze = e.T_freeze;
  E.LH_f0 = e.LH_f0;
  E.grav = e.grav;
  E.rhocp_l = e.cp_l * e.rho_l;
  E.rhocp_i = e.cp_i * e.rho_i;
  E.rho_i_over_rho_l = e.rho_i / e.rho_l;
  E.rho_l_over_rho_i = e.rho_l / e.rho_i;
  E.rho_i_LH_f0 = e.rho_i * e.LH_f0;
  E.grav_over_LH_f0 = e.grav / e.LH_f0;
  E.LH_f0_over_grav = e.LH_f0 / e.grav;
  E.inv_T_freeze = 1.0 / e.T_freeze;
  return E;
}

// Scalar EnergyHydrology parameters (energy_hydrology.jl:44-61).
struct EHScalars {
  double kersten_alpha, kersten_beta;
  double omega_ln10;  // Omega * ln(10): impedance 10^(-Omega f) = exp(-omega_ln10 f)
  double visc_gamma, visc_gamma_T_ref;
};

// van Genuchten closure of one column (retention_models.jl:354-368).
struct VG {
  double alpha, n, m;
  double inv_m, inv_n;     // 1/m, 1/n
  double inv_alpha;        // 1/alpha
  double coef_d;           // 1 / (alpha m n)
};

CLM_HD VG make_vg(double alpha, double n) {
  VG g;
  g.alpha = alpha;
  g.n = n;
  g.m = 1.0 - 1.0 / n;
  g.inv_m = 1.0 / g.m;
  g.inv_n = 1.0 / n;
  g.inv_alpha = 1.0 / alpha;
  g.coef_d = 1.0 / (alpha * g.m * n);
  return g;
}

// Brooks-Corey closure of one column (retention_models.jl:47-67).
struct BC {
  double psib, c;
  double neg_inv_c;  // -1/c
  double k_exp;      // 2/c + 3
  double coef_d;     // -psi_b / c
};

CLM_HD BC make_bc(double psib, double c) {
  BC g;
  g.psib = psib;
  g.c = c;
  g.neg_inv_c = -1.0 / c;
  g.k_exp = 2.0 / c + 3.0;
  g.coef_d = -psib / c;
  return g;
}

// The closure from parameter rows CLM_P_VG_ALPHA / CLM_P_VG_N
// (CLM_P_BC_PSI_B / CLM_P_BC_C): the reference dispatches on the type of
// hydrology_cm, the kernels on a template argument.
template <class CM>
CLM_HD CM make_cm(double row_a, double row_b);
template <>
CLM_HD VG make_cm<VG>(double alpha, double n) { return make_vg(alpha, n); }
template <>
CLM_HD BC make_cm<BC>(double psib, double c) { return make_bc(psib, c); }

// effective_saturation (soil_hydrology_parameterizations.jl:45-50), also
// returning the clipped vartheta and the clipped denominator.
struct Sat {
  double S, v_safe, nu_safe;
};

CLM_HD Sat saturation(double nu_eff, double vartheta, double theta_r) {
  Sat s;
  s.v_safe = fmax(vartheta, theta_r + kSqrtEps);
  s.nu_safe = fmax(nu_eff, theta_r + kSqrtEps);
  s.S = (s.v_safe - theta_r) / (s.nu_safe - theta_r);
  return s;
}

// 1 / (max(nu_eff, theta_r + sqrt(eps)) - theta_r): the reciprocal of the
// clipped denominator of effective_saturation, constant over a column
// (nu_eff = nu) or over a Newton solve (nu_eff = nu - theta_i, theta_i fixed).
// With it S = (vartheta_safe - theta_r) inv costs a product instead of a
// division (within an ulp of the quotient).
CLM_HD double sat_inv(double nu_eff, double theta_r) {
  return fm::rcp(fmax(nu_eff, theta_r + kSqrtEps) - theta_r);
}

CLM_HD double saturation_r(double inv, double vartheta, double theta_r) {
  return (fmax(vartheta, theta_r + kSqrtEps) - theta_r) * inv;
}

// pressure_head (:109-127) and dpsidvartheta (:135-152) at one point,
// sharing S^(-1/m) and log(S^(-1/m) - 1). want_d selects the derivative.
//   psi  = -(S^(-1/m) - 1)^(1/n) / alpha                 (S <= 1)
//        = (vartheta_safe - nu_safe) / S_s                (S > 1)
//   dpsi = (S^(-1/m) - 1)^(1/n - 1) S^(-1/m - 1) / (alpha m n (nu_safe - theta_r))
//        = 1 / S_s                                        (S >= 1)
template <bool want_d>
CLM_HD void psi_dpsi(const Tables& T, const VG& g, double nu_eff, double vartheta,
                     double theta_r, double S_s, double& psi, double& dpsi) {
  Sat s = saturation(nu_eff, vartheta, theta_r);
  if (s.S < 1.0) {
    const double u = fm::exp(T, -g.inv_m * fm::log(T, s.S));  // S^(-1/m)
    const double w = u - 1.0;
    const double w1n = fm::exp(T, g.inv_n * fm::log(T, w));  // w^(1/n)
    psi = -w1n * g.inv_alpha;
    if (want_d) dpsi = g.coef_d * w1n * u / (w * s.S * (s.nu_safe - theta_r));
  } else {
    // S == 1 gives psi = -0 in the reference (matric_potential(1)).
    psi = (s.S <= 1.0) ? -0.0 : (s.v_safe - s.nu_safe) / S_s;
    if (want_d) dpsi = 1.0 / S_s;
  }
}

// psi_dpsi with the reciprocal inv = sat_inv(nu_eff, theta_r) and 1/S_s given:
// no division on the unsaturated branch but dpsi's, whose factor
// S (nu_safe - theta_r) is vartheta_safe - theta_r itself.
template <bool want_d>
CLM_HD void psi_dpsi_r(const Tables& T, const VG& g, double nu_eff, double inv, double vartheta,
                       double theta_r, double inv_S_s, double& psi, double& dpsi) {
  const double vs = fmax(vartheta, theta_r + kSqrtEps);
  const double a = vs - theta_r;
  const double S = a * inv;
  if (S < 1.0) {
    const double u = fm::exp(T, -g.inv_m * fm::log(T, S));  // S^(-1/m)
    const double w = u - 1.0;
    const double w1n = fm::exp(T, g.inv_n * fm::log(T, w));  // w^(1/n)
    psi = -w1n * g.inv_alpha;
    if (want_d) dpsi = g.coef_d * w1n * u * fm::rcp(w * a);
  } else {
    psi = (S <= 1.0) ? -0.0 : (vs - fmax(nu_eff, theta_r + kSqrtEps)) * inv_S_s;
    if (want_d) dpsi = inv_S_s;
  }
}

// Brooks-Corey pressure_head (:268-287) and dpsidvartheta (:219-230),
// sharing S^(-1/c):
//   psi  = psi_b S^(-1/c)                                  (S <= 1)
//        = (vartheta_safe - nu_safe) / S_s + psi_b          (S > 1)
//   dpsi = -psi_b / (c (nu_safe - theta_r)) S^(-1/c) / S   (S < 1)
//        = 1 / S_s                                         (S >= 1)
template <bool want_d>
CLM_HD void psi_dpsi(const Tables& T, const BC& g, double nu_eff, double vartheta,
                     double theta_r, double S_s, double& psi, double& dpsi) {
  Sat s = saturation(nu_eff, vartheta, theta_r);
  if (s.S < 1.0) {
    const double u = fm::exp(T, g.neg_inv_c * fm::log(T, s.S));  // S^(-1/c)
    psi = g.psib * u;
    if (want_d) dpsi = g.coef_d * u / (s.S * (s.nu_safe - theta_r));
  } else {
    // S == 1: matric_potential(1) = psi_b
    psi = (s.S <= 1.0) ? g.psib : (s.v_safe - s.nu_safe) / S_s + g.psib;
    if (want_d) dpsi = 1.0 / S_s;
  }
}

template <bool want_d>
CLM_HD void psi_dpsi_r(const Tables& T, const BC& g, double nu_eff, double inv, double vartheta,
                       double theta_r, double inv_S_s, double& psi, double& dpsi) {
  const double vs = fmax(vartheta, theta_r + kSqrtEps);
  const double a = vs - theta_r;
  const double S = a * inv;
  if (S < 1.0) {
    const double u = fm::exp(T, g.neg_inv_c * fm::log(T, S));  // S^(-1/c)
    psi = g.psib * u;
    if (want_d) dpsi = g.coef_d * u * fm::rcp(a);
  } else {
    psi = (S <= 1.0) ? g.psib : (vs - fmax(nu_eff, theta_r + kSqrtEps)) * inv_S_s + g.psib;
    if (want_d) dpsi = inv_S_s;
  }
}

// hydraulic_conductivity (:161-173) of an effective saturation S:
//   K = K_sat sqrt(S) (1 - (1 - S^(1/m))^m)^2 (S < 1), K_sat otherwise.
CLM_HD double conductivity(const Tables& T, const VG& g, double K_sat, double S) {
  if (!(S < 1.0)) return K_sat;
  const double s1m = fm::exp(T, g.inv_m * fm::log(T, S));  // S^(1/m)
  const double t = fm::exp(T, g.m * fm::log(T, 1.0 - s1m));  // (1 - S^(1/m))^m
  const double f = 1.0 - t;
  return K_sat * (sqrt(S) * f * f);
}

// Brooks-Corey hydraulic_conductivity (:239-251): K_sat S^(2/c + 3) (S < 1).
CLM_HD double conductivity(const Tables& T, const BC& g, double K_sat, double S) {
  if (!(S < 1.0)) return K_sat;
  return K_sat * fm::exp(T, g.k_exp * fm::log(T, S));
}

// K_sat exp(lnf) k_r(S): the hydraulic conductivity times the impedance and
// viscosity factors exp(lnf) (EnergyHydrology update_aux!,
// energy_hydrology.jl:776-790), with the S-power of k_r inside the same
// exponential (sqrt(S) for van Genuchten, S^(2/c + 3) for Brooks-Corey).
CLM_HD double conductivity_scaled(const Tables& T, const VG& g, double K_sat, double S,
                                  double lnf) {
  if (!(S < 1.0)) return K_sat * fm::exp(T, lnf);
  const double lS = fm::log(T, S);
  const double s1m = fm::exp(T, g.inv_m * lS);                 // S^(1/m)
  const double tm = fm::exp(T, g.m * fm::log(T, 1.0 - s1m));   // (1 - S^(1/m))^m
  const double f = 1.0 - tm;
  return K_sat * (f * f) * fm::exp(T, lnf + 0.5 * lS);
}

CLM_HD double conductivity_scaled(const Tables& T, const BC& g, double K_sat, double S,
                                  double lnf) {
  if (!(S < 1.0)) return K_sat * fm::exp(T, lnf);
  return K_sat * fm::exp(T, lnf + g.k_exp * fm::log(T, S));
}

// Richards point: K, psi (and dpsi) sharing log(S) (nu_eff = nu), with the
// column's inv = sat_inv(nu, theta_r) and 1/S_s (as psi_dpsi_r).
template <bool want_d>
CLM_HD void richards_point(const Tables& T, const VG& g, double nu, double inv, double vartheta,
                           double theta_r, double inv_S_s, double K_sat, double& K, double& psi,
                           double& dpsi) {
  const double vs = fmax(vartheta, theta_r + kSqrtEps);
  const double a = vs - theta_r;
  const double S = a * inv;
  if (S < 1.0) {
    const double lS = fm::log(T, S);
    const double u = fm::exp(T, -g.inv_m * lS);  // S^(-1/m)
    const double w = u - 1.0;
    const double w1n = fm::exp(T, g.inv_n * fm::log(T, w));
    psi = -w1n * g.inv_alpha;
    if (want_d) dpsi = g.coef_d * w1n * u * fm::rcp(w * a);
    const double s1m = fm::exp(T, g.inv_m * lS);  // S^(1/m)
    const double t = fm::exp(T, g.m * fm::log(T, 1.0 - s1m));
    const double f = 1.0 - t;
    K = K_sat * (sqrt(S) * f * f);
  } else {
    psi = (S <= 1.0) ? -0.0 : (vs - fmax(nu, theta_r + kSqrtEps)) * inv_S_s;
    if (want_d) dpsi = inv_S_s;
    K = K_sat;
  }
}

// Brooks-Corey Richards point: K, psi (and dpsi) sharing log(S).
template <bool want_d>
CLM_HD void richards_point(const Tables& T, const BC& g, double nu, double inv, double vartheta,
                           double theta_r, double inv_S_s, double K_sat, double& K, double& psi,
                           double& dpsi) {
  const double vs = fmax(vartheta, theta_r + kSqrtEps);
  const double a = vs - theta_r;
  const double S = a * inv;
  if (S < 1.0) {
    const double lS = fm::log(T, S);
    const double u = fm::exp(T, g.neg_inv_c * lS);  // S^(-1/c)
    psi = g.psib * u;
    if (want_d) dpsi = g.coef_d * u * fm::rcp(a);
    K = K_sat * fm::exp(T, g.k_exp * lS);
  } else {
    psi = (S <= 1.0) ? g.psib : (vs - fmax(nu, theta_r + kSqrtEps)) * inv_S_s + g.psib;
    if (want_d) dpsi = inv_S_s;
    K = K_sat;
  }
}

// matric_potential of effective_saturation(nu, theta) (soil_Tf_depressed,
// phase_change_source). Returns S through *S_out.
CLM_HD double matric_of(const Tables& T, const VG& g, double nu, double theta,
                        double theta_r, double* S_out = nullptr) {
  Sat s = saturation(nu, theta, theta_r);
  if (S_out) *S_out = s.S;
  const double u = fm::exp(T, -g.inv_m * fm::log(T, s.S));
  const double w = u - 1.0;
  if (!(w > 0.0)) return -0.0;  // S >= 1 (theta <= nu keeps S <= 1)
  return -fm::exp(T, g.inv_n * fm::log(T, w)) * g.inv_alpha;
}

// Brooks-Corey: psi_b S^(-1/c) (matric_potential, :182-185).
CLM_HD double matric_of(const Tables& T, const BC& g, double nu, double theta,
                        double theta_r, double* S_out = nullptr) {
  Sat s = saturation(nu, theta, theta_r);
  if (S_out) *S_out = s.S;
  return g.psib * fm::exp(T, g.neg_inv_c * fm::log(T, s.S));
}

// matric_potential of a given effective saturation S <= 1.
CLM_HD double matric_S(const Tables& T, const VG& g, double S) {
  const double u = fm::exp(T, -g.inv_m * fm::log(T, S));
  const double w = u - 1.0;
  if (!(w > 0.0)) return -0.0;
  return -fm::exp(T, g.inv_n * fm::log(T, w)) * g.inv_alpha;
}

CLM_HD double matric_S(const Tables& T, const BC& g, double S) {
  return g.psib * fm::exp(T, g.neg_inv_c * fm::log(T, S));
}

// inverse_matric_potential (:72-77, :195-200) for psi <= 0:
//   van Genuchten (1 + (alpha |psi|)^n)^(-m), Brooks-Corey (psi / psi_b)^(-c).
CLM_HD double inverse_sat(const Tables& T, const VG& g, double psi) {
  const double x = fm::exp(T, g.n * fm::log(T, g.alpha * fabs(psi)));  // (alpha|psi|)^n
  return fm::exp(T, -g.m * fm::log(T, 1.0 + x));                     // (1 + x)^(-m)
}

CLM_HD double inverse_sat(const Tables& T, const BC& g, double psi) {
  return fm::exp(T, -g.c * fm::log(T, psi / g.psib));
}

// volumetric_heat_capacity (soil_heat_parameterizations.jl:157-171)
CLM_HD double heat_capacity(const Earth& E, double theta_l, double theta_i, double rhoc_ds) {
  return rhoc_ds + theta_l * E.rhocp_l + theta_i * E.rhocp_i;
}

// temperature_from_ρe_int (:180-192)
CLM_HD double temperature(const Earth& E, double rho_e, double theta_i, double rhoc) {
  return E.T_0 + (rho_e + theta_i * E.rho_i_LH_f0) / rhoc;
}

// volumetric_internal_energy_liq (:221-231)
CLM_HD double rho_e_liq(const Earth& E, double T) { return E.rhocp_l * (T - E.T_0); }

// Thermal conductivity kappa (energy_hydrology.jl:756-768): Balland-Arp
// Kersten number (:301-320) and kappa_sat (:243-256), with
// log(kappa_sat_unfrozen) and log(kappa_sat_frozen) precomputed per column.
CLM_HD double conductivity_heat(const Tables& T, const EHScalars& sc, double theta_l,
                                double theta_i, double nu, double kappa_dry, double k_unfrozen,
                                double k_frozen, double lku, double lkf, double nu_om,
                                double nu_quartz, double nu_gravel) {
  const double S_r = (theta_l + theta_i) / nu;  // relative_saturation
  double K_e;
  if (theta_i < kEps) {
    const double a = (1.0 + nu_om - sc.kersten_alpha * nu_quartz - nu_gravel) * 0.5;
    const double t1 = 1.0 + fm::exp(T, -sc.kersten_beta * S_r);
    const double t1m3 = 1.0 / (t1 * t1 * t1);
    const double h = (1.0 - S_r) * 0.5;
    const double base = t1m3 - h * h * h;
    K_e = fm::exp(T, a * fm::log(T, S_r) + (1.0 - nu_om) * fm::log(T, base));
  } else {
    K_e = fm::exp(T, (1.0 + nu_om) * fm::log(T, S_r));
  }
  const double theta_w = theta_l + theta_i;
  double ksat;
  if (theta_w < kEps)
    ksat = 0.5 * (k_unfrozen + k_frozen);
  else if (theta_i == 0.0)
    ksat = k_unfrozen;  // k_u^1 k_f^0
  else
    ksat = fm::exp(T, (theta_l * lku + theta_i * lkf) / theta_w);
  return K_e * ksat + (1.0 - K_e) * kappa_dry;
}

// Per-column constants of phase_change_r and phase_change_reduced.
struct PCCol {
  double nr;        // nu - theta_r
  double inv_den;   // 1 / (max(nu, theta_r + sqrt(eps)) - theta_r): effective_saturation(nu, .)
  double inv_3dz2;  // 1 / (3 dz^2): thermal_time
};

CLM_HD PCCol make_pc_col(double nu, double theta_r, double dz) {
  return PCCol{nu - theta_r, 1.0 / (fmax(nu, theta_r + kSqrtEps) - theta_r), 1.0 / (3.0 * (dz * dz))};
}

// Phase-change source (soil_heat_parameterizations.jl:89-122) including
// thermal_time (:60-62): (theta_l - theta_star) / tau, tau = 3 rho c dz^2 /
// kappa.
//
// phase_change (the FP64 path) evaluates the reference's own sequence:
// psi_w0 = matric_potential(S(theta_tot)), Tf = max(T_freeze exp(g psi_w0 /
// L_f), 1), psi_T = L_f/g log(T/Tf) heaviside(Tf - T), theta_star =
// inverse_matric_potential(psi_w0 + psi_T). For T >= T_freeze the heaviside
// factor is zero without evaluating Tf (Tf <= T_freeze), and theta_star is
// then inverse_matric_potential(matric_potential(S)) = S (nu - theta_r) +
// theta_r.
//
// phase_change_reduced (the mixed path) uses that with this Tf,
//   psi_w0 + L_f/g log(T/Tf) = L_f/g log(T/T_freeze) =: psi_T,
// independent of psi_w0, and Tf > T <=> psi_w0 > psi_T <=> S(theta_tot) > S_T
// with S_T = inverse_matric_potential(psi_T) (the matric potential increases
// with S, for either closure). So theta_star = min(S(theta_tot), S_T) (nu -
// theta_r) + theta_r: one log and inverse_matric_potential, no
// matric_potential and no Tf. The Tf >= 1 K clamp acts only where psi_w0 < -L_f/g
// log(T_freeze), where S(theta_tot) < S_T for every T > 1 K, so the min keeps
// S(theta_tot) as the clamped reference does; both branches agree at
// S(theta_tot) = S_T. It avoids the reference's cancellation of psi_w0
// against itself, which leaves up to ~1e-11 of theta_l / tau: columns whose
// trajectory switches a discontinuous closure (the Kersten number at
// theta_i = eps) follow that rounding, so the plain path keeps the
// reference's sequence.
//
// The column step passes the reciprocals it shares (PCCol below, and
// inv_rhoc = 1 / rho c, also used for T): products replace the divisions
// of S, tau and (theta_l - theta_star) / tau (each within an ulp or two).
template <class CM>
CLM_HD double phase_change(const Tables& T, const Earth& E, const CM& g, double nu,
                           double theta_r, double theta_l, double theta_i, double Tk,
                           double rhoc, double kappa, double dz, uint32_t& flags) {
  const double theta_tot = fmin(E.rho_i_over_rho_l * theta_i + theta_l, nu);
  double theta_star;
  double S;
  if (Tk >= E.T_freeze) {
    S = saturation(nu, theta_tot, theta_r).S;
    theta_star = S * (nu - theta_r) + theta_r;
  } else {
    const double psi_w0 = matric_of(T, g, nu, theta_tot, theta_r, &S);
    const double Tf = fmax(E.T_freeze * fm::exp(T, E.grav_over_LH_f0 * psi_w0), 1.0);
    if (Tf - Tk > kEps) {  // heaviside(Tf - T)
      const double psi = psi_w0 + E.LH_f0_over_grav * fm::log(T, Tk / Tf);
      if (psi > 0.0) flags |= CLM_COL_PSI_POSITIVE;
      theta_star = inverse_sat(T, g, psi) * (nu - theta_r) + theta_r;
    } else {
      if (psi_w0 > 0.0) flags |= CLM_COL_PSI_POSITIVE;
      theta_star = S * (nu - theta_r) + theta_r;
    }
  }
  const double tau = 3.0 * rhoc * (dz * dz) / kappa;
  return (theta_l - theta_star) / tau;
}


template <class CM>
CLM_HD double phase_change_r(const Tables& T, const Earth& E, const CM& g, double nu,
                             double theta_r, const PCCol& pcc, double theta_l, double theta_i,
                             double Tk, double inv_rhoc, double kappa, uint32_t& flags) {
  const double theta_tot = fmin(E.rho_i_over_rho_l * theta_i + theta_l, nu);
  const double S = (fmax(theta_tot, theta_r + kSqrtEps) - theta_r) * pcc.inv_den;
  double theta_star = S * pcc.nr + theta_r;
  if (Tk < E.T_freeze) {
    const double psi_w0 = matric_S(T, g, S);
    const double Tf = fmax(E.T_freeze * fm::exp(T, E.grav_over_LH_f0 * psi_w0), 1.0);
    if (Tf - Tk > kEps) {  // heaviside(Tf - T)
      const double psi = psi_w0 + E.LH_f0_over_grav * fm::log(T, Tk / Tf);
      if (psi > 0.0) flags |= CLM_COL_PSI_POSITIVE;
      theta_star = inverse_sat(T, g, psi) * pcc.nr + theta_r;
    } else if (psi_w0 > 0.0) {
      flags |= CLM_COL_PSI_POSITIVE;
    }
  }
  return (theta_l - theta_star) * kappa * inv_rhoc * pcc.inv_3dz2;
}

// The reduced form, with the divisions turned into products by reciprocals:
// the per-column ones above and inv_rhoc = 1 / rho c, which the caller also
// uses for the temperature.
template <class CM>
CLM_HD double phase_change_reduced(const Tables& T, const Earth& E, const CM& g, double nu,
                                   double theta_r, const PCCol& pcc, double theta_l,
                                   double theta_i, double Tk, double inv_rhoc, double kappa) {
  const double theta_tot = fmin(E.rho_i_over_rho_l * theta_i + theta_l, nu);
  double S = (fmax(theta_tot, theta_r + kSqrtEps) - theta_r) * pcc.inv_den;
  if (Tk < E.T_freeze) {
    const double psi_T = E.LH_f0_over_grav * fm::log(T, Tk * E.inv_T_freeze);
    S = fmin(S, inverse_sat(T, g, psi_T));
  }
  const double theta_star = S * pcc.nr + theta_r;
  return (theta_l - theta_star) * kappa * inv_rhoc * pcc.inv_3dz2;
}

// Root extraction of one column (src/integrated/soil_canopy_root_interactions.jl:8-39):
// the per-column canopy factors and the per-layer rate
//   re = hm(LAI, RAI) water_flux(z, h/2, psi_soil, psi_c, K_soil, K_c) root_distribution(z, d)
// with hm(x, y) = x y / max(x + y, eps) (plant_hydraulics.jl:170), water_flux =
// -hm(K1, K2) ((psi2 - psi1) / (z2 - z1) + 1) (:197-201), the Weibull plant
// conductivity K_c (:256-267) and root_distribution = exp(z / d) / d
// (biomass.jl:362-364).
CLM_HD double harmonic_mean(double x, double y) { return x * y / fmax(x + y, kEps); }

struct RootCol {
  double psi_c, hm_LR, z2, inv_d, K_c;
};

CLM_HD RootCol load_root_col(const Tables& T, const double* R, int stride, int s) {
  RootCol r;
  r.psi_c = R[CLM_RX_PSI_CANOPY * stride + s];
  r.hm_LR = harmonic_mean(R[CLM_RX_LAI * stride + s], R[CLM_RX_RAI * stride + s]);
  r.z2 = R[CLM_RX_HEIGHT * stride + s] / 2.0;
  r.inv_d = 1.0 / R[CLM_RX_ROOT_DEPTH * stride + s];
  const double Ksat = R[CLM_RX_K_SAT * stride + s];
  r.K_c = (r.psi_c <= 0.0)
              ? fm::exp(T, -fm::exp(T, R[CLM_RX_WEIBULL_C * stride + s] *
                                           fm::log(T, r.psi_c / R[CLM_RX_PSI63 * stride + s]))) *
                    Ksat
              : Ksat;
  return r;
}

CLM_HD double root_rate(const Tables& T, const RootCol& r, double z, double psi_soil,
                        double K_soil) {
  const double flux = -harmonic_mean(K_soil, r.K_c) * ((r.psi_c - psi_soil) / (r.z2 - z) + 1.0);
  return r.hm_LR * flux * (r.inv_d * fm::exp(T, z * r.inv_d));
}

// counter hash of the rain-pulse forcing (splitmix64 finaliser, Vigna):
// identical integer arithmetic on host and device.
CLM_HD uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

CLM_HD double hash01(uint64_t seed, uint64_t column, int64_t period) {
  uint64_t h = mix64(seed + 0x9E3779B97F4A7C15ULL * (column + 1ULL));
  h = mix64(h ^ ((uint64_t)period * 0xD1B54A32D192ED03ULL));
  return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

// Forcing descriptor value at time t for column `orig` (header comment of
// enum clm_forcing_field). F points to row 0 of a [CLM_F_NFIELDS][stride] block.
// col: the column's row in F; hash_col: its global index (rain-pulse hash).
CLM_HD double forcing_value(const double* F, int stride, int col, int64_t hash_col, double t,
                            uint64_t seed) {
  if (F == nullptr) return 0.0;
  double v = F[CLM_F_BASE * stride + col];
  const double amp = F[CLM_F_AMP * stride + col];
  if (amp != 0.0) v += amp * sin(F[CLM_F_OMEGA * stride + col] * t + F[CLM_F_PHASE * stride + col]);
  const double pp = F[CLM_F_PULSE_PERIOD * stride + col];
  if (pp > 0.0) {
    const int64_t k = (int64_t)floor(t / pp);
    if (hash01(seed, (uint64_t)hash_col, k) < F[CLM_F_PULSE_DUTY * stride + col])
      v += F[CLM_F_PULSE_AMP * stride + col];
  }
  return v;
}

}  // namespace clm
