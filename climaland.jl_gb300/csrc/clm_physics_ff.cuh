// Soil closures of the mixed path in double-float arithmetic (clm_ff.cuh).
//
// Same formulas as clm_physics.cuh (references there), evaluated on pairs of
// floats on the FP32 pipe; results are returned as FP64 for the FP64 residual
// assembly (psi, T, K, kappa) or as float for the FP32 Jacobian (dpsi). Each
// closure returns false when an intermediate would leave the double-float
// range (exponents beyond [kExpMin, kExpMax], arguments of log below 1e-30,
// saturated cells): the caller then evaluates that point with the FP64
// closure.
#pragma once

#include "clm_ff.cuh"
#include "clm_physics.cuh"

namespace clm {

using ff::F2;

// a < b for pairs
CLM_HD bool ff_lt(F2 a, F2 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
CLM_HD F2 ff_max(F2 a, F2 b) { return ff_lt(a, b) ? b : a; }
CLM_HD F2 ff_min(F2 a, F2 b) { return ff_lt(a, b) ? a : b; }

// Physical constants as pairs (LandParameters fields used in the closures).
struct EarthFF {
  F2 T_0, rhocp_l, rhocp_i, rho_i_LH_f0;
};

CLM_HD EarthFF make_earth_ff(const Earth& E) {
  return EarthFF{ff::from_double(E.T_0), ff::from_double(E.rhocp_l), ff::from_double(E.rhocp_i),
                 ff::from_double(E.rho_i_LH_f0)};
}

// Per-column constants of the mixed-path closures.
struct ColFF {
  F2 nu, theta_r, neg_inv_m, inv_m, m, inv_n, inv_alpha;
  float coef_d;  // 1 / (alpha m n) for the FP32 Jacobian
};

CLM_HD ColFF make_col_ff(double nu, double theta_r, const VG& g) {
  ColFF c;
  c.nu = ff::from_double(nu);
  c.theta_r = ff::from_double(theta_r);
  c.inv_m = ff::from_double(g.inv_m);
  c.neg_inv_m = ff::neg(c.inv_m);
  c.m = ff::from_double(g.m);
  c.inv_n = ff::from_double(g.inv_n);
  c.inv_alpha = ff::from_double(g.inv_alpha);
  c.coef_d = (float)g.coef_d;
  return c;
}

// pressure_head and dpsidvartheta (soil_hydrology_parameterizations.jl
// :109-152) at vartheta = v with nu_eff = nu - theta_i: for S < 1
//   psi = -(S^(-1/m) - 1)^(1/n) / alpha, dpsi = w^(1/n) u / (alpha m n w S (nu_safe - theta_r))
// with u = S^(-1/m), w = u - 1 (dpsi from the logs of its factors, in float);
// for S > 1 (saturated) psi = (v_safe - nu_safe) / S_s, dpsi = 1 / S_s.
// S = 1 exactly, and S within a float rounding below 1, take the FP64 closure.
CLM_HD bool psi_dpsi_ff(const ff::Tables& T, const ColFF& c, F2 nu_eff, F2 v, double inv_S_s,
                        double& psi, float& dpsi) {
  using namespace ff;
  const F2 guard = add_f(c.theta_r, 1.4901161193847656e-08f);  // theta_r + sqrt(eps)
  const F2 vs = ff_max(v, guard);
  const F2 ns = ff_max(nu_eff, guard);
  const F2 den = sub(ns, c.theta_r);
  const F2 S = div(sub(vs, c.theta_r), den);
  if (!(S.hi < 1.0f)) {
    const F2 d = sub(vs, ns);  // its sign is that of S - 1
    if (!(d.hi > 0.0f)) return false;
    psi = to_double(mul(d, from_double(inv_S_s)));
    dpsi = narrow_trunc(inv_S_s);
    return true;
  }
  if (!(S.hi > 1e-30f)) return false;
  const F2 L = log(T, S);
  const F2 a = mul(L, c.neg_inv_m);  // log u
  F2 lw;                             // log w
  if (a.hi <= kExpMax) {
    const F2 u = exp(T, a);
    const F2 w = add_f(u, -1.0f);
    if (!(w.hi > 1e-30f)) return false;
    lw = log(T, w);
  } else {
    // very dry (u = S^(-1/m) > e^80): log(u - 1) = log u + log(1 - 1/u), and
    // 1/u < 2e-35 is far below the pair's precision
    lw = a;
  }
  const F2 b = mul(lw, c.inv_n);  // log w^(1/n)
  if (!(b.hi >= kExpMin && b.hi <= kExpMax)) return false;
  psi = -to_double(mul(exp(T, b), c.inv_alpha));
  dpsi = ff::fast_div(c.coef_d * ff::exp_approx((b.hi - lw.hi) + (a.hi - L.hi)), den.hi);
  return true;
}

// Brooks-Corey constants of the mixed-path closures.
struct ColFFBC {
  F2 nu, theta_r, neg_inv_c, k_exp, psib;
  float coef_d;  // -psi_b / c for the FP32 Jacobian
};

CLM_HD ColFFBC make_col_ff(double nu, double theta_r, const BC& g) {
  ColFFBC c;
  c.nu = ff::from_double(nu);
  c.theta_r = ff::from_double(theta_r);
  c.neg_inv_c = ff::from_double(g.neg_inv_c);
  c.k_exp = ff::from_double(g.k_exp);
  c.psib = ff::from_double(g.psib);
  c.coef_d = (float)g.coef_d;
  return c;
}

// Per-column closure constants of the mixed path for closure CM.
template <class CM>
struct ColFFOf;
template <>
struct ColFFOf<VG> { using type = ColFF; };
template <>
struct ColFFOf<BC> { using type = ColFFBC; };

// Brooks-Corey pressure_head and dpsidvartheta (:219-230, :268-287): for S < 1
//   psi = psi_b u, dpsi = -psi_b u / (c S (nu_safe - theta_r)), u = S^(-1/c);
// for S > 1 psi = (v_safe - nu_safe) / S_s + psi_b, dpsi = 1 / S_s (S = 1, and
// S within a float rounding below 1, take the FP64 closure).
CLM_HD bool psi_dpsi_ff(const ff::Tables& T, const ColFFBC& c, F2 nu_eff, F2 v, double inv_S_s,
                        double& psi, float& dpsi) {
  using namespace ff;
  const F2 guard = add_f(c.theta_r, 1.4901161193847656e-08f);  // theta_r + sqrt(eps)
  const F2 vs = ff_max(v, guard);
  const F2 ns = ff_max(nu_eff, guard);
  const F2 den = sub(ns, c.theta_r);
  const F2 S = div(sub(vs, c.theta_r), den);
  if (!(S.hi < 1.0f)) {
    const F2 d = sub(vs, ns);  // its sign is that of S - 1
    if (!(d.hi > 0.0f)) return false;
    psi = to_double(add(mul(d, from_double(inv_S_s)), c.psib));
    dpsi = narrow_trunc(inv_S_s);
    return true;
  }
  if (!(S.hi > 1e-30f)) return false;
  const F2 L = log(T, S);
  const F2 a = mul(L, c.neg_inv_c);  // log u
  if (!(a.hi <= kExpMax)) return false;
  psi = to_double(mul(exp(T, a), c.psib));
  dpsi = ff::fast_div(c.coef_d * ff::exp_approx(a.hi - L.hi), den.hi);
  return true;
}

// RichardsModel point on the mixed path (update_aux! and dpsidvartheta at
// the iterate, rre.jl:368-380, 402-454): K and psi (FP64 results) and dpsi
// (float) sharing log S; van Genuchten's S^(1/m) is 1/S^(-1/m) (one
// division instead of an exponential) and sqrt(S) is exp(log(S)/2). False
// for saturated cells and outside the double-float range: the caller then
// evaluates the FP64 closure.
CLM_HD bool richards_point_ff(const ff::Tables& T, const ColFF& c, F2 K_sat, F2 v, double& K,
                              double& psi, float& dpsi) {
  using namespace ff;
  const F2 guard = add_f(c.theta_r, 1.4901161193847656e-08f);  // theta_r + sqrt(eps)
  const F2 vs = ff_max(v, guard);
  const F2 ns = ff_max(c.nu, guard);
  const F2 den = sub(ns, c.theta_r);
  const F2 S = div(sub(vs, c.theta_r), den);
  if (!(S.hi < 1.0f) || !(S.hi > 1e-30f)) return false;
  const F2 L = log(T, S);
  const F2 a = mul(L, c.neg_inv_m);  // log u, u = S^(-1/m)
  if (!(a.hi <= kExpMax)) return false;
  const F2 u = exp(T, a);
  const F2 w = add_f(u, -1.0f);
  if (!(w.hi > 1e-30f)) return false;
  const F2 lw = log(T, w);
  const F2 b = mul(lw, c.inv_n);  // log w^(1/n)
  if (!(b.hi >= kExpMin && b.hi <= kExpMax)) return false;
  psi = -to_double(mul(exp(T, b), c.inv_alpha));
  dpsi = fast_div(c.coef_d * exp_approx((b.hi - lw.hi) + (a.hi - L.hi)), den.hi);
  const F2 om = add_f(neg(div(make(1.0f), u)), 1.0f);  // 1 - S^(1/m)
  if (!(om.hi > 1e-30f)) return false;
  const F2 f = add_f(neg(exp(T, mul(log(T, om), c.m))), 1.0f);  // 1 - (1 - S^(1/m))^m
  const F2 h = mul_f(L, 0.5f);                                   // log sqrt(S)
  if (!(h.hi >= kExpMin)) return false;
  K = to_double(mul(mul(K_sat, mul(f, f)), exp(T, h)));
  return true;
}

CLM_HD bool richards_point_ff(const ff::Tables& T, const ColFFBC& c, F2 K_sat, F2 v, double& K,
                              double& psi, float& dpsi) {
  using namespace ff;
  const F2 guard = add_f(c.theta_r, 1.4901161193847656e-08f);
  const F2 vs = ff_max(v, guard);
  const F2 ns = ff_max(c.nu, guard);
  const F2 den = sub(ns, c.theta_r);
  const F2 S = div(sub(vs, c.theta_r), den);
  if (!(S.hi < 1.0f) || !(S.hi > 1e-30f)) return false;
  const F2 L = log(T, S);
  const F2 a = mul(L, c.neg_inv_c);  // log S^(-1/c)
  const F2 ek = mul(L, c.k_exp);     // log S^(2/c + 3)
  if (!(a.hi <= kExpMax) || !(ek.hi >= kExpMin)) return false;
  psi = to_double(mul(exp(T, a), c.psib));
  dpsi = fast_div(c.coef_d * exp_approx(a.hi - L.hi), den.hi);
  K = to_double(mul(K_sat, exp(T, ek)));
  return true;
}

// temperature_from_ρe_int with volumetric_heat_capacity
// (soil_heat_parameterizations.jl:157-192) at theta_l = tl, relative to T_0:
// (rho_e + theta_i rho_i L_f) / rho c, as a double (the Newton residual uses
// T - T_0 only).
CLM_HD double temperature_rel_ff(const EarthFF& E, F2 rho_e, F2 ti, F2 tl, F2 rhoc_ds) {
  using namespace ff;
  // rho c: three non-negative terms (no cancellation: the sloppy sum); the
  // numerator can cancel (T near T_0) and keeps the accurate one
  const F2 rc = add_small(add_small(rhoc_ds, mul(tl, E.rhocp_l)), mul(ti, E.rhocp_i));
  const F2 num = add(rho_e, mul(ti, E.rho_i_LH_f0));
  return to_double(div(num, rc));
}

// impedance_factor * viscosity_factor * hydraulic_conductivity
// (:161-173, :302-323): K_sat (1 - (1 - S^(1/m))^m)^2 exp(lnf + log(S)/2)
// with lnf = -Omega ln10 f_i + gamma (T - gamma_T_ref).
//
// Saturation is tested on the pair (S = 1 - 2^-26 rounds its high word to
// 1.0f; k_r is far from 1 there).
CLM_HD bool conductivity_ff(const ff::Tables& T, const ColFF& c, F2 K_sat, F2 S, F2 lnf,
                            double& K) {
  using namespace ff;
  if (!ff_lt(S, make(1.0f))) {
    if (!(lnf.hi >= kExpMin && lnf.hi <= kExpMax)) return false;
    K = to_double(mul(K_sat, exp(T, lnf)));
    return true;
  }
  if (!(S.hi > 1e-30f)) return false;
  const F2 L = log(T, S);
  const F2 a = mul(L, c.inv_m);  // log S^(1/m)
  if (!(a.hi >= kExpMin)) return false;
  const F2 om = add_f(neg(exp(T, a)), 1.0f);  // 1 - S^(1/m)
  if (!(om.hi > 1e-30f)) return false;
  const F2 tm = exp(T, mul(log(T, om), c.m));  // (1 - S^(1/m))^m
  const F2 f = add_f(neg(tm), 1.0f);
  const F2 e = add(lnf, mul_f(L, 0.5f));
  if (!(e.hi >= kExpMin && e.hi <= kExpMax)) return false;
  K = to_double(mul(mul(K_sat, mul(f, f)), exp(T, e)));
  return true;
}

// Brooks-Corey (:239-251): K_sat exp(lnf + (2/c + 3) log(S)).
CLM_HD bool conductivity_ff(const ff::Tables& T, const ColFFBC& c, F2 K_sat, F2 S, F2 lnf,
                            double& K) {
  using namespace ff;
  if (!ff_lt(S, make(1.0f))) {
    if (!(lnf.hi >= kExpMin && lnf.hi <= kExpMax)) return false;
    K = to_double(mul(K_sat, exp(T, lnf)));
    return true;
  }
  if (!(S.hi > 1e-30f)) return false;
  const F2 e = add(lnf, mul(log(T, S), c.k_exp));
  if (!(e.hi >= kExpMin && e.hi <= kExpMax)) return false;
  K = to_double(mul(K_sat, exp(T, e)));
  return true;
}

// Balland-Arp thermal conductivity (energy_hydrology.jl:756-768,
// soil_heat_parameterizations.jl:243-320): Kersten number and kappa_sat.
struct KappaFF {
  F2 nu, kdry, ku, kf, lku, lkf;
  F2 a_unfrozen;    // (1 + nu_om - alpha nu_quartz - nu_gravel) / 2
  F2 one_m_nuom;    // 1 - nu_om
  F2 one_p_nuom;    // 1 + nu_om
  F2 neg_beta;      // -kersten_beta
};

CLM_HD KappaFF make_kappa_ff(const EHScalars& sc, double nu, double kdry, double ku, double kf,
                             double lku, double lkf, double nuom, double nuq, double nug) {
  KappaFF k;
  k.nu = ff::from_double(nu);
  k.kdry = ff::from_double(kdry);
  k.ku = ff::from_double(ku);
  k.kf = ff::from_double(kf);
  k.lku = ff::from_double(lku);
  k.lkf = ff::from_double(lkf);
  k.a_unfrozen = ff::from_double((1.0 + nuom - sc.kersten_alpha * nuq - nug) * 0.5);
  k.one_m_nuom = ff::from_double(1.0 - nuom);
  k.one_p_nuom = ff::from_double(1.0 + nuom);
  k.neg_beta = ff::from_double(-sc.kersten_beta);
  return k;
}

// The branch decisions (theta_i < eps, theta_l + theta_i < eps, theta_i == 0)
// use the FP64 values, as the FP64 closure does: the Kersten number switches
// formula there.
CLM_HD bool kappa_ff(const ff::Tables& T, const KappaFF& k, double tl_d, double ti_d, F2 tl, F2 ti,
                     double& kappa) {
  using namespace ff;
  const F2 tw = add(tl, ti);
  const F2 S_r = div(tw, k.nu);  // relative_saturation
  if (!(S_r.hi > 1e-30f)) return false;
  const F2 lS = log(T, S_r);
  F2 arg;
  if (ti_d < kEps) {
    const F2 t1 = add_f(exp(T, mul(S_r, k.neg_beta)), 1.0f);
    const F2 t1m3 = div(make(1.0f), mul(mul(t1, t1), t1));
    const F2 h = mul_f(add_f(neg(S_r), 1.0f), 0.5f);
    const F2 base = sub(t1m3, mul(mul(h, h), h));
    if (!(base.hi > 1e-30f)) return false;
    arg = add(mul(k.a_unfrozen, lS), mul(k.one_m_nuom, log(T, base)));
  } else {
    arg = mul(k.one_p_nuom, lS);
  }
  if (!(arg.hi >= kExpMin && arg.hi <= kExpMax)) return false;
  const F2 Ke = exp(T, arg);
  F2 ksat;
  if (tl_d + ti_d < kEps) {
    ksat = mul_f(add(k.ku, k.kf), 0.5f);
  } else if (ti_d == 0.0) {
    ksat = k.ku;
  } else {
    const F2 e = div(add(mul(tl, k.lku), mul(ti, k.lkf)), tw);
    if (!(e.hi >= kExpMin && e.hi <= kExpMax)) return false;
    ksat = exp(T, e);
  }
  kappa = to_double(add(mul(Ke, ksat), mul(add_f(neg(Ke), 1.0f), k.kdry)));
  return true;
}

}  // namespace clm
