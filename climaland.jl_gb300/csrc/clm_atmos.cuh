// Atmosphere-driven top boundary of EnergyHydrology (CLM_BC_ATMOS):
// AtmosDrivenFluxBC with a prescribed atmosphere and radiation on a
// standalone soil column (src/standalone/Soil/boundary_conditions.jl:610-677,
// 870-936; energy_hydrology.jl:910-1368; shared_utilities/drivers.jl:
// 369-382, 699-716). Evaluated once per column and step at the explicit
// stage, in FP64 on both precision paths, from the update_aux values of the
// top layers:
//
//   surface state      T_sfc, psi_sfc, Tf_depressed_sfc of the top centre;
//                      theta_l extrapolated to the surface from the top two
//                      centres (Domains.jl:883-895);
//   humidity           q_vap_saturation (Clausius-Clapeyron with latent heat
//                      linear in T) over liquid, times the Kelvin factor
//                      exp(g min(psi, 0) M_w / (R T)), or over ice
//                      (energy_hydrology.jl:1037-1060);
//   soil conductance   D_vapor / max(dsl, eps), dsl the dry-layer thickness
//                      of Swenson et al. 2012 (:1338-1368);
//   turbulent fluxes   Monin-Obukhov similarity at point values with the
//                      reference's universal functions (Gryanik et al. 2020
//                      on the stable side, Businger-Dyer on the unstable
//                      side; Businger-Dyer on both with CLM_UF_BUSINGER):
//                      zeta = dz / L_MO from zeta F_h = Ri_b F_m^2 (stable
//                      Businger-Dyer: the quadratic's root; otherwise Newton
//                      steps), at most `iterations` steps
//                      (fewer once zeta moves by <= 1e-12 (1 + |zeta|)),
//                      the surface humidity re-evaluated from the
//                      heat conductance in each (update_q_vap_sfc_at_a_point,
//                      :1066-1099);
//   radiation          R_n = -(1 - alpha) SW_d - eps (LW_d - sigma T^4), the
//                      CLM two-band albedo over the top layers
//                      (soil_albedo.jl:146-198);
//   top fluxes         water I + E_liq, energy R_n + LHF + SHF +
//                      I rho e_liq(T_air), I the infiltrating part of P_liq
//                      after the runoff model (eh_runoff below); the
//                      sublimation part of E leaves theta_i (SoilSublimation,
//                      :931-947).
//
// SurfaceFluxes.jl and Thermodynamics.jl are not among the reference
// sources; the saturation humidity and the similarity solve restate the
// published formulations (constants in clm_atmos_params).

#pragma once

#include "clm_geometry.cuh"
#include "clm_physics.cuh"

namespace clm {

constexpr double kHalfPi = 1.57079632679489661923;

// Constants of the boundary, derived once per handle.
struct AtmosK {
  double stefan, D_vapor, LH_v0, cp_d, cp_v, von_karman;
  double R_d, R_v, delta;    // delta = R_v / R_d - 1
  double Mw_over_R;          // M_w / R (Kelvin factor)
  double Pr_0, a_m, a_h, a_h_over_Pr, b_m, b_h, zeta_max;
  int iterations;
  int gryanik;               // stable side: Gryanik et al. (2020) instead of Businger-Dyer
  double gb_m, gb_h;         // Gryanik's b_m, b_h
  double g3am, gah;          // 3 a_m / gb_m, a_h / gb_h
  // saturation vapour pressure, liquid [0] / ice [1]:
  // p_v = p_tr exp(ex ln(T / T_tr) + cc (1 / T_tr - 1 / T))
  double ex[2], cc[2];
  double inv_T_tr, p_tr_over_R_v;
};

inline AtmosK make_atmos_k(const clm_atmos_params& a, const clm_earth_params& e) {
  AtmosK K{};  // zeroed padding: handles compare the bytes
  K.stefan = a.stefan;
  K.D_vapor = a.D_vapor;
  K.LH_v0 = a.LH_v0;
  K.cp_d = a.cp_d;
  K.cp_v = a.cp_v;
  K.von_karman = a.von_karman;
  K.R_d = a.gas_constant / a.molmass_dryair;
  K.R_v = a.gas_constant / a.molmass_water;
  K.delta = K.R_v / K.R_d - 1.0;
  K.Mw_over_R = a.molmass_water / a.gas_constant;
  K.Pr_0 = a.Pr_0;
  K.a_m = a.a_m;
  K.a_h = a.a_h;
  K.a_h_over_Pr = a.a_h / a.Pr_0;
  K.b_m = a.b_m;
  K.b_h = a.b_h;
  K.zeta_max = a.zeta_max;
  K.iterations = a.iterations;
  K.gryanik = a.universal_functions == CLM_UF_GRYANIK;
  if (K.gryanik) {
    K.gb_m = a.gryanik_b_m;
    K.gb_h = a.gryanik_b_h;
    K.g3am = 3.0 * a.a_m / a.gryanik_b_m;
    K.gah = a.a_h / a.gryanik_b_h;
  }
  const double LH0[2] = {a.LH_v0, a.LH_s0};
  const double cpc[2] = {e.cp_l, e.cp_i};
  for (int i = 0; i < 2; ++i) {
    const double dcp = a.cp_v - cpc[i];
    K.ex[i] = dcp / K.R_v;
    K.cc[i] = (LH0[i] - dcp * e.T_0) / K.R_v;
  }
  K.inv_T_tr = 1.0 / a.T_triple;
  K.p_tr_over_R_v = a.press_triple / K.R_v;
  return K;
}

// x^y for x > 0
CLM_HD double powp(const Tables& Tb, double x, double y) { return fm::exp(Tb, y * fm::log(Tb, x)); }

// q_vap_saturation(T, rho, phase) = p_v,sat(T) / (rho R_v T)
CLM_HD double q_sat(const Tables& Tb, const AtmosK& K, double T, double rho, int ice) {
  const double pv_over_Rv =
      K.p_tr_over_R_v * fm::exp(Tb, K.ex[ice] * fm::log(Tb, T * K.inv_T_tr) + K.cc[ice] * (K.inv_T_tr - 1.0 / T));
  return pv_over_Rv / (rho * T);
}

// Businger-Dyer integrated stability functions (the stable side of
// CLM_UF_BUSINGER; the unstable side of both families)
CLM_HD double psi_m(const Tables& Tb, const AtmosK& K, double zeta) {
  if (zeta >= 0.0) return -K.a_m * zeta;
  const double x = sqrt(sqrt(1.0 - K.b_m * zeta));
  return 2.0 * fm::log(Tb, (1.0 + x) * 0.5) + fm::log(Tb, (1.0 + x * x) * 0.5) - 2.0 * atan(x) + kHalfPi;
}

CLM_HD double psi_h(const Tables& Tb, const AtmosK& K, double zeta) {
  if (zeta >= 0.0) return -K.a_h_over_Pr * zeta;
  return 2.0 * fm::log(Tb, (1.0 + sqrt(1.0 - K.b_h * zeta)) * 0.5);
}

// The stable root of zeta F_h(zeta) = Ri F_m(zeta)^2 (Ri >= 0): with the linear
// Businger-Dyer functions a quadratic A zeta^2 + B zeta + C = 0,
// A = a_h (1 - r_b) - Ri a_m^2 (1 - r_m)^2, B = Pr_0 lh - 2 Ri a_m (1 - r_m) lm,
// C = -Ri lm^2; the root continuous from zeta(0) = 0, or zeta_max above the
// critical Richardson number (no root).
CLM_HD double stable_zeta(const AtmosK& K, double Ri, double lm, double lh, double rm, double rb) {
  const double am = K.a_m * (1.0 - rm), ah = K.a_h * (1.0 - rb);
  const double A = ah - Ri * am * am, B = K.Pr_0 * lh - 2.0 * Ri * am * lm, C = -Ri * lm * lm;
  const double D = B * B - 4.0 * A * C;
  double z;
  if (B > 0.0 && D >= 0.0)
    z = -2.0 * C / (B + sqrt(D));
  else if (A > 0.0)
    z = (-B + sqrt(fmax(D, 0.0))) / (2.0 * A);
  else
    z = K.zeta_max;
  return fmin(fmax(z, 0.0), K.zeta_max);
}

// S_c of the closure (retention_models.jl:42, :64)
CLM_HD double closure_S_c(const Tables& Tb, const VG& g) {
  return powp(Tb, 1.0 + powp(Tb, (g.n - 1.0) * g.inv_n, 1.0 - 2.0 * g.n), -g.m);
}
CLM_HD double closure_S_c(const Tables& Tb, const BC& g) { return powp(Tb, 1.0 + 1.0 / g.c, -g.c); }

// The update_aux values the boundary reads.
struct AtmosSfc {
  double T, Tf, psi;    // top centre
  double th1, th2;      // theta_l of the top two centres
  double z1, z2;        // their coordinates
  double dz_top;        // top centre to the surface
  double th_alb;        // theta_l for the albedo (top-thickness mean or top centre)
  double ti;            // theta_i of the top centre
  double infil;         // infiltration of P_liq after the runoff model (EHRunoff)
};

struct AtmosOut {
  double top_w, top_h;  // top_bc.water, top_bc.heat
  double vice;          // turbulent_fluxes.vapor_flux_ice (sublimation source)
  double lhf, shf, vliq, R_n, q_sfc;
};

// Field f of slot s in the per-slot driver rows.
struct AtmosRow {
  const double* a;
  int st, s;
  CLM_HD double operator()(int f) const { return a[(int64_t)f * st + s]; }
};

template <class CM>
CLM_HD AtmosOut atmos_bc(const Tables& Tb, const AtmosK& K, const Earth& E, const AtmosRow& D,
                         const CM& g, double nu, double theta_r, const AtmosSfc& sf) {
  const double T_air = D(CLM_AT_T_AIR), q_air = D(CLM_AT_Q_AIR), h_air = D(CLM_AT_H_AIR);
  const double P_liq = D(CLM_AT_P_LIQ);
  const double grav = E.grav;
  // air and surface densities (ideal gas; adiabatic extrapolation to T_sfc)
  const double R_m = K.R_d + (K.R_v - K.R_d) * q_air;
  const double cv_d = K.cp_d - K.R_d;
  const double cv_m = cv_d + ((K.cp_v - K.R_v) - cv_d) * q_air;
  const double cp_m = K.cp_d + (K.cp_v - K.cp_d) * q_air;
  const double rho_air = D(CLM_AT_P_AIR) / (R_m * T_air);
  const double rho_sfc = rho_air * powp(Tb, sf.T / T_air, cv_m / R_m);
  // saturated surface humidity (component_specific_humidity)
  double qsat;
  if (sf.T > sf.Tf)
    qsat = q_sat(Tb, K, sf.T, rho_sfc, 0) *
           fm::exp(Tb, grav * fmin(sf.psi, 0.0) * K.Mw_over_R / sf.T);
  else
    qsat = q_sat(Tb, K, sf.T, rho_sfc, 1);
  // soil vapour conductance from the surface liquid fraction
  double th_sfc = (sf.th1 - sf.th2) / (sf.z1 - sf.z2) * (sf.dz_top + sf.z1 - sf.z2) + sf.th2;
  th_sfc = fmax(th_sfc, theta_r + kEps);
  const double S_l = saturation(nu, th_sfc, theta_r).S;
  const double aSc = fmin(fmax(D(CLM_AT_EVAP_ALPHA) * closure_S_c(Tb, g), 0.0), 1.0);
  const double dsl = S_l < aSc ? D(CLM_AT_D_DS) * powp(Tb, (aSc - S_l) / S_l, D(CLM_AT_EVAP_P)) : 0.0;
  const double g_soil = K.D_vapor / fmax(dsl, kEps);
  const double r = sf.ti / nu;
  const double beta_ice = (r * r) * (r * r);
  const bool subl = sf.T < sf.Tf;
  // Monin-Obukhov similarity
  const double dz = h_air;
  const double U = fmax(fabs(D(CLM_AT_U_AIR)), D(CLM_AT_GUSTINESS));
  const double z0m = D(CLM_AT_Z_0M), z0b = D(CLM_AT_Z_0B);
  const double lm = fm::log(Tb, dz / z0m), lh = fm::log(Tb, dz / z0b);
  const double thv_air = (T_air + grav * dz / K.cp_d) * (1.0 + K.delta * q_air);
  const double gU = grav * dz / (U * U);
  const double rm = z0m / dz, rb = z0b / dz;
  const double kk_U = K.von_karman * K.von_karman * U;
  double zeta = 0.0, g_h = 0.0, q_sfc = qsat;
  bool done = false;  // the last step moved zeta by at most 1e-12 (1 + |zeta|)
  for (int it = 0;; ++it) {
    // F_m = lm - psi_m(zeta) + psi_m(zeta z0m/dz), F_h = Pr_0 (lh - psi_h(zeta) +
    // psi_h(zeta z0b/dz)) and, on the unstable side, their zeta-derivatives
    // (psi'(zeta) = (1 - phi(zeta)) / zeta, phi_m = 1/x, phi_h = Pr_0 / y); the
    // two logarithms and arctangents of each pair combine into one
    // (atan x' - atan x = atan((x' - x) / (1 + x x')) for x, x' >= 1)
    double F_m, F_h, dF_m = 0.0, dF_h = 0.0;
    if (zeta >= 0.0 && K.gryanik) {
      // Gryanik et al. (2020): psi_m = -3 a_m / b_m ((1 + b_m zeta)^(1/3) - 1),
      // psi_h = -a_h / b_h ln(1 + b_h zeta); psi' = -a_m (1 + b_m zeta)^(-2/3),
      // -a_h / (1 + b_h zeta)
      const double c = cbrt(1.0 + K.gb_m * zeta), cp = cbrt(1.0 + K.gb_m * (zeta * rm));
      const double u = 1.0 + K.gb_h * zeta, up = 1.0 + K.gb_h * (zeta * rb);
      F_m = lm + K.g3am * (c - cp);
      F_h = K.Pr_0 * (lh + K.gah * fm::log(Tb, u * fm::rcp(up)));
      dF_m = K.a_m * (fm::rcp(c * c) - rm * fm::rcp(cp * cp));
      dF_h = K.Pr_0 * K.a_h * (fm::rcp(u) - rb * fm::rcp(up));
    } else if (zeta >= 0.0) {
      F_m = lm - psi_m(Tb, K, zeta) + psi_m(Tb, K, zeta * rm);
      F_h = K.Pr_0 * (lh - psi_h(Tb, K, zeta) + psi_h(Tb, K, zeta * rb));
    } else {
      // x = v^(1/4) and 1/x from s = sqrt(v) = x^2 and rsqrt(s); y and 1/y alike
      const double s = sqrt(1.0 - K.b_m * zeta), sp = sqrt(1.0 - K.b_m * (zeta * rm));
      const double ix = rsqrt(s), ixp = rsqrt(sp);
      const double x = s * ix, xp = sp * ixp;
      const double num = (1.0 + xp) * (1.0 + xp) * (1.0 + sp), den = (1.0 + x) * (1.0 + x) * (1.0 + s);
      F_m = lm + fm::log(Tb, num * fm::rcp(den)) - 2.0 * atan((xp - x) * fm::rcp(1.0 + x * xp));
      const double w = 1.0 - K.b_h * zeta, wp = 1.0 - K.b_h * (zeta * rb);
      const double iy = rsqrt(w), iyp = rsqrt(wp);
      const double y = w * iy, yp = wp * iyp;
      F_h = K.Pr_0 * (lh + 2.0 * fm::log(Tb, (1.0 + yp) * fm::rcp(1.0 + y)));
      const double iz = fm::rcp(zeta);
      dF_m = (ix - ixp) * iz;
      dF_h = K.Pr_0 * (iy - iyp) * iz;
    }
    g_h = kk_U * fm::rcp(F_m * F_h);
    if (subl)
      q_sfc = q_air < qsat ? beta_ice * qsat + (1.0 - beta_ice) * q_air : qsat;
    else  // (g_soil / g_h qsat + q_air) / (1 + g_soil / g_h)
      q_sfc = (g_soil * qsat + g_h * q_air) * fm::rcp(g_h + g_soil);
    if (it >= K.iterations || done) break;
    const double thv_sfc = sf.T * (1.0 + K.delta * q_sfc);
    const double Ri = gU * (thv_air - thv_sfc) * fm::rcp(thv_sfc);
    double zn;
    if (Ri >= 0.0 && (!K.gryanik || zeta <= 0.0)) {
      // Businger-Dyer: the exact root; Gryanik: its small-zeta form as the
      // start of the Newton steps
      zn = stable_zeta(K, Ri, lm, lh, rm, rb);
    } else if (Ri < 0.0 && zeta >= 0.0) {
      zn = Ri * lm * lm * fm::rcp(K.Pr_0 * lh);  // one fixed-point step from 0
    } else {
      // Newton on r = zeta F_h - Ri F_m^2 at fixed Ri
      const double r = zeta * F_h - Ri * F_m * F_m;
      const double dr = F_h + zeta * dF_h - 2.0 * Ri * F_m * dF_m;
      if (Ri < 0.0)
        zn = fmin(fmax(zeta - r * fm::rcp(dr), -K.zeta_max), 0.0);
      else
        zn = dr > 0.0 ? fmin(fmax(zeta - r * fm::rcp(dr), 0.0), K.zeta_max) : K.zeta_max;
    }
    done = fabs(zn - zeta) <= 1e-12 * (1.0 + fabs(zeta));
    zeta = zn;
  }
  AtmosOut o;
  const double Ev = -rho_sfc * g_h * (q_air - q_sfc);
  o.lhf = K.LH_v0 * Ev;
  o.shf = -rho_sfc * cp_m * g_h * (T_air + grav * dz / cp_m - sf.T);
  const double Et = Ev / E.rho_l;
  const double is_liq = (sf.T - sf.Tf > kEps) ? 1.0 : 0.0;
  o.vliq = Et * is_liq;
  o.vice = Et * (1.0 - is_liq);
  // net radiation with the two-band albedo
  const double S_a = saturation(nu, sf.th_alb, theta_r).S;
  const double a_par = (1.0 - S_a) * D(CLM_AT_PAR_ALBEDO_DRY) + S_a * D(CLM_AT_PAR_ALBEDO_WET);
  const double a_nir = (1.0 - S_a) * D(CLM_AT_NIR_ALBEDO_DRY) + S_a * D(CLM_AT_NIR_ALBEDO_WET);
  const double alpha = a_par * 0.5 + a_nir * 0.5;
  const double T2 = sf.T * sf.T;
  o.R_n = -(1.0 - alpha) * D(CLM_AT_SW_D) - D(CLM_AT_EMISSIVITY) * (D(CLM_AT_LW_D) - K.stefan * (T2 * T2));
  o.q_sfc = q_sfc;
  o.top_w = sf.infil + o.vliq;
  o.top_h = ((o.R_n + o.lhf) + o.shf) + sf.infil * rho_e_liq(E, T_air);
  return o;
}

// Runoff of the atmosphere-driven boundary on an EnergyHydrology column
// (src/standalone/Soil/Runoff/Runoff.jl): NoRunoff (:69-71), SurfaceRunoff
// (:129-148) and TOPMODELRunoff (:234-283) with the infiltration capacity
// -K_sat impedance viscosity of the top centre (:401-413), and TOPMODEL's
// implicit subsurface sink (:347-371): R_ss / max(h, eps) w_k on vartheta_l
// and R_ess / max(h, eps) w_k on rho e_int, w_k the liquid saturation weights.
struct EHRunoff {
  double infil;       // infiltration (m/s)
  double R_ss, R_ess; // subsurface water and energy runoff (TOPMODEL), else 0
  double cw, ce;      // R_ss / max(h, eps), R_ess / max(h, eps)
};

// H(vartheta - nu) (vartheta - theta_r) / (nu - theta_r) with the runoff
// heaviside (x > eps)
CLM_HD double sat_weight(double twc, double nr) { return ((twc - nr) - 0.0 > kEps ? 1.0 : 0.0) * twc / nr; }

// layer(k, v, ti, T) fills the layer's vartheta_l, theta_i and T
template <class Layer, class G_>
CLM_HD EHRunoff eh_runoff(const Tables& Tb, const Earth& E, const EHScalars& sc, int runoff,
                          const G_& G, double nu, double theta_r, double K_sat, double f_max,
                          double f_over, double R_sb, double tl_top, double input, Layer layer) {
  EHRunoff r{input, 0.0, 0.0, 0.0, 0.0};
  if (runoff == CLM_RUNOFF_NONE) return r;
  const int n = G.n;
  double v, ti, T;
  layer(n - 1, v, ti, T);
  const double ic = -K_sat * fm::exp(Tb, -sc.omega_ln10 * (ti / (tl_top + ti - theta_r))) *
                    fm::exp(Tb, sc.visc_gamma * (T - sc.visc_gamma_T_ref));
  if (runoff == CLM_RUNOFF_SURFACE) {
    const double is_sat = ((v + ti) - nu) - 0.0 > kEps ? 1.0 : 0.0;
    r.infil = (1.0 - is_sat) * fmax(ic, input);
    return r;
  }
  const double nr = nu - theta_r;
  double h_ice = 0.0, h = 0.0, Ew = 0.0;
  for (int k = 0; k < n; ++k) {
    layer(k, v, ti, T);
    const double dzk = G.width(k);
    h_ice += dzk * sat_weight(v + ti - theta_r, nr);
    const double w = sat_weight(v - theta_r, nr);
    h += dzk * w;
    Ew += dzk * (w * rho_e_liq(E, T));
  }
  const double depth = G.zhi - G.zlo;
  const double f_sat = fmin(f_max * fm::exp(Tb, -f_over / 2.0 * (depth - h_ice)), 1.0);
  r.infil = (1.0 - f_sat) * fmax(ic, input);
  r.R_ss = R_sb * fm::exp(Tb, -f_over * (depth - h));
  r.R_ess = Ew * (r.R_ss / fmax(h, kEps));
  r.cw = r.R_ss / fmax(h, kEps);
  r.ce = r.R_ess / fmax(h, kEps);
  return r;
}

// Tf_depressed as update_aux computes it (energy_hydrology.jl:797-808 passes
// (rho_l, rho_i) into the (rho_ice, rho_liq) slots of soil_Tf_depressed).
template <class CM>
CLM_HD double tf_depressed_aux(const Tables& Tb, const Earth& E, const CM& g, double nu,
                               double theta_r, double theta_l, double theta_i) {
  const double tt = fmin(E.rho_l / E.rho_i * theta_i + theta_l, nu);
  const double pw = matric_of(Tb, g, nu, tt, theta_r);
  return fmax(E.T_freeze * fm::exp(Tb, E.grav_over_LH_f0 * pw), 1.0);
}

// theta_l for the albedo: the mean over the layers centred within
// `thick` of the surface when the thinnest layer is thinner than it
// (column_integral_definite of H theta_l / N), else the top centre's.
template <class ThetaL, class G_>
CLM_HD double albedo_theta(const G_& G, double thick, ThetaL theta_l) {
  if (!(G.min_width() < thick)) return theta_l(G.n - 1);
  // H(thick + sqrt(eps) - (z_sfc - z_k)) rises with k: the layers k0..n-1
  auto H = [&](int k) { return (thick + kSqrtEps) - (G.zhi - G.centre(k)) > kEps; };
  int k0 = G.n;
  while (k0 > 0 && H(k0 - 1)) --k0;
  double N = 0.0;
  for (int k = k0; k < G.n; ++k) N += G.width(k);
  double I = 0.0;
  for (int k = k0; k < G.n; ++k) I += G.width(k) * (theta_l(k) / N);
  return I;
}

// SoilSublimation's factor for layer k: H(z_k + 2 dz_top) / (2 dz_top), with
// the reference's absolute coordinates.
template <class G_>
CLM_HD double sublimation_weight(const G_& G, int k, double dz_top) {
  return (((G.centre(k) + 2.0 * dz_top) - 0.0 > kEps) ? 1.0 : 0.0) / (2.0 * dz_top);
}

}  // namespace clm
