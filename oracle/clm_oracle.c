/*
 * ORACLE — test infrastructure only (see clm_oracle.h).
 *
 * FP64 CPU restatement of the ClimaLand.jl v1.11.2 soil column step. Each
 * function cites the reference lines it follows (paths relative to the
 * ClimaLand.jl tree). Third-party numerics that are not vendored in the
 * reference are restated from their published semantics:
 *   ClimaCore 0.15.2  InterpolateC2F (face = mean of the two centres),
 *                     GradientC2F (centre difference / centre spacing,
 *                     SetGradient(0) rows vanish at boundary faces),
 *                     DivergenceF2C (face difference / layer width,
 *                     SetValue supplies the boundary-face flux),
 *                     column_integral_definite! (sum of dz * f),
 *                     FieldMatrixSolver (Thomas per column; block lower
 *                     triangular for EnergyHydrology).
 *   ClimaTimeSteppers 0.10.6  IMEX ARS111 (explicit [0 0; 1 0], b = [1 0];
 *                     implicit [0 0; 0 1], b = [0 1]) with NewtonsMethod,
 *                     UpdateEvery(NewNewtonIteration). Assumed ordering:
 *                     cache_imp!(U) runs on the stage value before the
 *                     first residual; each iteration evaluates the
 *                     residual and the Jacobian at x, solves, sets
 *                     x -= delta and runs cache_imp!(x). The final state is
 *                     u + dt*T_exp[1] + dt*T_imp[2] with
 *                     T_imp[2] = (x - U) / dt.
 */
#include "clm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXL 256

static const double SQRT_EPS = 1.4901161193847656e-08; /* sqrt(eps(Float64)) */
static const double HALF_PI = 1.57079632679489661923;
static const double EPS64 = 2.220446049250313e-16;     /* eps(Float64)        */

/* ======================================================================
 * Pointwise hydrology: soil_hydrology_parameterizations.jl
 * ====================================================================== */

/* :22-31 */
double clmo_volumetric_liquid_fraction(double vartheta_l, double nu_eff,
                                       double theta_r) {
  double v_safe = fmax(vartheta_l, theta_r + SQRT_EPS);
  double nu_safe = fmax(nu_eff, theta_r + SQRT_EPS);
  return (v_safe < nu_safe) ? v_safe : nu_safe;
}

/* :45-50 */
double clmo_effective_saturation(double nu_eff, double vartheta_l,
                                 double theta_r) {
  double v_safe = fmax(vartheta_l, theta_r + SQRT_EPS);
  double nu_safe = fmax(nu_eff, theta_r + SQRT_EPS);
  return (v_safe - theta_r) / (nu_safe - theta_r);
}

/* :59-63 */
double clmo_matric_potential(double alpha, double n, double m, double S) {
  return -pow((pow(S, -1.0 / m) - 1.0) * pow(alpha, -n), 1.0 / n);
}

/* :72-77 (the reference raises an error for psi > 0; here a flag) */
double clmo_inverse_matric_potential(double alpha, double n, double m,
                                     double psi, int* psi_positive) {
  if (psi > 0 && psi_positive) *psi_positive = 1;
  return pow(1.0 + pow(alpha * fabs(psi), n), -m);
}

/* :109-127 */
double clmo_pressure_head(double alpha, double n, double m, double theta_r,
                          double vartheta_l, double nu_eff, double S_s) {
  double S = clmo_effective_saturation(nu_eff, vartheta_l, theta_r);
  double v_safe = fmax(vartheta_l, theta_r + SQRT_EPS);
  double nu_safe = fmax(nu_eff, theta_r + SQRT_EPS);
  if (S <= 1.0) return clmo_matric_potential(alpha, n, m, S);
  return (v_safe - nu_safe) / S_s;
}

/* :135-152 */
double clmo_dpsidvartheta(double alpha, double n, double m, double vartheta,
                          double nu_eff, double theta_r, double S_s) {
  double nu_safe = fmax(nu_eff, theta_r + SQRT_EPS);
  double S = clmo_effective_saturation(nu_safe, vartheta, theta_r);
  if (S < 1.0)
    return 1.0 / (alpha * m * n) / (nu_safe - theta_r) *
           pow(pow(S, -1.0 / m) - 1.0, 1.0 / n - 1.0) * pow(S, -1.0 / m - 1.0);
  return 1.0 / S_s;
}

/* :161-173 */
double clmo_hydraulic_conductivity(double m, double K_sat, double S) {
  double K;
  if (S < 1.0) {
    double f = 1.0 - pow(1.0 - pow(S, 1.0 / m), m);
    K = sqrt(S) * f * f;
  } else {
    K = 1.0;
  }
  return K * K_sat;
}

/* Brooks-Corey closure (retention_models.jl:47-67), :182-185 */
double clmo_bc_matric_potential(double c, double psib, double S) {
  return psib * pow(S, -1.0 / c);
}

/* :195-200 (the reference raises an error for psi > 0; here a flag) */
double clmo_bc_inverse_matric_potential(double c, double psib, double psi,
                                        int* psi_positive) {
  if (psi > 0 && psi_positive) *psi_positive = 1;
  return pow(psi / psib, -c);
}

/* :219-230 */
double clmo_bc_dpsidvartheta(double c, double psib, double vartheta,
                             double nu_eff, double theta_r, double S_s) {
  double nu_safe = fmax(nu_eff, theta_r + SQRT_EPS);
  double S = clmo_effective_saturation(nu_safe, vartheta, theta_r);
  if (S < 1.0) return -psib / (c * (nu_safe - theta_r)) * pow(S, -(1.0 + 1.0 / c));
  return 1.0 / S_s;
}

/* :239-251 */
double clmo_bc_hydraulic_conductivity(double c, double K_sat, double S) {
  double K = (S < 1.0) ? pow(S, 2.0 / c + 3.0) : 1.0;
  return K * K_sat;
}

/* :268-287: for Brooks-Corey S = 1 is psi = psi_b, not 0 */
double clmo_bc_pressure_head(double c, double psib, double theta_r,
                             double vartheta_l, double nu_eff, double S_s) {
  double S = clmo_effective_saturation(nu_eff, vartheta_l, theta_r);
  double v_safe = fmax(vartheta_l, theta_r + SQRT_EPS);
  double nu_safe = fmax(nu_eff, theta_r + SQRT_EPS);
  if (S <= 1.0) return clmo_bc_matric_potential(c, psib, S);
  return (v_safe - nu_safe) / S_s + psib;
}

/* The closure of one column: the reference dispatches on the type of
 * hydrology_cm (vanGenuchten / BrooksCorey). */
typedef struct {
  int bc;             /* CLM_CM_BROOKS_COREY?   */
  double alpha, n, m; /* vanGenuchten           */
  double c, psib;     /* BrooksCorey            */
} hcm_t;

static hcm_t hcm_vg(double alpha, double n, double m) {
  hcm_t h = {0, alpha, n, m, 0.0, 0.0};
  return h;
}

static double hcm_matric_potential(const hcm_t* h, double S) {
  return h->bc ? clmo_bc_matric_potential(h->c, h->psib, S)
               : clmo_matric_potential(h->alpha, h->n, h->m, S);
}

static double hcm_inverse_matric_potential(const hcm_t* h, double psi, int* pos) {
  return h->bc ? clmo_bc_inverse_matric_potential(h->c, h->psib, psi, pos)
               : clmo_inverse_matric_potential(h->alpha, h->n, h->m, psi, pos);
}

static double hcm_pressure_head(const hcm_t* h, double theta_r, double v,
                                double nu_eff, double S_s) {
  return h->bc ? clmo_bc_pressure_head(h->c, h->psib, theta_r, v, nu_eff, S_s)
               : clmo_pressure_head(h->alpha, h->n, h->m, theta_r, v, nu_eff, S_s);
}

static double hcm_dpsidvartheta(const hcm_t* h, double v, double nu_eff,
                                double theta_r, double S_s) {
  return h->bc ? clmo_bc_dpsidvartheta(h->c, h->psib, v, nu_eff, theta_r, S_s)
               : clmo_dpsidvartheta(h->alpha, h->n, h->m, v, nu_eff, theta_r, S_s);
}

static double hcm_hydraulic_conductivity(const hcm_t* h, double K_sat, double S) {
  return h->bc ? clmo_bc_hydraulic_conductivity(h->c, K_sat, S)
               : clmo_hydraulic_conductivity(h->m, K_sat, S);
}

/* ======================================================================
 * Root extraction helpers: src/standalone/Vegetation
 * ====================================================================== */

/* plant_hydraulics.jl:170 */
double clmo_harmonic_mean(double x, double y) {
  return x * y / fmax(x + y, EPS64);
}

/* plant_hydraulics.jl:197-201 */
double clmo_plant_water_flux(double z1, double z2, double psi1, double psi2,
                             double K1, double K2) {
  double K_eff = clmo_harmonic_mean(K1, K2);
  return -K_eff * ((psi2 - psi1) / (z2 - z1) + 1.0);
}

/* plant_hydraulics.jl:256-267 (Weibull) */
double clmo_weibull_conductivity(double K_sat, double psi63, double c,
                                 double psi) {
  double K = (psi <= 0.0) ? exp(-pow(psi / psi63, c)) : 1.0;
  return K * K_sat;
}

/* biomass.jl:362-364 */
double clmo_root_distribution(double z, double rooting_depth) {
  return (1.0 / rooting_depth) * exp(z / rooting_depth);
}

/* :302-305 */
double clmo_impedance_factor(double f_i, double Omega) {
  return pow(10.0, -Omega * f_i);
}

/* :320-323 */
double clmo_viscosity_factor(double T, double gamma, double gamma_T_ref) {
  return exp(gamma * (T - gamma_T_ref));
}

/* src/shared_utilities/utils.jl:95-101: 1 if x - a > eps(FT) else 0 */
double clmo_heaviside(double x, double a) {
  return (x - a > EPS64) ? 1.0 : 0.0;
}

/* ======================================================================
 * Pointwise heat: soil_heat_parameterizations.jl
 * ====================================================================== */

/* :35-52 (argument order as the reference signature: rho_ice, rho_liq) */
static double tf_depressed(double theta_l, double theta_i, double nu,
                           double theta_r, const hcm_t* h, double rho_ice,
                           double rho_liq, double T_freeze, double grav,
                           double LH_f0) {
  double theta_tot = fmin(rho_ice / rho_liq * theta_i + theta_l, nu);
  double psi_w0 = hcm_matric_potential(
      h, clmo_effective_saturation(nu, theta_tot, theta_r));
  return fmax(T_freeze * exp(grav * psi_w0 / LH_f0), 1.0);
}

double clmo_soil_Tf_depressed(double theta_l, double theta_i, double nu,
                              double theta_r, double alpha, double n,
                              double m, double rho_ice, double rho_liq,
                              double T_freeze, double grav, double LH_f0) {
  hcm_t h = hcm_vg(alpha, n, m);
  return tf_depressed(theta_l, theta_i, nu, theta_r, &h, rho_ice, rho_liq,
                      T_freeze, grav, LH_f0);
}

/* :60-62 */
double clmo_thermal_time(double rhoc, double dz, double kappa) {
  return 3.0 * rhoc * dz * dz / kappa;
}

/* :89-122 */
static double phase_change_source(double theta_l, double theta_i, double T,
                                  double tau, double nu, double theta_r,
                                  const hcm_t* h, double rho_i, double rho_l,
                                  double LH_f0, double T_freeze, double grav,
                                  int* psi_positive) {
  double Tf = tf_depressed(theta_l, theta_i, nu, theta_r, h, rho_i, rho_l,
                           T_freeze, grav, LH_f0);
  double psi_T = LH_f0 / grav * log(T / Tf) * clmo_heaviside(Tf - T, 0.0);
  double theta_tot = fmin(rho_i / rho_l * theta_i + theta_l, nu);
  double psi_w0 = hcm_matric_potential(
      h, clmo_effective_saturation(nu, theta_tot, theta_r));
  double theta_star =
      hcm_inverse_matric_potential(h, psi_w0 + psi_T, psi_positive) *
          (nu - theta_r) +
      theta_r;
  return (theta_l - theta_star) / tau;
}

double clmo_phase_change_source(double theta_l, double theta_i, double T,
                                double tau, double nu, double theta_r,
                                double alpha, double n, double m,
                                double rho_i, double rho_l, double LH_f0,
                                double T_freeze, double grav,
                                int* psi_positive) {
  hcm_t h = hcm_vg(alpha, n, m);
  return phase_change_source(theta_l, theta_i, T, tau, nu, theta_r, &h, rho_i,
                             rho_l, LH_f0, T_freeze, grav, psi_positive);
}

/* :157-171 */
double clmo_volumetric_heat_capacity(double theta_l, double theta_i,
                                     double rhoc_ds,
                                     const clm_earth_params* e) {
  double rhocp_i = e->cp_i * e->rho_i;
  double rhocp_l = e->cp_l * e->rho_l;
  return rhoc_ds + theta_l * rhocp_l + theta_i * rhocp_i;
}

/* :180-192 */
double clmo_temperature_from_rho_e_int(double rho_e_int, double theta_i,
                                       double rhoc_s,
                                       const clm_earth_params* e) {
  return e->T_0 + (rho_e_int + theta_i * e->rho_i * e->LH_f0) / rhoc_s;
}

/* :201-212 */
double clmo_volumetric_internal_energy(double theta_i, double rhoc_s,
                                       double T, const clm_earth_params* e) {
  return rhoc_s * (T - e->T_0) - theta_i * e->rho_i * e->LH_f0;
}

/* :221-231 */
double clmo_volumetric_internal_energy_liq(double T,
                                           const clm_earth_params* e) {
  double rhocp_l = e->cp_l * e->rho_l;
  return rhocp_l * (T - e->T_0);
}

/* :243-256 */
double clmo_kappa_sat(double theta_l, double theta_i, double k_unfrozen,
                      double k_frozen) {
  double theta_w = theta_l + theta_i;
  if (theta_w < EPS64) return (k_unfrozen + k_frozen) / 2.0;
  return pow(k_unfrozen, theta_l / theta_w) * pow(k_frozen, theta_i / theta_w);
}

/* :267-270 */
double clmo_thermal_conductivity(double kappa_dry, double K_e,
                                 double kappa_sat) {
  return K_e * kappa_sat + (1.0 - K_e) * kappa_dry;
}

/* :283-285 */
double clmo_relative_saturation(double theta_l, double theta_i, double nu) {
  return (theta_l + theta_i) / nu;
}

/* :301-320 */
double clmo_kersten_number(double theta_i, double S_r, double a, double b,
                           double nu_om, double nu_quartz, double nu_gravel) {
  if (theta_i < EPS64) {
    double t1 = pow(1.0 + exp(-b * S_r), -3.0);
    double t2 = pow((1.0 - S_r) / 2.0, 3.0);
    return pow(S_r, (1.0 + nu_om - a * nu_quartz - nu_gravel) / 2.0) *
           pow(t1 - t2, 1.0 - nu_om);
  }
  return pow(S_r, 1.0 + nu_om);
}

/* :338-348 */
double clmo_kappa_solid(double nu_om, double nu_quartz, double k_om,
                        double k_quartz, double k_minerals) {
  return pow(k_om, nu_om) * pow(k_quartz, nu_quartz) *
         pow(k_minerals, 1.0 - nu_om - nu_quartz);
}

/* :359-361 */
double clmo_kappa_sat_frozen(double kappa_solid, double nu, double kappa_ice) {
  return pow(kappa_solid, 1.0 - nu) * pow(kappa_ice, nu);
}

/* :371-373 */
double clmo_kappa_sat_unfrozen(double kappa_solid, double nu, double kappa_l) {
  return pow(kappa_solid, 1.0 - nu) * pow(kappa_l, nu);
}

/* :386-392 */
double clmo_kappa_dry(double rho_p, double nu, double kappa_solid,
                      double kappa_air) {
  const double a = 0.053;
  double rho_b_dry = (1.0 - nu) * rho_p;
  double num = (a * kappa_solid - kappa_air) * rho_b_dry + kappa_air * rho_p;
  double den = rho_p - (1.0 - a) * rho_b_dry;
  return num / den;
}

/* ======================================================================
 * Forcing descriptor (stands in for the bc(p, t) closures).
 * ====================================================================== */

static uint64_t mix64(uint64_t z) { /* splitmix64 finaliser (Vigna) */
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

double clm_forcing_hash01(uint64_t seed, uint64_t column, int64_t period) {
  uint64_t h = mix64(seed + 0x9E3779B97F4A7C15ULL * (column + 1ULL));
  h = mix64(h ^ ((uint64_t)period * 0xD1B54A32D192ED03ULL));
  return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

/* forcing row c; the rain-pulse hash uses the global column c + col0 */
double clmo_forcing_value(const double* F, int32_t ncol, int32_t c, double t,
                          uint64_t seed, int64_t col0) {
  if (!F) return 0.0;
  double v = F[CLM_F_BASE * ncol + c];
  double amp = F[CLM_F_AMP * ncol + c];
  if (amp != 0.0)
    v += amp * sin(F[CLM_F_OMEGA * ncol + c] * t + F[CLM_F_PHASE * ncol + c]);
  double pp = F[CLM_F_PULSE_PERIOD * ncol + c];
  if (pp > 0.0) {
    int64_t k = (int64_t)floor(t / pp);
    if (clm_forcing_hash01(seed, (uint64_t)(c + col0), k) < F[CLM_F_PULSE_DUTY * ncol + c])
      v += F[CLM_F_PULSE_AMP * ncol + c];
  }
  return v;
}

/* ======================================================================
 * Column model
 * ====================================================================== */

typedef struct {
  int n;
  int eh; /* EnergyHydrology? */
  /* geometry (Domains.jl:183-247, get_Δz :935-949) */
  double z[MAXL];     /* centre coordinates                     */
  double dzc[MAXL];   /* layer widths (ClimaCore Δz_field(z))   */
  double dzf[MAXL];   /* dzf[k]: centre spacing between k-1, k  */
  double dz_top, dz_bottom; /* centre-to-boundary distances      */
  /* parameters */
  double nu, K_sat, S_s, theta_r;
  hcm_t hcm; /* hydrology_cm */
  double kappa_dry, kappa_sat_frozen, kappa_sat_unfrozen, rhoc_ds;
  double nu_om, nu_quartz, nu_gravel;
  double f_max, f_over, R_sb; /* TOPMODEL (Runoff.jl:198-232)          */
  double depth;               /* model.domain.depth: z_hi - z_lo       */
  double z_sfc;               /* the top face (Domains.jl:1054)        */
  const clm_config* cfg;
  const clmo_problem* P;
  int c;
} col_t;

typedef struct { /* p.soil */
  double K[MAXL], psi[MAXL], theta_l[MAXL], T[MAXL], kappa[MAXL], Tf[MAXL];
  double top_w, top_h, bot_w, bot_h;
  int has_dflux;
  /* runoff (Runoff.jl): infiltration, surface runoff R_s, subsurface runoff
   * R_ss, saturated height h_sat, per-layer saturation weights */
  double infiltration, R_s, R_ss, h_sat, R_ess;
  double sat_w[MAXL];
  int runoff_sink;
  double dfluxBCdY;
  double total_water, total_energy;
  int psi_positive;
  /* RootExtraction (soil_canopy_root_interactions.jl:8-39) */
  double root_extraction[MAXL], root_energy_extraction[MAXL];
  /* AtmosDrivenFluxBC: turbulent_fluxes, R_n, q_sfc (CLM_AF_* order) */
  double atmos[CLM_AF_NFIELDS];
  int atmos_on;
} cache_t;

typedef struct {
  double v[MAXL], ti[MAXL], e[MAXL];
  double Fw, Fe;
} state_t;

typedef struct {
  double vv[3][MAXL], ev[3][MAXL], ee[3][MAXL];
} jac_t;

static void col_init(col_t* C, const clmo_problem* P, int c) {
  const clm_config* cfg = &P->cfg;
  int ncol = P->ncol;
  C->P = P;
  C->cfg = cfg;
  C->c = c;
  C->n = P->offsets[c + 1] - P->offsets[c];
  C->eh = (cfg->model == CLM_MODEL_ENERGY_HYDROLOGY);
  int n = C->n;
  double zlo = P->z_lo[c], zhi = P->z_hi[c];
  double zf[MAXL + 1] = {0.0};
  if (P->z_faces) {
    /* the caller's mesh (ClimaCore IntervalMesh faces, e.g. from
     * GeneralizedExponentialStretching): centres are the faces' midpoints,
     * the layer widths their differences (ClimaCore's FiniteDifferenceGrid) */
    const double* f = P->z_faces + P->offsets[c] + c;
    for (int k = 0; k <= n; ++k) zf[k] = f[k];
    zlo = zf[0];
    zhi = zf[n];
  } else {
    /* Column(; zlim, nelements): IntervalMesh with uniform faces */
    for (int k = 0; k <= n; ++k) zf[k] = zlo + (zhi - zlo) * ((double)k / n);
    zf[n] = zhi;
  }
  for (int k = 0; k < n; ++k) {
    C->z[k] = 0.5 * (zf[k] + zf[k + 1]);
    C->dzc[k] = zf[k + 1] - zf[k];
  }
  C->dzf[0] = 0.0;
  for (int k = 1; k < n; ++k) C->dzf[k] = C->z[k] - C->z[k - 1];
  C->dz_top = zf[n] - C->z[n - 1];
  C->dz_bottom = C->z[0] - zf[0];
  const double* p = P->params;
  C->nu = p[CLM_P_NU * ncol + c];
  C->K_sat = p[CLM_P_K_SAT * ncol + c];
  C->S_s = p[CLM_P_S_S * ncol + c];
  C->theta_r = p[CLM_P_THETA_R * ncol + c];
  if (cfg->hydrology_cm == CLM_CM_BROOKS_COREY) {
    memset(&C->hcm, 0, sizeof C->hcm);
    C->hcm.bc = 1;
    C->hcm.psib = p[CLM_P_BC_PSI_B * ncol + c];
    C->hcm.c = p[CLM_P_BC_C * ncol + c];
  } else {
    double vgn = p[CLM_P_VG_N * ncol + c];
    /* m = 1 - 1/n: retention_models.jl:364-368 */
    C->hcm = hcm_vg(p[CLM_P_VG_ALPHA * ncol + c], vgn, 1.0 - 1.0 / vgn);
  }
  C->depth = zhi - zlo;
  C->z_sfc = zhi;
  C->f_max = C->f_over = C->R_sb = 0.0;
  if (P->nparams >= CLM_NPARAM_MAX) {
    C->f_max = p[CLM_P_F_MAX * ncol + c];
    C->f_over = p[CLM_P_F_OVER * ncol + c];
    C->R_sb = p[CLM_P_R_SB * ncol + c];
  }
  if (C->eh) {
    C->kappa_dry = p[CLM_P_KAPPA_DRY * ncol + c];
    C->kappa_sat_frozen = p[CLM_P_KAPPA_SAT_FROZEN * ncol + c];
    C->kappa_sat_unfrozen = p[CLM_P_KAPPA_SAT_UNFROZEN * ncol + c];
    C->rhoc_ds = p[CLM_P_RHOC_DS * ncol + c];
    C->nu_om = p[CLM_P_NU_SS_OM * ncol + c];
    C->nu_quartz = p[CLM_P_NU_SS_QUARTZ * ncol + c];
    C->nu_gravel = p[CLM_P_NU_SS_GRAVEL * ncol + c];
  }
}

static void state_load(const col_t* C, state_t* Y, const double* v,
                       const double* ti, const double* e, const double* Fw,
                       const double* Fe) {
  int o = C->P->offsets[C->c];
  for (int k = 0; k < C->n; ++k) {
    Y->v[k] = v[o + k];
    Y->ti[k] = (C->eh && ti) ? ti[o + k] : 0.0;
    Y->e[k] = (C->eh && e) ? e[o + k] : 0.0;
  }
  Y->Fw = Fw ? Fw[C->c] : 0.0;
  Y->Fe = (C->eh && Fe) ? Fe[C->c] : 0.0;
}

static void state_store(const col_t* C, const state_t* Y, double* v,
                        double* ti, double* e, double* Fw, double* Fe) {
  int o = C->P->offsets[C->c];
  for (int k = 0; k < C->n; ++k) {
    if (v) v[o + k] = Y->v[k];
    if (C->eh && ti) ti[o + k] = Y->ti[k];
    if (C->eh && e) e[o + k] = Y->e[k];
  }
  if (Fw) Fw[C->c] = Y->Fw;
  if (C->eh && Fe) Fe[C->c] = Y->Fe;
}

/* Richards update_aux!: rre.jl:368-380 */
static void richards_update_aux(const col_t* C, const state_t* Y,
                                 cache_t* p) {
  double W = 0.0;
  for (int k = 0; k < C->n; ++k) {
    p->K[k] = hcm_hydraulic_conductivity(
        &C->hcm, C->K_sat,
        clmo_effective_saturation(C->nu, Y->v[k], C->theta_r));
    p->psi[k] = hcm_pressure_head(&C->hcm, C->theta_r, Y->v[k], C->nu, C->S_s);
    W += C->dzc[k] * Y->v[k]; /* rre.jl:502-511 */
  }
  p->total_water = W;
}

/* EnergyHydrology update_aux!: energy_hydrology.jl:722-814 */
static void eh_update_aux(const col_t* C, const state_t* Y, cache_t* p) {
  const clm_config* cfg = C->cfg;
  const clm_earth_params* e = &cfg->earth;
  double W = 0.0, E = 0.0;
  for (int k = 0; k < C->n; ++k) {
    double v = Y->v[k], ti = Y->ti[k];
    double tl = clmo_volumetric_liquid_fraction(v, C->nu - ti, C->theta_r);
    p->theta_l[k] = tl;
    p->kappa[k] = clmo_thermal_conductivity(
        C->kappa_dry,
        clmo_kersten_number(ti, clmo_relative_saturation(tl, ti, C->nu),
                            cfg->kersten_alpha, cfg->kersten_beta, C->nu_om,
                            C->nu_quartz, C->nu_gravel),
        clmo_kappa_sat(tl, ti, C->kappa_sat_unfrozen, C->kappa_sat_frozen));
    p->T[k] = clmo_temperature_from_rho_e_int(
        Y->e[k], ti, clmo_volumetric_heat_capacity(tl, ti, C->rhoc_ds, e), e);
    p->K[k] = clmo_impedance_factor(ti / (tl + ti - C->theta_r),
                                    cfg->ice_impedance_omega) *
              clmo_viscosity_factor(p->T[k], cfg->visc_gamma,
                                    cfg->visc_gamma_T_ref) *
              hcm_hydraulic_conductivity(
                  &C->hcm, C->K_sat,
                  clmo_effective_saturation(C->nu, v, C->theta_r));
    p->psi[k] = hcm_pressure_head(&C->hcm, C->theta_r, v, C->nu - ti, C->S_s);
    /* :797-808 passes (_ρ_l, _ρ_i) into the (_ρ_ice, _ρ_liq) slots. */
    p->Tf[k] = tf_depressed(tl, ti, C->nu, C->theta_r, &C->hcm, e->rho_l,
                            e->rho_i, e->T_freeze, e->grav, e->LH_f0);
    /* :1282-1320 */
    W += C->dzc[k] * (v + ti * e->rho_i / e->rho_l);
    E += C->dzc[k] * Y->e[k];
  }
  p->total_water = W;
  p->total_energy = E;
}

/* EnergyHydrology update_implicit_aux!: energy_hydrology.jl:427-445 */
static void eh_update_implicit_aux(const col_t* C, const state_t* Y,
                                   cache_t* p) {
  const clm_earth_params* e = &C->cfg->earth;
  for (int k = 0; k < C->n; ++k) {
    double v = Y->v[k], ti = Y->ti[k];
    p->T[k] = clmo_temperature_from_rho_e_int(
        Y->e[k], ti,
        clmo_volumetric_heat_capacity(fmin(C->nu - ti, v), ti, C->rhoc_ds, e),
        e);
    p->psi[k] = hcm_pressure_head(&C->hcm, C->theta_r, v, C->nu - ti, C->S_s);
  }
}

/* shared_utilities/boundary_conditions.jl:63-65 */
static double diffusive_flux(double K, double x2, double x1, double dz) {
  return -K * (x2 - x1) / dz;
}

/* Runoff of RichardsAtmosDrivenFluxBC (src/standalone/Soil/Runoff/Runoff.jl):
 * update_infiltration_water_flux! for NoRunoff (:69-80), SurfaceRunoff
 * (:129-145) and TOPMODELRunoff (:234-270) on a RichardsModel column (no ice:
 * model_agnostic_volumetric_ice_content is zero). precip is P_liq (m/s). */
static double runoff_heaviside(double x) { return (x - 0.0 > EPS64) ? 1.0 : 0.0; } /* utils.jl:83-100 */

static void richards_runoff(const col_t* C, const state_t* Y, cache_t* p, double precip) {
  const int n = C->n;
  const double ic = -1.0 * C->K_sat; /* soil_infiltration_capacity (Richards): -K_sat (:386-399) */
  switch (C->cfg->runoff) {
    case CLM_RUNOFF_SURFACE: {
      /* is_saturated(vartheta_l + theta_i, nu) at the top centre */
      const double is_sat = runoff_heaviside((Y->v[n - 1] + 0.0) - C->nu);
      p->infiltration = (1.0 - is_sat) * fmax(ic, precip); /* surface_infiltration (:107-109) */
      p->R_s = fabs(precip - p->infiltration);
      break;
    }
    case CLM_RUNOFF_TOPMODEL: {
      /* is_saturated(vartheta_l + theta_i - theta_r, nu - theta_r) weighted
       * by (vartheta_l + theta_i - theta_r) / (nu - theta_r); h_sat is its
       * column_integral_definite (sum of dz f, bottom to top) */
      double h = 0.0;
      for (int k = 0; k < n; ++k) {
        const double twc = Y->v[k] + 0.0 - C->theta_r, nr = C->nu - C->theta_r;
        p->sat_w[k] = runoff_heaviside(twc - nr) * twc / nr;
        h += C->dzc[k] * p->sat_w[k];
      }
      p->h_sat = h;
      const double zwt = C->depth - h;
      /* topmodel_surface_infiltration (:373-376) */
      const double f_sat = fmin(C->f_max * exp(-C->f_over / 2.0 * zwt), 1.0);
      p->infiltration = (1.0 - f_sat) * fmax(ic, precip);
      p->R_s = fabs(precip - p->infiltration);
      /* the liquid-only repetition gives the same weights without ice;
       * topmodel_ss_flux (:427-429) */
      p->R_ss = C->R_sb * exp(-C->f_over * zwt);
      p->runoff_sink = 1;
      break;
    }
    default: /* NoRunoff */
      p->infiltration = precip;
      p->R_s = 0.0;
  }
}

/* ======================================================================
 * Atmosphere-driven top boundary (CLM_BC_ATMOS): AtmosDrivenFluxBC with a
 * PrescribedAtmosphere and PrescribedRadiativeFluxes on a standalone
 * EnergyHydrology column (boundary_conditions.jl:610-677, 870-936).
 * SurfaceFluxes.jl and Thermodynamics.jl are not among the reference
 * sources: the saturation humidity and the Monin-Obukhov solve below are
 * restatements of the published formulations (Clausius-Clapeyron with a
 * latent heat linear in T; Businger et al. 1971 stability functions at
 * point values), not of those packages' code; the declaration of
 * clm_atmos_params spells them out.
 * ====================================================================== */

void clmo_atmos_params_default(clm_atmos_params* a) {
  memset(a, 0, sizeof *a);
  a->stefan = 5.670374419e-8;
  a->gas_constant = 8.3144598;
  a->molmass_dryair = 0.02897;
  a->molmass_water = 0.01801528;
  a->D_vapor = 2.5e-5;
  a->LH_v0 = 2500800.0;
  a->LH_s0 = 2834400.0;
  a->cp_d = 1004.5;
  a->cp_v = 1859.0;
  a->T_triple = 273.16;
  a->press_triple = 611.657;
  a->von_karman = 0.4;
  a->universal_functions = CLM_UF_GRYANIK;
  a->Pr_0 = 0.98;
  a->a_m = 5.0;
  a->a_h = 5.0;
  a->gryanik_b_m = 0.3;
  a->gryanik_b_h = 0.4;
  a->b_m = 15.0;
  a->b_h = 9.0;
  a->zeta_max = 100.0;
  a->iterations = 8;
}

/* q_vap_saturation(T, rho, Liquid() / Ice()): p_v,sat / (rho R_v T) with
 * p_v,sat = p_tr (T / T_tr)^(dcp / R_v) exp((LH_0 - dcp T_0) / R_v (1/T_tr - 1/T)),
 * dcp = cp_v - cp_l (cp_i), LH_0 = LH_v0 (LH_s0). */
double clmo_q_vap_saturation(double T, double rho, int ice,
                             const clm_atmos_params* a,
                             const clm_earth_params* e) {
  double R_v = a->gas_constant / a->molmass_water;
  double LH_0 = ice ? a->LH_s0 : a->LH_v0;
  double dcp = a->cp_v - (ice ? e->cp_i : e->cp_l);
  double p_v = a->press_triple * pow(T / a->T_triple, dcp / R_v) *
               exp((LH_0 - dcp * e->T_0) / R_v * (1.0 / a->T_triple - 1.0 / T));
  return p_v / (rho * R_v * T);
}

/* energy_hydrology.jl:1352-1368 */
double clmo_dry_soil_layer_thickness(double S_l, double aS_c, double d_ds,
                                     double p) {
  aS_c = fmin(fmax(aS_c, 0.0), 1.0);
  return S_l < aS_c ? d_ds * pow((aS_c - S_l) / S_l, p) : 0.0;
}

/* energy_hydrology.jl:1338-1350 */
double clmo_soil_conductance(double S_l, double S_c, double d_ds, double p,
                             double alpha, double D_vapor) {
  double dsl = clmo_dry_soil_layer_thickness(S_l, alpha * S_c, d_ds, p);
  return D_vapor / fmax(dsl, EPS64);
}

/* Gryanik et al. (2020) stable-side integrated stability functions, in the
 * convention F_h = Pr_0 (ln(dz/z_0b) - psi_h(zeta) + psi_h(zeta z_0b/dz)):
 * phi_m = 1 + a_m zeta / (1 + b_m zeta)^(2/3) gives
 * psi_m = -3 a_m / b_m ((1 + b_m zeta)^(1/3) - 1); phi_h = Pr_0 (1 + a_h
 * zeta / (1 + b_h zeta)) gives psi_h = -a_h / b_h ln(1 + b_h zeta), with
 * b_m, b_h = gryanik_b_m, gryanik_b_h. Gryanik, V. M., C. Lupkes, A. Grachev
 * and D. Sidorenko (2020), J. Atmos. Sci. 77, 2687-2716. */
double clmo_gryanik_psi_m(double zeta, const clm_atmos_params* a) {
  return -3.0 * a->a_m / a->gryanik_b_m * (cbrt(1.0 + a->gryanik_b_m * zeta) - 1.0);
}
double clmo_gryanik_psi_h(double zeta, const clm_atmos_params* a) {
  return -a->a_h / a->gryanik_b_h * log(1.0 + a->gryanik_b_h * zeta);
}

/* Businger-Dyer integrated stability functions */
double clmo_businger_psi_m(double zeta, const clm_atmos_params* a) {
  if (zeta >= 0.0) return -a->a_m * zeta;
  double x = sqrt(sqrt(1.0 - a->b_m * zeta));
  return 2.0 * log((1.0 + x) / 2.0) + log((1.0 + x * x) / 2.0) - 2.0 * atan(x) +
         HALF_PI;
}

double clmo_businger_psi_h(double zeta, const clm_atmos_params* a) {
  if (zeta >= 0.0) return -a->a_h * zeta / a->Pr_0;
  double y = sqrt(1.0 - a->b_h * zeta);
  return 2.0 * log((1.0 + y) / 2.0);
}

/* d psi / d zeta = (1 - phi(zeta)) / zeta on the unstable side:
 * phi_m = (1 - b_m zeta)^(-1/4), phi_h / Pr_0 = (1 - b_h zeta)^(-1/2) */
static double dpsi_m(double zeta, const clm_atmos_params* a) {
  return (1.0 - pow(1.0 - a->b_m * zeta, -0.25)) / zeta;
}
static double dpsi_h(double zeta, const clm_atmos_params* a) {
  return (1.0 - 1.0 / sqrt(1.0 - a->b_h * zeta)) / zeta;
}

/* The stable root of zeta F_h = Ri F_m^2 (Ri >= 0): with the linear
 * Businger-Dyer functions the quadratic A zeta^2 + B zeta + C = 0,
 * A = a_h (1 - r_b) - Ri a_m^2 (1 - r_m)^2, B = Pr_0 lh - 2 Ri a_m (1 - r_m) lm,
 * C = -Ri lm^2; its root continuous from zeta(0) = 0, or zeta_max above the
 * critical Richardson number. */
static double stable_zeta(const clm_atmos_params* a, double Ri, double lm,
                          double lh, double rm, double rb) {
  double am = a->a_m * (1.0 - rm), ah = a->a_h * (1.0 - rb);
  double A = ah - Ri * am * am, B = a->Pr_0 * lh - 2.0 * Ri * am * lm;
  double C = -Ri * lm * lm, D = B * B - 4.0 * A * C, z;
  if (B > 0.0 && D >= 0.0)
    z = -2.0 * C / (B + sqrt(D));
  else if (A > 0.0)
    z = (-B + sqrt(fmax(D, 0.0))) / (2.0 * A);
  else
    z = a->zeta_max;
  return fmin(fmax(z, 0.0), a->zeta_max);
}

/* The stability functions of the configured family (zeta >= 0: Businger-
 * Dyer or Gryanik; zeta < 0: Businger-Dyer) and d psi / d zeta. */
static double uf_psi_m(double zeta, const clm_atmos_params* a) {
  if (zeta >= 0.0 && a->universal_functions == CLM_UF_GRYANIK) return clmo_gryanik_psi_m(zeta, a);
  return clmo_businger_psi_m(zeta, a);
}
static double uf_psi_h(double zeta, const clm_atmos_params* a) {
  if (zeta >= 0.0 && a->universal_functions == CLM_UF_GRYANIK) return clmo_gryanik_psi_h(zeta, a);
  return clmo_businger_psi_h(zeta, a);
}
static double uf_dpsi_m(double zeta, const clm_atmos_params* a) {
  if (zeta >= 0.0) /* Gryanik: -a_m (1 + b_m zeta)^(-2/3); Businger: -a_m */
    return a->universal_functions == CLM_UF_GRYANIK
               ? -a->a_m / pow(1.0 + a->gryanik_b_m * zeta, 2.0 / 3.0) : -a->a_m;
  return dpsi_m(zeta, a);
}
static double uf_dpsi_h(double zeta, const clm_atmos_params* a) {
  if (zeta >= 0.0)
    return a->universal_functions == CLM_UF_GRYANIK ? -a->a_h / (1.0 + a->gryanik_b_h * zeta)
                                                    : -a->a_h / a->Pr_0;
  return dpsi_h(zeta, a);
}

/* Monin-Obukhov similarity at point values (the header's clm_atmos_params
 * comment): `iterations` steps from zeta = 0, each evaluating F_m, F_h, g_h,
 * the surface humidity (q_update, or thv_sfc fixed when q_update is NULL)
 * and Ri_b, then the next zeta from zeta F_h = Ri_b F_m^2 at fixed Ri_b
 * (exact for the linear Businger-Dyer stable functions, else one Newton
 * step). out: zeta, F_m, F_h, g_h, q_sfc, u*. */
typedef double (*mo_q_fn)(double g_h, const void* ctx);
static void mo_solve(const clm_atmos_params* a, double grav, double dz, double U, double z0m,
                     double z0b, double thv_air, double T_sfc, double delta, double q0,
                     mo_q_fn q_update, const void* ctx, double thv_sfc_fixed, double out[6]) {
  const double lm = log(dz / z0m), lh = log(dz / z0b);
  const double rm = z0m / dz, rb = z0b / dz;
  const int gry = a->universal_functions == CLM_UF_GRYANIK;
  double zeta = 0.0, F_m = 0.0, F_h = 0.0, g_h = 0.0, q_sfc = q0, ustar = 0.0;
  int done = 0; /* the last step moved zeta by at most 1e-12 (1 + |zeta|) */
  for (int it = 0;; ++it) {
    F_m = lm - uf_psi_m(zeta, a) + uf_psi_m(zeta * rm, a);
    F_h = a->Pr_0 * (lh - uf_psi_h(zeta, a) + uf_psi_h(zeta * rb, a));
    ustar = a->von_karman * U / F_m;
    g_h = a->von_karman * ustar / F_h;
    if (q_update) q_sfc = q_update(g_h, ctx);
    if (it >= a->iterations || done) break;
    const double thv_sfc = q_update ? T_sfc * (1.0 + delta * q_sfc) : thv_sfc_fixed;
    const double Ri = grav * dz * (thv_air - thv_sfc) / (thv_sfc * U * U);
    double zn;
    if (Ri >= 0.0 && (!gry || zeta <= 0.0)) {
      /* Businger-Dyer: the exact root; Gryanik: its small-zeta form as the
       * start of the Newton steps */
      zn = stable_zeta(a, Ri, lm, lh, rm, rb);
    } else if (Ri < 0.0 && zeta >= 0.0) {
      zn = Ri * lm * lm / (a->Pr_0 * lh); /* one fixed-point step from 0 */
    } else { /* Newton on r = zeta F_h - Ri F_m^2 at fixed Ri */
      const double dF_m = -uf_dpsi_m(zeta, a) + rm * uf_dpsi_m(zeta * rm, a);
      const double dF_h = a->Pr_0 * (-uf_dpsi_h(zeta, a) + rb * uf_dpsi_h(zeta * rb, a));
      const double r = zeta * F_h - Ri * F_m * F_m;
      const double dr = F_h + zeta * dF_h - 2.0 * Ri * F_m * dF_m;
      if (Ri < 0.0)
        zn = fmin(fmax(zeta - r / dr, -a->zeta_max), 0.0);
      else
        zn = dr > 0.0 ? fmin(fmax(zeta - r / dr, 0.0), a->zeta_max) : a->zeta_max;
    }
    done = fabs(zn - zeta) <= 1e-12 * (1.0 + fabs(zeta));
    zeta = zn;
  }
  out[0] = zeta;
  out[1] = F_m;
  out[2] = F_h;
  out[3] = g_h;
  out[4] = q_sfc;
  out[5] = ustar;
}

/* The similarity solve alone at a fixed surface virtual potential
 * temperature (for the known-answer tests). out: zeta, F_m, F_h, g_h, u*. */
int clmo_similarity(const clm_atmos_params* a, double grav, double dz, double U, double z0m,
                    double z0b, double thv_air, double thv_sfc, double* out) {
  if (!a || !out || !(dz > z0m) || !(dz > z0b) || !(U > 0)) return 1;
  double o[6];
  mo_solve(a, grav, dz, U, z0m, z0b, thv_air, 0.0, 0.0, 0.0, NULL, NULL, thv_sfc, o);
  out[0] = o[0];
  out[1] = o[1];
  out[2] = o[2];
  out[3] = o[3];
  out[4] = o[5];
  return 0;
}

/* S_c of the closure (retention_models.jl:42, :64) */
static double hcm_S_c(const hcm_t* h) {
  if (h->bc) return pow(1.0 + 1.0 / h->c, -h->c);
  return pow(1.0 + pow((h->n - 1.0) / h->n, 1.0 - 2.0 * h->n), -h->m);
}

/* update_q_vap_sfc_at_a_point (energy_hydrology.jl:1066-1099) */
static double q_sfc_update(double g_h, double q_air, double T_sfc, double Tf,
                           double g_soil, double beta_ice, double qsat) {
  if (T_sfc < Tf) {
    if (q_air < qsat) return beta_ice * qsat + (1.0 - beta_ice) * q_air;
    return qsat;
  }
  return (g_soil / g_h * qsat + q_air) / (1.0 + g_soil / g_h);
}
typedef struct {
  double q_air, T_sfc, Tf, g_soil, beta_ice, qsat;
} q_ctx_t;
static double q_sfc_of(double g_h, const void* ctx) {
  const q_ctx_t* q = (const q_ctx_t*)ctx;
  return q_sfc_update(g_h, q->q_air, q->T_sfc, q->Tf, q->g_soil, q->beta_ice, q->qsat);
}

/* Runoff of AtmosDrivenFluxBC on an EnergyHydrology column
 * (src/standalone/Soil/Runoff/Runoff.jl): update_infiltration_water_flux! for
 * NoRunoff (:69-71), SurfaceRunoff (:129-148) and TOPMODELRunoff (:234-283,
 * with update_subsurface_energy_runoff!), the infiltration capacity
 * -K_sat impedance(theta_i / (theta_l + theta_i - theta_r)) viscosity(T) of
 * the top centre (:401-413); input is P_liq. */
static void eh_runoff(const col_t* C, const state_t* Y, cache_t* p, double input) {
  const int n = C->n;
  const clm_config* cfg = C->cfg;
  const clm_earth_params* e = &cfg->earth;
  const double tl = p->theta_l[n - 1], ti = Y->ti[n - 1];
  const double ic = -C->K_sat * clmo_impedance_factor(ti / (tl + ti - C->theta_r), cfg->ice_impedance_omega) *
                    clmo_viscosity_factor(p->T[n - 1], cfg->visc_gamma, cfg->visc_gamma_T_ref);
  switch (cfg->runoff) {
    case CLM_RUNOFF_SURFACE: {
      const double is_sat = runoff_heaviside((Y->v[n - 1] + Y->ti[n - 1]) - C->nu);
      p->infiltration = (1.0 - is_sat) * fmax(ic, input);
      p->R_s = fabs(input - p->infiltration);
      break;
    }
    case CLM_RUNOFF_TOPMODEL: {
      const double nr = C->nu - C->theta_r;
      double h = 0.0;
      for (int k = 0; k < n; ++k) { /* weights with ice */
        const double twc = Y->v[k] + Y->ti[k] - C->theta_r;
        h += C->dzc[k] * (runoff_heaviside(twc - nr) * twc / nr);
      }
      const double f_sat = fmin(C->f_max * exp(-C->f_over / 2.0 * (C->depth - h)), 1.0);
      p->infiltration = (1.0 - f_sat) * fmax(ic, input);
      p->R_s = fabs(input - p->infiltration);
      h = 0.0; /* again with liquid water only, for the subsurface runoff */
      double E = 0.0;
      for (int k = 0; k < n; ++k) {
        const double twc = Y->v[k] - C->theta_r;
        p->sat_w[k] = runoff_heaviside(twc - nr) * twc / nr;
        h += C->dzc[k] * p->sat_w[k];
      }
      for (int k = 0; k < n; ++k)
        E += C->dzc[k] * (p->sat_w[k] * clmo_volumetric_internal_energy_liq(p->T[k], e));
      p->h_sat = h;
      p->R_ss = C->R_sb * exp(-C->f_over * (C->depth - h));
      p->R_ess = E * (p->R_ss / fmax(h, EPS64));
      p->runoff_sink = 1;
      break;
    }
    default:
      p->infiltration = input;
      p->R_s = 0.0;
  }
}

/* soil_boundary_fluxes!(::AtmosDrivenFluxBC, ::Val{(:soil,)}, ...) at the
 * update_aux values of Y: turbulent_fluxes!, net_radiation!, NoRunoff
 * infiltration and its energy, top_bc (boundary_conditions.jl:908-936). */
static void atmos_top_bc(const col_t* C, const state_t* Y, cache_t* p) {
  const clmo_problem* P = C->P;
  const clm_atmos_params* a = &P->atm;
  const clm_earth_params* e = &C->cfg->earth;
  const int ncol = P->ncol, c = C->c, n = C->n;
  const double* D = P->atmos;
#define AT(f) D[(f) * ncol + c]
  const double P_liq = AT(CLM_AT_P_LIQ), T_air = AT(CLM_AT_T_AIR);
  const double u_air = AT(CLM_AT_U_AIR), q_air = AT(CLM_AT_Q_AIR);
  const double P_air = AT(CLM_AT_P_AIR), h_air = AT(CLM_AT_H_AIR);
  /* surface values: the top centre (component_temperature etc.) */
  const double T_sfc = p->T[n - 1], Tf_sfc = p->Tf[n - 1], psi_sfc = p->psi[n - 1];
  const double grav = e->grav;
  const double R_d = a->gas_constant / a->molmass_dryair;
  const double R_v = a->gas_constant / a->molmass_water;
  /* air density and surface density (ideal gas; adiabatic extrapolation) */
  const double R_m = R_d + (R_v - R_d) * q_air;
  const double cv_m = (a->cp_d - R_d) + ((a->cp_v - R_v) - (a->cp_d - R_d)) * q_air;
  const double cp_m = a->cp_d + (a->cp_v - a->cp_d) * q_air;
  const double rho_air = P_air / (R_m * T_air);
  const double rho_sfc = rho_air * pow(T_sfc / T_air, cv_m / R_m);
  /* component_specific_humidity (:995-1060) */
  double qsat;
  if (T_sfc > Tf_sfc)
    qsat = clmo_q_vap_saturation(T_sfc, rho_sfc, 0, a, e) *
           exp(grav * fmin(psi_sfc, 0.0) * a->molmass_water / (a->gas_constant * T_sfc));
  else
    qsat = clmo_q_vap_saturation(T_sfc, rho_sfc, 1, a, e);
  /* surface liquid fraction extrapolated from the top two centres
   * (linear_interpolation_to_surface!, Domains.jl:883-895) */
  const double f1 = p->theta_l[n - 1], f2 = p->theta_l[n - 2];
  const double z1 = C->z[n - 1], z2 = C->z[n - 2];
  double th_sfc = (f1 - f2) / (z1 - z2) * (C->dz_top + z1 - z2) + f2;
  th_sfc = fmax(th_sfc, C->theta_r + EPS64);
  const double S_l_sfc = clmo_effective_saturation(C->nu, th_sfc, C->theta_r);
  const double g_soil = clmo_soil_conductance(S_l_sfc, hcm_S_c(&C->hcm), AT(CLM_AT_D_DS),
                                              AT(CLM_AT_EVAP_P), AT(CLM_AT_EVAP_ALPHA),
                                              a->D_vapor);
  const double r = Y->ti[n - 1] / C->nu;
  const double beta_ice = (r * r) * (r * r);
  /* Monin-Obukhov solve */
  const double dz = h_air;
  const double U = fmax(fabs(u_air), AT(CLM_AT_GUSTINESS));
  const double z0m = AT(CLM_AT_Z_0M), z0b = AT(CLM_AT_Z_0B);
  const double delta = R_v / R_d - 1.0;
  const double thv_air = (T_air + grav * dz / a->cp_d) * (1.0 + delta * q_air);
  const q_ctx_t qc = {q_air, T_sfc, Tf_sfc, g_soil, beta_ice, qsat};
  double mo[6];
  mo_solve(a, grav, dz, U, z0m, z0b, thv_air, T_sfc, delta, qsat, q_sfc_of, &qc, 0.0, mo);
  const double g_h = mo[3], q_sfc = mo[4];
  const double E = -rho_sfc * g_h * (q_air - q_sfc);
  const double lhf = a->LH_v0 * E;
  const double shf = -rho_sfc * cp_m * g_h * (T_air + grav * dz / cp_m - T_sfc);
  const double Et = E / e->rho_l;
  const double is_liq = clmo_heaviside(T_sfc, Tf_sfc);
  const double vliq = Et * is_liq, vice = Et * (1.0 - is_liq);
  /* CLMTwoBandSoilAlbedo (soil_albedo.jl:146-198) */
  const double thick = AT(CLM_AT_ALBEDO_TOP_THICKNESS);
  double dz_min = C->dzc[0];
  for (int k = 1; k < n; ++k) dz_min = fmin(dz_min, C->dzc[k]);
  double th_alb;
  if (dz_min < thick) {
    const double z_sfc = C->z_sfc;
    double N = 0.0, I = 0.0;
    for (int k = 0; k < n; ++k)
      N += C->dzc[k] * clmo_heaviside(thick + SQRT_EPS, z_sfc - C->z[k]);
    for (int k = 0; k < n; ++k)
      I += C->dzc[k] * (clmo_heaviside(thick + SQRT_EPS, z_sfc - C->z[k]) * p->theta_l[k] / N);
    th_alb = I;
  } else {
    th_alb = p->theta_l[n - 1];
  }
  const double S_sfc = clmo_effective_saturation(C->nu, th_alb, C->theta_r);
  const double a_par = (1.0 - S_sfc) * AT(CLM_AT_PAR_ALBEDO_DRY) + S_sfc * AT(CLM_AT_PAR_ALBEDO_WET);
  const double a_nir = (1.0 - S_sfc) * AT(CLM_AT_NIR_ALBEDO_DRY) + S_sfc * AT(CLM_AT_NIR_ALBEDO_WET);
  const double alpha = a_par / 2.0 + a_nir / 2.0;
  const double T2 = T_sfc * T_sfc;
  const double R_n = -(1.0 - alpha) * AT(CLM_AT_SW_D) -
                     AT(CLM_AT_EMISSIVITY) * (AT(CLM_AT_LW_D) - a->stefan * (T2 * T2));
  /* the runoff model splits P_liq; the infiltration carries the energy of
   * liquid water at the air temperature (boundary_conditions.jl:988-1003) */
  eh_runoff(C, Y, p, P_liq);
  p->top_w = p->infiltration + vliq;
  p->top_h = R_n + lhf + shf + p->infiltration * clmo_volumetric_internal_energy_liq(T_air, e);
  p->atmos[CLM_AF_LHF] = lhf;
  p->atmos[CLM_AF_SHF] = shf;
  p->atmos[CLM_AF_VAPOR_LIQ] = vliq;
  p->atmos[CLM_AF_VAPOR_ICE] = vice;
  p->atmos[CLM_AF_R_N] = R_n;
  p->atmos[CLM_AF_Q_SFC] = q_sfc;
  p->atmos[CLM_AF_TOP_WATER] = p->top_w;
  p->atmos[CLM_AF_TOP_HEAT] = p->top_h;
  p->atmos_on = 1;
#undef AT
}

/* Boundary fluxes.
 * Richards: rre.jl:111-149 with boundary_flux! methods
 *   WaterFluxBC :168-180, MoistureStateBC top :227-264 / bottom :278-315,
 *   FreeDrainage :340-353, set_dfluxBCdY! (MoistureStateBC top) :375-426.
 * EnergyHydrology: energy_hydrology.jl:273-298 with WaterHeatBC :709-724,
 *   HeatFluxBC :465-477, TemperatureStateBC :494-544,
 *   EnergyWaterFreeDrainage :590-608. */
static void update_boundary_fluxes(const col_t* C, const state_t* Y,
                                   cache_t* p, double t) {
  const clm_config* cfg = C->cfg;
  const clmo_problem* P = C->P;
  const clm_earth_params* e = &cfg->earth;
  int n = C->n, c = C->c, ncol = P->ncol;
  uint64_t seed = cfg->forcing_seed;
  int64_t col0 = cfg->column_offset;
  double f_tw = clmo_forcing_value(P->forcing[CLM_BC_TOP_WATER], ncol, c, t, seed, col0);
  double f_th = clmo_forcing_value(P->forcing[CLM_BC_TOP_HEAT], ncol, c, t, seed, col0);
  double f_bw = clmo_forcing_value(P->forcing[CLM_BC_BOTTOM_WATER], ncol, c, t, seed, col0);
  double f_bh = clmo_forcing_value(P->forcing[CLM_BC_BOTTOM_HEAT], ncol, c, t, seed, col0);
  double nu_top = C->nu, nu_bot = C->nu;

  /* water, top */
  p->runoff_sink = 0;
  p->atmos_on = 0;
  if (cfg->bc_top_water == CLM_BC_ATMOS) atmos_top_bc(C, Y, p);
  switch (cfg->bc_top_water) {
    case CLM_BC_ATMOS:
      break; /* set with the heat flux by atmos_top_bc */
    case CLM_BC_PRECIP_RUNOFF: /* RichardsAtmosDrivenFluxBC: boundary_conditions.jl:200-212 */
      richards_runoff(C, Y, p, f_tw);
      p->top_w = p->infiltration;
      break;
    case CLM_BC_STATE: {
      double psi_bc = hcm_pressure_head(&C->hcm, C->theta_r, f_tw, nu_top, C->S_s);
      p->top_w = diffusive_flux(p->K[n - 1], psi_bc + C->dz_top, p->psi[n - 1],
                                C->dz_top);
      break;
    }
    default:
      p->top_w = f_tw;
  }
  /* water, bottom */
  switch (cfg->bc_bottom_water) {
    case CLM_BC_FREE_DRAINAGE:
      p->bot_w = -1.0 * p->K[0];
      break;
    case CLM_BC_STATE: {
      double psi_bc = hcm_pressure_head(&C->hcm, C->theta_r, f_bw, nu_bot, C->S_s);
      p->bot_w = diffusive_flux(p->K[0], p->psi[0] + C->dz_bottom, psi_bc,
                                C->dz_bottom);
      break;
    }
    default:
      p->bot_w = f_bw;
  }
  if (C->eh) {
    switch (cfg->bc_top_heat) {
      case CLM_BC_ATMOS:
        break;
      case CLM_BC_STATE:
        p->top_h = diffusive_flux(p->kappa[n - 1], f_th, p->T[n - 1], C->dz_top);
        break;
      case CLM_BC_FLUX_ADVECTIVE: {
        double T_adv = P->forcing[CLM_BC_TOP_HEAT]
                           ? P->forcing[CLM_BC_TOP_HEAT][CLM_F_T_ADV * ncol + c]
                           : e->T_0;
        p->top_h = f_th + p->top_w * clmo_volumetric_internal_energy_liq(T_adv, e);
        break;
      }
      default:
        p->top_h = f_th;
    }
    switch (cfg->bc_bottom_heat) {
      case CLM_BC_FREE_DRAINAGE: /* EnergyWaterFreeDrainage */
        p->bot_h = -1.0 * p->K[0] * clmo_volumetric_internal_energy_liq(p->T[0], e);
        break;
      case CLM_BC_STATE:
        p->bot_h = diffusive_flux(p->kappa[0], p->T[0], f_bh, C->dz_bottom);
        break;
      default:
        p->bot_h = f_bh;
    }
  } else {
    p->top_h = p->bot_h = 0.0;
  }
  /* set_dfluxBCdY! exists for RichardsModel + MoistureStateBC at the top */
  p->has_dflux = (!C->eh && cfg->bc_top_water == CLM_BC_STATE);
  if (p->has_dflux) {
    p->dfluxBCdY = p->K[n - 1] *
                   hcm_dpsidvartheta(&C->hcm, Y->v[n - 1], C->nu, C->theta_r,
                                     C->S_s) /
                   C->dz_top;
  }
}

/* make_update_cache = update_aux! + update_boundary_fluxes! */
static void root_extraction(const col_t* C, cache_t* p);

static void update_cache(const col_t* C, const state_t* Y, cache_t* p,
                         double t) {
  if (C->eh)
    eh_update_aux(C, Y, p);
  else
    richards_update_aux(C, Y, p);
  if (C->eh && C->P->root) root_extraction(C, p);
  update_boundary_fluxes(C, Y, p, t);
}

/* make_update_implicit_cache (models.jl:238-246): implicit aux, then the
 * boundary fluxes only if dfluxBCdY is in the cache (rre.jl:460-468,
 * energy_hydrology.jl:447-455). Richards' implicit aux is the full aux
 * (models.jl:207-210). */
static void update_implicit_cache(const col_t* C, const state_t* Y,
                                  cache_t* p, double t) {
  if (C->eh)
    eh_update_implicit_aux(C, Y, p);
  else
    richards_update_aux(C, Y, p);
  if (p->has_dflux) update_boundary_fluxes(C, Y, p, t);
}

/* compute_exp_tendency!: rre.jl:214-243; energy_hydrology.jl:315-350 and
 * the PhaseChange source!: energy_hydrology.jl:838-906. */
/* update_root_extraction! (soil_canopy_root_interactions.jl:8-39), part of
 * the land model's update_boundary_fluxes! (soil_canopy_model.jl:266-268):
 * at the explicit stage only, from the soil aux psi, K, T of update_aux!. */
static void root_extraction(const col_t* C, cache_t* p) {
  const clmo_problem* P = C->P;
  const clm_earth_params* e = &C->cfg->earth;
  int ncol = P->ncol, c = C->c;
  const double* R = P->root;
  double psi_c = R[CLM_RX_PSI_CANOPY * ncol + c];
  double LAI = R[CLM_RX_LAI * ncol + c], RAI = R[CLM_RX_RAI * ncol + c];
  double h = R[CLM_RX_HEIGHT * ncol + c], rd = R[CLM_RX_ROOT_DEPTH * ncol + c];
  double K_can = clmo_weibull_conductivity(R[CLM_RX_K_SAT * ncol + c],
                                           R[CLM_RX_PSI63 * ncol + c],
                                           R[CLM_RX_WEIBULL_C * ncol + c], psi_c);
  for (int k = 0; k < C->n; ++k) {
    double re = clmo_harmonic_mean(LAI, RAI) *
                clmo_plant_water_flux(C->z[k], h / 2.0, p->psi[k], psi_c,
                                      p->K[k], K_can) *
                clmo_root_distribution(C->z[k], rd);
    p->root_extraction[k] = re;
    p->root_energy_extraction[k] =
        re * clmo_volumetric_internal_energy_liq(p->T[k], e);
  }
}

static void exp_tendency(const col_t* C, const state_t* Y, cache_t* p,
                         state_t* dY) {
  int n = C->n;
  for (int k = 0; k < n; ++k) dY->v[k] = dY->ti[k] = dY->e[k] = 0.0;
  dY->Fw = dY->Fe = 0.0;
  if (C->eh && C->cfg->phase_change) {
    const clm_earth_params* e = &C->cfg->earth;
    for (int k = 0; k < n; ++k) {
      double tl = p->theta_l[k], ti = Y->ti[k];
      double tau = clmo_thermal_time(
          clmo_volumetric_heat_capacity(tl, ti, C->rhoc_ds, e), C->dzc[k],
          p->kappa[k]);
      int pp = 0;
      double src = phase_change_source(
          tl, ti, p->T[k], tau, C->nu, C->theta_r, &C->hcm, e->rho_i, e->rho_l,
          e->LH_f0, e->T_freeze, e->grav, &pp);
      if (pp) p->psi_positive = 1;
      dY->v[k] += -src;
      dY->ti[k] += (e->rho_l / e->rho_i) * src;
    }
  }
  /* SoilSublimation source! (energy_hydrology.jl:931-947), appended after
   * the user sources by the EnergyHydrology constructor (:260-268) */
  if (C->eh && p->atmos_on) {
    const clm_earth_params* e = &C->cfg->earth;
    const double vice = p->atmos[CLM_AF_VAPOR_ICE];
    for (int k = 0; k < n; ++k)
      dY->ti[k] += -vice * e->rho_l / e->rho_i *
                   clmo_heaviside(C->z[k] + 2.0 * C->dz_top, 0.0) / (2.0 * C->dz_top);
    dY->Fw += -vice;
  }
  /* RootExtraction source! (soil_canopy_root_interactions.jl:139-159), after
   * PhaseChange in the sources tuple */
  if (C->eh && C->P->root) {
    double sw = 0.0, se = 0.0;
    for (int k = 0; k < n; ++k) {
      dY->v[k] += -1.0 * p->root_extraction[k];
      dY->e[k] += -1.0 * p->root_energy_extraction[k];
    }
    for (int k = 0; k < n; ++k) se += C->dzc[k] * p->root_energy_extraction[k];
    dY->Fe += se;
    for (int k = 0; k < n; ++k) sw += C->dzc[k] * p->root_extraction[k];
    dY->Fw += sw;
  }
}

/* Darcy + heat fluxes at faces and the divergence (ClimaCore
 * DivergenceF2C(SetValue) of -interp(K) * grad(psi + z), etc.):
 * rre.jl:161-203; energy_hydrology.jl:363-425. */
static void imp_tendency(const col_t* C, const state_t* Y, const cache_t* p,
                         state_t* dY) {
  int n = C->n;
  double Fw[MAXL + 1], Fe[MAXL + 1];
  const clm_earth_params* e = &C->cfg->earth;
  (void)Y;
  dY->Fw = -(p->top_w - p->bot_w);
  Fw[0] = p->bot_w;
  Fw[n] = p->top_w;
  for (int k = 1; k < n; ++k) {
    double Kf = 0.5 * (p->K[k - 1] + p->K[k]);
    double gh = ((p->psi[k] + C->z[k]) - (p->psi[k - 1] + C->z[k - 1])) / C->dzf[k];
    Fw[k] = -Kf * gh;
  }
  for (int k = 0; k < n; ++k) dY->v[k] = -((Fw[k + 1] - Fw[k]) / C->dzc[k]);
  if (p->runoff_sink) {
    /* TOPMODELSubsurfaceRunoff source! (Runoff.jl:321-345), an implicit
     * source with the cached R_ss, h_sat and saturation weights */
    for (int k = 0; k < n; ++k) dY->v[k] -= (p->R_ss / fmax(p->h_sat, EPS64)) * p->sat_w[k];
    dY->Fw -= p->R_ss;
  }
  if (C->eh) {
    dY->Fe = -(p->top_h - p->bot_h);
    Fe[0] = p->bot_h;
    Fe[n] = p->top_h;
    for (int k = 1; k < n; ++k) {
      double kf = 0.5 * (p->kappa[k - 1] + p->kappa[k]);
      double gT = (p->T[k] - p->T[k - 1]) / C->dzf[k];
      double gh = ((p->psi[k] + C->z[k]) - (p->psi[k - 1] + C->z[k - 1])) / C->dzf[k];
      double lk = 0.5 * (clmo_volumetric_internal_energy_liq(p->T[k - 1], e) * p->K[k - 1] +
                         clmo_volumetric_internal_energy_liq(p->T[k], e) * p->K[k]);
      Fe[k] = -kf * gT - lk * gh;
    }
    for (int k = 0; k < n; ++k) {
      dY->e[k] = -((Fe[k + 1] - Fe[k]) / C->dzc[k]);
      dY->ti[k] = 0.0;
    }
    if (p->runoff_sink) {
      /* TOPMODELSubsurfaceRunoff on EnergyHydrology (Runoff.jl:347-371): the
       * energy of the drained liquid water */
      for (int k = 0; k < n; ++k) dY->e[k] -= (p->R_ess / fmax(p->h_sat, EPS64)) * p->sat_w[k];
      dY->Fe -= p->R_ess;
    }
  } else {
    dY->Fe = 0.0;
  }
}

/* Assemble -dtγ * div * diag(coef_face) * grad * diag(d) - I as a
 * tridiagonal (lower, diag, upper) given face coefficients a_f at
 * interior faces (the MatrixFields.operator_matrix algebra of
 * rre.jl:402-454). coef_face[k] for k = 1..n-1 multiplies the (SetGradient
 * zero at the boundary) gradient at the face between centres k-1 and k. */
static void assemble_block(const col_t* C, double dtgamma,
                           const double* coef_face, const double* d,
                           double* L, double* M, double* U) {
  int n = C->n;
  for (int k = 0; k < n; ++k) {
    /* Row k of div * diag(-coef) * grad * diag(d):
     *   (1/dzc_k) [-a_up (d_{k+1} x_{k+1} - d_k x_k)
     *              + a_dn (d_k x_k - d_{k-1} x_{k-1})],
     * a = coef / dzf at interior faces; boundary-face rows are zero
     * (GradientC2F with SetGradient(0) at top and bottom). */
    int has_up = (k + 1 <= n - 1), has_dn = (k >= 1);
    double a_up = has_up ? coef_face[k + 1] / C->dzf[k + 1] : 0.0;
    double a_dn = has_dn ? coef_face[k] / C->dzf[k] : 0.0;
    double rowU = has_up ? -a_up * d[k + 1] / C->dzc[k] : 0.0;
    double rowL = has_dn ? -a_dn * d[k - 1] / C->dzc[k] : 0.0;
    double rowD = (a_up + a_dn) * d[k] / C->dzc[k];
    U[k] = -dtgamma * rowU;
    L[k] = -dtgamma * rowL;
    M[k] = -dtgamma * rowD - 1.0;
  }
}

/* Jacobian: Richards rre.jl:391-458, EnergyHydrology
 * energy_hydrology.jl:466-576 (including the "- I" on ∂ρe/∂ϑ,
 * :554-556). */
static void jacobian(const col_t* C, const state_t* Y, const cache_t* p,
                     double dtgamma, jac_t* J) {
  int n = C->n;
  const clm_earth_params* e = &C->cfg->earth;
  double D[MAXL], cf[MAXL + 1];
  for (int k = 0; k < n; ++k)
    D[k] = hcm_dpsidvartheta(&C->hcm, Y->v[k],
                             C->nu - (C->eh ? Y->ti[k] : 0.0), C->theta_r,
                             C->S_s);
  cf[0] = cf[n] = 0.0;
  for (int k = 1; k < n; ++k) cf[k] = 0.5 * (p->K[k - 1] + p->K[k]);
  assemble_block(C, dtgamma, cf, D, J->vv[0], J->vv[1], J->vv[2]);
  if (p->has_dflux) {
    /* LowerDiagonalMatrixRow(topBC_scratch) at the top face: adds
     * dfluxBCdY acting on the top cell, then -dtγ * div */
    J->vv[1][n - 1] += -dtgamma * (p->dfluxBCdY / C->dzc[n - 1]);
  }
  if (!C->eh) return;
  for (int k = 1; k < n; ++k)
    cf[k] = 0.5 * (clmo_volumetric_internal_energy_liq(p->T[k - 1], e) * p->K[k - 1] +
                   clmo_volumetric_internal_energy_liq(p->T[k], e) * p->K[k]);
  assemble_block(C, dtgamma, cf, D, J->ev[0], J->ev[1], J->ev[2]);
  double R[MAXL];
  for (int k = 0; k < n; ++k)
    R[k] = 1.0 / clmo_volumetric_heat_capacity(p->theta_l[k], Y->ti[k],
                                               C->rhoc_ds, e);
  for (int k = 1; k < n; ++k) cf[k] = 0.5 * (p->kappa[k - 1] + p->kappa[k]);
  assemble_block(C, dtgamma, cf, R, J->ee[0], J->ee[1], J->ee[2]);
}

/* Thomas algorithm for one tridiagonal system (bottom to top). */
static void thomas(int n, const double* L, const double* M, const double* U,
                   const double* f, double* x) {
  double cp[MAXL], dp[MAXL];
  cp[0] = U[0] / M[0];
  dp[0] = f[0] / M[0];
  for (int k = 1; k < n; ++k) {
    double den = M[k] - L[k] * cp[k - 1];
    cp[k] = U[k] / den;
    dp[k] = (f[k] - L[k] * dp[k - 1]) / den;
  }
  x[n - 1] = dp[n - 1];
  for (int k = n - 2; k >= 0; --k) x[k] = dp[k] - cp[k] * x[k + 1];
}

/* FieldMatrixSolver: BlockDiagonalSolve (Richards) or
 * BlockLowerTriangularSolve(soil.ϑ_l) (EnergyHydrology),
 * implicit_timestepping.jl:160-171; explicit blocks are -I. */
static void block_solve(const col_t* C, const jac_t* J, const state_t* f,
                        state_t* d) {
  int n = C->n;
  thomas(n, J->vv[0], J->vv[1], J->vv[2], f->v, d->v);
  d->Fw = -f->Fw;
  for (int k = 0; k < n; ++k) d->ti[k] = d->e[k] = 0.0;
  d->Fe = 0.0;
  if (C->eh) {
    double g[MAXL] = {0};
    for (int k = 0; k < n; ++k) {
      double w = J->ev[1][k] * d->v[k];
      if (k > 0) w += J->ev[0][k] * d->v[k - 1];
      if (k < n - 1) w += J->ev[2][k] * d->v[k + 1];
      g[k] = f->e[k] - w;
    }
    thomas(n, J->ee[0], J->ee[1], J->ee[2], g, d->e);
    for (int k = 0; k < n; ++k) d->ti[k] = -f->ti[k];
    d->Fe = -f->Fe;
  }
}

static int state_finite(const col_t* C, const state_t* Y) {
  for (int k = 0; k < C->n; ++k)
    if (!isfinite(Y->v[k]) || !isfinite(Y->ti[k]) || !isfinite(Y->e[k])) return 0;
  return isfinite(Y->Fw) && isfinite(Y->Fe);
}

/* One ARS111 step with NewtonsMethod (see the header comment). */
static void column_step(const col_t* C, state_t* Y, double t, double dt,
                        uint32_t* flag, int32_t* iters) {
  const clm_config* cfg = C->cfg;
  int n = C->n;
  cache_t p;
  memset(&p, 0, sizeof(p));
  state_t Te, U, x, Ti, f, d;
  jac_t J;
  /* stage 1: T_exp!(T_exp[1], u, p, t) = update_cache! + compute_exp_tendency! */
  update_cache(C, Y, &p, t);
  exp_tendency(C, Y, &p, &Te);
  /* stage 2: U = u + dt * a_exp[2,1] * T_exp[1] */
  for (int k = 0; k < n; ++k) {
    U.v[k] = Y->v[k] + dt * Te.v[k];
    U.ti[k] = Y->ti[k] + dt * Te.ti[k];
    U.e[k] = Y->e[k] + dt * Te.e[k];
  }
  U.Fw = Y->Fw + dt * Te.Fw;
  U.Fe = Y->Fe + dt * Te.Fe;
  x = U;
  double t_imp = t + dt;
  update_implicit_cache(C, &x, &p, t_imp);
  int it = 0;
  double prev_norm = INFINITY;
  int maxit = cfg->max_iters;
  for (it = 1; it <= maxit; ++it) {
    imp_tendency(C, &x, &p, &Ti);
    for (int k = 0; k < n; ++k) {
      f.v[k] = U.v[k] + dt * Ti.v[k] - x.v[k];
      f.ti[k] = U.ti[k] + dt * Ti.ti[k] - x.ti[k];
      f.e[k] = U.e[k] + dt * Ti.e[k] - x.e[k];
    }
    f.Fw = U.Fw + dt * Ti.Fw - x.Fw;
    f.Fe = U.Fe + dt * Ti.Fe - x.Fe;
    jacobian(C, &x, &p, dt, &J);
    block_solve(C, &J, &f, &d);
    double s2 = 0.0, se = cfg->energy_norm_scale;
    for (int k = 0; k < n; ++k) {
      x.v[k] -= d.v[k];
      x.ti[k] -= d.ti[k];
      x.e[k] -= d.e[k];
      s2 += d.v[k] * d.v[k] + d.ti[k] * d.ti[k] + (se * d.e[k]) * (se * d.e[k]);
    }
    x.Fw -= d.Fw;
    x.Fe -= d.Fe;
    s2 += d.Fw * d.Fw + d.Fe * d.Fe;
    update_implicit_cache(C, &x, &p, t_imp);
    double nrm = sqrt(s2);
    if (cfg->newton_mode == CLM_NEWTON_TOL) {
      if (nrm > prev_norm && it > 2) *flag |= CLM_COL_DIVERGED;
      prev_norm = nrm;
      if (nrm < cfg->newton_tol) break;
      if (it == maxit) *flag |= CLM_COL_NOT_CONVERGED;
    }
  }
  if (it > maxit) it = maxit;
  *iters = it;
  /* T_imp[2] = (U_2 - temp) / (dt * a_imp[2,2]);
   * u += dt * b_exp[1] * T_exp[1]; u += dt * b_imp[2] * T_imp[2] */
  for (int k = 0; k < n; ++k) {
    Y->v[k] = (Y->v[k] + dt * Te.v[k]) + dt * ((x.v[k] - U.v[k]) / dt);
    Y->ti[k] = (Y->ti[k] + dt * Te.ti[k]) + dt * ((x.ti[k] - U.ti[k]) / dt);
    Y->e[k] = (Y->e[k] + dt * Te.e[k]) + dt * ((x.e[k] - U.e[k]) / dt);
  }
  Y->Fw = (Y->Fw + dt * Te.Fw) + dt * ((x.Fw - U.Fw) / dt);
  Y->Fe = (Y->Fe + dt * Te.Fe) + dt * ((x.Fe - U.Fe) / dt);
  if (p.psi_positive) *flag |= CLM_COL_PSI_POSITIVE;
  if (!state_finite(C, Y)) *flag |= CLM_COL_NONFINITE;
}

/* ======================================================================
 * Batch entry points
 * ====================================================================== */

static int check_problem(const clmo_problem* P) {
  if (!P || P->ncol <= 0 || !P->offsets || !P->z_lo || !P->z_hi || !P->params)
    return CLM_ERR_ARG;
  int need = P->cfg.model == CLM_MODEL_ENERGY_HYDROLOGY ? CLM_NPARAM_EH
                                                        : CLM_NPARAM_RICHARDS;
  if (P->nparams < need) return CLM_ERR_ARG;
  if (P->root && P->cfg.model != CLM_MODEL_ENERGY_HYDROLOGY) return CLM_ERR_ARG;
  if (P->cfg.hydrology_cm != CLM_CM_VAN_GENUCHTEN &&
      P->cfg.hydrology_cm != CLM_CM_BROOKS_COREY)
    return CLM_ERR_ARG;
  if (P->cfg.bc_top_water == CLM_BC_ATMOS || P->cfg.bc_top_heat == CLM_BC_ATMOS) {
    if (P->cfg.model != CLM_MODEL_ENERGY_HYDROLOGY || P->cfg.bc_top_water != CLM_BC_ATMOS ||
        P->cfg.bc_top_heat != CLM_BC_ATMOS || P->cfg.runoff < CLM_RUNOFF_NONE ||
        P->cfg.runoff > CLM_RUNOFF_TOPMODEL || !P->atmos || P->root || P->atm.iterations < 1)
      return CLM_ERR_ARG;
    if (P->cfg.runoff == CLM_RUNOFF_TOPMODEL && P->nparams < CLM_NPARAM_MAX) return CLM_ERR_ARG;
  }
  if (P->cfg.bc_top_water == CLM_BC_PRECIP_RUNOFF) {
    if (P->cfg.model != CLM_MODEL_RICHARDS) return CLM_ERR_ARG;
    if (P->cfg.runoff < CLM_RUNOFF_NONE || P->cfg.runoff > CLM_RUNOFF_TOPMODEL) return CLM_ERR_ARG;
    if (P->cfg.runoff == CLM_RUNOFF_TOPMODEL && P->nparams < CLM_NPARAM_MAX) return CLM_ERR_ARG;
  }
  for (int c = 0; c < P->ncol; ++c) {
    int n = P->offsets[c + 1] - P->offsets[c];
    if (n < 2 || n > MAXL) return CLM_ERR_ARG;
  }
  return CLM_OK;
}

static void set_threads(const clmo_problem* P) {
#ifdef _OPENMP
  if (P->nthreads > 0) omp_set_num_threads(P->nthreads);
#else
  (void)P;
#endif
}

int clmo_atmos_fluxes(const clmo_problem* P, const double* v, const double* ti,
                      const double* e, double* out) {
  int rc = check_problem(P);
  if (rc) return rc;
  if (P->cfg.bc_top_water != CLM_BC_ATMOS || !out) return CLM_ERR_ARG;
  set_threads(P);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < P->ncol; ++c) {
    col_t C;
    col_init(&C, P, c);
    state_t Y;
    cache_t p;
    memset(&p, 0, sizeof(p));
    state_load(&C, &Y, v, ti, e, NULL, NULL);
    update_cache(&C, &Y, &p, 0.0);
    for (int f = 0; f < CLM_AF_NFIELDS; ++f) out[(size_t)f * P->ncol + c] = p.atmos[f];
  }
  return CLM_OK;
}

int clmo_update_cache(const clmo_problem* P, const double* v, const double* ti,
                      const double* e, double t, double* K, double* psi,
                      double* theta_l, double* T, double* kappa, double* Tf,
                      double* bc, double* total_water, double* total_energy) {
  int rc = check_problem(P);
  if (rc) return rc;
  set_threads(P);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < P->ncol; ++c) {
    col_t C;
    col_init(&C, P, c);
    state_t Y;
    cache_t p;
    memset(&p, 0, sizeof(p));
    state_load(&C, &Y, v, ti, e, NULL, NULL);
    update_cache(&C, &Y, &p, t);
    int o = P->offsets[c];
    for (int k = 0; k < C.n; ++k) {
      if (K) K[o + k] = p.K[k];
      if (psi) psi[o + k] = p.psi[k];
      if (C.eh) {
        if (theta_l) theta_l[o + k] = p.theta_l[k];
        if (T) T[o + k] = p.T[k];
        if (kappa) kappa[o + k] = p.kappa[k];
        if (Tf) Tf[o + k] = p.Tf[k];
      }
    }
    if (bc) {
      bc[0 * P->ncol + c] = p.top_w;
      bc[1 * P->ncol + c] = p.top_h;
      bc[2 * P->ncol + c] = p.bot_w;
      bc[3 * P->ncol + c] = p.bot_h;
    }
    if (total_water) total_water[c] = p.total_water;
    if (total_energy) total_energy[c] = p.total_energy;
  }
  return CLM_OK;
}

int clmo_exp_tendency(const clmo_problem* P, const double* v, const double* ti,
                      const double* e, double t, double* dv, double* dti,
                      double* de, double* dFw, double* dFe) {
  int rc = check_problem(P);
  if (rc) return rc;
  set_threads(P);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < P->ncol; ++c) {
    col_t C;
    col_init(&C, P, c);
    state_t Y, dY;
    cache_t p;
    memset(&p, 0, sizeof(p));
    state_load(&C, &Y, v, ti, e, NULL, NULL);
    update_cache(&C, &Y, &p, t);
    exp_tendency(&C, &Y, &p, &dY);
    state_store(&C, &dY, dv, dti, de, dFw, dFe);
  }
  return CLM_OK;
}

int clmo_imp_tendency(const clmo_problem* P, const double* v, const double* ti,
                      const double* e, double t, double* dv, double* dti,
                      double* de, double* dFw, double* dFe) {
  int rc = check_problem(P);
  if (rc) return rc;
  set_threads(P);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < P->ncol; ++c) {
    col_t C;
    col_init(&C, P, c);
    state_t Y, dY;
    cache_t p;
    memset(&p, 0, sizeof(p));
    state_load(&C, &Y, v, ti, e, NULL, NULL);
    update_cache(&C, &Y, &p, t);
    imp_tendency(&C, &Y, &p, &dY);
    state_store(&C, &dY, dv, dti, de, dFw, dFe);
  }
  return CLM_OK;
}

int clmo_jacobian(const clmo_problem* P, const double* v, const double* ti,
                  const double* e, double t, double dtgamma, double* W_vv,
                  double* W_ev, double* W_ee) {
  int rc = check_problem(P);
  if (rc) return rc;
  set_threads(P);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < P->ncol; ++c) {
    col_t C;
    col_init(&C, P, c);
    state_t Y;
    cache_t p;
    jac_t J;
    memset(&p, 0, sizeof(p));
    memset(&J, 0, sizeof(J));
    state_load(&C, &Y, v, ti, e, NULL, NULL);
    update_cache(&C, &Y, &p, t);
    jacobian(&C, &Y, &p, dtgamma, &J);
    int o = P->offsets[c];
    for (int k = 0; k < C.n; ++k)
      for (int j = 0; j < 3; ++j) {
        if (W_vv) W_vv[3 * (o + k) + j] = J.vv[j][k];
        if (C.eh && W_ev) W_ev[3 * (o + k) + j] = J.ev[j][k];
        if (C.eh && W_ee) W_ee[3 * (o + k) + j] = J.ee[j][k];
      }
  }
  return CLM_OK;
}

int clmo_solve(const clmo_problem* P, const double* W_vv, const double* W_ev,
               const double* W_ee, const double* f_v, const double* f_e,
               double* delta_v, double* delta_e) {
  int rc = check_problem(P);
  if (rc) return rc;
  set_threads(P);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < P->ncol; ++c) {
    col_t C;
    col_init(&C, P, c);
    jac_t J;
    state_t f, d;
    memset(&J, 0, sizeof(J));
    memset(&f, 0, sizeof(f));
    int o = P->offsets[c];
    for (int k = 0; k < C.n; ++k) {
      for (int j = 0; j < 3; ++j) {
        J.vv[j][k] = W_vv[3 * (o + k) + j];
        if (C.eh) {
          J.ev[j][k] = W_ev[3 * (o + k) + j];
          J.ee[j][k] = W_ee[3 * (o + k) + j];
        }
      }
      f.v[k] = f_v[o + k];
      if (C.eh) f.e[k] = f_e[o + k];
    }
    block_solve(&C, &J, &f, &d);
    for (int k = 0; k < C.n; ++k) {
      delta_v[o + k] = d.v[k];
      if (C.eh && delta_e) delta_e[o + k] = d.e[k];
    }
  }
  return CLM_OK;
}

int clmo_step(const clmo_problem* P, double* v, double* ti, double* e,
              double* Fw, double* Fe, double t, double dt, int32_t nsteps,
              uint32_t* flags, int32_t* iters) {
  int rc = check_problem(P);
  if (rc) return rc;
  if (!(dt > 0) || nsteps < 0 || P->cfg.max_iters < 1) return CLM_ERR_ARG;
  set_threads(P);
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(| : bad)
  for (int c = 0; c < P->ncol; ++c) {
    col_t C;
    col_init(&C, P, c);
    state_t Y;
    state_load(&C, &Y, v, ti, e, Fw, Fe);
    uint32_t fl = 0;
    int32_t it = 0;
    for (int s = 0; s < nsteps; ++s)
      column_step(&C, &Y, t + s * dt, dt, &fl, &it);
    state_store(&C, &Y, v, ti, e, Fw, Fe);
    if (flags) flags[c] = fl;
    if (iters) iters[c] = it;
    if (fl & CLM_COL_NONFINITE) bad = 1;
  }
  return bad ? CLM_ERR_NAN : CLM_OK;
}

/* Runoff diagnostics of the explicit-stage cache (per column): the
 * infiltration (the top water flux), R_s, R_ss and h_sat (p.soil.infiltration,
 * R_s, R_ss, h_grad of Runoff.jl). */
int clmo_runoff(const clmo_problem* P, const double* v, double t, double* infiltration,
                double* R_s, double* R_ss, double* h_sat) {
  int rc = check_problem(P);
  if (rc) return rc;
  if (P->cfg.bc_top_water != CLM_BC_PRECIP_RUNOFF) return CLM_ERR_ARG;
  set_threads(P);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < P->ncol; ++c) {
    col_t C;
    col_init(&C, P, c);
    state_t Y;
    cache_t p;
    memset(&p, 0, sizeof(p));
    state_load(&C, &Y, v, NULL, NULL, NULL, NULL);
    update_cache(&C, &Y, &p, t);
    infiltration[c] = p.infiltration;
    R_s[c] = p.R_s;
    R_ss[c] = p.R_ss;
    h_sat[c] = p.h_sat;
  }
  return CLM_OK;
}

int clmo_budgets(const clmo_problem* P, const double* v, const double* ti,
                 const double* e, double* total_water, double* total_energy) {
  int rc = check_problem(P);
  if (rc) return rc;
  const clm_earth_params* ep = &P->cfg.earth;
  int eh = P->cfg.model == CLM_MODEL_ENERGY_HYDROLOGY;
  for (int c = 0; c < P->ncol; ++c) {
    col_t C;
    col_init(&C, P, c);
    int o = P->offsets[c];
    double W = 0.0, E = 0.0;
    for (int k = 0; k < C.n; ++k) {
      W += C.dzc[k] * (v[o + k] + (eh ? ti[o + k] * ep->rho_i / ep->rho_l : 0.0));
      if (eh) E += C.dzc[k] * e[o + k];
    }
    if (total_water) total_water[c] = W;
    if (total_energy) total_energy[c] = eh ? E : 0.0;
  }
  return CLM_OK;
}
