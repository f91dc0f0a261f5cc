/*
 * ORACLE — test infrastructure only.
 *
 * A plain C, FP64, CPU restatement of the reference ClimaLand.jl soil column
 * step (RichardsModel / EnergyHydrology closures, ARS111 + Newton, the block
 * Thomas solve). It is the checker that tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg compare the CUDA library against; the product
 * (libclimaland_cuda) never links, loads or calls it.
 *
 * Layout: same as include/climaland_cuda.h (cell = offsets[c] + k, k = 0 the
 * bottom layer; per-column parameters and forcing as SoA rows of ncol).
 *
 * Pinning: the closures, tendencies, Jacobians and boundary conditions are
 * pinned by the reference's own known-answer tests (tests/
 * test_oracle_known_answers.py). The atmosphere-driven boundary's turbulent
 * fluxes and saturation humidity come from SurfaceFluxes.jl and
 * Thermodynamics.jl, which are not among the reference sources: they are
 * restated from the published formulations, and their parity is unpinned
 * (only the reference's identities around them are checked).
 */
#ifndef CLM_ORACLE_H
#define CLM_ORACLE_H

#include <stdint.h>
#include "../include/climaland_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct clmo_problem {
  clm_config cfg;          /* model, BC kinds, constants, Newton settings */
  int32_t ncol;
  const int32_t* offsets;  /* ncol + 1 */
  const double* z_lo;      /* ncol */
  const double* z_hi;      /* ncol */
  const double* params;    /* nparams x ncol */
  int32_t nparams;
  const double* forcing[4];/* CLM_F_NFIELDS x ncol per slot (NULL: zero)  */
  int32_t nthreads;        /* OpenMP threads (<= 0: library default)      */
  const double* root;      /* CLM_RX_NFIELDS x ncol root-extraction canopy
                              values (EnergyHydrology), or NULL            */
  const double* atmos;     /* CLM_AT_NFIELDS x ncol drivers of CLM_BC_ATMOS,
                              or NULL                                      */
  clm_atmos_params atm;    /* constants of CLM_BC_ATMOS                    */
  const double* z_faces;   /* face coordinates, column c's faces at
                              offsets[c] + c + j, j = 0..n (bottom to top):
                              a stretched column (Domains.jl:188-215 with
                              dz_tuple); NULL: n equal layers from z_lo to
                              z_hi                                         */
} clmo_problem;

/* ---- pointwise physics (names follow the reference functions) -------- */
double clmo_volumetric_liquid_fraction(double vartheta_l, double nu_eff,
                                       double theta_r);
double clmo_effective_saturation(double nu_eff, double vartheta_l,
                                 double theta_r);
double clmo_matric_potential(double alpha, double n, double m, double S);
double clmo_inverse_matric_potential(double alpha, double n, double m,
                                     double psi, int* psi_positive);
double clmo_pressure_head(double alpha, double n, double m, double theta_r,
                          double vartheta_l, double nu_eff, double S_s);
double clmo_dpsidvartheta(double alpha, double n, double m, double vartheta,
                          double nu_eff, double theta_r, double S_s);
double clmo_hydraulic_conductivity(double m, double K_sat, double S);
/* Brooks-Corey closure (soil_hydrology_parameterizations.jl:182-289) */
double clmo_bc_matric_potential(double c, double psib, double S);
double clmo_bc_inverse_matric_potential(double c, double psib, double psi,
                                        int* psi_positive);
double clmo_bc_pressure_head(double c, double psib, double theta_r,
                             double vartheta_l, double nu_eff, double S_s);
double clmo_bc_dpsidvartheta(double c, double psib, double vartheta,
                             double nu_eff, double theta_r, double S_s);
double clmo_bc_hydraulic_conductivity(double c, double K_sat, double S);
double clmo_impedance_factor(double f_i, double Omega);
/* canopy helpers of root extraction (src/standalone/Vegetation) */
double clmo_harmonic_mean(double x, double y);
double clmo_plant_water_flux(double z1, double z2, double psi1, double psi2,
                             double K1, double K2);
double clmo_weibull_conductivity(double K_sat, double psi63, double c,
                                 double psi);
double clmo_root_distribution(double z, double rooting_depth);
/* atmosphere-driven top boundary (CLM_BC_ATMOS) */
void clmo_atmos_params_default(clm_atmos_params* a);
/* The Monin-Obukhov solve at a fixed surface virtual potential temperature
 * (known-answer tests): out = zeta, F_m, F_h, g_h, u*; returns 0. */
int clmo_similarity(const clm_atmos_params* a, double grav, double dz, double U,
                    double z0m, double z0b, double thv_air, double thv_sfc,
                    double* out);
double clmo_gryanik_psi_m(double zeta, const clm_atmos_params* a);
double clmo_gryanik_psi_h(double zeta, const clm_atmos_params* a);
double clmo_q_vap_saturation(double T, double rho, int ice,
                             const clm_atmos_params* a,
                             const clm_earth_params* e);
double clmo_dry_soil_layer_thickness(double S_l, double aS_c, double d_ds,
                                     double p);
double clmo_soil_conductance(double S_l, double S_c, double d_ds, double p,
                             double alpha, double D_vapor);
double clmo_businger_psi_m(double zeta, const clm_atmos_params* a);
double clmo_businger_psi_h(double zeta, const clm_atmos_params* a);
/* the boundary's diagnostics (CLM_AF_NFIELDS x ncol) at a state */
int clmo_atmos_fluxes(const clmo_problem* P, const double* vartheta_l,
                      const double* theta_i, const double* rho_e_int,
                      double* out);
double clmo_viscosity_factor(double T, double gamma, double gamma_T_ref);
double clmo_heaviside(double x, double a);
double clmo_soil_Tf_depressed(double theta_l, double theta_i, double nu,
                              double theta_r, double alpha, double n,
                              double m, double rho_ice, double rho_liq,
                              double T_freeze, double grav, double LH_f0);
double clmo_thermal_time(double rhoc, double dz, double kappa);
double clmo_phase_change_source(double theta_l, double theta_i, double T,
                                double tau, double nu, double theta_r,
                                double alpha, double n, double m,
                                double rho_i, double rho_l, double LH_f0,
                                double T_freeze, double grav,
                                int* psi_positive);
double clmo_volumetric_heat_capacity(double theta_l, double theta_i,
                                     double rhoc_ds,
                                     const clm_earth_params* e);
double clmo_temperature_from_rho_e_int(double rho_e_int, double theta_i,
                                       double rhoc_s,
                                       const clm_earth_params* e);
double clmo_volumetric_internal_energy(double theta_i, double rhoc_s,
                                       double T, const clm_earth_params* e);
double clmo_volumetric_internal_energy_liq(double T,
                                           const clm_earth_params* e);
double clmo_kappa_sat(double theta_l, double theta_i, double k_unfrozen,
                      double k_frozen);
double clmo_thermal_conductivity(double kappa_dry, double K_e,
                                 double kappa_sat);
double clmo_relative_saturation(double theta_l, double theta_i, double nu);
double clmo_kersten_number(double theta_i, double S_r, double a, double b,
                           double nu_om, double nu_quartz, double nu_gravel);
double clmo_kappa_solid(double nu_om, double nu_quartz, double k_om,
                        double k_quartz, double k_minerals);
double clmo_kappa_sat_frozen(double kappa_solid, double nu, double kappa_ice);
double clmo_kappa_sat_unfrozen(double kappa_solid, double nu, double kappa_l);
double clmo_kappa_dry(double rho_p, double nu, double kappa_solid,
                      double kappa_air);
double clmo_forcing_value(const double* forcing, int32_t ncol, int32_t c,
                          double t, uint64_t seed, int64_t col0);

/* ---- closure level, whole batch --------------------------------------- *
 * State pointers: vartheta_l, theta_i, rho_e_int per cell; intF_w, intF_e
 * per column. theta_i / rho_e_int / intF_e are ignored for Richards. */

/* update_aux + update_boundary_fluxes at (state, t) (make_update_cache). */
/* runoff diagnostics of CLM_BC_PRECIP_RUNOFF (RichardsModel) */
int clmo_runoff(const clmo_problem* P, const double* vartheta_l, double t,
                double* infiltration, double* R_s, double* R_ss, double* h_sat);
int clmo_update_cache(const clmo_problem* P, const double* vartheta_l,
                      const double* theta_i, const double* rho_e_int,
                      double t, double* K, double* psi, double* theta_l,
                      double* T, double* kappa, double* Tf_depressed,
                      double* bc_fluxes, double* total_water,
                      double* total_energy);

/* exp_tendency (make_exp_tendency = update_cache + compute_exp_tendency). */
int clmo_exp_tendency(const clmo_problem* P, const double* vartheta_l,
                      const double* theta_i, const double* rho_e_int,
                      double t, double* dv, double* dti, double* de,
                      double* dFw, double* dFe);

/* compute_imp_tendency after update_cache at (state, t). */
int clmo_imp_tendency(const clmo_problem* P, const double* vartheta_l,
                      const double* theta_i, const double* rho_e_int,
                      double t, double* dv, double* dti, double* de,
                      double* dFw, double* dFe);

/* compute_jacobian after update_cache at (state, t); 3 values per cell. */
int clmo_jacobian(const clmo_problem* P, const double* vartheta_l,
                  const double* theta_i, const double* rho_e_int, double t,
                  double dtgamma, double* W_vv, double* W_ev, double* W_ee);

/* Block solve of W delta = f (BlockDiagonal / BlockLowerTriangular). */
int clmo_solve(const clmo_problem* P, const double* W_vv, const double* W_ev,
               const double* W_ee, const double* f_v, const double* f_e,
               double* delta_v, double* delta_e);

/* nsteps ARS111 steps from time t, in place. flags / iters per column may be
 * NULL. */
int clmo_step(const clmo_problem* P, double* vartheta_l, double* theta_i,
              double* rho_e_int, double* intF_w, double* intF_e, double t,
              double dt, int32_t nsteps, uint32_t* flags, int32_t* iters);

/* Column budgets of a state (column_integral_definite!). */
int clmo_budgets(const clmo_problem* P, const double* vartheta_l,
                 const double* theta_i, const double* rho_e_int,
                 double* total_water, double* total_energy);

#ifdef __cplusplus
}
#endif
#endif
