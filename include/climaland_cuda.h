/*
 * libclimaland_cuda — C ABI of the GB300 (sm_103a) soil column step.
 *
 * The library replaces, for one device, the model closures that ClimaLand
 * hands to ClimaTimeSteppers for a soil column model (RichardsModel or
 * EnergyHydrology) and the IMEX ARS111 + Newton step that drives them.
 * Every entry point below names the reference interface it stands in for
 * (paths relative to the ClimaLand.jl source tree).
 *
 * Conventions
 *  - All functions return an int status (CLM_OK = 0) and never abort, trap
 *    or throw across the ABI. clm_last_error() gives a readable message.
 *  - Host buffers are owned by the caller and copied in/out. Device buffers
 *    are owned by the handle.
 *  - Cell arrays use the reference's column layout: cell index =
 *    offsets[c] + k, level k = 0 is the bottom layer (ClimaCore level 1),
 *    levels contiguous within a column (ClimaCore VIJFH/VF "level fastest").
 *    For uniform columns offsets[c] = c * nlayers.
 *  - Per-column parameter blocks are structure-of-arrays: params[p*ncol + c].
 *  - One handle per host thread; each handle owns one CUDA stream.
 *    Calls are synchronous unless the _async form is used.
 */
#ifndef CLIMALAND_CUDA_H
#define CLIMALAND_CUDA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define CLM_OK 0
#define CLM_ERR_ARG 1         /* invalid argument (size, pointer, enum)    */
#define CLM_ERR_CUDA 2        /* a CUDA runtime call failed                */
#define CLM_ERR_TIMEOUT 3     /* a bounded device-side wait gave up        */
#define CLM_ERR_NAN 4         /* non-finite state detected (per-col flags) */
#define CLM_ERR_STATE 5       /* call order (e.g. step before set_state)   */
#define CLM_ERR_UNSUPPORTED 6 /* option not built in this library          */

/* ---- per-column status flags (clm_get_status) ------------------------ */
#define CLM_COL_NONFINITE 0x1u     /* NaN/Inf in the column state          */
#define CLM_COL_DIVERGED 0x2u      /* Newton increment norm grew           */
#define CLM_COL_NOT_CONVERGED 0x4u /* tolerance mode hit max_iters         */
#define CLM_COL_GUESS_FALLBACK 0x8u /* learned guess rejected, zero guess  */
#define CLM_COL_PSI_POSITIVE 0x10u /* inverse_matric_potential got psi > 0 */

/* ---- enums ------------------------------------------------------------ */
enum clm_model {
  CLM_MODEL_RICHARDS = 0,         /* src/standalone/Soil/rre.jl:67        */
  CLM_MODEL_ENERGY_HYDROLOGY = 1  /* src/standalone/Soil/energy_hydrology.jl:226 */
};

enum clm_precision {
  CLM_PREC_FP64 = 0,  /* plain path: everything in FP64 (drop-in)         */
  CLM_PREC_MIXED = 1  /* FP32 Jacobian + Thomas; FP64 residual, increment
                         accumulation, phase partition and budgets        */
};

enum clm_newton_mode {
  CLM_NEWTON_FIXED = 0, /* max_iters iterations, no convergence check
                           (Simulations.jl:127-135 default: 3)            */
  CLM_NEWTON_TOL = 1    /* stop when the column increment 2-norm is below
                           newton_tol (CTS MaximumError on the norm)       */
};

/* Newton starting point in tolerance mode (clm_config.learned_guess).
 * No reference counterpart: the reference starts every solve from U.
 * NETWORK: u_n plus the column's previous step increment plus the change
 *   the loaded network predicts (clm_load_mlp; one guess launch per step).
 * EXTRAPOLATE: u_n plus the previous step increment, computed inside the
 *   step kernel (no network, no extra launch); the handle keeps the state
 *   at the previous step's start, initialised at the first step call.
 * Both restart from U where the first Newton increment exceeds ten times
 * the guessed one, or where Newton from the guess stops contracting
 * (CLM_COL_GUESS_FALLBACK). */
enum clm_guess { CLM_GUESS_NONE = 0, CLM_GUESS_NETWORK = 1, CLM_GUESS_EXTRAPOLATE = 2 };

/* Tile order of the persistent step kernel (no reference counterpart: a
 * launch-configuration choice). Tiles of 32 columns are sorted deepest
 * first; results do not depend on the order. */
enum clm_schedule {
  CLM_SCHED_STATIC = 0,  /* warp w takes tiles w, w + W, w + 2W, ...        */
  CLM_SCHED_DYNAMIC = 1  /* warps claim the next tile from an atomic counter */
};

/* How tolerance-mode Newton maps columns to warps (clm_config.tol_regroup;
 * no reference counterpart: a scheduling choice). A warp runs its 32
 * columns in lockstep, as many iterations as its slowest column needs.
 * Results do not depend on the choice (the same arithmetic per column). */
enum clm_tol_schedule {
  CLM_TOL_TILES = 0,    /* the depth-sorted tiles                           */
  CLM_TOL_REGROUP = 1,  /* slots re-sorted after every step by the column's
                           last iteration count (without a Newton guess;
                           with one, the tiles)                             */
  CLM_TOL_SPLIT = 2,    /* EnergyHydrology: every step is two launches; the
                           first runs every column through two iterations,
                           the second finishes the columns that have not
                           converged, packed 32 to a warp in a queue the
                           handle keeps (about 96 n + 136 bytes per column
                           of n layers); RichardsModel: the tiles           */
  CLM_TOL_AUTO = 3      /* (default) CLM_TOL_REGROUP for FP64 without a
                           Newton guess and for RichardsModel, otherwise
                           CLM_TOL_SPLIT (each measured the faster there)   */
};

/* Boundary-condition kinds (src/standalone/Soil/boundary_conditions.jl). */
enum clm_bc_kind {
  CLM_BC_FLUX = 0,            /* WaterFluxBC / HeatFluxBC: F = f(t)        */
  CLM_BC_FREE_DRAINAGE = 1,   /* FreeDrainage (water, bottom): F = -K_1;
                                 as heat BC: EnergyWaterFreeDrainage
                                 F_e = -K_1 rho e_liq(T_1)                 */
  CLM_BC_STATE = 2,           /* MoistureStateBC / TemperatureStateBC      */
  CLM_BC_FLUX_ADVECTIVE = 3,  /* heat only: F_e = f(t) + F_w,top(t) *
                                 rho e_liq(T_adv), T_adv per column        */
  CLM_BC_PRECIP_RUNOFF = 4,   /* water, top, RichardsModel:
                                 RichardsAtmosDrivenFluxBC
                                 (boundary_conditions.jl:64-100, :200-212):
                                 the top-water forcing row is the liquid
                                 precipitation P(t) (< 0 into the soil),
                                 cfg->runoff turns it into the infiltration
                                 flux at the explicit stage               */
  CLM_BC_ATMOS = 5            /* water and heat, top, EnergyHydrology:
                                 AtmosDrivenFluxBC with a prescribed
                                 atmosphere and radiation, standalone soil
                                 (boundary_conditions.jl:610-677, 870-936):
                                 the drivers of clm_set_atmos; both top
                                 kinds must be CLM_BC_ATMOS; cfg->runoff
                                 splits P_liq (EnergyHydrology forms of
                                 Runoff.jl: infiltration capacity
                                 -K_sat impedance viscosity at the top,
                                 saturation with ice, and TOPMODEL's
                                 subsurface water and energy sink)        */
};

/* Per-column parameter rows for clm_set_params (SoA, row p of ncol). The
 * first CLM_NPARAM_RICHARDS rows are RichardsParameters (rre.jl:7-21); all
 * CLM_NPARAM_EH rows are the per-point EnergyHydrologyParameters
 * (energy_hydrology.jl:21-78). */
/* Runoff model of CLM_BC_PRECIP_RUNOFF and CLM_BC_ATMOS
 * (src/standalone/Soil/Runoff/Runoff.jl). */
enum clm_runoff {
  CLM_RUNOFF_NONE = 0,     /* NoRunoff: infiltration = P (:56-80)            */
  CLM_RUNOFF_SURFACE = 1,  /* SurfaceRunoff: (1 - H(theta_top - nu)) max(-K_sat, P)
                              (:85-145)                                      */
  CLM_RUNOFF_TOPMODEL = 2  /* TOPMODELRunoff (:198-270, :373-440): h_sat = sum dz
                              H(vartheta - nu) (vartheta - theta_r)/(nu - theta_r),
                              f_sat = min(f_max exp(-f_over z_wt / 2), 1),
                              infiltration (1 - f_sat) max(-K_sat, P), and the
                              TOPMODELSubsurfaceRunoff sink (:321-345) of
                              R_ss = R_sb exp(-f_over z_wt) spread over the
                              saturated layers, z_wt = depth - h_sat        */
};

/* Hydrology closure (src/standalone/Soil/retention_models.jl): how rows
 * 4 and 5 of the parameters are read. */
enum clm_hydrology_cm {
  CLM_CM_VAN_GENUCHTEN = 0, /* vanGenuchten{FT}(; alpha, n) (:354-368)          */
  CLM_CM_BROOKS_COREY = 1   /* BrooksCorey{FT}(; c, psi_b) (:47-67):
                               psi = psi_b S^(-1/c), K = K_sat S^(2/c + 3)
                               (soil_hydrology_parameterizations.jl:182-289) */
};

enum clm_param {
  CLM_P_NU = 0,            /* porosity nu                                 */
  CLM_P_K_SAT = 1,         /* saturated hydraulic conductivity (m/s)      */
  CLM_P_S_S = 2,           /* specific storativity (1/m)                  */
  CLM_P_THETA_R = 3,       /* residual water fraction                     */
  CLM_P_VG_ALPHA = 4,      /* van Genuchten alpha (1/m)                   */
  CLM_P_VG_N = 5,          /* van Genuchten n                             */
  CLM_P_BC_PSI_B = 4,      /* Brooks-Corey psi_b (m, < 0)                 */
  CLM_P_BC_C = 5,          /* Brooks-Corey c (> 0)                        */
  CLM_NPARAM_RICHARDS = 6,
  CLM_P_KAPPA_DRY = 6,          /* W/m/K                                   */
  CLM_P_KAPPA_SAT_FROZEN = 7,   /* W/m/K                                   */
  CLM_P_KAPPA_SAT_UNFROZEN = 8, /* W/m/K                                   */
  CLM_P_RHOC_DS = 9,            /* J/m^3/K                                 */
  CLM_P_NU_SS_OM = 10,
  CLM_P_NU_SS_QUARTZ = 11,
  CLM_P_NU_SS_GRAVEL = 12,
  CLM_NPARAM_EH = 13,
  /* TOPMODEL rows (CLM_RUNOFF_TOPMODEL; the reference's f_over and R_sb are
   * scalars, f_max a surface field) */
  CLM_P_F_MAX = 13,        /* maximum saturated fraction                      */
  CLM_P_F_OVER = 14,       /* 1/m                                             */
  CLM_P_R_SB = 15,         /* m/s                                             */
  CLM_NPARAM_MAX = 16
};

/* Forcing descriptor rows for clm_set_bc (SoA, row f of ncol). A boundary
 * value at time t for column c (original index) is
 *   base + amp * sin(omega * t + phase)
 *        + pulse_amp * [u(seed, c, floor(t / pulse_period)) < pulse_duty]
 * with u() the counter hash clm_forcing_hash01 below (pulse term off when
 * pulse_period <= 0). For CLM_BC_FLUX_ADVECTIVE row CLM_F_T_ADV is the
 * temperature carried by the top water flux. This replaces the reference's
 * Julia closure bc(p, t) (boundary_conditions.jl:168-180, 465-477), which
 * cannot cross a C ABI. */
enum clm_forcing_field {
  CLM_F_BASE = 0,
  CLM_F_AMP = 1,
  CLM_F_OMEGA = 2,
  CLM_F_PHASE = 3,
  CLM_F_PULSE_AMP = 4,
  CLM_F_PULSE_PERIOD = 5,
  CLM_F_PULSE_DUTY = 6,
  CLM_F_T_ADV = 7,
  CLM_F_NFIELDS = 8
};

/* Which boundary value clm_set_bc addresses. */
enum clm_bc_slot {
  CLM_BC_TOP_WATER = 0,
  CLM_BC_TOP_HEAT = 1,
  CLM_BC_BOTTOM_WATER = 2,
  CLM_BC_BOTTOM_HEAT = 3
};

/* Root extraction (EnergyHydrology with the RootExtraction source:
 * src/integrated/soil_canopy_root_interactions.jl:8-39, 139-159). Per-column
 * canopy values for clm_set_root_extraction (SoA, row f of ncol), held by
 * the caller's canopy model and frozen through a step. Each layer at centre
 * z loses (explicit stage)
 *   re = hm(LAI, RAI) water_flux(z, h/2, psi_soil, psi_canopy, K_soil,
 *        K_canopy(psi_canopy)) root_distribution(z, rooting_depth)     (1/s)
 * with hm(x, y) = x y / max(x + y, eps), water_flux = -hm(K1, K2) ((psi2 -
 * psi1) / (z2 - z1) + 1) (plant_hydraulics.jl:170, 197-201), the Weibull
 * conductivity K_sat exp(-(psi / psi63)^c) for psi <= 0, K_sat otherwise
 * (:256-267), root_distribution = exp(z / d) / d (biomass.jl:362-364), and
 * psi_soil, K_soil, T_soil the update_aux values at the step's start; rho e_int
 * loses re rho c_l (T_soil - T_0). As in the reference, the integrated fluxes
 * gain the column integrals of both (d intF_w += sum dz re, d intF_e += sum dz
 * re rho e_l): the reference adds the water extraction to intF_w with the
 * sign opposite to the state's change, so its water budget drifts by
 * 2 dt sum dz re per step; the library reproduces that. */
enum clm_root_field {
  CLM_RX_PSI_CANOPY = 0,  /* p.canopy.hydraulics.psi (m)                    */
  CLM_RX_LAI = 1,         /* leaf area index                                */
  CLM_RX_RAI = 2,         /* root area index                                */
  CLM_RX_HEIGHT = 3,      /* canopy height (m); the flux runs to h / 2      */
  CLM_RX_ROOT_DEPTH = 4,  /* rooting depth (m)                              */
  CLM_RX_K_SAT = 5,       /* Weibull K_sat of the plant (m/s)               */
  CLM_RX_PSI63 = 6,       /* Weibull psi63 (m, < 0)                         */
  CLM_RX_WEIBULL_C = 7,   /* Weibull c (> 0)                                */
  CLM_RX_NFIELDS = 8
};

/* Atmosphere-driven top boundary (CLM_BC_ATMOS). Per-column drivers and
 * surface parameters for clm_set_atmos (SoA, row f of ncol), frozen through
 * a step (the reference refreshes its drivers in a callback between steps).
 * At the explicit stage, from the update_aux values of the top layer:
 *   T_sfc = T_top, q_sfc from q_vap_saturation(T_sfc, rho_sfc) (liquid,
 *   times exp(g min(psi_top, 0) M_w / (R T_sfc)), when T_sfc > Tf_depressed_top;
 *   else ice) (energy_hydrology.jl:995-1060); the soil's vapour conductance
 *   D_vapor / max(dsl, eps) from the surface liquid fraction linearly
 *   extrapolated from the top two centres (:1062-1145, 1322-1368,
 *   Domains.jl:883-895); CLMTwoBandSoilAlbedo over the top
 *   ALBEDO_TOP_THICKNESS (soil_albedo.jl:146-198); net radiation
 *   -(1 - alpha) SW_d - eps (LW_d - sigma T_sfc^4) (drivers.jl:699-716);
 *   turbulent fluxes by Monin-Obukhov similarity (see clm_atmos_params);
 *   top water flux = infiltration + E / rho_l (liquid part), top energy flux =
 *   R_n + LHF + SHF + infiltration rho e_liq(T_air), the infiltration P_liq
 *   or, with cfg->runoff, its infiltrating part (boundary_conditions.jl:
 *   908-936, 988-1003); the sublimation part of E leaves theta_i of the
 *   layers with z + 2 dz_top > eps (the top layer for a surface at z = 0) and
 *   enters intF_w (SoilSublimation, energy_hydrology.jl:910-947). */
enum clm_atmos_field {
  CLM_AT_P_LIQ = 0,              /* liquid precipitation (m/s, < 0 downward)  */
  CLM_AT_T_AIR = 1,              /* air temperature (K)                       */
  CLM_AT_U_AIR = 2,              /* wind speed (m/s)                          */
  CLM_AT_Q_AIR = 3,              /* specific humidity (kg/kg)                 */
  CLM_AT_P_AIR = 4,              /* air pressure (Pa)                         */
  CLM_AT_SW_D = 5,               /* downwelling shortwave (W/m^2)             */
  CLM_AT_LW_D = 6,               /* downwelling longwave (W/m^2)              */
  CLM_AT_H_AIR = 7,              /* height of the atmospheric values (m)      */
  CLM_AT_GUSTINESS = 8,          /* gustiness (m/s): minimum wind speed       */
  CLM_AT_PAR_ALBEDO_DRY = 9,
  CLM_AT_NIR_ALBEDO_DRY = 10,
  CLM_AT_PAR_ALBEDO_WET = 11,
  CLM_AT_NIR_ALBEDO_WET = 12,    /* ConstantTwoBandSoilAlbedo: dry = wet      */
  CLM_AT_ALBEDO_TOP_THICKNESS = 13, /* m (CLMTwoBandSoilAlbedo default 0.02) */
  CLM_AT_EMISSIVITY = 14,
  CLM_AT_Z_0M = 15,              /* momentum roughness length (m)             */
  CLM_AT_Z_0B = 16,              /* scalar roughness length (m)               */
  CLM_AT_D_DS = 17,              /* maximum dry soil layer depth (m)          */
  CLM_AT_EVAP_P = 18,            /* evaporation exponent                      */
  CLM_AT_EVAP_ALPHA = 19,        /* evaporation scalar                        */
  CLM_AT_NFIELDS = 20
};

/* Universal functions of the similarity solve (clm_atmos_params). */
enum clm_universal_functions {
  CLM_UF_BUSINGER = 0, /* Businger-Dyer on both sides of neutral (Businger et
                          al. 1971; Paulson 1970 integral forms)            */
  CLM_UF_GRYANIK = 1   /* the reference's UF.GryanikParams
                          (src/shared_utilities/Parameters.jl:83): Gryanik
                          et al. (2020) on the stable side, Businger-Dyer on
                          the unstable side; the default                   */
};

/* Constants of the atmosphere-driven boundary (ClimaParams names). The
 * turbulent fluxes follow Monin-Obukhov similarity theory at point values
 * (as restated here from the published formulations, since SurfaceFluxes.jl
 * is not part of the reference sources):
 *   U = max(|u|, gustiness), dz = h_air, zeta = dz / L_MO,
 *   F_m = ln(dz/z_0m) - psi_m(zeta) + psi_m(zeta z_0m/dz),
 *   F_h = Pr_0 (ln(dz/z_0b) - psi_h(zeta) + psi_h(zeta z_0b/dz)),
 *   unstable (zeta < 0), Businger-Dyer:
 *   psi_m = 2 ln((1+x)/2) + ln((1+x^2)/2) - 2 atan x + pi/2, x = (1 - b_m zeta)^(1/4),
 *   psi_h = 2 ln((1+y)/2), y = (1 - b_h zeta)^(1/2);
 *   stable (zeta >= 0), Businger-Dyer: psi_m = -a_m zeta, psi_h = -a_h zeta / Pr_0;
 *   stable, Gryanik et al. (2020), phi_m = 1 + a_m zeta / (1 + gb_m zeta)^(2/3),
 *   phi_h = Pr_0 (1 + a_h zeta / (1 + gb_h zeta)):
 *   psi_m = -3 a_m / gb_m ((1 + gb_m zeta)^(1/3) - 1),
 *   psi_h = -a_h / gb_h ln(1 + gb_h zeta) (gb_m, gb_h: gryanik_b_m, gryanik_b_h);
 *   u* = kappa U / F_m, g_h = kappa u* / F_h; at most `iterations` steps from
 *   zeta = 0 (a column stops once a step moves zeta by <= 1e-12 (1 + |zeta|)),
 *   each re-evaluating F_m, F_h, g_h, q_sfc and
 *   Ri_b = g dz (theta_v,air - theta_v,sfc) / (theta_v,sfc U^2), then solving
 *   zeta F_h(zeta) = Ri_b F_m(zeta)^2 for the next zeta: for Ri_b >= 0 with
 *   Businger-Dyer exactly (a quadratic with the linear stable functions;
 *   zeta_max above the critical Richardson number), otherwise by a Newton
 *   step at fixed Ri_b (the first unstable one from Ri_b ln(dz/z_0m)^2 /
 *   (Pr_0 ln(dz/z_0b))), clamped to [-zeta_max, 0] or [0, zeta_max];
 *   theta_v,air = (T_air + g dz / cp_d)(1 + (R_v/R_d - 1) q_air),
 *   theta_v,sfc = T_sfc (1 + (R_v/R_d - 1) q_sfc), and q_sfc from g_h by the
 *   reference's update_q_vap_sfc_at_a_point
 *   (energy_hydrology.jl:1066-1099). Then
 *   E = -rho_sfc g_h (q_air - q_sfc), LHF = LH_v0 E,
 *   SHF = -rho_sfc cp_m g_h (T_air + g dz / cp_m - T_sfc),
 *   rho_sfc = rho_air (T_sfc / T_air)^(cv_m / R_m), rho_air = P / (R_m T_air). */
typedef struct clm_atmos_params {
  double stefan;          /* Stefan-Boltzmann constant (W/m^2/K^4)         */
  double gas_constant;    /* J/mol/K                                       */
  double molmass_dryair;  /* kg/mol                                        */
  double molmass_water;   /* kg/mol                                        */
  double D_vapor;         /* diffusivity of water vapour in air (m^2/s)    */
  double LH_v0, LH_s0;    /* latent heats at T_0 (J/kg)                    */
  double cp_d, cp_v;      /* isobaric specific heats (J/kg/K)              */
  double T_triple;        /* K                                             */
  double press_triple;    /* Pa                                            */
  double von_karman;
  double Pr_0, a_m, a_h;  /* Pr_0 and the stable-side a_m, a_h            */
  double b_m, b_h;        /* unstable-side Businger-Dyer b_m, b_h          */
  double zeta_max;        /* |zeta| bound of the iteration                 */
  int32_t iterations;     /* similarity iterations (>= 1; default 8)       */
  int32_t universal_functions; /* enum clm_universal_functions             */
  double gryanik_b_m, gryanik_b_h; /* stable-side b_m, b_h of CLM_UF_GRYANIK */
} clm_atmos_params;

/* Diagnostics of clm_atmos_fluxes (row f of ncol): the reference's
 * p.soil.turbulent_fluxes, R_n, q_sfc and top_bc at the current state. */
enum clm_atmos_flux {
  CLM_AF_LHF = 0, CLM_AF_SHF = 1, CLM_AF_VAPOR_LIQ = 2, CLM_AF_VAPOR_ICE = 3,
  CLM_AF_R_N = 4, CLM_AF_Q_SFC = 5, CLM_AF_TOP_WATER = 6, CLM_AF_TOP_HEAT = 7,
  CLM_AF_NFIELDS = 8
};

/* Physical constants (ClimaLand.Parameters.LandParameters,
 * src/shared_utilities/Parameters.jl:11-115). The Julia caller passes the
 * values of its own earth_param_set; clm_config_default fills ClimaParams
 * defaults. */
typedef struct clm_earth_params {
  double rho_l;    /* density_liquid_water (kg/m^3)                     */
  double rho_i;    /* density_ice_water (kg/m^3)                        */
  double cp_l;     /* isobaric_specific_heat_liquid (J/kg/K)            */
  double cp_i;     /* isobaric_specific_heat_ice (J/kg/K)               */
  double T_0;      /* thermodynamics_temperature_reference (K)          */
  double T_freeze; /* temperature_water_freeze (K)                      */
  double LH_f0;    /* LH_s0 - LH_v0 (J/kg), Parameters.jl:58            */
  double grav;     /* gravitational_acceleration (m/s^2)                */
} clm_earth_params;

typedef struct clm_config {
  int32_t model;          /* enum clm_model                                */
  int32_t ncol;           /* number of columns                             */
  int32_t nlayers;        /* >0: every column has nlayers layers;
                             0: per-column counts from clm_set_geometry    */
  int32_t precision;      /* enum clm_precision                            */
  int32_t newton_mode;    /* enum clm_newton_mode                          */
  int32_t max_iters;      /* Newton iterations (fixed) or cap (tolerance)  */
  double newton_tol;      /* tolerance-mode threshold                      */
  double energy_norm_scale; /* weight of rho e_int in the tolerance norm   */
  int32_t learned_guess;  /* enum clm_guess: where tolerance-mode Newton
                             starts (EnergyHydrology)                      */
  int32_t bc_top_water, bc_top_heat, bc_bottom_water, bc_bottom_heat;
  /* scalar EnergyHydrologyParameters (energy_hydrology.jl:44-61) */
  double kersten_alpha, kersten_beta, ice_impedance_omega;
  double visc_gamma, visc_gamma_T_ref;
  clm_earth_params earth;
  int32_t phase_change;   /* 1: PhaseChange source (energy_hydrology.jl:822)
                             in the explicit tendency (EnergyHydrology)    */
  int32_t pad0;
  uint64_t forcing_seed;  /* seed of the rain-pulse hash                   */
  int32_t cols_per_cta;   /* 0: default (32); clm_autotune may change it   */
  int32_t schedule;       /* enum clm_schedule; clm_autotune may change it  */
  int32_t graph;          /* 1: clm_step / clm_step_async replay their launch
                             sequence as CUDA graphs captured on first use
                             (t and dt go through a device array, so one
                             graph serves every call with the same nsteps) */
  int32_t hydrology_cm;   /* enum clm_hydrology_cm                          */
  int64_t column_offset;  /* global index of this handle's column 0 when a
                             domain is split across handles or GPUs: the
                             rain-pulse hash uses the global column index  */
  int32_t host_chunks;    /* clm_step_host pipeline depth (0: by size)      */
  int32_t runoff;         /* enum clm_runoff (CLM_BC_PRECIP_RUNOFF)         */
  int32_t tol_regroup;    /* enum clm_tol_schedule: how tolerance-mode
                             Newton maps columns to warps (default
                             CLM_TOL_AUTO). CLM_TOL_REGROUP keeps the
                             depth-sorted tiles when a Newton guess is set
                             (learned_guess != 0): the guess makes the last
                             count a poor predictor and the regrouped warps'
                             scattered loads cost more than they save.
                             Results do not depend on it                    */
  int32_t pad1;
} clm_config;

typedef struct clm_handle clm_handle;

/* Fill `cfg` with defaults: EnergyHydrology, FP64, fixed 3 Newton
 * iterations (Simulations.jl:127-135), flux top / free-drainage bottom,
 * Kersten alpha 0.24, beta 18.3, Omega 7, gamma 2.64e-2, gamma_T_ref 288
 * (test/standalone/Soil/soil_parameterizations.jl:71-75). */
void clm_config_default(clm_config* cfg);

/* Replaces LandSimulation's model set-up (Simulations.jl:115-245) and
 * initialize(model) (models.jl:493-499): allocates the device state. */
int clm_create(const clm_config* cfg, clm_handle** out);
void clm_destroy(clm_handle* h);
const char* clm_last_error(const clm_handle* h);

/* Column geometry (Domains.jl:183-247 Column, get_Δz :935-949): column c
 * spans [z_lo[c], z_hi[c]] with uniform layers; offsets (ncol+1 entries,
 * may be NULL when cfg->nlayers > 0) give the per-column layer counts. */
int clm_set_geometry(clm_handle* h, const double* z_lo, const double* z_hi,
                     const int32_t* offsets);

/* Per-layer geometry of stretched columns. Replaces the mesh of
 * Column(; zlim, nelements, dz_tuple) (Domains.jl:188-215: ClimaCore's
 * GeneralizedExponentialStretching, reverse_mode) and of the 3-D domains
 * built on it (global_domain's default dz_tuple = (10.0, 0.05), Domains.jl:
 * 1292-1298): z_faces holds each column's n + 1 face coordinates, bottom to
 * top, column c's at offsets[c] + c + j (the layout of a ClimaCore face
 * field: parent(coordinate_field(face_space).z) for a column space). The
 * library derives what ClimaCore's grid and get_Δz (:935-949) derive from
 * them: centres at the faces' midpoints, layer widths (divergence, column
 * integrals, thermal_time), centre spacings (gradients), Δz_top and
 * Δz_bottom (state boundary conditions, the atmosphere-driven boundary),
 * and sets z_lo / z_hi to the first and last face. Call after
 * clm_set_geometry (which returns the handle to uniform layers); NULL
 * returns to uniform layers. Faces must be finite and increasing. */
int clm_set_faces(clm_handle* h, const double* z_faces);

/* Per-column parameters, nparams rows of ncol (enum clm_param). Replaces
 * RichardsParameters / EnergyHydrologyParameters fields. */
int clm_set_params(clm_handle* h, const double* soa_params, int32_t nparams);

/* Boundary forcing for one slot, CLM_F_NFIELDS rows of ncol. Replaces the
 * bc closures evaluated by boundary_flux! (boundary_conditions.jl:168-608). */
int clm_set_bc(clm_handle* h, int32_t slot, const double* soa_forcing,
               int32_t nfields);

/* Root-extraction canopy values, CLM_RX_NFIELDS rows of ncol (enum
 * clm_root_field), or NULL to remove the source. Replaces the RootExtraction
 * source and update_root_extraction! (soil_canopy_root_interactions.jl:8-39,
 * 123-159). EnergyHydrology only (the reference defines the source for it
 * alone); the caller refreshes the values when its canopy state changes. */
int clm_set_root_extraction(clm_handle* h, const double* soa, int32_t nfields);

/* Drivers of the atmosphere-driven top boundary (CLM_BC_ATMOS): constants
 * `prm` (NULL: clm_atmos_params_default) and CLM_AT_NFIELDS x ncol values
 * (host pointer, SoA). Replaces the reference's update_drivers! of the
 * PrescribedAtmosphere / PrescribedRadiativeFluxes (drivers.jl) for the
 * soil; call again whenever the drivers change. soa = NULL removes them. */
void clm_atmos_params_default(clm_atmos_params* prm);
int clm_set_atmos(clm_handle* h, const clm_atmos_params* prm, const double* soa,
                  int32_t nfields);

/* The boundary's diagnostics at the current state (turbulent_fluxes!,
 * net_radiation!, component_specific_humidity, top_bc:
 * boundary_conditions.jl:908-936): CLM_AF_NFIELDS x ncol doubles written to
 * the host pointer `out` (SoA, original column order). */
int clm_atmos_fluxes(clm_handle* h, double* out, int32_t nfields);

/* Prognostic state Y.soil (energy_hydrology.jl:624-625, rre.jl:282).
 * theta_i, rho_e, intF_e may be NULL for RichardsModel. */
int clm_set_state(clm_handle* h, const double* vartheta_l,
                  const double* theta_i, const double* rho_e_int,
                  const double* intF_w, const double* intF_e);
int clm_get_state(clm_handle* h, double* vartheta_l, double* theta_i,
                  double* rho_e_int, double* intF_w, double* intF_e);

/* Same, with device pointers (caller-owned CuArray memory, reference
 * layout). Copies device-to-device on the handle's stream. */
int clm_set_state_device(clm_handle* h, const double* vartheta_l,
                         const double* theta_i, const double* rho_e_int,
                         const double* intF_w, const double* intF_e);
int clm_get_state_device(clm_handle* h, double* vartheta_l, double* theta_i,
                         double* rho_e_int, double* intF_w, double* intF_e);

/* Advance nsteps ARS111 steps of size dt from time t. Replaces
 * step!(landsim) (Simulations.jl:312-314) -> ClimaTimeSteppers IMEX ARS111
 * with NewtonsMethod (Simulations.jl:127-135) calling the closures
 * make_exp_tendency (models.jl:279-287), make_compute_imp_tendency,
 * make_compute_jacobian (rre.jl:161-458, energy_hydrology.jl:315-576),
 * make_update_implicit_cache (models.jl:238-246) and the block solve
 * selected in initialize_jacobian (implicit_timestepping.jl:63-172). */
int clm_step(clm_handle* h, double t, double dt, int32_t nsteps);
int clm_step_async(clm_handle* h, double t, double dt, int32_t nsteps);
int clm_sync(clm_handle* h);

/* Host-buffer step: the state in host memory (reference layout, updated in
 * place; pinned memory lets the copies overlap) is copied in, advanced
 * nsteps and copied back, pipelined over chunks of columns so that each
 * chunk's copies overlap the kernels of its neighbours. Replaces
 * step!(landsim) (Simulations.jl:312-314) for a host-resident Y.soil; the
 * same bits as clm_set_state + clm_step + clm_get_state (which it becomes,
 * without the overlap, when columns are not already in depth order or a
 * Newton guess is set: learned_guess != 0). With split Newton each chunk
 * runs the two launches of every step. */
int clm_step_host(clm_handle* h, double* vartheta_l, double* theta_i, double* rho_e_int,
                  double* intF_w, double* intF_e, double t, double dt, int32_t nsteps);

/* Launch-configuration autotuner (no reference counterpart; ClimaLand's
 * broadcasts are configured by ClimaCore). Times the step kernel on
 * probe_steps steps (1-64) from the handle's current state at time t, for
 * every columns-per-CTA (32 x warps, 1-4 warps that fit the shared memory)
 * and tile order, restores the state, flags and iteration counts, and keeps
 * the fastest configuration. `table` (may be NULL) receives up to
 * table_cap entries; *n_entries the number of candidates timed. */
typedef struct clm_tune_entry {
  int32_t cols_per_cta;   /* 32 x warps per CTA                            */
  int32_t schedule;       /* enum clm_schedule                              */
  int32_t grid;           /* resident CTAs (persistent grid)                */
  int32_t chosen;         /* 1 for the configuration kept                   */
  double ms_per_step;     /* CUDA-event time of the probe / probe_steps     */
} clm_tune_entry;
int clm_autotune(clm_handle* h, double t, double dt, int32_t probe_steps,
                 clm_tune_entry* table, int32_t table_cap, int32_t* n_entries);

/* The step kernel's current launch configuration. */
int clm_get_launch_config(const clm_handle* h, int32_t* cols_per_cta, int32_t* schedule,
                          int32_t* grid);

/* Run the handle's work on a caller-owned cudaStream_t (NULL restores the
 * handle's own stream). No reference counterpart: it lets a host that owns
 * the CUDA context (CUDA.jl, PyTorch) order and time the library's kernels
 * on its own stream. */
int clm_set_stream(clm_handle* h, void* cuda_stream);

/* Column budgets total_water / total_energy (rre.jl:502-511,
 * energy_hydrology.jl:1282-1320) of the current state, per column. */
int clm_get_budgets(clm_handle* h, double* total_water, double* total_energy);

/* Per-column status flags (CLM_COL_*, OR-ed over every step of the last
 * step call) and Newton iteration counts (of that call's last step); either
 * pointer may be NULL. Stands in for NaNCheckCallback (utils.jl:684-694). */
int clm_get_status(clm_handle* h, uint32_t* flags, int32_t* newton_iters);

/* ---- closure-level entry points (for parity of each closure) ---------
 * All operate on the handle's current state at time t; outputs are host
 * buffers in the reference layout. */

/* make_update_aux (rre.jl:368-380; energy_hydrology.jl:722-814) followed
 * by make_update_boundary_fluxes (rre.jl:111-149;
 * energy_hydrology.jl:273-298). Outputs per cell: K, psi and, for
 * EnergyHydrology, theta_l, T, kappa, Tf_depressed (NULL to skip); per
 * column: top/bottom water and heat fluxes (bc[4*ncol], slot-major). */
int clm_update_aux(clm_handle* h, double t, double* K, double* psi,
                   double* theta_l, double* T, double* kappa,
                   double* Tf_depressed, double* bc_fluxes);

/* make_exp_tendency (models.jl:279-287): update_aux + boundary fluxes +
 * compute_exp_tendency! (rre.jl:214-243; energy_hydrology.jl:315-350 with
 * the PhaseChange source :838-906). Outputs dY in the state layout. */
int clm_exp_tendency(clm_handle* h, double t, double* d_vartheta_l,
                     double* d_theta_i, double* d_rho_e_int, double* d_intF_w,
                     double* d_intF_e);

/* make_compute_imp_tendency (rre.jl:161-203; energy_hydrology.jl:363-425)
 * evaluated after make_update_cache at (state, t). */
int clm_imp_tendency(clm_handle* h, double t, double* d_vartheta_l,
                     double* d_theta_i, double* d_rho_e_int, double* d_intF_w,
                     double* d_intF_e);

/* make_compute_jacobian (rre.jl:391-458; energy_hydrology.jl:466-576)
 * after make_update_cache at (state, t): tridiagonal blocks
 * W = dtgamma * dT/dY - I, each 3 values per cell (lower, diag, upper):
 * W_vv (d vartheta / d vartheta), W_ev (d rho_e / d vartheta), W_ee. */
int clm_jacobian(clm_handle* h, double t, double dtgamma, double* W_vv,
                 double* W_ev, double* W_ee);

/* The block solve of initialize_jacobian's FieldMatrixSolver
 * (BlockDiagonalSolve / BlockLowerTriangularSolve(soil.ϑ_l),
 * implicit_timestepping.jl:160-171): given blocks and residual f, returns
 * delta with W delta = f per column (cell layout). f_e/W_e* may be NULL for
 * RichardsModel. */
int clm_solve(clm_handle* h, const double* W_vv, const double* W_ev,
              const double* W_ee, const double* f_v, const double* f_e,
              double* delta_v, double* delta_e);

/* ---- learned Newton guess (no reference counterpart) ------------------
 * A small MLP (inputs: the 20-layer vartheta_l, theta_i, T profiles, top
 * water and heat fluxes, alpha, n, nu, log10 K_sat, dt; two hidden layers
 * of 64 with GELU; outputs: 20-layer vartheta_l and rho_e_int) predicts how
 * each column's step increment changes from its previous step's. With
 * cfg->learned_guess = CLM_GUESS_NETWORK (EnergyHydrology, tolerance mode,
 * 20-layer columns) Newton starts from u_n + (u_n - u_{n-1}) + prediction,
 * u_{n-1} the state at the previous guess; a column whose first Newton
 * increment exceeds ten times its guessed one, or whose iteration from it
 * stops contracting, restarts from the plain start
 * (CLM_COL_GUESS_FALLBACK). clm_load_mlp restarts the history (the
 * first guess after it is the prediction alone); clm_set_state keeps it.
 * Weights are a blob of clm_mlp_blob_bytes() bytes written by clm_mlp_get. */
int clm_load_mlp(clm_handle* h, const void* weights, int64_t nbytes);

/* Raw network inputs of every 20-layer column at time t (device array of
 * ncol x 67 floats, original column order; other columns untouched). */
int clm_features(clm_handle* h, double t, double dt, float* X);

/* Trainer: FP32 master weights + Adam on the GPU; forward and backward
 * BF16 GEMMs on the tensor cores (FP32 accumulation). X (rows x 67) and
 * Y (rows x 40) are device arrays of raw inputs and targets; the
 * standardisation (per-feature mean and std, host arrays) is set first.
 * clm_mlp_train runs nsteps minibatches of `batch` consecutive rows,
 * wrapping at nrows, and returns each step's summed squared error (host
 * array of nsteps, may be NULL). clm_mlp_gradients returns the gradient
 * (host, clm_mlp_nparams() floats, parameter order W1 b1 W2 b2 W3 b3) of the
 * mean over rows of the squared standardised error, without updating. */
typedef struct clm_mlp clm_mlp;
int clm_mlp_create(uint64_t seed, clm_mlp** out);
void clm_mlp_destroy(clm_mlp* m);
int clm_mlp_set_normalization(clm_mlp* m, const float* in_mean, const float* in_std,
                              const float* out_mean, const float* out_std);
int clm_mlp_train(clm_mlp* m, const float* X, const float* Y, int64_t nrows,
                  int32_t batch, int32_t nsteps, float lr, float* loss,
                  void* cuda_stream);
int clm_mlp_gradients(clm_mlp* m, const float* X, const float* Y, int32_t nrows,
                      float* grad, float* loss);
int clm_mlp_predict(clm_mlp* m, const float* X, int64_t nrows, float* Y,
                    void* cuda_stream);
int64_t clm_mlp_blob_bytes(void);
int64_t clm_mlp_nparams(void);
int clm_mlp_get(const clm_mlp* m, void* blob, int64_t nbytes);
int clm_mlp_set(clm_mlp* m, const void* blob, int64_t nbytes);

/* ---- allocation-free step (no reference counterpart) -----------------
 * The EnergyHydrology step for callers that cannot allocate device memory:
 * hosts whose device heap belongs to another allocator (CUDA.jl or PyTorch
 * caching allocators under a fixed budget), time-stepping loops that cannot
 * take the synchronisation a cudaMalloc/cudaFree may bring, or embeddings
 * that forbid allocation after start-up.
 * Everything is caller-owned device memory in the reference layout: z_lo,
 * z_hi (ncol), params (CLM_NPARAM_EH rows of ncol), the state (cell = c * nlayers + k) and intF_w / intF_e (ncol),
 * updated in place; flags (ncol, CLM_COL_*) may be NULL. forcing is a
 * host array of 4 device pointers, one per clm_bc_slot (CLM_F_NFIELDS rows
 * of ncol each, or NULL); forcing itself may be NULL. cfg (host memory)
 * supplies the model constants and must ask for EnergyHydrology in FP64;
 * it passes clm_create's configuration checks, and neither the learned
 * guess nor the atmosphere-driven or precipitation/runoff top boundary is
 * available here. Limits: 2 <= nlayers <= 32, the same for every column;
 * otherwise CLM_ERR_ARG. The parameter rows are device memory and are not
 * validated: they must satisfy clm_set_params' constraints (a column whose
 * state turns non-finite gets CLM_COL_NONFINITE). The kernel's working
 * scratch is a fixed 24 MiB device array inside the library, held by every
 * GPU that loads it until the process exits. All calls share it: calls that
 * overlap on the GPU (other streams or host threads) race. The first call
 * on each device (and the first after a cudaDeviceReset) looks up that
 * array and configures the kernel, so make it before any stream capture.
 * Runs asynchronously on cuda_stream (a cudaStream_t, NULL for the legacy
 * default stream). */
int clm_step_eh_noalloc(const clm_config* cfg, int32_t ncol, int32_t nlayers,
                        const double* z_lo, const double* z_hi, const double* params,
                        const double* const* forcing, double* vartheta_l,
                        double* theta_i, double* rho_e_int, double* intF_w,
                        double* intF_e, uint32_t* flags, double t, double dt,
                        int32_t nsteps, void* cuda_stream);

/* Counter hash used by the rain-pulse forcing: uniform in [0, 1). Plain
 * integer arithmetic, identical on host and device. */
double clm_forcing_hash01(uint64_t seed, uint64_t column, int64_t period);

/* Library version string. */
const char* clm_version(void);

#ifdef __cplusplus
}
#endif

#endif /* CLIMALAND_CUDA_H */
