// Fused soil column step: IMEX ARS111 with a fixed-iteration (or
// tolerance-stopped) Newton loop, one thread per column, the column staged
// in shared memory.
//
// Reference path replaced (paths relative to the ClimaLand.jl tree):
//   stage 1   make_exp_tendency = update_aux! + update_boundary_fluxes! +
//             compute_exp_tendency! (models.jl:279-287; rre.jl:111-149,
//             214-243, 368-380; energy_hydrology.jl:273-350, 722-906)
//   stage 2   U = u + dt T_exp; Newton on U + dt T_imp(x) - x = 0 with
//             W = dt dT_imp/dY - I from make_compute_jacobian (rre.jl:391-458;
//             energy_hydrology.jl:466-576, including the "- I" on d(rho e)/d
//             vartheta), cache_imp! = make_update_implicit_cache
//             (models.jl:238-246; energy_hydrology.jl:427-455) and the block
//             Thomas solve chosen in initialize_jacobian
//             (implicit_timestepping.jl:160-171)
//   final     u_{n+1} = u + dt T_exp + dt (x - U) / dt
//
// Per Newton iteration the kernel makes four sweeps over the column:
//   1 (up)    T, psi, dpsi at x in a rolling 3-layer register window; face
//             fluxes, residual f, Jacobian rows and the Thomas forward
//             elimination of the vartheta block, all fused;
//   2 (down)  back substitution: delta vartheta;
//   3 (up)    energy right-hand side f_e - W_ev delta vartheta and the
//             forward elimination of the rho e block;
//   4 (down)  back substitution: delta rho e; x -= delta.
// JT is the type of the Jacobian and Thomas arrays: double for the plain
// path, float for the mixed-precision path (residual, increments, phase
// partition and budgets stay double; an FP64 column-sum projection restores
// the exact budget identity of the solve).

#include <cuda_runtime.h>

#include "clm_internal.cuh"

namespace clm {

// ---------------------------------------------------------------------------
// EnergyHydrology
// ---------------------------------------------------------------------------

// double arrays
enum { E_XV, E_XE, E_UV, E_UE, E_TI, E_K, E_KAP, E_IRC, E_FE, E_ND };
// JT arrays
enum { E_CP, E_DP, E_D, E_AE, E_DE, E_NJ };

template <typename JT>
__host__ __device__ constexpr size_t eh_smem_per_layer() {
  return E_ND * sizeof(double) + E_NJ * sizeof(JT);
}

struct EHCol {
  double nu, K_sat, S_s, theta_r;
  VG g;
  double kdry, ksf, ksu, rcds, nuom, nuq, nug, lku, lkf;
  double dz, inv_dz;
};

__device__ __forceinline__ EHCol load_eh_col(const StepArgs& A, int s, int n) {
  const int st = A.L.stride;
  const double* P = A.prm;
  EHCol c;
  c.nu = P[CLM_P_NU * st + s];
  c.K_sat = P[CLM_P_K_SAT * st + s];
  c.S_s = P[CLM_P_S_S * st + s];
  c.theta_r = P[CLM_P_THETA_R * st + s];
  c.g = make_vg(P[CLM_P_VG_ALPHA * st + s], P[CLM_P_VG_N * st + s]);
  c.kdry = P[CLM_P_KAPPA_DRY * st + s];
  c.ksf = P[CLM_P_KAPPA_SAT_FROZEN * st + s];
  c.ksu = P[CLM_P_KAPPA_SAT_UNFROZEN * st + s];
  c.rcds = P[CLM_P_RHOC_DS * st + s];
  c.nuom = P[CLM_P_NU_SS_OM * st + s];
  c.nuq = P[CLM_P_NU_SS_QUARTZ * st + s];
  c.nug = P[CLM_P_NU_SS_GRAVEL * st + s];
  c.lku = A.lkap[s];
  c.lkf = A.lkap[st + s];
  c.dz = (A.z_hi[s] - A.z_lo[s]) / n;
  c.inv_dz = 1.0 / c.dz;
  return c;
}

// Phase-change source (soil_heat_parameterizations.jl:89-122) divided out:
// returns (theta_l - theta_star) / tau with tau = 3 rho c dz^2 / kappa.
__device__ __forceinline__ double eh_phase_change(const Earth& E, const EHCol& c,
                                                  double theta_l, double theta_i,
                                                  double T, double rhoc,
                                                  double kappa, uint32_t& flags) {
  double theta_tot = fmin(E.rho_i_over_rho_l * theta_i + theta_l, c.nu);
  Sat s = saturation(c.nu, theta_tot, c.theta_r);
  double psi_w0;
  {
    double u = exp(-c.g.inv_m * log(s.S));
    double w = u - 1.0;
    psi_w0 = (w > 0.0) ? -exp(c.g.inv_n * log(w)) * c.g.inv_alpha : -0.0;
  }
  double Tf = fmax(E.T_freeze * exp(E.grav_over_LH_f0 * psi_w0), 1.0);
  double theta_star;
  if (Tf - T > kEps) {  // heaviside(Tf - T)
    double psi = psi_w0 + E.LH_f0_over_grav * log(T / Tf);
    if (psi > 0.0) flags |= CLM_COL_PSI_POSITIVE;
    double x = exp(c.g.n * log(c.g.alpha * fabs(psi)));  // (alpha |psi|)^n
    double Sst = exp(-c.g.m * log1p(x));                  // (1 + x)^(-m)
    theta_star = Sst * (c.nu - c.theta_r) + c.theta_r;
  } else {
    // psi_T = 0: inverse_matric_potential(matric_potential(S)) = S
    if (psi_w0 > 0.0) flags |= CLM_COL_PSI_POSITIVE;
    theta_star = s.S * (c.nu - c.theta_r) + c.theta_r;
  }
  double tau = 3.0 * rhoc * (c.dz * c.dz) / kappa;
  return (theta_l - theta_star) / tau;
}

// T and psi at the Newton iterate (update_implicit_aux!,
// energy_hydrology.jl:427-445) and dpsi/dvartheta (Jacobian, :503-512).
__device__ __forceinline__ void eh_iterate_point(const Earth& E, const EHCol& c,
                                                 double xv, double xe, double ti,
                                                 double& T, double& psi,
                                                 double& D) {
  double nu_eff = c.nu - ti;
  T = temperature(E, xe, ti, heat_capacity(E, fmin(nu_eff, xv), ti, c.rcds));
  psi_dpsi<true>(c.g, nu_eff, xv, c.theta_r, c.S_s, psi, D);
}

template <typename JT>
__global__ void __launch_bounds__(128, 1)
    eh_step_kernel(StepArgs A, double t0, double dt, int nsteps) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int wpc = blockDim.x >> 5;
  const int tile = blockIdx.x * wpc + warp;
  if (tile >= A.L.ntiles) return;
  const int nmax = A.L.nmax;
  double* dbase = reinterpret_cast<double*>(smem_raw) + (size_t)warp * E_ND * nmax * kTile;
  JT* jbase = reinterpret_cast<JT*>(reinterpret_cast<double*>(smem_raw) +
                                    (size_t)wpc * E_ND * nmax * kTile) +
              (size_t)warp * E_NJ * nmax * kTile;
  Tile<double> S{dbase, nmax, lane};
  Tile<JT> J{jbase, nmax, lane};

  const int s = tile * kTile + lane;
  const int n = A.L.col_n[s];
  if (n <= 0) return;
  const int orig = A.L.perm[s];
  const int64_t base = A.L.tile_off[tile] + lane;
  const Earth& E = A.E;
  const EHScalars& sc = A.sc;
  const EHCol c = load_eh_col(A, s, n);
  const int st = A.L.stride;
  uint32_t flags = 0;
  int iters_done = 0;

  // load the state into shared memory
  for (int k = 0; k < n; ++k) {
    S(E_XV, k) = A.v[base + (int64_t)k * kTile];
    S(E_TI, k) = A.ti[base + (int64_t)k * kTile];
    S(E_XE, k) = A.e[base + (int64_t)k * kTile];
  }
  double Fw = A.Fw[s], Fe = A.Fe[s];
  const double rdz = dt * c.inv_dz;

  for (int step = 0; step < nsteps; ++step) {
    const double t = t0 + step * dt;
    // ---------------- stage 1: aux at Y_n, explicit tendency, U ----------
    double K0 = 0, T0 = 0, kap0 = 0, psi0 = 0;
    double Kt = 0, Tt = 0, kapt = 0, psit = 0;
    for (int k = 0; k < n; ++k) {
      const double Yv = S(E_XV, k), Yti = S(E_TI, k), Ye = S(E_XE, k);
      const double nu_eff = c.nu - Yti;
      // volumetric_liquid_fraction (soil_hydrology_parameterizations.jl:22-31)
      const double v_safe = fmax(Yv, c.theta_r + kSqrtEps);
      const double nu_safe = fmax(nu_eff, c.theta_r + kSqrtEps);
      const double tl = (v_safe < nu_safe) ? v_safe : nu_safe;
      const double kap = conductivity_heat(sc, tl, Yti, c.nu, c.kdry, c.ksu, c.ksf,
                                           c.lku, c.lkf, c.nuom, c.nuq, c.nug);
      const double rc = heat_capacity(E, tl, Yti, c.rcds);
      const double T = temperature(E, Ye, Yti, rc);
      const Sat sK = saturation(c.nu, Yv, c.theta_r);
      const double fi = Yti / (tl + Yti - c.theta_r);
      const double K = exp(-sc.omega_ln10 * fi + sc.visc_gamma * (T - sc.visc_gamma_T_ref)) *
                       conductivity(c.g, c.K_sat, sK.S);
      double Uv = Yv, Uti = Yti;
      if (A.phase_change) {
        const double pc = eh_phase_change(E, c, tl, Yti, T, rc, kap, flags);
        Uv = Yv + dt * (-pc);
        Uti = Yti + dt * (E.rho_l_over_rho_i * pc);
      }
      S(E_XV, k) = Uv;
      S(E_UV, k) = Uv;
      S(E_TI, k) = Uti;
      S(E_XE, k) = Ye;
      S(E_UE, k) = Ye;
      S(E_K, k) = K;
      S(E_KAP, k) = kap;
      S(E_IRC, k) = 1.0 / heat_capacity(E, tl, Uti, c.rcds);
      if (k == 0) {
        K0 = K; T0 = T; kap0 = kap;
        if (A.bc_bw == CLM_BC_STATE) { double d; psi_dpsi<false>(c.g, nu_eff, Yv, c.theta_r, c.S_s, psi0, d); }
      }
      if (k == n - 1) {
        Kt = K; Tt = T; kapt = kap;
        if (A.bc_tw == CLM_BC_STATE) { double d; psi_dpsi<false>(c.g, nu_eff, Yv, c.theta_r, c.S_s, psit, d); }
      }
    }
    // boundary fluxes at t (frozen through the Newton solve)
    const double half = 0.5 * c.dz;  // centre-to-boundary distance
    double Ftw, Fth, Fbw, Fbh;
    {
      const double ftw = forcing_value(A.forc[CLM_BC_TOP_WATER], st, s, orig, t, A.seed);
      const double fth = forcing_value(A.forc[CLM_BC_TOP_HEAT], st, s, orig, t, A.seed);
      const double fbw = forcing_value(A.forc[CLM_BC_BOTTOM_WATER], st, s, orig, t, A.seed);
      const double fbh = forcing_value(A.forc[CLM_BC_BOTTOM_HEAT], st, s, orig, t, A.seed);
      if (A.bc_tw == CLM_BC_STATE) {
        double pb, d;
        psi_dpsi<false>(c.g, c.nu, ftw, c.theta_r, c.S_s, pb, d);
        Ftw = -Kt * ((pb + half) - psit) / half;
      } else {
        Ftw = ftw;
      }
      if (A.bc_bw == CLM_BC_FREE_DRAINAGE) {
        Fbw = -1.0 * K0;
      } else if (A.bc_bw == CLM_BC_STATE) {
        double pb, d;
        psi_dpsi<false>(c.g, c.nu, fbw, c.theta_r, c.S_s, pb, d);
        Fbw = -K0 * ((psi0 + half) - pb) / half;
      } else {
        Fbw = fbw;
      }
      if (A.bc_th == CLM_BC_STATE) {
        Fth = -kapt * (fth - Tt) / half;
      } else if (A.bc_th == CLM_BC_FLUX_ADVECTIVE) {
        const double* F = A.forc[CLM_BC_TOP_HEAT];
        const double Tadv = F ? F[CLM_F_T_ADV * st + s] : E.T_0;
        Fth = fth + Ftw * rho_e_liq(E, Tadv);
      } else {
        Fth = fth;
      }
      if (A.bc_bh == CLM_BC_FREE_DRAINAGE) {
        Fbh = -1.0 * K0 * rho_e_liq(E, T0);
      } else if (A.bc_bh == CLM_BC_STATE) {
        Fbh = -kap0 * (T0 - fbh) / half;
      } else {
        Fbh = fbh;
      }
    }
    const double UFw = Fw, UFe = Fe;
    double xFw = UFw, xFe = UFe;

    // ---------------- stage 2: Newton ------------------------------------
    double prev_norm = 1e300;
    int it = 0;
    for (it = 1; it <= A.max_iters; ++it) {
      // sweep 1 (bottom -> top)
      JT cp_prev = 0, dp_prev = 0;
      double Fw_dn = Fbw, Fe_dn = Fbh;
      double aw_dn = 0.0;
      JT D_prev = 0;
      double sum_fv = 0.0, sum_fe = 0.0;
      double Tc, psic, Dc;
      eh_iterate_point(E, c, S(E_XV, 0), S(E_XE, 0), S(E_TI, 0), Tc, psic, Dc);
      double Kc = S(E_K, 0), kapc = S(E_KAP, 0);
      double relKc = rho_e_liq(E, Tc) * Kc;
      for (int k = 0; k < n; ++k) {
        double Fw_up, Fe_up, aw_up = 0.0, ae_up = 0.0;
        double Tn = 0, psin = 0, Dn = 0, Kn = 0, kapn = 0, relKn = 0;
        if (k < n - 1) {
          eh_iterate_point(E, c, S(E_XV, k + 1), S(E_XE, k + 1), S(E_TI, k + 1), Tn, psin, Dn);
          Kn = S(E_K, k + 1);
          kapn = S(E_KAP, k + 1);
          relKn = rho_e_liq(E, Tn) * Kn;
          aw_up = 0.5 * (Kc + Kn) * c.inv_dz;
          const double ak_up = 0.5 * (kapc + kapn) * c.inv_dz;
          ae_up = 0.5 * (relKc + relKn) * c.inv_dz;
          const double dh = (psin - psic) + c.dz;
          Fw_up = -aw_up * dh;
          Fe_up = -ak_up * (Tn - Tc) - ae_up * dh;
        } else {
          Fw_up = Ftw;
          Fe_up = Fth;
        }
        const double Tv = -((Fw_up - Fw_dn) * c.inv_dz);
        const double Tee = -((Fe_up - Fe_dn) * c.inv_dz);
        const double fv = S(E_UV, k) + dt * Tv - S(E_XV, k);
        const double fe = S(E_UE, k) + dt * Tee - S(E_XE, k);
        sum_fv += fv;
        sum_fe += fe;
        // W_vv row and Thomas forward elimination
        const JT L = (JT)(rdz * aw_dn) * D_prev;
        const JT U = (k < n - 1) ? (JT)(rdz * aw_up * Dn) : (JT)0;
        const JT M = (JT)(-rdz * (aw_up + aw_dn) * Dc - 1.0);
        const JT inv = (JT)1 / (M - L * cp_prev);
        const JT cpk = U * inv;
        const JT dpk = ((JT)fv - L * dp_prev) * inv;
        J(E_CP, k) = cpk;
        J(E_DP, k) = dpk;
        J(E_D, k) = (JT)Dc;
        J(E_AE, k) = (JT)ae_up;
        S(E_FE, k) = fe;
        cp_prev = cpk;
        dp_prev = dpk;
        Fw_dn = Fw_up;
        Fe_dn = Fe_up;
        aw_dn = aw_up;
        D_prev = (JT)Dc;
        Tc = Tn; psic = psin; Dc = Dn; Kc = Kn; kapc = kapn; relKc = relKn;
      }
      // integrated fluxes (W = -I): x += f
      const double fFw = UFw + dt * (-(Ftw - Fbw)) - xFw;
      const double fFe = UFe + dt * (-(Fth - Fbh)) - xFe;
      xFw += fFw;
      xFe += fFe;
      // sweep 2 (top -> bottom): delta vartheta into E_DP
      {
        JT nxt = 0;
        for (int k = n - 1; k >= 0; --k) {
          const JT d = J(E_DP, k) - J(E_CP, k) * nxt;
          J(E_DP, k) = d;
          nxt = d;
        }
      }
      // FP64 column-sum projection (mixed path): sum(delta_v) = -sum(f_v)
      double corr_v = 0.0;
      if (sizeof(JT) < sizeof(double)) {
        double sd = 0.0;
        for (int k = 0; k < n; ++k) sd += (double)J(E_DP, k);
        corr_v = (sd + sum_fv) / n;
      }
      // sweep 3 (bottom -> top): energy right-hand side, rho e forward
      double norm2 = fFw * fFw + fFe * fFe;
      {
        JT c_prev = 0, d_prev = 0;
        double ak_dn = 0.0;
        JT dvm = 0, Dm = 0;  // k-1
        JT dv0 = J(E_DP, 0) - (JT)corr_v, D0 = J(E_D, 0);
        JT ae_dn = 0;
        double kap_c = S(E_KAP, 0), irc_c = S(E_IRC, 0), irc_m = 0.0;
        for (int k = 0; k < n; ++k) {
          JT dvp = 0, Dp = 0, ae_up = 0;
          double ak_up = 0.0, kap_n = 0.0, irc_n = 0.0;
          if (k < n - 1) {
            dvp = J(E_DP, k + 1) - (JT)corr_v;
            Dp = J(E_D, k + 1);
            ae_up = J(E_AE, k);
            kap_n = S(E_KAP, k + 1);
            irc_n = S(E_IRC, k + 1);
            ak_up = 0.5 * (kap_c + kap_n) * c.inv_dz;
          }
          const JT Gup = (k < n - 1) ? (Dp * dvp - D0 * dv0) : (JT)0;
          const JT Gdn = (k > 0) ? (D0 * dv0 - Dm * dvm) : (JT)0;
          const JT wev = (JT)rdz * (ae_up * Gup - ae_dn * Gdn) - dv0;
          const double g = S(E_FE, k) - (double)wev;
          const JT L = (JT)(rdz * ak_dn * irc_m);
          const JT U = (JT)(rdz * ak_up * irc_n);
          const JT M = (JT)(-rdz * (ak_up + ak_dn) * irc_c - 1.0);
          const JT inv = (JT)1 / (M - L * c_prev);
          const JT ck = U * inv;
          const JT dk = ((JT)g - L * d_prev) * inv;
          J(E_CP, k) = ck;
          J(E_DE, k) = dk;
          c_prev = ck;
          d_prev = dk;
          // x_v -= delta_v
          const double dvd = (double)dv0;
          S(E_XV, k) -= dvd;
          norm2 += dvd * dvd;
          dvm = dv0; Dm = D0; dv0 = dvp; D0 = Dp;
          ae_dn = ae_up;
          ak_dn = ak_up;
          irc_m = irc_c; irc_c = irc_n; kap_c = kap_n;
        }
      }
      // sweep 4 (top -> bottom): delta rho e
      {
        JT nxt = 0;
        double sd = 0.0;
        if (sizeof(JT) < sizeof(double)) {
          for (int k = n - 1; k >= 0; --k) {
            const JT d = J(E_DE, k) - J(E_CP, k) * nxt;
            J(E_DE, k) = d;
            sd += (double)d;
            nxt = d;
          }
        }
        // projection: W_ee and W_ev - (-I) have zero column sums, so
        // sum(delta_e) = -sum(g) = -sum(f_e) - sum(delta_v) = -sum(f_e) + sum(f_v)
        const double corr_e = (sizeof(JT) < sizeof(double)) ? (sd + sum_fe - sum_fv) / n : 0.0;
        nxt = 0;
        const double se = A.energy_scale;
        for (int k = n - 1; k >= 0; --k) {
          double d;
          if (sizeof(JT) < sizeof(double)) {
            d = (double)J(E_DE, k) - corr_e;
          } else {
            const JT dj = J(E_DE, k) - J(E_CP, k) * nxt;
            nxt = dj;
            d = (double)dj;
          }
          S(E_XE, k) -= d;
          norm2 += (se * d) * (se * d);
        }
      }
      iters_done = it;
      if (A.newton_mode == CLM_NEWTON_TOL) {
        const double nrm = sqrt(norm2);
        if (nrm > prev_norm && it > 2) flags |= CLM_COL_DIVERGED;
        prev_norm = nrm;
        if (nrm < A.tol) break;
        if (it == A.max_iters) flags |= CLM_COL_NOT_CONVERGED;
      }
    }
    // ---------------- final combination ---------------------------------
    const double inv_dt = 1.0 / dt;
    for (int k = 0; k < n; ++k) {
      const double Uv = S(E_UV, k), Ue = S(E_UE, k);
      S(E_XV, k) = Uv + dt * ((S(E_XV, k) - Uv) * inv_dt);
      S(E_XE, k) = Ue + dt * ((S(E_XE, k) - Ue) * inv_dt);
    }
    Fw = UFw + dt * ((xFw - UFw) * inv_dt);
    Fe = UFe + dt * ((xFe - UFe) * inv_dt);
  }
  // write back
  bool finite = isfinite(Fw) && isfinite(Fe);
  for (int k = 0; k < n; ++k) {
    const double v = S(E_XV, k), ti = S(E_TI, k), e = S(E_XE, k);
    finite = finite && isfinite(v) && isfinite(ti) && isfinite(e);
    A.v[base + (int64_t)k * kTile] = v;
    A.ti[base + (int64_t)k * kTile] = ti;
    A.e[base + (int64_t)k * kTile] = e;
  }
  A.Fw[s] = Fw;
  A.Fe[s] = Fe;
  if (!finite) flags |= CLM_COL_NONFINITE;
  A.flags[s] = flags;
  A.iters[s] = iters_done;
}

// ---------------------------------------------------------------------------
// RichardsModel
// ---------------------------------------------------------------------------

enum { R_XV, R_UV, R_ND };
enum { R_CP, R_DP, R_NJ };

template <typename JT>
__host__ __device__ constexpr size_t richards_smem_per_layer() {
  return R_ND * sizeof(double) + R_NJ * sizeof(JT);
}

template <typename JT>
__global__ void __launch_bounds__(128, 1)
    richards_step_kernel(StepArgs A, double t0, double dt, int nsteps) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int wpc = blockDim.x >> 5;
  const int tile = blockIdx.x * wpc + warp;
  if (tile >= A.L.ntiles) return;
  const int nmax = A.L.nmax;
  double* dbase = reinterpret_cast<double*>(smem_raw) + (size_t)warp * R_ND * nmax * kTile;
  JT* jbase = reinterpret_cast<JT*>(reinterpret_cast<double*>(smem_raw) +
                                    (size_t)wpc * R_ND * nmax * kTile) +
              (size_t)warp * R_NJ * nmax * kTile;
  Tile<double> S{dbase, nmax, lane};
  Tile<JT> J{jbase, nmax, lane};

  const int s = tile * kTile + lane;
  const int n = A.L.col_n[s];
  if (n <= 0) return;
  const int orig = A.L.perm[s];
  const int64_t base = A.L.tile_off[tile] + lane;
  const int st = A.L.stride;
  const double* P = A.prm;
  const double nu = P[CLM_P_NU * st + s];
  const double K_sat = P[CLM_P_K_SAT * st + s];
  const double S_s = P[CLM_P_S_S * st + s];
  const double theta_r = P[CLM_P_THETA_R * st + s];
  const VG g = make_vg(P[CLM_P_VG_ALPHA * st + s], P[CLM_P_VG_N * st + s]);
  const double dz = (A.z_hi[s] - A.z_lo[s]) / n;
  const double inv_dz = 1.0 / dz;
  const double half = 0.5 * dz;
  const double rdz = dt * inv_dz;
  // MoistureStateBC at the top carries dfluxBCdY (rre.jl:137-146, 460-468):
  // boundary fluxes are then refreshed with the implicit cache.
  const bool dflux = (A.bc_tw == CLM_BC_STATE);
  uint32_t flags = 0;
  int iters_done = 0;

  for (int k = 0; k < n; ++k) S(R_XV, k) = A.v[base + (int64_t)k * kTile];
  double Fw = A.Fw[s];

  for (int step = 0; step < nsteps; ++step) {
    const double t = t0 + step * dt;
    // explicit tendency is zero (no explicit sources): U = u
    for (int k = 0; k < n; ++k) S(R_UV, k) = S(R_XV, k);
    const double UFw = Fw;
    double xFw = UFw;
    const double t_bc = dflux ? t + dt : t;
    const double ftw = forcing_value(A.forc[CLM_BC_TOP_WATER], st, s, orig, t_bc, A.seed);
    const double fbw = forcing_value(A.forc[CLM_BC_BOTTOM_WATER], st, s, orig, t_bc, A.seed);
    double psi_tb = 0.0, psi_bb = 0.0;
    if (A.bc_tw == CLM_BC_STATE) { double d; psi_dpsi<false>(g, nu, ftw, theta_r, S_s, psi_tb, d); }
    if (A.bc_bw == CLM_BC_STATE) { double d; psi_dpsi<false>(g, nu, fbw, theta_r, S_s, psi_bb, d); }
    double Ftw = ftw, Fbw = fbw;  // frozen values when !dflux (set in iteration 1)
    double prev_norm = 1e300;
    int it;
    for (it = 1; it <= A.max_iters; ++it) {
      const bool refresh_bc = dflux || it == 1;
      JT cp_prev = 0, dp_prev = 0;
      double aw_dn = 0.0;
      JT D_prev = 0;
      double sum_f = 0.0;
      double Kc, psic, Dc;
      richards_point<true>(g, nu, S(R_XV, 0), theta_r, S_s, K_sat, Kc, psic, Dc);
      if (refresh_bc) {
        if (A.bc_bw == CLM_BC_FREE_DRAINAGE) Fbw = -1.0 * Kc;
        else if (A.bc_bw == CLM_BC_STATE) Fbw = -Kc * ((psic + half) - psi_bb) / half;
      }
      double Fw_dn = Fbw;
      double dflux_top = 0.0;
      for (int k = 0; k < n; ++k) {
        double Fw_up, aw_up = 0.0;
        double Kn = 0, psin = 0, Dn = 0;
        if (k < n - 1) {
          richards_point<true>(g, nu, S(R_XV, k + 1), theta_r, S_s, K_sat, Kn, psin, Dn);
          aw_up = 0.5 * (Kc + Kn) * inv_dz;
          Fw_up = -aw_up * ((psin - psic) + dz);
        } else {
          if (refresh_bc && A.bc_tw == CLM_BC_STATE) Ftw = -Kc * ((psi_tb + half) - psic) / half;
          if (dflux) dflux_top = Kc * Dc / half;  // set_dfluxBCdY! (boundary_conditions.jl:375-426)
          Fw_up = Ftw;
        }
        const double Tv = -((Fw_up - Fw_dn) * inv_dz);
        const double f = S(R_UV, k) + dt * Tv - S(R_XV, k);
        sum_f += f;
        const JT L = (JT)(rdz * aw_dn) * D_prev;
        const JT U = (k < n - 1) ? (JT)(rdz * aw_up * Dn) : (JT)0;
        double Md = -rdz * (aw_up + aw_dn) * Dc - 1.0;
        if (k == n - 1 && dflux) Md += -dt * (dflux_top * inv_dz);
        const JT M = (JT)Md;
        const JT inv = (JT)1 / (M - L * cp_prev);
        const JT cpk = U * inv;
        const JT dpk = ((JT)f - L * dp_prev) * inv;
        J(R_CP, k) = cpk;
        J(R_DP, k) = dpk;
        cp_prev = cpk;
        dp_prev = dpk;
        Fw_dn = Fw_up;
        aw_dn = aw_up;
        D_prev = (JT)Dc;
        Kc = Kn; psic = psin; Dc = Dn;
      }
      const double fFw = UFw + dt * (-(Ftw - Fbw)) - xFw;
      xFw += fFw;
      double norm2 = fFw * fFw;
      // back substitution and update
      if (sizeof(JT) < sizeof(double)) {
        JT nxt = 0;
        double sd = 0.0;
        for (int k = n - 1; k >= 0; --k) {
          const JT d = J(R_DP, k) - J(R_CP, k) * nxt;
          J(R_DP, k) = d;
          sd += (double)d;
          nxt = d;
        }
        const double corr = dflux ? 0.0 : (sd + sum_f) / n;
        for (int k = 0; k < n; ++k) {
          const double d = (double)J(R_DP, k) - corr;
          S(R_XV, k) -= d;
          norm2 += d * d;
        }
      } else {
        JT nxt = 0;
        for (int k = n - 1; k >= 0; --k) {
          const JT d = J(R_DP, k) - J(R_CP, k) * nxt;
          nxt = d;
          S(R_XV, k) -= (double)d;
          norm2 += (double)d * (double)d;
        }
      }
      iters_done = it;
      if (A.newton_mode == CLM_NEWTON_TOL) {
        const double nrm = sqrt(norm2);
        if (nrm > prev_norm && it > 2) flags |= CLM_COL_DIVERGED;
        prev_norm = nrm;
        if (nrm < A.tol) break;
        if (it == A.max_iters) flags |= CLM_COL_NOT_CONVERGED;
      }
    }
    const double inv_dt = 1.0 / dt;
    for (int k = 0; k < n; ++k) {
      const double Uv = S(R_UV, k);
      S(R_XV, k) = Uv + dt * ((S(R_XV, k) - Uv) * inv_dt);
    }
    Fw = UFw + dt * ((xFw - UFw) * inv_dt);
  }
  bool finite = isfinite(Fw);
  for (int k = 0; k < n; ++k) {
    const double v = S(R_XV, k);
    finite = finite && isfinite(v);
    A.v[base + (int64_t)k * kTile] = v;
  }
  A.Fw[s] = Fw;
  if (!finite) flags |= CLM_COL_NONFINITE;
  A.flags[s] = flags;
  A.iters[s] = iters_done;
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------

size_t step_smem_bytes(int model, int precision, int nmax, int wpc) {
  size_t per_layer;
  if (model == CLM_MODEL_ENERGY_HYDROLOGY)
    per_layer = precision == CLM_PREC_MIXED ? eh_smem_per_layer<float>() : eh_smem_per_layer<double>();
  else
    per_layer = precision == CLM_PREC_MIXED ? richards_smem_per_layer<float>()
                                            : richards_smem_per_layer<double>();
  return per_layer * (size_t)nmax * kTile * wpc;
}

cudaError_t launch_step(const StepArgs& A, int model, int precision, int wpc,
                        double t0, double dt, int nsteps, cudaStream_t stream) {
  const size_t smem = step_smem_bytes(model, precision, A.L.nmax, wpc);
  const int grid = (A.L.ntiles + wpc - 1) / wpc;
  const dim3 block(32 * wpc);
  void (*fn)(StepArgs, double, double, int);
  if (model == CLM_MODEL_ENERGY_HYDROLOGY)
    fn = precision == CLM_PREC_MIXED ? eh_step_kernel<float> : eh_step_kernel<double>;
  else
    fn = precision == CLM_PREC_MIXED ? richards_step_kernel<float> : richards_step_kernel<double>;
  cudaError_t err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  fn<<<grid, block, smem, stream>>>(A, t0, dt, nsteps);
  return cudaGetLastError();
}

}  // namespace clm
