// Closure-level kernels: each reference closure evaluated on its own, for
// per-closure parity checks and for callers that drive their own time
// stepper. One thread per column; cell arrays in the reference layout
// (cell = ref_off[c] + k), per-column arrays in sorted order (index s).
//
//   closure_kernel<AUX>  make_update_cache = update_aux! + boundary fluxes
//                        (rre.jl:111-149, 368-380;
//                         energy_hydrology.jl:273-298, 722-814)
//   closure_kernel<EXP>  make_exp_tendency (models.jl:279-287; rre.jl:214-243;
//                        energy_hydrology.jl:315-350, 838-906)
//   closure_kernel<IMP>  make_compute_imp_tendency (rre.jl:161-203;
//                        energy_hydrology.jl:363-425) after the cache update
//   closure_kernel<JAC>  make_compute_jacobian (rre.jl:391-458;
//                        energy_hydrology.jl:466-576) after the cache update
//   solve_kernel         FieldMatrixSolver block solve
//                        (implicit_timestepping.jl:160-171)

#include <cuda_runtime.h>

#include "clm_closures.cuh"

namespace clm {

template <int KIND, class CM, class Geom>
__device__ void closure_column(const ClosureArgs& C, const Tables& Tb) {
  const StepArgs& A = C.A;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= A.L.stride) return;
  const int n = A.L.col_n[s];
  if (n <= 0) return;
  const auto G = GeomOf<Geom::kStretched>::make(A, A.L.tile_off[s / kTile] + s % kTile, s, n);
  const int orig = A.L.perm[s];
  const int64_t o = C.ref_off[orig];
  const int st = A.L.stride;
  const int ncol = A.L.ncol;
  const bool eh = C.model == CLM_MODEL_ENERGY_HYDROLOGY;
  const Earth& E = A.E;
  const EHScalars& sc = A.sc;
  const double* P = A.prm;
  const double nu = P[CLM_P_NU * st + s], K_sat = P[CLM_P_K_SAT * st + s];
  const double S_s = P[CLM_P_S_S * st + s], theta_r = P[CLM_P_THETA_R * st + s];
  const CM g = make_cm<CM>(P[CLM_P_VG_ALPHA * st + s], P[CLM_P_VG_N * st + s]);
  double kdry = 0, ksf = 0, ksu = 0, rcds = 0, nuom = 0, nuq = 0, nug = 0, lku = 0, lkf = 0;
  if (eh) {
    kdry = P[CLM_P_KAPPA_DRY * st + s];
    ksf = P[CLM_P_KAPPA_SAT_FROZEN * st + s];
    ksu = P[CLM_P_KAPPA_SAT_UNFROZEN * st + s];
    rcds = P[CLM_P_RHOC_DS * st + s];
    nuom = P[CLM_P_NU_SS_OM * st + s];
    nuq = P[CLM_P_NU_SS_QUARTZ * st + s];
    nug = P[CLM_P_NU_SS_GRAVEL * st + s];
    lku = A.lkap[s];
    lkf = A.lkap[st + s];
  }
  double Kc[kMaxLayers], psic[kMaxLayers], Tc[kMaxLayers], kapc[kMaxLayers], tlc[kMaxLayers];
  // ---- update_aux ----
  for (int k = 0; k < n; ++k) {
    const double Yv = C.v[o + k];
    const double Yti = eh ? C.ti[o + k] : 0.0;
    const double nu_eff = nu - Yti;
    double d;
    psi_dpsi<false>(Tb, g, nu_eff, Yv, theta_r, S_s, psic[k], d);
    const Sat sK = saturation(nu, Yv, theta_r);
    double K = conductivity(Tb, g, K_sat, sK.S);
    if (eh) {
      const double Ye = C.e[o + k];
      const double v_safe = fmax(Yv, theta_r + kSqrtEps);
      const double nu_safe = fmax(nu_eff, theta_r + kSqrtEps);
      const double tl = (v_safe < nu_safe) ? v_safe : nu_safe;
      tlc[k] = tl;
      kapc[k] = conductivity_heat(Tb, sc, tl, Yti, nu, kdry, ksu, ksf, lku, lkf, nuom, nuq, nug);
      Tc[k] = temperature(E, Ye, Yti, heat_capacity(E, tl, Yti, rcds));
      const double fi = Yti / (tl + Yti - theta_r);
      K *= fm::exp(Tb, -sc.omega_ln10 * fi + sc.visc_gamma * (Tc[k] - sc.visc_gamma_T_ref));
    }
    Kc[k] = K;
  }
  // ---- boundary fluxes at t ----
  const double t = C.t;
  const double ftw = forcing_value(A.forc[CLM_BC_TOP_WATER], st, s, A.col0 + orig, t, A.seed);
  const double fth = forcing_value(A.forc[CLM_BC_TOP_HEAT], st, s, A.col0 + orig, t, A.seed);
  const double fbw = forcing_value(A.forc[CLM_BC_BOTTOM_WATER], st, s, A.col0 + orig, t, A.seed);
  const double fbh = forcing_value(A.forc[CLM_BC_BOTTOM_HEAT], st, s, A.col0 + orig, t, A.seed);
  double Ftw = ftw, Fth = 0, Fbw = fbw, Fbh = 0;
  if (A.bc_tw == CLM_BC_STATE) {
    double pb, d;
    psi_dpsi<false>(Tb, g, nu, ftw, theta_r, S_s, pb, d);
    Ftw = -Kc[n - 1] * ((pb + G.half_top()) - psic[n - 1]) / G.half_top();
  }
  if (A.bc_bw == CLM_BC_FREE_DRAINAGE) {
    Fbw = -1.0 * Kc[0];
  } else if (A.bc_bw == CLM_BC_STATE) {
    double pb, d;
    psi_dpsi<false>(Tb, g, nu, fbw, theta_r, S_s, pb, d);
    Fbw = -Kc[0] * ((psic[0] + G.half_bot()) - pb) / G.half_bot();
  }
  if (eh) {
    Fth = fth;
    if (A.bc_th == CLM_BC_STATE) Fth = -kapc[n - 1] * (fth - Tc[n - 1]) / G.half_top();
    else if (A.bc_th == CLM_BC_FLUX_ADVECTIVE) {
      const double* F = A.forc[CLM_BC_TOP_HEAT];
      Fth = fth + Ftw * rho_e_liq(E, F ? F[CLM_F_T_ADV * st + s] : E.T_0);
    }
    Fbh = fbh;
    if (A.bc_bh == CLM_BC_FREE_DRAINAGE) Fbh = -1.0 * Kc[0] * rho_e_liq(E, Tc[0]);
    else if (A.bc_bh == CLM_BC_STATE) Fbh = -kapc[0] * (Tc[0] - fbh) / G.half_bot();
  }
  const bool dflux = !eh && A.bc_tw == CLM_BC_STATE;
  // atmosphere-driven top boundary (CLM_BC_ATMOS) from the aux values above
  AtmosOut ab{};
  EHRunoff ro{0.0, 0.0, 0.0, 0.0, 0.0};
  double dz_top = 0.0;
  const bool atmos = eh && A.atm && A.bc_tw == CLM_BC_ATMOS;
  if (atmos) {
    AtmosSfc sf;
    sf.T = Tc[n - 1];
    sf.psi = psic[n - 1];
    sf.ti = C.ti[o + n - 1];
    sf.th1 = tlc[n - 1];
    sf.th2 = tlc[n - 2];
    sf.Tf = tf_depressed_aux(Tb, E, g, nu, theta_r, sf.th1, sf.ti);
    sf.z1 = G.centre(n - 1);
    sf.z2 = G.centre(n - 2);
    dz_top = G.top_gap();
    sf.dz_top = dz_top;
    const AtmosRow D{A.atm, st, s};
    sf.th_alb = albedo_theta(G, D(CLM_AT_ALBEDO_TOP_THICKNESS), [&](int k) { return tlc[k]; });
    ro = eh_runoff(Tb, E, sc, A.runoff, G, nu, theta_r, K_sat, P[CLM_P_F_MAX * st + s],
                   P[CLM_P_F_OVER * st + s], P[CLM_P_R_SB * st + s], tlc[n - 1], D(CLM_AT_P_LIQ),
                   [&](int k, double& v, double& ti, double& T) {
                     v = C.v[o + k];
                     ti = C.ti[o + k];
                     T = Tc[k];
                   });
    sf.infil = ro.infil;
    ab = atmos_bc(Tb, A.ak, E, D, g, nu, theta_r, sf);
    Ftw = ab.top_w;
    Fth = ab.top_h;
  }
  // RichardsAtmosDrivenFluxBC: the runoff model turns the precipitation into
  // the infiltration; TOPMODEL's implicit subsurface sink (Runoff.jl:129-148,
  // 234-270, 321-345, infiltration capacity -K_sat :386-389)
  if (!eh && A.bc_tw == CLM_BC_PRECIP_RUNOFF && A.runoff != CLM_RUNOFF_NONE) {
    const double ic = -1.0 * K_sat;
    if (A.runoff == CLM_RUNOFF_SURFACE) {
      const double is_sat = ((C.v[o + n - 1] + 0.0) - nu) > kEps ? 1.0 : 0.0;
      Ftw = (1.0 - is_sat) * fmax(ic, ftw);
    } else {
      const double nr = nu - theta_r;
      double h = 0.0;
      for (int k = 0; k < n; ++k) h += G.width(k) * sat_weight(C.v[o + k] + 0.0 - theta_r, nr);
      const double zwt = (G.zhi - G.zlo) - h;
      const double f_sat = fmin(P[CLM_P_F_MAX * st + s] * fm::exp(Tb, -P[CLM_P_F_OVER * st + s] / 2.0 * zwt), 1.0);
      Ftw = (1.0 - f_sat) * fmax(ic, ftw);
      ro.R_ss = P[CLM_P_R_SB * st + s] * fm::exp(Tb, -P[CLM_P_F_OVER * st + s] * zwt);
      ro.cw = ro.R_ss / fmax(h, kEps);
    }
  }
  if (KIND == CL_ATM) {
    if (atmos && C.atm_out) {
      const double vals[CLM_AF_NFIELDS] = {ab.lhf, ab.shf, ab.vliq, ab.vice, ab.R_n, ab.q_sfc, ab.top_w, ab.top_h};
      for (int f = 0; f < CLM_AF_NFIELDS; ++f) C.atm_out[(int64_t)f * ncol + orig] = vals[f];
    }
    return;
  }

  if (KIND == CL_AUX) {
    for (int k = 0; k < n; ++k) {
      if (C.K) C.K[o + k] = Kc[k];
      if (C.psi) C.psi[o + k] = psic[k];
      if (eh) {
        if (C.theta_l) C.theta_l[o + k] = tlc[k];
        if (C.T) C.T[o + k] = Tc[k];
        if (C.kappa) C.kappa[o + k] = kapc[k];
        if (C.Tf) {
          // energy_hydrology.jl:797-808 passes (rho_l, rho_i) into the
          // (rho_ice, rho_liq) slots of soil_Tf_depressed (:35-52).
          const double Yti = C.ti[o + k];
          const double tt = fmin(E.rho_l / E.rho_i * Yti + tlc[k], nu);
          const double pw = matric_of(Tb, g, nu, tt, theta_r);
          C.Tf[o + k] = fmax(E.T_freeze * fm::exp(Tb, E.grav_over_LH_f0 * pw), 1.0);
        }
      }
    }
    if (C.bc) {
      C.bc[0 * ncol + orig] = Ftw;
      C.bc[1 * ncol + orig] = Fth;
      C.bc[2 * ncol + orig] = Fbw;
      C.bc[3 * ncol + orig] = Fbh;
    }
    return;
  }
  if (KIND == CL_EXP) {
    // PhaseChange, then RootExtraction (soil_canopy_root_interactions.jl:139-159)
    const bool roots = eh && A.rx;
    RootCol rcol;
    if (roots) rcol = load_root_col(Tb, A.rx, st, s);
    double root_w = 0.0, root_e = 0.0;
    for (int k = 0; k < n; ++k) {
      double dv = 0.0, dti = 0.0, de = 0.0;
      if (eh && A.phase_change) {
        const double Yti = C.ti[o + k];
        const double rc = heat_capacity(E, tlc[k], Yti, rcds);
        uint32_t fl = 0;
        const double pc = phase_change(Tb, E, g, nu, theta_r, tlc[k], Yti, Tc[k], rc, kapc[k], G.width(k), fl);
        dv = -pc;
        dti = E.rho_l_over_rho_i * pc;
      }
      if (atmos) dti += -ab.vice * E.rho_l / E.rho_i * sublimation_weight(G, k, dz_top);
      if (roots) {
        const double re = root_rate(Tb, rcol, G.face_centre(k), psic[k], Kc[k]);
        const double ree = re * rho_e_liq(E, Tc[k]);
        dv += -1.0 * re;
        de += -1.0 * ree;
        root_e += G.width(k) * ree;
        root_w += G.width(k) * re;
      }
      if (C.dv) C.dv[o + k] = dv;
      if (eh && C.dti) C.dti[o + k] = dti;
      if (eh && C.de) C.de[o + k] = de;
    }
    if (C.dFw) C.dFw[orig] = atmos ? 0.0 + -ab.vice : root_w;
    if (eh && C.dFe) C.dFe[orig] = root_e;
    return;
  }
  if (KIND == CL_IMP) {
    double Fw_dn = Fbw, Fe_dn = Fbh;
    for (int k = 0; k < n; ++k) {
      double Fw_up, Fe_up = 0.0;
      if (k < n - 1) {
        const double rg = 2.0 * G.hinv_gap(k);  // 1 / gap
        const double dh = (psic[k + 1] - psic[k]) + G.gap(k);
        Fw_up = -0.5 * (Kc[k] + Kc[k + 1]) * rg * dh;
        if (eh) {
          const double ak = 0.5 * (kapc[k] + kapc[k + 1]) * rg;
          const double ae = 0.5 * (rho_e_liq(E, Tc[k]) * Kc[k] + rho_e_liq(E, Tc[k + 1]) * Kc[k + 1]) * rg;
          Fe_up = -ak * (Tc[k + 1] - Tc[k]) - ae * dh;
        }
      } else {
        Fw_up = Ftw;
        Fe_up = Fth;
      }
      // TOPMODEL's subsurface sink under the atmosphere-driven boundary
      const double w = (ro.cw != 0.0 || ro.ce != 0.0) ? sat_weight(C.v[o + k] - theta_r, nu - theta_r) : 0.0;
      if (C.dv) C.dv[o + k] = -((Fw_up - Fw_dn) * G.inv_width(k)) - ro.cw * w;
      if (eh) {
        if (C.de) C.de[o + k] = -((Fe_up - Fe_dn) * G.inv_width(k)) - ro.ce * w;
        if (C.dti) C.dti[o + k] = 0.0;
      }
      Fw_dn = Fw_up;
      Fe_dn = Fe_up;
    }
    if (C.dFw) C.dFw[orig] = -(Ftw - Fbw) - ro.R_ss;
    if (eh && C.dFe) C.dFe[orig] = -(Fth - Fbh) - ro.R_ess;
    return;
  }
  if (KIND == CL_JAC) {
    double D[kMaxLayers];
    for (int k = 0; k < n; ++k) {
      double p;
      const double Yti = eh ? C.ti[o + k] : 0.0;
      psi_dpsi<true>(Tb, g, nu - Yti, C.v[o + k], theta_r, S_s, p, D[k]);
    }
    for (int blk = 0; blk < (eh ? 3 : 1); ++blk) {
      double* W = blk == 0 ? C.Wvv : (blk == 1 ? C.Wev : C.Wee);
      if (!W) continue;
      for (int k = 0; k < n; ++k) {
        double cup = 0.0, cdn = 0.0, dm = 0.0, d0, dp = 0.0;
        auto coef = [&](int a) -> double {  // face coefficient between a, a+1
          if (blk == 0) return 0.5 * (Kc[a] + Kc[a + 1]);
          if (blk == 1) return 0.5 * (rho_e_liq(E, Tc[a]) * Kc[a] + rho_e_liq(E, Tc[a + 1]) * Kc[a + 1]);
          return 0.5 * (kapc[a] + kapc[a + 1]);
        };
        auto dd = [&](int a) -> double {
          if (blk < 2) return D[a];
          return 1.0 / heat_capacity(E, tlc[a], C.ti[o + a], rcds);
        };
        d0 = dd(k);
        const double rdz = C.dtgamma * G.inv_width(k);
        if (k < n - 1) { cup = coef(k) * (2.0 * G.hinv_gap(k)); dp = dd(k + 1); }
        if (k > 0) { cdn = coef(k - 1) * (2.0 * G.hinv_gap(k - 1)); dm = dd(k - 1); }
        double L = (k > 0) ? rdz * cdn * dm : 0.0;
        double U = (k < n - 1) ? rdz * cup * dp : 0.0;
        double M = -rdz * (cup + cdn) * d0 - 1.0;
        if (blk == 0 && dflux && k == n - 1)
          M += -C.dtgamma * ((Kc[n - 1] * D[n - 1] / G.half_top()) * G.inv_width(k));
        W[3 * (o + k) + 0] = L;
        W[3 * (o + k) + 1] = M;
        W[3 * (o + k) + 2] = U;
      }
    }
  }
}

template <int KIND>
__global__ void closure_kernel(ClosureArgs C) {
  __shared__ double tab[fm::TABLE_SIZE];
  const Tables Tb = fm::stage_tables(tab);
  __syncthreads();
  const bool str = C.A.geo.z != nullptr;
  if (C.A.cm == CLM_CM_BROOKS_COREY) {
    if (str) closure_column<KIND, BC, ColGeomS>(C, Tb);
    else closure_column<KIND, BC, ColGeom>(C, Tb);
  } else {
    if (str) closure_column<KIND, VG, ColGeomS>(C, Tb);
    else closure_column<KIND, VG, ColGeom>(C, Tb);
  }
}

__device__ void thomas_ref(int n, const double* W, const double* f, double* x) {
  double cp[kMaxLayers], dp[kMaxLayers];
  for (int k = 0; k < n; ++k) {
    const double L = W[3 * k], M = W[3 * k + 1], U = W[3 * k + 2];
    const double den = (k > 0) ? M - L * cp[k - 1] : M;
    cp[k] = U / den;
    dp[k] = (k > 0) ? (f[k] - L * dp[k - 1]) / den : f[k] / den;
  }
  x[n - 1] = dp[n - 1];
  for (int k = n - 2; k >= 0; --k) x[k] = dp[k] - cp[k] * x[k + 1];
}

__global__ void solve_kernel(SolveArgs S) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S.L.stride) return;
  const int n = S.L.col_n[s];
  if (n <= 0) return;
  const int64_t o = S.ref_off[S.L.perm[s]];
  thomas_ref(n, S.Wvv + 3 * o, S.fv + o, S.dv + o);
  if (S.Wev && S.Wee && S.fe && S.de) {
    double g[kMaxLayers];
    for (int k = 0; k < n; ++k) {
      double w = S.Wev[3 * (o + k) + 1] * S.dv[o + k];
      if (k > 0) w += S.Wev[3 * (o + k)] * S.dv[o + k - 1];
      if (k < n - 1) w += S.Wev[3 * (o + k) + 2] * S.dv[o + k + 1];
      g[k] = S.fe[o + k] - w;
    }
    thomas_ref(n, S.Wee + 3 * o, g, S.de + o);
  }
}

cudaError_t launch_closure(int kind, const ClosureArgs& C, cudaStream_t st) {
  const int blocks = (C.A.L.stride + 127) / 128;
  switch (kind) {
    case CL_AUX: closure_kernel<CL_AUX><<<blocks, 128, 0, st>>>(C); break;
    case CL_EXP: closure_kernel<CL_EXP><<<blocks, 128, 0, st>>>(C); break;
    case CL_IMP: closure_kernel<CL_IMP><<<blocks, 128, 0, st>>>(C); break;
    case CL_ATM: closure_kernel<CL_ATM><<<blocks, 128, 0, st>>>(C); break;
    default: closure_kernel<CL_JAC><<<blocks, 128, 0, st>>>(C); break;
  }
  return cudaGetLastError();
}

cudaError_t launch_solve(const SolveArgs& S, cudaStream_t st) {
  solve_kernel<<<(S.L.stride + 127) / 128, 128, 0, st>>>(S);
  return cudaGetLastError();
}

}  // namespace clm
