// One soil column through nsteps IMEX ARS111 steps (host and device code).
//
// Reference path replaced (paths relative to the ClimaLand.jl tree):
//   stage 1   make_exp_tendency = update_aux! + update_boundary_fluxes! +
//             compute_exp_tendency! (models.jl:279-287; rre.jl:111-149,
//             214-243, 368-380; energy_hydrology.jl:273-350, 722-906)
//   stage 2   U = u + dt T_exp; Newton on U + dt T_imp(x) - x = 0 with
//             W = dt dT_imp/dY - I from make_compute_jacobian (rre.jl:391-458;
//             energy_hydrology.jl:466-576, including the "- I" on
//             d(rho e)/d(vartheta)), cache_imp! = make_update_implicit_cache
//             (models.jl:238-246; energy_hydrology.jl:427-455) run on U
//             before the first iteration and after every update, and the
//             block Thomas solve of initialize_jacobian
//             (implicit_timestepping.jl:160-171)
//   final     u_{n+1} = u + dt T_exp + dt (x - U) / dt
//
// Storage (accessed through Col<T>, a strided view; stride 32 on the
// device where 32 columns are interleaved, 1 in a host replay):
//   g*    state arrays in the internal layout. During a step they hold the
//         stage value U (the explicit stage writes U over Y; U_e = Y_e), so
//         U costs no on-chip storage; the final combination overwrites them.
//   x*    Newton iterate and Thomas arrays: per-warp shared memory
//   K, kappa, 1/rho c, face coefficients (frozen through the Newton solve),
//         the f_e residual: per-warp scratch (L2-resident global memory).
//         The last step's state writes are evict-first (Col::store_last) so
//         that the state streaming through L2 does not push the scratch out.
//
// Per Newton iteration, four sweeps:
//   1 (up)    T, psi, dpsi at x in a rolling register window; face fluxes,
//             residual, Jacobian rows and the Thomas forward elimination of
//             the vartheta block, fused;
//   2 (down)  back substitution: delta vartheta;
//   3 (up)    energy right-hand side f_e - W_ev delta vartheta, forward
//             elimination of the rho e block, x_v -= delta_v;
//   4 (down)  back substitution: delta rho e, x_e -= delta_e.
// JT is the Jacobian/Thomas type: double (plain path) or float (mixed path,
// where an FP64 column-sum projection keeps the solve's exact budget identity).
//
// Mixed-path elimination. Every column of the water and energy blocks of
// W = dt dT_imp/dY - I sums to -1 (the face fluxes telescope), plus the
// MoistureStateBC term at the top. In stiff cells (saturated soil: dpsi =
// 1/S_s) the diagonal is -(off-diagonals) - 1 with off-diagonals near 1e7, and
// the "- 1" is below float resolution, so the textbook pivot M_k - L_k c'_{k-1}
// cancels. The float path therefore carries the reduced column sums s'_k of
// the Schur complement (Grassmann-Taksar-Heyman style): s'_k = s_k -
// U_{k-1} s'_{k-1} / piv_{k-1} and piv_k = s'_k - L_{k+1}, where every term
// has one sign (U, L >= 0; s', piv < 0): no cancellation at any stiffness.
// The FP64 path keeps the reference's Thomas recurrence.
#pragma once

#include "clm_internal.cuh"
#include "clm_physics_ff.cuh"
#include "clm_atmos.cuh"

namespace clm {

template <class CM>
struct EHCol {
  double nu, K_sat, S_s, theta_r;
  CM g;  // hydrology closure (VG or BC)
  double kdry, ksf, ksu, rcds, nuom, nuq, nug, lku, lkf;
  double inv_S_s;  // 1 / S_s
};

// kLogKappaHere: take log(kappa_sat_*) from the exp/log tables instead of
// the handle's precomputed per-column array (for callers without a handle).
template <class CM, bool kLogKappaHere = false>
CLM_HD EHCol<CM> load_eh_col(const StepArgs& A, const Tables& Tb, int s, int n) {
  const int st = A.L.stride;
  const double* P = A.prm;
  EHCol<CM> c;
  c.nu = P[CLM_P_NU * st + s];
  c.K_sat = P[CLM_P_K_SAT * st + s];
  c.S_s = P[CLM_P_S_S * st + s];
  c.theta_r = P[CLM_P_THETA_R * st + s];
  c.g = make_cm<CM>(P[CLM_P_VG_ALPHA * st + s], P[CLM_P_VG_N * st + s]);
  c.kdry = P[CLM_P_KAPPA_DRY * st + s];
  c.ksf = P[CLM_P_KAPPA_SAT_FROZEN * st + s];
  c.ksu = P[CLM_P_KAPPA_SAT_UNFROZEN * st + s];
  c.rcds = P[CLM_P_RHOC_DS * st + s];
  c.nuom = P[CLM_P_NU_SS_OM * st + s];
  c.nuq = P[CLM_P_NU_SS_QUARTZ * st + s];
  c.nug = P[CLM_P_NU_SS_GRAVEL * st + s];
  if (kLogKappaHere) {
    c.lku = fm::log(Tb, c.ksu);
    c.lkf = fm::log(Tb, c.ksf);
  } else {
    c.lku = A.lkap[s];
    c.lkf = A.lkap[st + s];
  }
  c.inv_S_s = 1.0 / c.S_s;
  return c;
}

// T and psi at the Newton iterate (update_implicit_aux!,
// energy_hydrology.jl:427-445) and dpsi/dvartheta for the Jacobian (:503-512).
// inv: sat_inv(nu - ti, theta_r), fixed through the Newton solve.
template <class CM>
CLM_HD void eh_iterate_point(const Tables& Tb, const Earth& E, const EHCol<CM>& c, double xv,
                             double xe, double ti, double inv, double& T, double& psi,
                             double& D) {
  const double nu_eff = c.nu - ti;
  T = E.T_0 + (xe + ti * E.rho_i_LH_f0) * fm::rcp(heat_capacity(E, fmin(nu_eff, xv), ti, c.rcds));
  psi_dpsi_r<true>(Tb, c.g, nu_eff, inv, xv, c.theta_r, c.inv_S_s, psi, D);
}

// Mixed path: T and psi in double-float (FP64 results), dpsi in float; points
// outside the double-float range fall back to the FP64 closure.
template <class CM>
struct EHMixed {
  ff::Tables FT;
  typename ColFFOf<CM>::type cf;
  EarthFF Ef;
  F2 rcds, K_sat, omega_ln10, visc_gamma, visc_T_ref;
  KappaFF kf;
};

template <class CM>
CLM_HD EHMixed<CM> make_eh_mixed(const Tables& Tb, const Earth& E, const EHScalars& sc,
                                 const EHCol<CM>& c) {
  EHMixed<CM> m;
  m.FT = ff::Tables{Tb.ff};
  m.cf = make_col_ff(c.nu, c.theta_r, c.g);
  m.Ef = make_earth_ff(E);
  m.rcds = ff::from_double(c.rcds);
  m.K_sat = ff::from_double(c.K_sat);
  m.omega_ln10 = ff::from_double(sc.omega_ln10);
  m.visc_gamma = ff::from_double(sc.visc_gamma);
  m.visc_T_ref = ff::from_double(sc.visc_gamma_T_ref);
  m.kf = make_kappa_ff(sc, c.nu, c.kdry, c.ksu, c.ksf, c.lku, c.lkf, c.nuom, c.nuq, c.nug);
  return m;
}

template <class CM>
CLM_HD void eh_iterate_point_mixed(const Tables& Tb, const EHCol<CM>& c, const EHMixed<CM>& M, double xv,
                                   double xe, double ti, double& q, double& psi, float& D) {
  const F2 ti_f = ff::from_double(ti);
  const F2 v = ff::from_double(xv);
  const F2 nu_eff = ff::sub(M.cf.nu, ti_f);
  q = temperature_rel_ff(M.Ef, ff::from_double(xe), ti_f, ff_min(nu_eff, v), M.rcds);
  if (!psi_dpsi_ff(M.FT, M.cf, nu_eff, v, c.inv_S_s, psi, D)) {
    double d;
    psi_dpsi<true>(Tb, c.g, c.nu - ti, xv, c.theta_r, c.S_s, psi, d);
    D = (float)d;
  }
}

// The temperature, psi and dpsi at the iterate (dpsi in the Jacobian type).
// The FP64 path returns T as the reference computes it; the mixed path
// returns q = T - T_0: the residual needs only temperature differences and
// volumetric_internal_energy_liq(T) = rho c_l (T - T_0), so the mixed
// iterate's temperature is carried relative to T_0 (no rounding of T to the
// ulp of ~273 K and no subtraction of T_0). The FP64 path keeps the
// reference's sequence: columns whose phase change sits on an unstable mode
// follow differences of a few ulp in rho e_int.
template <typename JT, class CM>
CLM_HD void eh_point(const Tables& Tb, const Earth& E, const EHCol<CM>& c, const EHMixed<CM>& M, double xv,
                     double xe, double ti, double inv, double& T, double& psi, JT& D) {
  if constexpr (sizeof(JT) < sizeof(double)) {
    eh_iterate_point_mixed(Tb, c, M, xv, xe, ti, T, psi, D);
  } else {
    eh_iterate_point(Tb, E, c, xv, xe, ti, inv, T, psi, D);
  }
}

struct EHBuffers {
  Col<double> gv, gti, ge;          // state (holds U during a step)
  Col<double> xv, xe, fe;           // iterate, energy residual
  Col<double> K, kap, irc;          // frozen aux: K, face kappa / dz (after stage 1), 1 / rho c
  // mixed path: the Jacobian's face products dt K_face / dz^2, dt kappa_face /
  // dz^2 and 1 / rho c in float (p == nullptr on the FP64 path)
  Col<float> awr{nullptr, 0}, akr{nullptr, 0}, ircf{nullptr, 0};
  // face water conductance K_face / dz, precomputed per step (p == nullptr:
  // computed in every Newton iteration, the same value)
  Col<double> aw{nullptr, 0};
  // FP64 path: sat_inv(nu - theta_i, theta_r) per layer for the Newton solve
  // (p == nullptr: computed at each use)
  Col<double> iden{nullptr, 0};
  // learned Newton guess: predicted u_{n+1} - u_n of vartheta_l and rho_e_int
  // (p == nullptr: no guess)
  Col<const float> guess_v{nullptr, 0}, guess_e{nullptr, 0};
  // extrapolated guess: vartheta_l and rho_e_int at the previous step's
  // start, read for the guess u_n + (u_n - u_{n-1}) and replaced by u_n
  // (p == nullptr: no extrapolation)
  Col<double> prev_v{nullptr, 0}, prev_e{nullptr, 0};
  // resumed solve (kResume): gv, gti, ge hold the saved stage value U and the
  // final state goes to the column's own state arrays ov, oe
  Col<double> ov{nullptr, 0}, oe{nullptr, 0};
};

// FP64 <-> Jacobian-type conversions: identities on the FP64 path; on the
// mixed path integer-only ones (clm_ff.cuh), which keep the FP64 pipe for
// the arithmetic.
template <typename JT>
CLM_HD JT to_jt(double x) {
  if constexpr (sizeof(JT) < sizeof(double))
    return ff::narrow_trunc(x);
  else
    return x;
}
template <typename JT>
CLM_HD double from_jt(JT x) {
  if constexpr (sizeof(JT) < sizeof(double))
    return ff::widen_fast(x);
  else
    return x;
}

// 1 / pivot of the Thomas recurrences: the Newton-Raphson FP64 reciprocal,
// or the float quotient on the mixed path.
template <typename JT>
CLM_HD JT rcp_jt(JT x) {
  if constexpr (sizeof(JT) < sizeof(double))
    return ff::fast_div(1.0f, x);
  else
    return fm::rcp(x);
}

template <typename JT>
struct EHJac {
  Col<JT> cp, dp, d, ae;            // Thomas c', d' (then delta_v, d''), dpsi, face coef
};

// What a column's Newton solve carries from one iteration to the next
// besides its arrays (the iterate x, the stage value U and the aux frozen
// through the solve): the split Newton schedule saves it after the first
// iterations of the columns that have not converged and resumes them in a
// second launch (eh_column's Defer and kResume).
struct EHNewtonCtx {
  double Ftw, Fth, Fbw, Fbh;  // boundary fluxes at Y_n, frozen through the solve
  double UFw, UFe, xFw, xFe;  // integrated fluxes: stage value and iterate
  double R_ss, R_ess;         // TOPMODEL's subsurface water and energy sinks
  double prev_norm, prev_state2, pred2;
  int it_start;               // iterations spent before a restart from U
  int it_done;                // the last iteration run
  bool use_guess;
};

// Deferral hook of eh_column: none (every column finishes its solve where
// it started). A deferring hook has kEnabled, `at` (the first iteration
// after which an unconverged column may leave; 0: never) and
// bool operator()(const EHBuffers&, int n, const EHNewtonCtx&), which saves
// the column and returns true, or returns false (the column carries on).
struct NoDefer {
  static constexpr bool kEnabled = false;
  int at = 0;
  template <class B, class X>
  CLM_HD bool operator()(const B&, int, const X&) const { return false; }
};

// Explicit sources and top boundaries compiled into a step kernel.
constexpr int kSrcNone = 0;
constexpr int kSrcRoots = 1;  // RootExtraction (A.rx)
constexpr int kSrcAtmos = 2;  // atmosphere-driven top boundary + SoilSublimation (A.atm)

// Newton mode of a column-code instantiation: fixed iterations or
// tolerance-stopped known when compiling (the step kernels instantiate both,
// so that each carries only its own mode's code), or read from
// StepArgs::newton_mode at run time.
constexpr int kNewtonFixed = 0;
constexpr int kNewtonTol = 1;
constexpr int kNewtonRuntime = 2;

// Geom: ColGeom (uniform layers) or ColGeomS (per-layer geometry); G holds
// the column's. On a uniform column rdz(k) = dt / dz and the face means
// 0.5 (a + b) / dz are exactly (a + b) hinv_gap(k).
// Defer / kResume (tolerance mode, one step per call): with a deferring
// hook, a column that has not converged after iteration defer.at is saved
// (arrays through the hook, the rest as an EHNewtonCtx) and left without its
// final combination; kResume runs such a column from its saved context
// (*resume) to the end of the step. The two launches run the same
// arithmetic in the same order as one uninterrupted solve.
template <typename JT, class CM, bool kLogKappaHere = false, int kSrc = kSrcNone,
          int kNewton = kNewtonRuntime, class Geom = ColGeom, class Defer = NoDefer,
          bool kResume = false>
CLM_HD void eh_column(const StepArgs& A, const Tables& Tb, int s, int n, int orig,
                      const EHBuffers& B, const EHJac<JT>& J, const Geom& G, double t0,
                      double dt, int nsteps, double& Fw, double& Fe, uint32_t& flags,
                      int& iters_done, const Defer& defer = Defer{},
                      const EHNewtonCtx* resume = nullptr) {
  const Earth& E = A.E;
  const EHScalars& sc = A.sc;
  const EHCol<CM> c = load_eh_col<CM, kLogKappaHere>(A, Tb, s, n);
  const int st = A.L.stride;
  constexpr bool kStr = Geom::kStretched;
  auto rdz = [&](int k) { return dt * G.inv_width(k); };
  // mixed: the energy advection coefficient at a face, 0.5 (rho e_l(T_k) K_k
  // + rho e_l(T_k+1) K_k+1) / dz, as the sum of the layers' q K (rho c_l 0.5 / dz)
  // (on a stretched column q K rho c_l, times 0.5 / gap at the face)
  const double c_adv = kStr ? E.rhocp_l : E.rhocp_l * G.hinv_gap(0);
  constexpr bool mixed = sizeof(JT) < sizeof(double);
  EHMixed<CM> MX;
  PCCol pcc = make_pc_col(c.nu, c.theta_r, G.width(0));
  if constexpr (mixed) MX = make_eh_mixed(Tb, E, sc, c);
  // the increment norms are needed only in tolerance mode
  const bool tol = kNewton == kNewtonRuntime ? A.newton_mode == CLM_NEWTON_TOL : kNewton == kNewtonTol;
  constexpr bool kRoots = kSrc == kSrcRoots;
  constexpr bool kAtmos = kSrc == kSrcAtmos;

  bool finite = true;  // the last step's state, checked as it is stored
  for (int step = 0; step < nsteps; ++step) {
    EHNewtonCtx X;
    bool& use_guess = X.use_guess;
    double& pred2 = X.pred2;
    double &Ftw = X.Ftw, &Fth = X.Fth, &Fbw = X.Fbw, &Fbh = X.Fbh;
    double &UFw = X.UFw, &UFe = X.UFe, &xFw = X.xFw, &xFe = X.xFe;
    double &prev_norm = X.prev_norm, &prev_state2 = X.prev_state2;
    int& it_start = X.it_start;
    int it_first = 1;
    if constexpr (kResume) {
      X = *resume;
      it_first = X.it_done + 1;
    } else {
      const double t = t0 + step * dt;
      // Newton guess (tolerance mode only): Newton starts from u_n + a guessed
      // increment instead of U -- the learned guess's (guess_v, guess_e) or the
      // previous step's increment (prev_v, prev_e) -- and falls back to U when
      // its first increment is more than ten times the guessed one (a grossly
      // wrong guess; one a little worse than U still converges about as fast,
      // while a restart costs the whole warp an iteration)
      const bool extrap = B.prev_v.p != nullptr && tol;
      use_guess = extrap || (B.guess_v.p != nullptr && tol && isfinite(B.guess_v[0]) &&
                             isfinite(B.guess_e[0]));
      pred2 = 0.0;
      // ---------------- stage 1: aux at Y_n, explicit tendency, U ----------
      double K0 = 0, T0 = 0, kap0 = 0, psi0 = 0;
      double Kt = 0, Tt = 0, kapt = 0, psit = 0;
      double kap_prev = 0.0, K_prev = 0.0;
      // RootExtraction (soil_canopy_root_interactions.jl:8-39, 139-159): the
      // explicit source at Y_n and its column integrals for intF_w / intF_e
      RootCol rcol;
      if constexpr (kRoots) rcol = load_root_col(Tb, A.rx, st, s);
      double root_w = 0.0, root_e = 0.0;
      // atmosphere-driven top boundary at Y_n (update_aux values of the top
      // layers), frozen through the Newton solve
      AtmosOut ab{};
      double dz_top = 0.0;
      double sub_top = 0.0;  // SoilSublimation's theta_i tendency in the layers k >= k_sub
      int k_sub = n;
      EHRunoff ro{0.0, 0.0, 0.0, 0.0, 0.0};
      if constexpr (kAtmos) {
        auto theta_l_of = [&](int k) {
          const double Yv = B.gv[k], nu_eff = c.nu - B.gti[k];
          const double v_safe = fmax(Yv, c.theta_r + kSqrtEps);
          const double nu_safe = fmax(nu_eff, c.theta_r + kSqrtEps);
          return (v_safe < nu_safe) ? v_safe : nu_safe;
        };
        const int k1 = n - 1;
        const double Yv = B.gv[k1], Yti = B.gti[k1], Ye = B.ge[k1];
        AtmosSfc sf;
        sf.th1 = theta_l_of(k1);
        sf.th2 = theta_l_of(k1 - 1);
        sf.T = E.T_0 + (Ye + Yti * E.rho_i_LH_f0) * fm::rcp(heat_capacity(E, sf.th1, Yti, c.rcds));
        double d;
        psi_dpsi<false>(Tb, c.g, c.nu - Yti, Yv, c.theta_r, c.S_s, sf.psi, d);
        sf.Tf = tf_depressed_aux(Tb, E, c.g, c.nu, c.theta_r, sf.th1, Yti);
        sf.z1 = G.centre(k1);
        sf.z2 = G.centre(k1 - 1);
        dz_top = G.top_gap();
        sf.dz_top = dz_top;
        sf.ti = Yti;
        const AtmosRow D{A.atm, st, s};
        sf.th_alb = albedo_theta(G, D(CLM_AT_ALBEDO_TOP_THICKNESS), theta_l_of);
        // the runoff model's infiltration (and TOPMODEL's subsurface sink) from
        // the update_aux values at Y_n
        const double* P = A.prm;
        ro = eh_runoff(Tb, E, sc, A.runoff, G, c.nu, c.theta_r, c.K_sat, P[CLM_P_F_MAX * st + s],
                       P[CLM_P_F_OVER * st + s], P[CLM_P_R_SB * st + s], sf.th1, D(CLM_AT_P_LIQ),
                       [&](int k, double& v, double& ti, double& T) {
                         v = B.gv[k];
                         ti = B.gti[k];
                         T = E.T_0 + (B.ge[k] + ti * E.rho_i_LH_f0) *
                                         fm::rcp(heat_capacity(E, theta_l_of(k), ti, c.rcds));
                       });
        sf.infil = ro.infil;
        ab = atmos_bc(Tb, A.ak, E, D, c.g, c.nu, c.theta_r, sf);
        // H(z_k + 2 dz_top) rises with k: the source reaches the layers from
        // k_sub up (the top layer alone for a surface at z = 0)
        while (k_sub > 0 && sublimation_weight(G, k_sub - 1, dz_top) != 0.0) --k_sub;
        sub_top = -ab.vice * E.rho_l / E.rho_i / (2.0 * dz_top);
      }
      for (int k = 0; k < n; ++k) {
        const double Yv = B.gv[k], Yti = B.gti[k], Ye = B.ge[k];
        const double nu_eff = c.nu - Yti;
        // volumetric_liquid_fraction (soil_hydrology_parameterizations.jl:22-31)
        const double v_safe = fmax(Yv, c.theta_r + kSqrtEps);
        const double nu_safe = fmax(nu_eff, c.theta_r + kSqrtEps);
        const double tl = (v_safe < nu_safe) ? v_safe : nu_safe;
        const double rc = heat_capacity(E, tl, Yti, c.rcds);
        // thermal_time's 1 / (3 dz^2) of this layer
        if constexpr (kStr) pcc.inv_3dz2 = fm::rcp(3.0 * (G.width(k) * G.width(k)));
        // one reciprocal of rho c for T and the phase change
        const double inv_rc = fm::rcp(rc);
        const double T = E.T_0 + (Ye + Yti * E.rho_i_LH_f0) * inv_rc;
        double kap = 0.0, K = 0.0;
        bool aux_ff = false;
        if constexpr (mixed) {
          // kappa and K in double-float
          const F2 tl_f = ff::from_double(tl), ti_f = ff::from_double(Yti);
          const F2 guard = ff::add_f(MX.cf.theta_r, 1.4901161193847656e-08f);
          const F2 S = ff::div(ff::sub(ff_max(ff::from_double(Yv), guard), MX.cf.theta_r),
                               ff::sub(ff_max(MX.cf.nu, guard), MX.cf.theta_r));
          // f_i = 0 without the division only where theta_i is exactly 0 (a
          // negative theta_i gives the reference's f_i < 0)
          const F2 fi = Yti != 0.0 ? ff::div(ti_f, ff::sub(ff::add(tl_f, ti_f), MX.cf.theta_r))
                                  : ff::make(0.0f);
          const F2 lnf = ff::add(ff::neg(ff::mul(MX.omega_ln10, fi)),
                                 ff::mul(MX.visc_gamma, ff::sub(ff::from_double(T), MX.visc_T_ref)));
          aux_ff = kappa_ff(MX.FT, MX.kf, tl, Yti, tl_f, ti_f, kap) &&
                   conductivity_ff(MX.FT, MX.cf, MX.K_sat, S, lnf, K);
        }
        if (!aux_ff) {
          kap = conductivity_heat(Tb, sc, tl, Yti, c.nu, c.kdry, c.ksu, c.ksf, c.lku, c.lkf, c.nuom,
                                  c.nuq, c.nug);
          const double SK = saturation_r(pcc.inv_den, Yv, c.theta_r);
          const double fi = Yti != 0.0 ? Yti / (tl + Yti - c.theta_r) : 0.0;
          // impedance_factor * viscosity_factor * hydraulic_conductivity, with
          // the sqrt(S) of the van Genuchten K inside the same exponential
          const double lnf = -sc.omega_ln10 * fi + sc.visc_gamma * (T - sc.visc_gamma_T_ref);
          K = conductivity_scaled(Tb, c.g, c.K_sat, SK, lnf);
        }
        double Uv = Yv, Uti = Yti, Ue = Ye;
        double pc = 0.0;
        if (A.phase_change) {
          pc = mixed ? phase_change_reduced(Tb, E, c.g, c.nu, c.theta_r, pcc, tl, Yti, T, inv_rc, kap)
                     : phase_change_r(Tb, E, c.g, c.nu, c.theta_r, pcc, tl, Yti, T, inv_rc, kap, flags);
          Uv = Yv + dt * (-pc);
          Uti = Yti + dt * (E.rho_l_over_rho_i * pc);
        }
        if constexpr (kAtmos) {
          // SoilSublimation after PhaseChange in the sources tuple
          const double sub = k >= k_sub ? sub_top : 0.0;
          Uti = Yti + dt * ((A.phase_change ? E.rho_l_over_rho_i * pc : 0.0) + sub);
        }
        if constexpr (kRoots) {
          // psi at Y_n (update_aux!), the layer centre z, K and T of this stage
          double psi_n, d;
          psi_dpsi<false>(Tb, c.g, nu_eff, Yv, c.theta_r, c.S_s, psi_n, d);
          const double re = root_rate(Tb, rcol, G.face_centre(k), psi_n, K);
          const double ree = re * rho_e_liq(E, T);
          Uv = Yv + dt * ((-pc) + (-1.0 * re));  // sources in the reference's order
          Ue = Ye + dt * (-1.0 * ree);
          root_e += G.width(k) * ree;
          root_w += G.width(k) * re;
          B.ge[k] = Ue;
        }
        B.gv[k] = Uv;
        B.gti[k] = Uti;
        if constexpr (kAtmos) {
          // TOPMODEL's implicit subsurface sink, constant through the Newton
          // solve: part of the residual's U + dt T_imp, not of the start x = U
          if (ro.cw != 0.0 || ro.ce != 0.0) {
            const double w = sat_weight(Yv - c.theta_r, c.nu - c.theta_r);
            B.gv[k] = Uv - dt * (ro.cw * w);
            B.ge[k] = Ue - dt * (ro.ce * w);
          }
        }
        if constexpr (!mixed)
          if (B.iden.p) B.iden[k] = sat_inv(c.nu - Uti, c.theta_r);
        if (use_guess) {
          double gv, ge;
          if (extrap) {
            gv = Yv - B.prev_v[k];
            ge = Ye - B.prev_e[k];
            // read again by the next step: evict-first when that is another
            // launch, kept in cache when it is this column's next step here
            if (nsteps == 1) {
              B.prev_v.store_last(k, Yv);
              B.prev_e.store_last(k, Ye);
            } else {
              B.prev_v[k] = Yv;
              B.prev_e[k] = Ye;
            }
          } else {
            gv = (double)B.guess_v[k];
            ge = (double)B.guess_e[k];
          }
          double xv0 = Yv + gv, xe0 = Ye + ge;
          // a zero guessed increment carries no information (the first step
          // of a history): the layer starts from U
          if (gv == 0.0 && ge == 0.0) {
            xv0 = Uv;
            xe0 = Ue;
          }
          // a layer whose guess leaves the retention curve's domain
          // (vartheta_l <= theta_r) or is not finite starts from U
          if (!(xv0 > c.theta_r + kSqrtEps) || !isfinite(xv0)) xv0 = Uv;
          if (!isfinite(xe0)) xe0 = Ue;
          B.xv[k] = xv0;
          B.xe[k] = xe0;
          const double dv = xv0 - Uv, de = A.energy_scale * (xe0 - Ue);
          pred2 += dv * dv + de * de;
        } else {
          B.xv[k] = Uv;
          B.xe[k] = Ue;
        }
        B.K[k] = K;
        // face conductances k-1|k, frozen through the Newton solve: kappa on
        // the face into kappa's slot (the cell value is not used after stage 1)
        if (k > 0) {
          const double ak = (kap_prev + kap) * G.hinv_gap(k - 1);
          const double aw = (K_prev + K) * G.hinv_gap(k - 1);
          B.kap[k - 1] = ak;
          if (B.aw.p) B.aw[k - 1] = aw;
          if constexpr (mixed) {
            // the float rows' face products: dt K_face / (dz gap) (uniform:
            // W's own rows), or dt K_face / gap (stretched: W's rows times the
            // layer width)
            const double fac = kStr ? dt : rdz(k - 1);
            B.awr[k - 1] = ff::narrow_trunc(fac * aw);
            B.akr[k - 1] = ff::narrow_trunc(fac * ak);
          }
        }
        kap_prev = kap;
        K_prev = K;
        if constexpr (mixed)
          B.ircf[k] = 1.0f / ff::narrow_trunc(heat_capacity(E, tl, Uti, c.rcds));
        else
          B.irc[k] = fm::rcp(heat_capacity(E, tl, Uti, c.rcds));
        if (k == 0) {
          K0 = K; T0 = T; kap0 = kap;
          if (A.bc_bw == CLM_BC_STATE) {
            double d;
            psi_dpsi<false>(Tb, c.g, nu_eff, Yv, c.theta_r, c.S_s, psi0, d);
          }
        }
        if (k == n - 1) {
          Kt = K; Tt = T; kapt = kap;
          if (A.bc_tw == CLM_BC_STATE) {
            double d;
            psi_dpsi<false>(Tb, c.g, nu_eff, Yv, c.theta_r, c.S_s, psit, d);
          }
        }
      }
      // boundary fluxes at t, frozen through the Newton solve
      {
        const double ftw = forcing_value(A.forc[CLM_BC_TOP_WATER], st, s, A.col0 + orig, t, A.seed);
        const double fth = forcing_value(A.forc[CLM_BC_TOP_HEAT], st, s, A.col0 + orig, t, A.seed);
        const double fbw = forcing_value(A.forc[CLM_BC_BOTTOM_WATER], st, s, A.col0 + orig, t, A.seed);
        const double fbh = forcing_value(A.forc[CLM_BC_BOTTOM_HEAT], st, s, A.col0 + orig, t, A.seed);
        if (kAtmos) {
          Ftw = ab.top_w;
        } else if (A.bc_tw == CLM_BC_STATE) {
          double pb, d;
          psi_dpsi<false>(Tb, c.g, c.nu, ftw, c.theta_r, c.S_s, pb, d);
          Ftw = -Kt * ((pb + G.half_top()) - psit) / G.half_top();  // diffusive_flux
        } else {
          Ftw = ftw;
        }
        if (A.bc_bw == CLM_BC_FREE_DRAINAGE) {
          Fbw = -1.0 * K0;
        } else if (A.bc_bw == CLM_BC_STATE) {
          double pb, d;
          psi_dpsi<false>(Tb, c.g, c.nu, fbw, c.theta_r, c.S_s, pb, d);
          Fbw = -K0 * ((psi0 + G.half_bot()) - pb) / G.half_bot();
        } else {
          Fbw = fbw;
        }
        if (kAtmos) {
          Fth = ab.top_h;
        } else if (A.bc_th == CLM_BC_STATE) {
          Fth = -kapt * (fth - Tt) / G.half_top();
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
          Fbh = -kap0 * (T0 - fbh) / G.half_bot();
        } else {
          Fbh = fbh;
        }
      }
      UFw = kRoots ? Fw + dt * root_w : kAtmos ? Fw + dt * (0.0 + -ab.vice) : Fw;
      UFe = kRoots ? Fe + dt * root_e : Fe;
      xFw = UFw;
      xFe = UFe;
      X.R_ss = ro.R_ss;
      X.R_ess = ro.R_ess;

      // ---------------- stage 2: Newton ------------------------------------
      prev_norm = 1e300;
      // a guess that moved no layer off U is no guess: plain start, plain test
      if (use_guess && !(pred2 > 0.0)) use_guess = false;
      prev_state2 = 0.0;  // the state increments' norm of the last iteration (guess test)
      it_start = 0;       // iterations spent before a restart from U
    }  // !kResume
    bool deferred = false;
    for (int it = it_first; it <= A.max_iters; ++it) {
      // sweep 1 (bottom -> top)
      JT cp_prev = 0, dp_prev = 0;
      JT U_prev = 0, sp_prev = -1, piv_prev = -1;  // mixed: reduced column sums
      double Fw_dn = Fbw, Fe_dn = Fbh;
      double aw_dn = 0.0;
      JT awr_dn = 0;  // mixed: dt K_face / dz^2 of the face below
      JT D_prev = 0;
      double sum_fv = 0.0, sum_fe = 0.0;
      double Tc, psic;  // Tc, Tn: T (FP64 path) or T - T_0 (mixed) at the iterate
      JT Dc;
      auto inv_of = [&](int k) {  // FP64 path: the layer's sat_inv
        if constexpr (mixed) return 0.0;
        else return B.iden.p ? B.iden[k] : sat_inv(c.nu - B.gti[k], c.theta_r);
      };
      eh_point<JT, CM>(Tb, E, c, MX, B.xv[0], B.xe[0], B.gti[0], inv_of(0), Tc, psic, Dc);
      double Kc = B.K[0];
      double relKc = mixed ? Tc * (Kc * c_adv) : rho_e_liq(E, Tc) * Kc;
      for (int k = 0; k < n; ++k) {
        double Fw_up, Fe_up, aw_up = 0.0, ae_up = 0.0;
        double Tn = 0, psin = 0, Kn = 0, relKn = 0;
        JT Dn = 0, awr_up = 0;
        if (k < n - 1) {
          eh_point<JT, CM>(Tb, E, c, MX, B.xv[k + 1], B.xe[k + 1], B.gti[k + 1], inv_of(k + 1), Tn,
                           psin, Dn);
          Kn = B.K[k + 1];
          relKn = mixed ? Tn * (Kn * c_adv) : rho_e_liq(E, Tn) * Kn;
          aw_up = B.aw.p ? B.aw[k] : (Kc + Kn) * G.hinv_gap(k);
          const double ak_up = B.kap[k];  // face k|k+1 (stage 1)
          ae_up = (mixed && !kStr) ? relKc + relKn : (relKc + relKn) * G.hinv_gap(k);
          const double dh = (psin - psic) + G.gap(k);
          Fw_up = -aw_up * dh;
          Fe_up = -ak_up * (Tn - Tc) - ae_up * dh;
          if constexpr (mixed) awr_up = B.awr[k];
        } else {
          Fw_up = Ftw;
          Fe_up = Fth;
        }
        double fv, fe;
        if constexpr (mixed) {
          // U + dt T - x with dt T = rdz (F_dn - F_up): one rounding fewer
          fv = (B.gv[k] - B.xv[k]) + rdz(k) * (Fw_dn - Fw_up);
          fe = (B.ge[k] - B.xe[k]) + rdz(k) * (Fe_dn - Fe_up);
        } else {
          const double Tv = -((Fw_up - Fw_dn) * G.inv_width(k));
          const double Tee = -((Fe_up - Fe_dn) * G.inv_width(k));
          fv = B.gv[k] + dt * Tv - B.xv[k];
          fe = B.ge[k] + dt * Tee - B.xe[k];
        }
        // the mixed path's weighted sums (row weight 1 on a uniform column)
        sum_fv += G.row_w(k) * fv;
        sum_fe += G.row_w(k) * fe;
        JT L, U, Md;
        if constexpr (mixed) {  // rows from the float face products
          L = awr_dn * D_prev;
          U = awr_up * Dn;
          Md = -(awr_up + awr_dn) * Dc - 1.0f;
        } else {
          L = (JT)(rdz(k) * aw_dn) * D_prev;
          U = (k < n - 1) ? (JT)(rdz(k) * aw_up * Dn) : (JT)0;
          Md = (JT)(-rdz(k) * (aw_up + aw_dn) * Dc - 1.0);
        }
        JT piv;
        if constexpr (mixed) {
          // the column sum of row k's block column: -(row weight)
          const JT wk = kStr ? (JT)G.row_w(k) : (JT)1;
          const JT sp = (k == 0) ? -wk : -wk - U_prev * (sp_prev / piv_prev);
          piv = sp - awr_up * Dc;  // L_{k+1} = dt K_face(k|k+1) / dz^2 dpsi_k
          U_prev = U;
          sp_prev = sp;
          piv_prev = piv;
        } else {
          piv = Md - L * cp_prev;
        }
        const JT inv = rcp_jt(piv);
        const JT cpk = U * inv;
        const JT dpk = (to_jt<JT>(kStr && mixed ? G.row_w(k) * fv : fv) - L * dp_prev) * inv;
        J.cp[k] = cpk;
        J.dp[k] = dpk;
        J.d[k] = Dc;
        J.ae[k] = to_jt<JT>(ae_up);
        B.fe[k] = fe;
        cp_prev = cpk;
        dp_prev = dpk;
        Fw_dn = Fw_up;
        Fe_dn = Fe_up;
        aw_dn = aw_up;
        awr_dn = awr_up;
        D_prev = Dc;
        Tc = Tn; psic = psin; Dc = Dn; Kc = Kn; relKc = relKn;
      }
      // integrated fluxes (their Jacobian block is -I): x += f
      const double fFw = UFw + dt * ((-(Ftw - Fbw)) - X.R_ss) - xFw;
      const double fFe = UFe + dt * ((-(Fth - Fbh)) - X.R_ess) - xFe;
      xFw += fFw;
      xFe += fFe;
      // sweep 2 (top -> bottom): delta vartheta into dp
      double sdv = 0.0;
      {
        JT nxt = 0;
        for (int k = n - 1; k >= 0; --k) {
          const JT d = J.dp[k] - J.cp[k] * nxt;
          J.dp[k] = d;
          nxt = d;
          if (mixed) sdv += G.row_w(k) * from_jt<JT>(d);
        }
      }
      // FP64 column-sum projection (mixed path): sum(w delta_v) = -sum(w f_v)
      const double corr_v = mixed ? (sdv + sum_fv) / G.wsum() : 0.0;
      const double flux2 = fFw * fFw + fFe * fFe;  // integrated fluxes
      double state2 = 0.0;                           // state increments
      // mixed path: the state increments' squares summed in float from the
      // float increments (the tolerance test needs a few digits of the norm;
      // the FP64 pipe is the mixed step's bound)
      float state2f = 0.0f;
      // sweep 3 (bottom -> top): energy right-hand side, rho e forward
      // elimination (c'' into cp, d'' into dp behind the read of delta_v)
      {
        JT c_prev = 0, d_prev = 0;
        JT U_prev = 0, sp_prev = -1, piv_prev = -1;  // mixed: reduced column sums
        double ak_dn = 0.0;
        JT akr_dn = 0;
        JT dvm = 0, Dm = 0;
        JT dv0 = J.dp[0] - (JT)corr_v, D0 = J.d[0];
        // the applied increment in FP64, so that the increments sum to
        // -sum(f_v) to FP64 rounding (the water budget identity)
        double dvd0 = from_jt<JT>(J.dp[0]) - corr_v;
        JT ae_dn = 0;
        double irc_c = 0.0, irc_m = 0.0;
        JT ircf_c = 0, ircf_m = 0;
        if constexpr (mixed)
          ircf_c = B.ircf[0];
        else
          irc_c = B.irc[0];
        for (int k = 0; k < n; ++k) {
          JT dvp = 0, Dp = 0, ae_up = 0;
          double dvdp = 0.0;
          double ak_up = 0.0, irc_n = 0.0;
          JT akr_up = 0, ircf_n = 0;
          if (k < n - 1) {
            dvp = J.dp[k + 1] - (JT)corr_v;
            dvdp = from_jt<JT>(J.dp[k + 1]) - corr_v;
            Dp = J.d[k + 1];
            ae_up = J.ae[k];
            if constexpr (mixed) {
              akr_up = B.akr[k];
              ircf_n = B.ircf[k + 1];
            } else {
              ak_up = B.kap[k];  // face k|k+1 (stage 1)
              irc_n = B.irc[k + 1];
            }
          }
          const JT Gup = (k < n - 1) ? (Dp * dvp - D0 * dv0) : (JT)0;
          const JT Gdn = (k > 0) ? (D0 * dv0 - Dm * dvm) : (JT)0;
          const JT wev = (JT)rdz(k) * (ae_up * Gup - ae_dn * Gdn) - dv0;
          const double g = B.fe[k] - from_jt<JT>(wev);
          JT L, U, Md;
          if constexpr (mixed) {
            L = akr_dn * ircf_m;
            U = akr_up * ircf_n;
            Md = -(akr_up + akr_dn) * ircf_c - 1.0f;
          } else {
            L = (JT)(rdz(k) * ak_dn * irc_m);
            U = (JT)(rdz(k) * ak_up * irc_n);
            Md = (JT)(-rdz(k) * (ak_up + ak_dn) * irc_c - 1.0);
          }
          JT piv;
          if constexpr (mixed) {
            const JT wk = kStr ? (JT)G.row_w(k) : (JT)1;
            const JT sp = (k == 0) ? -wk : -wk - U_prev * (sp_prev / piv_prev);
            piv = sp - akr_up * ircf_c;  // L_{k+1} = dt kappa_face(k|k+1) / dz^2 / rho c_k
            U_prev = U;
            sp_prev = sp;
            piv_prev = piv;
          } else {
            piv = Md - L * c_prev;
          }
          const JT inv = rcp_jt(piv);
          const JT ck = U * inv;
          const JT dk = (to_jt<JT>(kStr && mixed ? G.row_w(k) * g : g) - L * d_prev) * inv;
          J.cp[k] = ck;
          J.dp[k] = dk;
          c_prev = ck;
          d_prev = dk;
          const double dvd = dvd0;
          B.xv[k] -= dvd;
          if (tol) {
            if constexpr (mixed)
              state2f = fmaf(dv0, dv0, state2f);
            else
              state2 += dvd * dvd;
          }
          dvm = dv0; Dm = D0; dv0 = dvp; D0 = Dp;
          dvd0 = dvdp;
          ae_dn = ae_up;
          ak_dn = ak_up;
          akr_dn = akr_up;
          irc_m = irc_c; irc_c = irc_n;
          ircf_m = ircf_c; ircf_c = ircf_n;
        }
      }
      // sweep 4 (top -> bottom): delta rho e
      {
        const double se = A.energy_scale;
        JT nxt = 0;
        if (mixed) {
          double sde = 0.0;
          for (int k = n - 1; k >= 0; --k) {
            const JT d = J.dp[k] - J.cp[k] * nxt;
            J.dp[k] = d;
            sde += G.row_w(k) * from_jt<JT>(d);
            nxt = d;
          }
          // W_ee and W_ev + I have zero (width-weighted) column sums:
          // sum(w delta_e) = -sum(w f_e) - sum(w delta_v) = -sum(w f_e) + sum(w f_v)
          const double corr_e = (sde + sum_fe - sum_fv) / G.wsum();
          const float cef = ff::narrow_trunc(corr_e), sef = ff::narrow_trunc(se);
          for (int k = 0; k < n; ++k) {
            const double d = from_jt<JT>(J.dp[k]) - corr_e;
            B.xe[k] -= d;
            if (tol) {
              const float df = (J.dp[k] - cef) * sef;
              state2f = fmaf(df, df, state2f);
            }
          }
          state2 = ff::widen_fast(state2f);
        } else {
          for (int k = n - 1; k >= 0; --k) {
            const JT d = J.dp[k] - J.cp[k] * nxt;
            nxt = d;
            B.xe[k] -= (double)d;
            if (tol) state2 += (se * (double)d) * (se * (double)d);
          }
        }
      }
      iters_done = it;
      if (tol) {
        const double nrm = sqrt(flux2 + state2);
        // the guess is abandoned (restart from x = U) when its first
        // increment is more than ten times the guessed one, or when Newton
        // from it stops contracting or leaves the finite numbers; the tests
        // use the state part only (the integrated-flux increments do not
        // depend on the starting point)
        const bool drop_guess =
            use_guess && (it == 1 ? !(state2 <= 100.0 * pred2) && !(sqrt(state2) < A.tol)
                                  : !(state2 < prev_state2));
        if (drop_guess) {
          for (int k = 0; k < n; ++k) {
            B.xv[k] = B.gv[k];
            B.xe[k] = B.ge[k];
          }
          use_guess = false;
          flags |= CLM_COL_GUESS_FALLBACK;
          prev_norm = 1e300;
          it_start = it;
          // split Newton: the restart from U runs in the resuming launch
          if constexpr (Defer::kEnabled) {
            if (defer.at > 0 && it >= defer.at && it < A.max_iters) {
              X.it_done = it;
              if (defer(B, n, X)) {
                deferred = true;
                break;
              }
            }
          }
          continue;
        }
        prev_state2 = state2;
        if (nrm > prev_norm && it - it_start > 2) flags |= CLM_COL_DIVERGED;
        prev_norm = nrm;
        // with a guess, the integrated fluxes start from their value at the
        // guessed state (U_F + dt T_F(x0)): their first increment is that
        // start-up, not a Newton correction, and stays out of the test
        const double conv = (use_guess && it == 1) ? sqrt(state2) : nrm;
        if (conv < A.tol) break;
        if (it == A.max_iters) flags |= CLM_COL_NOT_CONVERGED;
        // split Newton: an unconverged column leaves after iteration
        // defer.at (or the first one after it that ends in this test) with
        // its context saved; it finishes in the resuming launch
        if constexpr (Defer::kEnabled) {
          if (defer.at > 0 && it >= defer.at && it < A.max_iters) {
            X.it_done = it;
            if (defer(B, n, X)) {
              deferred = true;
              break;
            }
          }
        }
      }
    }
    // ---------------- final combination ---------------------------------
    // (not for a deferred column: its solve ends in the resuming launch; a
    // deferring hook is used with one step per call, so the step loop needs
    // no second exit)
    if (!deferred) {
      const double inv_dt = 1.0 / dt;
      const bool last = step == nsteps - 1;
      const Col<double> OV = kResume ? B.ov : B.gv, OE = kResume ? B.oe : B.ge;
      for (int k = 0; k < n; ++k) {
        const double Uv = B.gv[k], Ue = B.ge[k];
        const double v = Uv + dt * ((B.xv[k] - Uv) * inv_dt);
        const double e = Ue + dt * ((B.xe[k] - Ue) * inv_dt);
        if (last) {
          OV.store_last(k, v);
          OE.store_last(k, e);
          finite = finite && isfinite(v) && isfinite(B.gti[k]) && isfinite(e);
        } else {
          OV[k] = v;
          OE[k] = e;
        }
      }
      Fw = UFw + dt * ((xFw - UFw) * inv_dt);
      Fe = UFe + dt * ((xFe - UFe) * inv_dt);
    }  // !deferred
  }
  finite = finite && isfinite(Fw) && isfinite(Fe);
  if (!finite) flags |= CLM_COL_NONFINITE;
}

// ---------------------------------------------------------------------------
// RichardsModel
// ---------------------------------------------------------------------------

struct RBuffers {
  Col<double> gv;   // state (U = u during a step: no explicit tendency)
  Col<double> xv;   // iterate
};

template <typename JT>
struct RJac {
  Col<JT> cp, dp;
  // mixed path: low words of the double-float right-hand side recurrence
  // (the residual is not rounded to float: in stiff columns it is far
  // larger than the smooth modes of the solution)
  Col<JT> dpl{nullptr, 0};
};

template <typename JT, class CM, class Geom = ColGeom>
CLM_HD void richards_column(const StepArgs& A, const Tables& Tb, int s, int n, int orig,
                            const RBuffers& B, const RJac<JT>& J, const Geom& G, double t0,
                            double dt, int nsteps, double& Fw, uint32_t& flags,
                            int& iters_done) {
  const int st = A.L.stride;
  const double* P = A.prm;
  const double nu = P[CLM_P_NU * st + s];
  const double K_sat = P[CLM_P_K_SAT * st + s];
  const double S_s = P[CLM_P_S_S * st + s];
  const double theta_r = P[CLM_P_THETA_R * st + s];
  const CM g = make_cm<CM>(P[CLM_P_VG_ALPHA * st + s], P[CLM_P_VG_N * st + s]);
  const double inv = sat_inv(nu, theta_r), inv_S_s = 1.0 / S_s;
  auto rdz = [&](int k) { return dt * G.inv_width(k); };
  constexpr bool kStr = Geom::kStretched;
  constexpr bool mixed = sizeof(JT) < sizeof(double);
  // mixed path: K, psi and dpsi in double-float (FP64 closure where it declines)
  typename ColFFOf<CM>::type cf;
  F2 K_sat_f;
  if constexpr (mixed) {
    cf = make_col_ff(nu, theta_r, g);
    K_sat_f = ff::from_double(K_sat);
  }
  const ff::Tables FT{Tb.ff};
  auto point = [&](double xv, double& K, double& psi, double& D) {
    if constexpr (mixed) {
      float d;
      if (richards_point_ff(FT, cf, K_sat_f, ff::from_double(xv), K, psi, d)) {
        D = d;
        return;
      }
    }
    richards_point<true>(Tb, g, nu, inv, xv, theta_r, inv_S_s, K_sat, K, psi, D);
  };
  // MoistureStateBC at the top carries dfluxBCdY (rre.jl:137-146, 460-468):
  // the boundary fluxes are then refreshed with the implicit cache.
  const bool dflux = (A.bc_tw == CLM_BC_STATE);
  const bool tol = A.newton_mode == CLM_NEWTON_TOL;  // the increment norm is needed only then

  for (int step = 0; step < nsteps; ++step) {
    const double t = t0 + step * dt;
    for (int k = 0; k < n; ++k) B.xv[k] = B.gv[k];
    const double UFw = Fw;
    double xFw = UFw;
    const double t_bc = dflux ? t + dt : t;
    const double ftw = forcing_value(A.forc[CLM_BC_TOP_WATER], st, s, A.col0 + orig, t_bc, A.seed);
    const double fbw = forcing_value(A.forc[CLM_BC_BOTTOM_WATER], st, s, A.col0 + orig, t_bc, A.seed);
    double psi_tb = 0.0, psi_bb = 0.0;
    if (A.bc_tw == CLM_BC_STATE) { double d; psi_dpsi<false>(Tb, g, nu, ftw, theta_r, S_s, psi_tb, d); }
    if (A.bc_bw == CLM_BC_STATE) { double d; psi_dpsi<false>(Tb, g, nu, fbw, theta_r, S_s, psi_bb, d); }
    // without dfluxBCdY the fluxes are those of the explicit stage at (u, t);
    // U = u, so iteration 1 (x = U) evaluates exactly those
    double Ftw = ftw, Fbw = fbw;
    // RichardsAtmosDrivenFluxBC (boundary_conditions.jl:200-212): the runoff
    // model (Runoff.jl) turns the precipitation ftw into the infiltration at
    // (u, t); TOPMODEL adds the implicit subsurface sink (Runoff.jl:321-345)
    // R_ss / max(h_sat, eps) on the saturated layers, not in the Jacobian.
    // All of it is frozen through the Newton solve.
    double R_ss = 0.0, q_sink = 0.0;
    const double nr = nu - theta_r;
    if (A.bc_tw == CLM_BC_PRECIP_RUNOFF) {
      const double ic = -1.0 * K_sat;  // soil_infiltration_capacity (Runoff.jl:386-399)
      if (A.runoff == CLM_RUNOFF_SURFACE) {
        const double is_sat = ((B.gv[n - 1] + 0.0) - nu) > kEps ? 1.0 : 0.0;
        Ftw = (1.0 - is_sat) * fmax(ic, ftw);
      } else if (A.runoff == CLM_RUNOFF_TOPMODEL) {
        double h = 0.0;  // column_integral_definite of the saturation weights
        for (int k = 0; k < n; ++k) {
          const double twc = B.gv[k] + 0.0 - theta_r;
          h += G.width(k) * ((twc - nr > kEps ? 1.0 : 0.0) * twc / nr);
        }
        const double zwt = (G.zhi - G.zlo) - h;
        const double f_sat = fmin(P[CLM_P_F_MAX * st + s] *
                                      fm::exp(Tb, -P[CLM_P_F_OVER * st + s] / 2.0 * zwt), 1.0);
        Ftw = (1.0 - f_sat) * fmax(ic, ftw);
        R_ss = P[CLM_P_R_SB * st + s] * fm::exp(Tb, -P[CLM_P_F_OVER * st + s] * zwt);
        q_sink = R_ss / fmax(h, kEps);
      }
    }
    double prev_norm = 1e300;
    for (int it = 1; it <= A.max_iters; ++it) {
      const bool refresh_bc = dflux || it == 1;
      JT cp_prev = 0, dp_prev = 0;
      JT U_prev = 0, sp_prev = -1, piv_prev = -1;  // mixed: reduced column sums
      F2 dpf_prev = ff::make(0.0f);                // mixed: double-float d'
      double aw_dn = 0.0;
      JT D_prev = 0;
      double sum_f = 0.0;
      double Kc, psic, Dc;
      point(B.xv[0], Kc, psic, Dc);
      if (refresh_bc) {
        if (A.bc_bw == CLM_BC_FREE_DRAINAGE) Fbw = -1.0 * Kc;
        else if (A.bc_bw == CLM_BC_STATE) Fbw = -Kc * ((psic + G.half_bot()) - psi_bb) / G.half_bot();
      }
      double Fw_dn = Fbw;
      for (int k = 0; k < n; ++k) {
        double Fw_up, aw_up = 0.0;
        double Kn = 0, psin = 0, Dn = 0;
        double Md_extra = 0.0;
        if (k < n - 1) {
          point(B.xv[k + 1], Kn, psin, Dn);
          aw_up = 0.5 * (Kc + Kn) * (2.0 * G.hinv_gap(k));
          Fw_up = -aw_up * ((psin - psic) + G.gap(k));
        } else {
          const double half = G.half_top();
          if (refresh_bc && A.bc_tw == CLM_BC_STATE) Ftw = -Kc * ((psi_tb + half) - psic) / half;
          // set_dfluxBCdY! (boundary_conditions.jl:375-426): K_N dpsi_N / dz_top;
          // the mixed path's weighted row (stretched) takes it without the 1 / dz
          if (dflux) Md_extra = (kStr && mixed) ? -dt * (Kc * Dc / half)
                                                : -dt * ((Kc * Dc / half) * G.inv_width(k));
          Fw_up = Ftw;
        }
        double Tv = -((Fw_up - Fw_dn) * G.inv_width(k));
        if (q_sink != 0.0) {
          const double twc = B.gv[k] + 0.0 - theta_r;  // U = u for Richards
          Tv -= q_sink * ((twc - nr > kEps ? 1.0 : 0.0) * twc / nr);
        }
        const double f = B.gv[k] + dt * Tv - B.xv[k];
        sum_f += G.row_w(k) * f;
        // rows of W; the mixed path on a stretched column uses W's rows times
        // the layer width (face products dt K_face / gap), whose block
        // columns sum to -width
        const double rk = (kStr && mixed) ? dt : rdz(k);
        const JT L = (JT)(rk * aw_dn) * D_prev;
        const JT U = (k < n - 1) ? (JT)(rk * aw_up * Dn) : (JT)0;
        const JT M = (JT)(-rdz(k) * (aw_up + aw_dn) * Dc - 1.0 + Md_extra);
        JT piv;
        if constexpr (mixed) {
          // column sum -1 (+ the MoistureStateBC term of the top column)
          const JT s_k = (JT)(-G.row_w(k) + Md_extra);
          const JT sp = (k == 0) ? s_k : s_k - U_prev * (sp_prev / piv_prev);
          piv = sp - ((k < n - 1) ? (JT)(rk * aw_up) * (JT)Dc : (JT)0);  // L_{k+1}
          U_prev = U;
          sp_prev = sp;
          piv_prev = piv;
        } else {
          piv = M - L * cp_prev;
        }
        const JT inv = rcp_jt(piv);
        const JT cpk = U * inv;
        J.cp[k] = cpk;
        if constexpr (mixed) {
          const F2 dpf = ff::mul_f(ff::sub(ff::from_double(kStr ? G.row_w(k) * f : f), ff::mul_f(dpf_prev, L)), inv);
          J.dp[k] = dpf.hi;
          J.dpl[k] = dpf.lo;
          dpf_prev = dpf;
        } else {
          const JT dpk = ((JT)f - L * dp_prev) * inv;
          J.dp[k] = dpk;
          dp_prev = dpk;
        }
        cp_prev = cpk;
        Fw_dn = Fw_up;
        aw_dn = aw_up;
        D_prev = (JT)Dc;
        Kc = Kn; psic = psin; Dc = Dn;
      }
      const double fFw = UFw + dt * ((-(Ftw - Fbw)) - R_ss) - xFw;
      xFw += fFw;
      double norm2 = fFw * fFw;
      if constexpr (mixed) {
        F2 nxt = ff::make(0.0f);
        double sd = 0.0;
        for (int k = n - 1; k >= 0; --k) {
          const F2 d = ff::sub(F2{J.dp[k], J.dpl[k]}, ff::mul_f(nxt, J.cp[k]));
          J.dp[k] = d.hi;
          J.dpl[k] = d.lo;
          sd += G.row_w(k) * ff::to_double(d);
          nxt = d;
        }
        const double corr = dflux ? 0.0 : (sd + sum_f) / G.wsum();
        for (int k = 0; k < n; ++k) {
          const double d = ff::to_double(F2{J.dp[k], J.dpl[k]}) - corr;
          B.xv[k] -= d;
          if (tol) norm2 += d * d;
        }
      } else {
        JT nxt = 0;
        for (int k = n - 1; k >= 0; --k) {
          const JT d = J.dp[k] - J.cp[k] * nxt;
          nxt = d;
          B.xv[k] -= (double)d;
          if (tol) norm2 += (double)d * (double)d;
        }
      }
      iters_done = it;
      if (tol) {
        const double nrm = sqrt(norm2);
        if (nrm > prev_norm && it > 2) flags |= CLM_COL_DIVERGED;
        prev_norm = nrm;
        if (nrm < A.tol) break;
        if (it == A.max_iters) flags |= CLM_COL_NOT_CONVERGED;
      }
    }
    const double inv_dt = 1.0 / dt;
    for (int k = 0; k < n; ++k) {
      const double Uv = B.gv[k];
      B.gv[k] = Uv + dt * ((B.xv[k] - Uv) * inv_dt);
    }
    Fw = UFw + dt * ((xFw - UFw) * inv_dt);
  }
  bool finite = isfinite(Fw);
  for (int k = 0; k < n; ++k) finite = finite && isfinite(B.gv[k]);
  if (!finite) flags |= CLM_COL_NONFINITE;
}

}  // namespace clm
