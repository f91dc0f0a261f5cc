// Host replay of the library's column code (climaland.jl_gb300/csrc/
// clm_column.cuh): the same eh_column / richards_column templates the step
// kernels run, compiled with g++ (no a*b+c contraction) and driven one column
// at a time on reference-layout arrays (cell stride 1). It checks the column
// algebra on the CPU (uniform and stretched geometry, FP64 and mixed
// Jacobian types) against the oracle; the device's own bits are checked by
// the GPU tests. Built as a shared library by tests/test_column_replay.py.
#define CLM_HD inline
#define __device__
#define __forceinline__ inline
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
using std::isfinite;
// the device's reciprocal square root, restated for the host
inline double rsqrt(double x) { return 1.0 / std::sqrt(x); }

#include "clm_column.cuh"

using namespace clm;

namespace {

// Split Newton emulation (clmr_set_split): iteration after which an
// unconverged column is saved and resumed from its saved context with fresh
// per-iteration arrays (0: one uninterrupted solve).
int g_split_at = 0;

// What the step kernel's deferring hook saves to the queue.
struct Saved {
  std::vector<double> uv, uti, ue, xv, xe, K, kap, aw, irc, iden;
  std::vector<float> ircf, awr, akr;
  EHNewtonCtx X{};
  bool done = false;
};

struct HostDefer {
  static constexpr bool kEnabled = true;
  int at;
  Saved* sv;
  bool mixed;
  bool operator()(const EHBuffers& B, int n, const EHNewtonCtx& X) const {
    auto take = [n](const Col<double>& c, std::vector<double>& out, int m) {
      out.assign(n, 0.0);
      for (int k = 0; k < m; ++k) out[k] = c[k];
    };
    auto takef = [n](const Col<float>& c, std::vector<float>& out, int m) {
      out.assign(n, 0.0f);
      for (int k = 0; k < m; ++k) out[k] = c[k];
    };
    take(B.gv, sv->uv, n);
    take(B.gti, sv->uti, n);
    take(B.ge, sv->ue, n);
    take(B.xv, sv->xv, n);
    take(B.xe, sv->xe, n);
    take(B.K, sv->K, n);
    take(B.kap, sv->kap, n - 1);
    take(B.aw, sv->aw, n - 1);
    if (mixed) {
      takef(B.ircf, sv->ircf, n);
      takef(B.awr, sv->awr, n - 1);
      takef(B.akr, sv->akr, n - 1);
    } else {
      take(B.irc, sv->irc, n);
      take(B.iden, sv->iden, n);
    }
    sv->X = X;
    sv->done = true;
    return true;
  }
};

template <typename JT, class CM, int kSrc, class Geom>
void eh_one(const StepArgs& A, const Tables& Tb, int c, int n, double* v, double* ti, double* e,
            const float* gv, const float* ge, double* pv, double* pe, const Geom& G, double t, double dt, int nsteps,
            double& Fw, double& Fe, uint32_t& fl, int& it) {
  constexpr bool mixed = sizeof(JT) < sizeof(double);
  std::vector<double> xv(n), xe(n), fe(n), K(n), kap(n), irc(n), aw(n), iden(n);
  std::vector<float> ircf(n), awr(n), akr(n);
  std::vector<JT> cp(n), dp(n), d(n), ae(n);
  EHBuffers B;
  B.gv = Col<double>{v, 1};
  B.gti = Col<double>{ti, 1};
  B.ge = Col<double>{e, 1};
  B.xv = Col<double>{xv.data(), 1};
  B.xe = Col<double>{xe.data(), 1};
  B.fe = Col<double>{fe.data(), 1};
  B.K = Col<double>{K.data(), 1};
  B.kap = Col<double>{kap.data(), 1};
  B.aw = Col<double>{aw.data(), 1};
  if (mixed) {
    B.ircf = Col<float>{ircf.data(), 1};
    B.awr = Col<float>{awr.data(), 1};
    B.akr = Col<float>{akr.data(), 1};
  } else {
    B.irc = Col<double>{irc.data(), 1};
    B.iden = Col<double>{iden.data(), 1};
  }
  EHJac<JT> J;
  J.cp = Col<JT>{cp.data(), 1};
  J.dp = Col<JT>{dp.data(), 1};
  J.d = Col<JT>{d.data(), 1};
  J.ae = Col<JT>{ae.data(), 1};
  if (gv && ge) {
    B.guess_v = Col<const float>{gv, 1};
    B.guess_e = Col<const float>{ge, 1};
  }
  if (pv && pe) {
    B.prev_v = Col<double>{pv, 1};
    B.prev_e = Col<double>{pe, 1};
  }
  if (!(g_split_at > 0 && nsteps == 1 && A.newton_mode == CLM_NEWTON_TOL)) {
    eh_column<JT, CM, false, kSrc>(A, Tb, c, n, c, B, J, G, t, dt, nsteps, Fw, Fe, fl, it);
    return;
  }
  Saved sv;
  eh_column<JT, CM, false, kSrc, kNewtonRuntime, Geom, HostDefer>(A, Tb, c, n, c, B, J, G, t, dt, 1, Fw, Fe,
                                                                   fl, it, HostDefer{g_split_at, &sv, mixed});
  if (!sv.done) return;
  // resume from the saved arrays and context only: the per-iteration arrays
  // start as NaN, so that anything the save left out shows in the result
  const double qnan = std::nan("");
  std::vector<double> fe2(n, qnan);
  std::vector<JT> cp2(n, (JT)qnan), dp2(n, (JT)qnan), d2(n, (JT)qnan), ae2(n, (JT)qnan);
  EHBuffers R;
  R.gv = Col<double>{sv.uv.data(), 1};
  R.gti = Col<double>{sv.uti.data(), 1};
  R.ge = Col<double>{sv.ue.data(), 1};
  R.xv = Col<double>{sv.xv.data(), 1};
  R.xe = Col<double>{sv.xe.data(), 1};
  R.fe = Col<double>{fe2.data(), 1};
  R.K = Col<double>{sv.K.data(), 1};
  R.kap = Col<double>{sv.kap.data(), 1};
  R.aw = Col<double>{sv.aw.data(), 1};
  if (mixed) {
    R.ircf = Col<float>{sv.ircf.data(), 1};
    R.awr = Col<float>{sv.awr.data(), 1};
    R.akr = Col<float>{sv.akr.data(), 1};
  } else {
    R.irc = Col<double>{sv.irc.data(), 1};
    R.iden = Col<double>{sv.iden.data(), 1};
  }
  R.ov = Col<double>{v, 1};
  R.oe = Col<double>{e, 1};
  EHJac<JT> J2;
  J2.cp = Col<JT>{cp2.data(), 1};
  J2.dp = Col<JT>{dp2.data(), 1};
  J2.d = Col<JT>{d2.data(), 1};
  J2.ae = Col<JT>{ae2.data(), 1};
  uint32_t fl2 = 0;
  eh_column<JT, CM, false, kSrcNone, kNewtonRuntime, Geom, NoDefer, true>(A, Tb, c, n, c, R, J2, G, t, dt, 1,
                                                                          Fw, Fe, fl2, it, NoDefer{}, &sv.X);
  fl |= fl2;
}

template <typename JT, class CM, class Geom>
void richards_one(const StepArgs& A, const Tables& Tb, int c, int n, double* v, const Geom& G,
                  double t, double dt, int nsteps, double& Fw, uint32_t& fl, int& it) {
  std::vector<double> xv(n);
  std::vector<JT> cp(n), dp(n), dpl(n);
  RBuffers B;
  B.gv = Col<double>{v, 1};
  B.xv = Col<double>{xv.data(), 1};
  RJac<JT> J;
  J.cp = Col<JT>{cp.data(), 1};
  J.dp = Col<JT>{dp.data(), 1};
  if (sizeof(JT) < sizeof(double)) J.dpl = Col<JT>{dpl.data(), 1};
  richards_column<JT, CM>(A, Tb, c, n, c, B, J, G, t, dt, nsteps, Fw, fl, it);
}

template <typename JT, class CM, class Geom>
void column(const StepArgs& A, const Tables& Tb, int model, int src, int c, int n, double* v,
            double* ti, double* e, const float* gv, const float* ge, double* pv, double* pe, const Geom& G, double t,
            double dt, int nsteps, double& Fw, double& Fe, uint32_t& fl, int& it) {
  if (model == CLM_MODEL_RICHARDS) {
    richards_one<JT, CM>(A, Tb, c, n, v, G, t, dt, nsteps, Fw, fl, it);
  } else if (src == kSrcRoots) {
    eh_one<JT, CM, kSrcRoots>(A, Tb, c, n, v, ti, e, gv, ge, pv, pe, G, t, dt, nsteps, Fw, Fe, fl, it);
  } else if (src == kSrcAtmos) {
    eh_one<JT, CM, kSrcAtmos>(A, Tb, c, n, v, ti, e, gv, ge, pv, pe, G, t, dt, nsteps, Fw, Fe, fl, it);
  } else {
    eh_one<JT, CM, kSrcNone>(A, Tb, c, n, v, ti, e, gv, ge, pv, pe, G, t, dt, nsteps, Fw, Fe, fl, it);
  }
}

template <typename JT, class CM>
void column_geom(const StepArgs& A, const Tables& Tb, int model, int src, int c, int n, int64_t o,
                 double* v, double* ti, double* e, const float* gv, const float* ge, double* pv, double* pe, double t,
                 double dt, int nsteps, double& Fw, double& Fe, uint32_t& fl, int& it) {
  if (A.geo.z) {
    const ColGeomS G(A.geo, o, 1, c, A.L.stride, A.z_lo[c], A.z_hi[c], n);
    column<JT, CM>(A, Tb, model, src, c, n, v, ti, e, gv, ge, pv, pe, G, t, dt, nsteps, Fw, Fe, fl, it);
  } else {
    const ColGeom G(A.z_lo[c], A.z_hi[c], n);
    column<JT, CM>(A, Tb, model, src, c, n, v, ti, e, gv, ge, pv, pe, G, t, dt, nsteps, Fw, Fe, fl, it);
  }
}

}  // namespace

// Split Newton emulation for later clmr_step calls (see g_split_at).
extern "C" void clmr_set_split(int at) { g_split_at = at; }

// One call advances every column nsteps steps in place (reference layout;
// forcing: 4 slot pointers or null; root, atmos: rows of ncol or null;
// z_faces: n + 1 faces per column at offsets[c] + c, or null for uniform
// layers; guess: a Newton starting increment of vartheta_l and rho_e_int
// per cell (EnergyHydrology, tolerance mode), or null; prev: the state at the
// previous step's start for the extrapolated guess, per cell, updated in
// place, or null). Returns 0, or 1 on an argument error.
extern "C" int clmr_step(const clm_config* cfg, int ncol, const int32_t* offsets, const double* z_lo,
                         const double* z_hi, const double* z_faces, const double* params, int nparams,
                         const double* const* forcing, const double* root, const double* atmos,
                         const clm_atmos_params* ap, double* v, double* ti, double* e, double* Fw,
                         double* Fe, double t, double dt, int nsteps, uint32_t* flags, int32_t* iters,
                         const float* guess_v, const float* guess_e, double* prev_v, double* prev_e) {
  if (!cfg || ncol <= 0 || nparams < 1 || nparams > CLM_NPARAM_MAX) return 1;
  const bool eh = cfg->model == CLM_MODEL_ENERGY_HYDROLOGY;
  std::vector<double> prm((size_t)CLM_NPARAM_MAX * ncol, 0.0), lkap(2 * (size_t)ncol, 0.0);
  std::memcpy(prm.data(), params, sizeof(double) * nparams * ncol);
  for (int c = 0; c < ncol && eh; ++c) {
    lkap[c] = std::log(prm[CLM_P_KAPPA_SAT_UNFROZEN * ncol + c]);
    lkap[ncol + c] = std::log(prm[CLM_P_KAPPA_SAT_FROZEN * ncol + c]);
  }
  std::vector<double> zlo(z_lo, z_lo + ncol), zhi(z_hi, z_hi + ncol);
  const int64_t nc = offsets[ncol];
  std::vector<double> geo, gcol;
  StepArgs A{};
  A.L.ncol = ncol;
  A.L.stride = ncol;
  if (z_faces) {
    geo.assign(5 * (size_t)nc, 0.0);
    gcol.assign(3 * (size_t)ncol, 0.0);
    for (int c = 0; c < ncol; ++c) {
      const int64_t o = offsets[c];
      const int n = offsets[c + 1] - offsets[c];
      const double* f = z_faces + o + c;
      const GeoColumn g = column_geometry(f, n, 1, &geo[o], &geo[nc + o], &geo[2 * nc + o],
                                          &geo[3 * nc + o], &geo[4 * nc + o]);
      gcol[c] = g.bot;
      gcol[ncol + c] = g.wmin;
      gcol[2 * ncol + c] = g.wsum;
      zlo[c] = f[0];
      zhi[c] = f[n];
    }
    A.geo = GeoArrays{geo.data(), geo.data() + nc, geo.data() + 2 * nc, geo.data() + 3 * nc,
                      geo.data() + 4 * nc, gcol.data()};
  }
  A.z_lo = zlo.data();
  A.z_hi = zhi.data();
  A.prm = prm.data();
  A.lkap = lkap.data();
  for (int i = 0; i < 4; ++i) A.forc[i] = forcing ? forcing[i] : nullptr;
  A.rx = eh ? root : nullptr;
  A.atm = (eh && cfg->bc_top_water == CLM_BC_ATMOS) ? atmos : nullptr;
  if (A.atm) {
    if (!ap) return 1;  // the caller passes the constants
    A.ak = make_atmos_k(*ap, cfg->earth);
  }
  A.E = make_earth(cfg->earth);
  A.sc.kersten_alpha = cfg->kersten_alpha;
  A.sc.kersten_beta = cfg->kersten_beta;
  A.sc.omega_ln10 = cfg->ice_impedance_omega * kLn10;
  A.sc.visc_gamma = cfg->visc_gamma;
  A.sc.visc_gamma_T_ref = cfg->visc_gamma_T_ref;
  A.bc_tw = cfg->bc_top_water;
  A.bc_th = cfg->bc_top_heat;
  A.bc_bw = cfg->bc_bottom_water;
  A.bc_bh = cfg->bc_bottom_heat;
  A.phase_change = eh ? cfg->phase_change : 0;
  A.runoff = cfg->runoff;
  A.cm = cfg->hydrology_cm;
  A.newton_mode = cfg->newton_mode;
  A.max_iters = cfg->max_iters;
  A.tol = cfg->newton_tol;
  A.energy_scale = cfg->energy_norm_scale;
  A.seed = cfg->forcing_seed;
  A.col0 = cfg->column_offset;
  const int src = A.atm ? kSrcAtmos : (A.rx ? kSrcRoots : kSrcNone);
  const Tables Tb = fm::host_tables();
  const bool mixed = cfg->precision == CLM_PREC_MIXED;
  const bool bc = cfg->hydrology_cm == CLM_CM_BROOKS_COREY;
#pragma omp parallel for schedule(dynamic, 16)
  for (int c = 0; c < ncol; ++c) {
    const int64_t o = offsets[c];
    const int n = offsets[c + 1] - offsets[c];
    double fw = Fw[c], fe = eh ? Fe[c] : 0.0;
    uint32_t fl = 0;
    int it = 0;
    double* cv = v + o;
    double* cti = eh ? ti + o : nullptr;
    double* ce = eh ? e + o : nullptr;
    const float* gv = guess_v ? guess_v + o : nullptr;
    const float* ge = guess_e ? guess_e + o : nullptr;
    double* pv = prev_v ? prev_v + o : nullptr;
    double* pe = prev_e ? prev_e + o : nullptr;
    if (mixed) {
      if (bc) column_geom<float, BC>(A, Tb, cfg->model, src, c, n, o, cv, cti, ce, gv, ge, pv, pe, t, dt, nsteps, fw, fe, fl, it);
      else column_geom<float, VG>(A, Tb, cfg->model, src, c, n, o, cv, cti, ce, gv, ge, pv, pe, t, dt, nsteps, fw, fe, fl, it);
    } else {
      if (bc) column_geom<double, BC>(A, Tb, cfg->model, src, c, n, o, cv, cti, ce, gv, ge, pv, pe, t, dt, nsteps, fw, fe, fl, it);
      else column_geom<double, VG>(A, Tb, cfg->model, src, c, n, o, cv, cti, ce, gv, ge, pv, pe, t, dt, nsteps, fw, fe, fl, it);
    }
    Fw[c] = fw;
    if (eh) Fe[c] = fe;
    if (flags) flags[c] = fl;
    if (iters) iters[c] = it;
  }
  return 0;
}
