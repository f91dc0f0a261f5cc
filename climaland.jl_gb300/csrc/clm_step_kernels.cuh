// Step kernels: persistent warps over 32-column tiles, one thread per
// column, running the column code of clm_column.cuh.
//
// Shared memory per CTA: the exp/log tables (2 KB; the mixed EnergyHydrology
// kernel also 0.5 KB of double-float pairs), then per warp the Newton
// iterate and the Thomas arrays of its tile. The arrays of EnergyHydrology
// that are written once per sweep and read once in a later sweep (the frozen
// aux K, kappa, 1/rho c, the face coefficients, the energy residual and the
// energy-advection face coefficient) live in a per-warp-slot global scratch
// area (`scratch`, sized by the launch grid, small enough to stay in L2):
// the smaller shared footprint leaves room for more resident warps when
// columns are deep (up to 30 layers: 8 instead of 5 warps per SM on the
// mixed path). The grid is the number of CTAs that
// fit on the device at once; each warp walks tiles w, w + W, w + 2W, ...
// (tiles are sorted deepest first, so the walk is balanced), or, with the
// dynamic order, claims the next unprocessed tile from an atomic counter
// (deepest first: longest-processing-time-first list scheduling).

#pragma once

#include <cuda_runtime.h>

#include "clm_column.cuh"

namespace clm {

template <typename JT>
__host__ __device__ constexpr size_t eh_smem_per_layer() {
  return 2 * sizeof(double) + 3 * sizeof(JT);  // xv, xe | cp, dp, d
}

template <typename JT>
__host__ __device__ constexpr int richards_jac_arrays() {
  return sizeof(JT) < sizeof(double) ? 3 : 2;  // cp, dp (| low words of dp)
}

template <typename JT>
__host__ __device__ constexpr size_t richards_smem_per_layer() {
  return sizeof(double) + richards_jac_arrays<JT>() * sizeof(JT);  // xv | cp, dp (, dp low)
}

// Per-warp scratch slots of nmax x 32 doubles. FP64 path: K, face kappa / dz,
// 1 / rho c, face K / dz, the energy residual, the energy-advection face
// coefficient, the layer's saturation reciprocal. Mixed: K, face kappa / dz,
// then the floats 1 / rho c, dt K_face / dz^2, dt kappa_face / dz^2 and the
// energy-advection face coefficient packed into two slots, face K / dz, the
// energy residual.
__host__ __device__ constexpr int eh_scratch_slots(bool mixed) { return mixed ? 6 : 7; }

// Split Newton queue. Entry e belongs to group e / 32 (one resuming warp,
// lane e % 32); a group is one contiguous block of kQArrays arrays of
// nmax x 32 doubles ([array][layer][lane], so that a warp's access to one
// layer is one 256-byte segment) followed by the scalars [kQScalars][32], so
// that one bulk prefetch brings a group into L2.
// Arrays: the stage value U (vartheta_l, theta_i, rho_e_int), the iterate,
// K, the face conductances kappa / dz and K / dz, two slots of aux (FP64:
// 1 / rho c and the saturation reciprocal; mixed: the floats 1 / rho c,
// dt K_face / dz^2, dt kappa_face / dz^2 and the energy-advection face
// coefficient), and the per-iteration energy residual and (FP64) advection
// face coefficient of the resumed solve.
constexpr int kQArrays = 12;
enum QueueArray { kQUv, kQUti, kQUe, kQXv, kQXe, kQK, kQKap, kQAw, kQAux0, kQAux1, kQFe, kQAe };
enum QueueScalar {
  kQsSlot, kQsFtw, kQsFth, kQsFbw, kQsFbh, kQsUFw, kQsUFe, kQsXFw, kQsXFe, kQsRss, kQsRess,
  kQsPrevNorm, kQsPrevState2, kQsPred2, kQsItStart, kQsItDone, kQsUseGuess, kQScalars
};

__host__ __device__ inline int64_t queue_doubles(int cap, int nmax) {
  return (int64_t)cap * ((int64_t)kQArrays * nmax + kQScalars);
}

struct QueueView {
  SplitQueue Q;
  __device__ int64_t lay() const { return (int64_t)Q.nmax * kTile; }
  // doubles per group block (a multiple of 32: 256-byte aligned blocks)
  __device__ int64_t block() const { return (int64_t)kQArrays * lay() + kQScalars * kTile; }
  __device__ double* group(int g) const { return Q.q + (int64_t)g * block(); }
  __device__ double* arr0(int e, int a) const { return group(e / kTile) + a * lay() + e % kTile; }
  __device__ Col<double> arr(int e, int a) const { return Col<double>{arr0(e, a), kTile}; }
  // the four float arrays of the mixed path's aux slots
  __device__ Col<float> farr(int e, int j) const {
    return Col<float>{reinterpret_cast<float*>(group(e / kTile) + kQAux0 * lay()) + j * lay() + e % kTile,
                      kTile};
  }
  __device__ double& scal(int e, int f) const {
    return group(e / kTile)[kQArrays * lay() + f * kTile + e % kTile];
  }
  // Bulk L2 prefetch of group g's block (TMA engine, no registers or shared
  // memory involved): lanes 0.. each issue one 16 KB piece. Every byte lies
  // inside the queue (g < cap / 32); sizes are multiples of 256 bytes.
  __device__ void prefetch_group(int g, int lane) const {
    const int64_t bytes = block() * (int64_t)sizeof(double);
    constexpr int64_t kPiece = 16384;
    const int64_t off = (int64_t)lane * kPiece;
    if (off < bytes) {
      const int64_t sz = bytes - off < kPiece ? bytes - off : kPiece;
      const char* p = reinterpret_cast<const char*>(group(g)) + off;
      asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"((unsigned)sz) : "memory");
    }
  }
};

// The step kernel's deferring hook: claims an entry (one atomic per lane, no
// warp collective inside the Newton loop) and copies the column's arrays and
// context with evict-first stores (the resuming launch prefetches them back;
// meanwhile they should not push the step kernel's L2-resident scratch out).
template <typename JT>
struct QueueDefer {
  static constexpr bool kEnabled = true;
  int at;
  QueueView V;
  int s;
  __device__ bool operator()(const EHBuffers& B, int n, const EHNewtonCtx& X) const {
    constexpr bool kMixed = sizeof(JT) < sizeof(double);
    const int e = atomicAdd(V.Q.count, 1);
    if (e >= V.Q.cap) return false;  // no room: the column finishes here
    const Col<double> uv = V.arr(e, kQUv), uti = V.arr(e, kQUti), ue = V.arr(e, kQUe);
    const Col<double> xv = V.arr(e, kQXv), xe = V.arr(e, kQXe), K = V.arr(e, kQK);
    const Col<double> kap = V.arr(e, kQKap), aw = V.arr(e, kQAw);
    for (int k = 0; k < n; ++k) {
      uv.store_last(k, B.gv[k]);
      uti.store_last(k, B.gti[k]);
      ue.store_last(k, B.ge[k]);
      xv.store_last(k, B.xv[k]);
      xe.store_last(k, B.xe[k]);
      K.store_last(k, B.K[k]);
      if constexpr (kMixed) {
        V.farr(e, 0).store_last(k, B.ircf[k]);
      } else {
        V.arr(e, kQAux0).store_last(k, B.irc[k]);
        V.arr(e, kQAux1).store_last(k, B.iden[k]);
      }
    }
    for (int k = 0; k < n - 1; ++k) {  // faces k|k+1
      kap.store_last(k, B.kap[k]);
      aw.store_last(k, B.aw[k]);
      if constexpr (kMixed) {
        V.farr(e, 1).store_last(k, B.awr[k]);
        V.farr(e, 2).store_last(k, B.akr[k]);
      }
    }
    auto put = [&](int f, double v) { __stcs(&V.scal(e, f), v); };
    put(kQsSlot, s);
    put(kQsFtw, X.Ftw);
    put(kQsFth, X.Fth);
    put(kQsFbw, X.Fbw);
    put(kQsFbh, X.Fbh);
    put(kQsUFw, X.UFw);
    put(kQsUFe, X.UFe);
    put(kQsXFw, X.xFw);
    put(kQsXFe, X.xFe);
    put(kQsRss, X.R_ss);
    put(kQsRess, X.R_ess);
    put(kQsPrevNorm, X.prev_norm);
    put(kQsPrevState2, X.prev_state2);
    put(kQsPred2, X.pred2);
    put(kQsItStart, X.it_start);
    put(kQsItDone, X.it_done);
    put(kQsUseGuess, X.use_guess ? 1.0 : 0.0);
    return true;
  }
};

// kSrc: the RootExtraction source (A.rx) or the atmosphere-driven top
// boundary (A.atm) compiled in; separate kernels so that their registers do
// not weigh on the step without them. kStr: per-layer geometry. kTol: 0
// fixed Newton iterations, 1 the tolerance-mode Newton (norms, stopping,
// guesses) compiled in, 2 that with split Newton's deferring hook (the
// first launch of a split step). Each carries only its own mode's code and
// has a smaller instruction footprint (with both Newton modes in one kernel,
// instruction-fetch stalls measured 0.81 cycles per issued instruction in
// tolerance mode with a guess, 0.23 in fixed mode; with the hook compiled
// into every tolerance kernel, never taken there, multi-step launches of the
// tiles measured 1.5-1.65x slower).
template <typename JT, class CM, int kSrc, bool kStr, int kTol = 0>
__global__ void __launch_bounds__(128, 1)
    eh_step_kernel(StepArgs A, double* __restrict__ scratch, StepClock clk, int nsteps) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* tab = reinterpret_cast<double*>(smem_raw);
  constexpr bool kMixed = sizeof(JT) < sizeof(double);
  constexpr int kTab = fm::stage_doubles<kMixed>();
  const Tables Tb = fm::stage_tables<kMixed>(tab);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int wpc = blockDim.x >> 5;
  const int nmax = A.L.nmax;
  const int64_t lay = (int64_t)nmax * kTile;
  double* dw = tab + kTab + (int64_t)warp * 2 * lay;
  JT* jw = reinterpret_cast<JT*>(tab + kTab + (int64_t)wpc * 2 * lay) + (int64_t)warp * 3 * lay;
  const int gwarp = blockIdx.x * wpc + warp;
  const int nwarps = gridDim.x * wpc;
  double* sw = scratch + (int64_t)gwarp * eh_scratch_slots(kMixed) * lay;
  EHBuffers B;
  B.xv = Col<double>{dw + lane, kTile};
  B.xe = Col<double>{dw + lay + lane, kTile};
  B.fe = Col<double>{sw + (kMixed ? 5 : 4) * lay + lane, kTile};
  B.K = Col<double>{sw + lane, kTile};
  B.kap = Col<double>{sw + lay + lane, kTile};
  B.aw = Col<double>{sw + (kMixed ? 4 : 3) * lay + lane, kTile};
  if constexpr (kMixed) {
    float* fw = reinterpret_cast<float*>(sw + 2 * lay);
    B.ircf = Col<float>{fw + lane, kTile};
    B.awr = Col<float>{fw + lay + lane, kTile};
    B.akr = Col<float>{fw + 2 * lay + lane, kTile};
  } else {
    B.irc = Col<double>{sw + 2 * lay + lane, kTile};
  }
  EHJac<JT> J;
  J.cp = Col<JT>{jw + lane, kTile};
  J.dp = Col<JT>{jw + lay + lane, kTile};
  J.d = Col<JT>{jw + 2 * lay + lane, kTile};
  if constexpr (kMixed)
    J.ae = Col<JT>{reinterpret_cast<JT*>(sw + 2 * lay) + 3 * lay + lane, kTile};
  else
    J.ae = Col<JT>{reinterpret_cast<JT*>(sw + 5 * lay) + lane, kTile};
  if constexpr (!kMixed) B.iden = Col<double>{sw + 6 * lay + lane, kTile};
  const double t0 = clk.start(), dt = clk.step();
  const bool dyn = A.tile_ctr != nullptr;
  const int tend = A.tile_end < 0 ? A.L.ntiles : A.tile_end;
  int tile = A.tile_begin + (dyn ? claim_tile(A.tile_ctr) : gwarp);
  while (tile < tend) {
    const int s = A.order ? A.order[tile * kTile + lane] : tile * kTile + lane;
    const int n = A.L.col_n[s];
    if (n > 0) {
      const int64_t base = A.L.tile_off[s / kTile] + s % kTile;
      B.gv = Col<double>{A.v + base, kTile};
      B.gti = Col<double>{A.ti + base, kTile};
      B.ge = Col<double>{A.e + base, kTile};
      if (A.guess) {
        B.guess_v = Col<const float>{A.guess + base, kTile};
        B.guess_e = Col<const float>{A.guess + A.L.ncells_int + base, kTile};
      }
      if (A.prev) {
        B.prev_v = Col<double>{A.prev + base, kTile};
        B.prev_e = Col<double>{A.prev + A.L.ncells_int + base, kTile};
      }
      double Fw = A.Fw[s], Fe = A.Fe[s];
      uint32_t flags = 0;
      int iters = 0;
      const auto G = GeomOf<kStr>::make(A, base, s, n);
      if constexpr (kTol == 2) {
        // split Newton: one-step launches with a queue defer their
        // unconverged columns after iteration split_at
        const QueueDefer<JT> D{(A.split.q && nsteps == 1) ? A.split_at : 0, QueueView{A.split}, s};
        eh_column<JT, CM, false, kSrc, kNewtonTol, typename GeomOf<kStr>::type, QueueDefer<JT>>(
            A, Tb, s, n, A.L.perm[s], B, J, G, t0, dt, nsteps, Fw, Fe, flags, iters, D);
      } else if constexpr (kTol == 1) {
        eh_column<JT, CM, false, kSrc, kNewtonTol>(A, Tb, s, n, A.L.perm[s], B, J, G, t0, dt, nsteps, Fw, Fe,
                                                   flags, iters);
      } else {
        eh_column<JT, CM, false, kSrc, kNewtonFixed>(A, Tb, s, n, A.L.perm[s], B, J, G, t0, dt, nsteps, Fw,
                                                     Fe, flags, iters);
      }
      A.Fw[s] = Fw;
      A.Fe[s] = Fe;
      A.flags[s] |= flags;  // cleared at the start of each step call
      A.iters[s] = iters;
    }
    tile = dyn ? A.tile_begin + claim_tile(A.tile_ctr) : tile + nwarps;
  }
  if (dyn) release_tiles(A.tile_ctr, nwarps);
}

// Split Newton, second launch: the queued columns, 32 to a warp in the order
// they were saved, from their saved context to the end of the step (the
// explicit source and top-boundary variants differ only before the Newton
// solve, so one kernel serves them all). Shared memory as the step kernel's:
// the tables, then per warp the iterate (copied in from the entry) and the
// Thomas arrays; U, the aux and the per-iteration residuals stay in the entry.
template <typename JT>
__host__ __device__ constexpr size_t eh_resume_smem_per_layer() {
  return eh_smem_per_layer<JT>();  // as the step kernel: xv, xe | cp, dp, d
}

template <typename JT, class CM, bool kStr>
__global__ void __launch_bounds__(128, 1) eh_resume_kernel(StepArgs A, StepClock clk) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* tab = reinterpret_cast<double*>(smem_raw);
  constexpr bool kMixed = sizeof(JT) < sizeof(double);
  constexpr int kTab = fm::stage_doubles<kMixed>();
  const Tables Tb = fm::stage_tables<kMixed>(tab);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int wpc = blockDim.x >> 5;
  const int64_t lay = (int64_t)A.L.nmax * kTile;
  double* dw = tab + kTab + (int64_t)warp * 2 * lay;
  JT* jw = reinterpret_cast<JT*>(tab + kTab + (int64_t)wpc * 2 * lay) + (int64_t)warp * 3 * lay;
  EHJac<JT> J;
  J.cp = Col<JT>{jw + lane, kTile};
  J.dp = Col<JT>{jw + lay + lane, kTile};
  J.d = Col<JT>{jw + 2 * lay + lane, kTile};
  const QueueView V{A.split};
  const int count = min(*A.split.count, A.split.cap);
  const int ngroups = (count + kTile - 1) / kTile;
  const double t0 = clk.start(), dt = clk.step();
  const int nw = gridDim.x * wpc;
  int grp = blockIdx.x * wpc + warp;
  if (grp < ngroups) V.prefetch_group(grp, lane);
  for (; grp < ngroups; grp += nw) {
    // the warp's next group comes into L2 while this one runs
    if (grp + nw < ngroups) V.prefetch_group(grp + nw, lane);
    const int e = grp * kTile + lane;
    if (e >= count) continue;  // the column code has no warp collectives
    const int s = (int)V.scal(e, kQsSlot);
    const int n = A.L.col_n[s];
    const int64_t base = A.L.tile_off[s / kTile] + s % kTile;
    EHBuffers B;
    B.gv = V.arr(e, kQUv);
    B.gti = V.arr(e, kQUti);
    B.ge = V.arr(e, kQUe);
    // the iterate in shared memory, as in the step kernel
    B.xv = Col<double>{dw + lane, kTile};
    B.xe = Col<double>{dw + lay + lane, kTile};
    {
      const Col<double> qv = V.arr(e, kQXv), qe = V.arr(e, kQXe);
      for (int k = 0; k < n; ++k) {
        B.xv[k] = qv[k];
        B.xe[k] = qe[k];
      }
    }
    B.K = V.arr(e, kQK);
    B.kap = V.arr(e, kQKap);
    B.aw = V.arr(e, kQAw);
    B.fe = V.arr(e, kQFe);
    if constexpr (kMixed) {
      B.ircf = V.farr(e, 0);
      B.awr = V.farr(e, 1);
      B.akr = V.farr(e, 2);
      J.ae = Col<JT>{reinterpret_cast<JT*>(V.farr(e, 3).p), kTile};
    } else {
      B.irc = V.arr(e, kQAux0);
      B.iden = V.arr(e, kQAux1);
      J.ae = Col<JT>{reinterpret_cast<JT*>(V.arr0(e, kQAe)), kTile};
    }
    B.ov = Col<double>{A.v + base, kTile};
    B.oe = Col<double>{A.e + base, kTile};
    EHNewtonCtx X;
    X.Ftw = V.scal(e, kQsFtw);
    X.Fth = V.scal(e, kQsFth);
    X.Fbw = V.scal(e, kQsFbw);
    X.Fbh = V.scal(e, kQsFbh);
    X.UFw = V.scal(e, kQsUFw);
    X.UFe = V.scal(e, kQsUFe);
    X.xFw = V.scal(e, kQsXFw);
    X.xFe = V.scal(e, kQsXFe);
    X.R_ss = V.scal(e, kQsRss);
    X.R_ess = V.scal(e, kQsRess);
    X.prev_norm = V.scal(e, kQsPrevNorm);
    X.prev_state2 = V.scal(e, kQsPrevState2);
    X.pred2 = V.scal(e, kQsPred2);
    X.it_start = (int)V.scal(e, kQsItStart);
    X.it_done = (int)V.scal(e, kQsItDone);
    X.use_guess = V.scal(e, kQsUseGuess) != 0.0;
    double Fw = A.Fw[s], Fe = A.Fe[s];
    uint32_t flags = 0;
    int iters = 0;
    const auto G = GeomOf<kStr>::make(A, base, s, n);
    eh_column<JT, CM, false, kSrcNone, kNewtonTol, typename GeomOf<kStr>::type, NoDefer, true>(
        A, Tb, s, n, A.L.perm[s], B, J, G, t0, dt, 1, Fw, Fe, flags, iters, NoDefer{}, &X);
    A.Fw[s] = Fw;
    A.Fe[s] = Fe;
    A.flags[s] |= flags;
    A.iters[s] = iters;
  }
}

template <typename JT, class CM, bool kStr>
__global__ void __launch_bounds__(128, 1)
    richards_step_kernel(StepArgs A, StepClock clk, int nsteps) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* tab = reinterpret_cast<double*>(smem_raw);
  constexpr bool kMixed = sizeof(JT) < sizeof(double);
  constexpr int kTab = fm::stage_doubles<kMixed>();
  const Tables Tb = fm::stage_tables<kMixed>(tab);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int wpc = blockDim.x >> 5;
  const int64_t lay = (int64_t)A.L.nmax * kTile;
  double* dw = tab + kTab + (int64_t)warp * lay;
  constexpr int kJA = richards_jac_arrays<JT>();
  JT* jw = reinterpret_cast<JT*>(tab + kTab + (int64_t)wpc * lay) + (int64_t)warp * kJA * lay;
  const int gwarp = blockIdx.x * wpc + warp;
  const int nwarps = gridDim.x * wpc;
  RBuffers B;
  B.xv = Col<double>{dw + lane, kTile};
  RJac<JT> J;
  J.cp = Col<JT>{jw + lane, kTile};
  J.dp = Col<JT>{jw + lay + lane, kTile};
  if (kJA > 2) J.dpl = Col<JT>{jw + 2 * lay + lane, kTile};
  const double t0 = clk.start(), dt = clk.step();
  const bool dyn = A.tile_ctr != nullptr;
  const int tend = A.tile_end < 0 ? A.L.ntiles : A.tile_end;
  int tile = A.tile_begin + (dyn ? claim_tile(A.tile_ctr) : gwarp);
  while (tile < tend) {
    const int s = A.order ? A.order[tile * kTile + lane] : tile * kTile + lane;
    const int n = A.L.col_n[s];
    if (n > 0) {
      const int64_t base = A.L.tile_off[s / kTile] + s % kTile;
      B.gv = Col<double>{A.v + base, kTile};
      double Fw = A.Fw[s];
      uint32_t flags = 0;
      int iters = 0;
      const auto G = GeomOf<kStr>::make(A, base, s, n);
      richards_column<JT, CM>(A, Tb, s, n, A.L.perm[s], B, J, G, t0, dt, nsteps, Fw, flags, iters);
      A.Fw[s] = Fw;
      A.flags[s] |= flags;  // cleared at the start of each step call
      A.iters[s] = iters;
    }
    tile = dyn ? A.tile_begin + claim_tile(A.tile_ctr) : tile + nwarps;
  }
  if (dyn) release_tiles(A.tile_ctr, nwarps);
}

// The explicit source / top boundary kernel variant of a launch.
inline int step_src(const StepArgs& A) {
  return A.atm ? kSrcAtmos : A.rx ? kSrcRoots : kSrcNone;
}

// The kernel of (model, precision, source variant) for closure CM and
// geometry kStr, and its launch.
template <class CM, bool kStr, int kTol>
void* eh_fn_t(bool mx, int src) {
  if (src == kSrcRoots)
    return mx ? (void*)eh_step_kernel<float, CM, kSrcRoots, kStr, kTol>
              : (void*)eh_step_kernel<double, CM, kSrcRoots, kStr, kTol>;
  if (src == kSrcAtmos)
    return mx ? (void*)eh_step_kernel<float, CM, kSrcAtmos, kStr, kTol>
              : (void*)eh_step_kernel<double, CM, kSrcAtmos, kStr, kTol>;
  return mx ? (void*)eh_step_kernel<float, CM, kSrcNone, kStr, kTol>
            : (void*)eh_step_kernel<double, CM, kSrcNone, kStr, kTol>;
}

// tol: 0 fixed iterations, 1 tolerance mode, 2 tolerance mode with split
// Newton's deferring hook
template <class CM, bool kStr>
void* step_fn_t(int model, int precision, int src = kSrcNone, int tol = 0) {
  if (model == CLM_MODEL_ENERGY_HYDROLOGY) {
    const bool mx = precision == CLM_PREC_MIXED;
    if (tol == 2) return eh_fn_t<CM, kStr, 2>(mx, src);
    return tol ? eh_fn_t<CM, kStr, 1>(mx, src) : eh_fn_t<CM, kStr, 0>(mx, src);
  }
  return precision == CLM_PREC_MIXED ? (void*)richards_step_kernel<float, CM, kStr>
                                     : (void*)richards_step_kernel<double, CM, kStr>;
}

template <typename JT, class CM, bool kStr, int kTol>
void launch_eh_mode(const StepArgs& A, int grid, dim3 block, size_t smem, double* scratch,
                    const StepClock& clk, int nsteps, cudaStream_t stream) {
  switch (step_src(A)) {
    case kSrcRoots:
      eh_step_kernel<JT, CM, kSrcRoots, kStr, kTol><<<grid, block, smem, stream>>>(A, scratch, clk, nsteps);
      break;
    case kSrcAtmos:
      eh_step_kernel<JT, CM, kSrcAtmos, kStr, kTol><<<grid, block, smem, stream>>>(A, scratch, clk, nsteps);
      break;
    default:
      eh_step_kernel<JT, CM, kSrcNone, kStr, kTol><<<grid, block, smem, stream>>>(A, scratch, clk, nsteps);
  }
}

template <typename JT, class CM, bool kStr>
void launch_eh_t(const StepArgs& A, int grid, dim3 block, size_t smem, double* scratch,
                 const StepClock& clk, int nsteps, cudaStream_t stream) {
  if (A.newton_mode == CLM_NEWTON_TOL && A.split.q && nsteps == 1)
    launch_eh_mode<JT, CM, kStr, 2>(A, grid, block, smem, scratch, clk, nsteps, stream);
  else if (A.newton_mode == CLM_NEWTON_TOL)
    launch_eh_mode<JT, CM, kStr, 1>(A, grid, block, smem, scratch, clk, nsteps, stream);
  else
    launch_eh_mode<JT, CM, kStr, 0>(A, grid, block, smem, scratch, clk, nsteps, stream);
}

template <class CM, bool kStr>
void launch_step_t(const StepArgs& A, int model, int precision, int grid, dim3 block, size_t smem,
                   double* scratch, const StepClock& clk, int nsteps, cudaStream_t stream) {
  if (model == CLM_MODEL_ENERGY_HYDROLOGY) {
    if (precision == CLM_PREC_MIXED)
      launch_eh_t<float, CM, kStr>(A, grid, block, smem, scratch, clk, nsteps, stream);
    else
      launch_eh_t<double, CM, kStr>(A, grid, block, smem, scratch, clk, nsteps, stream);
  } else {
    if (precision == CLM_PREC_MIXED)
      richards_step_kernel<float, CM, kStr><<<grid, block, smem, stream>>>(A, clk, nsteps);
    else
      richards_step_kernel<double, CM, kStr><<<grid, block, smem, stream>>>(A, clk, nsteps);
  }
}

template <class CM, bool kStr>
void* resume_fn_t(int precision) {
  return precision == CLM_PREC_MIXED ? (void*)eh_resume_kernel<float, CM, kStr>
                                     : (void*)eh_resume_kernel<double, CM, kStr>;
}

template <class CM, bool kStr>
void launch_resume_t(const StepArgs& A, int precision, int grid, dim3 block, size_t smem,
                     const StepClock& clk, cudaStream_t stream) {
  if (precision == CLM_PREC_MIXED)
    eh_resume_kernel<float, CM, kStr><<<grid, block, smem, stream>>>(A, clk);
  else
    eh_resume_kernel<double, CM, kStr><<<grid, block, smem, stream>>>(A, clk);
}

// One translation unit per (closure, geometry) instantiates these: the entry
// points each defines (clm_step.cu, clm_step_bc.cu, clm_step_s.cu,
// clm_step_bc_s.cu).
void* step_fn_vg(int model, int precision, int src, int tol);
void* step_fn_bc(int model, int precision, int src, int tol);
void* step_fn_vg_s(int model, int precision, int src, int tol);
void* step_fn_bc_s(int model, int precision, int src, int tol);
void launch_step_vg(const StepArgs& A, int model, int precision, int grid, dim3 block, size_t smem,
                    double* scratch, const StepClock& clk, int nsteps, cudaStream_t stream);
void launch_step_bc(const StepArgs& A, int model, int precision, int grid, dim3 block, size_t smem,
                    double* scratch, const StepClock& clk, int nsteps, cudaStream_t stream);
void launch_step_vg_s(const StepArgs& A, int model, int precision, int grid, dim3 block, size_t smem,
                      double* scratch, const StepClock& clk, int nsteps, cudaStream_t stream);
void launch_step_bc_s(const StepArgs& A, int model, int precision, int grid, dim3 block, size_t smem,
                      double* scratch, const StepClock& clk, int nsteps, cudaStream_t stream);
void* resume_fn_vg(int precision);
void* resume_fn_bc(int precision);
void* resume_fn_vg_s(int precision);
void* resume_fn_bc_s(int precision);
void launch_resume_vg(const StepArgs& A, int precision, int grid, dim3 block, size_t smem,
                      const StepClock& clk, cudaStream_t stream);
void launch_resume_bc(const StepArgs& A, int precision, int grid, dim3 block, size_t smem,
                      const StepClock& clk, cudaStream_t stream);
void launch_resume_vg_s(const StepArgs& A, int precision, int grid, dim3 block, size_t smem,
                        const StepClock& clk, cudaStream_t stream);
void launch_resume_bc_s(const StepArgs& A, int precision, int grid, dim3 block, size_t smem,
                        const StepClock& clk, cudaStream_t stream);

}  // namespace clm
