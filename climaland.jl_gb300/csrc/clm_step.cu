// Launch configuration of the step kernels (clm_step_kernels.cuh) and their
// van Genuchten instantiations on uniform columns; the Brooks-Corey ones and
// those with per-layer geometry compile in parallel in clm_step_bc.cu,
// clm_step_s.cu and clm_step_bc_s.cu.

#include "clm_step_kernels.cuh"

namespace clm {

void* step_fn_vg(int model, int precision, int src, int tol) {
  return step_fn_t<VG, false>(model, precision, src, tol);
}

void launch_step_vg(const StepArgs& A, int model, int precision, int grid, dim3 block, size_t smem,
                    double* scratch, const StepClock& clk, int nsteps, cudaStream_t stream) {
  launch_step_t<VG, false>(A, model, precision, grid, block, smem, scratch, clk, nsteps, stream);
}

void* resume_fn_vg(int precision) { return resume_fn_t<VG, false>(precision); }

void launch_resume_vg(const StepArgs& A, int precision, int grid, dim3 block, size_t smem,
                      const StepClock& clk, cudaStream_t stream) {
  launch_resume_t<VG, false>(A, precision, grid, block, smem, clk, stream);
}

// ---------------------------------------------------------------------------
// launch configuration
// ---------------------------------------------------------------------------

size_t step_smem_bytes(int model, int precision, int nmax, int wpc) {
  size_t per_layer;
  if (model == CLM_MODEL_ENERGY_HYDROLOGY)
    per_layer = precision == CLM_PREC_MIXED ? eh_smem_per_layer<float>() : eh_smem_per_layer<double>();
  else
    per_layer = precision == CLM_PREC_MIXED ? richards_smem_per_layer<float>()
                                            : richards_smem_per_layer<double>();
  const int tab = precision == CLM_PREC_MIXED ? fm::stage_doubles<true>() : fm::stage_doubles<false>();
  return tab * sizeof(double) + per_layer * (size_t)nmax * kTile * wpc;
}

static void* step_fn(int model, int precision, int cm, bool str, int src, int tol) {
  if (cm == CLM_CM_BROOKS_COREY)
    return str ? step_fn_bc_s(model, precision, src, tol) : step_fn_bc(model, precision, src, tol);
  return str ? step_fn_vg_s(model, precision, src, tol) : step_fn_vg(model, precision, src, tol);
}

// CTAs of `wpc` warps that can be resident on the whole device (the
// kernels of uniform columns, or with per-layer geometry when `str`; of
// tolerance-mode Newton when `tol`).
cudaError_t step_grid(int model, int precision, int cm, bool str, bool tol, int nmax, int wpc, int ntiles,
                      int* grid) {
  const size_t smem = step_smem_bytes(model, precision, nmax, wpc);
  cudaError_t err;
  // every variant of the launch shape: source kinds and Newton modes (fixed,
  // tolerance, tolerance with split Newton's deferring hook)
  for (int src : {kSrcNone, kSrcRoots, kSrcAtmos}) {
    for (int t : {0, 1, 2}) {
      if (model != CLM_MODEL_ENERGY_HYDROLOGY && (src != kSrcNone || t)) continue;
      if ((err = cudaFuncSetAttribute(step_fn(model, precision, cm, str, src, t),
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
        return err;
    }
  }
  void* fn = step_fn(model, precision, cm, str, kSrcNone, (tol && model == CLM_MODEL_ENERGY_HYDROLOGY) ? 1 : 0);
  int dev = 0, nsm = 0, per_sm = 0;
  if ((err = cudaGetDevice(&dev)) != cudaSuccess) return err;
  if ((err = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return err;
  if ((err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 32 * wpc, smem)) != cudaSuccess)
    return err;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  const int need = (ntiles + wpc - 1) / wpc;
  *grid = per_sm * nsm < need ? per_sm * nsm : need;
  return cudaSuccess;
}

// Split Newton's resuming kernel: its shared memory (tables and Thomas
// arrays) and the attribute that allows it; the queue's size in doubles.
size_t resume_smem_bytes(int precision, int nmax, int wpc) {
  const bool mx = precision == CLM_PREC_MIXED;
  const size_t per_layer = mx ? eh_resume_smem_per_layer<float>() : eh_resume_smem_per_layer<double>();
  const int tab = mx ? fm::stage_doubles<true>() : fm::stage_doubles<false>();
  return tab * sizeof(double) + per_layer * (size_t)nmax * kTile * wpc;
}

static void* resume_fn(int precision, int cm, bool str) {
  if (cm == CLM_CM_BROOKS_COREY) return str ? resume_fn_bc_s(precision) : resume_fn_bc(precision);
  return str ? resume_fn_vg_s(precision) : resume_fn_vg(precision);
}

// The attribute covers the largest CTA (up to wpc warps) whose shared memory
// the device offers, as the step kernel's launch shapes do.
cudaError_t resume_setup(int precision, int cm, bool str, int nmax, int wpc) {
  int dev = 0, cap = 0;
  cudaError_t err;
  if ((err = cudaGetDevice(&dev)) != cudaSuccess) return err;
  if ((err = cudaDeviceGetAttribute(&cap, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) != cudaSuccess)
    return err;
  size_t bytes = resume_smem_bytes(precision, nmax, 1);
  for (int w = wpc; w >= 1; --w)
    if (resume_smem_bytes(precision, nmax, w) <= (size_t)cap) {
      bytes = resume_smem_bytes(precision, nmax, w);
      break;
    }
  return cudaFuncSetAttribute(resume_fn(precision, cm, str), cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)bytes);
}

size_t split_queue_doubles(int cap, int nmax) { return (size_t)queue_doubles(cap, nmax); }

cudaError_t launch_resume(const StepArgs& A, int precision, int wpc, int grid, const StepClock& clk,
                          cudaStream_t stream) {
  const size_t smem = resume_smem_bytes(precision, A.L.nmax, wpc);
  const dim3 block(32 * wpc);
  const bool str = A.geo.z != nullptr;
  if (A.cm == CLM_CM_BROOKS_COREY) {
    if (str) launch_resume_bc_s(A, precision, grid, block, smem, clk, stream);
    else launch_resume_bc(A, precision, grid, block, smem, clk, stream);
  } else {
    if (str) launch_resume_vg_s(A, precision, grid, block, smem, clk, stream);
    else launch_resume_vg(A, precision, grid, block, smem, clk, stream);
  }
  return cudaGetLastError();
}

size_t step_scratch_doubles(int model, int precision, int nmax, int wpc, int grid) {
  if (model != CLM_MODEL_ENERGY_HYDROLOGY) return 0;
  return (size_t)grid * wpc * eh_scratch_slots(precision == CLM_PREC_MIXED) * nmax * kTile;
}

cudaError_t launch_step(const StepArgs& A, int model, int precision, int wpc, int grid,
                        double* scratch, const StepClock& clk, int nsteps, cudaStream_t stream) {
  const size_t smem = step_smem_bytes(model, precision, A.L.nmax, wpc);
  const dim3 block(32 * wpc);
  const bool str = A.geo.z != nullptr;
  if (A.cm == CLM_CM_BROOKS_COREY) {
    if (str) launch_step_bc_s(A, model, precision, grid, block, smem, scratch, clk, nsteps, stream);
    else launch_step_bc(A, model, precision, grid, block, smem, scratch, clk, nsteps, stream);
  } else {
    if (str) launch_step_vg_s(A, model, precision, grid, block, smem, scratch, clk, nsteps, stream);
    else launch_step_vg(A, model, precision, grid, block, smem, scratch, clk, nsteps, stream);
  }
  return cudaGetLastError();
}

}  // namespace clm
