// Step kernels of van Genuchten columns with per-layer geometry (stretched
// meshes, clm_set_faces), in their own translation unit so that they compile
// in parallel with the uniform ones.

#include "clm_step_kernels.cuh"

namespace clm {

void* step_fn_vg_s(int model, int precision, int src, int tol) {
  return step_fn_t<VG, true>(model, precision, src, tol);
}

void launch_step_vg_s(const StepArgs& A, int model, int precision, int grid, dim3 block, size_t smem,
                      double* scratch, const StepClock& clk, int nsteps, cudaStream_t stream) {
  launch_step_t<VG, true>(A, model, precision, grid, block, smem, scratch, clk, nsteps, stream);
}

void* resume_fn_vg_s(int precision) { return resume_fn_t<VG, true>(precision); }

void launch_resume_vg_s(const StepArgs& A, int precision, int grid, dim3 block, size_t smem,
                        const StepClock& clk, cudaStream_t stream) {
  launch_resume_t<VG, true>(A, precision, grid, block, smem, clk, stream);
}

}  // namespace clm
