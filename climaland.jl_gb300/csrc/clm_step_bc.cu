// Brooks-Corey instantiations of the step kernels (clm_step_kernels.cuh),
// in their own translation unit so that they compile in parallel with the
// van Genuchten ones.

#include "clm_step_kernels.cuh"

namespace clm {

void* step_fn_bc(int model, int precision, int src, int tol) {
  return step_fn_t<BC, false>(model, precision, src, tol);
}

void launch_step_bc(const StepArgs& A, int model, int precision, int grid, dim3 block, size_t smem,
                    double* scratch, const StepClock& clk, int nsteps, cudaStream_t stream) {
  launch_step_t<BC, false>(A, model, precision, grid, block, smem, scratch, clk, nsteps, stream);
}

void* resume_fn_bc(int precision) { return resume_fn_t<BC, false>(precision); }

void launch_resume_bc(const StepArgs& A, int precision, int grid, dim3 block, size_t smem,
                      const StepClock& clk, cudaStream_t stream) {
  launch_resume_t<BC, false>(A, precision, grid, block, smem, clk, stream);
}

}  // namespace clm
