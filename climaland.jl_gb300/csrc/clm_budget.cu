// Column budgets of the current state (column_integral_definite!):
//   total_water  = sum_k dz (vartheta_l + theta_i rho_i / rho_l)
//                  (rre.jl:502-511; energy_hydrology.jl:1282-1300)
//   total_energy = sum_k dz rho_e_int   (energy_hydrology.jl:1302-1320)
// One thread per column; sums accumulated in FP64 in layer order.

#include <cuda_runtime.h>

#include "clm_internal.cuh"

namespace clm {

__global__ void budgets_kernel(StepArgs A, int eh, double* __restrict__ W, double* __restrict__ Eo) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= A.L.stride) return;
  const int n = A.L.col_n[s];
  if (n <= 0) {
    W[s] = 0.0;
    Eo[s] = 0.0;
    return;
  }
  const int tile = s / kTile, lane = s % kTile;
  const int64_t base = A.L.tile_off[tile] + lane;
  const double dzu = (A.z_hi[s] - A.z_lo[s]) / n;
  const double r = A.E.rho_i_over_rho_l;
  double w = 0.0, e = 0.0;
  for (int k = 0; k < n; ++k) {
    const int64_t i = base + (int64_t)k * kTile;
    const double dz = A.geo.w ? A.geo.w[i] : dzu;  // layer width (stretched: per layer)
    double v = A.v[i];
    if (eh) {
      v += A.ti[i] * r;
      e += dz * A.e[i];
    }
    w += dz * v;
  }
  W[s] = w;
  Eo[s] = e;
}

cudaError_t launch_budgets(const StepArgs& A, int model, double* W, double* E, cudaStream_t st) {
  budgets_kernel<<<(A.L.stride + 127) / 128, 128, 0, st>>>(A, model == CLM_MODEL_ENERGY_HYDROLOGY, W, E);
  return cudaGetLastError();
}

}  // namespace clm
