// Argument blocks of the closure-level kernels (clm_closures.cu) and their
// C entry points (clm_closures_api.cu).
#pragma once

#include <cuda_runtime.h>

#include "clm_internal.cuh"

namespace clm {

enum ClosureKind { CL_AUX = 0, CL_EXP = 1, CL_IMP = 2, CL_JAC = 3, CL_ATM = 4 };

struct ClosureArgs {
  StepArgs A;              // parameters, forcing, config (state pointers unused)
  int model;               // enum clm_model
  const int32_t* ref_off;  // [ncol + 1]
  const double* v;         // state, reference layout
  const double* ti;
  const double* e;
  double t;
  double dtgamma;
  // outputs (reference layout; any may be null)
  double *K, *psi, *theta_l, *T, *kappa, *Tf;  // AUX
  double* bc;                                  // [4][ncol] original column order
  double *dv, *dti, *de, *dFw, *dFe;           // EXP / IMP
  double *Wvv, *Wev, *Wee;                     // JAC: 3 per cell
  double* atm_out;                             // ATM: [CLM_AF_NFIELDS][ncol] original order
};

struct SolveArgs {
  Layout L;
  const int32_t* ref_off;
  const double *Wvv, *Wev, *Wee, *fv, *fe;
  double *dv, *de;
};

cudaError_t launch_closure(int kind, const ClosureArgs& C, cudaStream_t st);
cudaError_t launch_solve(const SolveArgs& S, cudaStream_t st);

}  // namespace clm
