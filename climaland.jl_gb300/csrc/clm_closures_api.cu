// C entry points of the closure-level API (clm_update_aux, clm_exp_tendency,
// clm_imp_tendency, clm_jacobian, clm_solve). Each call converts the
// handle's state to the reference layout in a scratch buffer, runs one
// closure kernel (clm_closures.cu) and copies the requested outputs to the
// caller's host buffers. These entry points exist for per-closure parity
// and for callers with their own time stepper; the fused clm_step is the
// fast path.

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/climaland_cuda.h"
#include "clm_closures.cuh"

struct clm_handle;

namespace clm {
cudaError_t internal_to_ref(const Layout& L, const XFields& F, cudaStream_t st, int tile0 = 0,
                            int ntl = -1);
StepArgs handle_step_args(clm_handle* h);
Layout handle_layout(clm_handle* h);
int handle_ready(clm_handle* h);
int handle_fail(clm_handle* h, int code, const char* msg);
int handle_cuda_fail(clm_handle* h, cudaError_t e, const char* what);
cudaStream_t handle_stream(clm_handle* h);
const int32_t* handle_ref_off(clm_handle* h);
int64_t handle_ncells_ref(clm_handle* h);
int handle_ncol(clm_handle* h);
int handle_model(clm_handle* h);
double* handle_state_ptr(clm_handle* h, int which);
}  // namespace clm

using namespace clm;

namespace {

// Device scratch owned by one call.
struct Scratch {
  std::vector<double*> bufs;
  ~Scratch() {
    for (double* p : bufs) cudaFree(p);
  }
  double* get(size_t n, cudaError_t& err) {
    double* p = nullptr;
    if (err == cudaSuccess) err = cudaMalloc(&p, sizeof(double) * (n ? n : 1));
    if (err == cudaSuccess) bufs.push_back(p);
    return p;
  }
};

#define CLM_CUDA(h, call)                                          \
  do {                                                             \
    cudaError_t _e = (call);                                       \
    if (_e != cudaSuccess) return handle_cuda_fail((h), _e, #call); \
  } while (0)

// State in reference layout into scratch.
int state_ref(clm_handle* h, Scratch& S, const double** v, const double** ti, const double** e) {
  const bool eh = handle_model(h) == CLM_MODEL_ENERGY_HYDROLOGY;
  const int64_t nc = handle_ncells_ref(h);
  cudaError_t err = cudaSuccess;
  double* bv = S.get(nc, err);
  double* bt = eh ? S.get(nc, err) : nullptr;
  double* be = eh ? S.get(nc, err) : nullptr;
  if (err != cudaSuccess) return handle_cuda_fail(h, err, "cudaMalloc");
  Layout L = handle_layout(h);
  cudaStream_t st = handle_stream(h);
  XFields F{};
  F.nf = eh ? 3 : 1;
  double* outs[3] = {bv, bt, be};
  for (int i = 0; i < F.nf; ++i) {
    F.src[i] = handle_state_ptr(h, i);
    F.dst[i] = outs[i];
  }
  CLM_CUDA(h, internal_to_ref(L, F, st));
  *v = bv;
  *ti = bt;
  *e = be;
  return CLM_OK;
}

ClosureArgs base_args(clm_handle* h) {
  ClosureArgs C{};
  C.A = handle_step_args(h);
  C.model = handle_model(h);
  C.ref_off = handle_ref_off(h);
  return C;
}

int closure_ready(clm_handle* h) { return handle_ready(h); }

int copy_out(clm_handle* h, double* host, const double* dev, size_t n) {
  if (!host) return CLM_OK;
  CLM_CUDA(h, cudaMemcpyAsync(host, dev, sizeof(double) * n, cudaMemcpyDeviceToHost, handle_stream(h)));
  return CLM_OK;
}

int tendency(clm_handle* h, int kind, double t, double* dv, double* dti, double* de, double* dFw,
             double* dFe) {
  int rc = closure_ready(h);
  if (rc != CLM_OK) return rc;
  Scratch S;
  ClosureArgs C = base_args(h);
  rc = state_ref(h, S, &C.v, &C.ti, &C.e);
  if (rc != CLM_OK) return rc;
  const int64_t nc = handle_ncells_ref(h);
  const int ncol = handle_ncol(h);
  cudaError_t err = cudaSuccess;
  C.dv = S.get(nc, err);
  C.dti = S.get(nc, err);
  C.de = S.get(nc, err);
  C.dFw = S.get(ncol, err);
  C.dFe = S.get(ncol, err);
  if (err != cudaSuccess) return handle_cuda_fail(h, err, "cudaMalloc");
  C.t = t;
  CLM_CUDA(h, launch_closure(kind, C, handle_stream(h)));
  const bool eh = C.model == CLM_MODEL_ENERGY_HYDROLOGY;
  if ((rc = copy_out(h, dv, C.dv, nc))) return rc;
  if (eh) {
    if ((rc = copy_out(h, dti, C.dti, nc))) return rc;
    if ((rc = copy_out(h, de, C.de, nc))) return rc;
    if ((rc = copy_out(h, dFe, C.dFe, ncol))) return rc;
  }
  if ((rc = copy_out(h, dFw, C.dFw, ncol))) return rc;
  CLM_CUDA(h, cudaStreamSynchronize(handle_stream(h)));
  return CLM_OK;
}

}  // namespace

extern "C" {

int clm_update_aux(clm_handle* h, double t, double* K, double* psi, double* theta_l, double* T,
                   double* kappa, double* Tf, double* bc) {
  int rc = closure_ready(h);
  if (rc != CLM_OK) return rc;
  Scratch S;
  ClosureArgs C = base_args(h);
  rc = state_ref(h, S, &C.v, &C.ti, &C.e);
  if (rc != CLM_OK) return rc;
  const int64_t nc = handle_ncells_ref(h);
  const int ncol = handle_ncol(h);
  cudaError_t err = cudaSuccess;
  C.K = S.get(nc, err);
  C.psi = S.get(nc, err);
  const bool eh = C.model == CLM_MODEL_ENERGY_HYDROLOGY;
  if (eh) {
    C.theta_l = S.get(nc, err);
    C.T = S.get(nc, err);
    C.kappa = S.get(nc, err);
    C.Tf = S.get(nc, err);
  }
  C.bc = S.get(4 * (size_t)ncol, err);
  if (err != cudaSuccess) return handle_cuda_fail(h, err, "cudaMalloc");
  CLM_CUDA(h, cudaMemsetAsync(C.bc, 0, sizeof(double) * 4 * ncol, handle_stream(h)));
  C.t = t;
  CLM_CUDA(h, launch_closure(CL_AUX, C, handle_stream(h)));
  if ((rc = copy_out(h, K, C.K, nc))) return rc;
  if ((rc = copy_out(h, psi, C.psi, nc))) return rc;
  if (eh) {
    if ((rc = copy_out(h, theta_l, C.theta_l, nc))) return rc;
    if ((rc = copy_out(h, T, C.T, nc))) return rc;
    if ((rc = copy_out(h, kappa, C.kappa, nc))) return rc;
    if ((rc = copy_out(h, Tf, C.Tf, nc))) return rc;
  }
  if ((rc = copy_out(h, bc, C.bc, 4 * (size_t)ncol))) return rc;
  CLM_CUDA(h, cudaStreamSynchronize(handle_stream(h)));
  return CLM_OK;
}

int clm_atmos_fluxes(clm_handle* h, double* out, int32_t nfields) {
  int rc = closure_ready(h);
  if (rc != CLM_OK) return rc;
  if (handle_step_args(h).bc_tw != CLM_BC_ATMOS)
    return handle_fail(h, CLM_ERR_ARG, "the top boundary is not CLM_BC_ATMOS");
  if (!out || nfields != CLM_AF_NFIELDS) return handle_fail(h, CLM_ERR_ARG, "expected CLM_AF_NFIELDS rows");
  Scratch S;
  ClosureArgs C = base_args(h);
  rc = state_ref(h, S, &C.v, &C.ti, &C.e);
  if (rc != CLM_OK) return rc;
  const int ncol = handle_ncol(h);
  cudaError_t err = cudaSuccess;
  C.atm_out = S.get((size_t)CLM_AF_NFIELDS * ncol, err);
  if (err != cudaSuccess) return handle_cuda_fail(h, err, "cudaMalloc");
  CLM_CUDA(h, launch_closure(CL_ATM, C, handle_stream(h)));
  if ((rc = copy_out(h, out, C.atm_out, (size_t)CLM_AF_NFIELDS * ncol))) return rc;
  CLM_CUDA(h, cudaStreamSynchronize(handle_stream(h)));
  return CLM_OK;
}

int clm_exp_tendency(clm_handle* h, double t, double* dv, double* dti, double* de, double* dFw,
                     double* dFe) {
  return tendency(h, CL_EXP, t, dv, dti, de, dFw, dFe);
}

int clm_imp_tendency(clm_handle* h, double t, double* dv, double* dti, double* de, double* dFw,
                     double* dFe) {
  return tendency(h, CL_IMP, t, dv, dti, de, dFw, dFe);
}

int clm_jacobian(clm_handle* h, double t, double dtgamma, double* Wvv, double* Wev, double* Wee) {
  int rc = closure_ready(h);
  if (rc != CLM_OK) return rc;
  if (!Wvv) return handle_fail(h, CLM_ERR_ARG, "W_vv is required");
  Scratch S;
  ClosureArgs C = base_args(h);
  rc = state_ref(h, S, &C.v, &C.ti, &C.e);
  if (rc != CLM_OK) return rc;
  const int64_t nc = handle_ncells_ref(h);
  const bool eh = C.model == CLM_MODEL_ENERGY_HYDROLOGY;
  cudaError_t err = cudaSuccess;
  C.Wvv = S.get(3 * nc, err);
  if (eh) {
    C.Wev = S.get(3 * nc, err);
    C.Wee = S.get(3 * nc, err);
  }
  if (err != cudaSuccess) return handle_cuda_fail(h, err, "cudaMalloc");
  C.t = t;
  C.dtgamma = dtgamma;
  CLM_CUDA(h, launch_closure(CL_JAC, C, handle_stream(h)));
  if ((rc = copy_out(h, Wvv, C.Wvv, 3 * nc))) return rc;
  if (eh) {
    if ((rc = copy_out(h, Wev, C.Wev, 3 * nc))) return rc;
    if ((rc = copy_out(h, Wee, C.Wee, 3 * nc))) return rc;
  }
  CLM_CUDA(h, cudaStreamSynchronize(handle_stream(h)));
  return CLM_OK;
}

int clm_solve(clm_handle* h, const double* Wvv, const double* Wev, const double* Wee, const double* fv,
              const double* fe, double* dv, double* de) {
  if (!h) return CLM_ERR_ARG;
  const Layout L = handle_layout(h);
  if (!L.col_n) return handle_fail(h, CLM_ERR_STATE, "clm_set_geometry has not been called");
  if (!Wvv || !fv || !dv) return handle_fail(h, CLM_ERR_ARG, "W_vv, f_v and delta_v are required");
  const bool eh = handle_model(h) == CLM_MODEL_ENERGY_HYDROLOGY && Wev && Wee && fe && de;
  const int64_t nc = handle_ncells_ref(h);
  cudaStream_t st = handle_stream(h);
  Scratch S;
  cudaError_t err = cudaSuccess;
  SolveArgs A{};
  A.L = L;
  A.ref_off = handle_ref_off(h);
  double* wvv = S.get(3 * nc, err);
  double* f1 = S.get(nc, err);
  A.dv = S.get(nc, err);
  double *wev = nullptr, *wee = nullptr, *f2 = nullptr;
  if (eh) {
    wev = S.get(3 * nc, err);
    wee = S.get(3 * nc, err);
    f2 = S.get(nc, err);
    A.de = S.get(nc, err);
  }
  if (err != cudaSuccess) return handle_cuda_fail(h, err, "cudaMalloc");
  CLM_CUDA(h, cudaMemcpyAsync(wvv, Wvv, sizeof(double) * 3 * nc, cudaMemcpyHostToDevice, st));
  CLM_CUDA(h, cudaMemcpyAsync(f1, fv, sizeof(double) * nc, cudaMemcpyHostToDevice, st));
  if (eh) {
    CLM_CUDA(h, cudaMemcpyAsync(wev, Wev, sizeof(double) * 3 * nc, cudaMemcpyHostToDevice, st));
    CLM_CUDA(h, cudaMemcpyAsync(wee, Wee, sizeof(double) * 3 * nc, cudaMemcpyHostToDevice, st));
    CLM_CUDA(h, cudaMemcpyAsync(f2, fe, sizeof(double) * nc, cudaMemcpyHostToDevice, st));
  }
  A.Wvv = wvv;
  A.fv = f1;
  A.Wev = wev;
  A.Wee = wee;
  A.fe = f2;
  CLM_CUDA(h, launch_solve(A, st));
  CLM_CUDA(h, cudaMemcpyAsync(dv, A.dv, sizeof(double) * nc, cudaMemcpyDeviceToHost, st));
  if (eh) CLM_CUDA(h, cudaMemcpyAsync(de, A.de, sizeof(double) * nc, cudaMemcpyDeviceToHost, st));
  CLM_CUDA(h, cudaStreamSynchronize(st));
  return CLM_OK;
}

}  // extern "C"
