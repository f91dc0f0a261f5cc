// C entry points of the learned-guess network (no reference counterpart):
// a trainer object holding FP32 master weights, Adam moments and the
// input/output standardisation, trained on the GPU by the kernels of
// clm_mlp.cu, and its weight blob (the format clm_load_mlp accepts).

#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/climaland_cuda.h"
#include "clm_mlp.cuh"

namespace clm {
cudaError_t mlp_train_step(const float* P, const float* norm, const float* X, const float* Y,
                           int64_t row0, int nrows, float* grads, float* loss_sum, cudaStream_t st);
cudaError_t mlp_adam(float* P, float* G, float* M, float* V, int step, float lr, cudaStream_t st);
cudaError_t mlp_predict(const float* P, const float* norm, const float* X, int64_t nrows, float* Y,
                        cudaStream_t st);
}  // namespace clm

using namespace clm;

struct clm_mlp {
  float* P = nullptr;     // [kMlpParams]
  float* G = nullptr;     // gradient
  float* M = nullptr;     // Adam first moment
  float* V = nullptr;     // Adam second moment
  float* norm = nullptr;  // in_mean, in_std, out_mean, out_std
  float* loss = nullptr;  // per-step loss sums
  int loss_cap = 0;
  int adam_step = 0;
};

namespace {

uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

int ok(cudaError_t e) {
  if (e == cudaSuccess) return CLM_OK;
  cudaGetLastError();
  return CLM_ERR_CUDA;
}

}  // namespace

extern "C" {

int64_t clm_mlp_blob_bytes(void) { return kMlpBlobBytes; }

int64_t clm_mlp_nparams(void) { return kMlpParams; }

int clm_mlp_create(uint64_t seed, clm_mlp** out) {
  if (!out) return CLM_ERR_ARG;
  *out = nullptr;
  clm_mlp* m = new (std::nothrow) clm_mlp();
  if (!m) return CLM_ERR_ARG;
  const size_t pb = sizeof(float) * kMlpParams;
  const size_t nb = sizeof(float) * (2 * kMlpIn + 2 * kMlpOut);
  if (cudaMalloc(&m->P, pb) != cudaSuccess || cudaMalloc(&m->G, pb) != cudaSuccess ||
      cudaMalloc(&m->M, pb) != cudaSuccess || cudaMalloc(&m->V, pb) != cudaSuccess ||
      cudaMalloc(&m->norm, nb) != cudaSuccess) {
    cudaGetLastError();
    clm_mlp_destroy(m);
    return CLM_ERR_CUDA;
  }
  // Glorot-uniform weights, zero biases; identity standardisation.
  std::vector<float> P(kMlpParams, 0.0f);
  uint64_t s = seed ^ 0x5EEDULL;
  auto fill = [&](int base, int fan_in, int fan_out, int rows_used) {
    const float a = std::sqrt(6.0f / (float)(fan_in + fan_out));
    for (int i = 0; i < rows_used * fan_out; ++i) {
      const double u = (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
      P[base + i] = (float)((2.0 * u - 1.0) * a);
    }
  };
  fill(kMlpW1, kMlpIn, kMlpHidden, kMlpIn);  // padded input rows stay zero
  fill(kMlpW2, kMlpHidden, kMlpHidden, kMlpHidden);
  fill(kMlpW3, kMlpHidden, kMlpOut, kMlpHidden);
  std::vector<float> norm(2 * kMlpIn + 2 * kMlpOut, 0.0f);
  for (int i = 0; i < kMlpIn; ++i) norm[kMlpIn + i] = 1.0f;
  for (int i = 0; i < kMlpOut; ++i) norm[2 * kMlpIn + kMlpOut + i] = 1.0f;
  if (cudaMemcpy(m->P, P.data(), pb, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(m->G, 0, pb) != cudaSuccess || cudaMemset(m->M, 0, pb) != cudaSuccess ||
      cudaMemset(m->V, 0, pb) != cudaSuccess ||
      cudaMemcpy(m->norm, norm.data(), nb, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaGetLastError();
    clm_mlp_destroy(m);
    return CLM_ERR_CUDA;
  }
  *out = m;
  return CLM_OK;
}

void clm_mlp_destroy(clm_mlp* m) {
  if (!m) return;
  cudaFree(m->P);
  cudaFree(m->G);
  cudaFree(m->M);
  cudaFree(m->V);
  cudaFree(m->norm);
  cudaFree(m->loss);
  cudaGetLastError();
  delete m;
}

int clm_mlp_set_normalization(clm_mlp* m, const float* in_mean, const float* in_std,
                              const float* out_mean, const float* out_std) {
  if (!m || !in_mean || !in_std || !out_mean || !out_std) return CLM_ERR_ARG;
  std::vector<float> n(2 * kMlpIn + 2 * kMlpOut);
  std::memcpy(n.data(), in_mean, sizeof(float) * kMlpIn);
  std::memcpy(n.data() + kMlpIn, in_std, sizeof(float) * kMlpIn);
  std::memcpy(n.data() + 2 * kMlpIn, out_mean, sizeof(float) * kMlpOut);
  std::memcpy(n.data() + 2 * kMlpIn + kMlpOut, out_std, sizeof(float) * kMlpOut);
  for (int i = 0; i < kMlpOut; ++i)
    if (!(n[2 * kMlpIn + kMlpOut + i] > 0.0f)) return CLM_ERR_ARG;
  return ok(cudaMemcpy(m->norm, n.data(), sizeof(float) * n.size(), cudaMemcpyHostToDevice));
}

int clm_mlp_train(clm_mlp* m, const float* X, const float* Y, int64_t nrows, int32_t batch,
                  int32_t nsteps, float lr, float* loss_host, void* stream) {
  if (!m || !X || !Y || nrows <= 0 || batch <= 0 || nsteps < 0 || !(lr > 0)) return CLM_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (m->loss_cap < nsteps) {
    cudaFree(m->loss);
    m->loss = nullptr;
    if (cudaMalloc(&m->loss, sizeof(float) * (nsteps > 0 ? nsteps : 1)) != cudaSuccess) return ok(cudaErrorMemoryAllocation);
    m->loss_cap = nsteps;
  }
  if (nsteps > 0) {
    int rc = ok(cudaMemsetAsync(m->loss, 0, sizeof(float) * nsteps, st));
    if (rc) return rc;
  }
  int64_t row0 = 0;
  for (int i = 0; i < nsteps; ++i) {
    if (row0 >= nrows) row0 = 0;
    const int nb = (int)((nrows - row0) < batch ? (nrows - row0) : batch);
    int rc = ok(mlp_train_step(m->P, m->norm, X, Y, row0, nb, m->G, m->loss + i, st));
    if (rc) return rc;
    rc = ok(mlp_adam(m->P, m->G, m->M, m->V, ++m->adam_step, lr, st));
    if (rc) return rc;
    row0 += nb;
  }
  if (loss_host && nsteps > 0) {
    int rc = ok(cudaMemcpyAsync(loss_host, m->loss, sizeof(float) * nsteps, cudaMemcpyDeviceToHost, st));
    if (rc) return rc;
  }
  return ok(cudaStreamSynchronize(st));
}

int clm_mlp_gradients(clm_mlp* m, const float* X, const float* Y, int32_t nrows, float* grad_host,
                      float* loss_host) {
  if (!m || !X || !Y || nrows <= 0 || !grad_host) return CLM_ERR_ARG;
  float* loss = nullptr;
  int rc = ok(cudaMalloc(&loss, sizeof(float)));
  if (rc) return rc;
  rc = ok(cudaMemset(loss, 0, sizeof(float)));
  if (!rc) rc = ok(cudaMemset(m->G, 0, sizeof(float) * kMlpParams));
  if (!rc) rc = ok(mlp_train_step(m->P, m->norm, X, Y, 0, nrows, m->G, loss, nullptr));
  if (!rc) rc = ok(cudaMemcpy(grad_host, m->G, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
  if (!rc && loss_host) rc = ok(cudaMemcpy(loss_host, loss, sizeof(float), cudaMemcpyDeviceToHost));
  if (!rc) rc = ok(cudaMemset(m->G, 0, sizeof(float) * kMlpParams));
  cudaFree(loss);
  return rc;
}

int clm_mlp_predict(clm_mlp* m, const float* X, int64_t nrows, float* Y, void* stream) {
  if (!m || !X || !Y || nrows < 0) return CLM_ERR_ARG;
  if (nrows == 0) return CLM_OK;
  return ok(mlp_predict(m->P, m->norm, X, nrows, Y, static_cast<cudaStream_t>(stream)));
}

int clm_mlp_get(const clm_mlp* m, void* blob, int64_t nbytes) {
  if (!m || !blob || nbytes < kMlpBlobBytes) return CLM_ERR_ARG;
  MlpBlobHeader hd{kMlpMagic, kMlpIn, kMlpHidden, kMlpOut};
  unsigned char* b = static_cast<unsigned char*>(blob);
  std::memcpy(b, &hd, sizeof hd);
  float* f = reinterpret_cast<float*>(b + sizeof hd);
  int rc = ok(cudaMemcpy(f, m->norm, sizeof(float) * (2 * kMlpIn + 2 * kMlpOut), cudaMemcpyDeviceToHost));
  if (rc) return rc;
  return ok(cudaMemcpy(f + 2 * kMlpIn + 2 * kMlpOut, m->P, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
}

int clm_mlp_set(clm_mlp* m, const void* blob, int64_t nbytes) {
  if (!m || !blob || nbytes < kMlpBlobBytes) return CLM_ERR_ARG;
  MlpBlobHeader hd;
  std::memcpy(&hd, blob, sizeof hd);
  if (hd.magic != kMlpMagic || hd.nin != (uint32_t)kMlpIn || hd.nhidden != (uint32_t)kMlpHidden ||
      hd.nout != (uint32_t)kMlpOut)
    return CLM_ERR_ARG;
  const float* f = reinterpret_cast<const float*>(static_cast<const unsigned char*>(blob) + sizeof hd);
  int rc = ok(cudaMemcpy(m->norm, f, sizeof(float) * (2 * kMlpIn + 2 * kMlpOut), cudaMemcpyHostToDevice));
  if (rc) return rc;
  return ok(cudaMemcpy(m->P, f + 2 * kMlpIn + 2 * kMlpOut, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice));
}

}  // extern "C"
