// Layout conversion between the reference's column layout (cells of a
// column contiguous, level 0 at the bottom; what ClimaCore's VIJFH/VF data
// and the C ABI use) and the internal tiled layer-major layout
// (clm_internal.cuh). One CTA per 32-column tile: each warp reads whole
// columns with coalesced loads into shared memory, then the CTA writes the
// tile layer by layer with coalesced stores (and the reverse).

#include <cuda_runtime.h>

#include "clm_internal.cuh"

namespace clm {

constexpr int kXposeThreads = 256;
constexpr int kXposePad = kTile + 1;  // padded row (in doubles) of the staging tile

__global__ void __launch_bounds__(kXposeThreads)
    ref_to_internal_kernel(Layout L, const int32_t* __restrict__ ref_off,
                           const double* __restrict__ src, double* __restrict__ dst,
                           int ncomp, int tile0) {
  extern __shared__ double tileb[];  // [nmax * ncomp][kXposePad]
  const int tile = tile0 + blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = blockDim.x >> 5;
  const int nt = L.tile_n[tile];
  for (int j = warp; j < kTile; j += nw) {
    const int s = tile * kTile + j;
    const int n = L.col_n[s];
    if (n <= 0) continue;
    const int c = L.perm[s];
    const int64_t o = (int64_t)ref_off[c] * ncomp;
    for (int q = lane; q < n * ncomp; q += 32) tileb[q * kXposePad + j] = src[o + q];
  }
  __syncthreads();
  const int64_t to = L.tile_off[tile] * ncomp;
  for (int q = threadIdx.x; q < nt * ncomp * kTile; q += blockDim.x) {
    const int kk = q / kTile, j = q % kTile;
    const int s = tile * kTile + j;
    if (kk < L.col_n[s] * ncomp) dst[to + q] = tileb[kk * kXposePad + j];
  }
}

__global__ void __launch_bounds__(kXposeThreads)
    internal_to_ref_kernel(Layout L, const int32_t* __restrict__ ref_off,
                           const double* __restrict__ src, double* __restrict__ dst,
                           int ncomp, int tile0) {
  extern __shared__ double tileb[];
  const int tile = tile0 + blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = blockDim.x >> 5;
  const int nt = L.tile_n[tile];
  const int64_t to = L.tile_off[tile] * ncomp;
  for (int q = threadIdx.x; q < nt * ncomp * kTile; q += blockDim.x) {
    const int kk = q / kTile, j = q % kTile;
    const int s = tile * kTile + j;
    if (kk < L.col_n[s] * ncomp) tileb[kk * kXposePad + j] = src[to + q];
  }
  __syncthreads();
  for (int j = warp; j < kTile; j += nw) {
    const int s = tile * kTile + j;
    const int n = L.col_n[s];
    if (n <= 0) continue;
    const int c = L.perm[s];
    const int64_t o = (int64_t)ref_off[c] * ncomp;
    for (int q = lane; q < n * ncomp; q += 32) dst[o + q] = tileb[q * kXposePad + j];
  }
}

// per-column arrays: sorted <-> original order
__global__ void cols_to_sorted_kernel(Layout L, const double* __restrict__ src,
                                      double* __restrict__ dst) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= L.stride) return;
  const int c = L.perm[s];
  dst[s] = (c >= 0) ? src[c] : 0.0;
}

__global__ void cols_to_orig_kernel(Layout L, const double* __restrict__ src,
                                    double* __restrict__ dst) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= L.stride) return;
  const int c = L.perm[s];
  if (c >= 0) dst[c] = src[s];
}

size_t xpose_smem(const Layout& L, int ncomp) {
  return (size_t)L.nmax * ncomp * kXposePad * sizeof(double);
}

// tiles [tile0, tile0 + ntl) (ntl < 0: through the last tile)
cudaError_t ref_to_internal(const Layout& L, const int32_t* ref_off, const double* src,
                            double* dst, int ncomp, cudaStream_t st, int tile0, int ntl) {
  const size_t sm = xpose_smem(L, ncomp);
  cudaError_t e = cudaFuncSetAttribute(ref_to_internal_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  const int grid = ntl < 0 ? L.ntiles - tile0 : ntl;
  if (grid <= 0) return cudaSuccess;
  ref_to_internal_kernel<<<grid, kXposeThreads, sm, st>>>(L, ref_off, src, dst, ncomp, tile0);
  return cudaGetLastError();
}

cudaError_t internal_to_ref(const Layout& L, const int32_t* ref_off, const double* src,
                            double* dst, int ncomp, cudaStream_t st, int tile0, int ntl) {
  const size_t sm = xpose_smem(L, ncomp);
  cudaError_t e = cudaFuncSetAttribute(internal_to_ref_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  const int grid = ntl < 0 ? L.ntiles - tile0 : ntl;
  if (grid <= 0) return cudaSuccess;
  internal_to_ref_kernel<<<grid, kXposeThreads, sm, st>>>(L, ref_off, src, dst, ncomp, tile0);
  return cudaGetLastError();
}

cudaError_t cols_to_sorted(const Layout& L, const double* src, double* dst, cudaStream_t st) {
  cols_to_sorted_kernel<<<(L.stride + 255) / 256, 256, 0, st>>>(L, src, dst);
  return cudaGetLastError();
}

cudaError_t cols_to_orig(const Layout& L, const double* src, double* dst, cudaStream_t st) {
  cols_to_orig_kernel<<<(L.stride + 255) / 256, 256, 0, st>>>(L, src, dst);
  return cudaGetLastError();
}

}  // namespace clm
