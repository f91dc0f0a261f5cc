// Layout conversion between the reference's column layout (cells of a
// column contiguous, level 0 at the bottom; what ClimaCore's VIJFH/VF data
// and the C ABI use) and the internal tiled layer-major layout
// (clm_internal.cuh). One CTA per 32-column tile: each warp reads whole
// columns (contiguous runs) into a padded shared-memory tile, then the CTA
// writes the tile layer by layer with coalesced stores (and the reverse).

#include <cuda_runtime.h>

#include "clm_internal.cuh"

namespace clm {

constexpr int kXposeThreads = 256;
constexpr int kXposePad = kTile + 1;  // padded row (in doubles) of the staging tile

// Per tile, precomputed per layout: the first cell of each column in the
// reference layout and the column's layer count. A CTA starts its loads
// after one round of independent coalesced reads.
struct TileCols {
  int n[kTile];        // layer count of column j (0: padding)
  int64_t off[kTile];  // first cell of column j in the reference layout
};

__device__ __forceinline__ void tile_cols(const Layout& L, int tile, TileCols& tc) {
  const int i = threadIdx.x;
  if (i < kTile) {
    tc.n[i] = L.col_n[tile * kTile + i];
    tc.off[i] = L.slot_ref[tile * kTile + i];
  }
  __syncthreads();
}

// Each warp moves whole columns (lane k <-> layer k, up to 64 layers in two
// rounds); the CTA's 8 warps cover the tile's 32 columns, all loads of a
// warp issued before its stores.
constexpr int kXposeWarps = kXposeThreads / 32;
constexpr int kColsPerWarp = kTile / kXposeWarps;
constexpr int kRounds = (kMaxLayers + 31) / 32;
static_assert(kTile % kXposeWarps == 0, "warps must split the tile's columns evenly");

__global__ void __launch_bounds__(kXposeThreads)
    ref_to_internal_kernel(Layout L, const double* __restrict__ src, double* __restrict__ dst,
                           int tile0) {
  extern __shared__ double tileb[];  // [nmax][kXposePad]
  __shared__ TileCols tc;
  const int tile = tile0 + blockIdx.x;
  tile_cols(L, tile, tc);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double v[kColsPerWarp][kRounds];
#pragma unroll
  for (int c = 0; c < kColsPerWarp; ++c) {
    const int j = warp + c * kXposeWarps;
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
      const int k = lane + 32 * r;
      if (k < tc.n[j]) v[c][r] = src[tc.off[j] + k];
    }
  }
#pragma unroll
  for (int c = 0; c < kColsPerWarp; ++c) {
    const int j = warp + c * kXposeWarps;
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
      const int k = lane + 32 * r;
      if (k < tc.n[j]) tileb[k * kXposePad + j] = v[c][r];
    }
  }
  __syncthreads();
  const int nt = L.tile_n[tile];
  const int64_t to = L.tile_off[tile];
  for (int q = threadIdx.x; q < nt * kTile; q += blockDim.x) {
    const int k = q / kTile, jj = q % kTile;
    if (k < tc.n[jj]) dst[to + q] = tileb[k * kXposePad + jj];
  }
}

// Layer-major loads in flight per thread before their shared-memory stores.
constexpr int kXposeBatch = 4;

__global__ void __launch_bounds__(kXposeThreads)
    internal_to_ref_kernel(Layout L, const double* __restrict__ src, double* __restrict__ dst,
                           int tile0) {
  extern __shared__ double tileb[];
  __shared__ TileCols tc;
  const int tile = tile0 + blockIdx.x;
  tile_cols(L, tile, tc);
  const int nq = L.tile_n[tile] * kTile;
  const int64_t so = L.tile_off[tile];
  for (int base = 0; base < nq; base += blockDim.x * kXposeBatch) {
    double v[kXposeBatch];
    int q[kXposeBatch];
#pragma unroll
    for (int r = 0; r < kXposeBatch; ++r) {
      const int qq = base + r * blockDim.x + threadIdx.x;
      q[r] = -1;
      if (qq < nq && qq / kTile < tc.n[qq % kTile]) {
        q[r] = qq;
        v[r] = src[so + qq];
      }
    }
#pragma unroll
    for (int r = 0; r < kXposeBatch; ++r)
      if (q[r] >= 0) tileb[(q[r] / kTile) * kXposePad + q[r] % kTile] = v[r];
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int c = 0; c < kColsPerWarp; ++c) {
    const int j = warp + c * kXposeWarps;
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
      const int k = lane + 32 * r;
      if (k < tc.n[j]) dst[tc.off[j] + k] = tileb[k * kXposePad + j];
    }
  }
}

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

size_t xpose_smem(const Layout& L) { return (size_t)L.nmax * kXposePad * sizeof(double); }

// tiles [tile0, tile0 + ntl) (ntl < 0: through the last tile)
cudaError_t ref_to_internal(const Layout& L, const double* src, double* dst, cudaStream_t st,
                            int tile0, int ntl) {
  const size_t sm = xpose_smem(L);
  cudaError_t e = cudaFuncSetAttribute(ref_to_internal_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  const int grid = ntl < 0 ? L.ntiles - tile0 : ntl;
  if (grid <= 0) return cudaSuccess;
  ref_to_internal_kernel<<<grid, kXposeThreads, sm, st>>>(L, src, dst, tile0);
  return cudaGetLastError();
}

cudaError_t internal_to_ref(const Layout& L, const double* src, double* dst, cudaStream_t st,
                            int tile0, int ntl) {
  const size_t sm = xpose_smem(L);
  cudaError_t e = cudaFuncSetAttribute(internal_to_ref_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  const int grid = ntl < 0 ? L.ntiles - tile0 : ntl;
  if (grid <= 0) return cudaSuccess;
  internal_to_ref_kernel<<<grid, kXposeThreads, sm, st>>>(L, src, dst, tile0);
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
