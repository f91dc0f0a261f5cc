// Layout conversion between the reference's column layout (cells of a
// column contiguous, level 0 at the bottom; what ClimaCore's VIJFH/VF data
// and the C ABI use) and the internal tiled layer-major layout
// (clm_internal.cuh). One CTA per 32-column tile and up to three state
// fields: each warp reads whole columns (contiguous runs) of every field into
// padded shared-memory tiles, then the CTA writes them layer by layer with
// coalesced stores (and the reverse).

#include <cuda_runtime.h>

#include "clm_internal.cuh"

namespace clm {

constexpr int kXposeThreads = 256;
constexpr int kXposePad = kTile + 1;  // padded row (in doubles) of the staging tile

// Per tile, precomputed per layout: the first cell of each column in the
// reference layout and the column's layer count. A CTA starts its loads
// after one round of independent coalesced reads. `flat`: the tile's columns
// follow each other in the reference layout (columns kept in their order,
// as for equal depths), so the tile is one contiguous run of `total` cells;
// `nu`: their common layer count, or 0.
struct TileCols {
  int n[kTile];        // layer count of column j (0: padding)
  int64_t off[kTile];  // first cell of column j in the reference layout
  int pre[kTile + 1];  // prefix sums of n
  int flat, nu;
};

__device__ __forceinline__ void tile_cols(const Layout& L, int tile, TileCols& tc) {
  const int i = threadIdx.x;
  if (i < kTile) {
    const int n = L.col_n[tile * kTile + i];
    const int64_t off = L.slot_ref[tile * kTile + i];
    tc.n[i] = n;
    tc.off[i] = off;
    int x = n;  // inclusive warp scan
    for (int d = 1; d < 32; d <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, d);
      if (i >= d) x += y;
    }
    tc.pre[i + 1] = x;
    if (i == 0) tc.pre[0] = 0;
    // contiguous: the next column (if it holds cells) starts where this one ends
    const int64_t next_off = __shfl_down_sync(0xffffffffu, off, 1);
    const int next_n = __shfl_down_sync(0xffffffffu, n, 1);
    const bool ok = i == kTile - 1 || next_n == 0 || next_off == off + n;
    const int n0 = __shfl_sync(0xffffffffu, n, 0);
    const bool same = n == 0 || n == n0;
    const unsigned all_ok = __all_sync(0xffffffffu, ok);
    const unsigned all_same = __all_sync(0xffffffffu, same);
    if (i == 0) {
      tc.flat = all_ok ? 1 : 0;
      tc.nu = all_same ? n0 : 0;
    }
  }
  __syncthreads();
}

__device__ __forceinline__ int col_of(const TileCols& tc, int i) {
  if (tc.nu > 0) return i / tc.nu;
  int lo = 0, hi = kTile;  // pre[lo] <= i < pre[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (tc.pre[mid] <= i) lo = mid; else hi = mid;
  }
  return lo;
}

// Each warp moves whole columns (lane k <-> layer k, up to 64 layers in two
// rounds); the CTA's 8 warps cover the tile's 32 columns, all loads of a
// warp issued before its stores.
constexpr int kXposeWarps = kXposeThreads / 32;
constexpr int kColsPerWarp = kTile / kXposeWarps;
constexpr int kRounds = (kMaxLayers + 31) / 32;
static_assert(kTile % kXposeWarps == 0, "warps must split the tile's columns evenly");
constexpr int kXposeFlatBatch = 3;  // flat-run loads per thread and field in flight

__global__ void __launch_bounds__(kXposeThreads)
    ref_to_internal_kernel(Layout L, XFields F, int tile0) {
  extern __shared__ double tileb[];  // [nf][nmax][kXposePad]
  __shared__ TileCols tc;
  const int tile = tile0 + blockIdx.x;
  tile_cols(L, tile, tc);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t tb = (int64_t)L.nmax * kXposePad;  // doubles per field's staging tile
  if (tc.flat) {
    // one contiguous run per field: coalesced loads, kXposeBatch per thread
    // and field in flight
    const int total = tc.pre[kTile];
    const int64_t o0 = tc.off[0];
    for (int base = 0; base < total; base += blockDim.x * kXposeFlatBatch) {
      double v[kXposeMaxFields][kXposeFlatBatch];
#pragma unroll
      for (int r = 0; r < kXposeFlatBatch; ++r) {
        const int i = base + r * blockDim.x + threadIdx.x;
#pragma unroll
        for (int f = 0; f < kXposeMaxFields; ++f)
          if (f < F.nf && i < total) v[f][r] = F.src[f][o0 + i];
      }
#pragma unroll
      for (int r = 0; r < kXposeFlatBatch; ++r) {
        const int i = base + r * blockDim.x + threadIdx.x;
        if (i < total) {
          const int j = col_of(tc, i), k = i - tc.pre[j];
#pragma unroll
          for (int f = 0; f < kXposeMaxFields; ++f)
            if (f < F.nf) tileb[f * tb + k * kXposePad + j] = v[f][r];
        }
      }
    }
  } else {
    double v[kXposeMaxFields][kColsPerWarp][kRounds];
#pragma unroll
    for (int f = 0; f < kXposeMaxFields; ++f)
#pragma unroll
      for (int c = 0; c < kColsPerWarp; ++c) {
        const int j = warp + c * kXposeWarps;
#pragma unroll
        for (int r = 0; r < kRounds; ++r) {
          const int k = lane + 32 * r;
          if (f < F.nf && k < tc.n[j]) v[f][c][r] = F.src[f][tc.off[j] + k];
        }
      }
#pragma unroll
    for (int f = 0; f < kXposeMaxFields; ++f)
#pragma unroll
      for (int c = 0; c < kColsPerWarp; ++c) {
        const int j = warp + c * kXposeWarps;
#pragma unroll
        for (int r = 0; r < kRounds; ++r) {
          const int k = lane + 32 * r;
          if (f < F.nf && k < tc.n[j]) tileb[f * tb + k * kXposePad + j] = v[f][c][r];
        }
      }
  }
  __syncthreads();
  const int nt = L.tile_n[tile];
  const int64_t to = L.tile_off[tile];
  for (int f = 0; f < F.nf; ++f)
    for (int q = threadIdx.x; q < nt * kTile; q += blockDim.x) {
      const int k = q / kTile, jj = q % kTile;
      if (k < tc.n[jj]) F.dst[f][to + q] = tileb[f * tb + k * kXposePad + jj];
    }
}

// Layer-major loads in flight per thread and field before their
// shared-memory stores.
constexpr int kXposeBatch = 3;

__global__ void __launch_bounds__(kXposeThreads)
    internal_to_ref_kernel(Layout L, XFields F, int tile0) {
  extern __shared__ double tileb[];
  __shared__ TileCols tc;
  const int tile = tile0 + blockIdx.x;
  tile_cols(L, tile, tc);
  const int64_t tb = (int64_t)L.nmax * kXposePad;
  const int nq = L.tile_n[tile] * kTile;
  const int64_t so = L.tile_off[tile];
  for (int base = 0; base < nq; base += blockDim.x * kXposeBatch) {
    double v[kXposeMaxFields][kXposeBatch];
    int q[kXposeBatch];
#pragma unroll
    for (int r = 0; r < kXposeBatch; ++r) {
      const int qq = base + r * blockDim.x + threadIdx.x;
      q[r] = (qq < nq && qq / kTile < tc.n[qq % kTile]) ? qq : -1;
#pragma unroll
      for (int f = 0; f < kXposeMaxFields; ++f)
        if (f < F.nf && q[r] >= 0) v[f][r] = F.src[f][so + qq];
    }
#pragma unroll
    for (int r = 0; r < kXposeBatch; ++r)
#pragma unroll
      for (int f = 0; f < kXposeMaxFields; ++f)
        if (f < F.nf && q[r] >= 0) tileb[f * tb + (q[r] / kTile) * kXposePad + q[r] % kTile] = v[f][r];
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int f = 0; f < F.nf; ++f)
#pragma unroll
    for (int c = 0; c < kColsPerWarp; ++c) {
      const int j = warp + c * kXposeWarps;
#pragma unroll
      for (int r = 0; r < kRounds; ++r) {
        const int k = lane + 32 * r;
        if (k < tc.n[j]) F.dst[f][tc.off[j] + k] = tileb[f * tb + k * kXposePad + j];
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

size_t xpose_smem(const Layout& L, int nf) { return (size_t)nf * L.nmax * kXposePad * sizeof(double); }

// tiles [tile0, tile0 + ntl) (ntl < 0: through the last tile) of F.nf fields
cudaError_t ref_to_internal(const Layout& L, const XFields& F, cudaStream_t st, int tile0, int ntl) {
  if (F.nf < 1 || F.nf > kXposeMaxFields) return cudaErrorInvalidValue;
  const size_t sm = xpose_smem(L, F.nf);
  cudaError_t e = cudaFuncSetAttribute(ref_to_internal_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  const int grid = ntl < 0 ? L.ntiles - tile0 : ntl;
  if (grid <= 0) return cudaSuccess;
  ref_to_internal_kernel<<<grid, kXposeThreads, sm, st>>>(L, F, tile0);
  return cudaGetLastError();
}

cudaError_t internal_to_ref(const Layout& L, const XFields& F, cudaStream_t st, int tile0, int ntl) {
  if (F.nf < 1 || F.nf > kXposeMaxFields) return cudaErrorInvalidValue;
  const size_t sm = xpose_smem(L, F.nf);
  cudaError_t e = cudaFuncSetAttribute(internal_to_ref_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  const int grid = ntl < 0 ? L.ntiles - tile0 : ntl;
  if (grid <= 0) return cudaSuccess;
  internal_to_ref_kernel<<<grid, kXposeThreads, sm, st>>>(L, F, tile0);
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
