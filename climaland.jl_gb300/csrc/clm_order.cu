// Iteration-class order of the step kernel's columns (tolerance mode).
//
// A warp advances its 32 columns in lockstep, so in tolerance mode it runs
// as many Newton iterations as its slowest column. After each step the
// slots are sorted by (depth, last iteration count), deepest and slowest
// first, into `order`; the next launch's warp w takes slots order[32 w ..
// 32 w + 31], wherever they live in the tiled layout. A column's Newton
// iterations in one step are nearly always those of its previous step, so
// the warps' column sets become homogeneous in iteration count. Which lane
// and warp run a column does not change its arithmetic: the results are the
// same bits in any order.
//
// Counting sort over keys (kMaxLayers - n) * 32 + (31 - min(iters, 31)):
// warp-aggregated histogram (one atomic per distinct key per warp), an
// exclusive scan of the bins in one block, and a warp-aggregated scatter.

#include <cuda_runtime.h>

#include "clm_internal.cuh"

namespace clm {

constexpr int kOrderBins = (kMaxLayers + 1) * 32;

__device__ __forceinline__ int order_key(const Layout& L, const int32_t* iters, int s) {
  const int n = L.col_n[s];
  if (n <= 0) return kOrderBins - 1;  // padding slots last
  const int it = iters[s];
  const int c = it < 0 ? 0 : (it > 31 ? 31 : it);
  return (kMaxLayers - n) * 32 + (31 - c);
}

__global__ void order_hist_kernel(Layout L, const int32_t* __restrict__ iters, int* __restrict__ bins) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= L.stride) return;  // stride is a multiple of 32: whole warps
  const int key = order_key(L, iters, s);
  const unsigned same = __match_any_sync(0xffffffffu, key);
  if ((threadIdx.x & 31) == __ffs(same) - 1) atomicAdd(bins + key, __popc(same));
}

// bins -> exclusive prefix sums (one block of kOrderScanThreads)
constexpr int kOrderScanThreads = 1024;
__global__ void order_scan_kernel(int* __restrict__ bins) {
  __shared__ int part[kOrderScanThreads];
  constexpr int per = (kOrderBins + kOrderScanThreads - 1) / kOrderScanThreads;
  const int t = threadIdx.x;
  int loc[per];
  int sum = 0;
  for (int j = 0; j < per; ++j) {
    const int b = t * per + j;
    loc[j] = b < kOrderBins ? bins[b] : 0;
    sum += loc[j];
  }
  part[t] = sum;
  __syncthreads();
  for (int off = 1; off < kOrderScanThreads; off <<= 1) {  // Hillis-Steele inclusive scan
    const int v = t >= off ? part[t - off] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  int run = part[t] - sum;  // exclusive start of this thread's bins
  for (int j = 0; j < per; ++j) {
    const int b = t * per + j;
    if (b < kOrderBins) bins[b] = run;
    run += loc[j];
  }
}

__global__ void order_scatter_kernel(Layout L, const int32_t* __restrict__ iters, int* __restrict__ bins,
                                     int* __restrict__ order) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= L.stride) return;
  const int key = order_key(L, iters, s);
  const unsigned same = __match_any_sync(0xffffffffu, key);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(same) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(bins + key, __popc(same));
  base = __shfl_sync(same, base, leader);
  order[base + __popc(same & ((1u << lane) - 1u))] = s;
}

size_t order_bins_count() { return kOrderBins; }

// order <- slots sorted by (depth, iteration count); bins: kOrderBins ints
// of scratch, left zero for the next call.
cudaError_t regroup_slots(const Layout& L, const int32_t* iters, int* order, int* bins, cudaStream_t st) {
  const int blocks = (L.stride + 255) / 256;
  cudaError_t e = cudaMemsetAsync(bins, 0, sizeof(int) * kOrderBins, st);
  if (e != cudaSuccess) return e;
  order_hist_kernel<<<blocks, 256, 0, st>>>(L, iters, bins);
  order_scan_kernel<<<1, kOrderScanThreads, 0, st>>>(bins);
  order_scatter_kernel<<<blocks, 256, 0, st>>>(L, iters, bins, order);
  return cudaGetLastError();
}

}  // namespace clm
