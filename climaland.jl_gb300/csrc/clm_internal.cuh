// Internal device layout and kernel argument blocks of libclimaland_cuda.
//
// Columns are processed one per thread, 32 columns (one warp) per "tile".
// Cell arrays are stored tile by tile, layer-major inside a tile:
//   cell(tile, k, lane) = tile_off[tile] + k * 32 + lane
// so a warp's load of one layer is one contiguous 256-byte segment. Columns
// are sorted by layer count (descending) before tiling, so a tile holds
// columns of equal or nearly equal depth; tile_n is the deepest in the tile.
// Per-column arrays (parameters, forcing, integrated fluxes, status) are
// stored in the same sorted order with row stride `stride` (a multiple of 32).
#pragma once

#include <cstdint>

#include "clm_atmos.cuh"
#include "clm_physics.cuh"

namespace clm {

constexpr int kTile = 32;
constexpr int kMaxLayers = 64;

struct Layout {
  int ncol;        // real columns
  int stride;      // padded column count (multiple of 32)
  int ntiles;      // stride / 32
  int nmax;        // deepest column
  int64_t ncells_int;  // cells in the internal layout (incl. padding)
  const int64_t* tile_off;  // [ntiles]
  const int* tile_n;        // [ntiles]
  const int* col_n;         // [stride]  0 for padding lanes
  const int* perm;          // [stride]  original column index, -1 padding
  const int64_t* slot_ref;  // [stride]  first cell of the slot's column in the reference layout (0: padding)
};

// Up to three state fields converted by one layout-transpose launch.
constexpr int kXposeMaxFields = 3;
struct XFields {
  const double* src[kXposeMaxFields];
  double* dst[kXposeMaxFields];
  int nf;
};

// Split Newton (tolerance mode, EnergyHydrology): the columns that have not
// converged after the first iterations of a step, saved by the step kernel
// for the resuming kernel (clm_step_kernels.cuh has the entry layout).
struct SplitQueue {
  double* q = nullptr;   // entries (arrays and scalars), null: no split
  int* count = nullptr;  // entries written this step (zeroed before the step kernel)
  int cap = 0;           // capacity in entries, a multiple of 32
  int nmax = 0;          // layers per entry array
};

struct StepArgs {
  Layout L;
  const double* z_lo;   // [stride]
  const double* z_hi;   // [stride]
  // per-layer geometry of stretched columns (clm_set_faces; internal layout),
  // all null for uniform layers
  GeoArrays geo{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  const double* prm;    // [CLM_NPARAM_MAX][stride]
  const double* lkap;   // [2][stride] log kappa_sat_unfrozen, log kappa_sat_frozen
  const double* forc[4];  // [CLM_F_NFIELDS][stride] per slot, or null
  double* v;            // vartheta_l (internal layout)
  double* ti;           // theta_i
  double* e;            // rho_e_int
  double* Fw;           // intF_w  [stride]
  double* Fe;           // intF_e  [stride]
  uint32_t* flags;      // [stride]
  int32_t* iters;       // [stride]
  const float* guess = nullptr;  // learned Newton guess (internal layout, 2 per cell) or null
  // extrapolated Newton guess: vartheta_l then rho_e_int at the previous
  // step's start (internal layout, 2 x ncells_int), or null
  double* prev = nullptr;
  int* tile_ctr = nullptr;       // dynamic tile order: [next tile, warps done], or null (static)
  // iteration-class order (tolerance mode): warp w of the launch takes the
  // slots order[32 w + lane], or null for the tiles' own slots
  const int* order = nullptr;
  Earth E;
  EHScalars sc;
  int bc_tw, bc_th, bc_bw, bc_bh;
  int phase_change;
  int runoff;           // enum clm_runoff (CLM_BC_PRECIP_RUNOFF)
  int cm = CLM_CM_VAN_GENUCHTEN;  // enum clm_hydrology_cm
  const double* rx = nullptr;     // root-extraction canopy rows [CLM_RX_NFIELDS][stride], or null
  const double* atm = nullptr;    // atmosphere drivers [CLM_AT_NFIELDS][stride] (CLM_BC_ATMOS), or null
  AtmosK ak;                      // constants of CLM_BC_ATMOS
  int newton_mode;
  int max_iters;
  double tol;
  double energy_scale;
  uint64_t seed;
  int64_t col0 = 0;     // global index of column 0 (rain-pulse hash)
  int tile_begin = 0;   // the launch's tiles: [tile_begin, tile_end)
  int tile_end = -1;    // -1: through the last tile
  // split Newton: columns unconverged after iteration split_at go to
  // split.q (one-step launches of the tolerance-mode step kernel only)
  SplitQueue split;
  int split_at = 0;
};

// The column's geometry: uniform layers from z_lo, z_hi, or the per-layer
// arrays of a stretched mesh (A.geo, kStr).
template <bool kStr>
struct GeomOf {
  using type = ColGeom;
  static CLM_HD ColGeom make(const StepArgs& A, int64_t, int s, int n) {
    return ColGeom(A.z_lo[s], A.z_hi[s], n);
  }
};
template <>
struct GeomOf<true> {
  using type = ColGeomS;
  static CLM_HD ColGeomS make(const StepArgs& A, int64_t base, int s, int n) {
    return ColGeomS(A.geo, base, 32, s, A.L.stride, A.z_lo[s], A.z_hi[s], n);
  }
};

// Start time and step of a launch: by value, or (CUDA graph replay) read
// from a device array written before each replay: dev[slot] = t0 of this
// launch, dev[kClockSlots] = dt.
constexpr int kClockSlots = 64;
struct StepClock {
  double t0 = 0.0, dt = 0.0;
  const double* dev = nullptr;
  int slot = 0;
  CLM_HD double start() const { return dev ? dev[slot] : t0; }
  CLM_HD double step() const { return dev ? dev[kClockSlots] : dt; }
};

// Dynamic tile order: lane 0 claims the next tile for the warp. The last
// warp of the launch to finish resets the counter pair, so every launch
// (direct or replayed in a graph) starts from tile 0 without a memset.
#ifdef __CUDACC__
__device__ __forceinline__ int claim_tile(int* ctr) {
  int t = 0;
  if ((threadIdx.x & 31) == 0) t = atomicAdd(ctr, 1);
  return __shfl_sync(0xffffffffu, t, 0);
}

__device__ __forceinline__ void release_tiles(int* ctr, int nwarps) {
  if ((threadIdx.x & 31) == 0) {
    __threadfence();
    if (atomicAdd(ctr + 1, 1) == nwarps - 1) {
      atomicExch(ctr, 0);
      atomicExch(ctr + 1, 0);
    }
  }
  __syncwarp();
}
#endif

// clm_api.cu: the configuration checks of clm_create (CLM_OK or CLM_ERR_ARG),
// shared with the allocation-free entry point.
int check_config(const clm_config* cfg);

// Shared-memory view of one warp's column tile: array a, layer k.
template <typename T>
struct Tile {
  T* base;
  int nmax;
  int lane;
  __device__ __forceinline__ T& operator()(int a, int k) const {
    return base[(a * nmax + k) * kTile + lane];
  }
};

}  // namespace clm
