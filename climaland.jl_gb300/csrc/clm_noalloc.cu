// clm_step_eh_noalloc: the EnergyHydrology column step for callers that
// cannot allocate device memory.
//
// Some hosts run this library inside a memory budget they do not control:
// a CUDA.jl or PyTorch caching allocator that owns the device heap, a
// time-stepping loop that cannot afford the device-wide synchronisation a
// cudaMalloc/cudaFree may bring, or an embedding that forbids allocations
// after start-up. The handle API
// (clm_create) allocates its layout, staging and scratch buffers, so such
// callers cannot use it. This entry point takes every input and output as
// caller-owned device memory, in the reference's column layout, and keeps
// the one piece of working memory the kernel needs beyond those - the
// per-warp scratch for the frozen K, kappa and 1/(rho c) arrays - in a
// fixed file-scope device array, so the call allocates nothing.
//
// Limits and sharing:
//  * at most kNoAllocMaxLayers layers, all columns the same depth, FP64;
//  * the scratch array (kNoAllocScratchBytes, 24 MiB) is held by every GPU
//    that loads the library until the process exits;
//  * every call shares that array: calls that overlap on the GPU (other
//    streams, other host threads) race and corrupt each other's results.
//    Each call writes its scratch before reading it, so nothing needs to be
//    cleared between calls;
//  * the first call on each device looks up the array's device address
//    (cudaGetSymbolAddress) and configures the kernel; make that first call
//    before capturing the stream into a CUDA graph. Later calls repeat the
//    lookup and redo the configuration when the address has changed (a new
//    primary context after cudaDeviceReset);
//  * the parameter rows are device memory and are not validated: they must
//    satisfy clm_set_params' constraints (nu > theta_r >= 0, K_sat > 0, ...);
//    a column whose state becomes non-finite is flagged CLM_COL_NONFINITE.

#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "../../include/climaland_cuda.h"
#include "clm_column.cuh"

namespace clm {
namespace {

constexpr int kNoAllocMaxLayers = 32;
constexpr int kNoAllocSlots = 1024;  // warps (32-column tiles) resident at once
constexpr size_t kNoAllocScratchDoubles = (size_t)kNoAllocSlots * 3 * kNoAllocMaxLayers * kTile;
constexpr size_t kNoAllocScratchBytes = kNoAllocScratchDoubles * sizeof(double);
static_assert(kNoAllocScratchBytes == 24u << 20, "the documented scratch size is 24 MiB");

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

constexpr int kMaxDevices = 64;
struct DeviceSetup {
  double* scratch = nullptr;  // device address of g_noalloc_scratch
  int grid = 0;               // resident one-warp CTAs, capped at kNoAllocSlots
};
DeviceSetup g_setup[kMaxDevices];
std::mutex g_setup_mu;

size_t noalloc_smem(int n) {
  return fm::TABLE_SIZE * sizeof(double) + (size_t)7 * sizeof(double) * n * kTile;
}

// One warp per CTA; columns are read in the reference layout (cell =
// c * n + k), which the column code accesses through stride-1 views.
template <class CM>
__global__ void __launch_bounds__(32, 1)
    eh_step_noalloc_kernel(StepArgs A, double* __restrict__ scratch, int ncol, int n, double t0,
                           double dt, int nsteps, uint32_t* __restrict__ flags_out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* tab = reinterpret_cast<double*>(smem_raw);
  const Tables Tb = fm::stage_tables(tab);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t lay = (int64_t)n * kTile;
  double* w = tab + fm::TABLE_SIZE;
  double* sw = scratch + (int64_t)blockIdx.x * 3 * kNoAllocMaxLayers * kTile;
  EHBuffers B;
  B.xv = Col<double>{w + lane, kTile};
  B.xe = Col<double>{w + lay + lane, kTile};
  B.fe = Col<double>{w + 2 * lay + lane, kTile};
  B.K = Col<double>{sw + lane, kTile};
  B.kap = Col<double>{sw + lay + lane, kTile};
  B.irc = Col<double>{sw + 2 * lay + lane, kTile};
  EHJac<double> J;
  J.cp = Col<double>{w + 3 * lay + lane, kTile};
  J.dp = Col<double>{w + 4 * lay + lane, kTile};
  J.d = Col<double>{w + 5 * lay + lane, kTile};
  J.ae = Col<double>{w + 6 * lay + lane, kTile};
  const int ntiles = (ncol + kTile - 1) / kTile;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int c = tile * kTile + lane;
    if (c >= ncol) continue;
    const int64_t o = (int64_t)c * n;
    B.gv = Col<double>{A.v + o, 1};
    B.gti = Col<double>{A.ti + o, 1};
    B.ge = Col<double>{A.e + o, 1};
    double Fw = A.Fw[c], Fe = A.Fe[c];
    uint32_t fl = 0;
    int it = 0;
    const ColGeom G(A.z_lo[c], A.z_hi[c], n);
    eh_column<double, CM, true>(A, Tb, c, n, c, B, J, G, t0, dt, nsteps, Fw, Fe, fl, it);
    A.Fw[c] = Fw;
    A.Fe[c] = Fe;
    if (flags_out) flags_out[c] = fl;
  }
}

// Once per device: the scratch address and the launch configuration.
int setup_device(int dev, DeviceSetup* out) {
  std::lock_guard<std::mutex> lock(g_setup_mu);
  DeviceSetup& s = g_setup[dev];
  // the array's address in the current context: a context created after a
  // cudaDeviceReset places it anew and has lost the kernel attributes, so a
  // changed address repeats the set-up (the lookup allocates nothing)
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess) {
    cudaGetLastError();
    return CLM_ERR_CUDA;
  }
  if (s.scratch != static_cast<double*>(p)) {
    const size_t smem = noalloc_smem(kNoAllocMaxLayers);
    int nsm = 0, per_vg = 0, per_bc = 0;
    if (cudaFuncSetAttribute(eh_step_noalloc_kernel<VG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess ||
        cudaFuncSetAttribute(eh_step_noalloc_kernel<BC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_vg, eh_step_noalloc_kernel<VG>, 32, smem) !=
            cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_bc, eh_step_noalloc_kernel<BC>, 32, smem) !=
            cudaSuccess ||
        per_vg < 1 || per_bc < 1) {
      cudaGetLastError();
      return CLM_ERR_CUDA;
    }
    const int per_sm = per_vg < per_bc ? per_vg : per_bc;  // one grid for either closure
    s.grid = per_sm * nsm < kNoAllocSlots ? per_sm * nsm : kNoAllocSlots;
    s.scratch = static_cast<double*>(p);
  }
  *out = s;
  return CLM_OK;
}

}  // namespace
}  // namespace clm

using namespace clm;

extern "C" int clm_step_eh_noalloc(const clm_config* cfg, int32_t ncol, int32_t nlayers,
                                   const double* z_lo, const double* z_hi, const double* params,
                                   const double* const* forcing, double* vartheta_l,
                                   double* theta_i, double* rho_e_int, double* intF_w,
                                   double* intF_e, uint32_t* flags, double t, double dt,
                                   int32_t nsteps, void* cuda_stream) {
  // the checks of clm_create (enums, Newton settings, which boundary kind
  // each slot admits), then what this entry point does not carry: the mixed
  // path, the learned guess and the boundaries and sources that need
  // handle-owned driver arrays
  if (!cfg || check_config(cfg) != CLM_OK) return CLM_ERR_ARG;
  if (cfg->model != CLM_MODEL_ENERGY_HYDROLOGY || cfg->precision != CLM_PREC_FP64 || cfg->learned_guess)
    return CLM_ERR_ARG;
  if (cfg->bc_top_water == CLM_BC_ATMOS || cfg->bc_top_water == CLM_BC_PRECIP_RUNOFF) return CLM_ERR_ARG;
  if (ncol <= 0 || nlayers < 2 || nlayers > kNoAllocMaxLayers) return CLM_ERR_ARG;
  if (!z_lo || !z_hi || !params || !vartheta_l || !theta_i || !rho_e_int || !intF_w || !intF_e)
    return CLM_ERR_ARG;
  if (!(dt > 0) || !std::isfinite(t) || nsteps < 0) return CLM_ERR_ARG;
  if (nsteps == 0) return CLM_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return CLM_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) return CLM_ERR_UNSUPPORTED;
  DeviceSetup S;
  const int rc = setup_device(dev, &S);
  if (rc != CLM_OK) return rc;
  StepArgs A{};
  A.L.ncol = ncol;
  A.L.stride = ncol;  // parameter and forcing rows of ncol, original order
  A.L.nmax = nlayers;
  A.z_lo = z_lo;
  A.z_hi = z_hi;
  A.prm = params;
  A.lkap = nullptr;
  for (int i = 0; i < 4; ++i) A.forc[i] = forcing ? forcing[i] : nullptr;
  A.v = vartheta_l;
  A.ti = theta_i;
  A.e = rho_e_int;
  A.Fw = intF_w;
  A.Fe = intF_e;
  A.E = make_earth(cfg->earth);
  A.sc.kersten_alpha = cfg->kersten_alpha;
  A.sc.kersten_beta = cfg->kersten_beta;
  A.sc.omega_ln10 = cfg->ice_impedance_omega * kLn10;
  A.sc.visc_gamma = cfg->visc_gamma;
  A.sc.visc_gamma_T_ref = cfg->visc_gamma_T_ref;
  A.bc_tw = cfg->bc_top_water;
  A.bc_th = cfg->bc_top_heat;
  A.bc_bw = cfg->bc_bottom_water;
  A.bc_bh = cfg->bc_bottom_heat;
  A.phase_change = cfg->phase_change;
  A.newton_mode = cfg->newton_mode;
  A.max_iters = cfg->max_iters;
  A.tol = cfg->newton_tol;
  A.energy_scale = cfg->energy_norm_scale;
  A.seed = cfg->forcing_seed;
  A.col0 = cfg->column_offset;
  A.cm = cfg->hydrology_cm;
  const int ntiles = (ncol + kTile - 1) / kTile;
  const int grid = S.grid < ntiles ? S.grid : ntiles;
  const cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
  if (A.cm == CLM_CM_BROOKS_COREY)
    eh_step_noalloc_kernel<BC><<<grid, 32, noalloc_smem(nlayers), st>>>(A, S.scratch, ncol, nlayers, t,
                                                                          dt, nsteps, flags);
  else
    eh_step_noalloc_kernel<VG><<<grid, 32, noalloc_smem(nlayers), st>>>(A, S.scratch, ncol, nlayers, t,
                                                                          dt, nsteps, flags);
  if (cudaGetLastError() != cudaSuccess) return CLM_ERR_CUDA;
  return CLM_OK;
}
