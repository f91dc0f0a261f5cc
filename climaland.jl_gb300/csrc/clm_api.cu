// C ABI of libclimaland_cuda (include/climaland_cuda.h).
//
// The handle owns one CUDA stream, the device copies of the column layout,
// parameters, forcing and state, and (lazily) the scratch buffers of the
// closure-level entry points. No call throws, aborts or traps: CUDA errors
// become CLM_ERR_CUDA with a message in clm_last_error().

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/climaland_cuda.h"
#include "clm_internal.cuh"

namespace clm {
// clm_step.cu
cudaError_t launch_step(const StepArgs& A, int model, int precision, int wpc, int grid,
                        double* scratch, const StepClock& clk, int nsteps, cudaStream_t stream);
size_t step_smem_bytes(int model, int precision, int nmax, int wpc);
cudaError_t step_grid(int model, int precision, int cm, bool str, bool tol, int nmax, int wpc, int ntiles,
                      int* grid);
size_t step_scratch_doubles(int model, int precision, int nmax, int wpc, int grid);
cudaError_t resume_setup(int precision, int cm, bool str, int nmax, int wpc);
size_t split_queue_doubles(int cap, int nmax);
cudaError_t launch_resume(const StepArgs& A, int precision, int wpc, int grid, const StepClock& clk,
                          cudaStream_t stream);
// clm_layout.cu
cudaError_t ref_to_internal(const Layout& L, const XFields& F, cudaStream_t st, int tile0 = 0,
                            int ntl = -1);
cudaError_t internal_to_ref(const Layout& L, const XFields& F, cudaStream_t st, int tile0 = 0,
                            int ntl = -1);
cudaError_t cols_to_sorted(const Layout& L, const double* src, double* dst, cudaStream_t st);
cudaError_t cols_to_orig(const Layout& L, const double* src, double* dst, cudaStream_t st);
// clm_order.cu
cudaError_t regroup_slots(const Layout& L, const int32_t* iters, int* order, int* bins, cudaStream_t st);
size_t order_bins_count();
// clm_budget.cu
cudaError_t launch_budgets(const StepArgs& A, int model, double* W, double* E, cudaStream_t st);
// clm_mlp.cu
cudaError_t mlp_features(const StepArgs& A, double t, double dt, float* X, cudaStream_t st);
cudaError_t mlp_guess_setup(int64_t rows, int* grid);
cudaError_t mlp_guess(const StepArgs& A, const float* P, const float* norm, const StepClock& clk,
                      float* guess, double* prev, int grid, cudaStream_t st);
}  // namespace clm

#include "clm_mlp.cuh"

using namespace clm;

struct clm_handle {
  clm_config cfg{};
  int device = 0;
  cudaStream_t stream = nullptr;      // stream in use
  cudaStream_t own_stream = nullptr;  // created by clm_create
  std::string err;
  // layout (host copies)
  int ncol = 0, stride = 0, ntiles = 0, nmax = 0;
  int64_t ncells_ref = 0, ncells_int = 0;
  std::vector<int32_t> ref_off;
  std::vector<int> perm, col_n, tile_n;
  std::vector<int64_t> tile_off;
  // device
  int64_t* d_tile_off = nullptr;
  int* d_tile_n = nullptr;
  int* d_col_n = nullptr;
  int* d_perm = nullptr;
  int32_t* d_ref_off = nullptr;
  int64_t* d_slot_ref = nullptr;
  double *d_zlo = nullptr, *d_zhi = nullptr, *d_prm = nullptr, *d_lkap = nullptr;
  // per-layer geometry of clm_set_faces (null: uniform layers): 5 cell arrays
  // in the internal layout (centre, width, 1 / width, gap, 0.5 / gap) and 3
  // sorted per-column rows (Δz_bottom, thinnest width, sum of widths)
  double* d_geo = nullptr;
  double* d_geocol = nullptr;
  double* d_forc[4] = {nullptr, nullptr, nullptr, nullptr};
  double* d_rx = nullptr;  // root-extraction canopy rows (sorted), or null
  double* d_atm = nullptr; // atmosphere drivers of CLM_BC_ATMOS (sorted), or null
  AtmosK ak{};             // constants of CLM_BC_ATMOS
  double *d_v = nullptr, *d_ti = nullptr, *d_e = nullptr, *d_Fw = nullptr, *d_Fe = nullptr;
  uint32_t* d_flags = nullptr;
  int32_t* d_iters = nullptr;
  double* d_stage = nullptr;  // ncells_ref * 3 staging (reference layout)
  double* d_colstage = nullptr;  // 4 * stride: upload staging, W, E, spare
  float* d_guess = nullptr;  // learned guess, 2 x ncells_int (NaN: none)
  double* d_prev = nullptr;  // the state at the previous guess (vartheta_l, rho_e_int), 2 x ncells_int
  bool prev_valid = false;   // d_prev holds a state of this layout (extrapolated guess)
  float* d_mlp = nullptr;    // network parameters then standardisation
  bool have_geometry = false, have_params = false, have_state = false;
  int wpc = 1;   // warps (32-column tiles) per CTA of the step kernel
  int grid = 0;  // resident CTAs of the step kernel
  int sched = CLM_SCHED_STATIC;  // tile order of the step kernel
  int* d_ctr = nullptr;          // dynamic tile order: [next tile, warps done]
  int* d_order = nullptr;        // iteration-class slot order (tolerance mode)
  int* d_order_bins = nullptr;   // its counting-sort bins
  // split Newton: entries of the columns left unconverged by the step kernel
  // and their count (tolerance mode, CLM_TOL_SPLIT)
  double* d_queue = nullptr;
  int* d_qcount = nullptr;
  size_t queue_doubles = 0;
  double* d_scratch = nullptr;  // per-warp-slot frozen aux arrays
  size_t scratch_doubles = 0;
  int guess_grid = 0;           // persistent grid of the guess kernel
  bool perm_identity = false;   // columns already in depth order
  // clm_step_host pipeline: copy streams and one event pair per chunk
  cudaStream_t copy_in = nullptr, copy_out = nullptr;
  std::vector<cudaEvent_t> host_ev;
  // CUDA graph replay of clm_step_async: one executable graph per piece
  // length, captured on cap_stream, launched on `stream`; t and dt reach the
  // kernels through d_clock, filled from a pinned ring before each replay
  static constexpr int kGraphs = 4, kRing = 4;
  struct Graph {
    cudaGraphExec_t exec = nullptr;
    int nsteps = 0;
    uint64_t used = 0;
  } graphs[kGraphs];
  uint64_t graph_tick = 0;
  cudaStream_t cap_stream = nullptr;
  double* d_clock = nullptr;   // kClockSlots + 1
  double* h_clock = nullptr;   // pinned, kRing x (kClockSlots + 1)
  cudaEvent_t clock_ev[kRing] = {};
  int clock_next = 0;
  Earth E{};
  EHScalars sc{};
};

namespace {

int fail(clm_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

int cuda_fail(clm_handle* h, cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  cudaGetLastError();  // clear the (non-sticky) error state
  return fail(h, CLM_ERR_CUDA, m);
}

#define CLM_CUDA(h, call)                                   \
  do {                                                      \
    cudaError_t _e = (call);                                \
    if (_e != cudaSuccess) return cuda_fail((h), _e, #call); \
  } while (0)

template <typename T>
void dfree(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

bool is_eh(const clm_handle* h) { return h->cfg.model == CLM_MODEL_ENERGY_HYDROLOGY; }

// Tolerance mode groups columns into warps by their last Newton iteration
// count, re-sorted after every step (clm_order.cu).
// Warps regrouped by iteration count: tolerance mode without a Newton guess
// (with one, tile order measured faster: 19.5 against 21.0 ms per
// 1,048,576-column mixed step with the extrapolated start).
// The tolerance schedule in use: CLM_TOL_AUTO resolved by the measured rule
// (1,048,576 x 20 EnergyHydrology columns at tolerance 1e-8: FP64 from U
// 32.2 ms per step regrouped against 33.9 split; mixed from U 18.7 against
// 17.2; mixed from the extrapolated start 19.7 in tiles against 16.9 split).
int tol_schedule(const clm_handle* h) {
  const int t = h->cfg.tol_regroup;
  if (t != CLM_TOL_AUTO) return t;
  if (!is_eh(h) || (h->cfg.precision == CLM_PREC_FP64 && h->cfg.learned_guess == CLM_GUESS_NONE))
    return CLM_TOL_REGROUP;
  return CLM_TOL_SPLIT;
}

bool regroups(const clm_handle* h) {
  return h->cfg.newton_mode == CLM_NEWTON_TOL && tol_schedule(h) == CLM_TOL_REGROUP && h->d_order &&
         h->cfg.learned_guess == CLM_GUESS_NONE;
}

// Split Newton (EnergyHydrology, tolerance mode): each step is two launches,
// the step kernel running every column through its first kSplitIters
// iterations and the resuming kernel finishing the columns that have not
// converged, packed 32 to a warp. Warps in lockstep then run as many
// iterations as the columns need, not as the slowest of 32 neighbours.
constexpr int kSplitIters = 2;

bool splits(const clm_handle* h) {
  return h->cfg.newton_mode == CLM_NEWTON_TOL && tol_schedule(h) == CLM_TOL_SPLIT && is_eh(h) &&
         h->d_queue && h->cfg.max_iters > kSplitIters;
}

// Captured graphs hold kernel arguments by value (buffer pointers, launch
// shape): drop them whenever one of those changes.
void drop_graphs(clm_handle* h) {
  for (auto& g : h->graphs) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = clm_handle::Graph{};
  }
}

Layout layout_of(const clm_handle* h) {
  Layout L;
  L.ncol = h->ncol;
  L.stride = h->stride;
  L.ntiles = h->ntiles;
  L.nmax = h->nmax;
  L.ncells_int = h->ncells_int;
  L.tile_off = h->d_tile_off;
  L.tile_n = h->d_tile_n;
  L.col_n = h->d_col_n;
  L.perm = h->d_perm;
  L.slot_ref = h->d_slot_ref;
  return L;
}

StepArgs step_args(const clm_handle* h) {
  StepArgs A;
  A.L = layout_of(h);
  A.z_lo = h->d_zlo;
  A.z_hi = h->d_zhi;
  if (h->d_geo) {
    const int64_t ni = h->ncells_int;
    A.geo = GeoArrays{h->d_geo, h->d_geo + ni, h->d_geo + 2 * ni, h->d_geo + 3 * ni,
                      h->d_geo + 4 * ni, h->d_geocol};
  }
  A.prm = h->d_prm;
  A.lkap = h->d_lkap;
  for (int i = 0; i < 4; ++i) A.forc[i] = h->d_forc[i];
  A.rx = h->d_rx;
  A.atm = h->cfg.bc_top_water == CLM_BC_ATMOS ? h->d_atm : nullptr;
  A.ak = h->ak;
  A.v = h->d_v;
  A.ti = h->d_ti;
  A.e = h->d_e;
  A.Fw = h->d_Fw;
  A.Fe = h->d_Fe;
  A.flags = h->d_flags;
  A.iters = h->d_iters;
  A.guess = h->cfg.learned_guess == CLM_GUESS_NETWORK ? h->d_guess : nullptr;
  A.prev = h->cfg.learned_guess == CLM_GUESS_EXTRAPOLATE && h->prev_valid ? h->d_prev : nullptr;
  A.tile_ctr = h->sched == CLM_SCHED_DYNAMIC ? h->d_ctr : nullptr;
  A.order = regroups(h) ? h->d_order : nullptr;
  A.E = h->E;
  A.sc = h->sc;
  A.bc_tw = h->cfg.bc_top_water;
  A.bc_th = h->cfg.bc_top_heat;
  A.bc_bw = h->cfg.bc_bottom_water;
  A.bc_bh = h->cfg.bc_bottom_heat;
  A.phase_change = is_eh(h) ? h->cfg.phase_change : 0;
  A.newton_mode = h->cfg.newton_mode;
  A.runoff = h->cfg.runoff;
  A.cm = h->cfg.hydrology_cm;
  A.max_iters = h->cfg.max_iters;
  A.tol = h->cfg.newton_tol;
  A.energy_scale = h->cfg.energy_norm_scale;
  A.seed = h->cfg.forcing_seed;
  A.col0 = h->cfg.column_offset;
  return A;
}

// The persistent grid of the step kernel in use (uniform or per-layer
// geometry) for the current warps per CTA, and its scratch.
int configure_grid(clm_handle* h) {
  CLM_CUDA(h, step_grid(h->cfg.model, h->cfg.precision, h->cfg.hydrology_cm, h->d_geo != nullptr,
                        h->cfg.newton_mode == CLM_NEWTON_TOL, h->nmax, h->wpc, h->ntiles, &h->grid));
  const size_t nsc = step_scratch_doubles(h->cfg.model, h->cfg.precision, h->nmax, h->wpc, h->grid);
  if (nsc != h->scratch_doubles || (nsc && !h->d_scratch)) {
    dfree(h->d_scratch);
    if (nsc) CLM_CUDA(h, cudaMalloc(&h->d_scratch, sizeof(double) * nsc));
    h->scratch_doubles = nsc;
  }
  h->guess_grid = 0;
  // split Newton's queue: room for every column (each defers at most once a
  // step), allocated here so that no step call allocates
  if (h->cfg.newton_mode == CLM_NEWTON_TOL && tol_schedule(h) == CLM_TOL_SPLIT && is_eh(h)) {
    const size_t nq = split_queue_doubles(h->stride, h->nmax);
    if (nq != h->queue_doubles || !h->d_queue) {
      drop_graphs(h);  // captured launches hold the queue's address
      dfree(h->d_queue);
      h->queue_doubles = 0;
      CLM_CUDA(h, cudaMalloc(&h->d_queue, sizeof(double) * nq));
      h->queue_doubles = nq;
    }
    if (!h->d_qcount) CLM_CUDA(h, cudaMalloc(&h->d_qcount, sizeof(int)));
    // the resuming kernel's shared memory for the largest CTA clm_autotune tries
    CLM_CUDA(h, resume_setup(h->cfg.precision, h->cfg.hydrology_cm, h->d_geo != nullptr, h->nmax, 4));
  }
  return CLM_OK;
}

// Build the sorted, tiled layout from per-column layer counts.
int build_layout(clm_handle* h, const std::vector<int>& nl) {
  const int ncol = h->ncol;
  drop_graphs(h);
  // a new layout invalidates the per-layer geometry (clm_set_faces again)
  dfree(h->d_geo);
  dfree(h->d_geocol);
  h->ref_off.assign(ncol + 1, 0);
  for (int c = 0; c < ncol; ++c) {
    if (nl[c] < 2 || nl[c] > kMaxLayers)
      return fail(h, CLM_ERR_ARG, "layer count must be in [2, " + std::to_string(kMaxLayers) +
                                      "], column " + std::to_string(c) + " has " +
                                      std::to_string(nl[c]));
    h->ref_off[c + 1] = h->ref_off[c] + nl[c];
  }
  h->ncells_ref = h->ref_off[ncol];
  h->stride = (ncol + kTile - 1) / kTile * kTile;
  h->ntiles = h->stride / kTile;
  std::vector<int> order(ncol);
  std::iota(order.begin(), order.end(), 0);
  // deepest first: equal-depth columns share tiles, and the deep tiles are
  // scheduled first (longest-processing-time order)
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return nl[a] > nl[b]; });
  h->perm.assign(h->stride, -1);
  h->col_n.assign(h->stride, 0);
  for (int s = 0; s < ncol; ++s) {
    h->perm[s] = order[s];
    h->col_n[s] = nl[order[s]];
  }
  h->tile_n.assign(h->ntiles, 0);
  h->tile_off.assign(h->ntiles, 0);
  int64_t off = 0;
  int nmax = 0;
  for (int t = 0; t < h->ntiles; ++t) {
    int m = 0;
    for (int j = 0; j < kTile; ++j) m = std::max(m, h->col_n[t * kTile + j]);
    h->tile_n[t] = m;
    h->tile_off[t] = off;
    off += (int64_t)m * kTile;
    nmax = std::max(nmax, m);
  }
  h->ncells_int = off;
  h->perm_identity = true;
  for (int s = 0; s < ncol; ++s) h->perm_identity = h->perm_identity && h->perm[s] == s;
  h->nmax = nmax;
  // device copies
  // per-slot reference offsets (what the layout transposes read instead of
  // chasing perm -> ref_off)
  std::vector<int64_t> slot_ref(h->stride, 0);
  for (int s = 0; s < ncol; ++s) slot_ref[s] = h->ref_off[h->perm[s]];
  dfree(h->d_tile_off); dfree(h->d_tile_n); dfree(h->d_col_n); dfree(h->d_perm); dfree(h->d_ref_off);
  dfree(h->d_slot_ref);
  dfree(h->d_order);
  // the guesses and their history are per layout (a new layout needs
  // clm_load_mlp again for the network guess)
  dfree(h->d_guess);
  dfree(h->d_prev);
  h->prev_valid = false;
  cudaStream_t st = h->stream;
  CLM_CUDA(h, cudaMalloc(&h->d_tile_off, sizeof(int64_t) * h->ntiles));
  CLM_CUDA(h, cudaMalloc(&h->d_tile_n, sizeof(int) * h->ntiles));
  CLM_CUDA(h, cudaMalloc(&h->d_col_n, sizeof(int) * h->stride));
  CLM_CUDA(h, cudaMalloc(&h->d_perm, sizeof(int) * h->stride));
  CLM_CUDA(h, cudaMalloc(&h->d_ref_off, sizeof(int32_t) * (ncol + 1)));
  CLM_CUDA(h, cudaMemcpyAsync(h->d_tile_off, h->tile_off.data(), sizeof(int64_t) * h->ntiles, cudaMemcpyHostToDevice, st));
  CLM_CUDA(h, cudaMemcpyAsync(h->d_tile_n, h->tile_n.data(), sizeof(int) * h->ntiles, cudaMemcpyHostToDevice, st));
  CLM_CUDA(h, cudaMemcpyAsync(h->d_col_n, h->col_n.data(), sizeof(int) * h->stride, cudaMemcpyHostToDevice, st));
  CLM_CUDA(h, cudaMemcpyAsync(h->d_perm, h->perm.data(), sizeof(int) * h->stride, cudaMemcpyHostToDevice, st));
  CLM_CUDA(h, cudaMemcpyAsync(h->d_ref_off, h->ref_off.data(), sizeof(int32_t) * (ncol + 1), cudaMemcpyHostToDevice, st));
  CLM_CUDA(h, cudaMalloc(&h->d_slot_ref, sizeof(int64_t) * h->stride));
  CLM_CUDA(h, cudaMemcpyAsync(h->d_slot_ref, slot_ref.data(), sizeof(int64_t) * h->stride, cudaMemcpyHostToDevice, st));
  // iteration-class order: the tiles' own slots until a step has run
  std::vector<int> ident(h->stride);
  std::iota(ident.begin(), ident.end(), 0);
  CLM_CUDA(h, cudaMalloc(&h->d_order, sizeof(int) * h->stride));
  CLM_CUDA(h, cudaMemcpyAsync(h->d_order, ident.data(), sizeof(int) * h->stride, cudaMemcpyHostToDevice, st));
  if (!h->d_order_bins) CLM_CUDA(h, cudaMalloc(&h->d_order_bins, sizeof(int) * order_bins_count()));
  // the host vectors above go out of scope: wait for their copies
  CLM_CUDA(h, cudaStreamSynchronize(st));
  // per-layout buffers
  dfree(h->d_v); dfree(h->d_ti); dfree(h->d_e); dfree(h->d_stage);
  const int64_t ni = std::max<int64_t>(h->ncells_int, 1);
  CLM_CUDA(h, cudaMalloc(&h->d_v, sizeof(double) * ni));
  CLM_CUDA(h, cudaMemsetAsync(h->d_v, 0, sizeof(double) * ni, st));
  if (is_eh(h)) {
    CLM_CUDA(h, cudaMalloc(&h->d_ti, sizeof(double) * ni));
    CLM_CUDA(h, cudaMalloc(&h->d_e, sizeof(double) * ni));
    CLM_CUDA(h, cudaMemsetAsync(h->d_ti, 0, sizeof(double) * ni, st));
    CLM_CUDA(h, cudaMemsetAsync(h->d_e, 0, sizeof(double) * ni, st));
  }
  CLM_CUDA(h, cudaMalloc(&h->d_stage, sizeof(double) * std::max<int64_t>(h->ncells_ref, 1) * 3));
  // choose warps per CTA: as many tiles per CTA as fit in the shared memory
  // budget, up to 4 (cfg->cols_per_cta overrides)
  int dev_smem = 0;
  cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
  int want = h->cfg.cols_per_cta > 0 ? std::max(1, h->cfg.cols_per_cta / kTile) : 1;
  want = std::min(want, 4);
  while (want > 1 && step_smem_bytes(h->cfg.model, h->cfg.precision, h->nmax, want) > (size_t)dev_smem) --want;
  if (step_smem_bytes(h->cfg.model, h->cfg.precision, h->nmax, want) > (size_t)dev_smem)
    return fail(h, CLM_ERR_ARG, "column depth " + std::to_string(h->nmax) +
                                    " needs more shared memory than the device offers");
  h->wpc = want;
  return configure_grid(h);
}

// Start time of step s of a call that starts at t: the one expression both
// the direct launches and the graph clock use, so both give the same bits.
__attribute__((noinline)) double step_time(double t, int s, double dt) { return t + s * dt; }

// One kernel launch of a step sequence: `nsteps` steps from step `step` of
// the call, preceded by the guess kernel when `guess`.
struct Launch {
  int step, nsteps;
  bool guess;
};

// Steps are fused in one launch (a column stays in shared memory between
// steps), 64 per launch so that one launch stays short; with the learned
// guess, the network predicts each step's increment from the state at its
// start: one guess launch, then one step launch, per step; with tolerance
// regrouping, one step launch per step, each followed by the regrouping.
std::vector<Launch> launch_sequence(const clm_handle* h, int nsteps) {
  std::vector<Launch> seq;
  if (h->cfg.learned_guess == CLM_GUESS_NETWORK || regroups(h) || splits(h)) {  // one launch sequence per step
    const bool guess = h->cfg.learned_guess == CLM_GUESS_NETWORK;
    for (int i = 0; i < nsteps; ++i) seq.push_back({i, 1, guess});
  } else {
    const int chunk = 64;
    for (int s0 = 0; s0 < nsteps; s0 += chunk) seq.push_back({s0, std::min(chunk, nsteps - s0), false});
  }
  return seq;
}

int issue(clm_handle* h, const Launch& l, const StepClock& clk, cudaStream_t st) {
  const StepArgs A = step_args(h);
  if (l.guess) {
    const float* P = h->d_mlp;
    CLM_CUDA(h, mlp_guess(A, P, P + kMlpParams, clk, h->d_guess, h->d_prev, h->guess_grid, st));
  }
  if (splits(h) && l.nsteps == 1) {
    StepArgs S = A;
    S.split = SplitQueue{h->d_queue, h->d_qcount, h->stride, h->nmax};
    S.split_at = kSplitIters;
    CLM_CUDA(h, cudaMemsetAsync(h->d_qcount, 0, sizeof(int), st));
    CLM_CUDA(h, launch_step(S, h->cfg.model, h->cfg.precision, h->wpc, h->grid, h->d_scratch, clk, 1, st));
    CLM_CUDA(h, launch_resume(S, h->cfg.precision, h->wpc, h->grid, clk, st));
    return CLM_OK;
  }
  CLM_CUDA(h, launch_step(A, h->cfg.model, h->cfg.precision, h->wpc, h->grid, h->d_scratch, clk,
                          l.nsteps, st));
  if (A.order) CLM_CUDA(h, regroup_slots(A.L, h->d_iters, h->d_order, h->d_order_bins, st));
  return CLM_OK;
}

// Graph replay: the call is cut into pieces of at most kClockSlots launches;
// each piece length has one captured graph whose kernels read their start
// time from d_clock[slot] and dt from d_clock[kClockSlots].
int step_graph(clm_handle* h, double t, double dt, int nsteps) {
  if (!h->d_clock) {
    CLM_CUDA(h, cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking));
    CLM_CUDA(h, cudaMalloc(&h->d_clock, sizeof(double) * (kClockSlots + 1)));
    CLM_CUDA(h, cudaMallocHost(&h->h_clock, sizeof(double) * (kClockSlots + 1) * clm_handle::kRing));
    for (auto& ev : h->clock_ev) CLM_CUDA(h, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  }
  const int per_launch = (h->cfg.learned_guess == CLM_GUESS_NETWORK || regroups(h) || splits(h)) ? 1 : 64;
  const int piece_max = per_launch * kClockSlots;
  for (int s_begin = 0; s_begin < nsteps; s_begin += piece_max) {
    const int P = std::min(piece_max, nsteps - s_begin);
    const std::vector<Launch> seq = launch_sequence(h, P);
    clm_handle::Graph* g = nullptr;
    for (auto& c : h->graphs)
      if (c.exec && c.nsteps == P) g = &c;
    if (!g) {
      // evict the least recently used entry
      g = &h->graphs[0];
      for (auto& c : h->graphs)
        if (c.used < g->used) g = &c;
      if (g->exec) cudaGraphExecDestroy(g->exec);
      *g = clm_handle::Graph{};
      CLM_CUDA(h, cudaStreamBeginCapture(h->cap_stream, cudaStreamCaptureModeThreadLocal));
      int rc = CLM_OK;
      for (size_t j = 0; j < seq.size() && rc == CLM_OK; ++j) {
        StepClock clk;
        clk.dev = h->d_clock;
        clk.slot = (int)j;
        rc = issue(h, seq[j], clk, h->cap_stream);
      }
      cudaGraph_t graph = nullptr;
      const cudaError_t ec = cudaStreamEndCapture(h->cap_stream, &graph);
      if (rc != CLM_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
      }
      if (ec != cudaSuccess) return cuda_fail(h, ec, "cudaStreamEndCapture");
      const cudaError_t ei = cudaGraphInstantiate(&g->exec, graph, 0);
      cudaGraphDestroy(graph);
      if (ei != cudaSuccess) {
        g->exec = nullptr;
        return cuda_fail(h, ei, "cudaGraphInstantiate");
      }
      g->nsteps = P;
    }
    g->used = ++h->graph_tick;
    // the ring slot is free once the copy that last read it has run
    const int r = h->clock_next;
    h->clock_next = (r + 1) % clm_handle::kRing;
    CLM_CUDA(h, cudaEventSynchronize(h->clock_ev[r]));
    double* hc = h->h_clock + (size_t)r * (kClockSlots + 1);
    for (size_t j = 0; j < seq.size(); ++j) hc[j] = step_time(t, s_begin + seq[j].step, dt);
    hc[kClockSlots] = dt;
    CLM_CUDA(h, cudaMemcpyAsync(h->d_clock, hc, sizeof(double) * (kClockSlots + 1),
                                cudaMemcpyHostToDevice, h->stream));
    CLM_CUDA(h, cudaEventRecord(h->clock_ev[r], h->stream));
    CLM_CUDA(h, cudaGraphLaunch(g->exec, h->stream));
  }
  return CLM_OK;
}

int upload_cols_sorted(clm_handle* h, const double* host, double* dst, int rows) {
  // host rows of ncol (original order) -> device rows of stride (sorted)
  cudaStream_t st = h->stream;
  Layout L = layout_of(h);
  for (int r = 0; r < rows; ++r) {
    CLM_CUDA(h, cudaMemcpyAsync(h->d_colstage, host + (size_t)r * h->ncol, sizeof(double) * h->ncol,
                                cudaMemcpyHostToDevice, st));
    CLM_CUDA(h, cols_to_sorted(L, h->d_colstage, dst + (size_t)r * h->stride, st));
  }
  return CLM_OK;
}

int download_cols(clm_handle* h, const double* dsrc, double* host) {
  cudaStream_t st = h->stream;
  Layout L = layout_of(h);
  CLM_CUDA(h, cols_to_orig(L, dsrc, h->d_colstage, st));
  CLM_CUDA(h, cudaMemcpyAsync(host, h->d_colstage, sizeof(double) * h->ncol, cudaMemcpyDeviceToHost, st));
  return CLM_OK;
}

int ready(clm_handle* h) {
  if (!h) return CLM_ERR_ARG;
  if (!h->have_geometry) return fail(h, CLM_ERR_STATE, "clm_set_geometry has not been called");
  if (!h->have_params) return fail(h, CLM_ERR_STATE, "clm_set_params has not been called");
  if (!h->have_state) return fail(h, CLM_ERR_STATE, "clm_set_state has not been called");
  if (h->cfg.bc_top_water == CLM_BC_ATMOS && !h->d_atm)
    return fail(h, CLM_ERR_STATE, "clm_set_atmos has not been called");
  return CLM_OK;
}

// The guesses' history (the state at the previous step's start) restarts
// at the current state: at clm_load_mlp for the network guess, at the first
// step call for the extrapolated one; the first guess after it has no
// previous increment. clm_set_state keeps the history, so a caller that
// round-trips its state every step keeps it; a state unrelated to the
// previous one gives one poor first guess, which the step's restart rule
// replaces by the plain start where it is grossly off.
cudaError_t restart_guess_history(clm_handle* h) {
  if (!h->d_prev || !h->d_v || !h->d_e) return cudaSuccess;
  const size_t nb = sizeof(double) * (size_t)h->ncells_int;
  cudaError_t e = cudaMemcpyAsync(h->d_prev, h->d_v, nb, cudaMemcpyDeviceToDevice, h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h->d_prev + h->ncells_int, h->d_e, nb, cudaMemcpyDeviceToDevice, h->stream);
  return e;
}

int set_state_impl(clm_handle* h, const double* v, const double* ti, const double* e,
                   const double* Fw, const double* Fe, cudaMemcpyKind kind) {
  if (!h) return CLM_ERR_ARG;
  if (!h->have_geometry) return fail(h, CLM_ERR_STATE, "clm_set_geometry has not been called");
  if (!v || !Fw) return fail(h, CLM_ERR_ARG, "vartheta_l and intF_w are required");
  const bool eh = is_eh(h);
  if (eh && (!ti || !e || !Fe)) return fail(h, CLM_ERR_ARG, "EnergyHydrology needs theta_i, rho_e_int, intF_e");
  cudaStream_t st = h->stream;
  Layout L = layout_of(h);
  const size_t nb = sizeof(double) * h->ncells_ref;
  const double* src[3] = {v, ti, e};
  double* dst[3] = {h->d_v, h->d_ti, h->d_e};
  XFields F{};
  F.nf = eh ? 3 : 1;
  for (int i = 0; i < F.nf; ++i) {
    double* stg = h->d_stage + (size_t)i * h->ncells_ref;
    CLM_CUDA(h, cudaMemcpyAsync(stg, src[i], nb, kind, st));
    F.src[i] = stg;
    F.dst[i] = dst[i];
  }
  CLM_CUDA(h, ref_to_internal(L, F, st));
  const double* cs[2] = {Fw, Fe};
  double* cd[2] = {h->d_Fw, h->d_Fe};
  for (int i = 0; i < (eh ? 2 : 1); ++i) {
    CLM_CUDA(h, cudaMemcpyAsync(h->d_colstage, cs[i], sizeof(double) * h->ncol, kind, st));
    CLM_CUDA(h, cols_to_sorted(L, h->d_colstage, cd[i], st));
  }
  CLM_CUDA(h, cudaStreamSynchronize(st));
  h->have_state = true;
  return CLM_OK;
}

int get_state_impl(clm_handle* h, double* v, double* ti, double* e, double* Fw, double* Fe,
                   cudaMemcpyKind kind) {
  if (!h) return CLM_ERR_ARG;
  if (!h->have_state) return fail(h, CLM_ERR_STATE, "no state on the device");
  const bool eh = is_eh(h);
  cudaStream_t st = h->stream;
  Layout L = layout_of(h);
  const size_t nb = sizeof(double) * h->ncells_ref;
  double* outs[3] = {v, ti, e};
  const double* srcs[3] = {h->d_v, h->d_ti, h->d_e};
  XFields F{};
  for (int i = 0; i < (eh ? 3 : 1); ++i) {
    if (!outs[i]) continue;
    F.src[F.nf] = srcs[i];
    F.dst[F.nf++] = h->d_stage + (size_t)i * h->ncells_ref;
  }
  if (F.nf > 0) CLM_CUDA(h, internal_to_ref(L, F, st));
  for (int i = 0; i < (eh ? 3 : 1); ++i)
    if (outs[i])
      CLM_CUDA(h, cudaMemcpyAsync(outs[i], h->d_stage + (size_t)i * h->ncells_ref, nb, kind, st));
  double* co[2] = {Fw, Fe};
  const double* cs[2] = {h->d_Fw, h->d_Fe};
  for (int i = 0; i < (eh ? 2 : 1); ++i) {
    if (!co[i]) continue;
    CLM_CUDA(h, cols_to_orig(L, cs[i], h->d_colstage, st));
    CLM_CUDA(h, cudaMemcpyAsync(co[i], h->d_colstage, sizeof(double) * h->ncol, kind, st));
    CLM_CUDA(h, cudaStreamSynchronize(st));  // d_colstage is reused
  }
  CLM_CUDA(h, cudaStreamSynchronize(st));
  return CLM_OK;
}

}  // namespace

namespace clm {

// The configuration checks shared by clm_create and clm_step_eh_noalloc
// (sizes are checked by each): enums in range, the Newton settings, and the
// boundary kinds each slot and model admit.
int check_config(const clm_config* cfg) {
  if (!cfg) return CLM_ERR_ARG;
  if (cfg->model != CLM_MODEL_RICHARDS && cfg->model != CLM_MODEL_ENERGY_HYDROLOGY) return CLM_ERR_ARG;
  if (cfg->max_iters < 1 || cfg->max_iters > 1000) return CLM_ERR_ARG;
  if (cfg->precision != CLM_PREC_FP64 && cfg->precision != CLM_PREC_MIXED) return CLM_ERR_ARG;
  if (cfg->learned_guess != CLM_GUESS_NONE && cfg->learned_guess != CLM_GUESS_NETWORK &&
      cfg->learned_guess != CLM_GUESS_EXTRAPOLATE)
    return CLM_ERR_ARG;
  if (cfg->learned_guess && (cfg->model != CLM_MODEL_ENERGY_HYDROLOGY || cfg->newton_mode != CLM_NEWTON_TOL))
    return CLM_ERR_ARG;  // the guess only changes where tolerance-mode Newton starts
  if (cfg->newton_mode != CLM_NEWTON_FIXED && cfg->newton_mode != CLM_NEWTON_TOL) return CLM_ERR_ARG;
  if (cfg->schedule != CLM_SCHED_STATIC && cfg->schedule != CLM_SCHED_DYNAMIC) return CLM_ERR_ARG;
  if (cfg->graph != 0 && cfg->graph != 1) return CLM_ERR_ARG;
  if (cfg->tol_regroup < CLM_TOL_TILES || cfg->tol_regroup > CLM_TOL_AUTO) return CLM_ERR_ARG;
  if (cfg->cols_per_cta < 0) return CLM_ERR_ARG;
  if (cfg->hydrology_cm != CLM_CM_VAN_GENUCHTEN && cfg->hydrology_cm != CLM_CM_BROOKS_COREY)
    return CLM_ERR_ARG;
  const int kinds[4] = {cfg->bc_top_water, cfg->bc_top_heat, cfg->bc_bottom_water, cfg->bc_bottom_heat};
  for (int i = 0; i < 4; ++i) {
    const int k = kinds[i];
    const bool runoff_top = (i == 0 && k == CLM_BC_PRECIP_RUNOFF);
    const bool atmos_top = (i < 2 && k == CLM_BC_ATMOS);
    if (!runoff_top && !atmos_top && (k < CLM_BC_FLUX || k > CLM_BC_FLUX_ADVECTIVE)) return CLM_ERR_ARG;
  }
  if (cfg->bc_top_water == CLM_BC_PRECIP_RUNOFF &&
      (cfg->model != CLM_MODEL_RICHARDS || cfg->runoff < CLM_RUNOFF_NONE || cfg->runoff > CLM_RUNOFF_TOPMODEL))
    return CLM_ERR_ARG;
  // AtmosDrivenFluxBC sets both top fluxes of EnergyHydrology
  if ((cfg->bc_top_water == CLM_BC_ATMOS) != (cfg->bc_top_heat == CLM_BC_ATMOS)) return CLM_ERR_ARG;
  if (cfg->bc_top_water == CLM_BC_ATMOS &&
      (cfg->model != CLM_MODEL_ENERGY_HYDROLOGY || cfg->runoff < CLM_RUNOFF_NONE ||
       cfg->runoff > CLM_RUNOFF_TOPMODEL))
    return CLM_ERR_ARG;
  if (cfg->bc_top_water == CLM_BC_FREE_DRAINAGE || cfg->bc_top_water == CLM_BC_FLUX_ADVECTIVE ||
      cfg->bc_bottom_water == CLM_BC_FLUX_ADVECTIVE || cfg->bc_top_heat == CLM_BC_FREE_DRAINAGE ||
      cfg->bc_bottom_heat == CLM_BC_FLUX_ADVECTIVE)
    return CLM_ERR_ARG;
  return CLM_OK;
}

}  // namespace clm

extern "C" {

const char* clm_version(void) { return "libclimaland_cuda 0.1 (sm_103a)"; }

double clm_forcing_hash01(uint64_t seed, uint64_t column, int64_t period) {
  return hash01(seed, column, period);
}

void clm_config_default(clm_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->model = CLM_MODEL_ENERGY_HYDROLOGY;
  c->precision = CLM_PREC_FP64;
  c->newton_mode = CLM_NEWTON_FIXED;
  c->max_iters = 3;
  c->newton_tol = 1e-8;
  c->energy_norm_scale = 1.0;
  c->bc_top_water = CLM_BC_FLUX;
  c->bc_top_heat = CLM_BC_FLUX;
  c->bc_bottom_water = CLM_BC_FREE_DRAINAGE;
  c->bc_bottom_heat = CLM_BC_FREE_DRAINAGE;
  c->kersten_alpha = 0.24;
  c->kersten_beta = 18.3;
  c->ice_impedance_omega = 7.0;
  c->visc_gamma = 2.64e-2;
  c->visc_gamma_T_ref = 288.0;
  c->earth.rho_l = 1000.0;
  c->earth.rho_i = 916.7;
  c->earth.cp_l = 4181.0;
  c->earth.cp_i = 2100.0;
  c->earth.T_0 = 273.16;
  c->earth.T_freeze = 273.15;
  c->earth.LH_f0 = 2834400.0 - 2500800.0;
  c->earth.grav = 9.81;
  c->phase_change = 1;
  c->tol_regroup = CLM_TOL_AUTO;
}

int clm_create(const clm_config* cfg, clm_handle** out) {
  if (!cfg || !out) return CLM_ERR_ARG;
  *out = nullptr;
  if (check_config(cfg) != CLM_OK) return CLM_ERR_ARG;
  if (cfg->ncol <= 0 || cfg->nlayers < 0 || cfg->nlayers > kMaxLayers) return CLM_ERR_ARG;
  clm_handle* h = new (std::nothrow) clm_handle();
  if (!h) return CLM_ERR_ARG;
  h->cfg = *cfg;
  h->ncol = cfg->ncol;
  h->E = make_earth(cfg->earth);
  h->sc.kersten_alpha = cfg->kersten_alpha;
  h->sc.kersten_beta = cfg->kersten_beta;
  h->sc.omega_ln10 = cfg->ice_impedance_omega * kLn10;
  h->sc.visc_gamma = cfg->visc_gamma;
  h->sc.visc_gamma_T_ref = cfg->visc_gamma_T_ref;
  h->sched = cfg->schedule;
  cudaError_t e = cudaGetDevice(&h->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
  h->stream = h->own_stream;
  if (e != cudaSuccess) {
    cudaGetLastError();
    delete h;
    return CLM_ERR_CUDA;
  }
  const int stride = (h->ncol + kTile - 1) / kTile * kTile;
  const size_t cb = sizeof(double) * stride;
  bool ok = cudaMalloc(&h->d_zlo, cb) == cudaSuccess && cudaMalloc(&h->d_zhi, cb) == cudaSuccess &&
            cudaMalloc(&h->d_prm, cb * CLM_NPARAM_MAX) == cudaSuccess &&
            cudaMalloc(&h->d_lkap, cb * 2) == cudaSuccess && cudaMalloc(&h->d_Fw, cb) == cudaSuccess &&
            cudaMalloc(&h->d_Fe, cb) == cudaSuccess &&
            cudaMalloc(&h->d_flags, sizeof(uint32_t) * stride) == cudaSuccess &&
            cudaMalloc(&h->d_iters, sizeof(int32_t) * stride) == cudaSuccess &&
            cudaMalloc(&h->d_colstage, cb * 4) == cudaSuccess &&
            cudaMalloc(&h->d_ctr, sizeof(int) * 2) == cudaSuccess;
  if (ok) {
    ok = cudaMemsetAsync(h->d_prm, 0, cb * CLM_NPARAM_MAX, h->stream) == cudaSuccess &&
         cudaMemsetAsync(h->d_lkap, 0, cb * 2, h->stream) == cudaSuccess &&
         cudaMemsetAsync(h->d_Fw, 0, cb, h->stream) == cudaSuccess &&
         cudaMemsetAsync(h->d_Fe, 0, cb, h->stream) == cudaSuccess &&
         cudaMemsetAsync(h->d_flags, 0, sizeof(uint32_t) * stride, h->stream) == cudaSuccess &&
         cudaMemsetAsync(h->d_iters, 0, sizeof(int32_t) * stride, h->stream) == cudaSuccess &&
         cudaMemsetAsync(h->d_ctr, 0, sizeof(int) * 2, h->stream) == cudaSuccess;
  }
  if (!ok) {
    cudaGetLastError();
    clm_destroy(h);
    return CLM_ERR_CUDA;
  }
  if (cfg->nlayers > 0) {
    std::vector<int> nl(h->ncol, cfg->nlayers);
    int rc = build_layout(h, nl);
    if (rc != CLM_OK) {
      clm_destroy(h);
      return rc;
    }
  }
  *out = h;
  return CLM_OK;
}

void clm_destroy(clm_handle* h) {
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->own_stream && h->own_stream != h->stream) cudaStreamSynchronize(h->own_stream);
  dfree(h->d_tile_off); dfree(h->d_tile_n); dfree(h->d_col_n); dfree(h->d_perm); dfree(h->d_ref_off);
  dfree(h->d_slot_ref);
  dfree(h->d_zlo); dfree(h->d_zhi); dfree(h->d_prm); dfree(h->d_lkap);
  dfree(h->d_geo); dfree(h->d_geocol);
  for (auto& p : h->d_forc) dfree(p);
  dfree(h->d_rx);
  dfree(h->d_atm);
  dfree(h->d_v); dfree(h->d_ti); dfree(h->d_e); dfree(h->d_Fw); dfree(h->d_Fe);
  dfree(h->d_flags); dfree(h->d_iters); dfree(h->d_stage); dfree(h->d_colstage); dfree(h->d_guess);
  dfree(h->d_prev);
  dfree(h->d_scratch);
  dfree(h->d_mlp);
  dfree(h->d_ctr);
  dfree(h->d_order);
  dfree(h->d_order_bins);
  dfree(h->d_queue);
  dfree(h->d_qcount);
  drop_graphs(h);
  dfree(h->d_clock);
  if (h->h_clock) cudaFreeHost(h->h_clock);
  for (auto& ev : h->clock_ev)
    if (ev) cudaEventDestroy(ev);
  if (h->cap_stream) cudaStreamDestroy(h->cap_stream);
  for (auto& ev : h->host_ev) cudaEventDestroy(ev);
  if (h->copy_in) cudaStreamDestroy(h->copy_in);
  if (h->copy_out) cudaStreamDestroy(h->copy_out);
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
  cudaGetLastError();
  delete h;
}

const char* clm_last_error(const clm_handle* h) {
  if (!h) return "null handle";
  return h->err.c_str();
}

int clm_set_geometry(clm_handle* h, const double* z_lo, const double* z_hi, const int32_t* offsets) {
  if (!h || !z_lo || !z_hi) return h ? fail(h, CLM_ERR_ARG, "z_lo and z_hi are required") : CLM_ERR_ARG;
  for (int c = 0; c < h->ncol; ++c)
    if (!(z_hi[c] > z_lo[c]) || !std::isfinite(z_lo[c]) || !std::isfinite(z_hi[c]))
      return fail(h, CLM_ERR_ARG, "column " + std::to_string(c) + " needs z_lo < z_hi");
  if (h->cfg.nlayers == 0) {
    if (!offsets) return fail(h, CLM_ERR_ARG, "offsets are required when cfg.nlayers == 0");
    if (offsets[0] != 0) return fail(h, CLM_ERR_ARG, "offsets[0] must be 0");
    std::vector<int> nl(h->ncol);
    for (int c = 0; c < h->ncol; ++c) {
      nl[c] = offsets[c + 1] - offsets[c];
    }
    int rc = build_layout(h, nl);
    if (rc != CLM_OK) return rc;
  } else if (offsets) {
    for (int c = 0; c <= h->ncol; ++c)
      if (offsets[c] != c * h->cfg.nlayers)
        return fail(h, CLM_ERR_ARG, "offsets disagree with cfg.nlayers");
  }
  int rc = upload_cols_sorted(h, z_lo, h->d_zlo, 1);
  if (rc == CLM_OK) rc = upload_cols_sorted(h, z_hi, h->d_zhi, 1);
  if (rc != CLM_OK) return rc;
  CLM_CUDA(h, cudaStreamSynchronize(h->stream));
  h->have_geometry = true;
  if (h->d_geo) {  // uniform layers from here on: faces set earlier no longer apply
    drop_graphs(h);
    dfree(h->d_geo);
    dfree(h->d_geocol);
    return configure_grid(h);
  }
  return CLM_OK;
}

int clm_set_faces(clm_handle* h, const double* zf) {
  if (!h) return CLM_ERR_ARG;
  if (!h->have_geometry) return fail(h, CLM_ERR_STATE, "clm_set_geometry has not been called");
  drop_graphs(h);
  if (!zf) {  // back to uniform layers between the current z_lo and z_hi
    dfree(h->d_geo);
    dfree(h->d_geocol);
    return configure_grid(h);
  }
  const int ncol = h->ncol;
  const int64_t nc = h->ncells_ref;
  // the column geometry ClimaCore derives from the faces (midpoint centres,
  // widths, centre spacings, the boundary half-spacings), computed here once
  std::vector<double> g(5 * (size_t)nc, 0.0), rows(3 * (size_t)ncol), zlo(ncol), zhi(ncol);
  for (int c = 0; c < ncol; ++c) {
    const int64_t o = h->ref_off[c];
    const int n = h->ref_off[c + 1] - h->ref_off[c];
    const double* f = zf + o + c;
    for (int k = 0; k <= n; ++k)
      if (!std::isfinite(f[k]) || (k > 0 && !(f[k] > f[k - 1])))
        return fail(h, CLM_ERR_ARG, "column " + std::to_string(c) + " needs finite, increasing faces");
    const GeoColumn gc = column_geometry(f, n, 1, &g[0 * nc + o], &g[1 * nc + o], &g[2 * nc + o],
                                         &g[3 * nc + o], &g[4 * nc + o]);
    rows[c] = gc.bot;
    rows[ncol + c] = gc.wmin;
    rows[2 * (size_t)ncol + c] = gc.wsum;
    zlo[c] = f[0];
    zhi[c] = f[n];
  }
  cudaStream_t st = h->stream;
  Layout L = layout_of(h);
  const int64_t ni = std::max<int64_t>(h->ncells_int, 1);
  if (!h->d_geo) CLM_CUDA(h, cudaMalloc(&h->d_geo, sizeof(double) * 5 * ni));
  if (!h->d_geocol) CLM_CUDA(h, cudaMalloc(&h->d_geocol, sizeof(double) * 3 * h->stride));
  CLM_CUDA(h, cudaMemsetAsync(h->d_geo, 0, sizeof(double) * 5 * ni, st));
  CLM_CUDA(h, cudaMemsetAsync(h->d_geocol, 0, sizeof(double) * 3 * h->stride, st));
  for (int f0 = 0; f0 < 5; f0 += 3) {
    XFields F{};
    F.nf = std::min(3, 5 - f0);
    for (int i = 0; i < F.nf; ++i) {
      double* stg = h->d_stage + (size_t)i * nc;
      CLM_CUDA(h, cudaMemcpyAsync(stg, g.data() + (size_t)(f0 + i) * nc, sizeof(double) * nc,
                                  cudaMemcpyHostToDevice, st));
      F.src[i] = stg;
      F.dst[i] = h->d_geo + (f0 + i) * ni;
    }
    CLM_CUDA(h, ref_to_internal(L, F, st));
    CLM_CUDA(h, cudaStreamSynchronize(st));  // the staging is reused
  }
  int rc = upload_cols_sorted(h, rows.data(), h->d_geocol, 3);
  if (rc == CLM_OK) rc = upload_cols_sorted(h, zlo.data(), h->d_zlo, 1);
  if (rc == CLM_OK) rc = upload_cols_sorted(h, zhi.data(), h->d_zhi, 1);
  if (rc != CLM_OK) return rc;
  CLM_CUDA(h, cudaStreamSynchronize(st));
  return configure_grid(h);
}

int clm_set_params(clm_handle* h, const double* p, int32_t nparams) {
  if (!h) return CLM_ERR_ARG;
  if (!h->have_geometry) return fail(h, CLM_ERR_STATE, "clm_set_geometry has not been called");
  const bool topmodel = (h->cfg.bc_top_water == CLM_BC_PRECIP_RUNOFF || h->cfg.bc_top_water == CLM_BC_ATMOS) &&
                        h->cfg.runoff == CLM_RUNOFF_TOPMODEL;
  const int need = topmodel ? CLM_NPARAM_MAX : (is_eh(h) ? CLM_NPARAM_EH : CLM_NPARAM_RICHARDS);
  if (!p || nparams < need || nparams > CLM_NPARAM_MAX)
    return fail(h, CLM_ERR_ARG, "expected " + std::to_string(need) + " parameter rows");
  const int ncol = h->ncol;
  for (int c = 0; c < ncol; ++c) {
    const double nu = p[CLM_P_NU * ncol + c], Ks = p[CLM_P_K_SAT * ncol + c];
    const double Ss = p[CLM_P_S_S * ncol + c], tr = p[CLM_P_THETA_R * ncol + c];
    const double a = p[CLM_P_VG_ALPHA * ncol + c], n = p[CLM_P_VG_N * ncol + c];
    // van Genuchten alpha > 0, n > 1; Brooks-Corey psi_b < 0, c > 0
    const bool closure_ok = h->cfg.hydrology_cm == CLM_CM_BROOKS_COREY ? (a < 0 && n > 0) : (a > 0 && n > 1);
    if (!(nu > 0 && nu <= 1) || !(Ks >= 0) || !(Ss > 0) || !(tr >= 0 && tr < nu) || !closure_ok)
      return fail(h, CLM_ERR_ARG, "invalid hydraulic parameters in column " + std::to_string(c));
    if (topmodel) {
      const double fm = p[CLM_P_F_MAX * ncol + c], fo = p[CLM_P_F_OVER * ncol + c], rs = p[CLM_P_R_SB * ncol + c];
      if (!(fm >= 0 && fm <= 1) || !(fo >= 0) || !(rs >= 0))
        return fail(h, CLM_ERR_ARG, "invalid TOPMODEL parameters in column " + std::to_string(c));
    }
    if (is_eh(h)) {
      const double kd = p[CLM_P_KAPPA_DRY * ncol + c], kf = p[CLM_P_KAPPA_SAT_FROZEN * ncol + c];
      const double ku = p[CLM_P_KAPPA_SAT_UNFROZEN * ncol + c], rc = p[CLM_P_RHOC_DS * ncol + c];
      if (!(kd >= 0) || !(kf > 0) || !(ku > 0) || !(rc > 0))
        return fail(h, CLM_ERR_ARG, "invalid thermal parameters in column " + std::to_string(c));
    }
  }
  int rc = upload_cols_sorted(h, p, h->d_prm, nparams);
  if (rc != CLM_OK) return rc;
  if (is_eh(h)) {
    std::vector<double> lk((size_t)2 * ncol);
    for (int c = 0; c < ncol; ++c) {
      lk[c] = std::log(p[CLM_P_KAPPA_SAT_UNFROZEN * ncol + c]);
      lk[ncol + c] = std::log(p[CLM_P_KAPPA_SAT_FROZEN * ncol + c]);
    }
    rc = upload_cols_sorted(h, lk.data(), h->d_lkap, 2);
    if (rc != CLM_OK) return rc;
    CLM_CUDA(h, cudaStreamSynchronize(h->stream));
  }
  CLM_CUDA(h, cudaStreamSynchronize(h->stream));
  h->have_params = true;
  return CLM_OK;
}

int clm_set_bc(clm_handle* h, int32_t slot, const double* f, int32_t nfields) {
  if (!h) return CLM_ERR_ARG;
  if (!h->have_geometry) return fail(h, CLM_ERR_STATE, "clm_set_geometry has not been called");
  if (slot < 0 || slot > 3) return fail(h, CLM_ERR_ARG, "slot must be a clm_bc_slot");
  if (!f) {
    if (h->d_forc[slot]) drop_graphs(h);
    dfree(h->d_forc[slot]);
    return CLM_OK;
  }
  if (nfields < 1 || nfields > CLM_F_NFIELDS) return fail(h, CLM_ERR_ARG, "nfields out of range");
  for (int64_t i = 0; i < (int64_t)nfields * h->ncol; ++i)
    if (!std::isfinite(f[i])) return fail(h, CLM_ERR_ARG, "non-finite forcing value");
  if (!h->d_forc[slot]) {
    drop_graphs(h);
    CLM_CUDA(h, cudaMalloc(&h->d_forc[slot], sizeof(double) * h->stride * CLM_F_NFIELDS));
  }
  CLM_CUDA(h, cudaMemsetAsync(h->d_forc[slot], 0, sizeof(double) * h->stride * CLM_F_NFIELDS, h->stream));
  int rc = upload_cols_sorted(h, f, h->d_forc[slot], nfields);
  if (rc != CLM_OK) return rc;
  CLM_CUDA(h, cudaStreamSynchronize(h->stream));
  return CLM_OK;
}

int clm_set_root_extraction(clm_handle* h, const double* r, int32_t nfields) {
  if (!h) return CLM_ERR_ARG;
  if (!h->have_geometry) return fail(h, CLM_ERR_STATE, "clm_set_geometry has not been called");
  if (!r) {
    if (h->d_rx) drop_graphs(h);
    dfree(h->d_rx);
    return CLM_OK;
  }
  if (!is_eh(h))
    return fail(h, CLM_ERR_ARG, "root extraction is an EnergyHydrology source");
  if (h->cfg.bc_top_water == CLM_BC_ATMOS)
    return fail(h, CLM_ERR_UNSUPPORTED,
                "root extraction with the standalone-soil atmosphere-driven boundary");
  if (nfields != CLM_RX_NFIELDS) return fail(h, CLM_ERR_ARG, "expected CLM_RX_NFIELDS rows");
  const int ncol = h->ncol;
  for (int64_t i = 0; i < (int64_t)nfields * ncol; ++i)
    if (!std::isfinite(r[i])) return fail(h, CLM_ERR_ARG, "non-finite root-extraction value");
  for (int c = 0; c < ncol; ++c) {
    const double lai = r[CLM_RX_LAI * ncol + c], rai = r[CLM_RX_RAI * ncol + c];
    const double ht = r[CLM_RX_HEIGHT * ncol + c], d = r[CLM_RX_ROOT_DEPTH * ncol + c];
    const double ks = r[CLM_RX_K_SAT * ncol + c], p63 = r[CLM_RX_PSI63 * ncol + c];
    const double wc = r[CLM_RX_WEIBULL_C * ncol + c];
    if (!(lai >= 0) || !(rai >= 0) || !(ht > 0) || !(d > 0) || !(ks >= 0) || !(p63 < 0) || !(wc > 0))
      return fail(h, CLM_ERR_ARG, "invalid root-extraction values in column " + std::to_string(c));
  }
  if (!h->d_rx) {
    drop_graphs(h);
    CLM_CUDA(h, cudaMalloc(&h->d_rx, sizeof(double) * h->stride * CLM_RX_NFIELDS));
    CLM_CUDA(h, cudaMemsetAsync(h->d_rx, 0, sizeof(double) * h->stride * CLM_RX_NFIELDS, h->stream));
  }
  int rc = upload_cols_sorted(h, r, h->d_rx, nfields);
  if (rc != CLM_OK) return rc;
  CLM_CUDA(h, cudaStreamSynchronize(h->stream));
  return CLM_OK;
}

void clm_atmos_params_default(clm_atmos_params* a) {
  if (!a) return;
  std::memset(a, 0, sizeof *a);
  a->stefan = 5.670374419e-8;
  a->gas_constant = 8.3144598;
  a->molmass_dryair = 0.02897;
  a->molmass_water = 0.01801528;
  a->D_vapor = 2.5e-5;
  a->LH_v0 = 2500800.0;
  a->LH_s0 = 2834400.0;
  a->cp_d = 1004.5;
  a->cp_v = 1859.0;
  a->T_triple = 273.16;
  a->press_triple = 611.657;
  a->von_karman = 0.4;
  // ClimaParams' Gryanik coefficients (Gryanik et al. 2020), the
  // reference's universal functions; Businger-Dyer's b_m, b_h on the
  // unstable side
  a->universal_functions = CLM_UF_GRYANIK;
  a->Pr_0 = 0.98;
  a->a_m = 5.0;
  a->a_h = 5.0;
  a->gryanik_b_m = 0.3;
  a->gryanik_b_h = 0.4;
  a->b_m = 15.0;
  a->b_h = 9.0;
  a->zeta_max = 100.0;
  a->iterations = 8;
}

int clm_set_atmos(clm_handle* h, const clm_atmos_params* prm, const double* d, int32_t nfields) {
  if (!h) return CLM_ERR_ARG;
  if (!h->have_geometry) return fail(h, CLM_ERR_STATE, "clm_set_geometry has not been called");
  if (!d) {
    if (h->d_atm) drop_graphs(h);
    dfree(h->d_atm);
    return CLM_OK;
  }
  if (h->cfg.bc_top_water != CLM_BC_ATMOS)
    return fail(h, CLM_ERR_ARG, "the top boundary is not CLM_BC_ATMOS");
  if (nfields != CLM_AT_NFIELDS) return fail(h, CLM_ERR_ARG, "expected CLM_AT_NFIELDS rows");
  clm_atmos_params a;
  if (prm) a = *prm; else clm_atmos_params_default(&a);
  const double pos[] = {a.stefan, a.gas_constant, a.molmass_dryair, a.molmass_water, a.D_vapor,
                        a.cp_d, a.cp_v, a.T_triple, a.press_triple, a.von_karman, a.Pr_0,
                        a.zeta_max};
  for (double x : pos)
    if (!(x > 0) || !std::isfinite(x)) return fail(h, CLM_ERR_ARG, "invalid clm_atmos_params constant");
  const double fin[] = {a.LH_v0, a.LH_s0, a.a_m, a.a_h, a.b_m, a.b_h};
  for (double x : fin)
    if (!std::isfinite(x) || x < 0) return fail(h, CLM_ERR_ARG, "invalid clm_atmos_params constant");
  if (a.universal_functions != CLM_UF_BUSINGER && a.universal_functions != CLM_UF_GRYANIK)
    return fail(h, CLM_ERR_ARG, "universal_functions must be CLM_UF_BUSINGER or CLM_UF_GRYANIK");
  if (a.universal_functions == CLM_UF_GRYANIK && (!(a.gryanik_b_m > 0) || !(a.gryanik_b_h > 0) ||
                                                  !std::isfinite(a.gryanik_b_m) || !std::isfinite(a.gryanik_b_h)))
    return fail(h, CLM_ERR_ARG, "invalid Gryanik coefficients");
  if (a.iterations < 1 || a.iterations > 1000) return fail(h, CLM_ERR_ARG, "iterations must be in [1, 1000]");
  const int ncol = h->ncol;
  for (int64_t i = 0; i < (int64_t)nfields * ncol; ++i)
    if (!std::isfinite(d[i])) return fail(h, CLM_ERR_ARG, "non-finite atmosphere driver");
  for (int c = 0; c < ncol; ++c) {
    auto at = [&](int f) { return d[(int64_t)f * ncol + c]; };
    bool ok = at(CLM_AT_T_AIR) > 0 && at(CLM_AT_P_AIR) > 0 && at(CLM_AT_Q_AIR) >= 0 &&
              at(CLM_AT_Q_AIR) < 1 && at(CLM_AT_GUSTINESS) >= 0 &&
              (std::fabs(at(CLM_AT_U_AIR)) > 0 || at(CLM_AT_GUSTINESS) > 0) && at(CLM_AT_Z_0M) > 0 &&
              at(CLM_AT_Z_0B) > 0 && at(CLM_AT_H_AIR) > at(CLM_AT_Z_0M) && at(CLM_AT_H_AIR) > at(CLM_AT_Z_0B) &&
              at(CLM_AT_ALBEDO_TOP_THICKNESS) > 0 && at(CLM_AT_D_DS) >= 0 && at(CLM_AT_EVAP_ALPHA) >= 0 &&
              at(CLM_AT_EMISSIVITY) >= 0 && at(CLM_AT_EMISSIVITY) <= 1;
    for (int f = CLM_AT_PAR_ALBEDO_DRY; f <= CLM_AT_NIR_ALBEDO_WET; ++f) ok = ok && at(f) >= 0 && at(f) <= 1;
    if (!ok) return fail(h, CLM_ERR_ARG, "invalid atmosphere drivers in column " + std::to_string(c));
  }
  if (!h->d_atm) {
    drop_graphs(h);
    CLM_CUDA(h, cudaMalloc(&h->d_atm, sizeof(double) * h->stride * CLM_AT_NFIELDS));
    CLM_CUDA(h, cudaMemsetAsync(h->d_atm, 0, sizeof(double) * h->stride * CLM_AT_NFIELDS, h->stream));
  }
  // graphs hold StepArgs (with the constants) by value: new constants need
  // new graphs, new drivers in the same buffer do not
  const AtmosK ak = make_atmos_k(a, h->cfg.earth);
  if (std::memcmp(&ak, &h->ak, sizeof ak) != 0) drop_graphs(h);
  h->ak = ak;
  int rc = upload_cols_sorted(h, d, h->d_atm, nfields);
  if (rc != CLM_OK) return rc;
  CLM_CUDA(h, cudaStreamSynchronize(h->stream));
  return CLM_OK;
}

int clm_set_state(clm_handle* h, const double* v, const double* ti, const double* e, const double* Fw,
                  const double* Fe) {
  return set_state_impl(h, v, ti, e, Fw, Fe, cudaMemcpyHostToDevice);
}

int clm_get_state(clm_handle* h, double* v, double* ti, double* e, double* Fw, double* Fe) {
  return get_state_impl(h, v, ti, e, Fw, Fe, cudaMemcpyDeviceToHost);
}

int clm_set_state_device(clm_handle* h, const double* v, const double* ti, const double* e,
                         const double* Fw, const double* Fe) {
  return set_state_impl(h, v, ti, e, Fw, Fe, cudaMemcpyDeviceToDevice);
}

int clm_get_state_device(clm_handle* h, double* v, double* ti, double* e, double* Fw, double* Fe) {
  return get_state_impl(h, v, ti, e, Fw, Fe, cudaMemcpyDeviceToDevice);
}

int clm_step_async(clm_handle* h, double t, double dt, int32_t nsteps) {
  int rc = ready(h);
  if (rc != CLM_OK) return rc;
  if (!(dt > 0) || !std::isfinite(dt) || !std::isfinite(t) || nsteps < 0)
    return fail(h, CLM_ERR_ARG, "need dt > 0, finite t, nsteps >= 0");
  if (nsteps == 0) return CLM_OK;
  if (h->cfg.learned_guess == CLM_GUESS_NETWORK && (!h->d_mlp || !h->d_guess))
    return fail(h, CLM_ERR_STATE, "clm_load_mlp has not been called");
  if (h->cfg.learned_guess == CLM_GUESS_EXTRAPOLATE && !h->prev_valid) {
    // the history starts at the current state: the first step's guessed
    // increment is zero
    if (!h->d_prev)
      CLM_CUDA(h, cudaMalloc(&h->d_prev, sizeof(double) * 2 * (size_t)std::max<int64_t>(h->ncells_int, 1)));
    CLM_CUDA(h, restart_guess_history(h));
    h->prev_valid = true;
    drop_graphs(h);  // captured launches hold A.prev by value
  }
  // the step kernels OR each column's flags into d_flags: one call's flags
  // cover all of its steps, whatever its launches
  CLM_CUDA(h, cudaMemsetAsync(h->d_flags, 0, sizeof(uint32_t) * h->stride, h->stream));
  if (h->cfg.graph) {
    // a caller that is capturing the stream itself records the plain launches
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CLM_CUDA(h, cudaStreamIsCapturing(h->stream, &cs));
    if (cs == cudaStreamCaptureStatusNone) return step_graph(h, t, dt, nsteps);
  }
  const std::vector<Launch> seq = launch_sequence(h, nsteps);
  for (const Launch& l : seq) {
    StepClock clk;
    clk.t0 = step_time(t, l.step, dt);
    clk.dt = dt;
    rc = issue(h, l, clk, h->stream);
    if (rc != CLM_OK) return rc;
  }
  return CLM_OK;
}

int clm_step_host(clm_handle* h, double* v, double* ti, double* e, double* Fw, double* Fe,
                  double t, double dt, int32_t nsteps) {
  if (!h) return CLM_ERR_ARG;
  if (!h->have_geometry) return fail(h, CLM_ERR_STATE, "clm_set_geometry has not been called");
  if (!h->have_params) return fail(h, CLM_ERR_STATE, "clm_set_params has not been called");
  if (!(dt > 0) || !std::isfinite(dt) || !std::isfinite(t) || nsteps < 0)
    return fail(h, CLM_ERR_ARG, "need dt > 0, finite t, nsteps >= 0");
  const bool eh = is_eh(h);
  if (!v || !Fw || (eh && (!ti || !e || !Fe)))
    return fail(h, CLM_ERR_ARG, "every state array of the model is required");
  if (h->cfg.learned_guess || !h->perm_identity) {
    int rc = set_state_impl(h, v, ti, e, Fw, Fe, cudaMemcpyHostToDevice);
    if (rc == CLM_OK) rc = clm_step(h, t, dt, nsteps);
    if (rc == CLM_OK) rc = get_state_impl(h, v, ti, e, Fw, Fe, cudaMemcpyDeviceToHost);
    return rc;
  }
  if (!h->copy_in) {
    CLM_CUDA(h, cudaStreamCreateWithFlags(&h->copy_in, cudaStreamNonBlocking));
    CLM_CUDA(h, cudaStreamCreateWithFlags(&h->copy_out, cudaStreamNonBlocking));
  }
  const int nf = eh ? 3 : 1, nc = eh ? 2 : 1;
  const int64_t bytes = (int64_t)h->ncells_ref * nf * (int64_t)sizeof(double);
  // about 128 MB per chunk, at most 4 (each chunk's persistent launch ends
  // with a partial wave; measured on the 1,048,576 x 20 state: 4 chunks
  // 41.9 ms, 16 chunks 49.1 ms, unchunked 45.7 ms), chunks a whole number of
  // waves of the step grid's warps (one-wave first and last chunks: 34.6 vs
  // 36.1 ms per step with four equal chunks)
  int nch = h->cfg.host_chunks > 0
                ? h->cfg.host_chunks
                : (int)std::min<int64_t>(4, std::max<int64_t>(1, (bytes + (64 << 20)) >> 27));
  nch = std::max(1, std::min(nch, h->ntiles));
  const int wave = std::max(1, h->grid * h->wpc);
  // chunk boundaries (tiles): whole waves; with the automatic plan and at
  // least four waves, a one-wave first chunk (its copy in is the pipeline's
  // fill) and a last chunk of the final wave (its copy out is the drain)
  // around nch chunks of whole waves
  std::vector<int> bnd{0};
  const int nwaves = (h->ntiles + wave - 1) / wave;
  if (h->cfg.host_chunks <= 0 && nch > 1 && nwaves >= 4) {
    const int mid = nwaves - 2;  // waves between the first and the last
    const int per_w = (mid + nch - 1) / nch;
    bnd.push_back(wave);
    for (int w = 1 + per_w; w < nwaves - 1; w += per_w) bnd.push_back(w * wave);
    bnd.push_back((nwaves - 1) * wave);
    bnd.push_back(h->ntiles);
  } else {
    int per = (h->ntiles + nch - 1) / nch;
    if (per > wave) per = (per + wave - 1) / wave * wave;
    for (int T = per; T < h->ntiles; T += per) bnd.push_back(T);
    bnd.push_back(h->ntiles);
  }
  const int nchunks = (int)bnd.size() - 1;
  while ((int)h->host_ev.size() < 2 * nchunks) {
    cudaEvent_t ev;
    CLM_CUDA(h, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    h->host_ev.push_back(ev);
  }
  const Layout L = layout_of(h);
  StepArgs A = step_args(h);
  CLM_CUDA(h, cudaMemsetAsync(h->d_flags, 0, sizeof(uint32_t) * h->stride, h->stream));
  double* hf[3] = {v, ti, e};
  double* df[3] = {h->d_v, h->d_ti, h->d_e};
  double* hc[2] = {Fw, Fe};
  double* dc[2] = {h->d_Fw, h->d_Fe};
  for (int k = 0; k < nchunks; ++k) {
    const int T0 = bnd[k], T1 = bnd[k + 1];
    const int c0 = T0 * kTile, c1 = std::min(T1 * kTile, h->ncol);
    if (c0 >= c1) break;
    const int64_t a = h->ref_off[c0], b = h->ref_off[c1];
    cudaEvent_t ev_in = h->host_ev[2 * k], ev_done = h->host_ev[2 * k + 1];
    // in: this chunk's cells and per-column values (identity order: the
    // sorted index of a column is its own)
    for (int f = 0; f < nf; ++f)
      CLM_CUDA(h, cudaMemcpyAsync(h->d_stage + f * h->ncells_ref + a, hf[f] + a,
                                  sizeof(double) * (b - a), cudaMemcpyHostToDevice, h->copy_in));
    for (int f = 0; f < nc; ++f)
      CLM_CUDA(h, cudaMemcpyAsync(dc[f] + c0, hc[f] + c0, sizeof(double) * (c1 - c0),
                                  cudaMemcpyHostToDevice, h->copy_in));
    CLM_CUDA(h, cudaEventRecord(ev_in, h->copy_in));
    // transpose, step, transpose back on the handle's stream (step kernels
    // share the per-warp scratch, so they stay in one stream)
    CLM_CUDA(h, cudaStreamWaitEvent(h->stream, ev_in, 0));
    XFields Fi{}, Fo{};
    Fi.nf = Fo.nf = nf;
    for (int f = 0; f < nf; ++f) {
      Fi.src[f] = Fo.dst[f] = h->d_stage + f * h->ncells_ref;
      Fi.dst[f] = df[f];
      Fo.src[f] = df[f];
    }
    CLM_CUDA(h, ref_to_internal(L, Fi, h->stream, T0, T1 - T0));
    A.tile_begin = T0;
    A.tile_end = T1;
    A.order = nullptr;  // a chunk's launch covers its own tiles' columns
    if (splits(h)) {
      // split Newton per step: the chunk's tiles, then its deferred columns
      // (the queue serves one chunk at a time: the launches share the stream)
      StepArgs S = A;
      S.split = SplitQueue{h->d_queue, h->d_qcount, h->stride, h->nmax};
      S.split_at = kSplitIters;
      for (int s0 = 0; s0 < nsteps; ++s0) {
        StepClock clk;
        clk.t0 = step_time(t, s0, dt);
        clk.dt = dt;
        CLM_CUDA(h, cudaMemsetAsync(h->d_qcount, 0, sizeof(int), h->stream));
        CLM_CUDA(h, launch_step(S, h->cfg.model, h->cfg.precision, h->wpc, h->grid, h->d_scratch, clk, 1,
                                h->stream));
        CLM_CUDA(h, launch_resume(S, h->cfg.precision, h->wpc, h->grid, clk, h->stream));
      }
    } else {
      for (int s0 = 0; s0 < nsteps; s0 += 64) {
        StepClock clk;
        clk.t0 = step_time(t, s0, dt);
        clk.dt = dt;
        CLM_CUDA(h, launch_step(A, h->cfg.model, h->cfg.precision, h->wpc, h->grid, h->d_scratch, clk,
                                std::min(64, nsteps - s0), h->stream));
      }
    }
    CLM_CUDA(h, internal_to_ref(L, Fo, h->stream, T0, T1 - T0));
    CLM_CUDA(h, cudaEventRecord(ev_done, h->stream));
    // out
    CLM_CUDA(h, cudaStreamWaitEvent(h->copy_out, ev_done, 0));
    for (int f = 0; f < nf; ++f)
      CLM_CUDA(h, cudaMemcpyAsync(hf[f] + a, h->d_stage + f * h->ncells_ref + a, sizeof(double) * (b - a),
                                  cudaMemcpyDeviceToHost, h->copy_out));
    for (int f = 0; f < nc; ++f)
      CLM_CUDA(h, cudaMemcpyAsync(hc[f] + c0, dc[f] + c0, sizeof(double) * (c1 - c0),
                                  cudaMemcpyDeviceToHost, h->copy_out));
  }
  CLM_CUDA(h, cudaStreamSynchronize(h->copy_out));
  CLM_CUDA(h, cudaStreamSynchronize(h->stream));
  h->have_state = true;
  return CLM_OK;
}

int clm_autotune(clm_handle* h, double t, double dt, int32_t probe_steps, clm_tune_entry* table,
                 int32_t table_cap, int32_t* n_entries) {
  int rc = ready(h);
  if (rc != CLM_OK) return rc;
  if (!(dt > 0) || !std::isfinite(dt) || !std::isfinite(t) || probe_steps < 1 || probe_steps > 64)
    return fail(h, CLM_ERR_ARG, "need dt > 0, finite t, probe_steps in [1, 64]");
  if (table_cap < 0 || (table_cap > 0 && !table)) return fail(h, CLM_ERR_ARG, "bad table");
  // candidates: warps per CTA that fit the shared memory x tile order
  int dev_smem = 0;
  CLM_CUDA(h, cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device));
  std::vector<clm_tune_entry> cand;
  size_t need = 0;
  for (int w = 1; w <= 4; ++w) {
    if (step_smem_bytes(h->cfg.model, h->cfg.precision, h->nmax, w) > (size_t)dev_smem) break;
    int grid = 0;
    CLM_CUDA(h, step_grid(h->cfg.model, h->cfg.precision, h->cfg.hydrology_cm, h->d_geo != nullptr,
                          h->cfg.newton_mode == CLM_NEWTON_TOL, h->nmax, w, h->ntiles, &grid));
    need = std::max(need, step_scratch_doubles(h->cfg.model, h->cfg.precision, h->nmax, w, grid));
    for (int sch : {CLM_SCHED_STATIC, CLM_SCHED_DYNAMIC}) {
      clm_tune_entry e{};
      e.cols_per_cta = w * kTile;
      e.schedule = sch;
      e.grid = grid;
      cand.push_back(e);
    }
  }
  if (cand.empty()) return fail(h, CLM_ERR_ARG, "no launch configuration fits the shared memory");
  CLM_CUDA(h, cudaStreamSynchronize(h->stream));
  if (need > h->scratch_doubles) {
    dfree(h->d_scratch);
    CLM_CUDA(h, cudaMalloc(&h->d_scratch, sizeof(double) * need));
    h->scratch_doubles = need;
  }
  drop_graphs(h);
  // the probe advances the real state: keep a copy and put it back
  const int64_t ni = std::max<int64_t>(h->ncells_int, 1);
  const int nf = is_eh(h) ? 3 : 1;
  double* keep = nullptr;
  uint32_t* keep_fl = nullptr;
  int32_t* keep_it = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  auto cleanup = [&]() {
    if (keep) cudaFree(keep);
    if (keep_fl) cudaFree(keep_fl);
    if (keep_it) cudaFree(keep_it);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
  };
  auto bail = [&](cudaError_t err, const char* what) {
    cleanup();
    return cuda_fail(h, err, what);
  };
#define CLM_TRY(call)                               \
  do {                                              \
    cudaError_t _e = (call);                        \
    if (_e != cudaSuccess) return bail(_e, #call);  \
  } while (0)
  CLM_TRY(cudaMalloc(&keep, sizeof(double) * (nf * ni + 2 * h->stride)));
  CLM_TRY(cudaMalloc(&keep_fl, sizeof(uint32_t) * h->stride));
  CLM_TRY(cudaMalloc(&keep_it, sizeof(int32_t) * h->stride));
  CLM_TRY(cudaEventCreate(&e0));
  CLM_TRY(cudaEventCreate(&e1));
  double* fields[3] = {h->d_v, h->d_ti, h->d_e};
  auto save_restore = [&](bool save) -> cudaError_t {
    cudaError_t err = cudaSuccess;
    const cudaMemcpyKind k = cudaMemcpyDeviceToDevice;
    for (int f = 0; f < nf && err == cudaSuccess; ++f)
      err = save ? cudaMemcpyAsync(keep + f * ni, fields[f], sizeof(double) * ni, k, h->stream)
                 : cudaMemcpyAsync(fields[f], keep + f * ni, sizeof(double) * ni, k, h->stream);
    double* kf = keep + nf * ni;
    const size_t cb = sizeof(double) * h->stride;
    if (err == cudaSuccess)
      err = save ? cudaMemcpyAsync(kf, h->d_Fw, cb, k, h->stream) : cudaMemcpyAsync(h->d_Fw, kf, cb, k, h->stream);
    if (err == cudaSuccess && is_eh(h))
      err = save ? cudaMemcpyAsync(kf + h->stride, h->d_Fe, cb, k, h->stream)
                 : cudaMemcpyAsync(h->d_Fe, kf + h->stride, cb, k, h->stream);
    if (err == cudaSuccess)
      err = save ? cudaMemcpyAsync(keep_fl, h->d_flags, sizeof(uint32_t) * h->stride, k, h->stream)
                 : cudaMemcpyAsync(h->d_flags, keep_fl, sizeof(uint32_t) * h->stride, k, h->stream);
    if (err == cudaSuccess)
      err = save ? cudaMemcpyAsync(keep_it, h->d_iters, sizeof(int32_t) * h->stride, k, h->stream)
                 : cudaMemcpyAsync(h->d_iters, keep_it, sizeof(int32_t) * h->stride, k, h->stream);
    return err;
  };
  CLM_TRY(save_restore(true));
  const int wpc0 = h->wpc, grid0 = h->grid, sched0 = h->sched;
  int best = -1;
  for (size_t i = 0; i < cand.size(); ++i) {
    clm_tune_entry& c = cand[i];
    h->wpc = c.cols_per_cta / kTile;
    h->grid = c.grid;
    h->sched = c.schedule;
    StepArgs A = step_args(h);
    A.guess = nullptr;  // the probe times the step kernel alone
    A.prev = nullptr;   // and leaves the extrapolation history alone
    StepClock clk;
    clk.t0 = t;
    clk.dt = dt;
    // one untimed step (first-touch of the scratch slots), then the probe
    cudaError_t err = launch_step(A, h->cfg.model, h->cfg.precision, h->wpc, h->grid, h->d_scratch,
                                  clk, 1, h->stream);
    if (err == cudaSuccess) err = save_restore(false);
    if (err == cudaSuccess) err = cudaEventRecord(e0, h->stream);
    if (err == cudaSuccess)
      err = launch_step(A, h->cfg.model, h->cfg.precision, h->wpc, h->grid, h->d_scratch, clk,
                        probe_steps, h->stream);
    if (err == cudaSuccess) err = cudaEventRecord(e1, h->stream);
    if (err == cudaSuccess) err = save_restore(false);
    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
    if (err != cudaSuccess) {
      h->wpc = wpc0;
      h->grid = grid0;
      h->sched = sched0;
      return bail(err, "autotune probe");
    }
    c.ms_per_step = ms / probe_steps;
    if (best < 0 || c.ms_per_step < cand[best].ms_per_step) best = (int)i;
  }
#undef CLM_TRY
  h->wpc = cand[best].cols_per_cta / kTile;
  h->grid = cand[best].grid;
  h->sched = cand[best].schedule;
  cand[best].chosen = 1;
  const cudaError_t err = cudaStreamSynchronize(h->stream);
  cleanup();
  if (err != cudaSuccess) return cuda_fail(h, err, "autotune");
  for (int i = 0; i < (int)cand.size() && i < table_cap; ++i) table[i] = cand[i];
  if (n_entries) *n_entries = (int32_t)cand.size();
  return CLM_OK;
}

int clm_get_launch_config(const clm_handle* h, int32_t* cols_per_cta, int32_t* schedule, int32_t* grid) {
  if (!h) return CLM_ERR_ARG;
  if (cols_per_cta) *cols_per_cta = h->wpc * kTile;
  if (schedule) *schedule = h->sched;
  if (grid) *grid = h->grid;
  return CLM_OK;
}

int clm_sync(clm_handle* h) {
  if (!h) return CLM_ERR_ARG;
  CLM_CUDA(h, cudaStreamSynchronize(h->stream));
  return CLM_OK;
}

int clm_set_stream(clm_handle* h, void* cuda_stream) {
  if (!h) return CLM_ERR_ARG;
  CLM_CUDA(h, cudaStreamSynchronize(h->stream));
  h->stream = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : h->own_stream;
  return CLM_OK;
}

int clm_step(clm_handle* h, double t, double dt, int32_t nsteps) {
  int rc = clm_step_async(h, t, dt, nsteps);
  if (rc != CLM_OK) return rc;
  return clm_sync(h);
}

int clm_get_budgets(clm_handle* h, double* W, double* Eo) {
  int rc = ready(h);
  if (rc != CLM_OK) return rc;
  StepArgs A = step_args(h);
  double* dW = h->d_colstage + h->stride;
  double* dE = h->d_colstage + 2 * (size_t)h->stride;
  CLM_CUDA(h, launch_budgets(A, h->cfg.model, dW, dE, h->stream));
  if (W) {
    rc = download_cols(h, dW, W);
    if (rc != CLM_OK) return rc;
    CLM_CUDA(h, cudaStreamSynchronize(h->stream));
  }
  if (Eo) {
    if (is_eh(h)) {
      rc = download_cols(h, dE, Eo);
      if (rc != CLM_OK) return rc;
    } else {
      std::fill(Eo, Eo + h->ncol, 0.0);
    }
  }
  CLM_CUDA(h, cudaStreamSynchronize(h->stream));
  return CLM_OK;
}

int clm_get_status(clm_handle* h, uint32_t* flags, int32_t* iters) {
  if (!h) return CLM_ERR_ARG;
  if (!h->have_geometry) return fail(h, CLM_ERR_STATE, "clm_set_geometry has not been called");
  std::vector<uint32_t> f(h->stride);
  std::vector<int32_t> it(h->stride);
  CLM_CUDA(h, cudaMemcpyAsync(f.data(), h->d_flags, sizeof(uint32_t) * h->stride, cudaMemcpyDeviceToHost, h->stream));
  CLM_CUDA(h, cudaMemcpyAsync(it.data(), h->d_iters, sizeof(int32_t) * h->stride, cudaMemcpyDeviceToHost, h->stream));
  CLM_CUDA(h, cudaStreamSynchronize(h->stream));
  for (int s = 0; s < h->ncol; ++s) {
    const int c = h->perm[s];
    if (flags) flags[c] = f[s];
    if (iters) iters[c] = it[s];
  }
  return CLM_OK;
}

int clm_load_mlp(clm_handle* h, const void* weights, int64_t nbytes) {
  if (!h) return CLM_ERR_ARG;
  if (!is_eh(h)) return fail(h, CLM_ERR_UNSUPPORTED, "the learned guess is built for EnergyHydrology");
  if (!h->have_geometry) return fail(h, CLM_ERR_STATE, "clm_set_geometry has not been called");
  if (!weights || nbytes < kMlpBlobBytes) return fail(h, CLM_ERR_ARG, "weight blob too small");
  MlpBlobHeader hd;
  std::memcpy(&hd, weights, sizeof hd);
  if (hd.magic != kMlpMagic || hd.nin != (uint32_t)kMlpIn || hd.nhidden != (uint32_t)kMlpHidden ||
      hd.nout != (uint32_t)kMlpOut)
    return fail(h, CLM_ERR_ARG, "weight blob header does not match this library's network");
  const float* f = reinterpret_cast<const float*>(static_cast<const unsigned char*>(weights) + sizeof hd);
  const int nnorm = 2 * kMlpIn + 2 * kMlpOut;
  std::vector<float> buf((size_t)kMlpParams + nnorm);
  std::memcpy(buf.data(), f + nnorm, sizeof(float) * kMlpParams);  // parameters first
  std::memcpy(buf.data() + kMlpParams, f, sizeof(float) * nnorm);
  for (float x : buf)
    if (!std::isfinite(x)) return fail(h, CLM_ERR_ARG, "non-finite value in the weight blob");
  if (!h->d_mlp || !h->d_guess) drop_graphs(h);
  if (!h->d_mlp) CLM_CUDA(h, cudaMalloc(&h->d_mlp, sizeof(float) * buf.size()));
  if (!h->guess_grid) CLM_CUDA(h, mlp_guess_setup(h->stride, &h->guess_grid));
  CLM_CUDA(h, cudaMemcpyAsync(h->d_mlp, buf.data(), sizeof(float) * buf.size(), cudaMemcpyHostToDevice, h->stream));
  if (!h->d_guess) {
    const size_t gb = sizeof(float) * 2 * (size_t)std::max<int64_t>(h->ncells_int, 1);
    CLM_CUDA(h, cudaMalloc(&h->d_guess, gb));
    CLM_CUDA(h, cudaMemsetAsync(h->d_guess, 0xFF, gb, h->stream));  // NaN: no guess
  }
  if (!h->d_prev)
    CLM_CUDA(h, cudaMalloc(&h->d_prev, sizeof(double) * 2 * (size_t)std::max<int64_t>(h->ncells_int, 1)));
  CLM_CUDA(h, restart_guess_history(h));
  h->prev_valid = true;
  CLM_CUDA(h, cudaStreamSynchronize(h->stream));
  return CLM_OK;
}

int clm_features(clm_handle* h, double t, double dt, float* X) {
  int rc = ready(h);
  if (rc != CLM_OK) return rc;
  if (!is_eh(h)) return fail(h, CLM_ERR_UNSUPPORTED, "features are defined for EnergyHydrology");
  if (!X) return fail(h, CLM_ERR_ARG, "X is required");
  StepArgs A = step_args(h);
  CLM_CUDA(h, mlp_features(A, t, dt, X, h->stream));
  CLM_CUDA(h, cudaStreamSynchronize(h->stream));
  return CLM_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// internal accessors for clm_closures_api.cu
// ---------------------------------------------------------------------------
namespace clm {
StepArgs handle_step_args(clm_handle* h) { return step_args(h); }
Layout handle_layout(clm_handle* h) { return layout_of(h); }
int handle_ready(clm_handle* h) { return ready(h); }
int handle_fail(clm_handle* h, int code, const char* msg) { return fail(h, code, msg); }
int handle_cuda_fail(clm_handle* h, cudaError_t e, const char* what) { return cuda_fail(h, e, what); }
cudaStream_t handle_stream(clm_handle* h) { return h->stream; }
const int32_t* handle_ref_off(clm_handle* h) { return h->d_ref_off; }
int64_t handle_ncells_ref(clm_handle* h) { return h->ncells_ref; }
int handle_ncol(clm_handle* h) { return h->ncol; }
int handle_model(clm_handle* h) { return h->cfg.model; }
double* handle_state_ptr(clm_handle* h, int which) {
  return which == 0 ? h->d_v : (which == 1 ? h->d_ti : h->d_e);
}
}  // namespace clm
