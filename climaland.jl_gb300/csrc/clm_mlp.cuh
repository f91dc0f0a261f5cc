// Learned Newton initial guess: feature construction and the MLP shape.
//
// The network maps a column's state at the start of a step to the increment
// the converged Newton solve gives that step:
//   input  (kMlpIn, zero-padded to kMlpInPad): vartheta_l, theta_i and T of
//          the 20 layers (bottom first), the top water and heat fluxes at t,
//          alpha, n, nu, log10 K_sat, dt;
//   output (kMlpOut): delta vartheta_l and delta rho_e_int of the 20 layers
//          (u_{n+1} - u_n);
//   hidden 2 x 64, GELU; BF16 operands, FP32 accumulation.
// Inputs and outputs are standardised with per-feature mean / std stored
// with the weights.
#pragma once

#include <cstdint>

#include "clm_internal.cuh"

namespace clm {

constexpr int kMlpLayers = 20;  // columns the network is built for
constexpr int kMlpIn = 3 * kMlpLayers + 7;
constexpr int kMlpInPad = 80;
constexpr int kMlpHidden = 64;
constexpr int kMlpOut = 2 * kMlpLayers;
constexpr int kMlpOutPad = 48;

// Parameter block (FP32), one contiguous array:
//   W1 [kMlpInPad][kMlpHidden], b1 [kMlpHidden],
//   W2 [kMlpHidden][kMlpHidden], b2 [kMlpHidden],
//   W3 [kMlpHidden][kMlpOut], b3 [kMlpOut]
constexpr int kMlpW1 = 0;
constexpr int kMlpB1 = kMlpW1 + kMlpInPad * kMlpHidden;
constexpr int kMlpW2 = kMlpB1 + kMlpHidden;
constexpr int kMlpB2 = kMlpW2 + kMlpHidden * kMlpHidden;
constexpr int kMlpW3 = kMlpB2 + kMlpHidden;
constexpr int kMlpB3 = kMlpW3 + kMlpHidden * kMlpOut;
constexpr int kMlpParams = kMlpB3 + kMlpOut;

// Weight blob of clm_load_mlp / clm_mlp_get: header, normalisation, params.
struct MlpBlobHeader {
  uint32_t magic;    // kMlpMagic
  uint32_t nin, nhidden, nout;
};
constexpr uint32_t kMlpMagic = 0x504C4D43u;  // "CMLP"
// after the header: in_mean[kMlpIn], in_std[kMlpIn], out_mean[kMlpOut],
// out_std[kMlpOut], params[kMlpParams]  (all float)
constexpr int64_t kMlpBlobFloats = 2 * kMlpIn + 2 * kMlpOut + kMlpParams;
constexpr int64_t kMlpBlobBytes = sizeof(MlpBlobHeader) + kMlpBlobFloats * sizeof(float);

// Raw features of one column (layer k of the column through the strided
// views; n must be kMlpLayers). T from temperature_from_ρe_int with
// θ_l = volumetric_liquid_fraction, as update_aux! computes it. Layers
// [k0, k1) are written, and the seven column scalars when `tail`.
template <typename V>
CLM_HD void column_features(const StepArgs& A, int s, int orig, V v, V ti, V e, double t,
                            double dt, float* out, int k0 = 0, int k1 = kMlpLayers,
                            bool tail = true) {
  const int st = A.L.stride;
  const double* P = A.prm;
  const double nu = P[CLM_P_NU * st + s], thr = P[CLM_P_THETA_R * st + s];
  const double rcds = P[CLM_P_RHOC_DS * st + s];
  for (int k = k0; k < k1; ++k) {
    const double Yv = v[k], Yti = ti[k], Ye = e[k];
    const double v_safe = fmax(Yv, thr + kSqrtEps);
    const double nu_safe = fmax(nu - Yti, thr + kSqrtEps);
    const double tl = (v_safe < nu_safe) ? v_safe : nu_safe;
    out[k] = (float)Yv;
    out[kMlpLayers + k] = (float)Yti;
    out[2 * kMlpLayers + k] = (float)temperature(A.E, Ye, Yti, heat_capacity(A.E, tl, Yti, rcds));
  }
  if (!tail) return;
  out[60] = (float)forcing_value(A.forc[CLM_BC_TOP_WATER], st, s, A.col0 + orig, t, A.seed);
  out[61] = (float)forcing_value(A.forc[CLM_BC_TOP_HEAT], st, s, A.col0 + orig, t, A.seed);
  out[62] = (float)P[CLM_P_VG_ALPHA * st + s];
  out[63] = (float)P[CLM_P_VG_N * st + s];
  out[64] = (float)nu;
  out[65] = (float)log10(P[CLM_P_K_SAT * st + s]);
  out[66] = (float)dt;
}

}  // namespace clm
