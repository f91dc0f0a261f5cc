// Vertical geometry of one soil column, as the column code reads it.
//
// ClimaLand's soil domains are ClimaCore column spaces (Domains.jl:183-247):
// the mesh gives the face coordinates, the centres are the faces' midpoints,
// ClimaCore's Δz_field gives the layer widths (centre space) and the centre
// spacings (interior faces), and get_Δz (:935-949) halves the boundary
// faces' spacing for the centre-to-boundary distances Δz_top and Δz_bottom.
// The operators then read (rre.jl:161-203, energy_hydrology.jl:363-425):
//   GradientC2F at the face k|k+1   (x_{k+1} - x_k) / gap_k
//   InterpolateC2F                  (x_k + x_{k+1}) / 2
//   DivergenceF2C at the centre k   (F_{k+1/2} - F_{k-1/2}) / width_k
//   column_integral_definite!       sum_k width_k f_k
//
// ColGeom is a uniform column, Column(; zlim, nelements): n equal layers
// between z_lo and z_hi, everything from (z_hi - z_lo) / n.
// ColGeomS is a column with per-layer geometry (a stretched mesh,
// Column(; zlim, nelements, dz_tuple), or any mesh the caller passes as face
// coordinates to clm_set_faces): per-cell arrays in the internal layout,
// computed once on the host from the faces.
//
// Both expose the same accessors; the uniform one keeps the expressions the
// uniform path has always used (so its results do not change). The "row
// weight" is the factor by which the mixed path scales row k of its float
// Jacobian blocks so that every column of the scaled block sums to -weight
// (the face fluxes telescope under sum_k width_k): 1 on a uniform column
// (the unscaled rows already sum to -1), width_k on a stretched one.
#pragma once

#include <cstdint>

#include "clm_physics.cuh"

namespace clm {

template <typename T>
struct Col {
  T* p;
  int s;
  CLM_HD T& operator[](int k) const { return p[(int64_t)k * s]; }
  // a store this launch does not read back: cache-streaming (evict-first)
  CLM_HD void store_last(int k, T v) const {
#ifdef __CUDA_ARCH__
    __stcs(p + (int64_t)k * s, v);
#else
    p[(int64_t)k * s] = v;
#endif
  }
};

// Uniform column [z_lo, z_hi] with n layers: widths dz = (z_hi - z_lo) / n,
// centres z_lo + (k + 1/2) dz, the top face z_hi (the reference's column
// builds the faces as z_lo + (z_hi - z_lo) k / n; the two agree to rounding).
struct ColGeom {
  static constexpr bool kStretched = false;
  double zlo, zhi;
  int n;
  double dz, inv_dz;
  CLM_HD ColGeom(double lo, double hi, int nl)
      : zlo(lo), zhi(hi), n(nl), dz((hi - lo) / nl), inv_dz(1.0 / ((hi - lo) / nl)) {}
  CLM_HD double centre(int k) const { return zlo + (k + 0.5) * dz; }
  // the centre as the midpoint of the reference's faces (root extraction)
  CLM_HD double face_centre(int k) const {
    return 0.5 * ((zlo + (zhi - zlo) * ((double)k / n)) +
                  (k + 1 == n ? zhi : zlo + (zhi - zlo) * ((double)(k + 1) / n)));
  }
  CLM_HD double width(int) const { return dz; }
  CLM_HD double inv_width(int) const { return inv_dz; }
  CLM_HD double gap(int) const { return dz; }              // centre spacing k|k+1
  CLM_HD double hinv_gap(int) const { return 0.5 * inv_dz; }  // 0.5 / gap
  CLM_HD double half_top() const { return 0.5 * dz; }      // Δz_top
  CLM_HD double half_bot() const { return 0.5 * dz; }      // Δz_bottom
  CLM_HD double top_gap() const { return zhi - centre(n - 1); }  // surface to top centre
  CLM_HD double min_width() const { return dz; }
  CLM_HD double row_w(int) const { return 1.0; }
  CLM_HD double wsum() const { return (double)n; }
};

// Per-cell geometry arrays of a column in the internal layout (stride 32):
// centre z, width, 1 / width, gap (centre spacing to the layer above; for
// the top layer the distance from its centre to the surface, Δz_top) and
// 0.5 / gap; per column Δz_bottom, the thinnest width and the sum of widths.
struct GeoArrays {
  const double* z;
  const double* w;
  const double* rw;
  const double* gap;
  const double* hrg;
  const double* col;  // [3][stride]: Δz_bottom, min width, sum of widths
};

// Host side: the per-layer geometry of one column from its n + 1 faces f
// (finite, increasing), into the arrays of GeoArrays at cell stride cs:
// centres at the faces' midpoints, widths, centre spacings, Δz_top and
// Δz_bottom as distances from the boundary faces to the boundary centres.
// Returns Δz_bottom, the thinnest width and the sum of the widths.
struct GeoColumn {
  double bot, wmin, wsum;
};
inline GeoColumn column_geometry(const double* f, int n, int64_t cs, double* zc, double* w, double* rw,
                                 double* gap, double* hrg) {
  GeoColumn r{0.0, 0.0, 0.0};
  for (int k = 0; k < n; ++k) {
    const double wk = f[k + 1] - f[k];
    zc[k * cs] = 0.5 * (f[k] + f[k + 1]);
    w[k * cs] = wk;
    rw[k * cs] = 1.0 / wk;
    r.wmin = k == 0 ? wk : (wk < r.wmin ? wk : r.wmin);
    r.wsum += wk;
  }
  for (int k = 0; k < n; ++k) {
    const double g = k < n - 1 ? zc[(k + 1) * cs] - zc[k * cs] : f[n] - zc[k * cs];
    gap[k * cs] = g;
    hrg[k * cs] = k < n - 1 ? 0.5 / g : 0.0;
  }
  r.bot = zc[0] - f[0];
  return r;
}

struct ColGeomS {
  static constexpr bool kStretched = true;
  double zlo, zhi;
  int n;
  Col<const double> z, w, rw, gp, hrg;
  double bot, wmin, wtot;
  // base: the column's first cell; cs: the cell stride (32 in the internal
  // layout); s, stride: the column's slot in the per-column rows
  CLM_HD ColGeomS(const GeoArrays& g, int64_t base, int cs, int s, int stride, double lo, double hi,
                  int nl)
      : zlo(lo), zhi(hi), n(nl), z{g.z + base, cs}, w{g.w + base, cs}, rw{g.rw + base, cs},
        gp{g.gap + base, cs}, hrg{g.hrg + base, cs}, bot(g.col[s]), wmin(g.col[stride + s]),
        wtot(g.col[2 * stride + s]) {}
  CLM_HD double centre(int k) const { return z[k]; }
  CLM_HD double face_centre(int k) const { return z[k]; }
  CLM_HD double width(int k) const { return w[k]; }
  CLM_HD double inv_width(int k) const { return rw[k]; }
  CLM_HD double gap(int k) const { return gp[k]; }
  CLM_HD double hinv_gap(int k) const { return hrg[k]; }
  CLM_HD double half_top() const { return gp[n - 1]; }
  CLM_HD double half_bot() const { return bot; }
  CLM_HD double top_gap() const { return gp[n - 1]; }
  CLM_HD double min_width() const { return wmin; }
  CLM_HD double row_w(int k) const { return w[k]; }
  CLM_HD double wsum() const { return wtot; }
};

}  // namespace clm
