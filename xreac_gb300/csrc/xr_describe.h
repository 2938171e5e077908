// Host-side system descriptor shared by every entry point that runs the neighbour search
// (xr_eval / xr_eval_batch in xr_engine.cu, xr_count_neighbors_static in xr_static.cu): the cell
// checks, its inverse, the image scan reach and the FP32 error band of the distance screen. One
// definition, so the entry points cannot drift apart.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstring>

#include "xr_common.cuh"
#include "xreac_gb300.h"

namespace xr_host {

inline void inverse3(const double m[9], double inv[9], double* det_out) {
  const double a = m[0], b = m[1], c = m[2], d = m[3], e = m[4], f = m[5], g = m[6], h = m[7], i = m[8];
  const double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
  const double det = a * A + b * B + c * C;
  *det_out = det;
  inv[0] = A / det;
  inv[3] = B / det;
  inv[6] = C / det;
  inv[1] = -(b * i - c * h) / det;
  inv[4] = (a * i - c * g) / det;
  inv[7] = -(a * h - b * g) / det;
  inv[2] = (b * f - c * e) / det;
  inv[5] = -(a * f - c * d) / det;
  inv[8] = (a * e - b * d) / det;
}

// Fills S for system `in` with nonbonded cutoff rc: cell rows (identity when no direction is
// periodic) and inverse, pbc flags, image reach, the wrapped-coordinate origin and the bound on
// |FP32 squared distance - FP64 squared distance| (S.margin), the cutoffs. total_charge and
// has_guess are left to the caller. xpack (may be null) receives the positions as double4.
// Returns XR_OK, or XR_EINPUT with *msg set to xreac's message for the failed check.
//
// The error band covers every candidate image near a threshold, whichever list it comes from (the
// scan's images, a skin list, a caller's list): for such a candidate the image offset s in the
// wrapped frame has |s_k| < rc / h_k + 1 (h_k the cell height), which the reach below bounds.
//
// Cell rule of xreac's Boundary (src/xreac/geometry.py:37-39): det(cell) must exceed
// 1e-12 * |a1| |a2| |a3| ("nonsingular and right-handed").
// Image reach: where the cell height exceeds 2 rc only the nearest image can be within rc;
// otherwise +-(floor(rc / h + 1/2) + 1) cells around it are scanned (the supercell rule of
// src/xreac/geometry.py:58-79 as an image range).
inline int describe_system(const xr_system& in, int atom_off, double rc, XrSystem& S, double4_32a* xpack,
                           const char** msg) {
  std::memset(&S, 0, sizeof(S));
  S.atom_off = atom_off;
  S.natoms = in.natoms;
  bool any = false;
  for (int k = 0; k < 3; ++k) {
    S.periodic[k] = in.pbc[k] ? 1 : 0;
    any = any || S.periodic[k];
  }
  double cell[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  if (any) {
    if (!in.cell) {
      *msg = "A cell is required when pbc is enabled";
      return XR_EINPUT;
    }
    for (int k = 0; k < 9; ++k) cell[k] = in.cell[k];
    for (int k = 0; k < 9; ++k)
      if (!std::isfinite(cell[k])) {
        *msg = "cell must contain three finite lengths or a finite (3, 3) matrix";
        return XR_EINPUT;
      }
  }
  double lens[3];
  for (int k = 0; k < 3; ++k)
    lens[k] = std::sqrt(cell[3 * k] * cell[3 * k] + cell[3 * k + 1] * cell[3 * k + 1] + cell[3 * k + 2] * cell[3 * k + 2]);
  double inv[9], det;
  inverse3(cell, inv, &det);
  if (!(det > 1e-12 * lens[0] * lens[1] * lens[2]) || !std::isfinite(det)) {
    *msg = "Periodic cells must be nonsingular and right-handed";
    return XR_EINPUT;
  }
  for (int k = 0; k < 9; ++k) {
    S.cell[k] = cell[k];
    S.inv[k] = inv[k];
    S.cellf[k] = (float)cell[k];
  }
  for (int k = 0; k < 3; ++k) {
    const double height = 1.0 / std::sqrt(inv[k] * inv[k] + inv[3 + k] * inv[3 + k] + inv[6 + k] * inv[6 + k]);
    S.reach[k] = 0;
    if (S.periodic[k] && !(height > 2.0 * rc * (1.0 + 1e-9))) S.reach[k] = (int)std::floor(rc / height + 0.5) + 1;
  }
  // Wrapped positions (as the device computes them) bound the FP32 coordinate magnitudes.
  double origin[3] = {0, 0, 0};
  double ext = 0.0;
  for (int a = 0; a < in.natoms; ++a) {
    const double* p = in.positions + 3 * a;
    if (!std::isfinite(p[0]) || !std::isfinite(p[1]) || !std::isfinite(p[2])) {
      *msg = "positions must be a finite (N, 3) array in Angstrom";
      return XR_EINPUT;
    }
    double wr[3], xw[3];
    for (int k = 0; k < 3; ++k) {
      const double fk = p[0] * inv[k] + p[1] * inv[3 + k] + p[2] * inv[6 + k];
      wr[k] = S.periodic[k] ? std::floor(fk) : 0.0;
    }
    for (int q = 0; q < 3; ++q) xw[q] = p[q] - (wr[0] * cell[q] + wr[1] * cell[3 + q] + wr[2] * cell[6 + q]);
    if (a == 0)
      for (int q = 0; q < 3; ++q) origin[q] = xw[q];
    for (int q = 0; q < 3; ++q) ext = std::max(ext, std::fabs(xw[q] - origin[q]));
    if (xpack) xpack[a] = make_double4_32a(p[0], p[1], p[2], 0.0);
  }
  double img = 0.0;
  for (int k = 0; k < 3; ++k)
    if (S.periodic[k]) img += (S.reach[k] + 2) * lens[k];
  const double C = 2.0 * ext + img + 1.0;
  const double u = 1.0 / 16777216.0;  // 2^-24
  const double delta = 8.0 * u * C;    // per-component bound on |FP32 v - FP64 v|
  const double margin = 2.0 * std::sqrt(3.0) * (rc + 2.0 * delta) * delta + 3.0 * delta * delta + 8.0 * u * rc * rc;
  S.margin = (float)(4.0 * margin + 1e-6);
  for (int q = 0; q < 3; ++q) S.origin[q] = origin[q];
  S.rc = rc;
  S.inv_rc = 1.0 / rc;
  S.rc2 = rc * rc;
  S.bond_cut = std::min(5.0, rc);
  S.hb_cut = std::min(7.5, rc);
  S.rc2f = (float)S.rc2;
  S.bc2f = (float)(S.bond_cut * S.bond_cut);
  S.hc2f = (float)(S.hb_cut * S.hb_cut);
  return XR_OK;
}

// Cell grid of system S (already described) for a search within rl: cells at least rl / 2 high
// along each lattice direction (coarser where that would exceed max_cells cells), the cell offsets a
// search must visit, and the map from fractional coordinates to cells (wrapped coordinates in
// periodic directions; the range of the positions, from x, in the others). Fills S.cell_n,
// S.cell_reach, S.cell_f0 and S.cell_scale (S.cell_base is the caller's). Returns the number of cells
// and, in *visits, the expected image tests per atom pair of the system relative to the image scan
// (the fraction of the system's cells a search visits, over the scan's images per pair).
inline long long cell_grid(XrSystem& S, const double4_32a* x, int natoms, double rl, long long max_cells,
                           double* visits) {
  double h[3], fmin[3] = {0, 0, 0}, fmax[3] = {0, 0, 0};
  for (int k = 0; k < 3; ++k)
    h[k] = 1.0 / std::sqrt(S.inv[k] * S.inv[k] + S.inv[3 + k] * S.inv[3 + k] + S.inv[6 + k] * S.inv[6 + k]);
  for (int k = 0; k < 3; ++k) {
    if (S.periodic[k]) continue;
    double lo = INFINITY, hi = -INFINITY;
    for (int a = 0; a < natoms; ++a) {
      const double f = x[a].x * S.inv[k] + x[a].y * S.inv[3 + k] + x[a].z * S.inv[6 + k];
      lo = std::min(lo, f);
      hi = std::max(hi, f);
    }
    fmin[k] = lo;
    fmax[k] = hi;
  }
  double grow = 1.0;  // cell height multiplier, raised until the grid fits max_cells
  long long total = 1;
  for (int attempt = 0; attempt < 200; ++attempt) {
    total = 1;
    for (int k = 0; k < 3; ++k) {
      const double height = 0.5 * rl * grow;  // target cell height (A)
      if (S.periodic[k]) {
        const int n = std::max(1, (int)std::min(std::floor(h[k] / height), 1.0e6));
        S.cell_n[k] = n;
        S.cell_scale[k] = n;
        S.cell_f0[k] = 0.0;
      } else {
        // cells slightly wider than the target, so that the reach below is not one cell more by rounding
        const double wf = height / h[k] * (1.0 + 1e-6);
        const double f0 = fmin[k] - 1e-3 * wf;
        const double span = std::max(fmax[k] - f0, 0.0);
        const int n = (int)std::min(std::floor(span / wf) + 1.0, 1.0e6);
        S.cell_n[k] = n;
        S.cell_scale[k] = 1.0 / wf;
        S.cell_f0[k] = f0;
      }
      total *= S.cell_n[k];
    }
    if (total <= max_cells) break;
    grow *= 1.25;
  }
  double frac = 1.0;
  for (int k = 0; k < 3; ++k) {
    // an image within rl differs by at most rl / h_k in fractional coordinate k
    const double span = rl / h[k] * S.cell_scale[k] * (1.0 + 1e-9);
    S.cell_reach[k] = (int)std::min(std::ceil(span), 1.0e6);
    const int visited = 2 * S.cell_reach[k] + 1;
    frac *= (S.periodic[k] ? (double)visited : (double)std::min(visited, S.cell_n[k])) / S.cell_n[k];
    frac /= (2.0 * S.reach[k] + 1.0);
  }
  *visits = frac;
  return total;
}

}  // namespace xr_host
