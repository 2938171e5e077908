// Neighbour, pair and bond topology on the device.
//
// Restates the edge set of xreac's replicated_neighbors (src/xreac/neighbors.py:17-53): every image
// (j, S) of every atom with |x_j - x_i + S @ cell|^2 <= cutoff^2, zero-shift self edges excluded,
// in the canonical (i, j, Sx, Sy, Sz) order of Neighbors (src/xreac/neighbors.py:65-131).
//
// GB300 design: FP64 issues at 1/58 of the FP32 rate on this part, so the all-pairs scan runs in
// FP32 on cell-wrapped coordinates and only candidates whose squared distance lies inside a
// per-system error band of a threshold (cutoff, bond cutoff, hydrogen-bond cutoff) are re-tested
// with the reference's exact FP64 expression ((x_j - x_i) + S @ cell, ((vx^2 + vy^2) + vz^2)).
// A warp scans one source atom against 32 targets at a time in increasing j, and each lane visits
// its images in lexicographic shift order, so rows come out in canonical order without a sort.
#include "xr_common.cuh"

namespace {

constexpr int kHitBit = 1 << 30;

__global__ void k_prep(XrWork w) {
  int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= w.A) return;
  if (w.prep_zero) {
    // an evaluation's counters and scans start at zero (instead of a memset each; the status word
    // is cleared by the host before this kernel, since any block may flag it); cnt holds 4 (A + 1)
    // ints
    for (int k = 0; k < 4; ++k) w.cnt[4 * a + k] = 0;
    if (a == 0) {
      for (int k = 0; k < 4; ++k) w.cnt[4 * w.A + k] = 0;
      for (int k = 0; k < 8; ++k) w.counts[k] = 0;
      w.nmids[0] = 0;
      w.nmids[1] = 0;
      *w.bx_count = 0;
    }
    if (a < w.S) w.qiters[a] = 0;
    w.qb_first[a] = 0x7fffffff;
    w.qb_last[a] = -1;
  }
  const double4_32a p = w.x[a];
  int sys;
  if (w.types_in_x) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(p.w);
    int t = (int)(unsigned)(bits & 0xffffffffull);
    sys = (int)(unsigned)(bits >> 32);
    if (sys < 0 || sys >= w.S || t < 0) {  // not a packed word: flagged (the call fails), in-range indices kept
      atomicOr(w.status, XR_S_BAD_PACK);
      sys = 0;
      t = 0;
    }
    const_cast<int*>(w.type)[a] = t;
    const_cast<int*>(w.sys_of)[a] = sys;
  } else {
    sys = w.sys_of[a];
  }
  const XrSystem& S = w.sys[sys];
  const double xs[3] = {p.x, p.y, p.z};
  double f[3];
  int wr[3];
  for (int k = 0; k < 3; ++k) {
    f[k] = xs[0] * S.inv[0 * 3 + k] + xs[1] * S.inv[1 * 3 + k] + xs[2] * S.inv[2 * 3 + k];
    double fl = S.periodic[k] ? floor(f[k]) : 0.0;
    fl = fmin(fmax(fl, -1.0e6), 1.0e6);
    wr[k] = (int)fl;
    f[k] -= fl;
  }
  double xw[3];
  for (int c = 0; c < 3; ++c)
    xw[c] = xs[c] - (wr[0] * S.cell[0 * 3 + c] + wr[1] * S.cell[1 * 3 + c] + wr[2] * S.cell[2 * 3 + c]) - S.origin[c];
  w.wrap[a] = make_int4(wr[0], wr[1], wr[2], 0);
  w.xw[a] = make_float4((float)xw[0], (float)xw[1], (float)xw[2], 0.f);
  w.fw[a] = make_float4((float)f[0], (float)f[1], (float)f[2], 0.f);
  if (w.atom_cell) {
    // the cell of the wrapped position, from the same FP64 fractional coordinates as the wrap
    int cell = -1;
    if (S.cell_n[0] > 0) {
      int c[3];
      for (int k = 0; k < 3; ++k) {
        const double g = (S.periodic[k] ? f[k] : f[k] - S.cell_f0[k]) * S.cell_scale[k];
        c[k] = (int)fmin(fmax(floor(g), 0.0), (double)(S.cell_n[k] - 1));
      }
      cell = S.cell_base + (c[0] * S.cell_n[1] + c[1]) * S.cell_n[2] + c[2];
    }
    w.atom_cell[a] = cell;
  }
}

// Exact FP64 edge vector with the reference's association: (x_j - x_i) + S @ cell.
__device__ inline void exact_vector(const XrSystem& S, const double4_32a& xi, const double4_32a& xj, int sx, int sy, int sz,
                                    double v[3]) {
  const double xa[3] = {xi.x, xi.y, xi.z}, xb[3] = {xj.x, xj.y, xj.z};
  if ((sx | sy | sz) == 0) {  // no image shift: the offset is zero (the same values, FP64 work saved)
    for (int c = 0; c < 3; ++c) v[c] = __dsub_rn(xb[c], xa[c]);
    return;
  }
  for (int c = 0; c < 3; ++c) {
    double off = __dadd_rn(__dadd_rn(__dmul_rn((double)sx, S.cell[0 * 3 + c]), __dmul_rn((double)sy, S.cell[1 * 3 + c])),
                           __dmul_rn((double)sz, S.cell[2 * 3 + c]));
    v[c] = __dadd_rn(__dsub_rn(xb[c], xa[c]), off);
  }
}

__device__ inline double exact_d2(const double v[3]) {
  return __dadd_rn(__dadd_rn(__dmul_rn(v[0], v[0]), __dmul_rn(v[1], v[1])), __dmul_rn(v[2], v[2]));
}

// The FP32 screening constants of a system, held in registers for the candidate loop (the loop's
// status atomics would otherwise force the compiler to re-read them from global memory).
struct ScreenConsts {
  float cellf[9];
  float margin, rc2f, bc2f, hc2f;
};

__device__ inline ScreenConsts screen_consts(const XrSystem& S) {
  ScreenConsts c;
#pragma unroll
  for (int k = 0; k < 9; ++k) c.cellf[k] = S.cellf[k];
  c.margin = S.margin;
  c.rc2f = S.rc2f;
  c.bc2f = S.bc2f;
  c.hc2f = S.hc2f;
  return c;
}

// Classify one candidate image. Returns 0 (no edge) or kHitBit | code.
__device__ inline int classify(const XrWork& w, const XrSystem& S, const ScreenConsts& K, int i, int j, const float4& pi,
                               const float4& pj, const int4& wi, const int4& wj, int s0, int s1, int s2,
                               const double4_32a& xi) {
  const float vx = pj.x - pi.x + ((float)s0 * K.cellf[0] + (float)s1 * K.cellf[3] + (float)s2 * K.cellf[6]);
  const float vy = pj.y - pi.y + ((float)s0 * K.cellf[1] + (float)s1 * K.cellf[4] + (float)s2 * K.cellf[7]);
  const float vz = pj.z - pi.z + ((float)s0 * K.cellf[2] + (float)s1 * K.cellf[5] + (float)s2 * K.cellf[8]);
  const float r2 = vx * vx + vy * vy + vz * vz;
  const float mg = K.margin;
  const float rc2f = K.rc2f;
  if (r2 > rc2f + mg) return 0;
  const int sx = s0 - wj.x + wi.x, sy = s1 - wj.y + wi.y, sz = s2 - wj.z + wi.z;
  if (j == i && sx == 0 && sy == 0 && sz == 0) return 0;
  const float bc2f = K.bc2f, hc2f = K.hc2f;
  bool bond, hb;
  const bool exact = (r2 >= rc2f - mg) || (fabsf(r2 - bc2f) <= mg) || (fabsf(r2 - hc2f) <= mg) || (r2 < 1.0e-2f);
  if (exact) {
    double v[3];
    exact_vector(S, xi, w.x[j], sx, sy, sz, v);
    const double d2 = exact_d2(v);
    if (!(d2 <= S.rc2)) return 0;
    const double r = __dsqrt_rn(d2);
    if (r < 1e-6) atomicOr(w.status, XR_S_COINCIDENT);
    bond = r <= S.bond_cut;
    hb = r <= S.hb_cut;
  } else {
    bond = r2 < bc2f;
    hb = r2 < hc2f;
  }
  if (sx < -XR_SHIFT_MAX || sx > XR_SHIFT_MAX || sy < -XR_SHIFT_MAX || sy > XR_SHIFT_MAX || sz < -XR_SHIFT_MAX ||
      sz > XR_SHIFT_MAX) {
    atomicOr(w.status, XR_S_SHIFT_RANGE);
    return 0;
  }
  const bool neg = sx < 0 || (sx == 0 && (sy < 0 || (sy == 0 && sz < 0)));
  const bool half = (i < j) || (i == j && neg);
  return kHitBit | (int)(xr_pack_shift(sx, sy, sz) | (bond ? XR_CODE_BOND : 0u) | (hb ? XR_CODE_HB : 0u) |
                         (half ? XR_CODE_HALF : 0u));
}

// Writes edge e = (i -> j, code c) of the list and, for its flags, its pair p (half edges), bond b
// (half bond edges) and bond-row slot (bond edges); the other indices are -1.
__device__ inline void emit_edge(const XrWork& w, int i, int j, uint32_t c, int e, int p, int b, int slot) {
  w.edge[e] = make_int2(j, (int)c);
  w.edge_dbslot[e] = slot;
  if (p >= 0) {
    w.edge_pair[e] = p;
    w.pair_edge[p] = e;
    w.pair_i[p] = i;
    if (b >= 0) {
      w.pair_bond[p] = b;
      w.bond_pair[b] = p;
      w.bond_i[b] = i;
      w.bond_j[b] = j;
      w.dbrow[slot] = make_int2(b, 1);
    } else {
      w.pair_bond[p] = -1;
    }
  } else {
    w.edge_pair[e] = -1;
    if (slot >= 0) w.dbrow[slot] = make_int2(-1, -1);
  }
}

__device__ inline int warp_excl_scan(int v, int lane, int* total) {
  int x = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += y;
  }
  *total = __shfl_sync(0xffffffffu, x, 31);
  return x - v;
}

// One warp per source atom. FILL=false counts, FILL=true writes the rows.
template <bool FILL>
__global__ void k_neighbors(XrWork w) {
  const int lane = threadIdx.x & 31;
  const int i = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  if (i >= w.A) return;
  const XrSystem& S = w.sys[w.sys_of[i]];
  const float4 pi = w.xw[i], fi = w.fw[i];
  const int4 wi = w.wrap[i];
  const double4_32a xi = w.x[i];
  const int L = w.A + 1;
  int n_e = 0, n_h = 0, n_bh = 0, n_ba = 0;  // warp-uniform running totals
  int be = 0, bp = 0, bb = 0, bd = 0;
  if (FILL) {
    be = w.cnt[0 * L + i];
    bp = w.cnt[1 * L + i];
    bb = w.cnt[2 * L + i];
    bd = w.cnt[3 * L + i];
  }
  const int r0 = S.reach[0], r1 = S.reach[1], r2 = S.reach[2];
  // a lane's counts are at most its images, so 32 lanes' sums fit 16 bits when images < 2048
  const bool packed = (2 * r0 + 1) * (2 * r1 + 1) * (2 * r2 + 1) < 2048;
  const ScreenConsts K = screen_consts(S);
  const int natoms = S.natoms, atom_off = S.atom_off;
  const bool per0 = S.periodic[0] != 0, per1 = S.periodic[1] != 0, per2 = S.periodic[2] != 0;
  for (int jb = 0; jb < natoms; jb += 32) {
    const int jl = jb + lane;
    const bool valid = jl < natoms;
    const int j = atom_off + (valid ? jl : 0);
    const float4 pj = w.xw[j], fj = w.fw[j];
    const int4 wj = w.wrap[j];
    const int b0 = per0 ? -__float2int_rn(fj.x - fi.x) : 0;
    const int b1 = per1 ? -__float2int_rn(fj.y - fi.y) : 0;
    const int b2 = per2 ? -__float2int_rn(fj.z - fi.z) : 0;
    int c_e = 0, c_h = 0, c_bh = 0, c_ba = 0;
    if (valid) {
      for (int o0 = -r0; o0 <= r0; ++o0)
        for (int o1 = -r1; o1 <= r1; ++o1)
          for (int o2 = -r2; o2 <= r2; ++o2) {
            const int code = classify(w, S, K, i, j, pi, pj, wi, wj, b0 + o0, b1 + o1, b2 + o2, xi);
            if (code) {
              ++c_e;
              const bool half = code & XR_CODE_HALF, bond = code & XR_CODE_BOND;
              c_h += half;
              c_bh += half && bond;
              c_ba += bond;
            }
          }
    }
    int t_e, t_h, t_bh, t_ba;
    int o_e = 0, o_h = 0, o_bh = 0, o_ba = 0;
    if (!FILL) {  // the count pass needs the warp's totals only
      t_e = __reduce_add_sync(0xffffffffu, c_e);
      t_h = __reduce_add_sync(0xffffffffu, c_h);
      t_bh = __reduce_add_sync(0xffffffffu, c_bh);
      t_ba = __reduce_add_sync(0xffffffffu, c_ba);
    } else if (packed) {  // two counters per 32-bit scan: every prefix fits in 16 bits
      int t0, t1;
      const int s0 = warp_excl_scan(c_e | (c_h << 16), lane, &t0);
      const int s1 = warp_excl_scan(c_bh | (c_ba << 16), lane, &t1);
      o_e = s0 & 0xffff;
      o_h = s0 >> 16;
      o_bh = s1 & 0xffff;
      o_ba = s1 >> 16;
      t_e = t0 & 0xffff;
      t_h = t0 >> 16;
      t_bh = t1 & 0xffff;
      t_ba = t1 >> 16;
    } else {
      o_e = warp_excl_scan(c_e, lane, &t_e);
      o_h = warp_excl_scan(c_h, lane, &t_h);
      o_bh = warp_excl_scan(c_bh, lane, &t_bh);
      o_ba = warp_excl_scan(c_ba, lane, &t_ba);
    }
    if (FILL && c_e) {
      int k_e = 0, k_h = 0, k_bh = 0, k_ba = 0;
      for (int o0 = -r0; o0 <= r0; ++o0)
        for (int o1 = -r1; o1 <= r1; ++o1)
          for (int o2 = -r2; o2 <= r2; ++o2) {
            const int code = classify(w, S, K, i, j, pi, pj, wi, wj, b0 + o0, b1 + o1, b2 + o2, xi);
            if (!code) continue;
            const uint32_t c = (uint32_t)code & ~(uint32_t)kHitBit;
            const bool half = c & XR_CODE_HALF, bond = c & XR_CODE_BOND;
            const int e = be + n_e + o_e + k_e++;
            const int slot = bond ? bd + n_ba + o_ba + k_ba++ : -1;
            const int p = half ? bp + n_h + o_h + k_h++ : -1;
            const int b = half && bond ? bb + n_bh + o_bh + k_bh++ : -1;
            emit_edge(w, i, j, c, e, p, b, slot);
          }
    }
    n_e += t_e;
    n_h += t_h;
    n_bh += t_bh;
    n_ba += t_ba;
  }
  if (!FILL && lane == 0) {
    w.cnt[0 * L + i] = n_e;
    w.cnt[1 * L + i] = n_h;
    w.cnt[2 * L + i] = n_bh;
    w.cnt[3 * L + i] = n_ba;
  }
}

// Candidate list: every image (j, S) within the descriptor's cutoff (the list cutoff rc + 2 skin,
// from a second set of descriptors), in canonical order, without flags: one counter per atom
// (FILL=false, into cand_cnt) or the rows (FILL=true, cand_edge = {j, shift bits}).
template <bool FILL>
__global__ void k_candidates(XrWork w) {
  const int lane = threadIdx.x & 31;
  const int i = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  if (i >= w.A) return;
  const XrSystem& S = w.sys[w.sys_of[i]];
  const float4 pi = w.xw[i], fi = w.fw[i];
  const int4 wi = w.wrap[i];
  const double4_32a xi = w.x[i];
  const int r0 = S.reach[0], r1 = S.reach[1], r2 = S.reach[2];
  const ScreenConsts K = screen_consts(S);
  const int natoms = S.natoms, atom_off = S.atom_off;
  const bool per0 = S.periodic[0] != 0, per1 = S.periodic[1] != 0, per2 = S.periodic[2] != 0;
  int n_e = FILL ? w.cand_cnt[i] : 0;
  for (int jb = 0; jb < natoms; jb += 32) {
    const int jl = jb + lane;
    const bool valid = jl < natoms;
    const int j = atom_off + (valid ? jl : 0);
    const float4 pj = w.xw[j], fj = w.fw[j];
    const int4 wj = w.wrap[j];
    const int b0 = per0 ? -__float2int_rn(fj.x - fi.x) : 0;
    const int b1 = per1 ? -__float2int_rn(fj.y - fi.y) : 0;
    const int b2 = per2 ? -__float2int_rn(fj.z - fi.z) : 0;
    int c_e = 0;
    if (valid)
      for (int o0 = -r0; o0 <= r0; ++o0)
        for (int o1 = -r1; o1 <= r1; ++o1)
          for (int o2 = -r2; o2 <= r2; ++o2) c_e += classify(w, S, K, i, j, pi, pj, wi, wj, b0 + o0, b1 + o1, b2 + o2, xi) != 0;
    int t_e, o_e = 0;
    if (!FILL) {
      t_e = __reduce_add_sync(0xffffffffu, c_e);
    } else {
      o_e = warp_excl_scan(c_e, lane, &t_e);
      if (c_e) {
        int k = n_e + o_e;
        for (int o0 = -r0; o0 <= r0; ++o0)
          for (int o1 = -r1; o1 <= r1; ++o1)
            for (int o2 = -r2; o2 <= r2; ++o2) {
              const int code = classify(w, S, K, i, j, pi, pj, wi, wj, b0 + o0, b1 + o1, b2 + o2, xi);
              if (code) w.cand_edge[k++] = make_int2(j, (int)((uint32_t)code & XR_SHIFT_MASK));
            }
      }
    }
    n_e += t_e;
  }
  if (!FILL && lane == 0) w.cand_cnt[i] = n_e;
}

// ------------------------------------------------------------------------------ cell list
// Atoms binned into the cells k_prep assigned (order within a cell is that of the atomics; rows are
// sorted afterwards, so results do not depend on it).
__global__ void k_cell_count(XrWork w) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= w.A) return;
  const int c = w.atom_cell[a];
  if (c >= 0) w.atom_slot[a] = atomicAdd(w.cell_cnt + c, 1);
}

__global__ void k_cell_fill(XrWork w) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= w.A) return;
  const int c = w.atom_cell[a];
  if (c >= 0) w.cell_atoms[w.cell_cnt[c] + w.atom_slot[a]] = a;
}

__device__ inline int floor_div(int a, int n) { return a >= 0 ? a / n : -((-a + n - 1) / n); }

// Candidate images within the descriptor's cutoff from the cell list: one warp per source atom
// visits the cells within cell_reach of its own. Any image within the cutoff lies there: its
// fractional coordinates differ by at most cutoff / h_k (h_k the cell height), which is at most
// cell_reach cells. For fixed offsets in the first two directions the cells along the third are
// consecutive in cell_atoms, so their atoms are streamed as one range per image shift and the
// lanes stay busy however few atoms a cell holds. Each image is visited once: a cell offset fixes
// the wrapped cell and its shift. FILL=false counts (cand_cnt, and the longest row into counts[6]);
// FILL=true writes {j, shift bits} in visiting order.
template <bool FILL>
__global__ void k_cell_candidates(XrWork w) {
  const int lane = threadIdx.x & 31;
  const int i = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  if (i >= w.A) return;
  const XrSystem& S = w.sys[w.sys_of[i]];
  const float4 pi = w.xw[i];
  const int4 wi = w.wrap[i];
  const double4_32a xi = w.x[i];
  const ScreenConsts K = screen_consts(S);
  const int n0 = S.cell_n[0], n1 = S.cell_n[1], n2 = S.cell_n[2];
  const int m0 = S.cell_reach[0], m1 = S.cell_reach[1], m2 = S.cell_reach[2];
  const bool per0 = S.periodic[0] != 0, per1 = S.periodic[1] != 0, per2 = S.periodic[2] != 0;
  const int local = w.atom_cell[i] - S.cell_base;
  const int c2 = local % n2, c1 = (local / n2) % n1, c0 = local / (n1 * n2);
  const unsigned below = (1u << lane) - 1u;
  int n_e = FILL ? w.cand_cnt[i] : 0;
  for (int d0 = -m0; d0 <= m0; ++d0) {
    int e0 = c0 + d0, s0 = 0;
    if (per0) {
      s0 = floor_div(e0, n0);
      e0 -= s0 * n0;
    } else if (e0 < 0 || e0 >= n0) {
      continue;
    }
    for (int d1 = -m1; d1 <= m1; ++d1) {
      int e1 = c1 + d1, s1 = 0;
      if (per1) {
        s1 = floor_div(e1, n1);
        e1 -= s1 * n1;
      } else if (e1 < 0 || e1 >= n1) {
        continue;
      }
      const int rowbase = S.cell_base + (e0 * n1 + e1) * n2;
      int lo = c2 - m2, hi = c2 + m2;
      if (!per2) {
        lo = max(lo, 0);
        hi = min(hi, n2 - 1);
      }
      for (int e = lo; e <= hi;) {
        const int s2 = per2 ? floor_div(e, n2) : 0;
        const int seg_end = per2 ? min(hi, (s2 + 1) * n2 - 1) : hi;
        const int abeg = w.cell_cnt[rowbase + (e - s2 * n2)], aend = w.cell_cnt[rowbase + (seg_end - s2 * n2) + 1];
        for (int k0 = abeg; k0 < aend; k0 += 32) {
          const int k = k0 + lane;
          int code = 0, j = 0;
          if (k < aend) {
            j = w.cell_atoms[k];
            code = classify(w, S, K, i, j, pi, w.xw[j], wi, w.wrap[j], s0, s1, s2, xi);
          }
          const unsigned m = __ballot_sync(0xffffffffu, code != 0);
          if (FILL && code) w.cand_edge[n_e + __popc(m & below)] = make_int2(j, (int)((uint32_t)code & XR_SHIFT_MASK));
          n_e += __popc(m);
        }
        e = seg_end + 1;
      }
    }
  }
  if (!FILL && lane == 0) {
    w.cand_cnt[i] = n_e;
    atomicMax(w.counts + 6, n_e);
  }
}

// One block per candidate row: bitonic sort of the row's keys (j << 27 | shift bits, the canonical
// order) in shared memory, padded to a power of two.
__global__ void k_row_sort(XrWork w, int cap) {
  extern __shared__ unsigned long long keys[];
  const int i = blockIdx.x;
  const int beg = w.cand_cnt[i], len = w.cand_cnt[i + 1] - beg;
  if (len < 2) return;
  if (len > cap) {  // cannot happen: the host sized the buffer for the longest row
    if (threadIdx.x == 0) atomicOr(w.status, XR_S_LIMIT);
    return;
  }
  int P = 2;
  while (P < len) P <<= 1;
  for (int t = threadIdx.x; t < P; t += blockDim.x) {
    if (t < len) {
      const int2 c = w.cand_edge[beg + t];
      keys[t] = ((unsigned long long)(uint32_t)c.x << 27) | ((uint32_t)c.y & XR_SHIFT_MASK);
    } else {
      keys[t] = ~0ull;
    }
  }
  __syncthreads();
  for (int k = 2; k <= P; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = threadIdx.x; t < (P >> 1); t += blockDim.x) {
        const int lo = 2 * t - (t & (j - 1)), hi = lo + j;
        const bool up = (lo & k) == 0;
        const unsigned long long a = keys[lo], b = keys[hi];
        if ((a > b) == up) {
          keys[lo] = b;
          keys[hi] = a;
        }
      }
      __syncthreads();
    }
  for (int t = threadIdx.x; t < len; t += blockDim.x)
    w.cand_edge[beg + t] = make_int2((int)(keys[t] >> 27), (int)(keys[t] & XR_SHIFT_MASK));
}

// The edges within the cutoff of a candidate list (rows of {j, shift bits} in canonical order, a
// superset of the edges: a skin list of an earlier step, or a caller-supplied list), with their
// flags, classified exactly as k_neighbors classifies an image. One warp per source atom, 32
// candidates at a time; the kept candidates stay in row order, so the rows remain canonical.
// FILL=false counts per atom as k_neighbors<false> does; FILL=true writes the rows.
template <bool FILL>
__global__ void k_filter(XrWork w) {
  const int lane = threadIdx.x & 31;
  const int i = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  if (i >= w.A) return;
  const XrSystem& S = w.sys[w.sys_of[i]];
  const float4 pi = w.xw[i];
  const int4 wi = w.wrap[i];
  const double4_32a xi = w.x[i];
  const ScreenConsts K = screen_consts(S);
  const int L = w.A + 1;
  const int beg = w.cand_cnt[i], end = w.cand_cnt[i + 1];
  int n_e = 0, n_h = 0, n_bh = 0, n_ba = 0;
  if (FILL) {
    n_e = w.cnt[0 * L + i];
    n_h = w.cnt[1 * L + i];
    n_bh = w.cnt[2 * L + i];
    n_ba = w.cnt[3 * L + i];
  }
  const unsigned below = (1u << lane) - 1u;
  for (int k0 = beg; k0 < end; k0 += 32) {
    const int k = k0 + lane;
    int code = 0, j = 0;
    if (k < end) {
      const int2 cand = w.cand_edge[k];
      j = cand.x;
      const uint32_t sh = (uint32_t)cand.y;
      const int4 wj = w.wrap[j];
      code = classify(w, S, K, i, j, pi, w.xw[j], wi, wj, xr_sx(sh) + wj.x - wi.x, xr_sy(sh) + wj.y - wi.y,
                      xr_sz(sh) + wj.z - wi.z, xi);
    }
    const uint32_t c = (uint32_t)code & ~(uint32_t)kHitBit;
    const bool hit = code != 0, half = hit && (c & XR_CODE_HALF), bond = hit && (c & XR_CODE_BOND);
    const unsigned m_e = __ballot_sync(0xffffffffu, hit), m_h = __ballot_sync(0xffffffffu, half);
    const unsigned m_bh = __ballot_sync(0xffffffffu, half && bond), m_ba = __ballot_sync(0xffffffffu, bond);
    if (FILL && hit) {
      const int e = n_e + __popc(m_e & below);
      const int slot = bond ? n_ba + __popc(m_ba & below) : -1;
      const int p = half ? n_h + __popc(m_h & below) : -1;
      const int b = half && bond ? n_bh + __popc(m_bh & below) : -1;
      emit_edge(w, i, j, c, e, p, b, slot);
    }
    n_e += __popc(m_e);
    n_h += __popc(m_h);
    n_bh += __popc(m_bh);
    n_ba += __popc(m_ba);
  }
  if (!FILL && lane == 0) {
    w.cnt[0 * L + i] = n_e;
    w.cnt[1 * L + i] = n_h;
    w.cnt[2 * L + i] = n_bh;
    w.cnt[3 * L + i] = n_ba;
  }
}

// Reverse edges: a non-half edge (i -> j, S) takes the pair of (j -> i, -S), found by binary search
// in row j (rows are sorted by (j, shift bits), which is the canonical order).
__global__ void k_reverse(XrWork w) {
  const int lane = threadIdx.x & 31;
  const int i = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  if (i >= w.A) return;
  const int L = w.A + 1;
  const int beg = w.cnt[0 * L + i], end = w.cnt[0 * L + i + 1];
  for (int e = beg + lane; e < end; e += 32) {
    const int2 ed = w.edge[e];
    const uint32_t code = (uint32_t)ed.y;
    if (code & XR_CODE_HALF) continue;
    const int j = ed.x;
    const uint64_t key = ((uint64_t)(uint32_t)i << 27) | xr_neg_shift(code & XR_SHIFT_MASK);
    int lo = w.cnt[0 * L + j], hi = w.cnt[0 * L + j + 1];
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      const int2 m = w.edge[mid];
      const uint64_t k = ((uint64_t)(uint32_t)m.x << 27) | ((uint32_t)m.y & XR_SHIFT_MASK);
      if (k < key)
        lo = mid + 1;
      else
        hi = mid;
    }
    const int rowend = w.cnt[0 * L + j + 1];
    bool ok = lo < rowend;
    if (ok) {
      const int2 m = w.edge[lo];
      ok = m.x == i && (((uint32_t)m.y & XR_SHIFT_MASK) == xr_neg_shift(code & XR_SHIFT_MASK));
    }
    if (!ok) {
      // Inconsistent list (cannot happen for lists built here): record it and keep every index valid.
      atomicOr(w.status, XR_S_REVERSE);
      w.edge_pair[e] = 0;
      if (code & XR_CODE_BOND) w.dbrow[w.edge_dbslot[e]] = make_int2(0, -1);
      continue;
    }
    const int p = w.edge_pair[lo];
    w.edge_pair[e] = p;
    if (code & XR_CODE_BOND) w.dbrow[w.edge_dbslot[e]] = make_int2(w.pair_bond[p], -1);
  }
}

// ---------------------------------------------------------------- multi-array exclusive scan
// Scans the four count arrays cnt[k][0..A] in place (the last slot of each holds 0 on entry and
// the total on exit) and copies the totals to counts[0..3].
constexpr int kScanThreads = 1024;
constexpr int kScanPer = 4;
constexpr int kScanTile = kScanThreads * kScanPer;

__device__ inline int block_excl_scan(int v, int* smem, int* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += y;
  }
  if (lane == 31) smem[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int s = lane < (blockDim.x >> 5) ? smem[lane] : 0;
    int t = s;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, t, d);
      if (lane >= d) t += y;
    }
    smem[lane] = t - s;
    if (lane == 31) smem[32] = t;
  }
  __syncthreads();
  const int r = x - v + smem[wid];
  *total = smem[32];
  __syncthreads();
  return r;
}

__global__ void k_scan_blocks(int* base, int L, int* block_sums, int nblocks) {
  __shared__ int smem[33];
  const int k = blockIdx.y;
  int* a = base + (size_t)k * L;
  const int first = blockIdx.x * kScanTile + threadIdx.x * kScanPer;
  int s = 0;
  for (int t = 0; t < kScanPer; ++t) s += (first + t < L) ? a[first + t] : 0;
  int total;
  block_excl_scan(s, smem, &total);
  if (threadIdx.x == 0) block_sums[k * nblocks + blockIdx.x] = total;
}

__global__ void k_scan_sums(int* block_sums, int nblocks, int* totals) {
  __shared__ int smem[33];
  const int k = blockIdx.x;
  int carry = 0;
  for (int b0 = 0; b0 < nblocks; b0 += kScanThreads) {
    const int idx = b0 + threadIdx.x;
    const int v = idx < nblocks ? block_sums[k * nblocks + idx] : 0;
    int total;
    const int ex = block_excl_scan(v, smem, &total);
    if (idx < nblocks) block_sums[k * nblocks + idx] = ex + carry;
    carry += total;
  }
  if (threadIdx.x == 0) totals[k] = carry;
}

__global__ void k_scan_apply(int* base, int L, const int* block_sums, int nblocks) {
  __shared__ int smem[33];
  const int k = blockIdx.y;
  int* a = base + (size_t)k * L;
  const int first = blockIdx.x * kScanTile + threadIdx.x * kScanPer;
  int v[kScanPer];
  int s = 0;
  for (int t = 0; t < kScanPer; ++t) {
    v[t] = (first + t < L) ? a[first + t] : 0;
    s += v[t];
  }
  int total;
  int ex = block_excl_scan(s, smem, &total) + block_sums[k * nblocks + blockIdx.x];
  for (int t = 0; t < kScanPer; ++t) {
    if (first + t < L) a[first + t] = ex;
    ex += v[t];
  }
}

// Exclusive scans in place of `narrays` arrays of length L laid out one after another (the last
// slot of each holds 0 on entry and the total on exit); totals[k] receives each total. block_sums
// needs narrays * ceil(L / kScanTile) ints.
void scan_arrays(int* base, int L, int narrays, int* block_sums, int* totals, cudaStream_t st) {
  const int nblocks = (L + kScanTile - 1) / kScanTile;
  k_scan_blocks<<<dim3(nblocks, narrays), kScanThreads, 0, st>>>(base, L, block_sums, nblocks);
  k_scan_sums<<<narrays, kScanThreads, 0, st>>>(block_sums, nblocks, totals);
  k_scan_apply<<<dim3(nblocks, narrays), kScanThreads, 0, st>>>(base, L, block_sums, nblocks);
}

}  // namespace

void xr_launch_prep(const XrWork& w, cudaStream_t st) { k_prep<<<(w.A + 255) / 256, 256, 0, st>>>(w); }

void xr_launch_count(const XrWork& w, cudaStream_t st) {
  const int warps_per_block = 8;
  k_neighbors<false><<<(w.A + warps_per_block - 1) / warps_per_block, 32 * warps_per_block, 0, st>>>(w);
}

void xr_launch_topology(const XrWork& w, cudaStream_t st) {
  xr_launch_prep(w, st);
  xr_launch_count(w, st);
}

void xr_launch_rows(const XrWork& w, cudaStream_t st) {
  const int warps_per_block = 8;
  k_neighbors<true><<<(w.A + warps_per_block - 1) / warps_per_block, 32 * warps_per_block, 0, st>>>(w);
}

// Needs w.red to hold at least 4 * ceil((A+1)/4096) ints.
void xr_launch_scan(const XrWork& w, cudaStream_t st) {
  scan_arrays(w.cnt, w.A + 1, 4, reinterpret_cast<int*>(w.red), w.counts, st);
}

void xr_launch_candidates(const XrWork& w, bool fill, cudaStream_t st) {
  const int warps_per_block = 8;
  const int blocks = (w.A + warps_per_block - 1) / warps_per_block;
  if (fill) {
    k_candidates<true><<<blocks, 32 * warps_per_block, 0, st>>>(w);
  } else {
    k_candidates<false><<<blocks, 32 * warps_per_block, 0, st>>>(w);
    scan_arrays(w.cand_cnt, w.A + 1, 1, reinterpret_cast<int*>(w.red), w.counts + 5, st);
  }
}

void xr_launch_filter(const XrWork& w, bool fill, cudaStream_t st) {
  const int warps_per_block = 8;
  const int blocks = (w.A + warps_per_block - 1) / warps_per_block;
  if (fill)
    k_filter<true><<<blocks, 32 * warps_per_block, 0, st>>>(w);
  else
    k_filter<false><<<blocks, 32 * warps_per_block, 0, st>>>(w);
}

void xr_launch_cells(const XrWork& w, cudaStream_t st) {
  cudaMemsetAsync(w.cell_cnt, 0, sizeof(int) * ((size_t)w.ncells + 1), st);
  k_cell_count<<<(w.A + 255) / 256, 256, 0, st>>>(w);
  scan_arrays(w.cell_cnt, w.ncells + 1, 1, reinterpret_cast<int*>(w.red), w.counts + 7, st);
  k_cell_fill<<<(w.A + 255) / 256, 256, 0, st>>>(w);
}

void xr_launch_cell_candidates(const XrWork& w, bool fill, cudaStream_t st) {
  const int warps_per_block = 8;
  const int blocks = (w.A + warps_per_block - 1) / warps_per_block;
  if (fill) {
    k_cell_candidates<true><<<blocks, 32 * warps_per_block, 0, st>>>(w);
  } else {
    k_cell_candidates<false><<<blocks, 32 * warps_per_block, 0, st>>>(w);
    scan_arrays(w.cand_cnt, w.A + 1, 1, reinterpret_cast<int*>(w.red), w.counts + 5, st);
  }
}

void xr_launch_row_sort(const XrWork& w, int max_row, cudaStream_t st) {
  int cap = 2;
  while (cap < max_row) cap <<= 1;
  if (max_row < 2) return;
  const size_t bytes = sizeof(unsigned long long) * cap;
  if (bytes > 48 * 1024) cudaFuncSetAttribute(k_row_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  k_row_sort<<<w.A, 128, bytes, st>>>(w, cap);
}

void xr_launch_reverse(const XrWork& w, cudaStream_t st) {
  const int warps_per_block = 8;
  k_reverse<<<(w.A + warps_per_block - 1) / warps_per_block, 32 * warps_per_block, 0, st>>>(w);
}

void xr_launch_topology_fill(const XrWork& w, cudaStream_t st) {
  const int warps_per_block = 8;
  const int blocks = (w.A + warps_per_block - 1) / warps_per_block;
  k_neighbors<true><<<blocks, 32 * warps_per_block, 0, st>>>(w);
  k_reverse<<<blocks, 32 * warps_per_block, 0, st>>>(w);
}
