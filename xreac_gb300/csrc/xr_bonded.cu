// Bond orders, bonded energy terms and their hand-written adjoints (FP64).
//
// Forward equations restate src/xreac/energy.py:105-370 (bond orders and corrections, bond,
// lone-pair, over/under-coordination, C2 and triple-bond corrections, valence angle, penalty,
// angle conjugation, torsion, four-body conjugation and hydrogen bonds). Forces are the exact
// derivative of that energy at fixed charges, written by hand in reverse mode: every term kernel
// adds its sensitivities to
//   - per-bond accumulators  dE/d bo, dE/d pi, dE/d pp, dE/d sigma      (thresholded outputs)
//   - per-atom accumulators  dE/d total, dE/d d, dE/d db, dE/d sbo2
//   - atom gradients directly for the angular geometry,
// and the chain kernels then carry those back through the per-atom sums, the bond-order
// correction f1..f5 and the uncorrected bond orders to dE/dr per bond, which lands on the pair's
// radial accumulator. The near-collinear angle rule -1/max(sin, 1e-5) of xreac's fixed-charge
// forces (src/xreac/energy.py:49-55) is reproduced; thresholds are not differentiated, exactly as
// xreac's getval() masks are not.
//
// Layout: bonds are half pairs (each unordered image pair once); dbrow lists, per atom, its
// directed bond edges in canonical order as (bond id, +1 source / -1 target), so per-atom sums
// are gathers in the reference's order and need no atomics.
#include <algorithm>

#include "xr_common.cuh"
#include "xr_dfloat.cuh"  // xr_exp, xr_log: exp and log in double-float arithmetic on the FP32 pipe

namespace {

constexpr double THB_CUT = 0.001;
constexpr double THB_PRODUCT_CUT = 0.00001;
constexpr double HBOND_THRESHOLD = 0.01;

struct Ctx {
  XrWork w;
  XrFF ff;
};

#define AFV(k, a) w.a_fwd[(size_t)(k) * w.A + (a)]
#define AJV(k, a) w.a_adj[(size_t)(k) * w.A + (a)]
#define AEV(k, a) w.a_e[(size_t)(k) * w.A + (a)]
#define BFV(k, b) w.b_fwd[(size_t)(k) * w.cap_B + (b)]
#define BJV(k, b) w.b_adj[(size_t)(k) * w.cap_B + (b)]
#define BEV(k, b) w.b_e[(size_t)(k) * w.cap_B + (b)]

__device__ inline double atom_prm(const XrFF& ff, int t, int col) { return __ldg(ff.atom + t * XR_NATOM_COLS + col); }
__device__ inline double pair_prm(const XrFF& ff, int pt, int col) { return __ldg(ff.pair + pt * XR_NPAIR_COLS + col); }

__device__ inline void atomic_add3(double* f, int a, double gx, double gy, double gz) {
  atomicAdd(f + 3 * a + 0, gx);
  atomicAdd(f + 3 * a + 1, gy);
  atomicAdd(f + 3 * a + 2, gz);
}

// Vector from `atom` to the other end of bond b, for the bond-row entry direction `dir`.
__device__ inline void bond_vec(const XrWork& w, int b, int dir, double v[3]) {
  const double s = (double)dir;
  v[0] = s * w.b_v[0 * w.cap_B + b];
  v[1] = s * w.b_v[1 * w.cap_B + b];
  v[2] = s * w.b_v[2 * w.cap_B + b];
}
__device__ inline int bond_other(const XrWork& w, int b, int dir) { return dir > 0 ? w.bond_j[b] : w.bond_i[b]; }
// Image shift bits of the directed edge for a bond-row entry.
__device__ inline uint32_t bond_shift(const XrWork& w, int b, int dir) {
  const uint32_t c = (uint32_t)w.edge[w.pair_edge[w.bond_pair[b]]].y & XR_SHIFT_MASK;
  return dir > 0 ? c : xr_neg_shift(c);
}

// ------------------------------------------------------------------ uncorrected bond orders
// sigma' = (1+cut) exp(p_bo1 (r/r_s)^p_bo2), pi' = exp(p_bo3 (r/r_p)^p_bo4), pp' likewise;
// raw = sum; active when raw >= cut; bo0 = raw - cut (src/xreac/energy.py:130-149).
// One block-wide tile of bonds b (the whole warp takes part: the active ones are compacted with ballots).
__device__ inline void bo1_tile(const XrWork& w, const XrFF& ff0, int b, int nb) {
  const int lane = threadIdx.x & 31;
  bool mask = false;
  if (b < nb) {
    const int i = w.bond_i[b], j = w.bond_j[b];
    const XrFF ff = xr_ff_of(ff0, w, i);
    const uint32_t code = (uint32_t)w.edge[w.pair_edge[w.bond_pair[b]]].y;
    const XrSystem& S = w.sys[w.sys_of[i]];
    const int sx = xr_sx(code), sy = xr_sy(code), sz = xr_sz(code);
    const double4_32a xi = w.x[i], xj = w.x[j];
    const double xa[3] = {xi.x, xi.y, xi.z}, xb[3] = {xj.x, xj.y, xj.z};
    double v[3];
    const bool shifted = (code & XR_SHIFT_MASK) != xr_pack_shift(0, 0, 0);  // else the offset is zero
    for (int c = 0; c < 3; ++c) {
      v[c] = __dsub_rn(xb[c], xa[c]);
      if (shifted)
        v[c] = __dadd_rn(v[c], __dadd_rn(__dadd_rn(__dmul_rn((double)sx, S.cell[c]), __dmul_rn((double)sy, S.cell[3 + c])),
                                         __dmul_rn((double)sz, S.cell[6 + c])));
    }
    const double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(v[0], v[0]), __dmul_rn(v[1], v[1])), __dmul_rn(v[2], v[2])));
    w.b_r[b] = r;
    w.b_v[0 * w.cap_B + b] = v[0];
    w.b_v[1 * w.cap_B + b] = v[1];
    w.b_v[2 * w.cap_B + b] = v[2];
    const int ti = w.type[i], tj = w.type[j], T = ff.ntypes;
    const int pt = ti * T + tj;
    const double cut = 0.01 * ff.g[29];
    double sig = 0, pi = 0, pp = 0, dsig = 0, dpi = 0, dpp = 0;
    // Beyond the pair type's bound the uncorrected order is below a quarter of the cut: no term is
    // evaluated, the bond is inactive with zero orders (as the full expression would give).
    if (r <= __ldg(ff.pair_rmax + pt)) {
      const double lr = xr_log(r);
      if (atom_prm(ff, ti, A_R_S) > 0 && atom_prm(ff, tj, A_R_S) > 0) {
        const double p1 = pair_prm(ff, pt, P_BO1), p2 = pair_prm(ff, pt, P_BO2);
        const double t = xr_exp(p2 * (lr - __ldg(ff.pair_logr + 3 * pt + 0)));
        sig = (1.0 + cut) * xr_exp(p1 * t);
        dsig = sig * p1 * p2 * t / r;
      }
      if (atom_prm(ff, ti, A_R_PI) > 0 && atom_prm(ff, tj, A_R_PI) > 0) {
        const double p3 = pair_prm(ff, pt, P_BO3), p4 = pair_prm(ff, pt, P_BO4);
        const double t = xr_exp(p4 * (lr - __ldg(ff.pair_logr + 3 * pt + 1)));
        pi = xr_exp(p3 * t);
        dpi = pi * p3 * p4 * t / r;
      }
      if (atom_prm(ff, ti, A_R_PI_PI) > 0 && atom_prm(ff, tj, A_R_PI_PI) > 0) {
        const double p5 = pair_prm(ff, pt, P_BO5), p6 = pair_prm(ff, pt, P_BO6);
        const double t = xr_exp(p6 * (lr - __ldg(ff.pair_logr + 3 * pt + 2)));
        pp = xr_exp(p5 * t);
        dpp = pp * p5 * p6 * t / r;
      }
    }
    const double raw = sig + pi + pp;
    mask = raw >= cut;
    BFV(BF_BO0, b) = mask ? raw - cut : 0.0;
    BFV(BF_PI0, b) = mask ? pi : 0.0;
    BFV(BF_PP0, b) = mask ? pp : 0.0;
    BFV(BF_DSIG, b) = dsig;
    BFV(BF_DPI, b) = dpi;
    BFV(BF_DPP, b) = dpp;
    BFV(BF_MASK, b) = mask ? 1.0 : 0.0;
    if (!mask) {  // the corrected orders of an inactive bond are zero; k_bo2 visits active bonds only
      BFV(BF_BO, b) = 0.0;
      BFV(BF_PI, b) = 0.0;
      BFV(BF_PP, b) = 0.0;
      BFV(BF_SIG, b) = 0.0;
    }
  }
  // active bonds join the list of bonds the per-bond kernels visit (order is irrelevant: each
  // bond's results go to its own slots)
  const unsigned m = __ballot_sync(0xffffffffu, mask);
  int base = 0;
  if (lane == 0 && m) base = atomicAdd(w.nmask, __popc(m));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (mask) w.mlist[base + __popc(m & ((1u << lane) - 1u))] = b;
}

__global__ void k_bo1(XrWork w, XrFF ff0) {
  const int nb = xr_num_bonds(w);
  for (int b0 = blockIdx.x * blockDim.x; b0 < nb; b0 += gridDim.x * blockDim.x)  // uniform per block
    bo1_tile(w, ff0, b0 + threadIdx.x, nb);
}

// Delta'_a = sum of uncorrected bond orders over the atom's directed bond edges, one warp per atom.
// The same pass compacts the entries whose uncorrected order passed the cut into nzrow (canonical
// order kept): every other bond candidate within 5 A has zero bond orders and zero sensitivities,
// so the later per-atom loops visit only these few entries instead of all candidates.
__global__ void k_deltap(XrWork w) {
  const int lane = threadIdx.x & 31;
  const int a = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  if (a >= w.A) return;
  const int L = w.A + 1, beg = w.cnt[3 * L + a], end = w.cnt[3 * L + a + 1];
  double s = 0;
  int n = 0;
  for (int k0 = beg; k0 < end; k0 += 32) {
    const int k = k0 + lane;
    bool keep = false;
    int2 en = make_int2(0, 0);
    if (k < end) {
      en = w.dbrow[k];
      keep = BFV(BF_MASK, en.x) != 0.0;
      if (keep) s += BFV(BF_BO0, en.x);
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (keep) w.nzrow[beg + n + __popc(m & ((1u << lane) - 1u))] = en;
    n += __popc(m);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) {
    AFV(AF_DELTAP, a) = s;
    w.nnz[a] = n;
  }
}

// Corrected bond orders (src/xreac/energy.py:150-165).
__device__ inline void k_bo2_one(const XrWork& w, const XrFF& ff0, int b) {
  const int i = w.bond_i[b], j = w.bond_j[b];
  const XrFF ff = xr_ff_of(ff0, w, i);
  const int ti = w.type[i], tj = w.type[j], T = ff.ntypes, pt = ti * T + tj;
  const double* g = ff.g;
  const double bo0 = BFV(BF_BO0, b), pi0 = BFV(BF_PI0, b), pp0 = BFV(BF_PP0, b);
  const bool mask = BFV(BF_MASK, b) != 0.0;
  const double ovc = pair_prm(ff, pt, P_OVC), v13 = pair_prm(ff, pt, P_V13COR);
  const bool corrected = mask && (ovc >= 0.001 || v13 >= 0.001);
  double boc3 = pair_prm(ff, pt, P_BOC3), boc4 = pair_prm(ff, pt, P_BOC4), boc5 = pair_prm(ff, pt, P_BOC5);
  if (corrected && (!isfinite(boc3) || !isfinite(boc4) || !isfinite(boc5))) atomicOr(w.status, XR_S_BOC_NAN);
  if (!corrected) boc3 = boc4 = boc5 = 0.0;
  const double vi = atom_prm(ff, ti, A_VALENCY), vj = atom_prm(ff, tj, A_VALENCY);
  const double dpi_ = AFV(AF_DELTAP, i), dpj = AFV(AF_DELTAP, j);
  const double di = dpi_ - vi, dj = dpj - vj;
  const double dbi = dpi_ - atom_prm(ff, ti, A_VALENCY_VAL), dbj = dpj - atom_prm(ff, tj, A_VALENCY_VAL);
  double f1 = 1.0, df1i = 0.0, df1j = 0.0;
  if (ovc >= 0.001) {
    const double e2i = xr_exp(-g[0] * di), e2j = xr_exp(-g[0] * dj);
    const double f2 = e2i + e2j;
    const double e3i = xr_exp(-g[1] * di), e3j = xr_exp(-g[1] * dj);
    const double s3 = 0.5 * (e3i + e3j);
    const double f3 = -xr_log(s3) / g[1];
    const double Ai = vi + f2, Bi = Ai + f3, Aj = vj + f2, Bj = Aj + f3;
    f1 = 0.5 * (Ai / Bi + Aj / Bj);
    const double df1_df2 = 0.5 * (f3 / (Bi * Bi) + f3 / (Bj * Bj));
    const double df1_df3 = -0.5 * (Ai / (Bi * Bi) + Aj / (Bj * Bj));
    df1i = df1_df2 * (-g[0] * e2i) + df1_df3 * (0.5 * e3i / s3);
    df1j = df1_df2 * (-g[0] * e2j) + df1_df3 * (0.5 * e3j / s3);
  }
  const double f4 = 1.0 / (1.0 + xr_exp(-(boc4 * bo0 * bo0 - dbi) * boc3 + boc5));
  const double f5 = 1.0 / (1.0 + xr_exp(-(boc4 * bo0 * bo0 - dbj) * boc3 + boc5));
  const double f45 = v13 >= 0.001 ? f4 * f5 : 1.0;
  const double corr = f1 * f45;
  const double bo = bo0 * corr, pi = pi0 * corr * f1, pp = pp0 * corr * f1;
  const double sig = bo - pi - pp;
  BFV(BF_BO, b) = bo >= 1e-10 ? bo : 0.0;
  BFV(BF_PI, b) = pi >= 1e-10 ? pi : 0.0;
  BFV(BF_PP, b) = pp >= 1e-10 ? pp : 0.0;
  BFV(BF_SIG, b) = sig >= 1e-10 ? sig : 0.0;
  BFV(BF_F1, b) = f1;
  BFV(BF_F4, b) = f4;
  BFV(BF_F5, b) = f5;
  BFV(BF_CORR, b) = corr;
  BFV(BF_DF1I, b) = df1i;
  BFV(BF_DF1J, b) = df1j;
}

__global__ void k_bo2(XrWork w, XrFF ff) {
  const int nm = *w.nmask;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nm; q += gridDim.x * blockDim.x)
    k_bo2_one(w, ff, w.mlist[q]);
}

// Per-atom sums of corrected bond orders and the lone-pair quantities
// (src/xreac/energy.py:185-199, 295-296).
__global__ void k_atom1(XrWork w, XrFF ff0) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= w.A) return;
  const XrFF ff = xr_ff_of(ff0, w, a);
  const int L = w.A + 1, T = ff.ntypes, ta = w.type[a];
  const double* g = ff.g;
  double total = 0, sumpi = 0, prodsum = 0, ov1 = 0, n30 = 0;
  const int beg = w.cnt[3 * L + a];
  int nact = 0;
  for (int k = beg; k < beg + w.nnz[a]; ++k) {
    const int2 en = w.nzrow[k];
    const int b = en.x;
    const double bo = BFV(BF_BO, b);
    if (bo > THB_CUT) w.arow[beg + nact++] = en;  // bonded rows of src/xreac/energy.py:220
    total += bo;
    sumpi += BFV(BF_PI, b) + BFV(BF_PP, b);
    const double b2 = bo * bo, b4 = b2 * b2;
    prodsum += b4 * b4;
    const int pt = ta * T + w.type[bond_other(w, b, en.y)];
    ov1 += pair_prm(ff, pt, P_OVUN1) * pair_prm(ff, pt, P_DE_S) * bo;
    n30 += bo > 0.3 ? 1.0 : 0.0;
  }
  const double val = atom_prm(ff, ta, A_VALENCY), vale = atom_prm(ff, ta, A_VALENCY_E);
  const double de = total - vale;
  const double half = trunc(de / 2);
  const double vlpex = de - 2 * half;
  const double e15 = xr_exp(-g[15] * (2 + vlpex) * (2 + vlpex));
  const double nlp = e15 - half;
  const double dlp = 0.5 * (vale - val) - nlp;
  const double dlpt = atom_prm(ff, ta, A_MASS) > 21 ? 0.0 : dlp;
  const double elp = xr_exp(-75 * dlp);
  const double s = 1.0 / (1.0 + elp);
  const double plp2 = atom_prm(ff, ta, A_P_LP2);
  AEV(0, a) = plp2 * dlp * s;
  AJV(AJ_DLP, a) = plp2 * (s + 75.0 * dlp * elp * s * s);
  AFV(AF_TOTAL, a) = total;
  AFV(AF_NLP, a) = nlp;
  AFV(AF_VLPEX, a) = vlpex;
  AFV(AF_DLP, a) = dlp;
  AFV(AF_DLPT, a) = dlpt;
  AFV(AF_SUMPI, a) = sumpi;
  AFV(AF_PROD, a) = xr_exp(-prodsum);
  AFV(AF_OV1, a) = ov1;
  AFV(AF_COUNT30, a) = n30;
  AFV(AF_E15, a) = e15;
  w.nact[a] = nact;
}

__device__ inline double sbo2_of(double sbo, double p) {
  if (sbo <= 0) return 0.0;
  if (sbo <= 1) return xr_exp(p * xr_log(sbo));
  if (sbo < 2) return 2.0 - xr_exp(p * xr_log(2.0 - sbo));
  return 2.0;
}
__device__ inline double dsbo2_of(double sbo, double p) {
  if (sbo <= 0) return 0.0;
  if (sbo <= 1) return p * xr_exp((p - 1) * xr_log(sbo));
  if (sbo < 2) return p * xr_exp((p - 1) * xr_log(2.0 - sbo));
  return 0.0;
}

// Over/under-coordination and sbo (src/xreac/energy.py:201-212, 295-301), with their local adjoints.
__global__ void k_atom2(XrWork w, XrFF ff0) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= w.A) return;
  const XrFF ff = xr_ff_of(ff0, w, a);
  const int L = w.A + 1, ta = w.type[a];
  const double* g = ff.g;
  const double dfvl = atom_prm(ff, ta, A_MASS) <= 21 ? 1.0 : 0.0;
  double ov2 = 0;
  for (int k = w.cnt[3 * L + a]; k < w.cnt[3 * L + a] + w.nnz[a]; ++k) {
    const int2 en = w.nzrow[k];
    const int b = en.x, j = bond_other(w, b, en.y);
    const double dj = AFV(AF_TOTAL, j) - atom_prm(ff, w.type[j], A_VALENCY);
    ov2 += (dj - dfvl * AFV(AF_DLPT, j)) * (BFV(BF_PI, b) + BFV(BF_PP, b));
  }
  const double total = AFV(AF_TOTAL, a), val = atom_prm(ff, ta, A_VALENCY);
  const double d = total - val, db = total - atom_prm(ff, ta, A_VALENCY_BOC);
  const double dlpt = AFV(AF_DLPT, a), ov1 = AFV(AF_OV1, a);
  const double exov = xr_exp(g[31] * ov2);
  const double denc = 1.0 + g[32] * exov;
  const double dc = d - dfvl * dlpt / denc;
  const double po2 = atom_prm(ff, ta, A_P_OVUN2), p5 = atom_prm(ff, ta, A_P_OVUN5);
  const double D1 = dc + val + 1e-8;
  const double eo = xr_exp(po2 * dc);
  const double D2 = 1.0 + eo;
  const double over = ov1 * dc / D1 / D2;
  const double eu = xr_exp(g[6] * dc), em = xr_exp(-po2 * dc), e9 = xr_exp(g[9] * ov2);
  const double D3 = 1.0 + em, D4 = 1.0 + g[8] * e9;
  const double under = -p5 * (1.0 - eu) / D3 / D4;
  AEV(1, a) = over + under;
  const double dover_ddc = ov1 * (1.0 / (D1 * D2) - dc / (D1 * D1 * D2) - dc * po2 * eo / (D1 * D2 * D2));
  const double dunder_ddc = -p5 * (-g[6] * eu / (D3 * D4) + (1.0 - eu) * po2 * em / (D3 * D3 * D4));
  const double dunder_dov2 = -under * g[8] * g[9] * e9 / D4;
  const double A_dc = dover_ddc + dunder_ddc;
  AJV(AJ_OV1, a) = dc / (D1 * D2);
  AJV(AJ_OV2, a) = A_dc * dfvl * dlpt * g[32] * g[31] * exov / (denc * denc) + dunder_dov2;
  AJV(AJ_D, a) += A_dc;
  AJV(AJ_DLPT, a) = A_dc * (-dfvl / denc);
  const double vlpex = AFV(AF_VLPEX, a), nlp = AFV(AF_NLP, a), prod = AFV(AF_PROD, a);
  const double lpt = vlpex >= 0 ? 0.0 : nlp;
  const double sbo = AFV(AF_SUMPI, a) + (1.0 - prod) * (-db - g[33] * lpt);
  AFV(AF_OV2, a) = ov2;
  AFV(AF_DC, a) = dc;
  AFV(AF_SBO, a) = sbo;
  AFV(AF_SBO2, a) = sbo2_of(sbo, g[16]);
}

// Bond energy, C2 correction and triple-bond stabilisation, per half bond
// (src/xreac/energy.py:194-198, 231-246).
__device__ inline void k_bond_energy_one(const XrWork& w, const XrFF& ff0, int b) {
  const int i = w.bond_i[b], j = w.bond_j[b];
  const XrFF ff = xr_ff_of(ff0, w, i);
  const int ti = w.type[i], tj = w.type[j], T = ff.ntypes, pt = ti * T + tj;
  const double* g = ff.g;
  const double bo = BFV(BF_BO, b), pi = BFV(BF_PI, b), pp = BFV(BF_PP, b), sig = BFV(BF_SIG, b);
  const double Des = pair_prm(ff, pt, P_DE_S), Dep = pair_prm(ff, pt, P_DE_P), Depp = pair_prm(ff, pt, P_DE_PP);
  const double be1 = pair_prm(ff, pt, P_BE1), be2 = pair_prm(ff, pt, P_BE2);
  const double powv = sig > 0 ? xr_exp(be2 * xr_log(sig)) : 0.0;
  const double ex = xr_exp(be1 * (1.0 - powv));
  double e_bond = -(Des * sig * ex + Dep * pi + Depp * pp);
  BJV(BJ_SIG, b) = -Des * ex * (1.0 - be1 * be2 * powv);
  if (w.pgrad) {  // dE/d(De_s, De_p, De_pp, p_be1, p_be2)
    double* gp = xr_pgrad(w, i) + (size_t)pt * XR_NPAIR_COLS;
    atomicAdd(gp + P_DE_S, -sig * ex);
    if (pi != 0.0) atomicAdd(gp + P_DE_P, -pi);
    if (pp != 0.0) atomicAdd(gp + P_DE_PP, -pp);
    if (sig > 0) {
      atomicAdd(gp + P_BE1, -Des * sig * ex * (1.0 - powv));
      atomicAdd(gp + P_BE2, Des * sig * ex * be1 * powv * xr_log(sig));
    }
  }
  BJV(BJ_PI, b) += -Dep;
  BJV(BJ_PP, b) += -Depp;
  double e_c2 = 0.0, dbo = 0.0;
  if (g[5] > 0.001 && __ldg(ff.is_carbon + ti) && __ldg(ff.is_carbon + tj)) {
    const int ends[2] = {i, j};
    for (int s = 0; s < 2; ++s) {
      const int src = ends[s];
      const double d = AFV(AF_TOTAL, src) - atom_prm(ff, w.type[src], A_VALENCY);
      const double d2 = d * d;
      const double vov3 = bo - d - 0.040 * d2 * d2;
      if (vov3 > 3) {
        e_c2 += g[5] * (vov3 - 3) * (vov3 - 3);
        dbo += 2 * g[5] * (vov3 - 3);
        atomicAdd(&AJV(AJ_D, src), 2 * g[5] * (vov3 - 3) * (-1.0 - 0.16 * d2 * d));
      }
    }
  }
  const double mi = atom_prm(ff, ti, A_MASS), mj = atom_prm(ff, tj, A_MASS);
  const bool co = (mi == 12.0 && mj == 15.999) || (mj == 12.0 && mi == 15.999);
  const bool allowed = ((int)g[37] != 2) ? co : true;
  if (allowed && bo >= 1.0) {
    const double ti_ = AFV(AF_TOTAL, i), tj_ = AFV(AF_TOTAL, j);
    const double di = ti_ - atom_prm(ff, ti, A_VALENCY), dj = tj_ - atom_prm(ff, tj, A_VALENCY);
    const double e1 = xr_exp(-g[7] * (bo - 2.5) * (bo - 2.5));
    const double e4 = xr_exp(g[4] * (di + dj));
    const double D = 1.0 + 25.0 * e4;
    const double ei = xr_exp(-g[3] * (ti_ - bo)), ej = xr_exp(-g[3] * (tj_ - bo));
    const double stab = g[10] * e1 / D * (ei + ej);
    e_bond += stab;
    dbo += g[10] / D * (-2.0 * g[7] * (bo - 2.5) * e1 * (ei + ej) + e1 * g[3] * (ei + ej));
    const double dd = -g[10] * e1 * (ei + ej) * 25.0 * g[4] * e4 / (D * D);
    atomicAdd(&AJV(AJ_D, i), dd);
    atomicAdd(&AJV(AJ_D, j), dd);
    atomicAdd(&AJV(AJ_TOTAL, i), g[10] * e1 / D * (-g[3] * ei));
    atomicAdd(&AJV(AJ_TOTAL, j), g[10] * e1 / D * (-g[3] * ej));
  }
  if (dbo != 0.0) atomicAdd(&BJV(BJ_BO, b), dbo);
  BEV(0, b) = e_bond;
  BEV(1, b) = e_c2;
}

__global__ void k_bond_energy(XrWork w, XrFF ff) {
  const int nm = *w.nmask;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nm; q += gridDim.x * blockDim.x)
    k_bond_energy_one(w, ff, w.mlist[q]);
}

// ---------------------------------------------------------------------------------------------
// Many-body terms as compacted work items. A warp owns a chunk of kUnits units (valence centres or
// torsion middles). It enumerates the units' (left, right) combinations, keeps those that pass the
// cheap tests (bond-order product, parameter row), compacts them into shared memory with ballots
// and evaluates them 32 at a time, one per lane. An FP64 instruction occupies this part's FP64 pipe
// for the whole warp however few lanes are active, so a warp per centre (a handful of combinations)
// would spend most of the pipe on idle lanes. Per-unit sums (energies, the unit's own adjoints and
// force) are formed by a segmented warp reduction over the contiguous items of each unit, in lane
// and pass order, so energies are deterministic; contributions to other atoms and bonds use atomics.
constexpr int kUnits = 8;          // units per warp chunk
constexpr int kItemBuf = 64;       // per-warp item buffer: at most 31 left over + 32 new
constexpr int kBondedWarps = 4;    // warps per block of the item kernels

__device__ inline uint32_t pack_item(int u, int a, int c) { return ((uint32_t)u << 28) | ((uint32_t)a << 14) | (uint32_t)c; }
__device__ inline int item_unit(uint32_t it) { return (int)(it >> 28); }
__device__ inline int item_a(uint32_t it) { return (int)((it >> 14) & 16383u); }
__device__ inline int item_c(uint32_t it) { return (int)(it & 16383u); }

// Segmented sum over lanes whose items belong to the same unit (items of a unit are contiguous in
// lane order); the unit's first lane adds the sum into uacc[unit][*]. key < 0 marks an empty lane.
template <int NV>
__device__ inline void unit_sums(double (&v)[NV], int key, double* uacc) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int ko = __shfl_down_sync(0xffffffffu, key, o);
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const double t = __shfl_down_sync(0xffffffffu, v[k], o);
      if (lane + o < 32 && ko == key) v[k] += t;
    }
  }
  const int kp = __shfl_up_sync(0xffffffffu, key, 1);
  if (key >= 0 && (lane == 0 || kp != key))
#pragma unroll
    for (int k = 0; k < NV; ++k) uacc[key * NV + k] += v[k];
  __syncwarp();
}

// Appends the items flagged by `ok` to the warp's buffer and runs `process` on full batches of 32.
template <class Proc>
__device__ inline void push_items(uint32_t* buf, int& nbuf, bool ok, uint32_t item, Proc& process) {
  const int lane = threadIdx.x & 31;
  const unsigned m = __ballot_sync(0xffffffffu, ok);
  if (ok) buf[nbuf + __popc(m & ((1u << lane) - 1u))] = item;
  nbuf += __popc(m);
  __syncwarp();
  if (nbuf >= 32) {
    process(buf[lane], true);
    nbuf -= 32;
    const uint32_t moved = lane < nbuf ? buf[32 + lane] : 0u;
    __syncwarp();
    if (lane < nbuf) buf[lane] = moved;
    __syncwarp();
  }
}

// Valence angle, penalty and coalition terms (src/xreac/energy.py:278-318 with the angle rule of
// src/xreac/energy.py:49-55): units are centres j, items the pairs of j's active bonds.
__global__ void __launch_bounds__(32 * kBondedWarps) k_angles(XrWork w, XrFF ff0) {
  constexpr int NC = 8, NV = 10;
  __shared__ double ucon[kBondedWarps][kUnits][NC];
  __shared__ double uacc[kBondedWarps][kUnits][NV];
  __shared__ int ubeg[kBondedWarps][kUnits], ucnt[kBondedWarps][kUnits];
  __shared__ uint32_t buf[kBondedWarps][kItemBuf];
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  const int chunk = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  const int j0 = chunk * kUnits;
  if (j0 >= w.A) return;
  const int nu = min(kUnits, w.A - j0);
  const int L = w.A + 1, T = ff0.ntypes;
  const double* g = ff0.g;
  const bool lammps = !w.full_derivative;
  const double k180 = 3.14159265 / 180;
  // unit constants, one centre per lane
  if (lane < nu) {
    const int j = j0 + lane, tj = w.type[j];
    const XrFF ff = xr_ff_of(ff0, w, j);
    const double total_j = AFV(AF_TOTAL, j);
    const double d_j = total_j - atom_prm(ff, tj, A_VALENCY);
    const double sbo2 = AFV(AF_SBO2, j);
    const double ex3 = xr_exp(-g[20] * d_j), ex4 = xr_exp(g[21] * d_j);
    const double den34 = 1 + ex3 + ex4;
    const double e2 = xr_exp(g[2] * (total_j - atom_prm(ff, tj, A_VALENCY_VAL)));
    const double K1 = 1.0 / (1.0 + e2);
    double* cj = ucon[wl][lane];
    cj[0] = xr_exp(-g[17] * (2 - sbo2));
    cj[1] = (2 + ex3) / den34;
    cj[2] = (-g[20] * ex3 * den34 - (2 + ex3) * (-g[20] * ex3 + g[21] * ex4)) / (den34 * den34);
    cj[3] = K1;
    cj[4] = -g[2] * e2 * K1 * K1;
    cj[5] = total_j - atom_prm(ff, tj, A_VALENCY_BOC);
    cj[6] = atom_prm(ff, tj, A_P_VAL3);
    cj[7] = atom_prm(ff, tj, A_P_VAL5);
    ubeg[wl][lane] = w.cnt[3 * L + j];
    ucnt[wl][lane] = w.nact[j];
    if (w.nact[j] > 16383) atomicOr(w.status, XR_S_LIMIT);
#pragma unroll
    for (int k = 0; k < NV; ++k) uacc[wl][lane][k] = 0.0;
  }
  __syncwarp();
  double* acc = &uacc[wl][0][0];
  auto process = [&](uint32_t it, bool valid) {
    double v[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = 0.0;
    int key = -1;
    if (valid) {
      const int u = item_unit(it), a = item_a(it), c = item_c(it);
      key = u;
      const int j = j0 + u, tj = w.type[j];
      const XrFF ff = xr_ff_of(ff0, w, j);
      const double* cj = ucon[wl][u];
      const double e17 = cj[0], Fp = cj[1], dFp_dd = cj[2], K1 = cj[3], dK1_dt = cj[4], db_j = cj[5];
      const double pv3 = cj[6], pv5 = cj[7];
      const int2 ea = w.arow[ubeg[wl][u] + a], ec = w.arow[ubeg[wl][u] + c];
      const double bo_l = BFV(BF_BO, ea.x), bo_r = BFV(BF_BO, ec.x);
      const int i = bond_other(w, ea.x, ea.y), k = bond_other(w, ec.x, ec.y);
      const int key3 = (w.type[i] * T + tj) * T + w.type[k];
      const int first = __ldg(ff.angle_index + 2 * key3), count = __ldg(ff.angle_index + 2 * key3 + 1);
      double vl[3], vr[3];
      bond_vec(w, ea.x, ea.y, vl);
      bond_vec(w, ec.x, ec.y, vr);
      const double irl = 1.0 / w.b_r[ea.x], irr = 1.0 / w.b_r[ec.x];
      const double total_i = AFV(AF_TOTAL, i), total_k = AFV(AF_TOTAL, k);
      const double inv = irl * irr;
      const double cosv = (vl[0] * vr[0] + vl[1] * vr[1] + vl[2] * vr[2]) * inv;
      double theta, dth_dcos;
      if (lammps) {
        const double cc = fmin(fmax(cosv, -1.0), 1.0);
        theta = acos(cc);
        dth_dcos = -1.0 / fmax(sin(theta), 1e-5);
      } else {
        const double lo = -1 + 1e-14, hi = 1 - 1e-14;
        const double cc = fmin(fmax(cosv, lo), hi);
        theta = acos(cc);
        dth_dcos = (cosv > lo && cosv < hi) ? -1.0 / sqrt(1.0 - cc * cc) : 0.0;
      }
      const double bij = bo_l - THB_CUT, bjk = bo_r - THB_CUT;
      const double lbij = xr_log(bij), lbjk = xr_log(bjk);
      const double ibij = 1.0 / bij, ibjk = 1.0 / bjk;
      // terms that do not depend on the parameter record
      const double ti_b = total_i - bij, tk_b = total_k - bjk;
      double dE_dcos = 0, dbij = 0, dbjk = 0, dtot_i = 0, dtot_k = 0;
      for (int q = 0; q < count; ++q) {
        const double* prm = ff.angle + 7 * (first + q);
        const double th00 = __ldg(prm + 0), v1 = __ldg(prm + 1), v2 = __ldg(prm + 2), coa1 = __ldg(prm + 3);
        const double v7 = __ldg(prm + 4), pen1 = __ldg(prm + 5), v4 = __ldg(prm + 6);
        if (!(fabs(v1) > 0.001)) continue;
        const double theta0 = (180 - th00 * (1 - e17)) * k180;
        const double dth0_dsbo2 = th00 * k180 * g[17] * e17;
        const double pij = xr_exp(v4 * lbij), pjk = xr_exp(v4 * lbjk);
        const double A1 = xr_exp(-pv3 * pij), A2 = xr_exp(-pv3 * pjk);
        const double f7 = (1 - A1) * (1 - A2);
        const double df7_dbij = pv3 * v4 * pij * ibij * A1 * (1 - A2);
        const double df7_dbjk = (1 - A1) * pv3 * v4 * pjk * ibjk * A2;
        const double ex6 = xr_exp(g[14] * db_j), ex7 = xr_exp(-v7 * db_j);
        const double den8 = 1 + ex6 + ex7;
        const double f8 = pv5 - (pv5 - 1) * (2 + ex6) / den8;
        const double df8_ddb = -(pv5 - 1) * (g[14] * ex6 * den8 - (2 + ex6) * (g[14] * ex6 - v7 * ex7)) / (den8 * den8);
        const double dt = theta0 - theta;
        const double exang = xr_exp(-v2 * dt * dt);
        const double branch = v1 >= 0 ? 1 - exang : -exang;
        v[0] += f7 * f8 * v1 * branch;
        const double dE_ddt = f7 * f8 * v1 * 2 * v2 * dt * exang;
        dE_dcos += -dE_ddt * dth_dcos;
        v[3] += dE_ddt * dth0_dsbo2;
        dbij += f8 * v1 * branch * df7_dbij;
        dbjk += f8 * v1 * branch * df7_dbjk;
        v[4] += f7 * v1 * branch * df8_ddb;
        const double Gp = xr_exp(-g[19] * ((bij - 2) * (bij - 2) + (bjk - 2) * (bjk - 2)));
        const double ep = pen1 * Fp * Gp;
        if (w.pgrad) {
          // dE/d(theta00, v1, v2, coa1, v7, pen1, v4) of this record
          double* ga = xr_pgrad(w, j) + w.pgrad_angle_off + 7 * (size_t)(first + q);
          const double sgn_dt2 = dt * dt * exang;  // d branch / d v2 (either sign of v1)
          const double df7_dv4 = pv3 * pij * lbij * A1 * (1 - A2) + (1 - A1) * pv3 * pjk * lbjk * A2;
          const double df8_dv7 = (pv5 - 1) * (2 + ex6) / (den8 * den8) * (-db_j * ex7);
          atomicAdd(ga + 0, dE_ddt * (-(1 - e17) * k180));
          atomicAdd(ga + 1, f7 * f8 * branch);
          atomicAdd(ga + 2, f7 * f8 * v1 * sgn_dt2);
          atomicAdd(ga + 4, f7 * v1 * branch * df8_dv7);
          atomicAdd(ga + 5, Fp * Gp);
          atomicAdd(ga + 6, f8 * v1 * branch * df7_dv4);
        }
        v[1] += ep;
        v[5] += pen1 * dFp_dd * Gp;
        dbij += ep * (-2 * g[19] * (bij - 2));
        dbjk += ep * (-2 * g[19] * (bjk - 2));
        const double K2 = xr_exp(-g[38] * (ti_b * ti_b + tk_b * tk_b));
        const double K3 = xr_exp(-g[30] * ((bij - 1.5) * (bij - 1.5) + (bjk - 1.5) * (bjk - 1.5)));
        const double ec_ = coa1 * K1 * K2 * K3;
        if (w.pgrad) atomicAdd(xr_pgrad(w, j) + w.pgrad_angle_off + 7 * (size_t)(first + q) + 3, K1 * K2 * K3);
        v[2] += ec_;
        v[6] += coa1 * dK1_dt * K2 * K3;
        dtot_i += ec_ * (-2 * g[38] * ti_b);
        dtot_k += ec_ * (-2 * g[38] * tk_b);
        dbij += ec_ * (2 * g[38] * ti_b) + ec_ * (-2 * g[30] * (bij - 1.5));
        dbjk += ec_ * (2 * g[38] * tk_b) + ec_ * (-2 * g[30] * (bjk - 1.5));
      }
      if (dE_dcos != 0.0) {
        double gl[3], gr[3];
        for (int c3 = 0; c3 < 3; ++c3) {
          gl[c3] = dE_dcos * (vr[c3] * inv - cosv * vl[c3] * irl * irl);
          gr[c3] = dE_dcos * (vl[c3] * inv - cosv * vr[c3] * irr * irr);
          v[7 + c3] = -(gl[c3] + gr[c3]);
        }
        atomic_add3(w.f, i, gl[0], gl[1], gl[2]);
        atomic_add3(w.f, k, gr[0], gr[1], gr[2]);
      }
      if (dbij != 0.0) atomicAdd(&BJV(BJ_BO, ea.x), dbij);
      if (dbjk != 0.0) atomicAdd(&BJV(BJ_BO, ec.x), dbjk);
      if (dtot_i != 0.0) atomicAdd(&AJV(AJ_TOTAL, i), dtot_i);
      if (dtot_k != 0.0) atomicAdd(&AJV(AJ_TOTAL, k), dtot_k);
    }
    unit_sums<NV>(v, key, acc);
  };
  int nbuf = 0;
  for (int u = 0; u < nu; ++u) {
    const int m = ucnt[wl][u], beg = ubeg[wl][u];
    const int tj = w.type[j0 + u];
    const int npairs = m * (m - 1) / 2;
    for (int t0 = 0; t0 < npairs; t0 += 32) {
      const int t = t0 + lane;
      bool ok = false;
      uint32_t item = 0;
      if (t < npairs) {
        int a = 0, rem = t;
        while (rem >= m - 1 - a) {
          rem -= m - 1 - a;
          ++a;
        }
        const int c = a + 1 + rem;
        const int2 ea = w.arow[beg + a], ec = w.arow[beg + c];
        if (BFV(BF_BO, ea.x) * BFV(BF_BO, ec.x) > THB_PRODUCT_CUT) {
          const int i = bond_other(w, ea.x, ea.y), k = bond_other(w, ec.x, ec.y);
          const int key3 = (w.type[i] * T + tj) * T + w.type[k];
          ok = __ldg(ff0.angle_index + 2 * key3 + 1) > 0;
        }
        item = pack_item(u, a, c);
      }
      push_items(buf[wl], nbuf, ok, item, process);
    }
  }
  if (nbuf > 0) process(buf[wl][lane], lane < nbuf);
  if (lane < nu) {
    const int j = j0 + lane;
    const double* s = uacc[wl][lane];
    AEV(2, j) = s[0];
    AEV(3, j) = s[1];
    AEV(4, j) = s[2];
    if (s[3] != 0.0) atomicAdd(&AJV(AJ_SBO2, j), s[3]);
    if (s[4] != 0.0) atomicAdd(&AJV(AJ_DB, j), s[4]);
    if (s[5] != 0.0) atomicAdd(&AJV(AJ_D, j), s[5]);
    if (s[6] != 0.0) atomicAdd(&AJV(AJ_TOTAL, j), s[6]);
    if (s[7] != 0.0 || s[8] != 0.0 || s[9] != 0.0) atomic_add3(w.f, j, s[7], s[8], s[9]);
  }
}

__device__ inline void cross3(const double a[3], const double b[3], double c[3]) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

// Bonds with bo > 0.001 (the middles of torsion chains), compacted in bond order: the count of every
// tile of kMidTile bonds (k_mid_count), an exclusive scan of the tile counts in one block
// (k_mid_scan, which also stores the total in nmids), then each tile's middles at its offset
// (k_mid_fill). The order of mids decides which middles a warp of k_torsions takes together, and with
// that how each middle's items fall into the warp's batches of 32, i.e. the order in which they are
// summed: a fixed order keeps the torsion and conjugation energies the same bit for bit on every
// call. Launched with 128-thread blocks.
constexpr int kMidTile = 128;

__global__ void k_mid_count(XrWork w) {
  __shared__ int wc[kMidTile / 32];
  const int nb = xr_num_bonds(w), ntiles = (nb + kMidTile - 1) / kMidTile;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int b = t * kMidTile + threadIdx.x;
    const bool keep = b < nb && BFV(BF_BO, b) > THB_CUT;
    if (b < nb && !keep) {
      BEV(2, b) = 0.0;
      BEV(3, b) = 0.0;
    }
    const unsigned msk = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) wc[wid] = __popc(msk);
    __syncthreads();
    if (threadIdx.x == 0) {
      int c = 0;
      for (int k = 0; k < kMidTile / 32; ++k) c += wc[k];
      w.mid_tiles[t] = c;
    }
    __syncthreads();
  }
}

__global__ void k_mid_scan(XrWork w) {  // one block of 1024 threads
  __shared__ int part[32];
  __shared__ int carry_s;
  const int nb = xr_num_bonds(w), ntiles = (nb + kMidTile - 1) / kMidTile;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry_s = 0;
  __syncthreads();
  for (int base = 0; base < ntiles; base += blockDim.x) {
    const int t = base + threadIdx.x;
    const int v = t < ntiles ? w.mid_tiles[t] : 0;
    int x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, d);
      if (lane >= d) x += y;
    }
    if (lane == 31) part[wid] = x;
    __syncthreads();
    if (wid == 0) {
      const int p = part[lane];
      int q = p;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, q, d);
        if (lane >= d) q += y;
      }
      part[lane] = q - p;  // exclusive over warps
    }
    __syncthreads();
    const int carry = carry_s;
    if (t < ntiles) w.mid_tiles[t] = carry + part[wid] + x - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry_s = carry + part[wid] + x;
    __syncthreads();
  }
  if (threadIdx.x == 0) *w.nmids = carry_s;
}

__global__ void k_mid_fill(XrWork w) {
  __shared__ int wc[kMidTile / 32];
  const int nb = xr_num_bonds(w), ntiles = (nb + kMidTile - 1) / kMidTile;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int b = t * kMidTile + threadIdx.x;
    const bool keep = b < nb && BFV(BF_BO, b) > THB_CUT;
    const unsigned msk = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) wc[wid] = __popc(msk);
    __syncthreads();
    int off = w.mid_tiles[t];
    for (int k = 0; k < wid; ++k) off += wc[k];
    if (keep) w.mids[off + __popc(msk & ((1u << lane) - 1u))] = b;
    __syncthreads();
  }
}

// Torsion and four-body conjugation (src/xreac/energy.py:320-370): units are middle bonds j -> k
// (the half direction), items the (left, right) combinations of the two ends' active bond rows.
__global__ void __launch_bounds__(32 * kBondedWarps) k_torsions(XrWork w, XrFF ff0) {
  constexpr int NC = 10, NV = 11;
  struct UnitInt {
    int m, j, k, tj, tk, jb, kb, jn, kn;
    uint32_t sm;
  };
  __shared__ double ucon[kBondedWarps][kUnits][NC];
  __shared__ double uacc[kBondedWarps][kUnits][NV];
  __shared__ UnitInt uint_[kBondedWarps][kUnits];
  __shared__ uint32_t buf[kBondedWarps][kItemBuf];
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  const int warp = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
  const int T = ff0.ntypes;
  const int L = w.A + 1;
  const double* g = ff0.g;
  const int nm = *w.nmids;
  double* acc = &uacc[wl][0][0];
  for (int q0 = warp * kUnits; q0 < nm; q0 += nwarps * kUnits) {
    const int nu = min(kUnits, nm - q0);
    if (lane < nu) {
      UnitInt& ui = uint_[wl][lane];
      const int m = w.mids[q0 + lane];
      const int j = w.bond_i[m], k = w.bond_j[m];
      const int tj = w.type[j], tk = w.type[k];
      const XrFF ff = xr_ff_of(ff0, w, j);
      ui.m = m;
      ui.j = j;
      ui.k = k;
      ui.tj = tj;
      ui.tk = tk;
      ui.jb = w.cnt[3 * L + j];
      ui.kb = w.cnt[3 * L + k];
      ui.jn = w.nact[j];
      ui.kn = w.nact[k];
      if (ui.jn > 16383 || ui.kn > 16383) atomicOr(w.status, XR_S_LIMIT);
      ui.sm = (uint32_t)w.edge[w.pair_edge[w.bond_pair[m]]].y & XR_SHIFT_MASK;
      double* cm = ucon[wl][lane];
      double v[3];
      bond_vec(w, m, 1, v);
      const double db_j = AFV(AF_TOTAL, j) - atom_prm(ff, tj, A_VALENCY_BOC);
      const double db_k = AFV(AF_TOTAL, k) - atom_prm(ff, tk, A_VALENCY_BOC);
      const double ds = db_j + db_k;
      const double ex3 = xr_exp(-g[24] * ds), ex4 = xr_exp(g[25] * ds);
      const double den = 1 + ex3 + ex4;
      const double b2 = BFV(BF_BO, m) - THB_CUT;
      cm[0] = v[0];
      cm[1] = v[1];
      cm[2] = v[2];
      cm[3] = w.b_r[m];
      cm[4] = BFV(BF_PI, m);
      cm[5] = (2 + ex3) / den;  // f11
      cm[6] = (-g[24] * ex3 * den - (2 + ex3) * (-g[24] * ex3 + g[25] * ex4)) / (den * den);
      cm[7] = b2;
      cm[8] = xr_exp(-g[23] * b2);
      cm[9] = BFV(BF_BO, m);
#pragma unroll
      for (int c = 0; c < NV; ++c) uacc[wl][lane][c] = 0.0;
    }
    __syncwarp();
    auto process = [&](uint32_t it, bool valid) {
      double acc_v[NV];
#pragma unroll
      for (int c = 0; c < NV; ++c) acc_v[c] = 0.0;
      int key = -1;
      if (valid) {
        const int u = item_unit(it);
        key = u;
        const UnitInt& ui = uint_[wl][u];
        const double* cm = ucon[wl][u];
        const double v[3] = {cm[0], cm[1], cm[2]};
        const double rm = cm[3], pi_m = cm[4], f11 = cm[5], df11_dds = cm[6], b2 = cm[7], e2 = cm[8];
        const int2 el = w.arow[ui.jb + item_a(it)];
        const int2 er = w.arow[ui.kb + item_c(it)];
        const double bo_l = BFV(BF_BO, el.x), bo_r = BFV(BF_BO, er.x);
        const int i = bond_other(w, el.x, el.y), l = bond_other(w, er.x, er.y);
        const int row = __ldg(ff0.torsion_index + ((w.type[i] * T + ui.tj) * T + ui.tk) * T + w.type[l]);
        double u3[3], wv[3];
        bond_vec(w, el.x, el.y, u3);
        bond_vec(w, er.x, er.y, wv);
        const double rl = w.b_r[el.x], rr = w.b_r[er.x];
        double n1[3], n2[3];
        cross3(u3, v, n1);
        cross3(wv, v, n2);
        const double A1 = n1[0] * n1[0] + n1[1] * n1[1] + n1[2] * n1[2];
        const double A2 = n2[0] * n2[0] + n2[1] * n2[1] + n2[2] * n2[2];
        const double s1 = A1 / ((rl * rm) * (rl * rm));
        const double s2 = A2 / ((rm * rr) * (rm * rr));
        if (s1 < 1e-20 || s2 < 1e-20) {
          atomicOr(w.status, XR_S_COLLINEAR);
        } else {
          const double sinprod = sqrt(s1 * s2);
          const double isq = 1.0 / sqrt(A1 * A2);
          const double iA1 = 1.0 / A1, iA2 = 1.0 / A2;
          const double P = n1[0] * n2[0] + n1[1] * n2[1] + n1[2] * n2[2];
          const double cw = P * isq;
          const double* prm = xr_ff_of(ff0, w, ui.j).torsion + 5 * row;
          const double V1 = __ldg(prm + 0), V2 = __ldg(prm + 1), V3 = __ldg(prm + 2), tor1 = __ldg(prm + 3),
                       cot1 = __ldg(prm + 4);
          const double b1 = bo_l - THB_CUT, b3 = bo_r - THB_CUT;
          const double e1 = xr_exp(-g[23] * b1), e3 = xr_exp(-g[23] * b3);
          const double y = 2 - pi_m - f11;
          const double ex1 = xr_exp(tor1 * y * y);
          const double fn10 = (1 - e1) * (1 - e2) * (1 - e3);
          const double cv = 0.5 * (V1 * (1 + cw) + V2 * ex1 * (2 - 2 * cw * cw) + V3 * (1 + 4 * cw * cw * cw - 3 * cw));
          acc_v[0] = fn10 * sinprod * cv;
          const double q1 = b1 - 1.5, q2 = b2 - 1.5, q3 = b3 - 1.5;
          const double fn12 = xr_exp(-g[27] * (q1 * q1 + q2 * q2 + q3 * q3));
          const double conj = 1 + (cw * cw - 1) * sinprod;
          acc_v[1] = cot1 * fn12 * conj;
          const double dcv_dcw = 0.5 * (V1 - 4 * V2 * ex1 * cw + V3 * (12 * cw * cw - 3));
          const double dE_dcw = fn10 * sinprod * dcv_dcw + cot1 * fn12 * 2 * cw * sinprod;
          const double dE_dsp = fn10 * cv + cot1 * fn12 * (cw * cw - 1);
          const double dE_dex1 = fn10 * sinprod * 0.5 * V2 * (2 - 2 * cw * cw);
          const double dex1_dy = 2 * tor1 * y * ex1;
          acc_v[3] = -dE_dex1 * dex1_dy;             // pi of the middle
          acc_v[4] = -dE_dex1 * dex1_dy * df11_dds;  // db of both ends
          const double sc = sinprod * cv, cc = cot1 * conj;
          const double A_bol = sc * g[23] * e1 * (1 - e2) * (1 - e3) + cc * fn12 * (-2 * g[27] * q1);
          acc_v[2] = sc * g[23] * e2 * (1 - e1) * (1 - e3) + cc * fn12 * (-2 * g[27] * q2);
          const double A_bor = sc * g[23] * e3 * (1 - e1) * (1 - e2) + cc * fn12 * (-2 * g[27] * q3);
          atomicAdd(&BJV(BJ_BO, el.x), A_bol);
          atomicAdd(&BJV(BJ_BO, er.x), A_bor);
          double av[3], bv[3];
          for (int c3 = 0; c3 < 3; ++c3) {
            av[c3] = dE_dcw * (n2[c3] - (P * iA1) * n1[c3]) * isq + dE_dsp * sinprod * n1[c3] * iA1;
            bv[c3] = dE_dcw * (n1[c3] - (P * iA2) * n2[c3]) * isq + dE_dsp * sinprod * n2[c3] * iA2;
          }
          double gu[3], gv[3], gw[3], t1[3], t2[3];
          cross3(v, av, gu);
          cross3(av, u3, t1);
          cross3(bv, wv, t2);
          cross3(v, bv, gw);
          const double irl2 = 1.0 / (rl * rl), irm2 = 1.0 / (rm * rm), irr2 = 1.0 / (rr * rr);
          for (int c3 = 0; c3 < 3; ++c3) {
            gu[c3] += dE_dsp * (-sinprod) * u3[c3] * irl2;
            gv[c3] = t1[c3] + t2[c3] + dE_dsp * (-2 * sinprod) * v[c3] * irm2;
            gw[c3] += dE_dsp * (-sinprod) * wv[c3] * irr2;
            acc_v[5 + c3] = -gu[c3] - gv[c3];
            acc_v[8 + c3] = gv[c3] - gw[c3];
          }
          atomic_add3(w.f, i, gu[0], gu[1], gu[2]);
          atomic_add3(w.f, l, gw[0], gw[1], gw[2]);
        }
      }
      unit_sums<NV>(acc_v, key, acc);
    };
    int nbuf = 0;
    for (int u = 0; u < nu; ++u) {
      const UnitInt ui = uint_[wl][u];
      const double bo_m = ucon[wl][u][9];
      const int nit = ui.jn * ui.kn;
      for (int t0 = 0; t0 < nit; t0 += 32) {
        const int t = t0 + lane;
        bool ok = false;
        uint32_t item = 0;
        if (t < nit) {
          const int a = t / ui.kn, c = t % ui.kn;
          const int2 el = w.arow[ui.jb + a];
          const int2 er = w.arow[ui.kb + c];
          ok = !(el.x == ui.m && el.y > 0) && !(er.x == ui.m && er.y < 0);  // left == middle, right == reverse
          if (ok) {
            const int i = bond_other(w, el.x, el.y), l = bond_other(w, er.x, er.y);
            ok = __ldg(ff0.torsion_index + ((w.type[i] * T + ui.tj) * T + ui.tk) * T + w.type[l]) >= 0 &&
                 BFV(BF_BO, el.x) * bo_m * BFV(BF_BO, er.x) > THB_CUT;
            if (ok && i == l) {
              const uint32_t sl = bond_shift(w, el.x, el.y), sr = bond_shift(w, er.x, er.y);
              if (xr_sx(sl) == xr_sx(ui.sm) + xr_sx(sr) && xr_sy(sl) == xr_sy(ui.sm) + xr_sy(sr) &&
                  xr_sz(sl) == xr_sz(ui.sm) + xr_sz(sr))
                ok = false;  // the same atom image at both ends
            }
          }
          item = pack_item(u, a, c);
        }
        push_items(buf[wl], nbuf, ok, item, process);
      }
    }
    if (nbuf > 0) process(buf[wl][lane], lane < nbuf);
    if (lane < nu) {
      const UnitInt& ui = uint_[wl][lane];
      const double* s = uacc[wl][lane];
      BEV(2, ui.m) = s[0];
      BEV(3, ui.m) = s[1];
      if (s[2] != 0.0) atomicAdd(&BJV(BJ_BO, ui.m), s[2]);
      if (s[3] != 0.0) atomicAdd(&BJV(BJ_PI, ui.m), s[3]);
      if (s[4] != 0.0) {
        atomicAdd(&AJV(AJ_DB, ui.j), s[4]);
        atomicAdd(&AJV(AJ_DB, ui.k), s[4]);
      }
      if (s[5] != 0.0 || s[6] != 0.0 || s[7] != 0.0) atomic_add3(w.f, ui.j, s[5], s[6], s[7]);
      if (s[8] != 0.0 || s[9] != 0.0 || s[10] != 0.0) atomic_add3(w.f, ui.k, s[8], s[9], s[10]);
    }
    __syncwarp();
  }
}

constexpr int kHbWarps = 4;
constexpr int kHbDonors = 4;
constexpr int kHbBuf = 64;  // per-warp acceptor candidates: at most 31 left over + 32 new
struct HbDonor {
  double v[3];
  double ird, bo;  // 1 / |donor bond|, bond order
  int b, jd, td;
  uint32_t shift;
};

// Hydrogen bonds (src/xreac/energy.py:248-276), one warp per hydrogen (p_hbond = 1). Donors are the
// H's active bonds to p_hbond = 2 atoms with bo >= 0.01 (held in shared memory); acceptors are its
// edges within the H-bond cutoff to p_hbond = 2 atoms, other than the donor's own image. The warp
// first compacts the acceptor candidates of its row into shared memory with ballots, then gives
// each lane one candidate, so the FP64 work runs on full warps (an FP64 instruction costs the pipe
// the same for one active lane as for 32). Reciprocals are formed once per acceptor, per donor and
// per parameter row instead of once per (donor, acceptor) pair.
__global__ void __launch_bounds__(32 * kHbWarps, 4) k_hbonds(XrWork w, XrFF ff0) {
  __shared__ HbDonor don[kHbWarps][kHbDonors];
  __shared__ int2 cand[kHbWarps][kHbBuf];
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  const int h = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  if (h >= w.A) return;
  const XrFF ff = xr_ff_of(ff0, w, h);
  const int th = w.type[h], T = ff.ntypes;
  if (__ldg(ff.hb_role + th) != 1) {
    if (lane == 0) AEV(5, h) = 0.0;
    return;
  }
  const int L = w.A + 1;
  const XrSystem& S = w.sys[w.sys_of[h]];
  const double4_32a xh = w.x[h];
  const int abeg = w.cnt[3 * L + h], na = w.nact[h];
  const int ebeg = w.cnt[0 * L + h], eend = w.cnt[0 * L + h + 1];
  const unsigned lt = (1u << lane) - 1u;
  double E = 0;
  double gh[3] = {0, 0, 0};
  // Donor batches of up to kHbDonors (normally one batch holds them all).
  for (int dbase = 0; dbase < na; dbase += 32) {
    const int t = dbase + lane;
    bool is_donor = false;
    int2 en = make_int2(0, 0);
    if (t < na) {
      en = w.arow[abeg + t];
      const int jd = bond_other(w, en.x, en.y);
      is_donor = __ldg(ff.hb_role + w.type[jd]) == 2 && BFV(BF_BO, en.x) >= HBOND_THRESHOLD;
    }
    unsigned msk = __ballot_sync(0xffffffffu, is_donor);
    while (msk) {
      const int nd = min(__popc(msk), kHbDonors);
      const int rank = __popc(msk & lt);
      const bool mine = (msk >> lane & 1u) && rank < nd;
      if (mine) {
        HbDonor& d = don[wl][rank];
        d.b = en.x;
        d.jd = bond_other(w, en.x, en.y);
        d.td = w.type[d.jd];
        d.shift = bond_shift(w, en.x, en.y);
        d.bo = BFV(BF_BO, en.x);
        bond_vec(w, en.x, en.y, d.v);
        d.ird = 1.0 / w.b_r[en.x];
      }
      for (int q = 0; q < nd; ++q) msk &= msk - 1u;
      __syncwarp();
      // per-lane donor accumulators (registers; fixed indices after unrolling) and per-lane caches
      // of the last parameter row's constants and of exp(-hb2 bo) per donor
      double acc[kHbDonors][4];
      double eb_k[kHbDonors];
      int ebrow_k[kHbDonors];
#pragma unroll
      for (int k = 0; k < kHbDonors; ++k) {
        acc[k][0] = acc[k][1] = acc[k][2] = acc[k][3] = 0.0;
        eb_k[k] = 0.0;
        ebrow_k[k] = -1;
      }
      int crow = -1;
      double r0 = 0, ir0 = 0, hb1 = 0, hb2 = 0, hb3 = 0;
      auto process = [&](int2 ed) {
        const int ja = ed.x, ta = w.type[ja];
        const uint32_t sa = (uint32_t)ed.y & XR_SHIFT_MASK;
        double va[3];
        {
          const double4_32a xa = w.x[ja];
          const int sx = xr_sx(sa), sy = xr_sy(sa), sz = xr_sz(sa);
          const double p0[3] = {xh.x, xh.y, xh.z}, p1[3] = {xa.x, xa.y, xa.z};
          const bool shifted = sa != xr_pack_shift(0, 0, 0);  // else the offset is zero
          for (int c = 0; c < 3; ++c) {
            va[c] = __dsub_rn(p1[c], p0[c]);
            if (shifted)
              va[c] = __dadd_rn(va[c], __dadd_rn(__dadd_rn(__dmul_rn((double)sx, S.cell[c]), __dmul_rn((double)sy, S.cell[3 + c])),
                                                 __dmul_rn((double)sz, S.cell[6 + c])));
          }
        }
        const double ra = sqrt(va[0] * va[0] + va[1] * va[1] + va[2] * va[2]);
        const double ira = 1.0 / ra, ira2 = ira * ira;
        double ga[3] = {0, 0, 0};
#pragma unroll
        for (int k = 0; k < kHbDonors; ++k) {
          if (k >= nd) break;
          const HbDonor& d = don[wl][k];
          if (d.jd == ja && d.shift == sa) continue;  // same edge
          const int row = __ldg(ff.hbond_index + (d.td * T + th) * T + ta);
          if (row < 0) continue;
          if (row != crow) {
            const double* prm = ff.hbond + 4 * row;
            r0 = __ldg(prm + 0);
            hb1 = __ldg(prm + 1);
            hb2 = __ldg(prm + 2);
            hb3 = __ldg(prm + 3);
            ir0 = 1.0 / r0;
            crow = row;
          }
          if (!(r0 > 0)) continue;
          if (ebrow_k[k] != row) {
            eb_k[k] = xr_exp(-hb2 * d.bo);
            ebrow_k[k] = row;
          }
          const double eb = eb_k[k];
          const double inv = d.ird * ira;
          const double cosv = (d.v[0] * va[0] + d.v[1] * va[1] + d.v[2] * va[2]) * inv;
          const double cc = fmin(fmax(cosv, -1.0), 1.0);
          const double omc = 1 - cc;
          const double sin4 = 0.25 * omc * omc;
          const double Fb = hb1 * (1 - eb);
          const double E2 = xr_exp(-hb3 * (r0 * ira + ra * ir0 - 2));
          const double FE = Fb * E2;
          E += FE * sin4;
          acc[k][3] += hb1 * hb2 * eb * E2 * sin4;
          const double dE_dr_over_r = FE * sin4 * (-hb3) * (ir0 - r0 * ira2) * ira;
          const double dE_dcos = (cosv > -1.0 && cosv < 1.0) ? -0.5 * FE * omc : 0.0;
          const double ird2 = d.ird * d.ird;
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const double gdc = dE_dcos * (va[c] * inv - cosv * d.v[c] * ird2);
            const double gac = dE_dcos * (d.v[c] * inv - cosv * va[c] * ira2) + dE_dr_over_r * va[c];
            acc[k][c] += gdc;
            ga[c] += gac;
            gh[c] -= gdc + gac;
          }
        }
        if (ga[0] != 0.0 || ga[1] != 0.0 || ga[2] != 0.0) atomic_add3(w.f, ja, ga[0], ga[1], ga[2]);
      };
      // acceptor candidates: compacted in row order, processed 32 at a time
      int ncand = 0;
      for (int e0 = ebeg; e0 < eend; e0 += 32) {
        const int e = e0 + lane;
        bool ok = false;
        int2 ed = make_int2(0, 0);
        if (e < eend) {
          ed = w.edge[e];
          ok = ((uint32_t)ed.y & XR_CODE_HB) && __ldg(ff.hb_role + w.type[ed.x]) == 2;
        }
        const unsigned m = __ballot_sync(0xffffffffu, ok);
        if (ok) cand[wl][ncand + __popc(m & lt)] = ed;
        ncand += __popc(m);
        __syncwarp();
        if (ncand >= 32) {
          process(cand[wl][lane]);
          ncand -= 32;
          const int2 moved = lane < ncand ? cand[wl][32 + lane] : make_int2(0, 0);
          __syncwarp();
          if (lane < ncand) cand[wl][lane] = moved;
          __syncwarp();
        }
      }
      if (lane < ncand) process(cand[wl][lane]);
      // donor sensitivities: warp sums, then one update per donor
#pragma unroll
      for (int k = 0; k < kHbDonors; ++k) {
        if (k >= nd) break;
#pragma unroll
        for (int c = 0; c < 4; ++c)
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) acc[k][c] += __shfl_xor_sync(0xffffffffu, acc[k][c], o);
        if (lane == 0) {
          const HbDonor& d = don[wl][k];
          if (acc[k][3] != 0.0) atomicAdd(&BJV(BJ_BO, d.b), acc[k][3]);
          if (acc[k][0] != 0.0 || acc[k][1] != 0.0 || acc[k][2] != 0.0)
            atomic_add3(w.f, d.jd, acc[k][0], acc[k][1], acc[k][2]);
        }
      }
      __syncwarp();
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    E += __shfl_down_sync(0xffffffffu, E, o);
    gh[0] += __shfl_down_sync(0xffffffffu, gh[0], o);
    gh[1] += __shfl_down_sync(0xffffffffu, gh[1], o);
    gh[2] += __shfl_down_sync(0xffffffffu, gh[2], o);
  }
  if (lane == 0) {
    AEV(5, h) = E;
    if (gh[0] != 0.0 || gh[1] != 0.0 || gh[2] != 0.0) atomic_add3(w.f, h, gh[0], gh[1], gh[2]);
  }
}

// Per-atom chain: neighbours' over-coordination cross terms, lone pair, sbo, then dE/d total.
__global__ void k_chain_atom(XrWork w, XrFF ff0) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= w.A) return;
  const XrFF ff = xr_ff_of(ff0, w, a);
  const int L = w.A + 1, ta = w.type[a];
  const double* g = ff.g;
  double A_d = AJV(AJ_D, a), A_dlpt = AJV(AJ_DLPT, a);
  for (int k = w.cnt[3 * L + a]; k < w.cnt[3 * L + a] + w.nnz[a]; ++k) {
    const int2 en = w.nzrow[k];
    const int j = bond_other(w, en.x, en.y);
    const double P = BFV(BF_PI, en.x) + BFV(BF_PP, en.x);
    if (P == 0.0) continue;
    const double dfvl_j = atom_prm(ff, w.type[j], A_MASS) <= 21 ? 1.0 : 0.0;
    const double aov2 = AJV(AJ_OV2, j);
    A_d += aov2 * P;
    A_dlpt -= aov2 * dfvl_j * P;
  }
  const double mass = atom_prm(ff, ta, A_MASS);
  const double A_dlp = AJV(AJ_DLP, a) + (mass <= 21 ? A_dlpt : 0.0);
  const double sbo = AFV(AF_SBO, a), prod = AFV(AF_PROD, a), vlpex = AFV(AF_VLPEX, a), nlp = AFV(AF_NLP, a);
  const double db = AFV(AF_TOTAL, a) - atom_prm(ff, ta, A_VALENCY_BOC);
  const double lpt = vlpex >= 0 ? 0.0 : nlp;
  const double A_sbo = AJV(AJ_SBO2, a) * dsbo2_of(sbo, g[16]);
  const double A_prod = A_sbo * (db + g[33] * lpt);
  const double A_db = AJV(AJ_DB, a) - A_sbo * (1 - prod);
  double A_nlp = -A_dlp;
  if (vlpex < 0) A_nlp += -A_sbo * (1 - prod) * g[33];
  const double A_vlpex = A_nlp * (-2 * g[15] * (2 + vlpex) * AFV(AF_E15, a));
  AJV(AJ_SUMPI, a) = A_sbo;
  AJV(AJ_PRODSUM, a) = -prod * A_prod;
  AJV(AJ_TOTAL_ALL, a) = AJV(AJ_TOTAL, a) + A_d + A_db + A_vlpex;
}

// Per-bond chain: from the thresholded outputs back through f1, f4, f5 to the uncorrected orders.
__device__ inline void k_chain_bond_one(const XrWork& w, const XrFF& ff0, int b) {
  const int i = w.bond_i[b], j = w.bond_j[b];
  const XrFF ff = xr_ff_of(ff0, w, i);
  const int ti = w.type[i], tj = w.type[j], T = ff.ntypes, pt = ti * T + tj;
  const double bo = BFV(BF_BO, b), pi = BFV(BF_PI, b), pp = BFV(BF_PP, b), sig = BFV(BF_SIG, b);
  const double b2 = bo * bo, b4 = b2 * b2, b7 = b4 * b2 * bo;
  double A_bo = BJV(BJ_BO, b) + AJV(AJ_TOTAL_ALL, i) + AJV(AJ_TOTAL_ALL, j) +
                (AJV(AJ_OV1, i) + AJV(AJ_OV1, j)) * pair_prm(ff, pt, P_OVUN1) * pair_prm(ff, pt, P_DE_S) +
                (AJV(AJ_PRODSUM, i) + AJV(AJ_PRODSUM, j)) * 8.0 * b7;
  if (w.pgrad && bo != 0.0) {
    // De_s and p_ovun1 also weight the over-coordination sum ov1 = sum p_ovun1 De_s bo of both ends
    double* gp = xr_pgrad(w, i) + (size_t)pt * XR_NPAIR_COLS;
    const double a_ov = (AJV(AJ_OV1, i) + AJV(AJ_OV1, j)) * bo;
    atomicAdd(gp + P_DE_S, a_ov * pair_prm(ff, pt, P_OVUN1));
    atomicAdd(gp + P_OVUN1, a_ov * pair_prm(ff, pt, P_DE_S));
  }
  const double di = AFV(AF_TOTAL, i) - atom_prm(ff, ti, A_VALENCY), dj = AFV(AF_TOTAL, j) - atom_prm(ff, tj, A_VALENCY);
  const double dfi = atom_prm(ff, ti, A_MASS) <= 21 ? 1.0 : 0.0, dfj = atom_prm(ff, tj, A_MASS) <= 21 ? 1.0 : 0.0;
  const double A_P = AJV(AJ_OV2, i) * (dj - dfi * AFV(AF_DLPT, j)) + AJV(AJ_OV2, j) * (di - dfj * AFV(AF_DLPT, i)) +
                     AJV(AJ_SUMPI, i) + AJV(AJ_SUMPI, j);
  const double A_pi = BJV(BJ_PI, b) + A_P, A_pp = BJV(BJ_PP, b) + A_P, A_sig = BJV(BJ_SIG, b);
  const double gsig = sig != 0.0 ? A_sig : 0.0;
  const double g_bo = (bo != 0.0 ? A_bo : 0.0) + gsig;
  const double g_pi = (pi != 0.0 ? A_pi : 0.0) - gsig;
  const double g_pp = (pp != 0.0 ? A_pp : 0.0) - gsig;
  const double bo0 = BFV(BF_BO0, b), pi0 = BFV(BF_PI0, b), pp0 = BFV(BF_PP0, b);
  const double f1 = BFV(BF_F1, b), f4 = BFV(BF_F4, b), f5 = BFV(BF_F5, b), corr = BFV(BF_CORR, b);
  const double v13 = pair_prm(ff, pt, P_V13COR), ovc = pair_prm(ff, pt, P_OVC);
  const bool mask = BFV(BF_MASK, b) != 0.0;
  const bool corrected = mask && (ovc >= 0.001 || v13 >= 0.001);
  const double boc3 = corrected ? pair_prm(ff, pt, P_BOC3) : 0.0, boc4 = corrected ? pair_prm(ff, pt, P_BOC4) : 0.0;
  const double f45 = v13 >= 0.001 ? f4 * f5 : 1.0;
  double d_bo0 = g_bo * corr;
  const double d_pi0 = g_pi * corr * f1;
  const double d_pp0 = g_pp * corr * f1;
  const double d_corr = g_bo * bo0 + g_pi * pi0 * f1 + g_pp * pp0 * f1;
  const double d_f1 = (g_pi * pi0 + g_pp * pp0) * corr + d_corr * f45;
  double d_dbi = 0, d_dbj = 0;
  if (v13 >= 0.001) {
    const double d_f45 = d_corr * f1;
    const double dz4 = d_f45 * f5 * (-f4 * (1 - f4));
    const double dz5 = d_f45 * f4 * (-f5 * (1 - f5));
    d_bo0 += (dz4 + dz5) * (-2 * boc3 * boc4 * bo0);
    d_dbi = dz4 * boc3;
    d_dbj = dz5 * boc3;
  }
  BJV(BJ_BO0, b) = d_bo0;
  BJV(BJ_PI0, b) = d_pi0;
  BJV(BJ_PP0, b) = d_pp0;
  BJV(BJ_CI, b) = d_f1 * BFV(BF_DF1I, b) + d_dbi;
  BJV(BJ_CJ, b) = d_f1 * BFV(BF_DF1J, b) + d_dbj;
}

__global__ void k_chain_bond(XrWork w, XrFF ff) {
  const int nm = *w.nmask;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nm; q += gridDim.x * blockDim.x)
    k_chain_bond_one(w, ff, w.mlist[q]);
}

__global__ void k_chain_deltap(XrWork w) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= w.A) return;
  const int L = w.A + 1;
  double s = 0;
  for (int k = w.cnt[3 * L + a]; k < w.cnt[3 * L + a] + w.nnz[a]; ++k) {
    const int2 en = w.nzrow[k];
    s += en.y > 0 ? BJV(BJ_CI, en.x) : BJV(BJ_CJ, en.x);
  }
  AJV(AJ_DELTAP, a) = s;
}

// dE/dr of each bond from the uncorrected bond orders; added to the pair's radial accumulator.
__device__ inline void k_chain_radial_one(const XrWork& w, const XrFF& ff0, int b) {
  if (BFV(BF_MASK, b) == 0.0) return;
  const double d_bo0 = BJV(BJ_BO0, b) + AJV(AJ_DELTAP, w.bond_i[b]) + AJV(AJ_DELTAP, w.bond_j[b]);
  const double G = d_bo0 * BFV(BF_DSIG, b) + (d_bo0 + BJV(BJ_PI0, b)) * BFV(BF_DPI, b) +
                   (d_bo0 + BJV(BJ_PP0, b)) * BFV(BF_DPP, b);
  w.p_g[w.bond_pair[b]] += G;
  if (w.pgrad) {
    // dE/d(p_bo1..6, r_s, r_p, r_pp): the uncorrected orders' parameters, through the same chain
    // adjoints (dE/dsigma' = dE/dBO0, dE/dpi' = dE/dBO0 + dE/dPI0, dE/dpipi' = dE/dBO0 + dE/dPP0)
    const XrFF ff = xr_ff_of(ff0, w, w.bond_i[b]);
    const int ti = w.type[w.bond_i[b]], tj = w.type[w.bond_j[b]], T = ff.ntypes, pt = ti * T + tj;
    double* gp = xr_pgrad(w, w.bond_i[b]) + (size_t)pt * XR_NPAIR_COLS;
    const double r = w.b_r[b], lr = xr_log(r), cut = 0.01 * ff.g[29];
    const double adj[3] = {d_bo0, d_bo0 + BJV(BJ_PI0, b), d_bo0 + BJV(BJ_PP0, b)};
    const int cr[3] = {A_R_S, A_R_PI, A_R_PI_PI};
    const int ca[3] = {P_BO1, P_BO3, P_BO5}, cb[3] = {P_BO2, P_BO4, P_BO6}, cr0[3] = {P_RS, P_RP, P_RPP};
    for (int k = 0; k < 3; ++k) {
      if (!(atom_prm(ff, ti, cr[k]) > 0 && atom_prm(ff, tj, cr[k]) > 0) || adj[k] == 0.0) continue;
      const double pa = pair_prm(ff, pt, ca[k]), pb = pair_prm(ff, pt, cb[k]), r0 = pair_prm(ff, pt, cr0[k]);
      const double lt = lr - __ldg(ff.pair_logr + 3 * pt + k);
      const double t = xr_exp(pb * lt);
      const double bo = (k == 0 ? 1.0 + cut : 1.0) * xr_exp(pa * t);
      atomicAdd(gp + ca[k], adj[k] * bo * t);
      atomicAdd(gp + cb[k], adj[k] * bo * pa * t * lt);
      atomicAdd(gp + cr0[k], adj[k] * bo * pa * t * (-pb / r0));
    }
  }
}

__global__ void k_chain_radial(XrWork w, XrFF ff) {
  const int nm = *w.nmask;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nm; q += gridDim.x * blockDim.x)
    k_chain_radial_one(w, ff, w.mlist[q]);
}

}  // namespace

// Per-bond kernels after k_bo1 run over the active-bond list (bonds whose uncorrected order passed
// the cut), grid-striding over its device-side length.
static int active_grid(const XrWork& w, int tb) { return std::max(1, std::min((w.nB + tb - 1) / tb, 152 * 8)); }

void xr_launch_bond_orders(const XrWork& w, const XrFF& ff, cudaStream_t st) {
  const int tb = 128;
  const int gB = (w.nB + tb - 1) / tb;
  // (the torsion-middle and active-bond counters were zeroed by k_prep)
  if (w.nB > 0) k_bo1<<<gB, tb, 0, st>>>(w, ff);
  k_deltap<<<(w.A + 3) / 4, 128, 0, st>>>(w);
  if (w.nB > 0) k_bo2<<<active_grid(w, tb), tb, 0, st>>>(w, ff);
}

void xr_launch_bonded(const XrWork& w, const XrFF& ff, cudaStream_t st) {
  const int tb = 128;
  const int gA = (w.A + tb - 1) / tb;
  const int gB = (w.nB + tb - 1) / tb;
  const int gM = active_grid(w, tb);
  k_atom1<<<gA, tb, 0, st>>>(w, ff);
  k_atom2<<<gA, tb, 0, st>>>(w, ff);
  if (w.nB > 0) k_bond_energy<<<gM, tb, 0, st>>>(w, ff);
  {
    const int chunks = (w.A + kUnits - 1) / kUnits;
    k_angles<<<(chunks + kBondedWarps - 1) / kBondedWarps, 32 * kBondedWarps, 0, st>>>(w, ff);
  }
  if (w.nB > 0) {
    const int gT = std::min((w.nB + kMidTile - 1) / kMidTile, 152 * 16);
    k_mid_count<<<gT, kMidTile, 0, st>>>(w);
    k_mid_scan<<<1, 1024, 0, st>>>(w);
    k_mid_fill<<<gT, kMidTile, 0, st>>>(w);
    const int chunks = (w.nB + kUnits - 1) / kUnits;
    const int blocks = std::min((chunks + kBondedWarps - 1) / kBondedWarps, 152 * 16);
    k_torsions<<<blocks, 32 * kBondedWarps, 0, st>>>(w, ff);
  }
  k_hbonds<<<(w.A + kHbWarps - 1) / kHbWarps, 32 * kHbWarps, 0, st>>>(w, ff);
  k_chain_atom<<<gA, tb, 0, st>>>(w, ff);
  if (w.nB > 0) {
    k_chain_bond<<<gM, tb, 0, st>>>(w, ff);
    k_chain_deltap<<<gA, tb, 0, st>>>(w);
    k_chain_radial<<<gM, tb, 0, st>>>(w, ff);
  }
}
