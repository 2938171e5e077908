// Nonbonded pairs, QEq charges, Coulomb, force assembly and per-system reductions (FP64).
//
// - Taper, shielded Coulomb kernel and tapered vdW (shielding and/or inner core) restate
//   src/xreac/energy.py:89-92 and 213-219; each unordered image pair is evaluated once and counts
//   for both of xreac's directed edges.
// - QEq restates the KKT system of src/xreac/energy.py:95-102 (H = 14.4 * sum of shields +
//   diag(eta), self images on the diagonal, sum q = Q) and solves it by Jacobi-preconditioned
//   conjugate gradients projected onto sum q = Q (one solve; Gould, Hribar and Nocedal's projected
//   CG). Matrix rows are gathered from the full directed neighbour rows, so a matrix-vector product
//   needs no atomics and is deterministic.
// - A single large system runs the solver as one cooperative grid with a barrier whose every wait
//   is bounded; batches of systems give each system one thread block.
#include <algorithm>
#include <type_traits>

#include "xr_common.cuh"
#include "xr_dfloat.cuh"
#include "xreac_gb300.h"

namespace {

constexpr double C_ELE = 332.06371;
constexpr double QEQ_COULOMB = 14.4;
constexpr double SELF_CONVERSION = 23.02;

#define AEV(k, a) w.a_e[(size_t)(k) * w.A + (a)]
#define QW(k, a) w.qwork[(size_t)(k) * w.A + (a)]

__device__ inline double pair_prm(const XrFF& ff, int pt, int col) { return __ldg(ff.pair + pt * XR_NPAIR_COLS + col); }
__device__ inline double atom_prm(const XrFF& ff, int t, int col) { return __ldg(ff.atom + t * XR_NATOM_COLS + col); }
// The QEq solver sees one system at a time and reads only its parameter set's atom table.
__device__ inline double atom_prm(const double* atab, int t, int col) { return __ldg(atab + t * XR_NATOM_COLS + col); }
__device__ inline const double* atoms_of_system(const XrFF& ff, const XrSystem& S) {
  return xr_ff_at(ff, ff.nsets > 1 ? S.ff_set : 0).atom;
}

__device__ inline void edge_vector(const XrSystem& S, const double4_32a& xi, const double4_32a& xj, uint32_t code, double v[3]) {
  const double xa[3] = {xi.x, xi.y, xi.z}, xb[3] = {xj.x, xj.y, xj.z};
  if ((code & XR_SHIFT_MASK) == xr_pack_shift(0, 0, 0)) {  // no image shift: the offset is zero
    for (int c = 0; c < 3; ++c) v[c] = __dsub_rn(xb[c], xa[c]);
    return;
  }
  const int sx = xr_sx(code), sy = xr_sy(code), sz = xr_sz(code);
  for (int c = 0; c < 3; ++c) {
    const double off = __dadd_rn(__dadd_rn(__dmul_rn((double)sx, S.cell[c]), __dmul_rn((double)sy, S.cell[3 + c])),
                                 __dmul_rn((double)sz, S.cell[6 + c]));
    v[c] = __dadd_rn(__dsub_rn(xb[c], xa[c]), off);
  }
}

// t^(-1/3) for t in the float range: an FP32 seed, then two Newton-Raphson steps on f(z) = z^-3 - t,
// z <- z (4 - t z^3) / 3, each of which squares the relative error (about 1e-7, 1e-14, then FP64
// rounding). Multiplies only: it replaces a double cube root and the divisions by it. It stays FP64:
// the shield builds the QEq matrix, whose solve amplifies an entry's error by the matrix's condition
// (a double-float version, about 1e-14, moved the Coulomb energy of an ill-conditioned fixture by 2e-12
// of its value, beyond the parity tolerance).
__device__ inline double inv_cbrt(double t) {
  double z = (double)rcbrtf((float)t);
  z = z * (4.0 - t * z * z * z) * (1.0 / 3.0);
  z = z * (4.0 - t * z * z * z) * (1.0 / 3.0);
  return z;
}

// The QEq block-Jacobi groups: runs of at most kGroupMax consecutive atoms, each within kGroupBond of
// an earlier atom of its run (molecules).
constexpr int kGroupMax = 8;
constexpr double kGroupBond = 1.3;

// ------------------------------------------------------------------------------ pair kernel
__device__ inline void pair_one(const XrWork& w, const XrFF& ff0, int p) {
  const int e = w.pair_edge[p], i = w.pair_i[p];
  const int2 ed = w.edge[e];
  const int j = ed.x;
  const XrSystem& S = w.sys[w.sys_of[i]];
  const XrFF ff = xr_ff_at(ff0, ff0.nsets > 1 ? S.ff_set : 0);
  double v[3];
  edge_vector(S, w.x[i], w.x[j], (uint32_t)ed.y, v);
  const double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(v[0], v[0]), __dmul_rn(v[1], v[1])), __dmul_rn(v[2], v[2])));
  if (r < kGroupBond && i != j && abs(i - j) < kGroupMax) {  // a bond for the QEq preconditioner's groups
    const int lo = min(i, j), hi = max(i, j);
    atomicMin(w.qb_first + hi, lo);
    atomicMax(w.qb_last + hi, lo);
  }
  const double rc = S.rc;
  const int T = ff.ntypes, pt = w.type[i] * T + w.type[j];
  double taper = 0.0, dtaper = 0.0;
  if (r < rc) {
    const double u = r * S.inv_rc;
    taper = 1 + u * u * u * u * (-35 + u * (84 + u * (-70 + 20 * u)));
    const double um = u - 1;
    dtaper = 140.0 * S.inv_rc * u * u * u * um * um * um;
  }
  const double gam = pair_prm(ff, pt, P_GAMMA);
  const double z = inv_cbrt(r * r * r + gam);  // (r^3 + gamma)^(-1/3), FP64: the QEq matrix is built from it
  const double z2 = z * z;
  const double shield = taper * z;
  const double dshield = dtaper * z - taper * r * r * (z2 * z2);
  double f13 = r, df13 = 1.0;
  // exponentials and logarithms in double-float arithmetic on the FP32 pipe (xr_dfloat.cuh): they
  // were most of this kernel's FP64 issue. The shielding chain stays in double-floats from r to
  // f13 = (r^p + gw)^(1/p) and df13 / dr = r^(p-1) sum^(1/p-1) = exp((p-1) log r + (1/p-1) log sum).
  if (ff.vdw_type == 1 || ff.vdw_type == 3) {
    const xr_df lr = xr_df_log_df(xr_df_from_double(r));
    const xr_df rp = xr_df_exp_df(xr_df_mul(lr, {ff.vdw_p.x, ff.vdw_p.y}));
    const xr_df ls = xr_df_log_df(xr_df_add(rp, xr_df_from_double(__ldg(ff.pair_gw + pt))));
    const xr_df f = xr_df_exp_df(xr_df_mul(ls, {ff.vdw_invp.x, ff.vdw_invp.y}));
    const xr_df d = xr_df_exp_df(xr_df_add(xr_df_mul(lr, {ff.vdw_p_m1.x, ff.vdw_p_m1.y}),
                                           xr_df_mul(ls, {ff.vdw_invp_m1.x, ff.vdw_invp_m1.y})));
    f13 = (double)f.hi + (double)f.lo;
    df13 = (double)d.hi + (double)d.lo;
  }
  // reciprocals of the pair's radii from the table: multiplies instead of FP64 divisions
  const double D = pair_prm(ff, pt, P_D), alpha = pair_prm(ff, pt, P_ALPHA);
  const double2 inv = __ldg(reinterpret_cast<const double2*>(ff.pair_inv) + pt);  // 1/r_vdW, 1/rcore
  const double ev = xr_exp(0.5 * alpha * (1 - f13 * inv.x));
  const double dev = ev * (-0.5 * alpha * inv.x) * df13;
  double E = taper * D * (ev * ev - 2 * ev);
  double G = dtaper * D * (ev * ev - 2 * ev) + taper * D * (2 * ev - 2) * dev;
  if (ff.vdw_type == 2 || ff.vdw_type == 3) {
    const double ecore = pair_prm(ff, pt, P_ECORE), acore = pair_prm(ff, pt, P_ACORE);
    const double ec = ecore * xr_exp(acore * (1 - r * inv.y));
    E += taper * ec;
    G += dtaper * ec + taper * ec * (-acore * inv.y);
  }
  w.p_r[p] = r;
  w.p_shield[p] = shield;
  w.p_dshield[p] = dshield;
  w.p_evdw[p] = E;
  w.p_g[p] = G;
  if (w.pgrad && taper != 0.0) {
    // dE/d(D, alpha, r_vdW, gamma_w) of this pair's tapered vdW term (and the inner core's)
    const double rvdw = pair_prm(ff, pt, P_RVDW);
    double* gp = xr_pgrad(w, i) + (size_t)pt * XR_NPAIR_COLS;
    const double m = taper * D * (2 * ev - 2) * ev;  // dE/d(log ev) per unit of the exponent's argument
    atomicAdd(gp + P_D, taper * (ev * ev - 2 * ev));
    atomicAdd(gp + P_ALPHA, m * 0.5 * (1 - f13 / rvdw));
    atomicAdd(gp + P_RVDW, m * 0.5 * alpha * f13 / (rvdw * rvdw));
    if (ff.vdw_type == 1 || ff.vdw_type == 3) {
      // f13 = (r^p + gw)^(1/p) with gw = gamma_w^-p: d f13 / d gamma_w = -f13 gw / (sum gamma_w)
      const double pw = ff.g[28], gw = __ldg(ff.pair_gw + pt);
      const double sum = exp(pw * log(r)) + gw;
      const double gamw = pair_prm(ff, pt, P_GAMMA_W);
      atomicAdd(gp + P_GAMMA_W, m * (-0.5 * alpha / rvdw) * (-f13 * gw / (sum * gamw)));
    }
    if (ff.vdw_type == 2 || ff.vdw_type == 3) {
      const double ecore = pair_prm(ff, pt, P_ECORE), acore = pair_prm(ff, pt, P_ACORE), rcore = pair_prm(ff, pt, P_RCORE);
      const double ex = exp(acore * (1 - r / rcore));
      atomicAdd(gp + P_ECORE, taper * ex);
      atomicAdd(gp + P_ACORE, taper * ecore * ex * (1 - r / rcore));
      atomicAdd(gp + P_RCORE, taper * ecore * ex * acore * r / (rcore * rcore));
    }
  }
}

__global__ void k_hval(XrWork w) {
  const int ne = xr_num_edges(w);
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x) {
    const double h = QEQ_COULOMB * w.p_shield[w.edge_pair[e]];
    w.hval[e] = h;
    w.qch[e] = float(h);  // FP32 copy for the solver's row cache (which may overwrite it, scaled)
  }
}

// ---------------------------------------------------------------------------------- QEq
// Minimise 1/2 q'Hq + chi'q on {sum q = Q} -- the KKT system of src/xreac/energy.py:95-102 -- by
// projected preconditioned conjugate gradients (Gould, Hribar & Nocedal, SIAM J. Sci. Comput. 23,
// 1376 (2001)) with the Jacobi preconditioner D = diag(H): one solve instead of the two of the
// LAMMPS form, with the gradient re-projected every iteration (g <- g - lambda 1,
// lambda = <D^-1, g> / <D^-1, 1>) so the multiplier direction never accumulates.
// The product H z with z = D^-1 (g - lambda) is formed on the fly from a pre-scaled matrix
// H'_ij = H_ij / D_jj and row sums c_i = sum_j H'_ij, so no vector other than g is gathered.
// The gradient lives in two buffers used in turn. The multiplier part that a step adds,
// alpha <D^-1, Hp> / <D^-1, 1>, is reduced together with p'Hp, so the new gradient is written
// already projected and the second reduction only sees rounding-level drift; the squared norm
// g'D^-1 g is then free of cancellation against the multiplier direction (which grows towards
// -mu 1 at convergence), and the solver reaches the FP64 floor on every system.
// Per iteration: one matrix-vector product and two team-wide reductions (two barriers).
enum { Q_X = 0, Q_G, Q_P, Q_HP, Q_DINV, Q_C, Q_G2 };

__device__ inline unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Polls before a team wait gives up, and whether wait number `episode` of a team is the one a test
// made unsatisfiable (XrWork::wait_fail_at).
__device__ inline long long wait_cap(const XrWork& w, long long dflt) { return w.wait_polls > 0 ? w.wait_polls : dflt; }
__device__ inline bool wait_poisoned(const XrWork& w, unsigned episode) {
  return w.wait_fail_at > 0 && episode == (unsigned)w.wait_fail_at;
}

// Bounded grid barrier for a cooperative launch (all blocks co-resident): every block adds one to a
// monotonically increasing counter with release semantics and waits, with acquire loads, until it
// reaches the episode's target (number of blocks times episodes so far). Returns false when the
// wait ran out; every block then leaves the solver and the host reports the status bit.
__device__ bool grid_barrier(unsigned* bar, unsigned target, const XrWork& w, bool poisoned) {
  __syncthreads();
  __shared__ int ok;
  if (threadIdx.x == 0) {
    ok = 1;
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(bar) : "memory");
    const long long cap = wait_cap(w, 1ll << 24);
    long long it = 0;
    while (poisoned || ld_acquire(bar) < target) {
      if (++it > cap || ((it & 255) == 0 && (*(volatile int*)w.status & XR_S_BARRIER))) {
        atomicOr(w.status, XR_S_BARRIER);
        ok = 0;
        break;
      }
      if (it > 256) __nanosleep(32);
    }
  }
  __syncthreads();
  return ok;
}

// Team: the whole cooperative grid on one system, or one block on one system of a batch.
// Results of a reduction land in one of two result slots (by the parity of `slot`), so a reduction
// may write its totals while a slow warp still reads the previous reduction's.
// smem layout of the reductions: per-warp inputs at [k * 32 + warp] (k < 8), results from 256 on.
constexpr int kRedSmem = 8 * 32 + 16;
__device__ inline double* result_slot(double* smem, int slot) { return smem + 256 + 8 * (slot & 1); }

struct GridTeam {
  unsigned* bar;                // arrival counter of this team (zeroed before the launch)
  double* red;                  // the team's reduction slots: [slot][value][rank]
  int nb, rank;                 // blocks in the team and this block's rank
  mutable unsigned target = 0;  // barrier episodes so far times nb
  __device__ bool sync(const XrWork& w) const {
    target += nb;
    return grid_barrier(bar, target, w, wait_poisoned(w, target / nb));
  }
  // Team-wide sum of NV block totals held by lane 0 of warp 0, fused with the barrier: lane 0
  // publishes the block's values into a fixed slot and arrives (release); after the bounded wait
  // warp 0 adds all blocks' values in rank order (deterministic), thread 0 runs post() on the
  // totals (scalar work that then costs no extra synchronisation), and every thread receives them.
  template <int NV, class Post>
  __device__ bool reduce(const XrWork& w, double* v, double* smem, int slot, Post post) const {
    static_assert(NV <= 8, "at most eight values per reduction");
    __shared__ int ok;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    target += nb;
    double* res = result_slot(smem, slot);
    // Fixed-size slots ([rank][8] doubles); consecutive reductions never share one, so a block may
    // publish the next partials while a slower block still reads the previous ones.
    double* rs = red + (size_t)slot * 8 * nb;
    if (wid == 0) {
      int good = 1;
      __syncwarp();  // orders warp 0's row writes before lane 0's release
      if (lane == 0) {
        for (int k = 0; k < NV; ++k) rs[rank * 8 + k] = v[k];
        asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(bar) : "memory");
        const long long cap = wait_cap(w, 1ll << 24);
        const bool poisoned = wait_poisoned(w, target / nb);
        long long it = 0;
        while (poisoned || ld_acquire(bar) < target) {
          if (++it > cap || ((it & 255) == 0 && (*(volatile int*)w.status & XR_S_BARRIER))) {
            atomicOr(w.status, XR_S_BARRIER);
            good = 0;
            break;
          }
          if (it > 256) __nanosleep(32);
        }
        ok = good;
      }
      __syncwarp();
      // every lane issues all of its loads before adding (one memory round trip, not one per block);
      // lane sums in rank order, then a fixed shuffle tree: deterministic
      double t[NV];
#pragma unroll
      for (int k = 0; k < NV; ++k) t[k] = 0.0;
      for (int base = 0; base < nb; base += 5 * 32) {
        double x[5][NV];
#pragma unroll
        for (int u = 0; u < 5; ++u) {
          const int q = base + lane + 32 * u;
#pragma unroll
          for (int k = 0; k < NV; ++k) x[u][k] = q < nb ? __ldcg(rs + q * 8 + k) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 5; ++u)
#pragma unroll
          for (int k = 0; k < NV; ++k) t[k] += x[u][k];
      }
#pragma unroll
      for (int k = 0; k < NV; ++k) {
        double s = t[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) res[k] = s;
      }
      if (lane == 0) post(res);
    }
    __syncthreads();
    for (int k = 0; k < NV; ++k) v[k] = res[k];
    return ok;
  }
  // The same for NV <= 4 floats (the FP32 sweeps' scalars): slots of four floats per rank, one
  // 16-byte load per rank, and FP32 sums. An FP64 add occupies this part's FP64 pipe for 64
  // cycles per warp instruction, so the double form's 30 dependent adds for three values took
  // about 1 us of the reduction.
  template <int NV, class Post>
  __device__ bool reducef(const XrWork& w, float* v, double* smem, int slot, Post post) const {
    static_assert(NV <= 4, "at most four values per reduction");
    __shared__ int ok;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    target += nb;
    float* res = reinterpret_cast<float*>(result_slot(smem, slot));
    float* rs = reinterpret_cast<float*>(red + (size_t)slot * 8 * nb);  // [rank][4]
    if (wid == 0) {
      int good = 1;
      __syncwarp();  // orders warp 0's row writes before lane 0's release
      if (lane == 0) {
        float4 o = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (NV > 0) o.x = v[0];
        if (NV > 1) o.y = v[1];
        if (NV > 2) o.z = v[2];
        if (NV > 3) o.w = v[3];
        reinterpret_cast<float4*>(rs)[rank] = o;
        asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(bar) : "memory");
        const long long cap = wait_cap(w, 1ll << 24);
        const bool poisoned = wait_poisoned(w, target / nb);
        long long it = 0;
        while (poisoned || ld_acquire(bar) < target) {
          if (++it > cap || ((it & 255) == 0 && (*(volatile int*)w.status & XR_S_BARRIER))) {
            atomicOr(w.status, XR_S_BARRIER);
            good = 0;
            break;
          }
          if (it > 256) __nanosleep(32);
        }
        ok = good;
      }
      __syncwarp();
      // each lane adds its ranks in order, then a fixed shuffle tree: deterministic
      float t[4] = {0.0f, 0.0f, 0.0f, 0.0f};
      for (int base = 0; base < nb; base += 5 * 32) {
        float4 x[5];
#pragma unroll
        for (int u = 0; u < 5; ++u) {
          const int q = base + lane + 32 * u;
          x[u] = q < nb ? __ldcg(reinterpret_cast<const float4*>(rs) + q) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
#pragma unroll
        for (int u = 0; u < 5; ++u) {
          t[0] += x[u].x;
          t[1] += x[u].y;
          t[2] += x[u].z;
          t[3] += x[u].w;
        }
      }
#pragma unroll
      for (int k = 0; k < NV; ++k) {
        float s = t[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        t[k] = s;
      }
      if (lane == 0) {
        for (int k = 0; k < NV; ++k) res[k] = t[k];
        post(res);
      }
    }
    __syncthreads();
    for (int k = 0; k < NV; ++k) v[k] = res[k];
    return ok;
  }
};

struct BlockTeam {
  __device__ bool sync(const XrWork&) const {
    __syncthreads();
    return true;
  }
  template <int NV, class Post>
  __device__ bool reduce(const XrWork&, double* v, double* smem, int slot, Post post) const {
    double* res = result_slot(smem, slot);
    if (threadIdx.x == 0) {
      for (int k = 0; k < NV; ++k) res[k] = v[k];
      post(res);
    }
    __syncthreads();
    for (int k = 0; k < NV; ++k) v[k] = res[k];
    return true;
  }
};

// Team sum of NV values held by lane 0 of every warp: warp 0 first adds the block's warps.
// Distributed shared memory of a thread-block cluster (sm_90+): 32-bit shared-window addresses, the
// same variable in another block of the cluster, and mbarrier operations on it.
__device__ inline unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ inline unsigned cluster_map(unsigned addr, unsigned rank) {
  unsigned r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
__device__ inline unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ inline unsigned cluster_size() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}
// Hardware barrier of all threads of the cluster; only where every block is known to arrive (kernel
// entry and exit), never inside the solver.
__device__ inline void cluster_barrier_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Team of the blocks of one thread-block cluster (at most 8), exchanging through distributed shared
// memory. A reduction or barrier is one exchange, numbered m = 1, 2, ...: lane r of warp 0 of every
// block writes that block's partials into block r's slot array and then the exchange number into
// the entry's sequence word (a release store, cluster scope); lane r of each block waits (bounded,
// acquire loads) until entry r of its own slot array carries m. The partials are then added in rank
// order, so every block holds bit-identical totals and takes the same path. Two slot arrays
// alternate by the parity of m: block X writes exchange m + 2 into block Y only after seeing Y's
// entry of exchange m + 1, which Y wrote after reading exchange m.
struct ClusterTeam {
  double* slots;    // this block's partials, [parity][rank][value], 2 x 8 x 8
  unsigned* seqs;   // the exchange number of each entry, [parity][rank], 2 x 8 (zeroed at entry)
  int nb, rank;
  mutable unsigned count = 0;  // exchanges so far
  // Warp 0: push v[0..nv) (valid in lanes < nb) into every block's entry `rank` of slot array
  // `par`, then wait until this block's entries 0..nb-1 carry exchange number `count`. Lane r
  // (< nb) returns entry r's values in t. Bounded: false after about 2^22 polls or once another
  // wait has given up (the status bit).
  template <int NV>
  __device__ bool exchange(const XrWork& w, const double* v, unsigned par, double* t) const {
    const int lane = threadIdx.x & 31;
    const unsigned m = count;
    __syncwarp();
    if (lane < nb) {
      const unsigned dst = cluster_map(smem_u32(slots + (par * 8 + rank) * 8), lane);
#pragma unroll
      for (int k = 0; k < NV; ++k) asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(dst + 8 * k), "d"(v[k]) : "memory");
      asm volatile("st.release.cluster.shared::cluster.u32 [%0], %1;" ::"r"(cluster_map(smem_u32(seqs + par * 8 + rank), lane)),
                   "r"(m)
                   : "memory");
    }
    bool mine = lane >= nb;
    const unsigned mine_addr = smem_u32(seqs + par * 8 + (lane & 7));
    const long long cap = wait_cap(w, 1ll << 22);
    const bool poisoned = wait_poisoned(w, m);
    long long it = 0;
    int good = 1;
    for (;;) {
      if (!mine) {
        unsigned sq;
        asm volatile("ld.acquire.cluster.shared::cta.u32 %0, [%1];" : "=r"(sq) : "r"(mine_addr) : "memory");
        mine = sq == m && !poisoned;
      }
      if (__all_sync(0xffffffffu, mine)) break;
      bool stop = ++it > cap;
      if (lane == 0 && (it & 1023) == 0) stop = stop || (*(volatile int*)w.status & XR_S_BARRIER);
      if (__any_sync(0xffffffffu, stop)) {
        if (lane == 0) atomicOr(w.status, XR_S_BARRIER);
        good = 0;
        break;
      }
    }
    if (lane < nb) {
      const double* src = slots + (par * 8 + lane) * 8;
#pragma unroll
      for (int k = 0; k < NV; ++k) t[k] = src[k];
    } else {
#pragma unroll
      for (int k = 0; k < NV; ++k) t[k] = 0.0;
    }
    return good;
  }
  // exchange() for NV <= 8 floats (the FP32 sweeps' scalars): the same protocol on a float view of
  // the slot arrays, so that the totals are FP32 adds (an FP64 add occupies this part's FP64 pipe for
  // 64 cycles per warp instruction: the FP64 totals and post hook took about 0.45 us of each
  // reduction).
  template <int NV>
  __device__ bool exchangef(const XrWork& w, const float* v, unsigned par, float* t) const {
    const int lane = threadIdx.x & 31;
    const unsigned m = count;
    float* fslots = reinterpret_cast<float*>(slots);  // [parity][rank][16]
    __syncwarp();
    if (lane < nb) {
      const unsigned dst = cluster_map(smem_u32(fslots + (par * 8 + rank) * 16), lane);
#pragma unroll
      for (int k = 0; k < NV; ++k) asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(dst + 4 * k), "f"(v[k]) : "memory");
      asm volatile("st.release.cluster.shared::cluster.u32 [%0], %1;" ::"r"(cluster_map(smem_u32(seqs + par * 8 + rank), lane)),
                   "r"(m)
                   : "memory");
    }
    bool mine = lane >= nb;
    const unsigned mine_addr = smem_u32(seqs + par * 8 + (lane & 7));
    const long long cap = wait_cap(w, 1ll << 22);
    const bool poisoned = wait_poisoned(w, m);
    long long it = 0;
    int good = 1;
    for (;;) {
      if (!mine) {
        unsigned sq;
        asm volatile("ld.acquire.cluster.shared::cta.u32 %0, [%1];" : "=r"(sq) : "r"(mine_addr) : "memory");
        mine = sq == m && !poisoned;
      }
      if (__all_sync(0xffffffffu, mine)) break;
      bool stop = ++it > cap;
      if (lane == 0 && (it & 1023) == 0) stop = stop || (*(volatile int*)w.status & XR_S_BARRIER);
      if (__any_sync(0xffffffffu, stop)) {
        if (lane == 0) atomicOr(w.status, XR_S_BARRIER);
        good = 0;
        break;
      }
    }
    if (lane < nb) {
      const float* src = fslots + (par * 8 + lane) * 16;
#pragma unroll
      for (int k = 0; k < NV; ++k) t[k] = src[k];
    } else {
#pragma unroll
      for (int k = 0; k < NV; ++k) t[k] = 0.0f;
    }
    return good;
  }
  // Totals of the entries over lanes 0..7 of warp 0, a fixed tree (the same in every block).
  __device__ static float rank_totalf(float t) {
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    return t;
  }
  __device__ static double rank_total(double t) {
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    return t;
  }
  __device__ bool sync(const XrWork& w) const {
    __shared__ int ok;
    __syncthreads();
    const unsigned par = ++count & 1;
    if (threadIdx.x < 32) {
      if (threadIdx.x == 0) asm volatile("fence.acq_rel.cluster;" ::: "memory");
      double t[1];
      const bool g = exchange<0>(w, nullptr, par, t);
      if (threadIdx.x == 0) ok = g;
    }
    __syncthreads();
    return ok;
  }
  template <int NV, class Post>
  __device__ bool reduce(const XrWork& w, double* v, double* smem, int slot, Post post) const {
    static_assert(NV <= 8, "at most eight values per reduction");
    __shared__ int ok;
    double* res = result_slot(smem, slot);
    const unsigned par = ++count & 1;
    if (threadIdx.x < 32) {
      double t[NV > 0 ? NV : 1];
      const bool g = exchange<NV>(w, v, par, t);
#pragma unroll
      for (int k = 0; k < NV; ++k) t[k] = rank_total(t[k]);
      if (threadIdx.x == 0) {
        ok = g;
        for (int k = 0; k < NV; ++k) res[k] = t[k];
        post(res);
      }
    }
    __syncthreads();
    for (int k = 0; k < NV; ++k) v[k] = res[k];
    return ok;
  }
};

template <int NV, class Team, class Post>
__device__ bool team_sum(const Team& team, const XrWork& w, double* v, double* smem, int slot, Post post) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0)
    for (int k = 0; k < NV; ++k) smem[k * 32 + wid] = v[k];
  __syncthreads();
  if (wid == 0)
    for (int k = 0; k < NV; ++k) {
      double t = lane < nw ? smem[k * 32 + lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
      v[k] = t;
    }
  return team.template reduce<NV>(w, v, smem, slot, post);
}

// Per-row solver state of a block with at most 32 rows (the grid layout), indexed by row - r0.
template <class T>
struct QeqRows {
  T x[32], p[32], hp[32], di[32], c[32], eta_di[32], g[32];
};

// Block-shared state of one solve: the reductions' buffer, the iteration scalars (written by thread 0
// in the reductions' post hooks, in FP64 and as FP32 copies for the FP32 solve), the tile
// transposition buffers and the per-row state. One instance per kernel serves both team kinds.
struct QeqShared {
  double red[kRedSmem];
  double sc_lam, sc_alpha, sc_step, sc_beta;
  float sf_lam, sf_alpha, sf_step, sf_beta, sf_gz, sf_stop, sf_shift, sf_aold;
  double sd_s1w;  // <1, M^-1 1> of the FP32 row solver's block-Jacobi preconditioner
  // Scalars of the solve formed once, by the thread that runs a reduction's post hook (a division
  // done by every warp would cost the FP64 pipe once per warp): the start multipliers, the target,
  // the floor and the next sweep's stop ratio.
  double sd_l0, sd_lu, sd_target, sd_gfloor, sd_ratio;
  int sc_next;  // the next small system of the block (work sharing)
  int sc_groups;  // preconditioner groups of two or more rows (row solver setup)
  double cred[2][8][8];  // cluster team: partials pushed by the blocks of the cluster
  unsigned cseq[2][8];   // cluster team: exchange number of each pushed entry
  int sc_state;  // 0 iterate, 1 converged, 2 stop
  union {
    double d[32][33];
    float f[32][33];
  } part;
  union {
    double d[4][32];
    float f[4][32];
  } part4;
  QeqRows<double> rd;
  QeqRows<float> rf;
};

template <class T>
__device__ inline QeqRows<T>& qeq_rows(QeqShared& sh);
template <>
__device__ inline QeqRows<double>& qeq_rows<double>(QeqShared& sh) { return sh.rd; }
template <>
__device__ inline QeqRows<float>& qeq_rows<float>(QeqShared& sh) { return sh.rf; }
template <class T>
__device__ inline T (&qeq_part(QeqShared& sh))[32][33];
template <>
__device__ inline double (&qeq_part<double>(QeqShared& sh))[32][33] { return sh.part.d; }
template <>
__device__ inline float (&qeq_part<float>(QeqShared& sh))[32][33] { return sh.part.f; }
template <class T>
__device__ inline T (&qeq_part4(QeqShared& sh))[4][32];
template <>
__device__ inline double (&qeq_part4<double>(QeqShared& sh))[4][32] { return sh.part4.d; }
template <>
__device__ inline float (&qeq_part4<float>(QeqShared& sh))[4][32] { return sh.part4.f; }

template <class T>
__device__ inline T pick(double d, float f) {
  if constexpr (sizeof(T) == 8)
    return d;
  else
    return f;
}

template <class T>
__device__ inline T warp_total_t(T t) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  return t;
}

// Vectors of one conjugate-gradient solve (global, indexed by atom): the projected gradient in two
// buffers used in turn, the search direction, its product with H, and the accumulated step.
template <class T>
struct QeqVecs {
  T* g;
  T* g2;
  T* p;
  T* hp;
  T* y;
  // optional row constants in precision T (D^-1, eta D^-1, row sums), else formed from the FP64 ones
  const T* di = nullptr;
  const T* etadi = nullptr;
  const T* c = nullptr;
};

// Matrix rows of the owning block for the product: shared-memory cache of H'_ij = H_ij / D_jj with
// 16-bit columns (cached), else the global neighbour rows (hval holds H'_ij when `scaled`, else H_ij).
template <class T>
struct QeqMatrix {
  const T* cache_h;
  const unsigned short* cache_j;
  bool cached;
  bool scaled;
  int ebeg;
  T* gstage;  // the whole gradient of the system staged per iteration (or null)
};

// Projected, Jacobi-preconditioned conjugate gradients in precision T on
//   minimise 1/2 y'Hy + g0'y  subject to  sum y = 0,
// starting from y = v.y (its current content, normally 0 or the start point) with the projected
// gradient in v.g. Gould, Hribar and Nocedal's projected CG with z = D^-1 (g - lambda): the products
// use the pre-scaled rows (H z = H'(g - lambda) with row sums c), and the multiplier change of a
// step, alpha <D^-1, Hp> / <D^-1, 1>, is reduced together with p'Hp, so the gradient is written
// already projected and its norm g'D^-1 g is free of cancellation. Stops when that norm is at most
// `stop`, at `max_it` iterations (flagging XR_S_CG when `flag_limit`), or on breakdown.
// Per iteration: one product and two team-wide reductions. Returns the iterations taken, or -1
// when a team barrier gave up.
template <class Team, class T>
__device__ int qeq_cg(const XrWork& w, const double* atab, const Team& team, QeqShared& sh, int a0, int n, int r0,
                      int r1, QeqVecs<T> v, const QeqMatrix<T>& M, double s1, double gz_start, double stop,
                      double gfloor, int max_it, bool flag_limit, int& slot) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const double* DI = &QW(Q_DINV, 0);
  const double* Cr = &QW(Q_C, 0);
  QeqRows<T>& R = qeq_rows<T>(sh);
  auto& part = qeq_part<T>(sh);
  auto& part4 = qeq_part4<T>(sh);
  const bool row_smem = (r1 - r0) <= 32;
  double gz = gz_start;  // meaningful in thread 0
  if (threadIdx.x == 0) {
    sh.sc_beta = 0.0;
    sh.sf_beta = 0.0f;
    sh.sc_lam = 0.0;
    sh.sf_lam = 0.0f;
    sh.sc_state = (!(gz_start > gfloor) || n < 2 || gz_start <= stop) ? 1 : 0;
  }
  if (row_smem && wid == 0 && r0 + lane < r1) {
    const int a = a0 + r0 + lane;
    const double di = DI[a];
    R.x[lane] = v.y[a];
    R.p[lane] = T(0);
    R.hp[lane] = T(0);
    R.di[lane] = T(di);
    R.c[lane] = T(Cr[a]);
    R.eta_di[lane] = T(atom_prm(atab, w.type[a], A_ETA) * di);
    R.g[lane] = v.g[a];
  }
  __syncthreads();
  T* G = v.g;
  T* G2 = v.g2;
  int it = 0;
  while (sh.sc_state == 0) {
    if (++it > max_it) {
      if (flag_limit && threadIdx.x == 0) atomicOr(w.status, XR_S_CG);
      --it;
      break;
    }
    const T lam = pick<T>(sh.sc_lam, sh.sf_lam);
    const T beta = pick<T>(sh.sc_beta, sh.sf_beta);
    // p = -z + beta p,  Hp = -H z + beta Hp,  z = D^-1 (g - lambda); the next buffer gets g - lambda
    if (M.gstage) {  // the whole gradient of the system in shared memory: the gathers stay on-chip
      for (int q = threadIdx.x; q < n; q += blockDim.x) M.gstage[q] = __ldcg(G + a0 + q);
      __syncthreads();
    }
    T php0 = T(0), php1 = T(0);  // lane partials in warp 0: p'Hp and <D^-1, Hp>
    for (int tb = r0; tb < r1; tb += 32) {
      const int r = tb + wid;
      T hz = T(0);
      if (wid < 32 && r < r1) {
        const int a = a0 + r;
        const int eb = w.cnt[a], ee = w.cnt[a + 1];
        if (M.cached && M.gstage) {
          for (int e = eb + lane; e < ee; e += 32) hz += M.cache_h[e - M.ebeg] * M.gstage[M.cache_j[e - M.ebeg]];
        } else if (M.cached) {
          for (int e = eb + lane; e < ee; e += 32) hz += M.cache_h[e - M.ebeg] * __ldcg(G + a0 + M.cache_j[e - M.ebeg]);
        } else {
          for (int e = eb + lane; e < ee; e += 32) {
            const int j = w.edge[e].x;
            const double h = M.scaled ? w.hval[e] : w.hval[e] * __ldcg(DI + j);
            hz += T(h) * __ldcg(G + j);
          }
        }
      }
      if (wid < 32) part[wid][lane] = hz;
      __syncthreads();
      if (wid < 4) {  // lane = row of the tile; warp k adds lanes 8k .. 8k+7 of the row's partials
        T s = part[lane][8 * wid];
#pragma unroll
        for (int k = 1; k < 8; ++k) s += part[lane][8 * wid + k];
        part4[wid][lane] = s;
      }
      __syncthreads();
      if (wid == 0 && tb + lane < r1) {
        const int rr = tb + lane, a = a0 + rr;
        T h = (part4[0][lane] + part4[1][lane]) + (part4[2][lane] + part4[3][lane]);
        const T ga = row_smem ? R.g[lane] : (M.gstage ? M.gstage[rr] : G[a]);
        const T di = row_smem ? R.di[lane] : (v.di ? v.di[a] : T(DI[a]));
        const T etadi = row_smem ? R.eta_di[lane] : (v.etadi ? v.etadi[a] : T(atom_prm(atab, w.type[a], A_ETA) * DI[a]));
        const T cr = row_smem ? R.c[lane] : (v.c ? v.c[a] : T(Cr[a]));
        const T p_old = row_smem ? R.p[lane] : v.p[a];
        const T hp_old = row_smem ? R.hp[lane] : v.hp[a];
        h += etadi * ga - lam * cr;
        const T z = di * (ga - lam);
        const T p = -z + beta * p_old;
        const T hp = -h + beta * hp_old;
        if (row_smem) {
          R.p[lane] = p;
          R.hp[lane] = hp;
          R.g[lane] = ga - lam;
        } else {
          v.p[a] = p;
          v.hp[a] = hp;
          G2[a] = ga - lam;
        }
        php0 += p * hp;
        php1 += di * hp;
      }
    }
    double pHp[2] = {0.0, 0.0};
    if (wid == 0) {
      pHp[0] = double(warp_total_t<T>(php0));
      pHp[1] = double(warp_total_t<T>(php1));
    }
    if (!team.template reduce<2>(w, pHp, sh.red, slot, [&](double* t) {
          // The QEq matrix of a close-packed geometry can have a negative eigenvalue (the reference's
          // direct KKT solve accepts it); CG then takes steps of negative curvature (alpha < 0) and
          // still converges. Only an exactly vanishing or non-finite p'Hp is a breakdown, and a
          // non-positive one at rounding level means the solve has converged.
          const bool rounding = gz <= 1e4 * gfloor;
          if (!(fabs(t[0]) > 0.0) || !isfinite(t[0]) || (t[0] < 0.0 && rounding)) {
            if (!rounding && flag_limit) atomicOr(w.status, XR_S_NONSPD);
            sh.sc_state = 2;
          } else {
            sh.sc_alpha = gz / t[0];
            sh.sc_step = sh.sc_alpha * t[1] / s1;
            sh.sf_alpha = float(sh.sc_alpha);
            sh.sf_step = float(sh.sc_step);
          }
        }))
      return -1;
    slot = slot == 1 ? 2 : 1;
    if (sh.sc_state != 0) break;
    // Step: y += alpha p, g += alpha Hp - (multiplier change), one row per lane of warp 0.
    const T alpha = pick<T>(sh.sc_alpha, sh.sf_alpha);
    const T step_lam = pick<T>(sh.sc_step, sh.sf_step);
    double u[2] = {0, 0};
    if (wid == 0) {
      T u0 = T(0), u1 = T(0);
      for (int rr = r0 + lane; rr < r1; rr += 32) {
        const int a = a0 + rr;
        if (row_smem) {
          const T g = (R.g[lane] + alpha * R.hp[lane]) - step_lam;
          R.x[lane] += alpha * R.p[lane];
          R.g[lane] = g;
          G2[a] = g;  // published for the other rows' products
          u0 += R.di[lane] * g;
          u1 += R.di[lane] * g * g;
        } else {
          const T g = (G2[a] + alpha * v.hp[a]) - step_lam;
          v.y[a] += alpha * v.p[a];
          G2[a] = g;
          const T di = v.di ? v.di[a] : T(DI[a]);
          u0 += di * g;
          u1 += di * g * g;
        }
      }
      u[0] = double(warp_total_t<T>(u0));
      u[1] = double(warp_total_t<T>(u1));
    }
    if (!team.template reduce<2>(w, u, sh.red, slot, [&](double* t) {
          sh.sc_lam = t[0] / s1;
          sh.sf_lam = float(sh.sc_lam);
          const double gz_new = t[1] - sh.sc_lam * t[0];
          if (gz_new <= stop) sh.sc_state = 1;
          sh.sc_beta = gz_new / gz;
          sh.sf_beta = float(sh.sc_beta);
          gz = gz_new;
        }))
      return -1;
    slot = slot == 1 ? 2 : 1;
    T* tmp = G;  // the buffer just written becomes the one read next
    G = G2;
    G2 = tmp;
  }
  if (row_smem && wid == 0 && r0 + lane < r1) v.y[a0 + r0 + lane] = R.x[lane];
  __syncthreads();
  return it;
}

// Every lane of the warp gets the warp's totals of v[0..NV) (fixed shuffle tree: deterministic).
template <int NV>
__device__ inline void warp_sum_all(double* v) {
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = warp_total_t<double>(v[k]);
}

// warp_sum_all after a loop of one row per thread over this block's m rows: the warps past the rows
// hold zeros and skip the shuffle tree, which costs the FP64 pipe as much for idle warps as for busy
// ones.
template <int NV>
__device__ inline void rows_sum_all(double* v, int m) {
  if ((int)(threadIdx.x & ~31u) < m) warp_sum_all<NV>(v);
}

// Lanes per matrix row in the per-row loops over a block's m rows: as many as keep the rows within
// two passes of the block's warps (at least 4), so short rows of small systems do not leave most
// lanes idle; each lane keeps four entries' loads in flight.
__device__ inline int row_group(int m) {
  int g = 32;
  while (g > 4 && m * g > 2048) g >>= 1;
  return g;
}

// Sum of NV floats over the team: every thread passes its values; the block totals are formed in
// warp 0 and, for a cluster or grid team, exchanged and added in rank order; thread 0 of each block
// runs post(t) on the totals t[0..NV) (bit-identical in every block) and the block waits for it.
// Returns false when a team exchange gave up.
template <int NV, class Team, class Post>
__device__ inline bool team_sumf(const Team& team, const XrWork& w, float* v, float* smem, Post post, int* slot) {
  constexpr bool kCluster = std::is_same<Team, ClusterTeam>::value;
  constexpr bool kGrid = std::is_same<Team, GridTeam>::value;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = warp_total_t<float>(v[k]);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) smem[32 * k + wid] = v[k];
  __syncthreads();
  if constexpr (kGrid) {
    float f[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) f[k] = wid == 0 ? warp_total_t<float>(lane < nw ? smem[32 * k + lane] : 0.0f) : 0.0f;
    const bool ok = team.template reducef<NV>(w, f, reinterpret_cast<double*>(smem), *slot, post);
    *slot = *slot == 1 ? 2 : 1;
    return ok;
  }
  bool good = true;
  if (wid == 0) {
    float x[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) x[k] = warp_total_t<float>(lane < nw ? smem[32 * k + lane] : 0.0f);
    if constexpr (kCluster) {
      const unsigned par = ++team.count & 1;
      float t[NV];
      good = team.template exchangef<NV>(w, x, par, t);
#pragma unroll
      for (int k = 0; k < NV; ++k) x[k] = ClusterTeam::rank_totalf(t[k]);
    }
    if (lane == 0) {
      post(x);
      if (!good) smem[32 * NV] = -1.0f;
    }
  }
  if constexpr (kCluster) {
    if (threadIdx.x == 0 && good) smem[32 * NV] = 0.0f;
  }
  __syncthreads();
  if constexpr (kCluster) return smem[32 * NV] == 0.0f;
  return true;
}

// Shared-memory layout of the FP32 row solver, at the start of the kernel's dynamic shared memory,
// for a system of n atoms of which this block owns m rows (r0 .. r1):
//   yt[n4]  D v for every row of the system (v = M^-1 of the vector being multiplied), the vector the
//           product gathers; n4 = n rounded up to a multiple of 4; two such buffers for a cluster
//   own rows, m floats each: the constants D_ii, eta D^-1, c = H w1, w1 = M^-1 1, then the solver's
//           x (the correction), p, s, r, u, and for the pipelined solver of grid teams q, z, w, m~
//   binv[8m] row r of its group's inverse block (columns: the group's rows in order)
//   rp[m + 1] row starts relative to the cache; first[m], size[m] the group of each row (16-bit)
// M is block-Jacobi: groups of at most 8 consecutive own rows whose atoms are joined by distances
// below 1.3 A (molecules), each block H restricted to the group. One-row groups are Jacobi.
// Stop of an FP32 sweep of the row solver: its squared preconditioned norm falls by this factor, or to
// a hundredth of the final target. 1e-10 (1e-5 in norm) for the textbook CG of blocks and clusters,
// 1e-7 (about 3e-4) for the pipelined CG of grid teams.
template <class Team>
__host__ __device__ constexpr double sweep_ratio32() {
  return std::is_same<Team, GridTeam>::value ? 1e-7 : 1e-10;
}

// A team splits a system's rows between its blocks, and each block forms its block-Jacobi groups from
// its own rows. A split between local rows r - 1 and r cuts no group when no bond shorter than
// kGroupBond joins a row of [r, r + kGroupMax - 1) to one of the kGroupMax - 1 rows before r (a group
// only joins rows that close). A molecule cut in two loses its strong intramolecular couplings to the
// plain Jacobi part of the preconditioner: on the 4,608-atom water box that took 84 CG iterations
// instead of 69, on 300-atom clusters 52 instead of 39.
// Whether row i (local) has such a bond to a row in [max(0, i - 7), r): the first bonded atom of that
// window, which k_pairs recorded, lies before r.
__device__ inline bool qeq_row_bonded_before(const XrWork& w, int a0, int i, int r) {
  return __ldcg(w.qb_first + a0 + i) < a0 + r;
}

// The nearest split at or after r (within kGroupMax - 1 rows) that cuts no group, else r; one warp,
// its lanes checking the candidate splits' rows in parallel. Every split is computed once per
// boundary, so neighbouring blocks of a team agree on their common boundary.
__device__ inline int qeq_aligned_split_warp(const XrWork& w, int a0, int n, int r) {
  const int lane = threadIdx.x & 31;
  unsigned bad = 0u;  // bit k: split r + k cuts a group
  for (int c = lane; c < kGroupMax * (kGroupMax - 1); c += 32) {
    const int k = c / (kGroupMax - 1), t = c % (kGroupMax - 1);
    const int b = r + k, i = b + t;
    const bool cut = b > 0 && b < n && i < n && qeq_row_bonded_before(w, a0, i, b);
    if (cut) bad |= 1u << k;
  }
  for (int o = 16; o > 0; o >>= 1) bad |= __shfl_xor_sync(0xffffffffu, bad, o);
  for (int k = 0; k < kGroupMax; ++k)
    if (!(bad >> k & 1u) || r + k >= n) return min(r + k, n);
  return r;
}

struct Rows32 {
  float *yt, *dd, *etadi, *cw, *wv, *x, *p, *s, *rr, *u, *q, *z, *wq, *mt, *binv;
  int* rp;
  unsigned short *first, *size;
  int n4;
  // nyt gathered-vector buffers; nvec per-row vectors (rows32_vectors)
  __device__ Rows32(unsigned char* base, int n, int m, int nyt, int nvec) {
    float* f = reinterpret_cast<float*>(base);
    n4 = (n + 3) / 4 * 4;
    yt = f;
    dd = f + nyt * n4;
    etadi = dd + m;
    cw = etadi + m;
    wv = cw + m;
    x = wv + m;
    p = x + m;
    s = p + m;
    rr = s + m;
    u = rr + m;
    q = u + m;  // q, z, w, m~: the pipelined solver's only
    z = q + m;
    wq = z + m;
    mt = wq + m;
    binv = dd + nvec * m;
    rp = reinterpret_cast<int*>(binv + kGroupMax * m);
    first = reinterpret_cast<unsigned short*>(rp + m + 1);
    size = first + m;
  }
  // FP32 scratch of the setup, 8 per row over dd .. rr
  __device__ float* scratch32() const { return dd; }
  // buffer k of the gathered vector (a cluster team alternates two)
  __device__ float* ytb(int k) const { return yt + (k & 1) * n4; }
};

// Buffers of the gathered vector: two for a cluster team, whose blocks write into each other's.
template <class Team>
__host__ __device__ constexpr int rows32_yt_buffers() {
  return std::is_same<Team, ClusterTeam>::value ? 2 : 1;
}

// Per-row vectors: the constants D, eta D^-1, c, w1 and the textbook solver's x, p, s, r, u; the
// pipelined solver of grid teams adds q, z, w, m~.
template <class Team>
__host__ __device__ constexpr int rows32_vectors() {
  return std::is_same<Team, GridTeam>::value ? 13 : 9;
}

template <class Team>
__host__ __device__ constexpr size_t rows32_bytes(int n, int m) {
  return (4 * (size_t)rows32_yt_buffers<Team>() * ((n + 3) / 4 * 4) + 4 * (size_t)(rows32_vectors<Team>() + kGroupMax) * m +
          4 * (size_t)(m + 1) + 4 * (size_t)m + 15) /
         16 * 16;
}

// Setup of the row solver's preconditioner and constants, once per solve (after the Jacobi diagonal
// and the row cache are in place): the groups, their inverse blocks, w = M^-1 1, D, eta D^-1, the
// row starts, s1 = <1, w> (team total, into sh.sd_s1w) and c = H w. Returns false when a team
// exchange gave up.
template <class Team>
__device__ __noinline__ bool qeq_rows32_setup(const XrWork& w, const double* atab, const Team& team, QeqShared& sh, int a0,
                                              int n, int r0, int r1, const QeqMatrix<float>& M, float* gyt) {
  extern __shared__ __align__(16) unsigned char qeq_dyn[];
  constexpr bool kCluster = std::is_same<Team, ClusterTeam>::value;
  constexpr bool kGrid = std::is_same<Team, GridTeam>::value;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5, tid = threadIdx.x;
  const int m = r1 - r0;
  Rows32 R(qeq_dyn, n, m, rows32_yt_buffers<Team>(), rows32_vectors<Team>());
  const double* DI = &QW(Q_DINV, 0);
  const int gs = row_group(m), sub = lane & (gs - 1), gpw = 32 / gs;
  // 1. for every own row, the latest of the kGroupMax - 1 own rows before it that is bonded to it
  //    (distance below kGroupBond, recorded by k_pairs); rows further back cannot share its group
  int* prev = reinterpret_cast<int*>(R.binv);  // scratch until the inverses are written
  for (int i = tid; i < m; i += blockDim.x) {
    const int last = __ldcg(w.qb_last + a0 + r0 + i);
    prev[i] = last >= a0 + r0 ? last - (a0 + r0) : -1;
  }
  __syncthreads();
  // 2. groups: runs of consecutive rows, each bonded to an earlier row of its run, at most kGroupMax
  if (tid == 0) {
    int start = 0;
    for (int i = 0; i < m; ++i) {
      if (!(i > start && prev[i] >= start && i - start < kGroupMax)) start = i;
      R.first[i] = (unsigned short)start;
    }
    int end = m;
    for (int i = m - 1; i >= 0; --i) {
      R.size[i] = (unsigned short)(end - R.first[i]);
      if (R.first[i] == i) end = i;
    }
  }
  __syncthreads();
  // 3. each row of a group of two or more: its row of the group's block (FP32: the inverse is
  //    stored in FP32), into the scratch. The off-diagonal entries are read from hval, and only
  //    those in the group.
  float* B = R.scratch32();
  for (int ib = wid * gpw; ib < m; ib += nw * gpw) {
    const int i = ib + lane / gs;
    const int k = i < m ? R.size[i] : 1;
    if (__all_sync(0xffffffffu, k < 2)) continue;
    float acc[kGroupMax];
#pragma unroll
    for (int b = 0; b < kGroupMax; ++b) acc[b] = 0.0f;
    if (i < m && k > 1) {
      const int f = R.first[i], a = a0 + r0 + i;
      for (int e = w.cnt[a] + sub; e < w.cnt[a + 1]; e += gs) {
        const int b = int(M.cache_j[e - M.ebeg]) - r0 - f;
        if (b >= 0 && b < k && b != i - f) {
          const float h = float(w.hval[e]);
#pragma unroll
          for (int q = 0; q < kGroupMax; ++q)
            if (q == b) acc[q] += h;
        }
      }
    }
#pragma unroll
    for (int b = 0; b < kGroupMax; ++b)
      for (int o = gs / 2; o > 0; o >>= 1) acc[b] += __shfl_xor_sync(0xffffffffu, acc[b], o);
    if (sub == 0 && i < m && k > 1) {
      const int f = R.first[i];
      const float d = 1.0f / float(DI[a0 + r0 + i]);
#pragma unroll
      for (int b = 0; b < kGroupMax; ++b) B[kGroupMax * i + b] = b == i - f ? d : acc[b];
    }
  }
  // 4. inverse blocks by Gauss-Jordan elimination without pivoting: a group's block is symmetric
  //    and, for a molecule, positive definite, so its pivots are positive; a block with a pivot
  //    that is not (H can be indefinite for close-packed atoms) falls back to Jacobi. Eight lanes
  //    per group, lane r holding row r of the block (rows past the group's size padded with the
  //    identity); the groups' first rows are listed in rp (written in step 5).
  int* list = R.rp;
  if (tid == 0) sh.sc_groups = 0;
  __syncthreads();
  for (int i = tid; i < m; i += blockDim.x)
    if (R.first[i] == i && R.size[i] > 1) list[atomicAdd(&sh.sc_groups, 1)] = i;
  __syncthreads();
  const int ngroups = sh.sc_groups;
  for (int g0 = wid * 4; g0 < ngroups; g0 += nw * 4) {
    const int g = g0 + (lane >> 3), r = lane & 7;
    const bool active = g < ngroups;
    const int f = active ? list[g] : 0;
    const int k = active ? (int)R.size[f] : 0;
    float a[kGroupMax];
#pragma unroll
    for (int q = 0; q < kGroupMax; ++q) a[q] = (r < k && q < k) ? B[kGroupMax * (f + r) + q] : (q == r ? 1.0f : 0.0f);
    bool ok = true;
#pragma unroll
    for (int c = 0; c < kGroupMax; ++c) {
      float pr[kGroupMax];  // pivot row c, from lane c of the eight
#pragma unroll
      for (int q = 0; q < kGroupMax; ++q) pr[q] = __shfl_sync(0xffffffffu, a[q], c, 8);
      const float piv = pr[c];
      ok = ok && piv > 0.0f && isfinite(piv);
      const float inv = 1.0f / piv, fr = a[c];
#pragma unroll
      for (int q = 0; q < kGroupMax; ++q) {
        if (q == c) a[q] = r == c ? inv : -fr * inv;
        else a[q] = r == c ? pr[q] * inv : a[q] - fr * (pr[q] * inv);
      }
    }
    if (active && r < k) {
      const float di = float(DI[a0 + r0 + f + r]);
#pragma unroll
      for (int q = 0; q < kGroupMax; ++q) R.binv[kGroupMax * (f + r) + q] = q >= k ? 0.0f : ok ? a[q] : (q == r ? di : 0.0f);
    }
  }
  __syncthreads();  // the scratch (dd .. rr) is free again
  // 5. Jacobi rows, w = M^-1 1 (the stored inverse rows' sums), D, eta D^-1, the row starts
  double s1[1] = {0.0};
  for (int i = tid; i < m; i += blockDim.x) {
    const int a = a0 + r0 + i;
    const double di = DI[a];
    float wsum = float(di);
    if (R.size[i] < 2) {
      R.binv[kGroupMax * i] = float(di);
      for (int c = 1; c < kGroupMax; ++c) R.binv[kGroupMax * i + c] = 0.0f;
    } else {
      wsum = 0.0f;
      for (int c = 0; c < kGroupMax; ++c) wsum += R.binv[kGroupMax * i + c];
    }
    R.wv[i] = wsum;
    R.dd[i] = float(1.0 / di);
    R.etadi[i] = float(atom_prm(atab, w.type[a], A_ETA) * di);
    R.rp[i] = w.cnt[a] - M.ebeg;
    s1[0] += double(wsum);
  }
  if (tid == 0) R.rp[m] = w.cnt[a0 + r1] - M.ebeg;
  __syncthreads();
  rows_sum_all<1>(s1, m);
  auto keep = [&](double* t) { sh.sd_s1w = t[0]; };
  if (!team_sum<1>(team, w, s1, sh.red, 0, keep)) return false;
  // 5. c = H w: D w of the own rows into every block's yt, then the product over the cached rows
  unsigned remote = 0;
  if constexpr (kCluster) remote = smem_u32(R.yt + r0);
  for (int i = tid; i < m; i += blockDim.x) {
    const float v = R.wv[i] * R.dd[i];
    R.yt[r0 + i] = v;
    if constexpr (kCluster) {
      for (int r = 0; r < team.nb; ++r)
        if (r != team.rank) asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(cluster_map(remote + 4 * i, r)), "f"(v) : "memory");
    }
    if constexpr (kGrid) gyt[a0 + r0 + i] = v;
  }
  if (!team.sync(w)) return false;
  if constexpr (kGrid) {
    for (int q = tid; q < n; q += blockDim.x) R.yt[q] = __ldcg(gyt + a0 + q);
    __syncthreads();
  }
  for (int ib = wid * gpw; ib < m; ib += nw * gpw) {
    const int i = ib + lane / gs;
    float t = 0.0f;
    if (i < m)
      for (int e = R.rp[i] + sub; e < R.rp[i + 1]; e += gs) t += M.cache_h[e] * R.yt[M.cache_j[e]];
    for (int o = gs / 2; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (sub == 0 && i < m) R.cw[i] = t + R.etadi[i] * R.yt[r0 + i];
  }
  __syncthreads();
  return true;
}

// The FP32 solve of a refinement sweep with every vector in shared memory (layout Rows32) for a system
// of at most 1024 atoms solved by one block (rows [0, n)) or by a thread-block cluster. Projected
// PCG with the block-Jacobi M of the setup: z = M^-1 (g - lambda 1) with lambda = <w1, g> / <w1, 1>;
// the product gathers yt = D M^-1 g over the pre-scaled rows (H'_ij = H_ij / D_jj), so
// H z = H'yt - lambda c. g is kept projected (shifted by the multiplier each step), so <g, z> is free
// of cancellation. A group of lanes per row forms the product and its first lane the first update;
// a thread per row the second update and the group products M^-1 g. Two team reductions per
// iteration: p'Hp with <w1, Hp> after the product, the new norm after the preconditioner. In a
// cluster each block writes its rows' D M^-1 g into every other block's yt before the second
// reduction, whose exchange publishes it; the writes alternate between two yt buffers, so that
// the first one cannot reach a block still gathering the setup's vector. Stops when <g, z> falls
// to `ratio` times its start value (the vectors g, Hp and y of the description live in the
// layout's r, s and u). The correction x of the own rows is written to y_out (global, by atom).
template <class Team>
__device__ __noinline__ int qeq_cg_rows32(const XrWork& w, const Team& team, QeqShared& sh, int a0, int n, int r0,
                                          int r1, const QeqMatrix<float>& M, float* y_out, double ratio, int max_it, int* slot) {
  extern __shared__ __align__(16) unsigned char qeq_dyn[];
  constexpr bool kCluster = std::is_same<Team, ClusterTeam>::value;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5, tid = threadIdx.x;
  const int m = r1 - r0;
  Rows32 R(qeq_dyn, n, m, rows32_yt_buffers<Team>(), rows32_vectors<Team>());
  // the row cache: in this block's shared memory, or FP32 rows in global memory
  const bool cache_shared = __isShared(M.cache_h);
  const float* const ch_g = M.cache_h;
  const unsigned short* const cj_g = M.cache_j;
  const float* const ch_s =
      reinterpret_cast<const float*>(qeq_dyn + (cache_shared ? (reinterpret_cast<const unsigned char*>(M.cache_h) - qeq_dyn) : 0));
  const unsigned short* const cj_s = reinterpret_cast<const unsigned short*>(
      qeq_dyn + (cache_shared ? (reinterpret_cast<const unsigned char*>(M.cache_j) - qeq_dyn) : 0));
  const double* G = &QW(Q_G, 0);
  float* red = reinterpret_cast<float*>(sh.red);
  const float s1 = float(sh.sd_s1w);
  // exchange parity: the setup's product gathered buffer 0, so the first publish writes buffer 1 (a
  // cluster's blocks write into each other's; a block alone has one buffer)
  int buf = 1;
  auto yt_of = [&](int k) -> float* { return kCluster ? R.ytb(k) : R.yt; };
  auto publish = [&](int i, float v) {  // D M^-1 g of own row i, here and in the other blocks
    float* yt = yt_of(buf);
    yt[r0 + i] = v;
    if constexpr (kCluster) {
      const unsigned remote = smem_u32(yt + r0 + i);
      for (int r = 0; r < team.nb; ++r)
        if (r != team.rank) asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(cluster_map(remote, r)), "f"(v) : "memory");
    }
  };
  auto group_apply = [&](int i) {  // (M^-1 g)_i over the group of row i
    const int f = R.first[i], k = R.size[i];
    const float* bi = R.binv + kGroupMax * i;
    float t = 0.0f;
    for (int b = 0; b < k; ++b) t += bi[b] * R.rr[f + b];
    return t;
  };
  for (int i = tid; i < m; i += blockDim.x) {
    R.rr[i] = float(__ldcg(G + a0 + r0 + i));
    R.p[i] = 0.0f;
    R.s[i] = 0.0f;
    R.x[i] = 0.0f;
  }
  __syncthreads();
  float u0 = 0.0f, u1 = 0.0f;
  for (int i = tid; i < m; i += blockDim.x) {
    const float y = group_apply(i);
    R.u[i] = y;
    publish(i, y * R.dd[i]);
    u0 += R.wv[i] * R.rr[i];
    u1 += R.rr[i] * y;
  }
  // start: lambda = <w, g> / <w, 1>, and <g - lambda, M^-1 (g - lambda)> = <g, M^-1 g> - lambda <w, g>
  float acc[2] = {u0, u1};
  if (!team_sumf<2>(team, w, acc, red, [&](const float* t) {
        const float lam = t[0] / s1;
        const float gz = t[1] - lam * t[0];
        sh.sf_lam = lam;
        sh.sf_beta = 0.0f;
        sh.sf_gz = gz;
        sh.sf_stop = float(ratio) * gz;
        sh.sc_state = (!(gz > 0.0f) || n < 2) ? 1 : 0;
      }, slot))
    return -1;
  const float* yt = yt_of(buf);
  const float fstop = sh.sf_stop;
  const int gs = row_group(m), sub = lane & (gs - 1), gpw = 32 / gs;
  int it = 0;
  while (sh.sc_state == 0) {
    if (++it > max_it) {
      --it;
      break;
    }
    const float lam = sh.sf_lam, beta = sh.sf_beta;
    // H y over the cached rows (gs lanes per row); the group's first lane then updates the row:
    // z = y - lambda w, Hz = Hy - lambda c, p = -z + beta p, Hp = -Hz + beta Hp, g -= lambda
    float php0 = 0.0f, php1 = 0.0f;
    // four entries per lane in flight: the rows may stream from L2 rather than shared memory
    auto row_dot = [&](const float* ch, const unsigned short* cj, int e, int ee) {
      float s = 0.0f;
      for (; e + 3 * gs < ee; e += 4 * gs) {
        const float h0 = ch[e], h1 = ch[e + gs], h2 = ch[e + 2 * gs], h3 = ch[e + 3 * gs];
        const int j0 = cj[e], j1 = cj[e + gs], j2 = cj[e + 2 * gs], j3 = cj[e + 3 * gs];
        s += h0 * yt[j0];
        s += h1 * yt[j1];
        s += h2 * yt[j2];
        s += h3 * yt[j3];
      }
      for (; e < ee; e += gs) s += ch[e] * yt[cj[e]];
      return s;
    };
    for (int ib = wid * gpw; ib < m; ib += nw * gpw) {
      const int i = ib + lane / gs;
      float s = 0.0f;
      if (i < m)
        s = cache_shared ? row_dot(ch_s, cj_s, R.rp[i] + sub, R.rp[i + 1]) : row_dot(ch_g, cj_g, R.rp[i] + sub, R.rp[i + 1]);
      for (int o = gs / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (sub == 0 && i < m) {
        const float hz = s + R.etadi[i] * yt[r0 + i] - lam * R.cw[i];
        const float z = R.u[i] - lam * R.wv[i];
        const float pv = -z + beta * R.p[i];
        const float hpv = -hz + beta * R.s[i];
        R.p[i] = pv;
        R.s[i] = hpv;
        R.rr[i] -= lam;
        php0 += pv * hpv;
        php1 += R.wv[i] * hpv;
      }
    }
    acc[0] = php0;
    acc[1] = php1;
    if (!team_sumf<2>(team, w, acc, red, [&](const float* t) {
          const float gz = sh.sf_gz;
          if (!(fabsf(t[0]) > 0.0f) || !isfinite(t[0])) {
            sh.sc_state = 2;  // breakdown: the FP64 residual of the sweep decides what follows
          } else {
            sh.sf_alpha = gz / t[0];
            sh.sf_step = sh.sf_alpha * t[1] / s1;
          }
        }, slot))
      return -1;
    if (sh.sc_state != 0) break;
    const float alpha = sh.sf_alpha, step = sh.sf_step;
    for (int i = tid; i < m; i += blockDim.x) {
      R.rr[i] = (R.rr[i] + alpha * R.s[i]) - step;
      R.x[i] += alpha * R.p[i];
    }
    __syncthreads();  // the group products read the other rows of the group
    u0 = 0.0f;
    u1 = 0.0f;
    buf ^= 1;
    for (int i = tid; i < m; i += blockDim.x) {
      const float y = group_apply(i);
      R.u[i] = y;
      publish(i, y * R.dd[i]);
      u0 += R.wv[i] * R.rr[i];
      u1 += R.rr[i] * y;
    }
    acc[0] = u0;
    acc[1] = u1;
    if (!team_sumf<2>(team, w, acc, red, [&](const float* t) {
          const float lamn = t[0] / s1;
          const float gzn = t[1] - lamn * t[0];
          sh.sf_lam = lamn;
          sh.sf_beta = gzn / sh.sf_gz;
          sh.sf_gz = gzn;
          if (gzn <= fstop) sh.sc_state = 1;
        }, slot))
      return -1;
    yt = yt_of(buf);
  }
  for (int i = tid; i < m; i += blockDim.x) y_out[a0 + r0 + i] = R.x[i];
  __syncthreads();
  return it;
}

// The FP32 solve of a refinement sweep of a grid-wide team (this block's rows [r0, r1) of a system
// above the cluster sizes), every vector in shared memory (layout Rows32).
//
// Pipelined projected PCG (Ghysels and Vanroose's recurrences) with the block-Jacobi M of the
// setup, on  minimise 1/2 y'Hy + g0'y  subject to  sum y = 0,  with residual r = -g:
//   u = P r, w = H u with P = M^-1 - w1 w1' / s1 (w1 = M^-1 1, s1 = <1, w1>: z = P r sums to zero);
//   per iteration gamma = r'u, delta = w'u and pi = <w1, w> are reduced together, while the
//   preconditioned m~ = M^-1 w is exchanged in the same team operation; after it m = m~ - w1 pi/s1,
//   n = H m = H m~ - c pi/s1 (c = H w1 from the setup), beta = gamma / gamma_old,
//   alpha = gamma / (delta - beta gamma / alpha_old), and the recurrences
//   z = n + beta z, q = m + beta q, s = w + beta s, p = u + beta p,
//   y += alpha p, r -= alpha s, u -= alpha q, w -= alpha z.
// One grid-wide reduction per iteration instead of the textbook form's two (about 4 us each on the
// water box). The extra recurrences lose accuracy in FP32 over long runs, so a sweep stops at a
// relative norm of about 3e-4 (sweep_ratio32) and the FP64 refinement restarts it: on the water
// box, the C/H/O box and the stream's 500-atom systems an FP32 emulation took 1-5 % more
// iterations than the textbook form, over four sweeps instead of three. Block and cluster teams,
// whose reductions cost far less, keep the textbook form (qeq_cg_rows32): there the extra sweep
// cost more than the saved reductions.
//
// The product gathers yt = D m~ over the pre-scaled rows (H'_ij = H_ij / D_jj). A group of lanes
// per row forms the product and its first lane the updates; a thread per row the partial sums and
// the group products M^-1 w. Every block writes its rows' D m~ to global memory before the
// reduction and stages the whole vector after it, alternating two global buffers (gyt0, gyt1): a
// block writes buffer k & 1 for exchange k only after exchange k - 1, which every block entered
// after staging exchange k - 2's buffer. (Written for any team: a cluster alternates two shared
// buffers the same way.) The iteration stops when gamma falls to `ratio` times its start value.
// The correction y of the own rows is written to y_out (global, indexed by atom).
template <class Team>
__device__ __noinline__ int qeq_cg_rows32_pipelined(const XrWork& w, const Team& team, QeqShared& sh, int a0, int n,
                                                    int r0, int r1, const QeqMatrix<float>& M, float* y_out,
                                                    double ratio, int max_it, float* gyt0, float* gyt1, int* slot) {
  extern __shared__ __align__(16) unsigned char qeq_dyn[];
  constexpr bool kCluster = std::is_same<Team, ClusterTeam>::value;
  constexpr bool kGrid = std::is_same<Team, GridTeam>::value;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5, tid = threadIdx.x;
  const int m = r1 - r0;
  Rows32 R(qeq_dyn, n, m, rows32_yt_buffers<Team>(), rows32_vectors<Team>());
  // the row cache: in this block's shared memory, or FP32 rows in global memory
  const bool cache_shared = __isShared(M.cache_h);
  const float* const ch_g = M.cache_h;
  const unsigned short* const cj_g = M.cache_j;
  const float* const ch_s =
      reinterpret_cast<const float*>(qeq_dyn + (cache_shared ? (reinterpret_cast<const unsigned char*>(M.cache_h) - qeq_dyn) : 0));
  const unsigned short* const cj_s = reinterpret_cast<const unsigned short*>(
      qeq_dyn + (cache_shared ? (reinterpret_cast<const unsigned char*>(M.cache_j) - qeq_dyn) : 0));
  const double* G = &QW(Q_G, 0);
  float* red = reinterpret_cast<float*>(sh.red);
  const float s1 = float(sh.sd_s1w);
  // exchange parity: the setup's product gathered buffer 0, so the first exchange writes buffer 1
  int buf = 1;
  auto yt_of = [&](int k) -> float* { return kCluster ? R.ytb(k) : R.yt; };
  auto publish = [&](int i, float v) {  // D m~ of own row i, here and in the other blocks
    float* yt = yt_of(buf);
    yt[r0 + i] = v;
    if constexpr (kCluster) {
      const unsigned remote = smem_u32(yt + r0 + i);
      for (int r = 0; r < team.nb; ++r)
        if (r != team.rank) asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(cluster_map(remote, r)), "f"(v) : "memory");
    }
    if constexpr (kGrid) (buf ? gyt1 : gyt0)[a0 + r0 + i] = v;  // the other blocks stage it after the reduction
  };
  auto stage = [&]() {  // a grid team's whole yt from global memory, after the reduction that published it
    if constexpr (kGrid) {
      const float* src = (buf ? gyt1 : gyt0) + a0;
      // 16-byte loads from the first 16-byte boundary on; the few elements before it and after the
      // last whole vector one by one
      const int head = min(n, int((16 - (reinterpret_cast<uintptr_t>(src) & 15)) & 15) / 4);
      const int nv4 = (n - head) / 4;
      const float4* src4 = reinterpret_cast<const float4*>(src + head);
      for (int q = tid; q < nv4; q += blockDim.x) {
        const float4 v = __ldcg(src4 + q);
        float* d = R.yt + head + 4 * q;
        d[0] = v.x;
        d[1] = v.y;
        d[2] = v.z;
        d[3] = v.w;
      }
      const int rest = head + 4 * nv4;
      if (tid < head) R.yt[tid] = __ldcg(src + tid);
      if (tid < n - rest) R.yt[rest + tid] = __ldcg(src + rest + tid);
      __syncthreads();
    }
  };
  auto group_apply = [&](const float* v, int i) {  // (M^-1 v)_i over the group of row i
    const int f = R.first[i], k = R.size[i];
    const float* bi = R.binv + kGroupMax * i;
    float t = 0.0f;
    for (int b = 0; b < k; ++b) t += bi[b] * v[f + b];
    return t;
  };
  // lanes per row: the fewest that take the block's rows in one pass over its warps (a block of 33
  // rows would otherwise give its first warp a second row, and the team waits for that block)
  int gs = 32;
  while (gs > 4 && m * gs > (int)blockDim.x) gs >>= 1;
  const int sub = lane & (gs - 1), gpw = 32 / gs;
  // The product H'yt over the cached rows (gs lanes per row, four entries per lane in flight: the rows
  // may stream from L2 rather than shared memory); the first lane of the row's group then runs
  // epi(i, sum) with the off-diagonal sum (the diagonal term is etadi * yt).
  auto product = [&](auto epi) {
    const float* yt = yt_of(buf);
    auto row_dot = [&](const float* ch, const unsigned short* cj, int e, int ee) {
      float t = 0.0f;
      for (; e + 3 * gs < ee; e += 4 * gs) {
        const float h0 = ch[e], h1 = ch[e + gs], h2 = ch[e + 2 * gs], h3 = ch[e + 3 * gs];
        const int j0 = cj[e], j1 = cj[e + gs], j2 = cj[e + 2 * gs], j3 = cj[e + 3 * gs];
        t += h0 * yt[j0];
        t += h1 * yt[j1];
        t += h2 * yt[j2];
        t += h3 * yt[j3];
      }
      for (; e < ee; e += gs) t += ch[e] * yt[cj[e]];
      return t;
    };
    for (int ib = wid * gpw; ib < m; ib += nw * gpw) {
      const int i = ib + lane / gs;
      float t = 0.0f;
      if (i < m)
        t = cache_shared ? row_dot(ch_s, cj_s, R.rp[i] + sub, R.rp[i + 1]) : row_dot(ch_g, cj_g, R.rp[i] + sub, R.rp[i + 1]);
      for (int o = gs / 2; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
      if (sub == 0 && i < m) epi(i, t + R.etadi[i] * yt[r0 + i]);
    }
  };
  // start: r = -g0, u~ = M^-1 r exchanged with the reduction of <w1, r> and <r, u~>; then
  // u = u~ - w1 <w1, r>/s1 and w = H u = H u~ - c <w1, r>/s1
  for (int i = tid; i < m; i += blockDim.x) {
    R.rr[i] = -float(__ldcg(G + a0 + r0 + i));
    R.x[i] = 0.0f;
    R.p[i] = 0.0f;
    R.s[i] = 0.0f;
    R.q[i] = 0.0f;
    R.z[i] = 0.0f;
  }
  __syncthreads();
  float acc[3] = {0.0f, 0.0f, 0.0f};
  for (int i = tid; i < m; i += blockDim.x) {
    const float t = group_apply(R.rr, i);
    R.u[i] = t;
    publish(i, t * R.dd[i]);
    acc[0] += R.wv[i] * R.rr[i];
    acc[1] += R.rr[i] * t;
  }
  if (!team_sumf<2>(team, w, acc, red, [&](const float* t) {
        const float shift = t[0] / s1;
        const float gam = t[1] - shift * t[0];  // <r, P r>
        sh.sf_shift = shift;
        sh.sf_stop = float(ratio) * gam;
        sh.sc_state = (!(gam > 0.0f) || n < 2) ? 1 : 0;
      }, slot))
    return -1;
  stage();
  if (sh.sc_state == 0) {
    const float shift = sh.sf_shift;
    product([&](int i, float hv) {
      R.wq[i] = hv - shift * R.cw[i];
      R.u[i] -= shift * R.wv[i];
    });
    __syncthreads();  // the group products read the other rows of the group
  }
  const float fstop = sh.sf_stop;
  int it = 0;
  while (sh.sc_state == 0) {
    buf ^= 1;
    acc[0] = acc[1] = acc[2] = 0.0f;
    for (int i = tid; i < m; i += blockDim.x) {
      const float t = group_apply(R.wq, i);
      R.mt[i] = t;
      publish(i, t * R.dd[i]);
      acc[0] += R.rr[i] * R.u[i];
      acc[1] += R.wq[i] * R.u[i];
      acc[2] += R.wv[i] * R.wq[i];
    }
    const bool more = it < max_it;
    if (!team_sumf<3>(team, w, acc, red, [&](const float* t) {
          const float gam = t[0], dlt = t[1];
          if (gam <= fstop || !more) {
            sh.sc_state = 1;
            return;
          }
          const float beta = it == 0 ? 0.0f : gam / sh.sf_gz;
          const float php = it == 0 ? dlt : dlt - beta * gam / sh.sf_aold;  // p'Hp
          if (!(fabsf(php) > 0.0f) || !isfinite(php) || !isfinite(gam)) {
            sh.sc_state = 2;  // breakdown: the FP64 residual of the sweep decides what follows
            return;
          }
          const float alpha = gam / php;
          sh.sf_beta = beta;
          sh.sf_alpha = alpha;
          sh.sf_aold = alpha;
          sh.sf_gz = gam;
          sh.sf_shift = t[2] / s1;
        }, slot))
      return -1;
    if (sh.sc_state != 0) break;
    stage();
    const float alpha = sh.sf_alpha, beta = sh.sf_beta, shift = sh.sf_shift;
    product([&](int i, float hv) {
      const float nv = hv - shift * R.cw[i];
      const float mv = R.mt[i] - shift * R.wv[i];
      const float zv = nv + beta * R.z[i];
      const float qv = mv + beta * R.q[i];
      const float sv = R.wq[i] + beta * R.s[i];
      const float pv = R.u[i] + beta * R.p[i];
      R.z[i] = zv;
      R.q[i] = qv;
      R.s[i] = sv;
      R.p[i] = pv;
      R.x[i] += alpha * pv;
      R.rr[i] -= alpha * sv;
      R.u[i] -= alpha * qv;
      R.wq[i] -= alpha * zv;
    });
    __syncthreads();  // the group products read the other rows of the group
    ++it;
  }
  for (int i = tid; i < m; i += blockDim.x) y_out[a0 + r0 + i] = R.x[i];
  __syncthreads();
  return it;
}

// FP64 gradient of the QEq energy at the current charges X for the owned rows, projected onto
// sum q = Q: g = H x + chi, lambda = <D^-1, g> / <D^-1, 1>, G = g - lambda, and its norm
// <D^-1, G^2> (from the projected values, so free of cancellation). Two team reductions.
template <class Team>
__device__ bool qeq_residual(const XrWork& w, const double* atab, const Team& team, QeqShared& sh, int a0, int r0, int r1,
                             double s1, double target, double* gz_out, int& slot, bool adjoint) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double* X = &QW(Q_X, 0);
  double* G = &QW(Q_G, 0);
  const double* DI = &QW(Q_DINV, 0);
  const int gs = row_group(r1 - r0), sub = lane & (gs - 1), gpw = 32 / gs;
  double acc[1] = {0.0};
  for (int rb = r0 + wid * gpw; rb < r1; rb += nw * gpw) {
    const int r = rb + lane / gs, a = a0 + r;
    double hx = 0;
    if (r < r1) {
      const int ee = w.cnt[a + 1];
      int e = w.cnt[a] + sub;
      for (; e + 3 * gs < ee; e += 4 * gs) {
        int j[4];
        double h[4], x[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          j[u] = w.edge[e + u * gs].x;
          h[u] = w.hval[e + u * gs];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) x[u] = __ldcg(X + j[u]);
#pragma unroll
        for (int u = 0; u < 4; ++u) hx += h[u] * x[u];
      }
      for (; e < ee; e += gs) hx += w.hval[e] * __ldcg(X + w.edge[e].x);
    }
    for (int o = gs / 2; o > 0; o >>= 1) hx += __shfl_xor_sync(0xffffffffu, hx, o);
    if (sub == 0 && r < r1) G[a] = hx;  // finished one row per thread below
  }
  __syncthreads();
  for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    const int a = a0 + r, t = w.type[a];
    const double g = G[a] + atom_prm(atab, t, A_ETA) * X[a] + (adjoint ? w.qrhs[a] : atom_prm(atab, t, A_CHI));
    G[a] = g;
    acc[0] += DI[a] * g;
  }
  rows_sum_all<1>(acc, r1 - r0);
  if (!team_sum<1>(team, w, acc, sh.red, slot, [&](double* t) { t[0] = t[0] / s1; })) return false;
  slot = slot == 1 ? 2 : 1;
  const double lam = acc[0];
  double acc2[1] = {0.0};
  for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    const int a = a0 + r;
    const double g = G[a] - lam;
    G[a] = g;
    acc2[0] += DI[a] * g * g;
  }
  rows_sum_all<1>(acc2, r1 - r0);
  // (and the stop ratio of the row solver's next sweep from here: sweep_ratio32 of the norm, no
  // further than 1e-2 of the target)
  auto ratio = [&](double* t) {
    sh.sd_ratio = t[0] > 0.0 ? fmax(sweep_ratio32<Team>() * t[0], 0.01 * target) / t[0] : 1.0;
  };
  if (!team_sum<1>(team, w, acc2, sh.red, slot, ratio)) return false;
  slot = slot == 1 ? 2 : 1;
  *gz_out = acc2[0];
  return true;
}

// Rows [r0, r1) of the system starting at atom a0 belong to this block. The matrix-vector product
// runs on tiles of 32 rows, one row per warp; the lanes' partial row sums are transposed through
// shared memory so that one warp owns the 32 rows of a tile, one row per lane, for the row
// reductions and every per-row scalar update. On this part an FP64 instruction costs the FP64 pipe
// the same whether one lane or 32 are active, so scalar row work done by lane 0 of 32 warps would
// cost 32 times the issue slots of the same work spread over the lanes of one warp.
//
// Mixed precision (when the block's rows fit the shared-memory cache as FP32): iterative refinement
// around FP32 solves. Each sweep solves the correction problem (the current projected FP64
// gradient as g0) with the FP32 projected CG to a relative norm of 1e-5, adds the correction to
// the FP64 charges and recomputes the projected gradient in FP64 from the unscaled matrix. FP32
// issues at 64 times the FP64 rate here, so a sweep costs a fraction of the FP64 iterations it
// replaces, and the FP64 residual decides convergence against the same tolerance as the FP64
// solve. If a sweep fails to cut the residual by 1e3 the FP64 solve takes over from the current
// charges.
//
// When `cache_j` is non-null the block's matrix rows are kept in shared memory (FP32 in the mixed
// mode, else FP64); when `gstage` is non-null the whole gradient is staged in shared memory.
template <class Team>
__device__ void qeq_solve(const XrWork& w, const double* atab, const Team& team, int a0, int n, int r0, int r1,
                          double Q, bool warm, QeqShared& sh, unsigned char* dyn, int dyn_bytes, bool adjoint) {
  double* smem = sh.red;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double* X = &QW(Q_X, 0);
  double* G = &QW(Q_G, 0);
  double* DI = &QW(Q_DINV, 0);
  double* Cr = &QW(Q_C, 0);
  float* F = reinterpret_cast<float*>(&QW(7, 0));  // FP32 vectors and row constants: 8 x A floats in slots 7..10
  auto noop = [](double*) {};
  const double x0 = Q == 0.0 ? 0.0 : Q / n;
  const int ebeg = w.cnt[a0 + r0], eend = w.cnt[a0 + r1];
  const int nent = eend - ebeg;
  // Shared-memory plan: [gradient stage: n doubles when it takes at most half the space][row cache].
  // The cache holds FP32 values + 16-bit columns (6 B per entry, mixed precision) when the block's
  // rows fit, else FP64 values + columns (10 B), else nothing (rows read from global memory).
  // A block that solves a system of at most 1024 atoms alone keeps every row's FP32 state in shared
  // memory instead, and so does each block of a cluster team for its rows plus the whole vector the
  // product gathers (layout Rows32: 4 B per atom of the system, 8 B in a cluster, and 76 B per own row, 92 B in a
  // grid team), and at least
  // the n doubles of the FP64 stage of a fallback.
  constexpr bool kBlock = std::is_same<Team, BlockTeam>::value;
  constexpr bool kCluster = std::is_same<Team, ClusterTeam>::value;
  // (the same for every block of a team: it depends on the system only)
  constexpr bool kGridTeam = std::is_same<Team, GridTeam>::value;
  int team_rows = n;  // the most rows any block of the team owns (the same value in every block)
  if constexpr (kGridTeam) team_rows = min(n, ((n + team.nb - 1) / team.nb + 31) / 32 * 32 + kGroupMax);
  const bool small_rows =
      dyn != nullptr && ((kBlock || kCluster) ? n <= 1024 : rows32_bytes<Team>(n, team_rows) <= (size_t)dyn_bytes / 2);
  const int stage_n = (dyn != nullptr && (small_rows || n * 8 <= dyn_bytes / 2)) ? n : 0;
  const size_t stage_bytes =
      small_rows ? std::max<size_t>(rows32_bytes<Team>(n, r1 - r0), 8 * (size_t)n) : 8 * (size_t)stage_n;
  void* gstage = stage_n > 0 ? dyn : nullptr;
  unsigned char* region = dyn != nullptr ? dyn + stage_bytes : nullptr;
  const long long region_bytes = dyn != nullptr ? dyn_bytes - (long long)stage_bytes : 0;
  // Rows that do not fit are kept in FP32 in global memory (L2-resident for a batch) instead, so the
  // solve stays mixed-precision; FP64 rows from hval are the path without that buffer.
  const bool cols16 = n <= 65536;
  const bool fits32 = region != nullptr && cols16 && nent <= region_bytes / 6;
  const bool glob32 = !fits32 && cols16 && w.qch != nullptr;
  const bool mixed = fits32 || glob32;
  const bool cached64 = !mixed && region != nullptr && cols16 && nent <= region_bytes / 10;
  void* cache_h = region;
  unsigned short* cache_j = nullptr;
  if (fits32) cache_j = reinterpret_cast<unsigned short*>(region + 4 * (size_t)(region_bytes / 6));
  if (glob32) {
    cache_h = w.qch + ebeg;
    cache_j = w.qcj + ebeg;
  }
  if (cached64) cache_j = reinterpret_cast<unsigned short*>(region + 8 * (size_t)(region_bytes / 10));
  // 1. Jacobi diagonal (eta + self-image shields) of the owned rows, and the start point: the
  //    uniform x0 = Q/n, or the caller's charges of an earlier step (already summing to Q).
  const int gs = row_group(r1 - r0), sub = lane & (gs - 1), gpw = 32 / gs;
  for (int rb = r0 + wid * gpw; rb < r1; rb += nw * gpw) {
    const int r = rb + lane / gs, a = a0 + r;
    double d = 0;
    if (r < r1) {
      const int ee = w.cnt[a + 1];
      int e = w.cnt[a] + sub;
      for (; e + 3 * gs < ee; e += 4 * gs) {
        int j[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) j[u] = w.edge[e + u * gs].x;
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (j[u] == a) d += w.hval[e + u * gs];
      }
      for (; e < ee; e += gs)
        if (w.edge[e].x == a) d += w.hval[e];
    }
    if (__any_sync(0xffffffffu, d != 0.0))  // self images: small periodic cells only
      for (int o = gs / 2; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
    if (sub == 0 && r < r1) DI[a] = d;  // the shield sum; the diagonal follows one row per thread
  }
  __syncthreads();
  for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    const int a = a0 + r;
    const double di = 1.0 / (atom_prm(atab, w.type[a], A_ETA) + DI[a]);
    DI[a] = di;
    F[5 * w.A + a] = float(di);
    X[a] = warm ? w.qguess[a] : x0;
  }
  if (!team.sync(w)) return;
  // 2. Pre-scaled rows H'_ij = H_ij / D_jj (cached in FP32 or FP64, or in hval in place), row sums
  //    c_i = sum_j H'_ij + eta_i D_ii^-1, and the start gradient g = H x + chi. The FP64 sums are
  //    formed only where they are read: the row sums r_i = sum_j H_ij for a uniform start x0 != 0,
  //    H x for a warm start, and c for the solves other than the shared-memory row solver (whose
  //    FP64 fallback forms c itself). A cold neutral start with FP32 rows needs no FP64 per entry:
  //    its cache entries are hval's FP32 copy times the FP32 diagonal.
  const bool need_rs = x0 != 0.0;
  const bool need_cs = !(small_rows && mixed);
  const bool fast = mixed && !need_rs && !need_cs && !warm;
  const float* const DI32 = F + 5 * w.A;
  for (int rb = r0 + wid * gpw; rb < r1 && fast; rb += nw * gpw) {
    const int r = rb + lane / gs, a = a0 + r;
    if (r < r1) {
      float* const ch = reinterpret_cast<float*>(cache_h);
      const int ee = w.cnt[a + 1];
      int e = w.cnt[a] + sub;
      for (; e + 3 * gs < ee; e += 4 * gs) {
        int j[4];
        float h[4], dj[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          j[u] = w.edge[e + u * gs].x;
          h[u] = w.qch[e + u * gs];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) dj[u] = __ldcg(DI32 + j[u]);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          cache_j[e + u * gs - ebeg] = (unsigned short)(j[u] - a0);
          ch[e + u * gs - ebeg] = h[u] * dj[u];
        }
      }
      for (; e < ee; e += gs) {
        const int j = w.edge[e].x;
        const float h = w.qch[e];
        cache_j[e - ebeg] = (unsigned short)(j - a0);
        ch[e - ebeg] = h * __ldcg(DI32 + j);
      }
    }
  }
  for (int rb = r0 + wid * gpw; rb < r1 && !fast; rb += nw * gpw) {
    const int r = rb + lane / gs, a = a0 + r;
    double rs = 0, cs = 0, hx = 0;
    auto put = [&](int e, int j, double h, double dj, double xj) {
      const double hp = h * dj;
      rs += h;
      cs += hp;
      if (warm) hx += h * xj;
      if (mixed) {
        cache_j[e - ebeg] = (unsigned short)(j - a0);
        reinterpret_cast<float*>(cache_h)[e - ebeg] = float(hp);
      } else if (cached64) {
        cache_j[e - ebeg] = (unsigned short)(j - a0);
        reinterpret_cast<double*>(cache_h)[e - ebeg] = hp;
      } else {
        w.hval[e] = hp;  // scaled in place; hval is not read after the solve
      }
    };
    if (r < r1) {
      const int ee = w.cnt[a + 1];
      int e = w.cnt[a] + sub;
      for (; e + 3 * gs < ee; e += 4 * gs) {
        int j[4];
        double h[4], dj[4], xj[4] = {0, 0, 0, 0};
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          j[u] = w.edge[e + u * gs].x;
          h[u] = w.hval[e + u * gs];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          dj[u] = __ldcg(DI + j[u]);
          if (warm) xj[u] = __ldcg(X + j[u]);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) put(e + u * gs, j[u], h[u], dj[u], xj[u]);
      }
      for (; e < ee; e += gs) {
        const int j = w.edge[e].x;
        put(e, j, w.hval[e], __ldcg(DI + j), warm ? __ldcg(X + j) : 0.0);
      }
    }
    for (int o = gs / 2; o > 0; o >>= 1) {
      if (need_rs) rs += __shfl_xor_sync(0xffffffffu, rs, o);
      if (need_cs) cs += __shfl_xor_sync(0xffffffffu, cs, o);
      if (warm) hx += __shfl_xor_sync(0xffffffffu, hx, o);
    }
    if (sub == 0 && r < r1) {  // the row's sums, finished one row per thread below
      Cr[a] = cs;
      QW(Q_HP, a) = rs;
      G[a] = hx;
    }
  }
  __syncthreads();
  double acc[5] = {0, 0, 0, 0, 0};
  for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    const int a = a0 + r, t = w.type[a];
    const double eta = atom_prm(atab, t, A_ETA), di = DI[a], chi = adjoint ? w.qrhs[a] : atom_prm(atab, t, A_CHI);
    const double gu = need_rs ? x0 * (QW(Q_HP, a) + eta) + chi : chi;
    const double g = warm ? G[a] + eta * X[a] + chi : gu;
    if (need_cs) Cr[a] = Cr[a] + eta * di;
    G[a] = g;
    QW(Q_HP, a) = gu;  // parked for the projection step below
    acc[0] += di;
    acc[1] += di * g;
    acc[2] += di * g * g;
    acc[3] += di * gu;
    acc[4] += di * gu * gu;
  }
  rows_sum_all<5>(acc, r1 - r0);
  if (!team_sum<5>(team, w, acc, smem, 0, [&](double* t) {
        sh.sd_l0 = t[1] / t[0];
        sh.sd_lu = t[3] / t[0];
      }))
    return;
  const double s1 = acc[0];
  // 3. Project the start gradient explicitly (g - lambda with lambda = <D^-1, g> / <D^-1, 1>) and take
  //    its norm from the projected values: sum D^-1 g^2 - lambda sum D^-1 g cancels to rounding noise
  //    of the unprojected gradient when the start is (nearly) the solution, e.g. q = 0 for identical
  //    atoms. The uniform start's projected norm sets the convergence scale.
  const double lam0 = sh.sd_l0, lamu = sh.sd_lu;
  double acc2[3] = {0, 0, 0};  // <D^-1, g~^2>, <D^-1, g~_u^2>, <D^-1, g~>
  for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    {
      const int a = a0 + r;
      const double di = DI[a];
      const double gt = G[a] - lam0;
      const double gut = QW(Q_HP, a) - lamu;
      G[a] = gt;
      acc2[0] += di * gt * gt;
      acc2[1] += di * gut * gut;
      acc2[2] += di * gt;
    }
  }
  rows_sum_all<3>(acc2, r1 - r0);
  // the target: tol^2 of the uniform start's projected norm (= the start's when cold)
  if (!team_sum<3>(team, w, acc2, smem, 1, [&](double* t) {
        sh.sd_target = w.cg_tol * w.cg_tol * t[1];
        sh.sd_gfloor = 1e-28 * fmax(acc[2], acc[4]);
        sh.sd_ratio = t[0] > 0.0 ? fmax(sweep_ratio32<Team>() * t[0], 0.01 * sh.sd_target) / t[0] : 1.0;
      }))
    return;
  const double target = sh.sd_target, gfloor = sh.sd_gfloor;
  double gz = acc2[0];
  int slot = 2;
  int iters = 0;
  bool fp64 = !mixed;
  if (mixed) {
    // 4a. Iterative refinement around FP32 solves of the correction problem.
    const size_t A = w.A;
    QeqVecs<float> v32{F, F + A, F + 2 * A, F + 3 * A, F + 4 * A, F + 5 * A, F + 6 * A, F + 7 * A};
    for (int r = r0 + threadIdx.x; r < r1 && !small_rows; r += blockDim.x) {
      const int a = a0 + r;
      F[5 * A + a] = float(DI[a]);
      F[6 * A + a] = float(atom_prm(atab, w.type[a], A_ETA) * DI[a]);
      F[7 * A + a] = float(Cr[a]);
    }
    QeqMatrix<float> M32{reinterpret_cast<const float*>(cache_h), cache_j, true, true, ebeg,
                         reinterpret_cast<float*>(gstage)};
    if (small_rows && gz > target && gz > gfloor && n >= 2 && !qeq_rows32_setup(w, atab, team, sh, a0, n, r0, r1, M32, v32.g))
      return;
    for (int sweep = 0; sweep < 8; ++sweep) {
      if (!(gz > target) || !(gz > gfloor) || n < 2) break;
      // the iteration limit bounds the FP32 and FP64 iterations together
      const int budget = min(400, w.cg_max_iter - iters);
      if (budget <= 0) break;
      if (!small_rows) {  // the shared-memory solver reads the FP64 gradient itself (published by the
                          // reduction that ended the residual)
        for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
          const int a = a0 + r;
          v32.g[a] = float(G[a]);
          v32.p[a] = 0.0f;
          v32.hp[a] = 0.0f;
          v32.y[a] = 0.0f;
        }
        if (!team.sync(w)) return;
      }
      // the correction's own projected norm starts at gz; the row solver stops at sweep_ratio32 of it
      // per sweep (sd_ratio), the FP32 CG over global rows at 1e-10 (1e-5 in norm), both no further
      // than a hundredth of the final target
      int it = 0;
      if (small_rows) {
        if constexpr (kGridTeam)
          it = qeq_cg_rows32_pipelined(w, team, sh, a0, n, r0, r1, M32, v32.y, sh.sd_ratio, budget, v32.g, v32.g2, &slot);
        else
          it = qeq_cg_rows32(w, team, sh, a0, n, r0, r1, M32, v32.y, sh.sd_ratio, budget, &slot);
      } else {
        it = qeq_cg<Team, float>(w, atab, team, sh, a0, n, r0, r1, v32, M32, s1, gz, fmax(1e-10 * gz, 0.01 * target), 0.0,
                                 budget, false, slot);
      }
      if (it < 0) return;
      iters += it;
      // x += y, then restore sum x = Q exactly: the FP32 step keeps sum y = 0 only to FP32 rounding,
      // and the residual must be taken at a point on the constraint (a uniform shift added after
      // convergence would change the projected gradient)
      double sx[1] = {0.0};
      for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        const int a = a0 + r;
        X[a] += double(v32.y[a]);
        sx[0] += X[a];
      }
      rows_sum_all<1>(sx, r1 - r0);
      if (!team_sum<1>(team, w, sx, smem, slot, [&](double* t) { t[0] = (Q - t[0]) / n; })) return;
      slot = slot == 1 ? 2 : 1;
      const double shift = sx[0];
      for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) X[a0 + r] += shift;
      if (!team.sync(w)) return;
      double gz_new = 0.0;
      if (!qeq_residual(w, atab, team, sh, a0, r0, r1, s1, target, &gz_new, slot, adjoint)) return;
      const bool stalled = gz_new > 1e-3 * gz;
      gz = gz_new;
      if (stalled && gz > target) {
        fp64 = true;  // FP32 solves no longer reduce the residual: finish in FP64
        break;
      }
    }
    if (!fp64 && gz > target && gz > gfloor && n >= 2) fp64 = true;  // sweep limit
  }
  if (fp64) {
    // 4b. FP64 projected CG from the current charges (cold: the start point) to the tolerance.
    if (!need_cs) {  // its row sums c, which the row solver's setup did not need
      for (int rb = r0 + wid * gpw; rb < r1; rb += nw * gpw) {
        const int r = rb + lane / gs, a = a0 + r;
        double cs = 0;
        if (r < r1)
          for (int e = w.cnt[a] + sub; e < w.cnt[a + 1]; e += gs) cs += w.hval[e] * __ldcg(DI + w.edge[e].x);
        for (int o = gs / 2; o > 0; o >>= 1) cs += __shfl_xor_sync(0xffffffffu, cs, o);
        if (sub == 0 && r < r1) Cr[a] = cs + atom_prm(atab, w.type[a], A_ETA) * DI[a];
      }
      __syncthreads();
    }
    QeqVecs<double> v64{G, &QW(Q_G2, 0), &QW(Q_P, 0), &QW(Q_HP, 0), X};
    QeqMatrix<double> M64{reinterpret_cast<const double*>(cache_h), cache_j, cached64, !mixed, ebeg,
                          reinterpret_cast<double*>(gstage)};
    for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
      QW(Q_P, a0 + r) = 0.0;
      QW(Q_HP, a0 + r) = 0.0;
    }
    __syncthreads();
    // what the FP32 sweeps left of the iteration limit (none: the limit is flagged unless converged)
    const int it = qeq_cg<Team, double>(w, atab, team, sh, a0, n, r0, r1, v64, M64, s1, gz, target, gfloor,
                                        max(0, w.cg_max_iter - iters), true, slot);
    if (it < 0) return;
    iters += it;
  }
  if (threadIdx.x == 0) {
    atomicMax(w.counts + 4, iters);
    atomicMax(w.qiters + w.sys_of[a0], iters);
  }
  // 5. Final charges; the constraint is restored exactly against accumulated rounding.
  double sx[1] = {0.0};
  for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) sx[0] += X[a0 + r];
  rows_sum_all<1>(sx, r1 - r0);
  if (!team_sum<1>(team, w, sx, smem, 3, [&](double* t) { t[0] = (Q - t[0]) / n; })) return;
  const double shift = sx[0];
  for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    const int a = a0 + r;
    const double q = X[a] + shift;
    if (adjoint) {
      w.qadj[a] = q;
      continue;
    }
    w.q[a] = q;
    const int t = w.type[a];
    AEV(6, a) = SELF_CONVERSION * (atom_prm(atab, t, A_CHI) * q + 0.5 * atom_prm(atab, t, A_ETA) * q * q);
  }
}

// Dynamic shared memory of the solver kernel: [gradient stage: n doubles][row cache values][row
// cache columns (16-bit, local to the system)]. Each system's solve splits it the same way.
constexpr int kQeqMaxDyn = 208 * 1024;

// The systems solved by one block each, largest first, taken one at a time from a shared counter
// by whichever block is free (a block of a team joins once its team's system is solved).
__device__ void qeq_small_systems(const XrWork& w, const XrFF& ff, const int* small, int nsmall, unsigned* next,
                                  int adjoint, QeqShared& sh, unsigned char* dyn) {
  for (;;) {
    if (threadIdx.x == 0) sh.sc_next = (int)atomicAdd(next, 1u);
    __syncthreads();
    const int k = sh.sc_next;
    __syncthreads();
    if (k >= nsmall) return;
    const XrSystem& S = w.sys[small[k]];
    BlockTeam team;
    qeq_solve(w, atoms_of_system(ff, S), team, S.atom_off, S.natoms, 0, S.natoms, adjoint ? 0.0 : S.total_charge,
              !adjoint && S.has_guess != 0, sh, dyn, kQeqMaxDyn, adjoint != 0);
    __syncthreads();
  }
}

// Cooperative solver launch for a batch: the first nteam blocks form teams, one per large system
// (map[b] = {system, rank, team size, first block of the team}); each team splits its system's rows
// and synchronises through its own bounded counter. The remaining blocks each solve a share of the
// small systems (small[k], k = b - nteam, b - nteam + (gridDim.x - nteam), ...) alone, with block
// barriers only. All blocks are co-resident (cooperative launch, one block per SM).
__global__ void __launch_bounds__(1024, 1) k_qeq_grid(XrWork w, XrFF ff, const int4* map, int nteam, const int* small,
                                                      int nsmall, int adjoint) {
  __shared__ QeqShared sh;
  extern __shared__ __align__(16) unsigned char dyn[];
  if ((int)blockIdx.x < nteam) {
    const int4 m = map[blockIdx.x];
    const XrSystem& S = w.sys[m.x];
    // the rows of this block (k_qeq_splits: equal shares of 32-row multiples, no molecule cut)
    const int r0 = w.qsplit[2 * blockIdx.x], r1 = max(r0, w.qsplit[2 * blockIdx.x + 1]);
    GridTeam team{w.barrier + m.w, w.red + (size_t)32 * m.w, m.z, m.y};
    qeq_solve(w, atoms_of_system(ff, S), team, S.atom_off, S.natoms, r0, r1, adjoint ? 0.0 : S.total_charge,
              !adjoint && S.has_guess != 0, sh, dyn, kQeqMaxDyn, adjoint != 0);
    __syncthreads();
  }
  qeq_small_systems(w, ff, small, nsmall, w.barrier + nteam, adjoint, sh, dyn);
}

// Row splits of the QEq teams, one warp per split, before the solver (so that its registers stay with
// the solve). Cluster teams (map == null): qsplit[k * (csize + 1) + q] for system big[k] and
// q = 0 .. csize, at about the same number of matrix entries per block. Grid teams: qsplit[2 b] and
// qsplit[2 b + 1] for team block b (map[b] = {system, rank, team size, first block}), at the team's
// equal shares of 32-row multiples. Each split then moves to the nearest one that cuts no molecule.
__global__ void k_qeq_splits(XrWork w, const int* big, int nbig, int csize, const int4* map, int nteam) {
  const int t = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  int sys, r;
  if (map == nullptr) {
    if (t >= nbig * (csize + 1)) return;
    const int k = t / (csize + 1), q = t % (csize + 1);
    sys = big[k];
    const XrSystem& S = w.sys[sys];
    const int* cnt = w.cnt + S.atom_off;
    const long long E = cnt[S.natoms] - cnt[0];
    r = S.natoms;
    if (q < csize) {
      const long long target = cnt[0] + E * q / csize;
      int lo = 0, hi = S.natoms;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (cnt[mid] < target) lo = mid + 1;
        else hi = mid;
      }
      r = lo;
    }
  } else {
    if (t >= 2 * nteam) return;
    const int4 m = map[t >> 1];
    sys = m.x;
    const int n = w.sys[sys].natoms;
    const int per = ((n + m.z - 1) / m.z + 31) / 32 * 32;
    r = min(n, (m.y + (t & 1)) * per);
  }
  const XrSystem& S = w.sys[sys];
  const int v = qeq_aligned_split_warp(w, S.atom_off, S.natoms, r);
  if (lane == 0) w.qsplit[t] = v;
}

// Solver on thread-block clusters (4 or 8 blocks, set at launch), one block per SM: the systems of
// `big` (largest first) are each solved by a whole cluster, rows split over its blocks, with
// reductions through distributed shared memory; then every block takes systems of `small` alone.
// A cluster's leader draws the next big system from a counter and the draw reaches the other
// blocks through an exchange. Ordinary launch: no block waits on a block of another cluster.
__global__ void __launch_bounds__(1024, 1) k_qeq_cluster(XrWork w, XrFF ff, const int* big, int nbig, const int* small,
                                                         int nsmall, int adjoint) {
  __shared__ QeqShared sh;
  extern __shared__ __align__(16) unsigned char dyn[];
  const unsigned rank = cluster_rank(), nb = cluster_size();
  if (threadIdx.x < 16) (&sh.cseq[0][0])[threadIdx.x] = 0u;
  cluster_barrier_all();  // every block's sequence words are zero before the first remote write
  ClusterTeam team{&sh.cred[0][0][0], &sh.cseq[0][0], (int)nb, (int)rank};
  auto noop = [](double*) {};
  for (;;) {
    double v[1] = {0.0};
    if (threadIdx.x < 32) {
      double d = 0.0;
      if (rank == 0 && threadIdx.x == 0) d = (double)atomicAdd(w.barrier, 1u);
      v[0] = __shfl_sync(0xffffffffu, d, 0);
    }
    if (!team.template reduce<1>(w, v, sh.red, 0, noop)) break;
    const int k = (int)v[0];
    if (k >= nbig) break;
    const XrSystem& S = w.sys[big[k]];
    // the rows of this block (k_qeq_splits: equal numbers of matrix entries, no molecule cut)
    const int r0 = w.qsplit[k * (nb + 1) + rank], r1 = max(r0, w.qsplit[k * (nb + 1) + rank + 1]);
    qeq_solve(w, atoms_of_system(ff, S), team, S.atom_off, S.natoms, r0, r1, adjoint ? 0.0 : S.total_charge,
              !adjoint && S.has_guess != 0, sh, dyn, kQeqMaxDyn, adjoint != 0);
    __syncthreads();
    if (*(volatile int*)w.status & XR_S_BARRIER) break;
  }
  qeq_small_systems(w, ff, small, nsmall, w.barrier + 1, adjoint, sh, dyn);
  cluster_barrier_all();  // no block leaves while a peer may still write into its shared memory
}

// Fallback without cooperative launch: one block per system, no shared-memory row cache.
__global__ void __launch_bounds__(1024, 1) k_qeq_block(XrWork w, XrFF ff, int adjoint) {
  __shared__ QeqShared sh;
  const XrSystem& S = w.sys[blockIdx.x];
  BlockTeam team;
  qeq_solve(w, atoms_of_system(ff, S), team, S.atom_off, S.natoms, 0, S.natoms, adjoint ? 0.0 : S.total_charge,
            !adjoint && S.has_guess != 0, sh, nullptr, 0, adjoint != 0);
}

__global__ void k_pairs(XrWork w, XrFF ff0) {
  const int np = xr_num_pairs(w);
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) pair_one(w, ff0, p);
}

// ------------------------------------------------------------------------ force assembly
// The pair's shielded Coulomb energy 332.06371 q_i q_j shield(r) is formed here, with the final
// charges, and its dE/dr joins the pair's radial sensitivity (vdW, charge response, bond-order
// chain): dE/dx_j += G v/r, dE/dx_i -= G v/r.
__device__ inline void pair_force_one(const XrWork& w, int p) {
  const int i = w.pair_i[p];
  const int2 ed = w.edge[w.pair_edge[p]];
  const int j = ed.x;
  const double qq = C_ELE * w.q[i] * w.q[j];
  w.p_ecoul[p] = qq * w.p_shield[p];
  const double G = w.p_g[p] + qq * w.p_dshield[p];
  if (G == 0.0 || i == j) return;  // a self-image pair moves both ends together: no net force
  const XrSystem& S = w.sys[w.sys_of[i]];
  double v[3];
  edge_vector(S, w.x[i], w.x[j], (uint32_t)ed.y, v);
  const double s = G / w.p_r[p];
  for (int c = 0; c < 3; ++c) {
    atomicAdd(w.f + 3 * j + c, s * v[c]);
    atomicAdd(w.f + 3 * i + c, -s * v[c]);
  }
}

__global__ void k_pair_forces(XrWork w) {
  const int np = xr_num_pairs(w);
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) pair_force_one(w, p);
}

// ------------------------------------------------------------------------ reductions
// Energies land per item (pair, bond, atom). The atoms of each system are cut into fixed chunks of
// at most XR_CHUNK_ATOMS, numbered in system order from XrSystem::chunk0; pairs and half bonds are
// stored by their first atom, so a chunk's atoms own contiguous ranges of both, and one block sums
// the chunk's pair, bond and atom terms directly. One block per system then adds its chunks in
// order. Every sum has a fixed order (the system's chunks, each in thread and lane order), so
// energies, charges and dipoles are bitwise reproducible from call to call. The adds are FP64 (a
// warp instruction takes 64 cycles of the FP64 pipe), so chunks are small enough to spread over the
// SMs, and the block's partials are summed slot by slot (a few adds per lane, then five shuffles)
// rather than each warp reducing all 23 slots.
constexpr int kReduceThreads = 128;

// Partial slots: 0..13 components, 14 mass, 15..17 mass * x, 18 charge, 19..21 charge * x, 22 finite.
__global__ void __launch_bounds__(kReduceThreads) k_reduce_chunk(XrWork w, XrFF ff) {
  __shared__ double part[XR_PART_N][kReduceThreads];
  // the chunk's system: the last one that starts at or before it (a system without atoms has no
  // chunks and starts where the next one does)
  const int chunk = blockIdx.x;
  int lo = 0, hi = w.S - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (w.sys[mid].chunk0 <= chunk)
      lo = mid;
    else
      hi = mid - 1;
  }
  const XrSystem& S = w.sys[lo];
  const int a_beg = S.atom_off + (chunk - S.chunk0) * XR_CHUNK_ATOMS;
  const int4 ch = make_int4(lo, a_beg, min(S.atom_off + S.natoms, a_beg + XR_CHUNK_ATOMS), 0);
  const int L = w.A + 1, tid = threadIdx.x;
  const double* atab = atoms_of_system(ff, S);
  double v[XR_PART_N];
#pragma unroll
  for (int k = 0; k < XR_PART_N; ++k) v[k] = 0.0;
#pragma unroll 4
  for (int p = w.cnt[1 * L + ch.y] + tid; p < w.cnt[1 * L + ch.z]; p += kReduceThreads) {
    v[C_VDW] += w.p_evdw[p];
    v[C_COULOMB] += w.p_ecoul[p];
  }
#pragma unroll 2
  for (int b = w.cnt[2 * L + ch.y] + tid; b < w.cnt[2 * L + ch.z]; b += kReduceThreads) {
    v[C_BOND] += w.b_e[0 * w.cap_B + b];
    v[C_LONE_PAIR] += w.b_e[1 * w.cap_B + b];
    v[C_TORSION] += w.b_e[2 * w.cap_B + b];
    v[C_CONJ] += w.b_e[3 * w.cap_B + b];
  }
  double finite = 1.0;
  for (int a = ch.y + tid; a < ch.z; a += kReduceThreads) {
    v[C_LONE_PAIR] += AEV(0, a);
    v[C_ATOM] += AEV(1, a);
    v[C_ANGLE] += AEV(2, a);
    v[C_PENALTY] += AEV(3, a);
    v[C_ANGLE_CONJ] += AEV(4, a);
    v[C_HBOND] += AEV(5, a);
    v[C_QEQ] += AEV(6, a);
    const double m = atom_prm(atab, w.type[a], A_MASS);
    const double4_32a x = w.x[a];
    const double q = w.q[a];
    v[14] += m;
    v[15] += m * x.x;
    v[16] += m * x.y;
    v[17] += m * x.z;
    v[18] += q;
    v[19] += q * x.x;
    v[20] += q * x.y;
    v[21] += q * x.z;
    if (!(isfinite(q) && isfinite(w.f[3 * a]) && isfinite(w.f[3 * a + 1]) && isfinite(w.f[3 * a + 2]))) finite = 0.0;
  }
  v[22] = finite;
#pragma unroll
  for (int k = 0; k < XR_PART_N; ++k) part[k][tid] = v[k];
  __syncthreads();
  // slot k by warp k % 4: four partials per lane in thread order, then the warp's butterfly (finite
  // combines by min)
  const int lane = tid & 31, wid = tid >> 5;
  for (int k = wid; k < XR_PART_N; k += kReduceThreads / 32) {
    double s = part[k][lane];
    for (int t = lane + 32; t < kReduceThreads; t += 32) s = k == 22 ? fmin(s, part[k][t]) : s + part[k][t];
    for (int o = 16; o > 0; o >>= 1) {
      const double y = __shfl_xor_sync(0xffffffffu, s, o);
      s = k == 22 ? fmin(s, y) : s + y;
    }
    if (lane == 0) w.chunk_part[(size_t)blockIdx.x * XR_PART_N + k] = s;
  }
}

// One block per system: warp k % 8 sums slot k over the system's chunks (a strided pass per lane in
// chunk order, then the warp's butterfly).
constexpr int kFinalThreads = 256;
__global__ void __launch_bounds__(kFinalThreads) k_reduce_final(XrWork w) {
  const int s = blockIdx.x;
  const int c0 = w.sys[s].chunk0, c1 = c0 + (w.sys[s].natoms + XR_CHUNK_ATOMS - 1) / XR_CHUNK_ATOMS;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, k = threadIdx.x;
  __shared__ double tot[XR_PART_N];
  for (int slot = wid; slot < XR_PART_N; slot += kFinalThreads / 32) {
    double acc = slot == 22 ? 1.0 : 0.0;
    for (int c = c0 + lane; c < c1; c += 32) {
      const double v = w.chunk_part[(size_t)c * XR_PART_N + slot];
      acc = slot == 22 ? fmin(acc, v) : acc + v;
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double y = __shfl_xor_sync(0xffffffffu, acc, o);
      acc = slot == 22 ? fmin(acc, y) : acc + y;
    }
    if (lane == 0) tot[slot] = acc;
  }
  __syncthreads();
  if (k == 0) {
    double total = 0;
    bool fin = tot[22] > 0.5;
    for (int c = 0; c < XR_NCOMP; ++c) {
      w.energy[16 * s + c] = tot[c];
      total += tot[c];
      if (!isfinite(tot[c])) fin = false;
    }
    w.energy[16 * s + 14] = total;
    w.energy[16 * s + 15] = 0.0;
    // dipole about the mass centre: sum q (x - c) = sum q x - c sum q (src/xreac/energy.py:171-177)
    for (int d = 0; d < 3; ++d) w.props[4 * s + d] = tot[19 + d] - tot[15 + d] / tot[14] * tot[18];
    w.props[4 * s + 3] = 0.0;
    if (!fin) atomicOr(w.status, XR_S_NONFINITE);
  }
}

// -dE/dq per atom (warp per atom over its directed edges).
__global__ void k_qeq_rhs(XrWork w, XrFF ff) {
  const int lane = threadIdx.x & 31;
  const int a = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  if (a >= w.A) return;
  double s = 0;
  for (int e = w.cnt[a] + lane; e < w.cnt[a + 1]; e += 32) s += w.q[w.edge[e].x] * w.p_shield[w.edge_pair[e]];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) {
    const int t = w.type[a];
    const double* atab = atoms_of_system(ff, w.sys[w.sys_of[a]]);
    const double dEdq = C_ELE * s + SELF_CONVERSION * (atom_prm(atab, t, A_CHI) + atom_prm(atab, t, A_ETA) * w.q[a]);
    w.qrhs[a] = -dEdq;
  }
}

__global__ void k_charge_response_radial(XrWork w) {
  const int np = xr_num_pairs(w);
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
    const int i = w.pair_i[p], j = w.edge[w.pair_edge[p]].x;
    w.p_g[p] += -QEQ_COULOMB * (w.qadj[i] * w.q[j] + w.qadj[j] * w.q[i]) * w.p_dshield[p];
  }
}

// dE/d(chi, eta, gamma) through the charges: with the KKT system H q + chi = mu 1, sum q = Q and the
// adjoint lambda (H lambda = dE/dq - nu 1, sum lambda = 0, from the adjoint solve), the total
// derivative of a parameter theta is dE/dtheta|_q - lambda' (dH/dtheta q + dchi/dtheta). So
// dE/dchi_i = 23.02 q_i - lambda_i, dE/deta_i = 11.51 q_i^2 - lambda_i q_i (H_ii = eta_i + self
// images), and for a pair's gamma (shield = taper (r^3 + gamma)^(-1/3), H_ij = 14.4 shield),
// (332.06371 q_i q_j - 14.4 (lambda_i q_j + lambda_j q_i)) dshield/dgamma with
// dshield/dgamma = -shield / (3 (r^3 + gamma)). Summed per element and per pair type.
__global__ void k_qeq_param_grad(XrWork w, XrFF ff0) {
  const int stride = gridDim.x * blockDim.x;
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < w.A; a += stride) {
    const double q = w.q[a], lam = w.qadj[a];
    double* ga = xr_pgrad(w, a) + w.pgrad_atom_off + (size_t)w.type[a] * XR_NATOM_COLS;
    atomicAdd(ga + A_CHI, SELF_CONVERSION * q - lam);
    atomicAdd(ga + A_ETA, 0.5 * SELF_CONVERSION * q * q - lam * q);
  }
  const int np = xr_num_pairs(w);
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += stride) {
    const int i = w.pair_i[p], j = w.edge[w.pair_edge[p]].x;
    const double sh = w.p_shield[p];
    if (sh == 0.0) continue;
    const XrFF ff = xr_ff_of(ff0, w, i);
    const int pt = w.type[i] * ff.ntypes + w.type[j];
    const double r = w.p_r[p], gam = pair_prm(ff, pt, P_GAMMA);
    const double dsh = -sh / (3.0 * (r * r * r + gam));
    const double c = C_ELE * w.q[i] * w.q[j] - QEQ_COULOMB * (w.qadj[i] * w.q[j] + w.qadj[j] * w.q[i]);
    atomicAdd(xr_pgrad(w, i) + (size_t)pt * XR_NPAIR_COLS + P_GAMMA, c * dsh);
  }
}

}  // namespace

void xr_launch_qeq_param_gradient(const XrWork& w, const XrFF& ff, cudaStream_t st) {
  const int n = std::max(w.A, std::max(w.nP, 1));
  k_qeq_param_grad<<<std::min((n + 255) / 256, 152 * 8), 256, 0, st>>>(w, ff);
}

void xr_launch_charge_response(const XrWork& w, const XrFF& ff, cudaStream_t st, int stage) {
  if (stage == 0) {
    k_qeq_rhs<<<(w.A + 3) / 4, 128, 0, st>>>(w, ff);
    if (w.nE > 0) k_hval<<<(w.nE + 255) / 256, 256, 0, st>>>(w);  // the solve may have scaled them in place
  } else if (w.nP > 0) {
    k_charge_response_radial<<<(w.nP + 255) / 256, 256, 0, st>>>(w);
  }
}

void xr_launch_pairs(const XrWork& w, const XrFF& ff, cudaStream_t st) {
  if (w.nP > 0) k_pairs<<<(w.nP + 127) / 128, 128, 0, st>>>(w, ff);
  if (w.nE > 0) k_hval<<<(w.nE + 255) / 256, 256, 0, st>>>(w);
}

int xr_qeq_coop_blocks_per_sm() {
  cudaFuncSetAttribute(k_qeq_grid, cudaFuncAttributeMaxDynamicSharedMemorySize, kQeqMaxDyn);
  int nb = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_qeq_grid, 1024, kQeqMaxDyn);
  return nb;
}

namespace {
cudaLaunchConfig_t cluster_config(int csize, int nblocks, cudaStream_t st, cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nblocks);
  cfg.blockDim = dim3(1024);
  cfg.dynamicSmemBytes = kQeqMaxDyn;
  cfg.stream = st;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}
}  // namespace

int xr_qeq_max_clusters(int csize) {
  if (cudaFuncSetAttribute(k_qeq_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, kQeqMaxDyn) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = cluster_config(csize, csize, nullptr, attr);
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, (void*)k_qeq_cluster, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

int xr_launch_qeq_cluster(const XrWork& w, const XrFF& ff, cudaStream_t st, int csize, int nblocks, const int* list,
                          int nbig, int nsmall, bool adjoint) {
  cudaMemsetAsync(w.barrier, 0, 2 * sizeof(unsigned), st);  // big-system and small-system counters
  if (nbig > 0) {
    const int n = nbig * (csize + 1);  // one warp each
    k_qeq_splits<<<(n + 3) / 4, 128, 0, st>>>(w, list, nbig, csize, nullptr, 0);
  }
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = cluster_config(csize, nblocks, st, attr);
  const int* small = list + nbig;
  int adj = adjoint ? 1 : 0;
  return (int)cudaLaunchKernelEx(&cfg, k_qeq_cluster, w, ff, list, nbig, small, nsmall, adj);
}

// Returns 0 on success or a CUDA error code from the launch. With nblocks > 0 the cooperative
// solver runs nblocks blocks (nteam team blocks described by map, the rest over the small list);
// nblocks = 0 selects the one-block-per-system fallback.
int xr_launch_qeq(const XrWork& w, const XrFF& ff, cudaStream_t st, int nblocks, const int4* map, int nteam,
                  const int* small, int nsmall, bool adjoint) {
  int adj = adjoint ? 1 : 0;
  if (nblocks > 0) {
    // team barrier counters, then the small-system counter
    cudaMemsetAsync(w.barrier, 0, sizeof(unsigned) * (size_t)(nteam + 1), st);
    if (nteam > 0) k_qeq_splits<<<(2 * nteam + 3) / 4, 128, 0, st>>>(w, nullptr, 0, 0, map, nteam);
    if (nteam == 0) {  // no block waits on another: an ordinary launch, which may overlap other streams' work
      k_qeq_grid<<<nblocks, 1024, kQeqMaxDyn, st>>>(w, ff, map, nteam, small, nsmall, adj);
      return (int)cudaGetLastError();
    }
    void* args[] = {(void*)&w, (void*)&ff, (void*)&map, (void*)&nteam, (void*)&small, (void*)&nsmall, (void*)&adj};
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)k_qeq_grid, dim3(nblocks), dim3(1024), args, kQeqMaxDyn, st);
    return (int)e;
  }
  k_qeq_block<<<w.S, 1024, 0, st>>>(w, ff, adj);
  return (int)cudaGetLastError();
}

// Charge-response (full-derivative) forces, xreac's full_derivative=True (src/xreac/calculator.py:
// 134-148 differentiates through the KKT solve of src/xreac/energy.py:95-102). With E(q(x), x) and
// H q + chi = mu 1, sum q = Q, the adjoint lambda solves H lambda = dE/dq - nu 1, sum lambda = 0, and
// dE/dx = dE/dx|_q - lambda' (dH/dx) q. dE/dq_k = 332.06371 sum_(k->j) q_j shield + 23.02 (chi_k +
// eta_k q_k) (the Coulomb and self energies; the QEq matrix uses 14.4, so E is not stationary in q).
// stage 0: the adjoint right-hand side -dE/dq (the solver's "chi") and the unscaled matrix entries;
// stage 1: each pair's radial term -14.4 (lambda_i q_j + lambda_j q_i) dshield/dr.



void xr_launch_forces(const XrWork& w, const XrFF& ff, cudaStream_t st) {
  (void)ff;
  if (w.nP > 0) k_pair_forces<<<(w.nP + 255) / 256, 256, 0, st>>>(w);
}

void xr_launch_reduce(const XrWork& w, const XrFF& ff, cudaStream_t st) {
  k_reduce_chunk<<<w.nchunks, kReduceThreads, 0, st>>>(w, ff);
  k_reduce_final<<<w.S, kFinalThreads, 0, st>>>(w);
}

namespace {
__global__ void k_math_test(int fn, const double* in, double* out, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double x = in[i];
    out[i] = fn == 0 ? xr_exp(x) : fn == 1 ? exp(x) : fn == 2 ? xr_log(x) : log(x);
  }
}
}  // namespace

extern "C" int xr_test_math(int fn, const double* in, double* out, int n) {
  if (fn < 0 || fn > 3 || n < 0 || (n > 0 && (!in || !out))) return XR_EINPUT;
  if (n == 0) return XR_OK;
  k_math_test<<<std::min((n + 255) / 256, 4096), 256>>>(fn, in, out, n);
  if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return XR_ECUDA;
  return XR_OK;
}
