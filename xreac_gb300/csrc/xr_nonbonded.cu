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
#include "xr_common.cuh"

namespace {

constexpr double C_ELE = 332.06371;
constexpr double QEQ_COULOMB = 14.4;
constexpr double SELF_CONVERSION = 23.02;

#define AEV(k, a) w.a_e[(size_t)(k) * w.A + (a)]
#define QW(k, a) w.qwork[(size_t)(k) * w.A + (a)]

__device__ inline double pair_prm(const XrFF& ff, int pt, int col) { return __ldg(ff.pair + pt * XR_NPAIR_COLS + col); }
__device__ inline double atom_prm(const XrFF& ff, int t, int col) { return __ldg(ff.atom + t * XR_NATOM_COLS + col); }

__device__ inline void edge_vector(const XrSystem& S, const double4_32a& xi, const double4_32a& xj, uint32_t code, double v[3]) {
  const int sx = xr_sx(code), sy = xr_sy(code), sz = xr_sz(code);
  const double xa[3] = {xi.x, xi.y, xi.z}, xb[3] = {xj.x, xj.y, xj.z};
  for (int c = 0; c < 3; ++c) {
    const double off = __dadd_rn(__dadd_rn(__dmul_rn((double)sx, S.cell[c]), __dmul_rn((double)sy, S.cell[3 + c])),
                                 __dmul_rn((double)sz, S.cell[6 + c]));
    v[c] = __dadd_rn(__dsub_rn(xb[c], xa[c]), off);
  }
}

// ------------------------------------------------------------------------------ pair kernel
__global__ void k_pairs(XrWork w, XrFF ff) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= w.nP) return;
  const int e = w.pair_edge[p], i = w.pair_i[p];
  const int2 ed = w.edge[e];
  const int j = ed.x;
  const XrSystem& S = w.sys[w.sys_of[i]];
  double v[3];
  edge_vector(S, w.x[i], w.x[j], (uint32_t)ed.y, v);
  const double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(v[0], v[0]), __dmul_rn(v[1], v[1])), __dmul_rn(v[2], v[2])));
  const double rc = S.rc;
  const int T = ff.ntypes, pt = w.type[i] * T + w.type[j];
  double taper = 0.0, dtaper = 0.0;
  if (r < rc) {
    const double u = r / rc;
    taper = 1 + u * u * u * u * (-35 + u * (84 + u * (-70 + 20 * u)));
    const double um = u - 1;
    dtaper = 140.0 / rc * u * u * u * um * um * um;
  }
  const double gam = pair_prm(ff, pt, P_GAMMA);
  const double c = cbrt(r * r * r + gam);
  const double shield = taper / c;
  const double dshield = dtaper / c - taper * r * r / (c * c * c * c);
  double f13 = r, df13 = 1.0;
  if (ff.vdw_type == 1 || ff.vdw_type == 3) {
    const double pw = ff.g[28];
    const double rp = exp(pw * log(r));
    const double sum = rp + __ldg(ff.pair_gw + pt);
    f13 = exp(log(sum) / pw);
    df13 = f13 * rp / (sum * r);
  }
  const double D = pair_prm(ff, pt, P_D), alpha = pair_prm(ff, pt, P_ALPHA), rvdw = pair_prm(ff, pt, P_RVDW);
  const double ev = exp(0.5 * alpha * (1 - f13 / rvdw));
  const double dev = ev * (-0.5 * alpha / rvdw) * df13;
  double E = taper * D * (ev * ev - 2 * ev);
  double G = dtaper * D * (ev * ev - 2 * ev) + taper * D * (2 * ev - 2) * dev;
  if (ff.vdw_type == 2 || ff.vdw_type == 3) {
    const double ecore = pair_prm(ff, pt, P_ECORE), acore = pair_prm(ff, pt, P_ACORE), rcore = pair_prm(ff, pt, P_RCORE);
    const double ec = ecore * exp(acore * (1 - r / rcore));
    E += taper * ec;
    G += dtaper * ec + taper * ec * (-acore / rcore);
  }
  w.p_r[p] = r;
  w.p_shield[p] = shield;
  w.p_dshield[p] = dshield;
  w.p_evdw[p] = E;
  w.p_g[p] = G;
}

__global__ void k_hval(XrWork w) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= w.nE) return;
  w.hval[e] = QEQ_COULOMB * w.p_shield[w.edge_pair[e]];
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

// Bounded grid barrier for a cooperative launch (all blocks co-resident): every block adds one to a
// monotonically increasing counter with release semantics and waits, with acquire loads, until it
// reaches the episode's target (number of blocks times episodes so far). Returns false when the
// wait ran out; every block then leaves the solver and the host reports the status bit.
__device__ bool grid_barrier(unsigned* bar, unsigned target, int* status) {
  __syncthreads();
  __shared__ int ok;
  if (threadIdx.x == 0) {
    ok = 1;
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(bar) : "memory");
    long long it = 0;
    while (ld_acquire(bar) < target) {
      if (++it > (1ll << 24) || (*(volatile int*)status & XR_S_BARRIER)) {
        atomicOr(status, XR_S_BARRIER);
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
    return grid_barrier(bar, target, w.status);
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
    // Fixed-size slots; consecutive reductions never share one, so a block may publish the next
    // partials while a slower block still reads the previous ones.
    double* rs = red + (size_t)slot * 8 * nb;
    if (wid == 0) {
      int good = 1;
      __syncwarp();  // orders warp 0's row writes before lane 0's release
      if (lane == 0) {
        for (int k = 0; k < NV; ++k) rs[k * nb + rank] = v[k];
        asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(bar) : "memory");
        long long it = 0;
        while (ld_acquire(bar) < target) {
          if (++it > (1ll << 24) || (*(volatile int*)w.status & XR_S_BARRIER)) {
            atomicOr(w.status, XR_S_BARRIER);
            good = 0;
            break;
          }
          if (it > 256) __nanosleep(32);
        }
        ok = good;
      }
      __syncwarp();
      for (int k = 0; k < NV; ++k) {
        double t = 0;
        for (int q = lane; q < nb; q += 32) t += __ldcg(rs + k * nb + q);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) res[k] = t;
      }
      if (lane == 0) post(res);
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

// Warp-0 sum of a per-lane value (the block total ends in every lane of warp 0).
__device__ inline double warp_total(double t) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  return t;
}

// Block-shared state of one solve: the reductions' buffer, the iteration scalars (written by thread 0
// in the reductions' post hooks), the tile transposition buffers and, for blocks of at most 32 rows,
// the rows' solver state indexed by row - r0. One instance per kernel serves both team kinds.
struct QeqShared {
  double red[kRedSmem];
  double sc_lam, sc_alpha, sc_step, sc_beta;
  int sc_state;  // 0 iterate, 1 converged, 2 stop
  double part[32][33];
  double part4[4][32];
  double rs_x[32], rs_p[32], rs_hp[32], rs_di[32], rs_c[32], rs_eta[32], rs_g[32];
};

// Rows [r0, r1) of the system starting at atom a0 belong to this block. The matrix-vector product
// runs on tiles of 32 rows, one row per warp; the lanes' partial row sums are transposed through
// shared memory so that one warp owns the 32 rows of a tile, one row per lane, for the row
// reductions and every per-row scalar update. On this part an FP64 instruction costs the FP64 pipe
// the same whether one lane or 32 are active, so scalar row work done by lane 0 of 32 warps would
// cost 32 times the issue slots of the same work spread over the lanes of one warp.
// When `cache_j` is non-null the block's matrix rows (column, H'_ij) are kept in shared memory;
// when `gstage` is non-null the whole gradient is staged in shared memory every iteration.
template <class Team>
__device__ void qeq_solve(const XrWork& w, const XrFF& ff, const Team& team, int a0, int n, int r0, int r1,
                          double Q, bool warm, QeqShared& sh, unsigned short* cache_j, double* cache_h,
                          int cache_cap, double* gstage) {
  double* smem = sh.red;
  double &sc_lam = sh.sc_lam, &sc_alpha = sh.sc_alpha, &sc_step = sh.sc_step, &sc_beta = sh.sc_beta;
  int& sc_state = sh.sc_state;
  auto& part = sh.part;
  auto& part4 = sh.part4;
  double *rs_x = sh.rs_x, *rs_p = sh.rs_p, *rs_hp = sh.rs_hp, *rs_di = sh.rs_di, *rs_c = sh.rs_c, *rs_eta = sh.rs_eta,
         *rs_g = sh.rs_g;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double* X = &QW(Q_X, 0);
  double* G = &QW(Q_G, 0);
  double* G2 = &QW(Q_G2, 0);
  double* Pv = &QW(Q_P, 0);
  double* HP = &QW(Q_HP, 0);
  double* DI = &QW(Q_DINV, 0);
  double* Cr = &QW(Q_C, 0);
  auto noop = [](double*) {};
  const double x0 = Q / n;
  // 1. Jacobi diagonal (eta + self-image shields) of the owned rows, and the start point: the
  //    uniform x0 = Q/n, or the caller's charges of an earlier step (already summing to Q).
  for (int r = r0 + wid; r < r1; r += nw) {
    const int a = a0 + r;
    double d = 0;
    for (int e = w.cnt[a] + lane; e < w.cnt[a + 1]; e += 32)
      if (w.edge[e].x == a) d += w.hval[e];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
    if (lane == 0) {
      DI[a] = 1.0 / (atom_prm(ff, w.type[a], A_ETA) + d);
      X[a] = warm ? w.qguess[a] : x0;
    }
  }
  if (!team.sync(w)) return;
  // 2. Pre-scaled rows H'_ij = H_ij / D_jj (cached or in hval), row sums, and the start point
  //    x0 = Q/n with gradient g0 = H x0 + chi = (Q/n) * rowsum(H) + chi.
  const int ebeg = w.cnt[a0 + r0], eend = w.cnt[a0 + r1];
  const bool cached = cache_j != nullptr && (eend - ebeg) <= cache_cap;
  // <D^-1, 1>, <D^-1, g>, <D^-1, g^2> at the start point, and <D^-1, g_u>, <D^-1, g_u^2> at the
  // uniform start x0, whose projected norm sets the convergence scale for cold and warm starts alike
  double acc[5] = {0, 0, 0, 0, 0};
  for (int r = r0 + wid; r < r1; r += nw) {
    const int a = a0 + r;
    const int t = w.type[a];
    double rs = 0, cs = 0, hx = 0;
    for (int e = w.cnt[a] + lane; e < w.cnt[a + 1]; e += 32) {
      const int j = w.edge[e].x;
      const double h = w.hval[e];
      const double hp = h * __ldcg(DI + j);
      rs += h;
      cs += hp;
      if (warm) hx += h * __ldcg(X + j);
      if (cached) {
        cache_j[e - ebeg] = (unsigned short)(j - a0);
        cache_h[e - ebeg] = hp;
      } else {
        w.hval[e] = hp;  // scaled in place; hval is not read after the solve
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      rs += __shfl_xor_sync(0xffffffffu, rs, o);
      cs += __shfl_xor_sync(0xffffffffu, cs, o);
      if (warm) hx += __shfl_xor_sync(0xffffffffu, hx, o);
    }
    if (lane == 0) {
      const double eta = atom_prm(ff, t, A_ETA), di = DI[a], chi = atom_prm(ff, t, A_CHI);
      const double gu = x0 * (rs + eta) + chi;
      const double g = warm ? hx + eta * X[a] + chi : gu;
      Cr[a] = cs + eta * di;
      G[a] = g;
      Pv[a] = 0.0;
      HP[a] = gu;  // kept for the projection step below, then cleared
      acc[0] += di;
      acc[1] += di * g;
      acc[2] += di * g * g;
      acc[3] += di * gu;
      acc[4] += di * gu * gu;
    }
  }
  if (!team_sum<5>(team, w, acc, smem, 0, noop)) return;
  // Iteration scalars are computed by thread 0 alone (in the reductions' post hooks) and shared.
  const double s1 = acc[0];
  // 3. Project the start gradient explicitly (g - lambda with lambda = <D^-1, g> / <D^-1, 1>) and take
  //    its norm from the projected values: sum D^-1 g^2 - lambda sum D^-1 g cancels to rounding noise
  //    of the unprojected gradient when the start is (nearly) the solution, e.g. q = 0 for identical
  //    atoms. The uniform start's projected norm sets the convergence scale.
  const double lam0 = acc[1] / s1, lamu = acc[3] / s1;
  double acc2[3] = {0, 0, 0};  // <D^-1, g~^2>, <D^-1, g~_u^2>, <D^-1, g~>
  for (int r = r0 + wid; r < r1; r += nw) {
    const int a = a0 + r;
    if (lane == 0) {
      const double di = DI[a];
      const double gt = G[a] - lam0;
      const double gut = HP[a] - lamu;  // the uniform start's gradient, parked in HP by step 2
      G[a] = gt;
      HP[a] = 0.0;
      acc2[0] += di * gt * gt;
      acc2[1] += di * gut * gut;
      acc2[2] += di * gt;
    }
  }
  const double tol2 = w.cg_tol * w.cg_tol;
  const double gfloor = 1e-28 * fmax(acc[2], acc[4]);
  double gz = 0.0, gz0 = 0.0;
  if (!team_sum<3>(team, w, acc2, smem, 1, noop)) return;
  if (threadIdx.x == 0) {
    gz = acc2[0];
    gz0 = acc2[1];  // the uniform start's projected norm (= gz when cold)
    sc_lam = acc2[2] / s1;  // rounding-level drift of the projection, removed in the first step
    sc_beta = 0.0;
    // Nothing to solve when the projected gradient is already at rounding level (one atom, a start
    // that is exact by symmetry) or a warm start already meets the tolerance.
    sc_state = (!(gz > gfloor) || n < 2 || gz <= tol2 * gz0) ? 1 : 0;
  }
  // For blocks of at most 32 rows (the grid layout) the rows' solver state lives in shared memory.
  const bool row_smem = (r1 - r0) <= 32;
  if (row_smem && wid == 0 && r0 + lane < r1) {
    const int a = a0 + r0 + lane;
    rs_x[lane] = X[a];
    rs_p[lane] = 0.0;
    rs_hp[lane] = 0.0;
    rs_di[lane] = DI[a];
    rs_c[lane] = Cr[a];
    rs_eta[lane] = atom_prm(ff, w.type[a], A_ETA);
    rs_g[lane] = G[a];
  }
  __syncthreads();
  int it = 0;
  int slot = 2;
  while (sc_state == 0) {
    if (++it > w.cg_max_iter) {
      if (threadIdx.x == 0) atomicOr(w.status, XR_S_CG);
      break;
    }
    const double lam = sc_lam, beta = sc_beta;
    // p = -z + beta p,  Hp = -H z + beta Hp,  z = D^-1 (g - lambda); the next buffer gets g - lambda
    if (gstage) {  // the whole gradient of the system in shared memory: the gathers below stay on-chip
      for (int q = threadIdx.x; q < n; q += blockDim.x) gstage[q] = __ldcg(G + a0 + q);
      __syncthreads();
    }
    double pHp[2] = {0.0, 0.0};  // lane partials in warp 0: p'Hp and <D^-1, Hp>
    for (int tb = r0; tb < r1; tb += 32) {
      const int r = tb + wid;
      double hz = 0;
      if (wid < 32 && r < r1) {
        const int a = a0 + r;
        const int eb = w.cnt[a], ee = w.cnt[a + 1];
        if (cached && gstage) {
          for (int e = eb + lane; e < ee; e += 32) hz += cache_h[e - ebeg] * gstage[cache_j[e - ebeg]];
        } else if (cached) {
          for (int e = eb + lane; e < ee; e += 32) hz += cache_h[e - ebeg] * __ldcg(G + a0 + cache_j[e - ebeg]);
        } else {
          double h0 = 0, h1 = 0;
          int e = eb + lane;
          for (; e + 32 < ee; e += 64) {
            const double g0 = __ldcg(G + w.edge[e].x), g1 = __ldcg(G + w.edge[e + 32].x);
            h0 += w.hval[e] * g0;
            h1 += w.hval[e + 32] * g1;
          }
          if (e < ee) h0 += w.hval[e] * __ldcg(G + w.edge[e].x);
          hz = h0 + h1;
        }
      }
      if (wid < 32) part[wid][lane] = hz;
      __syncthreads();
      if (wid < 4) {  // lane = row of the tile; warp k adds lanes 8k .. 8k+7 of the row's partials
        double s = part[lane][8 * wid];
#pragma unroll
        for (int k = 1; k < 8; ++k) s += part[lane][8 * wid + k];
        part4[wid][lane] = s;
      }
      __syncthreads();
      if (wid == 0 && tb + lane < r1) {
        const int rr = tb + lane, a = a0 + rr;
        double h = (part4[0][lane] + part4[1][lane]) + (part4[2][lane] + part4[3][lane]);
        const double ga = row_smem ? rs_g[lane] : (gstage ? gstage[rr] : G[a]);
        const double di = row_smem ? rs_di[lane] : DI[a];
        const double eta = row_smem ? rs_eta[lane] : atom_prm(ff, w.type[a], A_ETA);
        const double cr = row_smem ? rs_c[lane] : Cr[a];
        const double p_old = row_smem ? rs_p[lane] : Pv[a];
        const double hp_old = row_smem ? rs_hp[lane] : HP[a];
        h += eta * di * ga - lam * cr;
        const double z = di * (ga - lam);
        const double p = -z + beta * p_old;
        const double hp = -h + beta * hp_old;
        if (row_smem) {
          rs_p[lane] = p;
          rs_hp[lane] = hp;
          rs_g[lane] = ga - lam;
        } else {
          Pv[a] = p;
          HP[a] = hp;
          G2[a] = ga - lam;
        }
        pHp[0] += p * hp;
        pHp[1] += di * hp;
      }
    }
    if (wid == 0) {
      pHp[0] = warp_total(pHp[0]);
      pHp[1] = warp_total(pHp[1]);
    }
    if (!team.template reduce<2>(w, pHp, smem, slot, [&](double* t) {
          // The QEq matrix of a close-packed geometry can have a negative eigenvalue (the reference's
          // direct KKT solve accepts it); CG then takes steps of negative curvature (alpha < 0) and
          // still converges. Only an exactly vanishing or non-finite p'Hp is a breakdown, and a
          // non-positive one at rounding level means the solve has converged.
          const bool rounding = gz <= 1e4 * gfloor;
          if (!(fabs(t[0]) > 0.0) || !isfinite(t[0]) || (t[0] < 0.0 && rounding)) {
            if (!rounding) atomicOr(w.status, XR_S_NONSPD);
            sc_state = 2;
          } else {
            sc_alpha = gz / t[0];
            sc_step = sc_alpha * t[1] / s1;
          }
        }))
      return;
    slot = slot == 1 ? 2 : 1;
    if (sc_state != 0) break;
    // Step: x += alpha p, g += alpha Hp - (multiplier change), one row per lane of warp 0.
    const double alpha = sc_alpha, step_lam = sc_step;
    double u[2] = {0, 0};
    if (wid == 0) {
      for (int rr = r0 + lane; rr < r1; rr += 32) {
        const int a = a0 + rr;
        if (row_smem) {
          const double g = (rs_g[lane] + alpha * rs_hp[lane]) - step_lam;
          rs_x[lane] += alpha * rs_p[lane];
          rs_g[lane] = g;
          G2[a] = g;  // published for the other rows' products
          u[0] += rs_di[lane] * g;
          u[1] += rs_di[lane] * g * g;
        } else {
          const double g = (G2[a] + alpha * HP[a]) - step_lam;
          X[a] += alpha * Pv[a];
          G2[a] = g;
          const double di = DI[a];
          u[0] += di * g;
          u[1] += di * g * g;
        }
      }
      u[0] = warp_total(u[0]);
      u[1] = warp_total(u[1]);
    }
    if (!team.template reduce<2>(w, u, smem, slot, [&](double* t) {
          sc_lam = t[0] / s1;
          const double gz_new = t[1] - sc_lam * t[0];
          if (gz_new <= tol2 * gz0) sc_state = 1;
          sc_beta = gz_new / gz;
          gz = gz_new;
        }))
      return;
    slot = slot == 1 ? 2 : 1;
    double* tmp = G;  // the buffer just written becomes the one read next
    G = G2;
    G2 = tmp;
  }
  if (row_smem && wid == 0 && r0 + lane < r1) X[a0 + r0 + lane] = rs_x[lane];
  __syncthreads();
  if (threadIdx.x == 0) atomicMax(w.counts + 4, it);
  // Final charges; the constraint is restored exactly against accumulated rounding.
  double sx[1] = {0.0};
  if (lane == 0)
    for (int r = r0 + wid; r < r1; r += nw) sx[0] += X[a0 + r];
  if (!team_sum<1>(team, w, sx, smem, 3, noop)) return;
  const double shift = (Q - sx[0]) / n;
  for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    const int a = a0 + r;
    const double q = X[a] + shift;
    w.q[a] = q;
    const int t = w.type[a];
    AEV(6, a) = SELF_CONVERSION * (atom_prm(ff, t, A_CHI) * q + 0.5 * atom_prm(ff, t, A_ETA) * q * q);
  }
}

// Dynamic shared memory of the solver kernel: [gradient stage: n doubles][row cache values][row
// cache columns (16-bit, local to the system)]. Each system's solve splits it the same way.
constexpr int kQeqMaxDyn = 208 * 1024;

__device__ inline void qeq_smem_plan(unsigned char* dyn, int n, double** gstage, double** cache_h,
                                     unsigned short** cache_j, int* cache_cap) {
  // stage the gradient when it takes at most half the space; 16-bit cache columns need n <= 65536
  const int stage_n = (n * 8 <= kQeqMaxDyn / 2) ? n : 0;
  const int cap = n <= 65536 ? (int)((kQeqMaxDyn - (size_t)stage_n * 8) / (sizeof(double) + sizeof(unsigned short))) : 0;
  *gstage = stage_n > 0 ? reinterpret_cast<double*>(dyn) : nullptr;
  *cache_h = reinterpret_cast<double*>(dyn + sizeof(double) * (size_t)stage_n);
  *cache_j = cap > 0 ? reinterpret_cast<unsigned short*>(dyn + sizeof(double) * ((size_t)stage_n + cap)) : nullptr;
  *cache_cap = cap;
}

// Cooperative solver launch for a batch: the first nteam blocks form teams, one per large system
// (map[b] = {system, rank, team size, first block of the team}); each team splits its system's rows
// and synchronises through its own bounded counter. The remaining blocks each solve a share of the
// small systems (small[k], k = b - nteam, b - nteam + (gridDim.x - nteam), ...) alone, with block
// barriers only. All blocks are co-resident (cooperative launch, one block per SM).
__global__ void __launch_bounds__(1024, 1) k_qeq_grid(XrWork w, XrFF ff, const int4* map, int nteam, const int* small,
                                                      int nsmall) {
  __shared__ QeqShared sh;
  extern __shared__ __align__(16) unsigned char dyn[];
  double *gstage, *cache_h;
  unsigned short* cache_j;
  int cache_cap;
  if ((int)blockIdx.x < nteam) {
    const int4 m = map[blockIdx.x];
    const XrSystem& S = w.sys[m.x];
    const int per = ((S.natoms + m.z - 1) / m.z + 31) / 32 * 32;
    const int r0 = min(S.natoms, m.y * per), r1 = min(S.natoms, r0 + per);
    qeq_smem_plan(dyn, S.natoms, &gstage, &cache_h, &cache_j, &cache_cap);
    GridTeam team{w.barrier + m.w, w.red + (size_t)32 * m.w, m.z, m.y};
    qeq_solve(w, ff, team, S.atom_off, S.natoms, r0, r1, S.total_charge, S.has_guess != 0, sh, cache_j, cache_h,
              cache_cap, gstage);
    return;
  }
  const int nsb = (int)gridDim.x - nteam;
  for (int k = (int)blockIdx.x - nteam; k < nsmall; k += nsb) {
    const XrSystem& S = w.sys[small[k]];
    qeq_smem_plan(dyn, S.natoms, &gstage, &cache_h, &cache_j, &cache_cap);
    BlockTeam team;
    qeq_solve(w, ff, team, S.atom_off, S.natoms, 0, S.natoms, S.total_charge, S.has_guess != 0, sh, cache_j, cache_h,
              cache_cap, gstage);
    __syncthreads();
  }
}

// Fallback without cooperative launch: one block per system, no shared-memory row cache.
__global__ void __launch_bounds__(1024, 1) k_qeq_block(XrWork w, XrFF ff) {
  __shared__ QeqShared sh;
  const XrSystem& S = w.sys[blockIdx.x];
  BlockTeam team;
  qeq_solve(w, ff, team, S.atom_off, S.natoms, 0, S.natoms, S.total_charge, S.has_guess != 0, sh, nullptr, nullptr,
            0, nullptr);
}

// ------------------------------------------------------------------------------ Coulomb
__global__ void k_coulomb(XrWork w) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= w.nP) return;
  const int i = w.pair_i[p], j = w.edge[w.pair_edge[p]].x;
  const double qq = C_ELE * w.q[i] * w.q[j];
  w.p_ecoul[p] = qq * w.p_shield[p];
  w.p_g[p] += qq * w.p_dshield[p];
}

// ------------------------------------------------------------------------ force assembly
// Every radial sensitivity (vdW, Coulomb, bond-order chain) sits on its pair: dE/dx_j += G v/r,
// dE/dx_i -= G v/r.
__global__ void k_pair_forces(XrWork w) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= w.nP) return;
  const double G = w.p_g[p];
  if (G == 0.0) return;
  const int i = w.pair_i[p];
  const int2 ed = w.edge[w.pair_edge[p]];
  const int j = ed.x;
  if (i == j) return;  // a self-image pair moves both ends together: no net force
  const XrSystem& S = w.sys[w.sys_of[i]];
  double v[3];
  edge_vector(S, w.x[i], w.x[j], (uint32_t)ed.y, v);
  const double s = G / w.p_r[p];
  for (int c = 0; c < 3; ++c) {
    atomicAdd(w.f + 3 * j + c, s * v[c]);
    atomicAdd(w.f + 3 * i + c, -s * v[c]);
  }
}

// ------------------------------------------------------------------------ reductions
// Energies land per item (pair, bond, atom). A warp per atom first folds its own pairs and half
// bonds into per-atom component sums; fixed chunks of at most XR_CHUNK_ATOMS atoms of one system
// are then summed by one block each, and one block per system adds its chunks in order. Every sum
// has a fixed order, so energies, charges and dipoles are bitwise reproducible.
#define ESUM(k, a) w.esum[(size_t)(k) * w.A + (a)]

__global__ void k_energy_gather(XrWork w) {
  const int lane = threadIdx.x & 31;
  const int a = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  if (a >= w.A) return;
  const int L = w.A + 1;
  double ev = 0, ec = 0, eb = 0, ec2 = 0, et = 0, eco = 0;
  for (int p = w.cnt[1 * L + a] + lane; p < w.cnt[1 * L + a + 1]; p += 32) {
    ev += w.p_evdw[p];
    ec += w.p_ecoul[p];
  }
  for (int b = w.cnt[2 * L + a] + lane; b < w.cnt[2 * L + a + 1]; b += 32) {
    eb += w.b_e[0 * w.cap_B + b];
    ec2 += w.b_e[1 * w.cap_B + b];
    et += w.b_e[2 * w.cap_B + b];
    eco += w.b_e[3 * w.cap_B + b];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ev += __shfl_xor_sync(0xffffffffu, ev, o);
    ec += __shfl_xor_sync(0xffffffffu, ec, o);
    eb += __shfl_xor_sync(0xffffffffu, eb, o);
    ec2 += __shfl_xor_sync(0xffffffffu, ec2, o);
    et += __shfl_xor_sync(0xffffffffu, et, o);
    eco += __shfl_xor_sync(0xffffffffu, eco, o);
  }
  if (lane == 0) {
    ESUM(C_BOND, a) = eb;
    ESUM(C_ATOM, a) = AEV(1, a);
    ESUM(C_LONE_PAIR, a) = AEV(0, a) + ec2;
    ESUM(C_MOLECULE, a) = 0.0;
    ESUM(C_ANGLE, a) = AEV(2, a);
    ESUM(C_PENALTY, a) = AEV(3, a);
    ESUM(C_ANGLE_CONJ, a) = AEV(4, a);
    ESUM(C_HBOND, a) = AEV(5, a);
    ESUM(C_TORSION, a) = et;
    ESUM(C_CONJ, a) = eco;
    ESUM(C_VDW, a) = ev;
    ESUM(C_COULOMB, a) = ec;
    ESUM(C_EFIELD, a) = 0.0;
    ESUM(C_QEQ, a) = AEV(6, a);
  }
}

// Partial slots: 0..13 components, 14 mass, 15..17 mass * x, 18 charge, 19..21 charge * x, 22 finite.
__global__ void k_reduce_chunk(XrWork w, XrFF ff) {
  __shared__ double smem[XR_PART_N * 32];
  const int4 ch = w.chunks[blockIdx.x];
  double v[XR_PART_N];
  for (int k = 0; k < XR_PART_N; ++k) v[k] = 0.0;
  double finite = 1.0;
  for (int a = ch.y + threadIdx.x; a < ch.z; a += blockDim.x) {
    for (int k = 0; k < XR_NCOMP; ++k) v[k] += ESUM(k, a);
    const double m = atom_prm(ff, w.type[a], A_MASS);
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
  // block sum (finite combines by min)
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k = 0; k < XR_PART_N; ++k)
    for (int o = 16; o > 0; o >>= 1) {
      const double y = __shfl_xor_sync(0xffffffffu, v[k], o);
      v[k] = (k == 22) ? fmin(v[k], y) : v[k] + y;
    }
  if (lane == 0)
    for (int k = 0; k < XR_PART_N; ++k) smem[k * 32 + wid] = v[k];
  __syncthreads();
  if (threadIdx.x < XR_PART_N) {
    const int k = threadIdx.x;
    double s = k == 22 ? 1.0 : 0.0;
    for (int q = 0; q < nw; ++q) s = (k == 22) ? fmin(s, smem[k * 32 + q]) : s + smem[k * 32 + q];
    w.chunk_part[(size_t)blockIdx.x * XR_PART_N + k] = s;
  }
}

__global__ void k_reduce_final(XrWork w) {
  const int s = blockIdx.x;
  const int2 r = w.sys_chunks[s];
  const int k = threadIdx.x;
  __shared__ double tot[XR_PART_N];
  if (k < XR_PART_N) {
    double acc = k == 22 ? 1.0 : 0.0;
    for (int c = r.x; c < r.y; ++c) {
      const double v = w.chunk_part[(size_t)c * XR_PART_N + k];
      acc = (k == 22) ? fmin(acc, v) : acc + v;
    }
    tot[k] = acc;
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

}  // namespace

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

// Returns 0 on success or a CUDA error code from the launch. With nblocks > 0 the cooperative
// solver runs nblocks blocks (nteam team blocks described by map, the rest over the small list);
// nblocks = 0 selects the one-block-per-system fallback.
int xr_launch_qeq(const XrWork& w, const XrFF& ff, cudaStream_t st, int nblocks, const int4* map, int nteam,
                  const int* small, int nsmall) {
  if (nblocks > 0) {
    if (nteam > 0) cudaMemsetAsync(w.barrier, 0, sizeof(unsigned) * (size_t)nteam, st);
    void* args[] = {(void*)&w, (void*)&ff, (void*)&map, (void*)&nteam, (void*)&small, (void*)&nsmall};
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)k_qeq_grid, dim3(nblocks), dim3(1024), args, kQeqMaxDyn, st);
    return (int)e;
  }
  k_qeq_block<<<w.S, 1024, 0, st>>>(w, ff);
  return (int)cudaGetLastError();
}

void xr_launch_coulomb(const XrWork& w, const XrFF& ff, cudaStream_t st) {
  (void)ff;
  if (w.nP > 0) k_coulomb<<<(w.nP + 255) / 256, 256, 0, st>>>(w);
}

void xr_launch_forces(const XrWork& w, const XrFF& ff, cudaStream_t st) {
  (void)ff;
  if (w.nP > 0) k_pair_forces<<<(w.nP + 255) / 256, 256, 0, st>>>(w);
}

void xr_launch_reduce(const XrWork& w, const XrFF& ff, cudaStream_t st) {
  k_energy_gather<<<(w.A + 7) / 8, 256, 0, st>>>(w);
  k_reduce_chunk<<<w.nchunks, 256, 0, st>>>(w, ff);
  k_reduce_final<<<w.S, 32, 0, st>>>(w);
}
