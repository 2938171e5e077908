// Shared device-side definitions for the GB300 ReaxFF evaluator.
//
// Data model (one "batch" = one or more independent systems evaluated together):
//   atoms      : concatenated over systems; system s owns atoms [atom_off, atom_off + natoms).
//   edges      : full directed neighbour list within the nonbonded cutoff, CSR by source atom,
//                rows in canonical (j, Sx, Sy, Sz) order -- the order of xreac's Neighbors
//                (src/xreac/neighbors.py:65-98). Each edge is int2 {j, code}.
//   pairs      : the "half" edges (i < j, or i == j with a lexicographically negative shift),
//                one per unordered image pair; nonbonded energies and forces run over pairs.
//   bonds      : pairs within min(5 A, cutoff) (bond-order candidates, src/xreac/energy.py:109).
//   bond rows  : per atom, its directed bond edges in canonical order, as (bond id, direction).
// Pairs and bonds are numbered in source-atom order, so every system owns contiguous ranges of
// atoms, edges, pairs and bonds. All physics is FP64; FP32 is used only to pre-classify squared
// distances that lie far from a threshold.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define XR_NATOM_COLS 24
#define XR_NPAIR_COLS 28
#define XR_NGENERAL 39
#define XR_NCOMP 14

// Atom table columns (xreac_gb300/forcefield.py: ATOM_COLUMNS).
enum AtomCol {
  A_R_S = 0, A_VALENCY, A_MASS, A_R_VDW, A_EPSILON, A_GAMMA, A_R_PI, A_VALENCY_E, A_ALPHA, A_GAMMA_W,
  A_VALENCY_BOC, A_P_OVUN5, A_CHI, A_ETA, A_P_HBOND, A_R_PI_PI, A_P_LP2, A_P_OVUN2, A_P_VAL3,
  A_VALENCY_VAL, A_P_VAL5, A_RCORE, A_ECORE, A_ACORE
};
// Pair table columns (xreac_gb300/forcefield.py: PAIR_COLUMNS).
enum PairCol {
  P_DE_S = 0, P_DE_P, P_DE_PP, P_BE1, P_BE2, P_BO1, P_BO2, P_BO3, P_BO4, P_BO5, P_BO6, P_OVUN1, P_OVC,
  P_V13COR, P_RS, P_RP, P_RPP, P_BOC3, P_BOC4, P_BOC5, P_D, P_ALPHA, P_GAMMA_W, P_RVDW, P_RCORE,
  P_ECORE, P_ACORE, P_GAMMA
};
// Energy components, in xreac's order (src/xreac/energy.py:26-41).
enum Comp {
  C_BOND = 0, C_ATOM, C_LONE_PAIR, C_MOLECULE, C_ANGLE, C_PENALTY, C_ANGLE_CONJ, C_HBOND, C_TORSION,
  C_CONJ, C_VDW, C_COULOMB, C_EFIELD, C_QEQ
};

// Status bits written by kernels instead of trapping; the host maps them to errors.
enum XrStatusBits {
  XR_S_CAPACITY = 1 << 0,     // a list outgrew its buffer: the host grows it and retries
  XR_S_SHIFT_RANGE = 1 << 1,  // an image shift does not fit the packed edge code
  XR_S_COLLINEAR = 1 << 2,    // collinear atoms in an active torsion
  XR_S_BOC_NAN = 1 << 3,      // NaN p_boc mixing on an active bond-order correction
  XR_S_CG = 1 << 4,           // QEq conjugate gradient hit its iteration limit
  XR_S_NONFINITE = 1 << 5,    // non-finite energy, charge or force
  XR_S_COINCIDENT = 1 << 6,   // two atoms closer than 1e-6 A
  XR_S_NONSPD = 1 << 7,       // QEq matrix not positive definite along a CG direction
  XR_S_BARRIER = 1 << 8,      // a grid barrier wait reached its iteration limit
  XR_S_REVERSE = 1 << 9,      // an edge without its reverse (internal consistency check)
  XR_S_LIMIT = 1 << 10,       // an atom has more active bonds than the packed item indices hold
  XR_S_BAD_PACK = 1 << 11,    // an atom's packed type and system word was out of range (internal check)
};

// Edge code: three 9-bit signed image shifts plus flags. Sx sits in the highest shift bits so the
// integer order of the 27 shift bits is the lexicographic order of (Sx, Sy, Sz).
#define XR_CODE_BOND (1u << 27)   // r <= min(5, cutoff): bond-order candidate
#define XR_CODE_HB (1u << 28)     // r <= min(7.5, cutoff): hydrogen-bond acceptor range
#define XR_CODE_HALF (1u << 29)   // canonical half edge (owns the pair)
#define XR_SHIFT_MASK ((1u << 27) - 1u)
#define XR_SHIFT_MAX 255

__host__ __device__ inline uint32_t xr_pack_shift(int sx, int sy, int sz) {
  return ((uint32_t)(sx + 256) << 18) | ((uint32_t)(sy + 256) << 9) | (uint32_t)(sz + 256);
}
__host__ __device__ inline int xr_sx(uint32_t c) { return (int)((c >> 18) & 511u) - 256; }
__host__ __device__ inline int xr_sy(uint32_t c) { return (int)((c >> 9) & 511u) - 256; }
__host__ __device__ inline int xr_sz(uint32_t c) { return (int)(c & 511u) - 256; }
// Shift bits of the reverse edge (-S).
__host__ __device__ inline uint32_t xr_neg_shift(uint32_t c) {
  return xr_pack_shift(-xr_sx(c), -xr_sy(c), -xr_sz(c));
}

// Per-system description (host-filled, uploaded with the batch).
struct XrSystem {
  int atom_off;          // first atom of the system
  int natoms;
  int periodic[3];       // pbc flags
  int reach[3];          // image scan half-width per direction (0 non-periodic, 0 for large cells)
  double cell[9];        // row vectors (identity when non-periodic)
  double inv[9];         // inverse of cell (row-vector convention: frac = x @ inv)
  double origin[3];      // reference point subtracted before FP32 rounding
  double total_charge;
  int has_guess;         // QEq starts from w.qguess (charges of an earlier step) instead of Q/n
  int ff_set;            // parameter set of the force field this system is evaluated with
  int chunk0;            // the system's first energy-reduction chunk (XR_CHUNK_ATOMS atoms each) in the batch
  // Cell list (when the call bins its atoms): cells per lattice direction (0: not binned), cell
  // offsets searched per direction, the system's first cell in the batch's cell arrays, and the map
  // of a fractional coordinate f to its cell, floor((f - cell_f0) * cell_scale) (wrapped f in
  // periodic directions, where cell_f0 = 0 and cell_scale = cells).
  int cell_n[3];
  int cell_reach[3];
  int cell_base;
  double cell_f0[3];
  double cell_scale[3];
  double rc, rc2, bond_cut, hb_cut;     // cutoff, cutoff^2, min(5, rc), min(7.5, rc)
  double inv_rc;                        // 1 / rc
  float cellf[9];
  float margin;          // bound on |FP32 squared distance - FP64 squared distance| (A^2)
  float rc2f, bc2f, hc2f;  // FP32 squared cutoff, bond cutoff and hydrogen-bond cutoff
};

// Force-field tables on the device (uploaded once per force field). A force field holds one or more
// parameter sets of the same elements and records: the general parameters and the three index tables
// (angle_index, torsion_index, hbond_index) are shared, every other table is per set. The pointers
// below are set 0's; set s's tables sit s * set_stride bytes after them (xr_ff_at).
struct XrFF {
  int ntypes;
  int vdw_type;
  int nsets;                  // parameter sets (1 unless the host loaded more)
  long long set_stride;       // bytes from one set's tables to the next set's
  double g[XR_NGENERAL];
  const double* atom;         // [T][XR_NATOM_COLS]
  const double* pair;         // [T*T][XR_NPAIR_COLS]
  const double* pair_gw;      // [T*T] (1/gamma_w)^g28 for shielded vdW
  const double* pair_logr;    // [T*T][3] log(r_s), log(r_p), log(r_pp) (0 where unused)
  const double* pair_rmax;    // [T*T] distance beyond which the uncorrected bond order stays below cut/4
  const double* pair_inv;     // [T*T][2] 1 / r_vdW, 1 / rcore (IEEE: infinite for a zero rcore)
  double inv_g28;             // 1 / g[28], the vdW shielding exponent
  // p = g[28], 1 / p, 1 / p - 1 and p - 1 as double-floats (hi, lo) for the pair kernel's vdW
  // shielding chain in double-float arithmetic
  float2 vdw_p, vdw_invp, vdw_invp_m1, vdw_p_m1;
  const int* is_carbon;       // [T] label is "C" (case-insensitive): C2 correction applies
  const int* hb_role;         // [T] 1 hydrogen-bond hydrogen, 2 donor/acceptor (p_hbond), 0 otherwise
  const int* angle_index;     // [T^3][2] first, count
  const double* angle;        // [R][7]
  const int* torsion_index;   // [T^4] row or -1 (rows with a nonzero V1, V2, V3 or V_conj)
  const double* torsion;      // [Q][5]
  const int* hbond_index;     // [T^3] row or -1
  const double* hbond;        // [H][4]
};

// Device work state of one batch. Sizes: A atoms, E edges, P pairs, B bonds, D = 2B bond-row
// entries, S systems. Capacities (cap_*) are the allocated lengths; counts live on the device.
struct XrWork {
  int A, S;
  int nE, nP, nB, nD;         // list sizes (known on the host once the count pass has been scanned)
  long long cap_E, cap_P, cap_B;
  int full_derivative;
  int cg_max_iter;
  double cg_tol;
  // Team waits of the QEq solver: polls before a wait gives up (0: the defaults, 2^22 for a cluster
  // exchange and 2^24 for a grid barrier), and, for tests of the give-up path, the number of the
  // team wait (1, 2, ...; 0: none) that waits for an arrival that never comes.
  long long wait_polls;
  int wait_fail_at;
  const XrSystem* sys;
  int* status;                // one int of XR_S_* bits
  int* counts;                // [8]: E, P, B, D totals (last entries of the scans), [4] QEq iterations, [5] candidates,
                              // [6] the longest candidate row of a cell-list build, [7] binned atoms
  // atoms
  const double4_32a* x;           // positions (w unused)
  const int* type;
  const int* sys_of;
  // Set when the host packed each atom's type and system into the unused 8 bytes of its position
  // (low and high 32 bits of x[a].w): k_prep then writes type and sys_of itself, and a call uploads
  // one array instead of three.
  int types_in_x;
  int prep_zero;              // k_prep zeroes the call's counters (evaluations; not the static count)
  // [A] the QEq preconditioner's bonds: the first and the last atom j of the kGroupMax - 1 atoms
  // before a that lies within 1.3 A of a (an image counts), or INT_MAX / -1 (set by k_pairs)
  int* qb_first;
  int* qb_last;
  int* bx_count;              // exported bonds of the call (zeroed by k_prep)
  int4* wrap;                 // integer lattice wrap of each atom
  float4* xw;                 // wrapped position minus origin, FP32
  float4* fw;                 // wrapped fractional coordinates, FP32
  int* cnt;                   // [4][A+1] counts, then exclusive scans in place:
                              //   0: edges, 1: half edges (pairs), 2: half bonds, 3: bond rows
  // candidate list: per atom, a superset of its edges as {j, shift bits} in canonical order (a skin
  // list kept from an earlier call, or a caller-supplied list); CSR by cand_cnt [A+1]
  int* cand_cnt;
  int2* cand_edge;
  // cell list of the call's atoms: atom_cell [A] (global cell index, -1 unbinned), atom_slot [A], the
  // cells' atom ranges cell_cnt [ncells + 1] (counts, then their exclusive scan) and cell_atoms [A]
  int* atom_cell;
  int* atom_slot;
  int* cell_cnt;
  int* cell_atoms;
  int ncells;
  // edges
  int2* edge;                 // {j, code}
  int* edge_pair;             // pair id of every edge (its own or its reverse's)
  int* edge_dbslot;           // bond-row slot of bond edges, -1 otherwise
  double* hval;               // per edge: 14.4 * shield of its pair (QEq matrix row entries)
  float* qch;                 // per edge: FP32 hval, then (a system whose rows exceed shared memory)
  unsigned short* qcj;        //   the pre-scaled row entry H_ij / D_jj and its column within the system
  // pairs
  int* pair_edge;             // half edge of each pair
  int* pair_i;                // source atom of each pair
  int* pair_bond;             // bond id or -1
  double* p_r;                // pair distance
  double* p_shield;           // shield(r)
  double* p_dshield;          // d shield / d r
  double* p_g;                // accumulated dE/dr on the pair (nonbonded, bonded and H-bond radial parts)
  double* p_evdw;             // vdW energy of the pair (both directions)
  double* p_ecoul;            // Coulomb energy of the pair
  // bonds
  int* bond_pair;
  int* bond_i;
  int* bond_j;
  double* b_r;                // bond length
  double* b_v;                // [3][B] bond vector from bond_i to bond_j's image
  double* b_fwd;              // [BF_N][B] forward intermediates (structure of arrays)
  double* b_adj;              // [BJ_N][B] adjoint accumulators
  double* b_e;                // [4][B] energies: bond, lone-pair C2, torsion, conjugation
  int2* dbrow;                // [D] {bond id, +1 if the atom is the bond's source else -1}
  int2* arow;                 // [D] active bond-row entries (bo > 0.001) at the start of each atom's range
  int* nact;                  // [A] number of active entries per atom
  int2* nzrow;                // [D] bond-row entries whose uncorrected bond order passed the cut (bo' > 0)
  int* nnz;                   // [A] number of such entries per atom (every other entry has zero bond orders)
  int* mids;                  // [B] bonds with bo > 0.001 (torsion middles), compacted
  int* nmids;                 // device count of mids
  int* mid_tiles;             // [ceil(cap_B / 128)] per-tile counts, then offsets, of the middles
  int* mlist;                 // [B] active bonds (uncorrected order passed the cut), in any order
  int* nmask;                 // length of mlist (device)
  // per-atom forward intermediates [AF_N][A] and adjoints [AJ_N][A] (structure of arrays)
  double* a_fwd;
  double* a_adj;
  double* a_e;                // [8][A] per-atom energies: lp, atom, angle, penalty, coa, hb, qeq, spare
  // charges and forces
  double* q;
  const double* qguess;       // [A] initial QEq charges of systems with has_guess (sum = total charge)
  int* qiters;                // [S] QEq conjugate-gradient iterations of each system
  double* qrhs;               // [A] adjoint QEq right-hand side (-dE/dq), full-derivative forces
  double* qadj;               // [A] adjoint QEq solution lambda (sum lambda = 0 per system)
  // Force-field parameter gradient dE/dtheta (null unless requested), summed over the batch:
  // [T*T][XR_NPAIR_COLS] pair-table columns, then [R][7] angle records.
  double* pgrad;
  int pgrad_angle_off;
  int pgrad_atom_off;         // [T][XR_NATOM_COLS] atom-table columns after the angle records (chi, eta)
  long long pgrad_stride;     // doubles per system: each system accumulates its own gradient
  double* f;                  // [A][3] gradient dE/dx accumulator (forces = -f)
  double* qwork;              // [XR_QW_N][A] QEq solver vectors
  double* red;                // reduction scratch for solvers
  unsigned* barrier;          // [2048] arrival counters of the QEq teams (indexed by a team's first block)
  int* qsplit;                // row splits of the cluster teams' systems (k_qeq_splits)
  // outputs
  double* energy;             // [S][16]: 14 components, total, pad
  double* props;              // [S][4]: dipole xyz, pad
  // deterministic per-system reductions: fixed atom chunks per system (XrSystem::chunk0 onwards)
  double* chunk_part;         // [nchunks][XR_PART_N]
  int nchunks;
};

// List sizes of the call as the device holds them (the totals of the count scans, counts[0..2]).
// Kernels over edges, pairs and bonds read these and stride over them, so a launch sequence
// recorded for one call (a CUDA graph) stays correct when it is replayed for a call whose lists
// have other sizes.
__device__ __forceinline__ int xr_num_edges(const XrWork& w) { return *(volatile const int*)(w.counts + 0); }
__device__ __forceinline__ int xr_num_pairs(const XrWork& w) { return *(volatile const int*)(w.counts + 1); }
__device__ __forceinline__ int xr_num_bonds(const XrWork& w) { return *(volatile const int*)(w.counts + 2); }

// The parameter-gradient block of the system of `atom` (pair table, then angle records).
__device__ inline double* xr_pgrad(const XrWork& w, int atom) { return w.pgrad + (size_t)w.sys_of[atom] * w.pgrad_stride; }

template <class P>
__device__ __forceinline__ const P* xr_byte_offset(const P* p, long long bytes) {
  return reinterpret_cast<const P*>(reinterpret_cast<const char*>(p) + bytes);
}

// The force field as seen by one parameter set: the per-set table pointers moved to that set.
__device__ __forceinline__ XrFF xr_ff_at(const XrFF& ff, int set) {
  XrFF f = ff;
  const long long o = (long long)set * ff.set_stride;
  f.atom = xr_byte_offset(ff.atom, o);
  f.pair = xr_byte_offset(ff.pair, o);
  f.pair_gw = xr_byte_offset(ff.pair_gw, o);
  f.pair_logr = xr_byte_offset(ff.pair_logr, o);
  f.pair_rmax = xr_byte_offset(ff.pair_rmax, o);
  f.pair_inv = xr_byte_offset(ff.pair_inv, o);
  f.is_carbon = xr_byte_offset(ff.is_carbon, o);
  f.hb_role = xr_byte_offset(ff.hb_role, o);
  f.angle = xr_byte_offset(ff.angle, o);
  f.torsion = xr_byte_offset(ff.torsion, o);
  f.hbond = xr_byte_offset(ff.hbond, o);
  return f;
}

// Parameter set of the system that `atom` belongs to (0 when the force field has one set).
__device__ __forceinline__ int xr_set_of(const XrFF& ff, const XrWork& w, int atom) {
  return ff.nsets > 1 ? w.sys[w.sys_of[atom]].ff_set : 0;
}

// The force field of the system that `atom` belongs to.
__device__ __forceinline__ XrFF xr_ff_of(const XrFF& ff, const XrWork& w, int atom) {
  return xr_ff_at(ff, xr_set_of(ff, w, atom));
}

// Per-atom forward slots in a_fwd.
enum AF { AF_DELTAP = 0, AF_TOTAL, AF_NLP, AF_VLPEX, AF_DLP, AF_DLPT, AF_SUMPI, AF_PROD, AF_OV1, AF_OV2, AF_DC,
          AF_SBO, AF_SBO2, AF_COUNT30, AF_E15, AF_N };
// Per-atom adjoint slots in a_adj. AJ_TOTAL, AJ_D, AJ_DB and AJ_SBO2 collect the direct
// sensitivities of the energy terms to total, d = total - valency, db = total - valency_boc and
// sbo2; the rest are filled by the chain kernels.
enum AJ { AJ_TOTAL = 0, AJ_D, AJ_DB, AJ_SBO2, AJ_OV1, AJ_OV2, AJ_DLPT, AJ_DLP, AJ_SUMPI, AJ_PRODSUM,
          AJ_TOTAL_ALL, AJ_DELTAP, AJ_N };
// Per-bond forward slots in b_fwd.
enum BF { BF_BO0 = 0, BF_PI0, BF_PP0, BF_DSIG, BF_DPI, BF_DPP, BF_BO, BF_PI, BF_PP, BF_SIG, BF_F1, BF_F4, BF_F5,
          BF_CORR, BF_MASK, BF_DF1I, BF_DF1J, BF_N };
// Per-bond adjoint slots in b_adj: direct sensitivities to the thresholded bo, pi, pp, sigma, then
// the chain's partial derivatives with respect to the uncorrected bond orders and the two ends' Delta'.
enum BJ { BJ_BO = 0, BJ_PI, BJ_PP, BJ_SIG, BJ_BO0, BJ_PI0, BJ_PP0, BJ_CI, BJ_CJ, BJ_N };

#define XR_QW_N 12
#define XR_PART_N 24
#define XR_CHUNK_ATOMS 32

// Kernel launchers (defined in the .cu files, called by the engine).
void xr_launch_topology(const XrWork& w, cudaStream_t st);  // xr_launch_prep, then xr_launch_count
void xr_launch_prep(const XrWork& w, cudaStream_t st);      // wrapped FP32 coordinates (k_prep)
void xr_launch_count(const XrWork& w, cudaStream_t st);     // all-pairs image scan, counts (k_neighbors<false>)
void xr_launch_rows(const XrWork& w, cudaStream_t st);      // all-pairs image scan, rows (k_neighbors<true>)
void xr_launch_scan(const XrWork& w, cudaStream_t st);
void xr_launch_topology_fill(const XrWork& w, cudaStream_t st);
// Candidate list at the cutoff of w.sys (descriptors at rc + 2 skin): fill=false counts into cand_cnt
// and scans it (total into counts[5]); fill=true writes cand_edge.
void xr_launch_candidates(const XrWork& w, bool fill, cudaStream_t st);
// The edges within the cutoff of the candidate list: fill=false counts into cnt (scanned by
// xr_launch_scan), fill=true writes the rows, pairs and bonds.
void xr_launch_filter(const XrWork& w, bool fill, cudaStream_t st);
// Cell list of the atoms binned by k_prep (atom_cell): counts per cell, their scan, cell_atoms.
void xr_launch_cells(const XrWork& w, cudaStream_t st);
// Candidate list at the cutoff of w.sys from the cell list, in no particular order within a row:
// fill=false counts into cand_cnt, scans it (total into counts[5]) and records the longest row in
// counts[6]; fill=true writes cand_edge.
void xr_launch_cell_candidates(const XrWork& w, bool fill, cudaStream_t st);
// Sorts every candidate row into canonical (j, Sx, Sy, Sz) order; rows hold at most max_row entries
// (at most XR_ROW_SORT_MAX).
void xr_launch_row_sort(const XrWork& w, int max_row, cudaStream_t st);
#define XR_ROW_SORT_MAX 8192
void xr_launch_reverse(const XrWork& w, cudaStream_t st);
void xr_launch_pairs(const XrWork& w, const XrFF& ff, cudaStream_t st);
int xr_launch_qeq(const XrWork& w, const XrFF& ff, cudaStream_t st, int nblocks, const int4* map, int nteam,
                  const int* small, int nsmall, bool adjoint = false);
void xr_launch_charge_response(const XrWork& w, const XrFF& ff, cudaStream_t st, int stage);
// Parameter gradient of the QEq parameters from the charges and the adjoint solution (qadj):
// chi and eta of every atom's type, the pair table's gamma of every pair's type.
void xr_launch_qeq_param_gradient(const XrWork& w, const XrFF& ff, cudaStream_t st);
int xr_qeq_coop_blocks_per_sm();
// Thread-block-cluster QEq solver: `csize` blocks per cluster (kQeqClusterBatch for batches, whose
// many systems share the SMs; kQeqClusterSingle for a single system, whose solve time is the call's
// latency); how many such clusters can be resident at once (0: unavailable); and its launch over
// `list` = nbig cluster systems followed by nsmall single-block systems (nblocks a multiple of csize).
constexpr int kQeqClusterBatch = 4;
constexpr int kQeqClusterSingle = 8;
int xr_qeq_max_clusters(int csize);
int xr_launch_qeq_cluster(const XrWork& w, const XrFF& ff, cudaStream_t st, int csize, int nblocks, const int* list,
                          int nbig, int nsmall, bool adjoint = false);
void xr_launch_bond_orders(const XrWork& w, const XrFF& ff, cudaStream_t st);  // k_bo1, k_deltap, k_bo2
void xr_launch_bonded(const XrWork& w, const XrFF& ff, cudaStream_t st);       // energy terms and adjoint chain
void xr_launch_forces(const XrWork& w, const XrFF& ff, cudaStream_t st);
void xr_launch_reduce(const XrWork& w, const XrFF& ff, cudaStream_t st);
