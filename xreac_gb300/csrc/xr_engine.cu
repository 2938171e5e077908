// C ABI and orchestration of one evaluation (or a ragged batch of them) on the device.
//
// Sequence per call: upload positions and system descriptors -> count neighbour rows -> scan ->
// (grow buffers) -> fill rows, pairs, bonds, reverse map -> pair kernel (vdW, shield) -> QEq ->
// bond orders, bonded energies and adjoints -> Coulomb energy and force assembly -> per-system
// reductions -> one copy of the packed per-atom results back to the host (or straight into device outputs).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "xr_common.cuh"
#include "xr_describe.h"
#include "xr_lists.h"
#include "xreac_gb300.h"

namespace {

// Most co-resident blocks of the QEq solver kernel (its team map and barrier counters).
constexpr int kQeqBlocks = 2048;

template <class T>
bool grow(T** p, size_t* cap, size_t need) {
  if (*p && *cap >= need) return true;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  size_t n = std::max<size_t>(need, 1);
  n = n + n / 4 + 64;
  if (cudaMalloc((void**)p, n * sizeof(T)) != cudaSuccess) {
    *p = nullptr;
    return false;
  }
  *cap = n;
  return true;
}

}  // namespace

// Per-set tables of a force field, in their order inside a set's block.
enum FFPart { FP_ATOM = 0, FP_PAIR, FP_GW, FP_LOGR, FP_RMAX, FP_PINV, FP_CARBON, FP_HBROLE, FP_ANGLE, FP_TORSION, FP_HBOND,
              FP_N };

struct xr_ff {
  XrFF d{};
  // Device layout (one allocation): nsets blocks of set_bytes, one per parameter set, then the shared
  // index tables (angle, torsion, hydrogen bond) in shared_bytes.
  void* blob = nullptr;
  size_t blob_bytes = 0;
  size_t set_bytes = 0, shared_bytes = 0;
  size_t part_off[FP_N] = {};        // offsets of the per-set tables inside a block
  size_t shared_off[3] = {};         // offsets of the index tables inside the shared region
  std::vector<unsigned char> set0;   // host copy of set 0's block (the default for tables not given)
  int nsets = 1;
  int device = 0;
  int nangle = 0, ntorsion = 0, nhbond = 0;
};

struct xr_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  double cg_tol = 1e-13;
  int cg_max = 2000;
  long long wait_polls = 0;  // QEq team waits: poll limit (0: defaults) and the wait a test makes run out
  int wait_fail_at = 0;
  // Candidate lists (a superset of each atom's edges, {j, shift bits} rows in canonical order): the
  // skin list kept for reuse, or the rows of a caller-supplied list.
  int* cand_cnt = nullptr;  // [A+1] row offsets
  size_t ccand_cnt = 0;
  int2* cand_edge = nullptr;
  size_t ccand_edge = 0;
  XrSystem* sys_list = nullptr;  // descriptors at the list cutoff rc + 2 skin (builds only)
  size_t csys_list = 0;
  int* h_cand_cnt = nullptr;  // pinned staging of a supplied list
  size_t ch_cand_cnt = 0;
  int2* h_cand_edge = nullptr;
  size_t ch_cand_edge = 0;
  XrSystem* h_sys_list = nullptr;
  size_t ch_sys_list = 0;
  // Device bytes the context holds (its buffers, as grown; xr_ctx_memory).
  long long dev_bytes = 0;
  // CUDA graphs of the launch sequence after the list count (xr_ctx_set_graphs): a sequence is
  // recorded the second time its launch key occurs and replayed whenever the key occurs again; the
  // kGraphCache most recently used graphs are kept.
  bool graphs = true;
  struct GraphEntry {
    cudaGraphExec_t exec;
    long long launches;       // kernels in the recorded sequence
    unsigned long long used;  // clock of the last use
  };
  std::unordered_map<std::string, GraphEntry> gcache;
  std::unordered_map<std::string, int> gseen;  // keys not recorded yet: occurrences (-1: not recordable)
  unsigned long long gclock = 0;
  static constexpr size_t kGraphCache = 128;
  static constexpr size_t kGraphSeen = 4096;
  int last_graph = 0;  // of the last call: 0 launched directly, 1 recorded, 2 replayed
  // Cell list (xr_ctx_set_cell_list): 0 chooses per call, 1 always, -1 never.
  int cell_mode = 0;
  int* atom_cell = nullptr;
  size_t catom_cell = 0;
  int* atom_slot = nullptr;
  size_t catom_slot = 0;
  int* cell_cnt = nullptr;
  size_t ccell_cnt = 0;
  int* cell_atoms = nullptr;
  size_t ccell_atoms = 0;
  // Skin reuse (xr_ctx_set_skin): the list of the last call is reused by a call on the same systems
  // (atom counts, types, cells, pbc, cutoff) in which no atom moved more than `skin` from where it was
  // when the list was built; the list holds every image within rc + 2 skin then (ASE's convention).
  double skin = 0.0;
  bool cache_valid = false;
  double cache_rc = 0.0, cache_skin = 0.0;
  std::vector<double> cache_x0;   // [3A] positions at the build
  std::vector<int> cache_types;   // [A]
  std::vector<int> cache_shape;   // per system: natoms, pbc[3]
  std::vector<double> cache_cell; // per system: 9 cell entries (identity when not periodic)
  long long list_builds = 0;      // candidate lists built since the context was made
  int list_mode = 0;              // of the last call: 0 scanned, 1 list built, 2 list reused, 3 supplied,
                                  // 4 cell-list search, 5 list built from the cell list
  int nsm = 0;
  int coop_per_sm = 0;
  int max_clusters = 0;  // resident thread-block clusters of the cluster QEq solver (0: unavailable),
  int max_clusters_batch = 0;  // for the single-system and the batch cluster size
  long long launches = 0;
  long long h2d_bytes = 0, d2h_bytes = 0;  // host<->device bytes moved by the last evaluation
  int qeq_iterations = 0;                   // CG iterations of the last evaluation (largest system)
  long long list_sizes[6] = {};             // edges, pairs, bond candidates, bond rows, active bonds, middles
  int* qiters = nullptr;                    // [S] per-system iterations (device)
  size_t cqiters = 0;
  std::vector<int> h_qiters;
  // last batch layout (host copies for export)
  std::vector<XrSystem> host_sys;
  std::vector<int> host_cnt;  // [4][A+1] scans of the last evaluation
  int last_A = 0;
  // atom-sized buffers
  size_t capA = 0;
  double4_32a* x = nullptr;
  size_t cx = 0;
  int* type = nullptr;
  size_t ctype = 0;
  int* sys_of = nullptr;
  size_t csys_of = 0;
  int4* wrap = nullptr;
  size_t cwrap = 0;
  float4* xw = nullptr;
  size_t cxw = 0;
  float4* fw = nullptr;
  size_t cfw = 0;
  int* cnt = nullptr;
  size_t ccnt = 0;
  double* a_fwd = nullptr;
  size_t ca_fwd = 0;
  double* a_adj = nullptr;
  size_t ca_adj = 0;
  double* a_e = nullptr;
  size_t ca_e = 0;
  double* q = nullptr;
  size_t cq = 0;
  double* qguess = nullptr;
  size_t cqguess = 0;
  double* qrhs = nullptr;
  size_t cqrhs = 0;
  double* pgrad = nullptr;  // force-field parameter gradient of the last call (when requested)
  size_t cpgrad = 0;
  std::vector<double> h_pgrad;
  long long pgrad_pairs = 0, pgrad_angles = 0, pgrad_atoms = 0;
  int pgrad_systems = 0;  // systems of the last call with XR_FLAG_PARAM_GRADIENT (one block each)
  double* qadj = nullptr;
  size_t cqadj = 0;
  double* f = nullptr;
  size_t cf = 0;
  double* qwork = nullptr;
  size_t cqwork = 0;
  double* outbuf = nullptr;
  size_t coutbuf = 0;
  int2* arow = nullptr;
  size_t carow = 0;
  int2* nzrow = nullptr;
  int* nnz = nullptr;
  size_t cnnz = 0;
  int* mids = nullptr;
  int* nmids = nullptr;  // [2] torsion middles, active bonds
  int* mid_tiles = nullptr;  // per 128-bond tile: middles counts, then offsets
  size_t cmid_tiles = 0;
  int* qsplit = nullptr;     // row splits of the cluster teams' systems
  size_t cqsplit = 0;
  int* mlist = nullptr;
  int* nact = nullptr;
  size_t cnact = 0;
  int* qb_first = nullptr;
  size_t cqb_first = 0;
  int* qb_last = nullptr;
  size_t cqb_last = 0;
  double* chunk_part = nullptr;
  size_t cchunk_part = 0;
  // edge / pair / bond buffers
  int2* edge = nullptr;
  size_t cedge = 0;
  int* edge_pair = nullptr;
  size_t cedge_pair = 0;
  int* edge_dbslot = nullptr;
  size_t cedge_dbslot = 0;
  double* hval = nullptr;
  size_t chval = 0;
  float* qch = nullptr;  // FP32 pre-scaled QEq rows of systems whose rows exceed shared memory
  size_t cqch = 0;
  unsigned short* qcj = nullptr;
  size_t cqcj = 0;
  int *pair_edge = nullptr, *pair_i = nullptr, *pair_bond = nullptr;
  size_t cpair_edge = 0, cpair_i = 0, cpair_bond = 0;
  double *p_r = nullptr, *p_shield = nullptr, *p_dshield = nullptr, *p_g = nullptr, *p_evdw = nullptr, *p_ecoul = nullptr;
  size_t cp_r = 0, cp_shield = 0, cp_dshield = 0, cp_g = 0, cp_evdw = 0, cp_ecoul = 0;
  int *bond_pair = nullptr, *bond_i = nullptr, *bond_j = nullptr;
  size_t cbond_pair = 0, cbond_i = 0, cbond_j = 0;
  double *b_r = nullptr, *b_v = nullptr, *b_fwd = nullptr, *b_adj = nullptr, *b_e = nullptr;
  size_t cb_r = 0, cb_v = 0, cb_fwd = 0, cb_adj = 0, cb_e = 0;
  size_t capB = 0;
  int2* dbrow = nullptr;
  size_t cdbrow = 0;
  // system-sized and misc
  XrSystem* sys = nullptr;
  size_t csys = 0;
  double* energy = nullptr;
  size_t cenergy = 0;
  double* props = nullptr;
  size_t cprops = 0;
  int* status = nullptr;
  int* counts = nullptr;
  unsigned* barrier = nullptr;
  int4* qmap = nullptr;  // [2048] QEq team blocks of the current batch
  int* qsmall = nullptr;
  size_t cqsmall = 0;
  std::vector<int4> h_qmap;
  std::vector<int> h_qsmall;
  double* red = nullptr;
  size_t cred = 0;
  // per-stage timing (CUDA events on the context stream), enabled by xr_ctx_set_profiling
  bool profile = false;
  static constexpr int kStages = 9;
  cudaEvent_t ev[kStages + 1] = {};
  double stage_ms[kStages] = {};
  long long stage_calls = 0;
  // compact export of nonzero bonds: {bond, i, j, code} and bo
  int* bx_count = nullptr;
  std::vector<int4> h_bx_meta;
  std::vector<double> h_bx_bo;
  // pinned host staging (every host<->device copy of a call is asynchronous from/to these)
  double4_32a* h_x = nullptr;
  size_t ch_x = 0;
  int* h_types = nullptr;
  size_t ch_types = 0;
  int* h_sysof = nullptr;
  size_t ch_sysof = 0;
  XrSystem* h_sysd = nullptr;
  size_t ch_sysd = 0;
  int4* h_qmap_p = nullptr;
  size_t ch_qmap_p = 0;
  int* h_qsmall_p = nullptr;
  size_t ch_qsmall_p = 0;
  double* h_pg = nullptr;
  size_t ch_pg = 0;
  double* h_out = nullptr;
  size_t ch_out = 0;
  double* h_guess = nullptr;
  size_t ch_guess = 0;
  int* h_small = nullptr;  // status + counts
};

namespace {

// grow() for a context's buffer, keeping the context's device-byte count.
template <class T>
bool grow(xr_ctx* c, T** p, size_t* cap, size_t need) {
  const long long before = *p ? (long long)(*cap * sizeof(T)) : 0;
  const bool ok = grow(p, cap, need);
  c->dev_bytes += (*p ? (long long)(*cap * sizeof(T)) : 0) - before;
  return ok;
}

int cuda_fail(xr_ctx* c, cudaError_t e, const char* where) {
  c->err = std::string("CUDA error in ") + where + ": " + cudaGetErrorString(e);
  return XR_ECUDA;
}

template <class T>
bool host_grow(T** p, size_t* cap, size_t need) {
  if (*p && *cap >= need) return true;
  if (*p) cudaFreeHost(*p);
  *p = nullptr;
  *cap = 0;
  size_t n = std::max<size_t>(need, 1);
  n = n + n / 4 + 64;
  if (cudaMallocHost((void**)p, n * sizeof(T)) != cudaSuccess) {
    *p = nullptr;
    return false;
  }
  *cap = n;
  return true;
}

// Per-system descriptor (xr_describe.h) plus the system's total charge.
int build_system(xr_ctx* c, const xr_system& in, int atom_off, double rc, XrSystem& S, double4_32a* xpack) {
  const char* msg = "";
  const int code = xr_host::describe_system(in, atom_off, rc, S, xpack, &msg);
  if (code != XR_OK) {
    c->err = msg;
    return code;
  }
  S.total_charge = in.total_charge;
  return XR_OK;
}

#define GROW(field, n)                                      \
  do {                                                      \
    if (!grow(c, &c->field, &c->c##field, (size_t)(n))) return false; \
  } while (0)

bool ensure_atoms(xr_ctx* c, int A, int S) {
  GROW(x, A);
  GROW(type, A);
  GROW(sys_of, A);
  GROW(wrap, A);
  GROW(xw, A);
  GROW(fw, A);
  GROW(cnt, 4 * (size_t)(A + 1));
  GROW(a_fwd, (size_t)AF_N * A);
  GROW(a_adj, (size_t)AJ_N * A);
  GROW(a_e, 8 * (size_t)A);
  GROW(q, A);
  GROW(qguess, A);
  GROW(qrhs, A);
  GROW(qadj, A);
  GROW(f, 3 * (size_t)A);
  GROW(qwork, (size_t)XR_QW_N * A);
  GROW(outbuf, 8 * (size_t)A);
  GROW(nact, A);
  GROW(nnz, A);
  GROW(qb_first, A);
  GROW(qb_last, A);
  GROW(qsmall, S);
  GROW(qiters, S);
  GROW(sys, S);
  GROW(qsplit, 9 * (size_t)S + 2 * (size_t)kQeqBlocks + 9);  // cluster teams' splits, or two per grid-team block
  GROW(energy, 16 * (size_t)S);
  GROW(props, 4 * (size_t)S);
  const size_t scan_ints = 4 * ((size_t)(A + 1) / 4096 + 2);
  const size_t red = std::max<size_t>(scan_ints / 2 + 8, (size_t)4 * 8 * 2048);
  GROW(red, red);
  return true;
}

// Device bytes per bond slot of the bond arrays (structures of arrays with stride capB).
constexpr long long kBondBytes = 3 * sizeof(int) + 4 * sizeof(double) + (BF_N + BJ_N + 4) * sizeof(double) +
                                 6 * sizeof(int2) + 2 * sizeof(int);

bool ensure_lists(xr_ctx* c, long long E, long long P, long long B) {
  GROW(mid_tiles, B / 128 + 2);
  GROW(edge, E);
  GROW(edge_pair, E);
  GROW(edge_dbslot, E);
  GROW(hval, E);
  GROW(qch, E);
  GROW(qcj, E);
  GROW(pair_edge, P);
  GROW(pair_i, P);
  GROW(pair_bond, P);
  GROW(p_r, P);
  GROW(p_shield, P);
  GROW(p_dshield, P);
  GROW(p_g, P);
  GROW(p_evdw, P);
  GROW(p_ecoul, P);
  // bond arrays are structures of arrays with stride capB
  if (c->capB < (size_t)B || !c->b_fwd) {
    size_t nb = std::max<size_t>((size_t)B, 1);
    nb = nb + nb / 4 + 64;
    c->dev_bytes -= (long long)(c->b_fwd ? c->capB : 0) * kBondBytes;
    cudaFree(c->bond_pair);
    cudaFree(c->bond_i);
    cudaFree(c->bond_j);
    cudaFree(c->b_r);
    cudaFree(c->b_v);
    cudaFree(c->b_fwd);
    cudaFree(c->b_adj);
    cudaFree(c->b_e);
    cudaFree(c->dbrow);
    cudaFree(c->arow);
    cudaFree(c->nzrow);
    cudaFree(c->mids);
    cudaFree(c->mlist);
    c->mlist = nullptr;
    c->arow = nullptr;
    c->nzrow = nullptr;
    c->mids = nullptr;
    c->bond_pair = c->bond_i = c->bond_j = nullptr;
    c->b_r = c->b_v = c->b_fwd = c->b_adj = c->b_e = nullptr;
    c->dbrow = nullptr;
    bool ok = cudaMalloc((void**)&c->bond_pair, nb * sizeof(int)) == cudaSuccess &&
              cudaMalloc((void**)&c->bond_i, nb * sizeof(int)) == cudaSuccess &&
              cudaMalloc((void**)&c->bond_j, nb * sizeof(int)) == cudaSuccess &&
              cudaMalloc((void**)&c->b_r, nb * sizeof(double)) == cudaSuccess &&
              cudaMalloc((void**)&c->b_v, 3 * nb * sizeof(double)) == cudaSuccess &&
              cudaMalloc((void**)&c->b_fwd, (size_t)BF_N * nb * sizeof(double)) == cudaSuccess &&
              cudaMalloc((void**)&c->b_adj, (size_t)BJ_N * nb * sizeof(double)) == cudaSuccess &&
              cudaMalloc((void**)&c->b_e, 4 * nb * sizeof(double)) == cudaSuccess &&
              cudaMalloc((void**)&c->dbrow, 2 * nb * sizeof(int2)) == cudaSuccess &&
              cudaMalloc((void**)&c->arow, 2 * nb * sizeof(int2)) == cudaSuccess &&
              cudaMalloc((void**)&c->nzrow, 2 * nb * sizeof(int2)) == cudaSuccess &&
              cudaMalloc((void**)&c->mids, nb * sizeof(int)) == cudaSuccess &&
              cudaMalloc((void**)&c->mlist, nb * sizeof(int)) == cudaSuccess;
    if (!ok) return false;
    c->capB = nb;
    c->dev_bytes += (long long)nb * kBondBytes;
  }
  return true;
}

void fill_work(xr_ctx* c, XrWork& w, int A, int S, unsigned flags) {
  std::memset(&w, 0, sizeof(w));
  w.A = A;
  w.S = S;
  w.full_derivative = (flags & XR_FLAG_FULL_DERIVATIVE) ? 1 : 0;
  w.cg_max_iter = c->cg_max;
  w.cg_tol = c->cg_tol;
  w.wait_polls = c->wait_polls;
  w.wait_fail_at = c->wait_fail_at;
  w.sys = c->sys;
  w.status = c->status;
  w.counts = c->counts;
  w.x = c->x;
  w.type = c->type;
  w.sys_of = c->sys_of;
  w.bx_count = c->bx_count;
  w.qb_first = c->qb_first;
  w.qb_last = c->qb_last;
  w.wrap = c->wrap;
  w.xw = c->xw;
  w.fw = c->fw;
  w.cnt = c->cnt;
  w.a_fwd = c->a_fwd;
  w.a_adj = c->a_adj;
  w.a_e = c->a_e;
  w.q = c->q;
  w.f = c->f;
  w.qwork = c->qwork;
  w.red = c->red;
  w.barrier = c->barrier;
  w.qsplit = c->qsplit;
  w.energy = c->energy;
  w.props = c->props;
  w.nact = c->nact;
  w.nnz = c->nnz;
  w.chunk_part = c->chunk_part;
}

void attach_lists(xr_ctx* c, XrWork& w) {
  w.cand_cnt = c->cand_cnt;
  w.cand_edge = c->cand_edge;
  w.cap_E = (long long)c->cedge;
  w.cap_P = (long long)c->cpair_edge;
  w.cap_B = (long long)c->capB;
  w.edge = c->edge;
  w.edge_pair = c->edge_pair;
  w.edge_dbslot = c->edge_dbslot;
  w.hval = c->hval;
  w.qch = c->qch;
  w.qcj = c->qcj;
  w.pair_edge = c->pair_edge;
  w.pair_i = c->pair_i;
  w.pair_bond = c->pair_bond;
  w.p_r = c->p_r;
  w.p_shield = c->p_shield;
  w.p_dshield = c->p_dshield;
  w.p_g = c->p_g;
  w.p_evdw = c->p_evdw;
  w.p_ecoul = c->p_ecoul;
  w.bond_pair = c->bond_pair;
  w.bond_i = c->bond_i;
  w.bond_j = c->bond_j;
  w.b_r = c->b_r;
  w.b_v = c->b_v;
  w.b_fwd = c->b_fwd;
  w.b_adj = c->b_adj;
  w.b_e = c->b_e;
  w.dbrow = c->dbrow;
  w.arow = c->arow;
  w.nzrow = c->nzrow;
  w.mids = c->mids;
  w.mid_tiles = c->mid_tiles;
  w.nmids = c->nmids;
  w.nmask = c->nmids + 1;
  w.qguess = c->qguess;
  w.qrhs = c->qrhs;
  w.qadj = c->qadj;
  w.qiters = c->qiters;
  w.mlist = c->mlist;
}

// One exported bond: (bond id, i, j, image code) and its corrected order.
struct __align__(16) XrBondRecord {
  int4 meta;
  double bo;
  double pad;
};

// The result block of a call, in doubles from the start of outbuf (device) and h_out (host): per-atom
// values [8 A], energies [16 S], properties [4 S], the tail of ints (kTailInts counters, the systems'
// QEq iterations [S], the scans [4 (A + 1)]), then the exported bonds as 32-byte records. Kernels
// write all of it, so one copy brings a call's results back.
constexpr int kTailInts = 5;  // status, exported bonds, QEq iterations, torsion middles, active bonds
struct ResultLayout {
  size_t energy, props, tail, bonds, end;
};
ResultLayout result_layout(int A, int nsys, long long nB) {
  ResultLayout L;
  L.energy = 8 * (size_t)A;
  L.props = L.energy + 16 * (size_t)nsys;
  L.tail = L.props + 4 * (size_t)nsys;
  const size_t tail_ints = kTailInts + (size_t)nsys + 4 * (size_t)(A + 1);
  L.bonds = (L.tail + (tail_ints + 1) / 2 + 3) / 4 * 4;
  L.end = L.bonds + 4 * (size_t)std::max<long long>(nB, 0);
  return L;
}

// Packs forces (-dE/dx), charges, total bond orders, lone pairs and bond counts per atom.
__global__ void k_pack(XrWork w, double* out) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= w.A) return;
  out[8 * a + 0] = -w.f[3 * a + 0];
  out[8 * a + 1] = -w.f[3 * a + 1];
  out[8 * a + 2] = -w.f[3 * a + 2];
  out[8 * a + 3] = w.q[a];
  out[8 * a + 4] = w.a_fwd[(size_t)AF_TOTAL * w.A + a];
  out[8 * a + 5] = w.a_fwd[(size_t)AF_NLP * w.A + a];
  out[8 * a + 6] = w.a_fwd[(size_t)AF_COUNT30 * w.A + a];
  out[8 * a + 7] = 0.0;
}

// Device-output variant for a single system: writes straight into the caller's arrays.
__global__ void k_unpack_device(XrWork w, double* forces, double* charges, double* tbo, double* nlp, int* counts) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= w.A) return;
  if (forces) {
    forces[3 * a + 0] = -w.f[3 * a + 0];
    forces[3 * a + 1] = -w.f[3 * a + 1];
    forces[3 * a + 2] = -w.f[3 * a + 2];
  }
  if (charges) charges[a] = w.q[a];
  if (tbo) tbo[a] = w.a_fwd[(size_t)AF_TOTAL * w.A + a];
  if (nlp) nlp[a] = w.a_fwd[(size_t)AF_NLP * w.A + a];
  if (counts) counts[a] = (int)w.a_fwd[(size_t)AF_COUNT30 * w.A + a];
}

// Energies, properties and the tail of ints into the result block (its layout: result_layout), after
// every other kernel of the call.
__global__ void k_gather_tail(XrWork w, double* block, size_t energy_off, size_t tail_off) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
  double* e = block + energy_off;
  for (int k = t; k < 20 * w.S; k += nt) e[k] = k < 16 * w.S ? w.energy[k] : w.props[k - 16 * w.S];
  int* ti = reinterpret_cast<int*>(block + tail_off);
  if (t == 0) {
    ti[0] = *w.status;
    ti[1] = *w.bx_count;
    ti[2] = w.counts[4];
    ti[3] = w.nmids[0];
    ti[4] = w.nmids[1];
  }
  for (int k = t; k < w.S; k += nt) ti[kTailInts + k] = w.qiters[k];
  int* tc = ti + kTailInts + w.S;
  const int nc = 4 * (w.A + 1);
  for (int k = t; k < nc; k += nt) tc[k] = w.cnt[k];
}

__global__ void k_positions_from_device(const double* pos, double4_32a* x, int n) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  x[a] = make_double4_32a(pos[3 * a], pos[3 * a + 1], pos[3 * a + 2], 0.0);
}

// Nonzero corrected bond orders, compacted with warp-aggregated atomics; the host restores bond order.
__global__ void k_bond_export(XrWork w, XrBondRecord* rec, int* counter) {
  const int nb = xr_num_bonds(w);
  const int lane = threadIdx.x & 31;
  for (int b0 = blockIdx.x * blockDim.x; b0 < nb; b0 += gridDim.x * blockDim.x) {  // uniform per block
    const int b = b0 + threadIdx.x;
    const double bo = b < nb ? w.b_fwd[(size_t)BF_BO * w.cap_B + b] : 0.0;
    const bool keep = b < nb && bo != 0.0;
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    int base = 0;
    if (lane == 0 && m) base = atomicAdd(counter, __popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (keep) {
      const int slot = base + __popc(m & ((1u << lane) - 1u));
      const int code = w.edge[w.pair_edge[w.bond_pair[b]]].y;
      XrBondRecord r;
      r.meta = make_int4(b, w.bond_i[b], w.bond_j[b], code);
      r.bo = bo;
      r.pad = 0.0;
      rec[slot] = r;
    }
  }
}

void stage(xr_ctx* c, int k, cudaStream_t st) {
  if (c->profile) cudaEventRecord(c->ev[k], st);
}

int status_to_code(xr_ctx* c, int st) {
  if (st & XR_S_COINCIDENT) {
    c->err = "Coincident atoms are not supported";
    return XR_ECOINCIDENT;
  }
  if (st & (XR_S_SHIFT_RANGE | XR_S_CAPACITY)) {
    c->err = "An image shift exceeds the supported range of +-255 cells; wrap the positions into the cell";
    return XR_ECAPACITY;
  }
  if (st & XR_S_LIMIT) {
    c->err = "An atom has more than 16383 active bonds; the many-body item lists cannot index them";
    return XR_ECAPACITY;
  }
  if (st & XR_S_REVERSE) {
    c->err = "neighbors must include both directions: (i, j, S) and (j, i, -S)";
    return XR_EINPUT;
  }
  if (st & XR_S_BAD_PACK) {
    c->err = "internal error: an atom's packed type and system were out of range";
    return XR_ECUDA;
  }
  if (st & XR_S_BOC_NAN) {
    c->err = "Invalid p_boc mixing for an active bond-order correction";
    return XR_EBADPARAM;
  }
  if (st & XR_S_COLLINEAR) {
    c->err = "Collinear atoms in an active torsion: the dihedral derivative is undefined; perturb the geometry";
    return XR_ECOLLINEAR;
  }
  if (st & XR_S_BARRIER) {
    c->err = "A device-side wait of the QEq solver gave up (a scheduling failure, not an input error); "
             "the evaluation may be repeated";
    return XR_EWAIT;
  }
  if (st & XR_S_NONSPD) {
    c->err = "Singular QEq system; check the geometry and parameters";
    return XR_ESINGULAR;
  }
  if (st & XR_S_CG) {
    c->err = "QEq did not converge within the iteration limit; raise it (set_qeq) or check the geometry and "
             "parameters";
    return XR_ECG_NOCONV;
  }
  if (st & XR_S_NONFINITE) {
    c->err = "Non-finite energy, charges, or forces; check the geometry";
    return XR_ENONFINITE;
  }
  return XR_OK;
}

// QEq work plan of a batch for the solver kernel (at most kQeqBlocks co-resident blocks). A team
// of ceil(n / 32) blocks (32 rows per 1024-thread block) solves a large system with grid-level
// reductions, which shortens one solve; a single block solves a system with block barriers only,
// which costs the fewest SM-cycles. So a single-system call gives a team to a system above
// kQeqSmall atoms, and a batch (throughput) only to systems above kQeqBatchBlock atoms. Teams are
// scaled down when they do not fit; the other systems are taken, largest first, by whichever block
// is free. A one-block team is no team: such a system joins the small ones.
constexpr int kQeqSmall = 160;
#ifndef XR_QEQ_TEAM_ROWS
#define XR_QEQ_TEAM_ROWS 32
#endif
constexpr int kQeqTeamRows = XR_QEQ_TEAM_ROWS;  // rows per block of a grid-wide team (a multiple of 32)
constexpr int kQeqBatchBlock = 1024;

void plan_qeq(xr_ctx* c, const xr_system* sys, int nsys, int* nblocks, int* nteam, int* nsmall) {
  const int budget = std::min(c->nsm * c->coop_per_sm, kQeqBlocks);
  const int team_above = nsys > 1 ? kQeqBatchBlock : kQeqSmall;
  std::vector<int> large, small;
  for (int s = 0; s < nsys; ++s) (sys[s].natoms > team_above ? large : small).push_back(s);
  std::sort(large.begin(), large.end(), [&](int a, int b) { return sys[a].natoms > sys[b].natoms; });
  std::vector<int> team(large.size());
  for (;;) {
    const int small_blocks = small.empty() ? 0 : (large.empty() ? std::min<int>((int)small.size(), budget)
                                                                 : std::min<int>((int)small.size(), std::max(1, budget / 4)));
    const int avail = budget - small_blocks;
    long long want = 0;
    for (size_t k = 0; k < large.size(); ++k) want += (sys[large[k]].natoms + kQeqTeamRows - 1) / kQeqTeamRows;
    long long have = 0;
    for (size_t k = 0; k < large.size(); ++k) {
      const long long d = (sys[large[k]].natoms + kQeqTeamRows - 1) / kQeqTeamRows;
      team[k] = (int)std::max<long long>(2, want > avail ? d * avail / std::max<long long>(want, 1) : d);
      have += team[k];
    }
    if (have <= avail || large.empty()) {
      *nsmall = (int)small.size();
      std::sort(small.begin(), small.end(), [&](int a, int b) { return sys[a].natoms > sys[b].natoms; });
      c->h_qsmall.assign(small.begin(), small.end());
      c->h_qmap.clear();
      for (size_t k = 0; k < large.size(); ++k) {
        const int first = (int)c->h_qmap.size();
        for (int r = 0; r < team[k]; ++r) c->h_qmap.push_back(make_int4(large[k], r, team[k], first));
      }
      *nteam = (int)c->h_qmap.size();
      *nblocks = *nteam + small_blocks;
      return;
    }
    small.push_back(large.back());  // the smallest large system is solved by one block
    large.pop_back();
    team.pop_back();
  }
}

// Cluster plan: every system above kQeqSmall atoms is solved by one thread-block cluster
// (4 blocks in a batch, 8 for a single system; rows split over them, reductions in distributed
// shared memory), the others
// by single blocks. Taken when no system is too large for a cluster to be the better choice: above
// kQeqClusterMax atoms a single-system call spreads the rows over a grid-wide team instead, and
// above kQeqBatchBlock atoms a batch does. h_qsmall receives the cluster systems, then the others,
// each largest first.
constexpr int kQeqClusterMax = 640;

bool plan_qeq_cluster(xr_ctx* c, const xr_system* sys, int nsys, int* csize, int* nblocks, int* nbig, int* nsmall) {
  *csize = nsys > 1 ? kQeqClusterBatch : kQeqClusterSingle;
  if ((nsys > 1 ? c->max_clusters_batch : c->max_clusters) < 1) return false;
  const int cs = *csize;
  const int limit = nsys > 1 ? kQeqBatchBlock : kQeqClusterMax;
  std::vector<int> big, small;
  for (int s = 0; s < nsys; ++s) {
    if (sys[s].natoms > limit) return false;
    (sys[s].natoms > kQeqSmall ? big : small).push_back(s);
  }
  auto larger = [&](int a, int b) { return sys[a].natoms > sys[b].natoms; };
  std::sort(big.begin(), big.end(), larger);
  std::sort(small.begin(), small.end(), larger);
  const int clusters = std::max(1, std::min(c->nsm / cs, (int)big.size() + ((int)small.size() + cs - 1) / cs));
  *nblocks = clusters * cs;
  *nbig = (int)big.size();
  *nsmall = (int)small.size();
  c->h_qsmall.assign(big.begin(), big.end());
  c->h_qsmall.insert(c->h_qsmall.end(), small.begin(), small.end());
  return true;
}

// Whether the kept skin list serves this call: the same systems (atom counts, types, pbc, cells) at
// the same cutoff and skin, and no atom further than `skin` from its position at the build (the rule
// of ASE's PrimitiveNeighborList.update: a rebuild once any atom moved more than the skin).
bool skin_list_valid(const xr_ctx* c, int nsys, int A, double rc) {
  if (!c->cache_valid || c->cache_rc != rc || c->cache_skin != c->skin || (int)c->cache_types.size() != A ||
      (int)c->cache_shape.size() != 4 * nsys)
    return false;
  for (int s = 0; s < nsys; ++s) {
    const XrSystem& S = c->host_sys[s];
    const int* sh = c->cache_shape.data() + 4 * s;
    if (sh[0] != S.natoms || sh[1] != S.periodic[0] || sh[2] != S.periodic[1] || sh[3] != S.periodic[2]) return false;
    if (std::memcmp(c->cache_cell.data() + 9 * s, S.cell, 9 * sizeof(double)) != 0) return false;
  }
  if (std::memcmp(c->cache_types.data(), c->h_types, sizeof(int) * (size_t)A) != 0) return false;
  const double lim = c->skin * c->skin;
  for (int a = 0; a < A; ++a) {
    const double dx = c->h_x[a].x - c->cache_x0[3 * a], dy = c->h_x[a].y - c->cache_x0[3 * a + 1],
                 dz = c->h_x[a].z - c->cache_x0[3 * a + 2];
    if (dx * dx + dy * dy + dz * dz > lim) return false;
  }
  return true;
}

void keep_skin_list(xr_ctx* c, int nsys, int A, double rc) {
  c->cache_rc = rc;
  c->cache_skin = c->skin;
  c->cache_types.assign(c->h_types, c->h_types + A);
  c->cache_x0.resize(3 * (size_t)A);
  for (int a = 0; a < A; ++a) {
    c->cache_x0[3 * a] = c->h_x[a].x;
    c->cache_x0[3 * a + 1] = c->h_x[a].y;
    c->cache_x0[3 * a + 2] = c->h_x[a].z;
  }
  c->cache_shape.resize(4 * (size_t)nsys);
  c->cache_cell.resize(9 * (size_t)nsys);
  for (int s = 0; s < nsys; ++s) {
    const XrSystem& S = c->host_sys[s];
    int* sh = c->cache_shape.data() + 4 * s;
    sh[0] = S.natoms;
    sh[1] = S.periodic[0];
    sh[2] = S.periodic[1];
    sh[3] = S.periodic[2];
    std::memcpy(c->cache_cell.data() + 9 * s, S.cell, 9 * sizeof(double));
  }
  c->cache_valid = true;
}

enum ListMode { kScan = 0, kBuild = 1, kReuse = 2, kSupplied = 3, kCell = 4 };

// Cell-list choice of a call whose list comes from a search (an image scan, or a skin-list build at
// rl): per system, the grid of cell_grid stored in both descriptor sets; used when the searches'
// expected image tests fall below half of the image scan's (or when the context forces it).
// Systems smaller than kCellMinAtoms cost little either way. Returns the batch's number of cells
// (0: no cell list).
constexpr int kCellMinAtoms = 1024;

long long plan_cells(xr_ctx* c, int nsys, const xr_system* sys, double rl, XrSystem* list_desc) {
  if (c->cell_mode < 0) return 0;
  double scan = 0.0, cells = 0.0;
  long long total = 0;
  int largest = 0;
  for (int s = 0, o = 0; s < nsys; o += sys[s].natoms, ++s) {
    XrSystem& S = list_desc ? list_desc[s] : c->host_sys[s];
    const int n = sys[s].natoms;
    largest = std::max(largest, n);
    double visits = 1.0;
    const long long nc = xr_host::cell_grid(S, c->h_x + o, n, rl, std::max<long long>(64, 2ll * n), &visits);
    S.cell_base = (int)total;
    total += nc;
    double images = 1.0;
    for (int k = 0; k < 3; ++k) images *= 2.0 * S.reach[k] + 1.0;
    scan += (double)n * n * images;
    cells += (double)n * n * images * visits + 64.0 * n;  // plus the row sort
    if (total > (1ll << 30)) return 0;
  }
  const bool use = c->cell_mode > 0 || (largest >= kCellMinAtoms && cells < 0.5 * scan);
  for (int s = 0; s < nsys; ++s) {
    XrSystem& S = list_desc ? list_desc[s] : c->host_sys[s];
    if (!use) S.cell_n[0] = S.cell_n[1] = S.cell_n[2] = 0;
    if (list_desc) {  // k_prep bins with the main descriptors: the same grid in both sets
      XrSystem& M = c->host_sys[s];
      for (int k = 0; k < 3; ++k) {
        M.cell_n[k] = S.cell_n[k];
        M.cell_reach[k] = S.cell_reach[k];
        M.cell_f0[k] = S.cell_f0[k];
        M.cell_scale[k] = S.cell_scale[k];
      }
      M.cell_base = S.cell_base;
    }
  }
  return use ? total : 0;
}

// Everything the launch sequence after the list count depends on, other than data in device memory:
// the work descriptor (pointers, capacities, atom and system counts; the list sizes are read from
// the device), the force field's view, and the host-side launch choices.
std::vector<unsigned char> launch_key(const XrWork& w, const XrFF& ff, const int* ints, int nints, const void* const* ptrs,
                                      int nptrs) {
  XrWork wk = w;  // padding is zero: fill_work clears the whole structure
  wk.nE = wk.nP = wk.nB = wk.nD = 0;
  std::vector<unsigned char> k(sizeof(XrWork) + sizeof(XrFF) + sizeof(int) * nints + sizeof(void*) * nptrs);
  unsigned char* q = k.data();
  std::memcpy(q, &wk, sizeof(XrWork));
  std::memcpy(q + sizeof(XrWork), &ff, sizeof(XrFF));
  std::memcpy(q + sizeof(XrWork) + sizeof(XrFF), ints, sizeof(int) * nints);
  std::memcpy(q + sizeof(XrWork) + sizeof(XrFF) + sizeof(int) * nints, ptrs, sizeof(void*) * nptrs);
  return k;
}

int run_batch(xr_ctx* c, const xr_ff* ff, int nsys, const xr_system* sys, unsigned flags, xr_result* out,
              const xr_neighbors* nb = nullptr, const int* sets = nullptr) {
  if (!c || !ff || nsys < 1 || !sys) {
    if (c) c->err = "invalid arguments";
    return XR_EINPUT;
  }
  if (sets)
    for (int s = 0; s < nsys; ++s)
      if (sets[s] < 0 || sets[s] >= ff->nsets) {
        c->err = "parameter set index out of range";
        return XR_EINPUT;
      }
  if (nb && nsys != 1) {
    c->err = "a supplied neighbour list belongs to a single-system call";
    return XR_EINPUT;
  }
  const bool dev_io = (flags & XR_FLAG_DEVICE_IO) != 0;
  if (dev_io && nsys != 1) {
    c->err = "device input/output is supported for single-system calls";
    return XR_EINPUT;
  }
  cudaSetDevice(c->device);
  const double rc = ff->d.g[12];
  long long A64 = 0;
  for (int s = 0; s < nsys; ++s) {
    if (sys[s].natoms < 1 || !sys[s].types || !sys[s].positions) {
      c->err = "A nonempty sequence of parameter-file atom labels is required";
      return XR_EINPUT;
    }
    A64 += sys[s].natoms;
  }
  if (A64 > (1ll << 26)) {
    c->err = "batch too large";
    return XR_EINPUT;
  }
  const int A = (int)A64;
  if (!ensure_atoms(c, A, nsys) || !host_grow(&c->h_x, &c->ch_x, (size_t)A))
    return cuda_fail(c, cudaErrorMemoryAllocation, "allocation");
  c->host_sys.resize(nsys);
  if (!host_grow(&c->h_types, &c->ch_types, (size_t)A) || !host_grow(&c->h_sysof, &c->ch_sysof, (size_t)A) ||
      !host_grow(&c->h_sysd, &c->ch_sysd, (size_t)nsys))
    return cuda_fail(c, cudaErrorMemoryAllocation, "allocation");
  int* types = c->h_types;
  int* sys_of = c->h_sysof;
  bool any_guess = false;
  int off = 0;
  for (int s = 0; s < nsys; ++s) {
    const xr_system& in = sys[s];
    if (dev_io) {
      // positions live on the device: descriptor from a host-side copy of the cell only
      std::vector<double> hp(3 * (size_t)in.natoms);
      cudaMemcpy(hp.data(), in.positions, hp.size() * sizeof(double), cudaMemcpyDeviceToHost);
      xr_system tmp = in;
      tmp.positions = hp.data();
      int rcode = build_system(c, tmp, off, rc, c->host_sys[s], c->h_x + off);
      if (rcode) return rcode;
    } else {
      int rcode = build_system(c, in, off, rc, c->host_sys[s], c->h_x + off);
      if (rcode) return rcode;
    }
    c->host_sys[s].ff_set = sets ? sets[s] : 0;
    for (int a = 0; a < in.natoms; ++a) {
      const int t = in.types[a];
      if (t < 0 || t >= ff->d.ntypes) {
        c->err = "Atom types absent from the force field";
        return XR_EINPUT;
      }
      types[off + a] = t;
      sys_of[off + a] = s;
      if (!dev_io) {
        const unsigned long long bits = (unsigned long long)(unsigned)t | ((unsigned long long)(unsigned)s << 32);
        std::memcpy(&c->h_x[off + a].w, &bits, sizeof(bits));
      }
    }
    if (in.charges_guess) {
      // starting charges of the QEq solve (a warm start), shifted onto sum q = total_charge
      if (!host_grow(&c->h_guess, &c->ch_guess, (size_t)A)) return cuda_fail(c, cudaErrorMemoryAllocation, "allocation");
      double* hg = c->h_guess + off;
      if (dev_io) {
        cudaMemcpy(hg, in.charges_guess, sizeof(double) * in.natoms, cudaMemcpyDeviceToHost);
      } else {
        std::memcpy(hg, in.charges_guess, sizeof(double) * in.natoms);
      }
      double sum = 0;
      for (int a = 0; a < in.natoms; ++a) {
        if (!std::isfinite(hg[a])) {
          c->err = "initial charges must be finite";
          return XR_EINPUT;
        }
        sum += hg[a];
      }
      const double shift = (in.total_charge - sum) / in.natoms;
      for (int a = 0; a < in.natoms; ++a) hg[a] += shift;
      c->host_sys[s].has_guess = 1;
      any_guess = true;
    }
    off += in.natoms;
  }
  // Where the rows come from: the all-pairs image scan, a skin list (built now, or kept from an
  // earlier call), or the caller's list.
  ListMode mode = kScan;
  if (nb) {
    std::vector<int> start;
    std::vector<int2> rows;
    int maxs[3];
    std::string msg;
    const int code = xr_host::canonical_list(sys[0].natoms, sys[0].pbc, *nb, start, rows, maxs, msg);
    if (code != XR_OK) {
      c->err = msg;
      return code;
    }
    if (!grow(c, &c->cand_cnt, &c->ccand_cnt, (size_t)A + 1) || !grow(c, &c->cand_edge, &c->ccand_edge, std::max<size_t>(rows.size(), 1)) ||
        !host_grow(&c->h_cand_cnt, &c->ch_cand_cnt, (size_t)A + 1) ||
        !host_grow(&c->h_cand_edge, &c->ch_cand_edge, std::max<size_t>(rows.size(), 1)))
      return cuda_fail(c, cudaErrorMemoryAllocation, "allocation");
    std::memcpy(c->h_cand_cnt, start.data(), sizeof(int) * ((size_t)A + 1));
    if (!rows.empty()) std::memcpy(c->h_cand_edge, rows.data(), sizeof(int2) * rows.size());
    c->cache_valid = false;  // the candidate arrays now hold the caller's list
    mode = kSupplied;
  } else if (c->skin > 0.0) {
    mode = skin_list_valid(c, nsys, A, rc) ? kReuse : kBuild;
    if (mode == kBuild) {
      if (!host_grow(&c->h_sys_list, &c->ch_sys_list, (size_t)nsys) || !grow(c, &c->sys_list, &c->csys_list, (size_t)nsys) ||
          !grow(c, &c->cand_cnt, &c->ccand_cnt, (size_t)A + 1))
        return cuda_fail(c, cudaErrorMemoryAllocation, "allocation");
      const double rl = rc + 2.0 * c->skin;
      for (int s = 0, o = 0; s < nsys; o += sys[s].natoms, ++s) {
        const char* msg = "";
        xr_system in = sys[s];
        in.positions = nullptr;  // positions come from the packed copy below
        XrSystem& L = c->h_sys_list[s];
        // the list cutoff's descriptor: the same cell and wrap, the list cutoff's reach and band
        std::vector<double> px(3 * (size_t)in.natoms);
        for (int a = 0; a < in.natoms; ++a) {
          px[3 * a] = c->h_x[o + a].x;
          px[3 * a + 1] = c->h_x[o + a].y;
          px[3 * a + 2] = c->h_x[o + a].z;
        }
        in.positions = px.data();
        const int code = xr_host::describe_system(in, o, rl, L, nullptr, &msg);
        if (code != XR_OK) {
          c->err = msg;
          return code;
        }
      }
      c->cache_valid = false;  // rebuilt below
    }
  }
  long long ncells = 0;
  if (mode == kScan || mode == kBuild) {
    ncells = plan_cells(c, nsys, sys, mode == kBuild ? rc + 2.0 * c->skin : rc, mode == kBuild ? c->h_sys_list : nullptr);
    if (ncells > 0) {
      if (!grow(c, &c->atom_cell, &c->catom_cell, (size_t)A) || !grow(c, &c->atom_slot, &c->catom_slot, (size_t)A) ||
          !grow(c, &c->cell_atoms, &c->ccell_atoms, (size_t)A) || !grow(c, &c->cell_cnt, &c->ccell_cnt, (size_t)ncells + 1) ||
          !grow(c, &c->cand_cnt, &c->ccand_cnt, (size_t)A + 1))
        return cuda_fail(c, cudaErrorMemoryAllocation, "allocation");
      if (mode == kScan) mode = kCell;
    }
  }
  // energy-reduction chunks: each system's atoms in runs of XR_CHUNK_ATOMS, numbered in system order
  size_t nchunk = 0;
  for (int s = 0; s < nsys; ++s) {
    c->host_sys[s].chunk0 = (int)nchunk;
    nchunk += (size_t)(sys[s].natoms + XR_CHUNK_ATOMS - 1) / XR_CHUNK_ATOMS;
  }
  if (!grow(c, &c->chunk_part, &c->cchunk_part, nchunk * (size_t)XR_PART_N))
    return cuda_fail(c, cudaErrorMemoryAllocation, "allocation");
  std::memcpy(c->h_sysd, c->host_sys.data(), sizeof(XrSystem) * nsys);
  cudaStream_t st = c->stream;
  long long launches = 0;
  long long h2d = 0, d2h = 0;
  cudaError_t e;
  if (dev_io) {
    k_positions_from_device<<<(A + 255) / 256, 256, 0, st>>>(sys[0].positions, c->x, A);
    ++launches;
  } else {
    cudaMemcpyAsync(c->x, c->h_x, sizeof(double4_32a) * A, cudaMemcpyHostToDevice, st);
    h2d += sizeof(double4_32a) * (long long)A;
  }
  if (any_guess) {
    cudaMemcpyAsync(c->qguess, c->h_guess, sizeof(double) * A, cudaMemcpyHostToDevice, st);
    h2d += sizeof(double) * (long long)A;
  }
  if (dev_io) {  // else types and systems travel in the positions' fourth words, unpacked by k_prep
    cudaMemcpyAsync(c->type, types, sizeof(int) * A, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(c->sys_of, sys_of, sizeof(int) * A, cudaMemcpyHostToDevice, st);
    h2d += 2 * sizeof(int) * (long long)A;
  }
  cudaMemcpyAsync(c->sys, c->h_sysd, sizeof(XrSystem) * nsys, cudaMemcpyHostToDevice, st);
  h2d += sizeof(XrSystem) * (long long)nsys;
  // (counts, QEq iterations, scans, torsion-middle and exported-bond counters: zeroed by k_prep)
  cudaMemsetAsync(c->status, 0, sizeof(int), st);
  XrWork w;
  fill_work(c, w, A, nsys, flags);
  w.types_in_x = dev_io ? 0 : 1;
  w.prep_zero = 1;
  w.nchunks = (int)nchunk;
  c->pgrad_pairs = c->pgrad_angles = 0;
  if (flags & XR_FLAG_PARAM_GRADIENT) {
    // one gradient block per system: [pair table][angle records][atom table]
    const long long np = (long long)ff->d.ntypes * ff->d.ntypes * XR_NPAIR_COLS, na = 7ll * ff->nangle;
    const long long nat = (long long)ff->d.ntypes * XR_NATOM_COLS;
    const size_t all = (size_t)(np + na + nat) * nsys;
    if (!grow(c, &c->pgrad, &c->cpgrad, all + 1)) return cuda_fail(c, cudaErrorMemoryAllocation, "allocation");
    cudaMemsetAsync(c->pgrad, 0, sizeof(double) * all, st);
    w.pgrad = c->pgrad;
    w.pgrad_angle_off = (int)np;
    w.pgrad_atom_off = (int)(np + na);
    w.pgrad_stride = np + na + nat;
    c->pgrad_pairs = np;
    c->pgrad_angles = na;
    c->pgrad_atoms = nat;
    c->pgrad_systems = nsys;
  }
  attach_lists(c, w);
  if (ncells > 0) {
    w.atom_cell = c->atom_cell;
    w.atom_slot = c->atom_slot;
    w.cell_cnt = c->cell_cnt;
    w.cell_atoms = c->cell_atoms;
    w.ncells = (int)ncells;
  }
  stage(c, 0, st);
  xr_launch_prep(w, st);  // also assigns every atom its cell when the call uses the cell list
  launches += 1;
  if (mode == kScan || mode == kSupplied) {
    // the image scan; for a supplied list only its coincident-atom check counts (xreac checks every
    // pair's minimum image whatever list it is given), and the filter's counts replace its own
    xr_launch_count(w, st);
    launches += 1;
  }
  if (mode == kSupplied) {
    cudaMemcpyAsync(c->cand_cnt, c->h_cand_cnt, sizeof(int) * ((size_t)A + 1), cudaMemcpyHostToDevice, st);
    const long long m = c->h_cand_cnt[A];
    if (m > 0) cudaMemcpyAsync(c->cand_edge, c->h_cand_edge, sizeof(int2) * (size_t)m, cudaMemcpyHostToDevice, st);
    h2d += sizeof(int) * ((long long)A + 1) + sizeof(int2) * m;
  }
  if (mode == kBuild || mode == kCell) {
    // every image within the list cutoff (rc + 2 skin for a skin list, with its descriptors; rc for
    // a cell-list search), from the cell list or the image scan
    XrWork wl = w;
    if (mode == kBuild) {
      cudaMemcpyAsync(c->sys_list, c->h_sys_list, sizeof(XrSystem) * nsys, cudaMemcpyHostToDevice, st);
      h2d += sizeof(XrSystem) * (long long)nsys;
      wl.sys = c->sys_list;
    }
    cudaMemsetAsync(c->cand_cnt, 0, sizeof(int) * ((size_t)A + 1), st);
    wl.cand_cnt = c->cand_cnt;
    if (ncells > 0) {
      xr_launch_cells(wl, st);
      xr_launch_cell_candidates(wl, false, st);
      launches += 8;
    } else {
      xr_launch_candidates(wl, false, st);
      launches += 4;
    }
    cudaMemcpyAsync(c->h_small + 9, c->counts + 5, 2 * sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(c->h_small + 4, c->status, sizeof(int), cudaMemcpyDeviceToHost, st);
    d2h += 3 * sizeof(int);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(c, e, "neighbour list count");
    if (int code = status_to_code(c, c->h_small[4])) return code;
    const int m = c->h_small[9], longest = c->h_small[10];
    if (!grow(c, &c->cand_edge, &c->ccand_edge, std::max<size_t>((size_t)m, 1)))
      return cuda_fail(c, cudaErrorMemoryAllocation, "list allocation");
    wl.cand_edge = w.cand_edge = c->cand_edge;
    if (ncells > 0 && longest <= XR_ROW_SORT_MAX) {
      xr_launch_cell_candidates(wl, true, st);
      xr_launch_row_sort(wl, longest, st);
      launches += 2;
    } else {
      // the image scan finds the same candidates (its rows come out in canonical order): used where
      // a row is too long for the shared-memory sort
      xr_launch_candidates(wl, true, st);
      launches += 1;
    }
    if (mode == kBuild) ++c->list_builds;
  }
  if (mode != kScan) {
    w.cand_cnt = c->cand_cnt;
    w.cand_edge = c->cand_edge;
    xr_launch_filter(w, false, st);
    launches += 1;
  }
  xr_launch_scan(w, st);
  launches += 3;
  cudaMemcpyAsync(c->h_small, c->counts, 4 * sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(c->h_small + 4, c->status, sizeof(int), cudaMemcpyDeviceToHost, st);
  d2h += 5 * sizeof(int);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(c, e, "neighbour count");
  const int nE = c->h_small[0], nP = c->h_small[1], nB = c->h_small[2], nD = c->h_small[3];
  if (int code = status_to_code(c, c->h_small[4])) return code;
  if (mode == kBuild) keep_skin_list(c, nsys, A, rc);
  c->list_mode = mode == kBuild && ncells > 0 ? 5 : (int)mode;
  if (!ensure_lists(c, nE, nP, nB)) return cuda_fail(c, cudaErrorMemoryAllocation, "list allocation");
  attach_lists(c, w);
  w.nE = nE;
  w.nP = nP;
  w.nB = nB;
  w.nD = nD;
  // Host-side choices of the launch sequence, made before it so that it can be recorded: the QEq
  // plan (its tables go through pinned buffers that a replay copies again) and the bond export.
  int qblocks = 0, qteam = 0, qsmall = 0, qbig = 0, qcsize = 0, nlist = 0;
  bool qcluster = false;
  if (c->coop_per_sm > 0) {
    qcluster = plan_qeq_cluster(c, sys, nsys, &qcsize, &qblocks, &qbig, &qsmall);
    if (!qcluster) plan_qeq(c, sys, nsys, &qblocks, &qteam, &qsmall);
    nlist = qbig + qsmall;
    if (!host_grow(&c->h_qmap_p, &c->ch_qmap_p, (size_t)std::max(qteam, 1)) ||
        !host_grow(&c->h_qsmall_p, &c->ch_qsmall_p, (size_t)std::max(nlist, 1)))
      return cuda_fail(c, cudaErrorMemoryAllocation, "allocation");
    if (qteam > 0) std::memcpy(c->h_qmap_p, c->h_qmap.data(), sizeof(int4) * qteam);
    if (nlist > 0) std::memcpy(c->h_qsmall_p, c->h_qsmall.data(), sizeof(int) * nlist);
    h2d += sizeof(int4) * (long long)qteam + sizeof(int) * (long long)nlist;
  }
  const ResultLayout RL = result_layout(A, nsys, nB);
  if (!grow(c, &c->outbuf, &c->coutbuf, RL.end) || !host_grow(&c->h_out, &c->ch_out, RL.end))
    return cuda_fail(c, cudaErrorMemoryAllocation, "result block");
  XrBondRecord* const bx_rec = reinterpret_cast<XrBondRecord*>(c->outbuf + RL.bonds);
  auto launch_qeq = [&](bool adjoint) {
    return qcluster ? xr_launch_qeq_cluster(w, ff->d, st, qcsize, qblocks, c->qsmall, qbig, qsmall, adjoint)
                    : xr_launch_qeq(w, ff->d, st, qblocks, c->qmap, qteam, c->qsmall, qsmall, adjoint);
  };
  // The launch sequence: rows, pairs, QEq, bond orders, bonded terms, Coulomb energy and forces,
  // reductions, bond export. Returns 0 or a CUDA error of a launch.
  auto sequence = [&]() -> int {
    stage(c, 1, st);
    if (mode == kScan)
      xr_launch_rows(w, st);
    else
      xr_launch_filter(w, true, st);
    xr_launch_reverse(w, st);
    launches += 2;
    cudaMemsetAsync(c->a_adj, 0, sizeof(double) * (size_t)AJ_N * A, st);
    cudaMemsetAsync(c->f, 0, sizeof(double) * 3 * (size_t)A, st);
    cudaMemsetAsync(c->b_adj, 0, sizeof(double) * (size_t)BJ_N * c->capB, st);
    cudaMemsetAsync(c->b_e, 0, sizeof(double) * 4 * c->capB, st);
    stage(c, 2, st);
    xr_launch_pairs(w, ff->d, st);
    launches += 2;
    stage(c, 3, st);
    if (qteam > 0) cudaMemcpyAsync(c->qmap, c->h_qmap_p, sizeof(int4) * qteam, cudaMemcpyHostToDevice, st);
    if (nlist > 0) cudaMemcpyAsync(c->qsmall, c->h_qsmall_p, sizeof(int) * nlist, cudaMemcpyHostToDevice, st);
    if (int le = launch_qeq(false)) return le;
    launches += (qcluster ? qbig > 0 : qteam > 0) ? 2 : 1;  // the teams' row splits, then the solver
    stage(c, 4, st);
    const bool qeq_grad = w.pgrad && (flags & XR_FLAG_QEQ_GRADIENT);
    if (w.full_derivative || qeq_grad) {
      // the adjoint QEq solve with the same plan: charge-response forces (its radial pair terms)
      // and the QEq parameters' gradient
      xr_launch_charge_response(w, ff->d, st, 0);
      if (int le = launch_qeq(true)) return le;
      launches += (qcluster ? qbig > 0 : qteam > 0) ? 4 : 3;
      if (w.full_derivative) {
        xr_launch_charge_response(w, ff->d, st, 1);
        launches += 1;
      }
      if (qeq_grad) {
        xr_launch_qeq_param_gradient(w, ff->d, st);
        launches += 1;
      }
    }
    stage(c, 5, st);
    xr_launch_bond_orders(w, ff->d, st);
    launches += 3;
    stage(c, 6, st);
    xr_launch_bonded(w, ff->d, st);
    launches += 13;
    stage(c, 7, st);
    xr_launch_forces(w, ff->d, st);
    launches += 1;
    xr_launch_reduce(w, ff->d, st);
    launches += 2;
    if (nB > 0) {  // (its counter was zeroed by k_prep)
      k_bond_export<<<(nB + 255) / 256, 256, 0, st>>>(w, bx_rec, c->bx_count);
      ++launches;
    }
    return (int)cudaGetLastError();
  };
  // A sequence is recorded as a CUDA graph the second time its launch key occurs (a relaxation or MD
  // step, a repeated request, a request size seen before) and replayed on later occurrences: one
  // launch instead of about 30 kernel launches and their memsets. The key holds every pointer and
  // size the recorded launches use, so a cached graph matches only calls whose buffers it addresses.
  // Not with stage timing, nor with grid-wide QEq teams (their co-residency needs a cooperative launch).
  c->last_graph = 0;
  bool done = false;
  if (c->graphs && !c->profile && qteam == 0) {
    const int ints[] = {(int)mode, qcluster ? 1 : 0, qcsize, qblocks, qteam, qsmall, qbig, nlist, nE > 0, nP > 0, nB > 0,
                        (int)flags};
    const void* ptrs[] = {c->h_qmap_p, c->h_qsmall_p, c->qmap, c->qsmall, bx_rec, c->bx_count, c->outbuf};
    const int nptrs = (int)(sizeof(ptrs) / sizeof(ptrs[0]));
    const std::vector<unsigned char> kv = launch_key(w, ff->d, ints, (int)(sizeof(ints) / sizeof(int)), ptrs, nptrs);
    const std::string key(reinterpret_cast<const char*>(kv.data()), kv.size());
    auto hit = c->gcache.find(key);
    if (hit != c->gcache.end()) {
      if (cudaGraphLaunch(hit->second.exec, st) == cudaSuccess) {
        launches += hit->second.launches;
        hit->second.used = ++c->gclock;
        c->last_graph = 2;
        done = true;
      } else {
        cudaGetLastError();
      }
    } else {
      int& seen = c->gseen[key];
      if (seen >= 0 && ++seen >= 2) {
        const long long before = launches;
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ex = nullptr;
        if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
          const int rc = sequence();
          const cudaError_t ce = cudaStreamEndCapture(st, &g);
          if (rc != 0 || ce != cudaSuccess || !g || cudaGraphInstantiate(&ex, g, 0) != cudaSuccess) ex = nullptr;
          if (g) cudaGraphDestroy(g);
        }
        if (ex && cudaGraphLaunch(ex, st) == cudaSuccess) {
          if (c->gcache.size() >= xr_ctx::kGraphCache) {  // evict the least recently used
            auto lru = c->gcache.begin();
            for (auto it = c->gcache.begin(); it != c->gcache.end(); ++it)
              if (it->second.used < lru->second.used) lru = it;
            cudaGraphExecDestroy(lru->second.exec);
            c->gcache.erase(lru);
          }
          c->gcache.emplace(key, xr_ctx::GraphEntry{ex, launches - before, ++c->gclock});
          c->gseen.erase(key);
          c->last_graph = 1;
          done = true;
        } else {  // not recordable here: launch directly, and do not try this key again
          if (ex) cudaGraphExecDestroy(ex);
          cudaGetLastError();
          launches = before;
          seen = -1;
        }
      }
      if (c->gseen.size() > xr_ctx::kGraphSeen) c->gseen.clear();
    }
  }
  if (!done)
    if (int le = sequence()) return cuda_fail(c, (cudaError_t)le, "launch");
  // Results: the per-atom values (k_pack, or the caller's device arrays), then energies, properties,
  // counters, QEq iterations and scans (k_gather_tail) into the result block, where k_bond_export has
  // written the exported bonds (at most nB records); one copy brings the block back, and the call
  // synchronises once more only at its end. The parameter gradient, when asked for, comes separately.
  if (dev_io) {
    const xr_result& r = out[0];
    k_unpack_device<<<(A + 255) / 256, 256, 0, st>>>(w, r.forces, r.charges, r.total_bond_orders, r.lone_pairs,
                                                    r.bond_counts);
  } else {
    k_pack<<<(A + 255) / 256, 256, 0, st>>>(w, c->outbuf);
  }
  {
    const long long tail_n = 20ll * nsys + 4ll * (A + 1) + nsys;
    const int gb = (int)std::min<long long>((tail_n + 255) / 256, 152 * 4);
    k_gather_tail<<<gb, 256, 0, st>>>(w, c->outbuf, RL.energy, RL.tail);
  }
  launches += 2;
  {
    const size_t from = dev_io ? RL.energy : 0;
    const size_t count = RL.bonds + 4 * (size_t)std::max(nB, 0) - from;
    cudaMemcpyAsync(c->h_out + from, c->outbuf + from, sizeof(double) * count, cudaMemcpyDeviceToHost, st);
    d2h += (long long)(sizeof(double) * count);
  }
  if (c->pgrad_pairs > 0) {
    const size_t all = (size_t)(c->pgrad_pairs + c->pgrad_angles + c->pgrad_atoms) * nsys;
    if (!host_grow(&c->h_pg, &c->ch_pg, all)) return cuda_fail(c, cudaErrorMemoryAllocation, "allocation");
    cudaMemcpyAsync(c->h_pg, c->pgrad, sizeof(double) * all, cudaMemcpyDeviceToHost, st);
    d2h += (long long)(sizeof(double) * all);
  }
  stage(c, 8, st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(c, e, "evaluation");
  if (c->profile) {
    for (int k = 0; k < 8; ++k) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, c->ev[k], c->ev[k + 1]) == cudaSuccess) c->stage_ms[k] += ms;
    }
    ++c->stage_calls;
  }
  const int* tail = reinterpret_cast<const int*>(c->h_out + RL.tail);
  const XrBondRecord* recs = reinterpret_cast<const XrBondRecord*>(c->h_out + RL.bonds);
  {
    const int nx = std::min(tail[1], std::max(nB, 0));
    d2h += (sizeof(int4) + sizeof(double)) * (long long)nB;
    // exported in arrival order; sorted by bond id (system, then pair order) for the exporters
    std::vector<int> order(nx);
    for (int k = 0; k < nx; ++k) order[k] = k;
    std::sort(order.begin(), order.end(), [&](int a, int b) { return recs[a].meta.x < recs[b].meta.x; });
    c->h_bx_meta.resize(nx);
    c->h_bx_bo.resize(nx);
    for (int k = 0; k < nx; ++k) {
      c->h_bx_meta[k] = recs[order[k]].meta;
      c->h_bx_bo[k] = recs[order[k]].bo;
    }
  }
  c->h_qiters.assign(tail + kTailInts, tail + kTailInts + nsys);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(c, e, "kernel launch");
  c->launches = launches;
  c->qeq_iterations = tail[2];
  c->list_sizes[0] = nE;
  c->list_sizes[1] = nP;
  c->list_sizes[2] = nB;
  c->list_sizes[3] = nD;
  c->list_sizes[4] = tail[4];  // active bonds (uncorrected order passed the cut)
  c->list_sizes[5] = tail[3];  // torsion middles (bo > 0.001)
  if (c->pgrad_pairs > 0)
    c->h_pgrad.assign(c->h_pg, c->h_pg + (c->pgrad_pairs + c->pgrad_angles + c->pgrad_atoms) * nsys);
  c->last_A = A;
  // keep the scans for export
  c->host_cnt.assign(tail + kTailInts + nsys, tail + kTailInts + nsys + 4 * (size_t)(A + 1));
  c->h2d_bytes = h2d;
  c->d2h_bytes = d2h;
  if (int code = status_to_code(c, tail[0])) return code;
  if (dev_io) {
    const xr_result& r = out[0];
    if (r.energy)
      for (int k = 0; k < 15; ++k) r.energy[k] = c->h_out[RL.energy + k];
    if (r.dipole)
      for (int k = 0; k < 3; ++k) r.dipole[k] = c->h_out[RL.props + k];
    return XR_OK;
  }
  off = 0;
  for (int s = 0; s < nsys; ++s) {
    const xr_result& r = out[s];
    const int n = sys[s].natoms;
    const double* pa = c->h_out + 8 * (size_t)off;
    const double* pe = c->h_out + RL.energy + 16 * s;
    const double* pp = c->h_out + RL.props + 4 * s;
    if (r.energy)
      for (int k = 0; k < 15; ++k) r.energy[k] = pe[k];
    if (r.dipole)
      for (int k = 0; k < 3; ++k) r.dipole[k] = pp[k];
    for (int a = 0; a < n; ++a) {
      const double* v = pa + 8 * a;
      if (r.forces) {
        r.forces[3 * a + 0] = v[0];
        r.forces[3 * a + 1] = v[1];
        r.forces[3 * a + 2] = v[2];
      }
      if (r.charges) r.charges[a] = v[3];
      if (r.total_bond_orders) r.total_bond_orders[a] = v[4];
      if (r.lone_pairs) r.lone_pairs[a] = v[5];
      if (r.bond_counts) r.bond_counts[a] = (int)v[6];
    }
    // the charge constraint check of src/xreac/calculator.py:153-154
    if (r.charges) {
      double sq = 0;
      for (int a = 0; a < n; ++a) sq += r.charges[a];
      if (std::fabs(sq - sys[s].total_charge) > 1e-8) {
        c->err = "QEq charge constraint failed";
        return XR_ECHARGE;
      }
    }
    off += n;
  }
  return XR_OK;
}

// Derived per-set tables of one parameter set (host): the vdW shielding term, log radii, bond-order
// distance bound and reciprocal radii per pair type, and the hydrogen-bond role per element.
void ff_derive(int T, const double* general, const double* atom, const double* pair, double* gw, double* logr,
               double* rmax, double* pinv, int* hb_role) {
  for (int pt = 0; pt < T * T; ++pt) {
    const double* p = pair + pt * XR_NPAIR_COLS;
    gw[pt] = std::pow(1.0 / p[P_GAMMA_W], general[28]);
    logr[3 * pt + 0] = p[P_RS] > 0 ? std::log(p[P_RS]) : 0.0;
    logr[3 * pt + 1] = p[P_RP] > 0 ? std::log(p[P_RP]) : 0.0;
    logr[3 * pt + 2] = p[P_RPP] > 0 ? std::log(p[P_RPP]) : 0.0;
    pinv[2 * pt] = 1.0 / p[P_RVDW];
    pinv[2 * pt + 1] = 1.0 / p[P_RCORE];
  }
  // Per pair type, a distance beyond which the uncorrected bond order sigma' + pi' + pi-pi' stays
  // below a quarter of the cut (k_bo1 skips the terms there: the bond is inactive either way). Each
  // used term c exp(p_odd (r / r0)^p_even) decreases with r when p_odd < 0 < p_even, and stays below
  // target / n (n used terms) for r > r0 (ln(target / (n c)) / p_odd)^(1 / p_even); the largest of
  // these bounds the sum. Otherwise no bound is used (infinity) and every candidate is evaluated.
  const double cut = 0.01 * general[29];
  for (int pt = 0; pt < T * T; ++pt) {
    const double* p = pair + pt * XR_NPAIR_COLS;
    const double* ai = atom + (pt / T) * XR_NATOM_COLS;
    const double* aj = atom + (pt % T) * XR_NATOM_COLS;
    const bool use[3] = {ai[A_R_S] > 0 && aj[A_R_S] > 0, ai[A_R_PI] > 0 && aj[A_R_PI] > 0,
                         ai[A_R_PI_PI] > 0 && aj[A_R_PI_PI] > 0};
    const double pa[3] = {p[P_BO1], p[P_BO3], p[P_BO5]}, pb[3] = {p[P_BO2], p[P_BO4], p[P_BO6]};
    const double r0[3] = {p[P_RS], p[P_RP], p[P_RPP]};
    bool monotone = cut > 0;
    int n = 0;
    for (int k = 0; k < 3; ++k) {
      if (!use[k]) continue;
      ++n;
      if (!(pa[k] < 0 && pb[k] > 0 && r0[k] > 0 && std::isfinite(pa[k]) && std::isfinite(pb[k]))) monotone = false;
    }
    double bound = INFINITY;
    if (monotone) {
      const double share = 0.25 * cut / std::max(n, 1);
      bound = 1e-6;
      for (int k = 0; k < 3; ++k) {
        if (!use[k]) continue;
        const double c = k == 0 ? 1.0 + cut : 1.0;
        if (c <= share) continue;  // the term never reaches its share
        const double u = std::log(share / c) / pa[k];  // > 0: (r / r0)^p_even must exceed it
        bound = std::max(bound, r0[k] * std::pow(u, 1.0 / pb[k]) * (1.0 + 1e-12));
      }
      if (!std::isfinite(bound)) bound = INFINITY;
    }
    rmax[pt] = bound;
  }
  for (int t = 0; t < T; ++t) {
    const double ph = atom[t * XR_NATOM_COLS + A_P_HBOND];
    hb_role[t] = ph == 1.0 ? 1 : (ph == 2.0 ? 2 : 0);  // the reference compares p_hbond exactly
  }
}

// Sizes in bytes of the per-set tables and of the shared index tables.
void ff_part_bytes(const xr_ff* f, size_t bytes[FP_N], size_t shared[3]) {
  const size_t T = (size_t)f->d.ntypes, TT = T * T;
  bytes[FP_ATOM] = sizeof(double) * T * XR_NATOM_COLS;
  bytes[FP_PAIR] = sizeof(double) * TT * XR_NPAIR_COLS;
  bytes[FP_GW] = sizeof(double) * TT;
  bytes[FP_LOGR] = sizeof(double) * 3 * TT;
  bytes[FP_RMAX] = sizeof(double) * TT;
  bytes[FP_PINV] = sizeof(double) * 2 * TT;
  bytes[FP_CARBON] = sizeof(int) * T;
  bytes[FP_HBROLE] = sizeof(int) * T;
  bytes[FP_ANGLE] = sizeof(double) * 7 * (size_t)f->nangle;
  bytes[FP_TORSION] = sizeof(double) * 5 * (size_t)f->ntorsion;
  bytes[FP_HBOND] = sizeof(double) * 4 * (size_t)f->nhbond;
  shared[0] = sizeof(int) * 2 * TT * T;
  shared[1] = sizeof(int) * TT * TT;
  shared[2] = sizeof(int) * TT * T;
}

inline size_t round256(size_t n) { return (n + 255) / 256 * 256; }

// Writes one set's block (host, set_bytes long): the given tables, set 0's where a table is null
// (is_carbon always set 0's), and the tables derived from this set's atom and pair values.
void ff_fill_set(const xr_ff* f, const double* general, const double* atom, const double* pair, const int* is_carbon,
                 const double* angle, const double* torsion, const double* hbond, unsigned char* block) {
  size_t bytes[FP_N], shared[3];
  ff_part_bytes(f, bytes, shared);
  const unsigned char* base = f->set0.empty() ? nullptr : f->set0.data();
  auto put = [&](int part, const void* src) {
    const void* from = src ? src : (base ? base + f->part_off[part] : nullptr);
    if (from && bytes[part]) std::memcpy(block + f->part_off[part], from, bytes[part]);
  };
  put(FP_ATOM, atom);
  put(FP_PAIR, pair);
  put(FP_CARBON, is_carbon);
  put(FP_ANGLE, angle);
  put(FP_TORSION, torsion);
  put(FP_HBOND, hbond);
  const int T = f->d.ntypes;
  ff_derive(T, general, reinterpret_cast<const double*>(block + f->part_off[FP_ATOM]),
            reinterpret_cast<const double*>(block + f->part_off[FP_PAIR]),
            reinterpret_cast<double*>(block + f->part_off[FP_GW]), reinterpret_cast<double*>(block + f->part_off[FP_LOGR]),
            reinterpret_cast<double*>(block + f->part_off[FP_RMAX]), reinterpret_cast<double*>(block + f->part_off[FP_PINV]),
            reinterpret_cast<int*>(block + f->part_off[FP_HBROLE]));
}

// Points the device view at the blob: set 0's tables, the shared index tables, the set stride.
void ff_bind(xr_ff* f) {
  unsigned char* b = static_cast<unsigned char*>(f->blob);
  XrFF& d = f->d;
  d.nsets = f->nsets;
  d.set_stride = (long long)f->set_bytes;
  d.atom = reinterpret_cast<const double*>(b + f->part_off[FP_ATOM]);
  d.pair = reinterpret_cast<const double*>(b + f->part_off[FP_PAIR]);
  d.pair_gw = reinterpret_cast<const double*>(b + f->part_off[FP_GW]);
  d.pair_logr = reinterpret_cast<const double*>(b + f->part_off[FP_LOGR]);
  d.pair_rmax = reinterpret_cast<const double*>(b + f->part_off[FP_RMAX]);
  d.pair_inv = reinterpret_cast<const double*>(b + f->part_off[FP_PINV]);
  d.is_carbon = reinterpret_cast<const int*>(b + f->part_off[FP_CARBON]);
  d.hb_role = reinterpret_cast<const int*>(b + f->part_off[FP_HBROLE]);
  d.angle = reinterpret_cast<const double*>(b + f->part_off[FP_ANGLE]);
  d.torsion = reinterpret_cast<const double*>(b + f->part_off[FP_TORSION]);
  d.hbond = reinterpret_cast<const double*>(b + f->part_off[FP_HBOND]);
  unsigned char* sh = b + (size_t)f->nsets * f->set_bytes;
  d.angle_index = reinterpret_cast<const int*>(sh + f->shared_off[0]);
  d.torsion_index = reinterpret_cast<const int*>(sh + f->shared_off[1]);
  d.hbond_index = reinterpret_cast<const int*>(sh + f->shared_off[2]);
}

// The force field's device tables with one parameter set: set 0's block and the shared index tables,
// laid out in one allocation (each table 256-byte aligned) and filled with one copy. The first call
// allocates; later calls (xr_ff_update) overwrite the same layout and drop any further sets.
int ff_pack(xr_ff* f, const double* general, const double* atom, const double* pair, const int* is_carbon, int vdw_type,
            const int* angle_index, const double* angle, const int* torsion_index, const double* torsion,
            const int* hbond_index, const double* hbond) {
  XrFF& d = f->d;
  size_t bytes[FP_N], shared[3];
  ff_part_bytes(f, bytes, shared);
  size_t set_bytes = 0, shared_bytes = 0;
  for (int k = 0; k < FP_N; ++k) {
    f->part_off[k] = set_bytes;
    set_bytes += round256(bytes[k]);
  }
  for (int k = 0; k < 3; ++k) {
    f->shared_off[k] = shared_bytes;
    shared_bytes += round256(shared[k]);
  }
  if (f->blob && (set_bytes != f->set_bytes || shared_bytes != f->shared_bytes)) return XR_EINPUT;
  const size_t total = std::max<size_t>(set_bytes + shared_bytes, 256);
  if (f->blob && f->nsets != 1) {  // back to one set
    cudaFree(f->blob);
    f->blob = nullptr;
  }
  if (!f->blob) {
    if (cudaMalloc(&f->blob, total) != cudaSuccess) {
      f->blob = nullptr;
      return XR_ECUDA;
    }
    f->blob_bytes = total;
  }
  f->set_bytes = set_bytes;
  f->shared_bytes = shared_bytes;
  f->nsets = 1;
  d.vdw_type = vdw_type;
  for (int k = 0; k < XR_NGENERAL; ++k) d.g[k] = general[k];
  d.inv_g28 = 1.0 / d.g[28];
  auto as_df = [](double v) {
    const float h = (float)v;
    return make_float2(h, (float)(v - (double)h));
  };
  d.vdw_p = as_df(d.g[28]);
  d.vdw_invp = as_df(d.inv_g28);
  d.vdw_invp_m1 = as_df(d.inv_g28 - 1.0);
  d.vdw_p_m1 = as_df(d.g[28] - 1.0);
  std::vector<unsigned char> host(total, 0);
  f->set0.clear();
  ff_fill_set(f, general, atom, pair, is_carbon, angle, torsion, hbond, host.data());
  const int* idx[3] = {angle_index, torsion_index, hbond_index};
  for (int k = 0; k < 3; ++k)
    if (shared[k]) std::memcpy(host.data() + set_bytes + f->shared_off[k], idx[k], shared[k]);
  f->set0.assign(host.begin(), host.begin() + set_bytes);
  if (cudaMemcpy(f->blob, host.data(), total, cudaMemcpyHostToDevice) != cudaSuccess) return XR_ECUDA;
  ff_bind(f);
  return XR_OK;
}

}  // namespace

extern "C" {

int xr_ff_create(const double* general, int ntypes, const double* atom, const double* pair, const int* is_carbon,
                 int vdw_type, const int* angle_index, const double* angle, int nangle, const int* torsion_index,
                 const double* torsion, int ntorsion, const int* hbond_index, const double* hbond, int nhbond,
                 xr_ff** out) {
  if (!out || !general || ntypes < 1 || !atom || !pair || !is_carbon || !angle_index || !torsion_index || !hbond_index)
    return XR_EINPUT;
  if (vdw_type < 1 || vdw_type > 3 || nangle < 0 || ntorsion < 0 || nhbond < 0) return XR_EINPUT;
  xr_ff* f = new xr_ff();
  cudaGetDevice(&f->device);
  f->nangle = nangle;
  f->ntorsion = ntorsion;
  f->nhbond = nhbond;
  f->d.ntypes = ntypes;
  const int code = ff_pack(f, general, atom, pair, is_carbon, vdw_type, angle_index, angle, torsion_index, torsion,
                           hbond_index, hbond);
  if (code != XR_OK) {
    xr_ff_destroy(f);
    return code;
  }
  *out = f;
  return XR_OK;
}

int xr_ff_update(xr_ff* f, const double* general, const double* atom, const double* pair, const int* is_carbon,
                 int vdw_type, const int* angle_index, const double* angle, const int* torsion_index,
                 const double* torsion, const int* hbond_index, const double* hbond) {
  if (!f || !general || !atom || !pair || !is_carbon || !angle_index || !torsion_index || !hbond_index || vdw_type < 1 ||
      vdw_type > 3)
    return XR_EINPUT;
  cudaSetDevice(f->device);
  return ff_pack(f, general, atom, pair, is_carbon, vdw_type, angle_index, angle, torsion_index, torsion, hbond_index,
                 hbond);
}

int xr_ff_set_count(xr_ff* f, int nsets) {
  if (!f || nsets < 1 || nsets > XR_MAX_PARAMETER_SETS) return XR_EINPUT;
  if (nsets == f->nsets) return XR_OK;
  cudaSetDevice(f->device);
  const size_t total = std::max<size_t>((size_t)nsets * f->set_bytes + f->shared_bytes, 256);
  void* blob = nullptr;
  if (cudaMalloc(&blob, total) != cudaSuccess) return XR_ECUDA;
  unsigned char* nb = static_cast<unsigned char*>(blob);
  const unsigned char* ob = static_cast<const unsigned char*>(f->blob);
  const int keep = std::min(nsets, f->nsets);
  cudaError_t e = cudaMemcpy(nb, ob, (size_t)keep * f->set_bytes, cudaMemcpyDeviceToDevice);
  for (int s = keep; s < nsets && e == cudaSuccess; ++s)
    e = cudaMemcpy(nb + (size_t)s * f->set_bytes, ob, f->set_bytes, cudaMemcpyDeviceToDevice);
  if (e == cudaSuccess && f->shared_bytes)
    e = cudaMemcpy(nb + (size_t)nsets * f->set_bytes, ob + (size_t)f->nsets * f->set_bytes, f->shared_bytes,
                   cudaMemcpyDeviceToDevice);
  if (e != cudaSuccess) {
    cudaFree(blob);
    return XR_ECUDA;
  }
  cudaFree(f->blob);
  f->blob = blob;
  f->blob_bytes = total;
  f->nsets = nsets;
  ff_bind(f);
  return XR_OK;
}

int xr_ff_set_count_of(const xr_ff* f) { return f ? f->nsets : 0; }

int xr_ff_update_sets(xr_ff* f, int first, int count, const double* atom, const double* pair, const double* angle,
                      const double* torsion, const double* hbond) {
  if (!f || first < 0 || count < 0 || first > f->nsets - count) return XR_EINPUT;
  if (count == 0) return XR_OK;
  cudaSetDevice(f->device);
  size_t bytes[FP_N], shared[3];
  ff_part_bytes(f, bytes, shared);
  const size_t T = (size_t)f->d.ntypes;
  const size_t stride[FP_N] = {T * XR_NATOM_COLS, T * T * XR_NPAIR_COLS, 0, 0, 0, 0, 0, 0, 7 * (size_t)f->nangle,
                               5 * (size_t)f->ntorsion, 4 * (size_t)f->nhbond};
  std::vector<unsigned char> host((size_t)count * f->set_bytes, 0);
  for (int s = 0; s < count; ++s)
    ff_fill_set(f, f->d.g, atom ? atom + s * stride[FP_ATOM] : nullptr, pair ? pair + s * stride[FP_PAIR] : nullptr,
                nullptr, angle ? angle + s * stride[FP_ANGLE] : nullptr,
                torsion ? torsion + s * stride[FP_TORSION] : nullptr, hbond ? hbond + s * stride[FP_HBOND] : nullptr,
                host.data() + (size_t)s * f->set_bytes);
  if (first == 0) f->set0.assign(host.begin(), host.begin() + f->set_bytes);
  if (cudaMemcpy(static_cast<unsigned char*>(f->blob) + (size_t)first * f->set_bytes, host.data(), host.size(),
                 cudaMemcpyHostToDevice) != cudaSuccess)
    return XR_ECUDA;
  return XR_OK;
}

void xr_ff_destroy(xr_ff* ff) {
  if (!ff) return;
  if (ff->blob) cudaFree(ff->blob);
  delete ff;
}

int xr_ctx_create(int device, void* stream, xr_ctx** out) {
  if (!out) return XR_EINPUT;
  xr_ctx* c = new xr_ctx();
  c->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    delete c;
    return XR_ECUDA;
  }
  if (stream) {
    c->stream = (cudaStream_t)stream;
  } else {
    cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    c->own_stream = true;
  }
  cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device);
  c->coop_per_sm = xr_qeq_coop_blocks_per_sm();
  c->max_clusters = xr_qeq_max_clusters(kQeqClusterSingle);
  c->max_clusters_batch = xr_qeq_max_clusters(kQeqClusterBatch);
  int coop_ok = 0;
  cudaDeviceGetAttribute(&coop_ok, cudaDevAttrCooperativeLaunch, device);
  if (!coop_ok) c->coop_per_sm = 0;
  bool ok = cudaMalloc((void**)&c->status, sizeof(int)) == cudaSuccess &&
            cudaMalloc((void**)&c->counts, 8 * sizeof(int)) == cudaSuccess &&
            cudaMalloc((void**)&c->barrier, (kQeqBlocks + 1) * sizeof(unsigned)) == cudaSuccess &&
            cudaMalloc((void**)&c->qmap, kQeqBlocks * sizeof(int4)) == cudaSuccess &&
            cudaMalloc((void**)&c->bx_count, sizeof(int)) == cudaSuccess &&
            cudaMalloc((void**)&c->nmids, 2 * sizeof(int)) == cudaSuccess &&
            cudaMallocHost((void**)&c->h_small, 16 * sizeof(int)) == cudaSuccess;
  if (!ok) {
    xr_ctx_destroy(c);
    return XR_ECUDA;
  }
  *out = c;
  return XR_OK;
}

void xr_ctx_destroy(xr_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (auto& e : c->gcache) cudaGraphExecDestroy(e.second.exec);
  void* bufs[] = {c->x, c->type, c->sys_of, c->wrap, c->xw, c->fw, c->cnt, c->a_fwd, c->a_adj, c->a_e, c->q, c->f,
                  c->qwork, c->outbuf, c->edge, c->edge_pair, c->edge_dbslot, c->hval, c->qch, c->qcj, c->pair_edge, c->pair_i,
                  c->pair_bond, c->p_r, c->p_shield, c->p_dshield, c->p_g, c->p_evdw, c->p_ecoul, c->bond_pair,
                  c->bond_i, c->bond_j, c->b_r, c->b_v, c->b_fwd, c->b_adj, c->b_e, c->dbrow, c->sys, c->energy,
                  c->props, c->status, c->counts, c->barrier, c->qmap, c->qsmall, c->qiters, c->red, c->qguess, c->qrhs, c->qadj, c->pgrad, c->bx_count,
                  c->arow, c->nact, c->nzrow, c->nnz, c->qb_first, c->qb_last, c->chunk_part, c->mids, c->nmids, c->mlist,
                  c->cand_cnt, c->cand_edge, c->sys_list, c->atom_cell, c->atom_slot, c->cell_cnt, c->cell_atoms,
                  c->mid_tiles, c->qsplit};
  for (void* p : bufs)
    if (p) cudaFree(p);
  if (c->h_x) cudaFreeHost(c->h_x);
  if (c->h_out) cudaFreeHost(c->h_out);
  if (c->h_guess) cudaFreeHost(c->h_guess);
  for (void* hp : {(void*)c->h_types, (void*)c->h_sysof, (void*)c->h_sysd,
                   (void*)c->h_qmap_p, (void*)c->h_qsmall_p, (void*)c->h_pg, (void*)c->h_cand_cnt, (void*)c->h_cand_edge, (void*)c->h_sys_list})
    if (hp) cudaFreeHost(hp);
  if (c->h_small) cudaFreeHost(c->h_small);
  for (int k = 0; k <= xr_ctx::kStages; ++k)
    if (c->ev[k]) cudaEventDestroy(c->ev[k]);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char* xr_last_error(const xr_ctx* c) { return c ? c->err.c_str() : "null context"; }

int xr_ctx_set_qeq(xr_ctx* c, double tolerance, int max_iterations) {
  if (!c || !(tolerance > 0) || max_iterations < 1) return XR_EINPUT;
  c->cg_tol = tolerance;
  c->cg_max = max_iterations;
  return XR_OK;
}

int xr_ctx_set_wait_test(xr_ctx* c, long long polls, int fail_at) {
  if (!c || polls < 0 || fail_at < 0) return XR_EINPUT;
  c->wait_polls = polls;
  c->wait_fail_at = fail_at;
  return XR_OK;
}

int xr_eval(xr_ctx* c, const xr_ff* ff, const xr_system* sys, unsigned flags, xr_result* out) {
  return run_batch(c, ff, 1, sys, flags, out);
}

int xr_eval_neighbors(xr_ctx* c, const xr_ff* ff, const xr_system* sys, const xr_neighbors* nb, unsigned flags,
                      xr_result* out) {
  if (c && !nb) {
    c->err = "neighbors must be a tuple (i, j, S)";
    return XR_EINPUT;
  }
  return run_batch(c, ff, 1, sys, flags, out, nb);
}

int xr_ctx_set_skin(xr_ctx* c, double skin) {
  if (!c || !(skin >= 0.0) || !std::isfinite(skin)) return XR_EINPUT;
  c->cache_valid = false;  // setting the skin, even to its current value, drops the kept list
  c->skin = skin;
  return XR_OK;
}

int xr_ctx_set_graphs(xr_ctx* c, int enable) {
  if (!c) return XR_EINPUT;
  c->graphs = enable != 0;
  if (!c->graphs && !c->gcache.empty()) {
    cudaSetDevice(c->device);
    for (auto& e : c->gcache) cudaGraphExecDestroy(e.second.exec);
    c->gcache.clear();
  }
  c->gseen.clear();
  return XR_OK;
}

int xr_last_graph(const xr_ctx* c) { return c ? c->last_graph : -1; }

int xr_ctx_set_cell_list(xr_ctx* c, int mode) {
  if (!c || mode < -1 || mode > 1) return XR_EINPUT;
  c->cell_mode = mode;
  return XR_OK;
}

int xr_last_list_info(const xr_ctx* c, int* mode, long long* builds) {
  if (!c) return XR_EINPUT;
  if (mode) *mode = c->list_mode;
  if (builds) *builds = c->list_builds;
  return XR_OK;
}

int xr_eval_batch(xr_ctx* c, const xr_ff* ff, int nsys, const xr_system* sys, unsigned flags, xr_result* out) {
  return run_batch(c, ff, nsys, sys, flags, out);
}

int xr_eval_batch_sets(xr_ctx* c, const xr_ff* ff, int nsys, const xr_system* sys, const int* sets, unsigned flags,
                       xr_result* out) {
  if (c && !sets) {
    c->err = "parameter sets require one set index per system";
    return XR_EINPUT;
  }
  return run_batch(c, ff, nsys, sys, flags, out, nullptr, sets);
}

long long xr_last_launches(const xr_ctx* c) { return c ? c->launches : 0; }

int xr_last_list_sizes(const xr_ctx* c, long long* sizes, int n) {
  if (!c || !sizes || n < 0) return XR_EINPUT;
  for (int k = 0; k < n && k < 6; ++k) sizes[k] = c->list_sizes[k];
  return XR_OK;
}

int xr_last_qeq_iterations(const xr_ctx* c) { return c ? c->qeq_iterations : 0; }

int xr_get_param_gradient_system(const xr_ctx* c, int index, double* pair_grad, long long npair, double* angle_grad,
                                 long long nangle) {
  if (!c || c->pgrad_pairs == 0 || index < -1 || index >= c->pgrad_systems) return XR_EINPUT;
  if (npair != c->pgrad_pairs || nangle != c->pgrad_angles || !pair_grad || (nangle > 0 && !angle_grad)) return XR_EINPUT;
  const long long stride = npair + nangle + c->pgrad_atoms;
  const int s0 = index < 0 ? 0 : index, s1 = index < 0 ? c->pgrad_systems : index + 1;
  for (long long k = 0; k < npair; ++k) pair_grad[k] = 0.0;
  for (long long k = 0; k < nangle; ++k) angle_grad[k] = 0.0;
  for (int sy = s0; sy < s1; ++sy) {  // systems in call order: the same sum on every call
    const double* g = c->h_pgrad.data() + (size_t)sy * stride;
    for (long long k = 0; k < npair; ++k) pair_grad[k] += g[k];
    for (long long k = 0; k < nangle; ++k) angle_grad[k] += g[npair + k];
  }
  return XR_OK;
}

int xr_get_param_gradient_atoms(const xr_ctx* c, int index, double* atom_grad, long long natom) {
  if (!c || c->pgrad_pairs == 0 || index < -1 || index >= c->pgrad_systems || natom != c->pgrad_atoms || !atom_grad)
    return XR_EINPUT;
  const long long stride = c->pgrad_pairs + c->pgrad_angles + c->pgrad_atoms;
  const int s0 = index < 0 ? 0 : index, s1 = index < 0 ? c->pgrad_systems : index + 1;
  for (long long k = 0; k < natom; ++k) atom_grad[k] = 0.0;
  for (int sy = s0; sy < s1; ++sy) {
    const double* g = c->h_pgrad.data() + (size_t)sy * stride + c->pgrad_pairs + c->pgrad_angles;
    for (long long k = 0; k < natom; ++k) atom_grad[k] += g[k];
  }
  return XR_OK;
}

int xr_get_param_gradient_blocks(const xr_ctx* c, double* out, long long count) {
  if (!c || c->pgrad_pairs == 0 || !out) return XR_EINPUT;
  const long long all = (c->pgrad_pairs + c->pgrad_angles + c->pgrad_atoms) * (long long)c->pgrad_systems;
  if (count != all) return XR_EINPUT;
  std::memcpy(out, c->h_pgrad.data(), sizeof(double) * (size_t)all);
  return XR_OK;
}

int xr_get_param_gradient(const xr_ctx* c, double* pair_grad, long long npair, double* angle_grad, long long nangle) {
  return xr_get_param_gradient_system(c, -1, pair_grad, npair, angle_grad, nangle);
}

int xr_last_qeq_work(const xr_ctx* c, long long* iterations, double* matvec_bytes) {
  if (!c || !iterations || !matvec_bytes) return XR_EINPUT;
  const int L = c->last_A + 1;
  long long its = 0;
  double bytes = 0;
  for (size_t s = 0; s < c->h_qiters.size() && s < c->host_sys.size(); ++s) {
    const XrSystem& sy = c->host_sys[s];
    const long long pairs = c->host_cnt[1 * L + sy.atom_off + sy.natoms] - c->host_cnt[1 * L + sy.atom_off];
    its += c->h_qiters[s];
    bytes += (double)c->h_qiters[s] * (8.0 * (double)pairs + 16.0 * sy.natoms);
  }
  *iterations = its;
  *matvec_bytes = bytes;
  return XR_OK;
}

int xr_last_transfer_bytes(const xr_ctx* c, long long* h2d, long long* d2h) {
  if (!c) return XR_EINPUT;
  if (h2d) *h2d = c->h2d_bytes;
  if (d2h) *d2h = c->d2h_bytes;
  return XR_OK;
}

int xr_get_neighbors(xr_ctx* c, int index, int* i, int* j, int* S, long long capacity, long long* count) {
  if (!c || index < 0 || index >= (int)c->host_sys.size() || !count) return XR_EINPUT;
  const int L = c->last_A + 1;
  const XrSystem& sy = c->host_sys[index];
  const int a0 = sy.atom_off, a1 = sy.atom_off + sy.natoms;
  const int e0 = c->host_cnt[a0], e1 = c->host_cnt[a1];
  *count = e1 - e0;
  if (capacity < e1 - e0 || !i || !j || !S) return XR_OK;
  std::vector<int2> ed(e1 - e0);
  cudaMemcpy(ed.data(), c->edge + e0, sizeof(int2) * (e1 - e0), cudaMemcpyDeviceToHost);
  (void)L;
  for (int a = a0; a < a1; ++a)
    for (int e = c->host_cnt[a]; e < c->host_cnt[a + 1]; ++e) {
      const int k = e - e0;
      const uint32_t code = (uint32_t)ed[k].y;
      i[k] = a - a0;
      j[k] = ed[k].x - a0;
      S[3 * k + 0] = xr_sx(code);
      S[3 * k + 1] = xr_sy(code);
      S[3 * k + 2] = xr_sz(code);
    }
  return XR_OK;
}

int xr_get_bonds(xr_ctx* c, int index, int* i, int* j, int* S, double* bo, long long capacity, long long* count) {
  if (!c || index < -1 || index >= (int)c->host_sys.size() || !count) return XR_EINPUT;
  const int L = c->last_A + 1;
  // index -1: every system of the batch, atom indices counted over the concatenated systems
  const int a0 = index < 0 ? 0 : c->host_sys[index].atom_off;
  const int a1 = index < 0 ? c->last_A : a0 + c->host_sys[index].natoms;
  const int b0 = c->host_cnt[2 * L + a0], b1 = c->host_cnt[2 * L + a1];
  // exported entries are sorted by bond id: the system's are one contiguous run
  const auto& m = c->h_bx_meta;
  const auto lo = std::lower_bound(m.begin(), m.end(), b0, [](const int4& v, int key) { return v.x < key; });
  const auto hi = std::lower_bound(m.begin(), m.end(), b1, [](const int4& v, int key) { return v.x < key; });
  const long long n = hi - lo;
  *count = n;
  if (capacity < n || !i || !j || !S || !bo) return XR_OK;
  long long k = 0;
  for (auto it = lo; it != hi; ++it, ++k) {
    const uint32_t code = (uint32_t)it->w;
    i[k] = it->y - a0;
    j[k] = it->z - a0;
    S[3 * k + 0] = xr_sx(code);
    S[3 * k + 1] = xr_sy(code);
    S[3 * k + 2] = xr_sz(code);
    bo[k] = c->h_bx_bo[it - m.begin()];
  }
  return XR_OK;
}

int xr_ctx_reserve(xr_ctx* c, int atoms, int systems, long long edges, long long bonds) {
  if (!c || atoms < 1 || systems < 1 || edges < 0 || bonds < 0) return XR_EINPUT;
  cudaSetDevice(c->device);
  const long long chunks = (long long)systems + atoms / XR_CHUNK_ATOMS + 1;
  // pinned host buffers too: a call within the reservation allocates and frees no page-locked memory
  // (whose allocation stalls, and whose release waits for the whole device, other threads' work included)
  if (!ensure_atoms(c, atoms, systems) || !host_grow(&c->h_x, &c->ch_x, (size_t)atoms) ||
      !host_grow(&c->h_guess, &c->ch_guess, (size_t)atoms) || !host_grow(&c->h_types, &c->ch_types, (size_t)atoms) ||
      !host_grow(&c->h_sysof, &c->ch_sysof, (size_t)atoms) || !host_grow(&c->h_sysd, &c->ch_sysd, (size_t)systems) ||
      !host_grow(&c->h_qsmall_p, &c->ch_qsmall_p, (size_t)systems) ||
      !host_grow(&c->h_qmap_p, &c->ch_qmap_p, (size_t)std::max(1, std::min(c->nsm * c->coop_per_sm, kQeqBlocks))) ||
      !ensure_lists(c, edges, edges / 2, bonds) ||
      !grow(c, &c->chunk_part, &c->cchunk_part, (size_t)chunks * XR_PART_N) ||
      !grow(c, &c->outbuf, &c->coutbuf, result_layout(atoms, systems, bonds).end) ||
      !host_grow(&c->h_out, &c->ch_out, result_layout(atoms, systems, bonds).end) ||
      // candidate rows and the cell list, for calls that search by cells
      !grow(c, &c->cand_cnt, &c->ccand_cnt, (size_t)atoms + 1) ||
      !grow(c, &c->cand_edge, &c->ccand_edge, (size_t)std::max<long long>(edges, 1)) ||
      !grow(c, &c->atom_cell, &c->catom_cell, (size_t)atoms) || !grow(c, &c->atom_slot, &c->catom_slot, (size_t)atoms) ||
      !grow(c, &c->cell_atoms, &c->ccell_atoms, (size_t)atoms) ||
      !grow(c, &c->cell_cnt, &c->ccell_cnt, 2 * (size_t)atoms + 64 * (size_t)systems + 1))
    return cuda_fail(c, cudaErrorMemoryAllocation, "reservation");
  return XR_OK;
}

int xr_ctx_memory(const xr_ctx* c, long long* device_bytes, long long* caps, int n) {
  if (!c || n < 0 || (n > 0 && !caps)) return XR_EINPUT;
  if (device_bytes) *device_bytes = c->dev_bytes;
  const long long v[6] = {(long long)c->cx, (long long)c->csys, (long long)c->cedge, (long long)c->cpair_edge,
                          (long long)c->capB, (long long)c->ccand_edge};
  for (int k = 0; k < n && k < 6; ++k) caps[k] = v[k];
  return XR_OK;
}

long long xr_footprint_bytes(int atoms, int systems, long long edges, long long bonds) {
  if (atoms < 1 || systems < 1 || edges < 0 || bonds < 0) return -1;
  // the buffers of ensure_atoms, ensure_lists and xr_ctx_reserve, per element
  const long long per_atom = sizeof(double4_32a) + 2 * sizeof(int) + sizeof(int4) + 2 * sizeof(float4) + 4 * sizeof(int) +
                             (AF_N + AJ_N + 8 + 4 + 3 + XR_QW_N + 8) * sizeof(double) + 8 * sizeof(int);
  const long long per_system = sizeof(int2) + 3 * sizeof(int) + sizeof(XrSystem) + 20 * sizeof(double);
  const long long per_edge = sizeof(int2) + 2 * sizeof(int) + sizeof(double) + sizeof(float) + sizeof(unsigned short);
  const long long per_pair = 3 * sizeof(int) + 6 * sizeof(double);
  const long long per_bond = kBondBytes + 32;  // + the exported-bond record of the result block
  const long long chunks = (long long)systems + atoms / XR_CHUNK_ATOMS + 1;
  const long long per_cells = 4 * sizeof(int) + 2 * sizeof(int);  // cand_cnt, atom_cell, atom_slot, cell_atoms, cell_cnt
  const long long base = (long long)atoms * (per_atom + per_cells) + (long long)systems * (per_system + 64 * sizeof(int)) +
                         edges * (per_edge + sizeof(int2)) + (edges / 2) * per_pair + bonds * per_bond +
                         chunks * XR_PART_N * sizeof(double);
  const long long red = (long long)sizeof(double) * 4 * 8 * 2048;  // reduction scratch, at least this
  // grow()'s headroom (n + n/4 + 64 elements per buffer), rounded up by 2 %
  return (base + red) * 5 / 4 + (base + red) / 50 + 64ll * 64 * 16;
}

int xr_ctx_set_profiling(xr_ctx* c, int enable) {
  if (!c) return XR_EINPUT;
  cudaSetDevice(c->device);
  if (enable && !c->ev[0])
    for (int k = 0; k <= xr_ctx::kStages; ++k) cudaEventCreate(&c->ev[k]);
  c->profile = enable != 0;
  for (int k = 0; k < xr_ctx::kStages; ++k) c->stage_ms[k] = 0.0;
  c->stage_calls = 0;
  return XR_OK;
}

int xr_ctx_stage_times(const xr_ctx* c, double* ms, int n, long long* calls) {
  if (!c || !ms) return XR_EINPUT;
  for (int k = 0; k < n && k < xr_ctx::kStages; ++k) ms[k] = c->stage_ms[k];
  if (calls) *calls = c->stage_calls;
  return XR_OK;
}

}  // extern "C"
