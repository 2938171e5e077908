/*
 * xreac_gb300 -- C ABI of the GB300 ReaxFF evaluator.
 *
 * The entry points replace the evaluation path behind hsulab/xreac's Python API:
 *   ForceField.from_file / bundled          (src/xreac/forcefield.py:84-95, 120-315) -> xr_ff_create
 *   Calculator(force_field)                  (src/xreac/calculator.py:69-74)          -> xr_ctx_create
 *   Calculator.evaluate(symbols, positions, total_charge, cell, pbc, full_derivative)
 *                                            (src/xreac/calculator.py:76-165)         -> xr_eval
 *   one evaluate per request, batched        (no reference counterpart; serving)      -> xr_eval_batch
 *   the ValueError raised by evaluate        (src/xreac/calculator.py:58-66, 149-154) -> return code + xr_last_error
 *   Neighbors(i, j, S) of an evaluation      (src/xreac/neighbors.py:101-131)         -> xr_get_neighbors
 *   Evaluation.bond_orders (sparse form)     (src/xreac/energy.py:167-178)            -> xr_get_bonds
 *
 * Plain pointers and sizes only. Units: Angstrom, kcal/mol, kcal/mol/Angstrom, elementary charge.
 * All floating point is IEEE double. Arrays are C-contiguous.
 */
#ifndef XREAC_GB300_H
#define XREAC_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* Return codes. xr_last_error(ctx) gives the message, worded as xreac's ValueError texts. */
enum xr_status {
  XR_OK = 0,
  XR_EINPUT = 1,        /* invalid arguments (shapes, types, cell) */
  XR_ECOINCIDENT = 2,   /* "Coincident atoms are not supported" */
  XR_ESINGULAR = 3,     /* "Singular QEq system; check the geometry and parameters" */
  XR_ENONFINITE = 4,    /* "Non-finite energy, charges, or forces; check the geometry" */
  XR_ECHARGE = 5,       /* "QEq charge constraint failed" */
  XR_ECOLLINEAR = 6,    /* "Collinear atoms in an active torsion: ..." */
  XR_ECAPACITY = 7,     /* a device list outgrew its limit (image shifts beyond +-255 cells) */
  XR_EBADPARAM = 8,     /* "Invalid p_boc* mixing for an active bond-order correction" */
  XR_ECUDA = 9,         /* CUDA runtime failure */
  XR_EUNSUPPORTED = 10, /* requested option not available */
  XR_ECG_NOCONV = 11,   /* the QEq conjugate gradient reached its iteration limit (xr_ctx_set_qeq) */
  XR_EWAIT = 12         /* a device-side wait of the QEq solver gave up: a scheduling failure, not an
                           input error; the context stays usable and the call may be repeated */
};

/* Evaluation flags. */
#define XR_FLAG_FULL_DERIVATIVE 1u /* charge-response forces (xreac full_derivative=True) */
#define XR_FLAG_DEVICE_IO 2u       /* positions and result arrays are device pointers */
#define XR_FLAG_PARAM_GRADIENT 4u  /* also dE/dtheta for bond, angle and vdW parameters (xr_get_param_gradient) */
#define XR_FLAG_QEQ_GRADIENT 8u    /* with XR_FLAG_PARAM_GRADIENT: also chi, eta (xr_get_param_gradient_atoms) and the
                                    * pair table's gamma, through an adjoint QEq solve */

typedef struct xr_ff xr_ff;
typedef struct xr_ctx xr_ctx;

/* One system. positions: natoms x 3. cell: 9 doubles (three row vectors) or NULL when no
 * direction is periodic. types: element numbers in parameter-file order. charges_guess: NULL, or
 * natoms starting charges for the QEq solve (e.g. the previous step's charges of the same system;
 * shifted to sum to total_charge). It changes only the iteration count: convergence is measured
 * against the projected residual of the uniform start, so the result meets the same tolerance. */
typedef struct {
  int natoms;
  const int* types;
  const double* positions;
  const double* cell;
  int pbc[3];
  double total_charge;
  const double* charges_guess;
} xr_system;

/* A caller-supplied directed neighbour list of one system, xreac's neighbors=(i, j, S)
 * (src/xreac/calculator.py:113-120, src/xreac/neighbors.py:101-131): edge e points from atom i[e] to
 * the image of atom j[e] at x[j] + S[e] @ cell. Both directions of every pair, any order, no
 * zero-shift self edge; edges beyond the cutoff (a skin) are allowed. Host pointers. */
typedef struct {
  long long count;  /* number of directed edges */
  const int* i;     /* count source atoms */
  const int* j;     /* count target atoms */
  const int* S;     /* count x 3 integer lattice shifts */
} xr_neighbors;

/* Results of one system. Any pointer may be NULL to skip that output.
 * energy: 15 doubles = the 14 components in xreac's order (bond, atom, lone_pair, molecule, angle,
 * penalty, angle_conjugation, hydrogen_bond, torsion, conjugation, vdw, coulomb, electric_field,
 * qeq) followed by the total. */
typedef struct {
  double* energy;
  double* forces;            /* natoms x 3 */
  double* charges;           /* natoms */
  double* total_bond_orders; /* natoms */
  double* lone_pairs;        /* natoms */
  int* bond_counts;          /* natoms */
  double* dipole;            /* 3 */
} xr_result;

/* Force field: packed tables as produced by xreac_gb300.forcefield.ForceField.tables().
 * general: 39; atom: ntypes x 24; pair: ntypes^2 x 28; is_carbon: ntypes;
 * angle_index: ntypes^3 x 2 (first, count) into angle (nangle x 7);
 * torsion_index: ntypes^4 (row or -1) into torsion (ntorsion x 5);
 * hbond_index: ntypes^3 (row or -1) into hbond (nhbond x 4). vdw_type: 1, 2 or 3. */
int xr_ff_create(const double* general, int ntypes, const double* atom, const double* pair, const int* is_carbon,
                 int vdw_type, const int* angle_index, const double* angle, int nangle, const int* torsion_index,
                 const double* torsion, int ntorsion, const int* hbond_index, const double* hbond, int nhbond,
                 xr_ff** out);
void xr_ff_destroy(xr_ff* ff);

/* Replace the parameter values of a force field in place (no reference counterpart; the reference
 * rebuilds its per-edge parameter arrays on every evaluation): the same table shapes as at
 * xr_ff_create (ntypes, angle, torsion and hydrogen-bond record counts), new values; one host-to-
 * device copy, no allocation. No evaluation that uses this force field may be in flight. For
 * parameter fitting and perturbation studies that evaluate many variants of one force field. */
int xr_ff_update(xr_ff* ff, const double* general, const double* atom, const double* pair, const int* is_carbon,
                 int vdw_type, const int* angle_index, const double* angle, const int* torsion_index,
                 const double* torsion, const int* hbond_index, const double* hbond);

/* Parameter sets (no reference counterpart; the reference evaluates one force field per call).
 * A force field can hold nsets variants of its parameters, each with the elements and records of
 * xr_ff_create: the general parameters and the angle / torsion / hydrogen-bond index tables are
 * shared, while the atom, pair, angle, torsion and hydrogen-bond values (and the tables derived
 * from them) are per set. xr_eval_batch_sets then evaluates every system with its own set, so many
 * perturbed or fitted copies of a force field run in one batch. Set 0 is the force field of
 * xr_ff_create / xr_ff_update; xr_ff_update returns the force field to that single set.
 *
 * xr_ff_set_count: resize to nsets (1 <= nsets <= XR_MAX_PARAMETER_SETS); sets kept keep their
 * values, new ones start as copies of set 0. Reallocates the device tables: no evaluation that uses
 * this force field may be in flight.
 * xr_ff_update_sets: values of sets first .. first + count - 1, one host-to-device copy. Each table
 * pointer is NULL (every one of these sets takes set 0's values) or holds count consecutive tables of
 * the xr_ff_create shapes: atom count x ntypes x 24, pair count x ntypes^2 x 28, angle count x
 * nangle x 7, torsion count x ntorsion x 5, hbond count x nhbond x 4. */
#define XR_MAX_PARAMETER_SETS 65536
int xr_ff_set_count(xr_ff* ff, int nsets);
int xr_ff_set_count_of(const xr_ff* ff);
int xr_ff_update_sets(xr_ff* ff, int first, int count, const double* atom, const double* pair, const double* angle,
                      const double* torsion, const double* hbond);

/* Context: device work buffers (grown on demand, reused across calls) and a CUDA stream.
 * stream may be NULL (the context creates its own) or a cudaStream_t owned by the caller.
 * A context is used by one host thread at a time. */
int xr_ctx_create(int device, void* stream, xr_ctx** out);
void xr_ctx_destroy(xr_ctx* ctx);
const char* xr_last_error(const xr_ctx* ctx);

/* Pre-size the context's device and pinned host buffers for batches of up to `atoms` atoms in
 * `systems` systems with `edges` directed neighbour edges and `bonds` bond candidates (r <= 5 A),
 * so later calls within these sizes never allocate (no reference counterpart; serving). Buffers
 * otherwise grow on demand, and a growth frees and reallocates device memory, which synchronises
 * the whole device. */
int xr_ctx_reserve(xr_ctx* ctx, int atoms, int systems, long long edges, long long bonds);

/* Solver settings: QEq conjugate-gradient relative residual and iteration limit. */
int xr_ctx_set_qeq(xr_ctx* ctx, double tolerance, int max_iterations);

/* Tests of the failure path of the QEq solver's team waits (no reference counterpart). Every wait
 * of a thread-block cluster or grid team is bounded; polls > 0 replaces the default limits (2^22
 * polls for a cluster exchange, 2^24 for a grid barrier; 0 restores them). fail_at > 0 makes team
 * wait number fail_at of each solve wait for an arrival that never comes, so it runs out, the call
 * returns XR_EWAIT and the context stays usable; 0 turns this off. Systems of at most 160 atoms
 * (a single block, no team waits) are not affected. */
int xr_ctx_set_wait_test(xr_ctx* ctx, long long polls, int fail_at);

/* Test of the device math (no reference counterpart): out[i] = f(in[i]) for n device-resident
 * doubles on the current device's default stream, f = the double-float exp (fn 0) or log (fn 2) that
 * the pair and bond-order kernels use, or CUDA's FP64 exp (fn 1) or log (fn 3) to compare with.
 * Returns XR_OK, XR_EINPUT for a bad fn or n, or XR_ECUDA. */
int xr_test_math(int fn, const double* in, double* out, int n);

/* Evaluate one system (energy, fixed-charge forces, QEq charges, per-atom bond properties). */
int xr_eval(xr_ctx* ctx, const xr_ff* ff, const xr_system* sys, unsigned flags, xr_result* out);

/* Evaluate one system on exactly the edges of a caller-supplied list: Calculator.evaluate with
 * neighbors=(i, j, S) (src/xreac/calculator.py:113-120). The list is validated with xreac's rules and
 * messages (XR_EINPUT: indices out of range, nonzero shifts in non-periodic directions, zero-shift self
 * edges, duplicates, a missing reverse direction), put in canonical order, and reduced on the device
 * to its edges within the cutoff, which are the only ones that contribute; pairs missing from the list
 * contribute nothing, as in xreac. Shifts beyond +-255 cells give XR_ECAPACITY. */
int xr_eval_neighbors(xr_ctx* ctx, const xr_ff* ff, const xr_system* sys, const xr_neighbors* nb, unsigned flags,
                      xr_result* out);

/* The validation of xr_eval_neighbors alone, on the host (no device work): XR_OK, or the status and,
 * in msg (msg_len bytes, NUL-terminated), the message xreac's ValueError carries. pbc: 3 flags. */
int xr_neighbors_check(int natoms, const int* pbc, const xr_neighbors* nb, char* msg, int msg_len);

/* Neighbour-list reuse across calls, as ASE's skin list does (src/xreac/ase.py:107-131): with
 * skin > 0 each xr_eval / xr_eval_batch call keeps on the device a list of every image within
 * cutoff + 2 skin, and a later call on the same systems (atom counts, types, pbc, cells, cutoff)
 * reuses it while no atom has moved more than `skin` from its position at the build; the edges
 * within the cutoff are then re-selected from that list by exact distance tests, so results equal
 * those of a fresh list. skin = 0 (the default) scans every call. Setting the skin, even to its
 * current value, drops the kept list. */
int xr_ctx_set_skin(xr_ctx* ctx, double skin);

/* CUDA graphs (no reference counterpart): with enable != 0 (the default) the second call with a
 * given launch sequence (the same systems' sizes and periodicity, force field, flags and buffers, as
 * in relaxation or MD steps or a request size seen before) records the kernels after the neighbour
 * count as a CUDA graph, and later calls with that sequence replay it as one launch; a context keeps
 * its 128 most recently used graphs. The kernels read the list sizes from device memory, so a replay
 * is the same computation. Not used with stage timing (xr_ctx_set_profiling) or with grid-wide QEq
 * teams. xr_last_graph: 0 launched directly, 1 recorded, 2 replayed (-1 for a null context).
 * xr_ctx_set_graphs(ctx, 0) releases the context's graphs. */
int xr_ctx_set_graphs(xr_ctx* ctx, int enable);
int xr_last_graph(const xr_ctx* ctx);

/* Cell-list neighbour search (no reference counterpart; xreac enumerates every atom pair over the
 * replicated images, src/xreac/neighbors.py:17-53). mode 0 (the default) uses it for a call whose
 * largest system has at least 1,024 atoms when it halves the expected image tests; 1 always; -1
 * never. Either way the list is the image scan's, in the same canonical order: the cell search
 * yields the same candidate images, each row is then sorted. */
int xr_ctx_set_cell_list(xr_ctx* ctx, int mode);

/* How the last call got its neighbour rows (mode: 0 image scan, 1 skin list built, 2 skin list
 * reused, 3 supplied list, 4 cell-list search, 5 skin list built from the cell list) and how many
 * skin lists the context has built (no reference counterpart; instrumentation). */
int xr_last_list_info(const xr_ctx* ctx, int* mode, long long* builds);

/* Evaluate nsys independent systems in one ragged batch with per-system offsets. */
int xr_eval_batch(xr_ctx* ctx, const xr_ff* ff, int nsys, const xr_system* sys, unsigned flags, xr_result* out);

/* As xr_eval_batch, system s evaluated with parameter set sets[s] of ff (0 <= sets[s] < the set
 * count). With XR_FLAG_PARAM_GRADIENT each system's gradient is with respect to its own set. */
int xr_eval_batch_sets(xr_ctx* ctx, const xr_ff* ff, int nsys, const xr_system* sys, const int* sets, unsigned flags,
                       xr_result* out);

/* Neighbour list of the last evaluation of system `index` of the last batch, in canonical
 * (i, j, Sx, Sy, Sz) order: i, j (capacity entries each), S (capacity x 3). *count receives the
 * number of directed edges; nothing is written when capacity is too small. Host pointers. */
int xr_get_neighbors(xr_ctx* ctx, int index, int* i, int* j, int* S, long long capacity, long long* count);

/* Nonzero corrected bond orders of the last evaluation of system `index`, one entry per unordered
 * image pair (i, j, S) in pair order; the directed pair (j, i, -S) carries the same value.
 * index -1 returns those of every system of the batch at once, with atom indices counted over the
 * systems concatenated in call order. Host pointers; *count as for xr_get_neighbors. */
int xr_get_bonds(xr_ctx* ctx, int index, int* i, int* j, int* S, double* bo, long long capacity, long long* count);

/* Gradient of the total energy, summed over the systems of the last call made with
 * XR_FLAG_PARAM_GRADIENT, with respect to force-field parameters (no reference counterpart; the
 * reference has no parameter derivatives): pair_grad[(s*ntypes + t)*28 + column] over the pair-table
 * columns of xr_ff_create (filled: De_s, De_p, De_pp, p_be1, p_be2, p_ovun1, p_bo1..p_bo6, r_s, r_p, r_pp, D,
 * alpha, gamma_w, r_vdW, rcore, ecore, acore; others 0), and angle_grad[row*7 + k] over the angle
 * records (theta00, p_val1, p_val2, p_coa1, p_val7, p_pen1, p_val4). A parameter stored once for
 * both orders of a pair (or for both ends of an angle) gets the sum of its rows. Charges do not
 * depend on these parameters, so this is the total derivative. npair = ntypes^2 * 28 and
 * nangle = 7 * (angle records) must match. */
int xr_get_param_gradient(const xr_ctx* ctx, double* pair_grad, long long npair, double* angle_grad, long long nangle);

/* As xr_get_param_gradient for the energy of system `index` of that call alone (index -1: the sum
 * over its systems, which is xr_get_param_gradient). Every system of a call keeps its own gradient,
 * so several evaluations (e.g. the displaced geometries of a finite difference) share one call. */
int xr_get_param_gradient_system(const xr_ctx* ctx, int index, double* pair_grad, long long npair, double* angle_grad,
                                 long long nangle);

/* The atom-table part of that gradient: atom_grad[t*24 + column] over the atom-table columns of
 * xr_ff_create, filled for chi and eta when the call had XR_FLAG_QEQ_GRADIENT (then the pair table's
 * gamma column is filled too); natom = ntypes * 24. The QEq parameters change the charges, so these
 * total derivatives come from an adjoint QEq solve: dE/dchi = 23.02 q - lambda, dE/deta = 11.51 q^2 -
 * lambda q per atom, with lambda the solution of H lambda = dE/dq on sum lambda = 0 (no reference
 * counterpart). index as for xr_get_param_gradient_system. */
int xr_get_param_gradient_atoms(const xr_ctx* ctx, int index, double* atom_grad, long long natom);

/* Every system's gradient block of that call at once: out[s * (npair + nangle + natom) + k], the pair
 * columns (k < npair), the angle records, then the atom-table columns, for s in call order;
 * count = systems x (npair + nangle + natom). */
int xr_get_param_gradient_blocks(const xr_ctx* ctx, double* out, long long count);

/* Device memory of a context (no reference counterpart; for admission by footprint): the bytes its
 * buffers hold, and their capacities caps[0..n) = atoms, systems, directed edges, pairs, bonds,
 * candidate edges (a call within them allocates nothing). */
int xr_ctx_memory(const xr_ctx* ctx, long long* device_bytes, long long* caps, int n);

/* Device bytes a context needs for calls of up to `atoms` atoms in `systems` systems with `edges`
 * directed edges and `bonds` bond candidates (what xr_ctx_reserve would allocate), or -1 for invalid
 * sizes. Needs no device. */
long long xr_footprint_bytes(int atoms, int systems, long long edges, long long bonds);

/* Number of CUDA kernels the last xr_eval / xr_eval_batch call launched. */
long long xr_last_launches(const xr_ctx* ctx);

/* List sizes of the last call, summed over its systems (no reference counterpart; instrumentation):
 * sizes[0] directed edges within the cutoff, [1] unordered pairs, [2] bond candidates (pairs with
 * r <= 5 A), [3] directed bond-row entries, [4] active bonds (uncorrected order at or above the cut),
 * [5] torsion middle bonds (bo > 0.001). The first n (at most 6) are written. */
int xr_last_list_sizes(const xr_ctx* ctx, long long* sizes, int n);

/* QEq conjugate-gradient iterations of the last call (largest over its systems; no reference
 * counterpart: the reference solves the KKT system directly). */
int xr_last_qeq_iterations(const xr_ctx* ctx);

/* QEq work of the last call (no reference counterpart; instrumentation): the conjugate-gradient
 * iterations summed over its systems, and the algorithmic bytes of a matrix-free product summed
 * over every iteration of every system: iterations x (8 B per unordered pair + 16 B per atom). */
int xr_last_qeq_work(const xr_ctx* ctx, long long* iterations, double* matvec_bytes);

/* Host-to-device and device-to-host bytes the last call moved (no reference counterpart). */
int xr_last_transfer_bytes(const xr_ctx* ctx, long long* h2d, long long* d2h);

/* Per-stage device timing with CUDA events on the context stream (no reference counterpart;
 * instrumentation). enable=1 resets the accumulators. Stages: 0 neighbour count + scan (including
 * the host read of the list sizes), 1 row fill + reverse map, 2 pair kernel (vdW, shield) and QEq
 * matrix rows, 3 QEq solve, 4 charge response (the adjoint QEq solve; empty unless the call asks
 * for the charge-response derivative or the QEq parameters' gradient), 5 bond orders (uncorrected,
 * Delta', corrected), 6 bonded terms + adjoint chain, 7 Coulomb energy + force assembly +
 * reductions + result packing. ms receives the summed
 * milliseconds of the first n (at most 8) stages over *calls evaluations. */
int xr_ctx_set_profiling(xr_ctx* ctx, int enable);
int xr_ctx_stage_times(const xr_ctx* ctx, double* ms, int n, long long* calls);

/* Allocation-free neighbour counting (no counterpart in the reference, which always allocates
 * through NumPy). For callers that cannot allocate device memory where they need the count: a
 * process whose device memory belongs to a framework's pool allocator, a step loop that cannot
 * take the device-wide synchronisation of cudaFree, or a caller sizing its own neighbour buffers.
 * Writes counts[a] = number of directed neighbours (j, S) of atom a with |x_j - x_a + S @ cell|
 * <= cutoff, zero-shift self pairs excluded -- the row lengths of xr_get_neighbors's list for the
 * same cutoff -- and *total (may be NULL) = their sum. positions, cell and counts are HOST
 * pointers; types is not read. Work is issued on `stream` (a cudaStream_t of the current device,
 * NULL = default stream; a stream of another device is rejected with XR_EINPUT), which the call
 * synchronises before returning.
 * All device scratch is one static array of the library: no cudaMalloc, cudaFree or allocating
 * library call. natoms above XR_STATIC_MAX_ATOMS is rejected with XR_ECAPACITY. Calls that overlap
 * in time on one device (two threads, or unordered streams) race on the shared scratch. The first
 * call on a device performs the set-up (a cudaGetSymbolAddress with that device current); make it
 * before any stream capture begins. The address found then is kept for the life of the process, so
 * do not call this again on a device after cudaDeviceReset. Cells follow xr_eval's rules (finite,
 * nonsingular, right-handed). xr_static_last_error() gives the message of this thread's last
 * failed call. */
#define XR_STATIC_MAX_ATOMS 16384
int xr_count_neighbors_static(const xr_system* sys, double cutoff, void* stream, int* counts, long long* total);
const char* xr_static_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* XREAC_GB300_H */
