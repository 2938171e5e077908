"""Seeded synthetic systems with the shapes, sizes and compositions of the benchmark workloads.

There is no public dataset behind these workloads; every structure is generated
here from a fixed seed, so the benchmark and the tests see identical inputs.

- ``water_cluster``: rigid H2O (O-H 0.97 A, H-O-H 104.5 deg) with uniformly placed
  oxygens, a minimum O-O distance enforced by rejection and uniformly random
  orientations; non-periodic (64 H2O in a 12 A cube, seed 1).
- ``water_box``: the same molecules in a periodic cube with minimum-image
  rejection and Gaussian jitter on every atom (1,536 H2O in 35.8 A, seed 2).
- ``cho_mixture``: CH4 / O2 / H2O / CO2 with ideal geometries in a periodic cube
  sized to a mass density, inter-molecular heavy-atom distance enforced.
- ``request_stream``: a stream of uneven-size evaluation requests (clusters and
  small periodic cells of the molecules above, two force fields, repeats with
  small jitter, Poisson arrival times).

Positions are float64 Angstrom; cells are (3, 3) row-vector matrices.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

MASS = {"H": 1.008, "C": 12.011, "O": 15.999}
AVOGADRO_A3 = 0.602214076  # g/cm^3 -> amu per A^3 conversion factor


def _rotation(rng):
    """Uniformly random proper rotation (QR of a Gaussian matrix, sign-fixed)."""
    q, r = np.linalg.qr(rng.normal(size=(3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def _water():
    half = np.deg2rad(104.5 / 2)
    return ["O", "H", "H"], np.array(
        [[0.0, 0.0, 0.0], [0.97 * np.cos(half), 0.97 * np.sin(half), 0.0], [0.97 * np.cos(half), -0.97 * np.sin(half), 0.0]]
    )


def _methane():
    d = 1.09 / np.sqrt(3.0)
    return ["C", "H", "H", "H", "H"], np.array(
        [[0.0, 0, 0], [d, d, d], [d, -d, -d], [-d, d, -d], [-d, -d, d]]
    )


def _oxygen():
    return ["O", "O"], np.array([[-0.605, 0.0, 0.0], [0.605, 0.0, 0.0]])


def _co2():
    return ["C", "O", "O"], np.array([[0.0, 0, 0], [1.16, 0, 0], [-1.16, 0, 0]])


MOLECULES = {"H2O": _water, "CH4": _methane, "O2": _oxygen, "CO2": _co2}


@dataclass
class System:
    symbols: list
    positions: np.ndarray
    cell: np.ndarray | None = None
    pbc: bool = False
    total_charge: float = 0.0
    force_field: str = "ffield.reax.HO.2015"

    @property
    def n(self):
        return len(self.symbols)


def _place(rng, molecules, box, min_dist, periodic, max_trials=2_000_000):
    """Random sequential placement of rigid molecules, checking heavy-atom distances.

    ``molecules`` is a list of (symbols, local_coords) drawn in order. Each
    molecule's centre is uniform in the box and its orientation uniform; it is
    accepted when every heavy atom (C or O) is at least ``min_dist`` from every
    previously accepted heavy atom (minimum image when periodic).
    """
    symbols, coords, heavy = [], [], np.zeros((0, 3))
    trials = 0
    for mol_symbols, local in molecules:
        is_heavy = np.array([s != "H" for s in mol_symbols])
        while True:
            trials += 1
            if trials > max_trials:
                raise RuntimeError("Molecule placement did not converge; lower the density")
            centre = rng.uniform(0.0, box, 3)
            xyz = local @ _rotation(rng).T + centre
            cand = xyz[is_heavy]
            if len(heavy):
                d = cand[:, None, :] - heavy[None, :, :]
                if periodic:
                    d -= box * np.rint(d / box)
                if np.min(np.einsum("abk,abk->ab", d, d)) < min_dist * min_dist:
                    continue
            break
        symbols.extend(mol_symbols)
        coords.append(xyz)
        heavy = np.vstack((heavy, cand))
    return symbols, np.vstack(coords)


def water_cluster(n_mol=64, box=12.0, min_oo=2.6, seed=1, jitter=0.0):
    """Non-periodic rigid-water cluster: oxygens uniform in a cube of side ``box``."""
    rng = np.random.default_rng(seed)
    mols = [_water() for _ in range(n_mol)]
    # Oxygens (not centres of mass) are uniform in the cube: local frame has O at 0.
    symbols, x = _place(rng, mols, box, min_oo, periodic=False)
    if jitter:
        x = x + rng.normal(0.0, jitter, x.shape)
    return System(symbols, x, None, False, 0.0, "ffield.reax.HO.2015")


def water_box(n_mol=1536, box=35.8, min_oo=2.5, seed=2, jitter=0.05):
    """Periodic liquid-density water: 1,536 H2O in a 35.8 A cube by default (1.0 g/cm^3)."""
    rng = np.random.default_rng(seed)
    mols = [_water() for _ in range(n_mol)]
    symbols, x = _place(rng, mols, box, min_oo, periodic=True)
    if jitter:
        x = x + rng.normal(0.0, jitter, x.shape)
    return System(symbols, x, np.diag([box] * 3), True, 0.0, "ffield.reax.HO.2015")


def cho_mixture(counts=(300, 300, 300, 100), density=0.6, min_heavy=2.4, seed=3, jitter=0.05):
    """Periodic CH4 / O2 / H2O / CO2 mixture in a cube sized to ``density`` g/cm^3.

    ``counts`` are the numbers of CH4, O2, H2O and CO2 molecules, placed in a
    seeded random order. 300/300/300/100 molecules give 3,300 atoms.
    """
    rng = np.random.default_rng(seed)
    kinds = ["CH4"] * counts[0] + ["O2"] * counts[1] + ["H2O"] * counts[2] + ["CO2"] * counts[3]
    kinds = [kinds[k] for k in rng.permutation(len(kinds))]
    mols = [MOLECULES[k]() for k in kinds]
    mass = sum(MASS[s] for m in mols for s in m[0])
    box = (mass / (density * AVOGADRO_A3)) ** (1.0 / 3.0)
    symbols, x = _place(rng, mols, box, min_heavy, periodic=True)
    if jitter:
        x = x + rng.normal(0.0, jitter, x.shape)
    return System(symbols, x, np.diag([box] * 3), True, 0.0, "ffield.reax.CHO.2008")


@dataclass
class Request:
    index: int
    arrival: float
    system: System
    repeat_of: int | None = None


def _cluster_of_size(rng, target, ff):
    """Random molecular cluster with about ``target`` atoms (at least one molecule)."""
    if ff == "ffield.reax.HO.2015":
        pool = ["H2O"]
    else:
        pool = ["CH4", "O2", "H2O", "CO2"]
    mols, n = [], 0
    while n < target:
        kind = pool[rng.integers(len(pool))]
        m = MOLECULES[kind]()
        if n and n + len(m[0]) > target + 1:
            break
        mols.append(m)
        n += len(m[0])
    return mols


def request_stream(n_requests=4096, min_atoms=3, max_atoms=512, rate=2000.0, seed=4,
                   periodic_fraction=0.10, charged_fraction=0.01, repeat_fraction=0.25,
                   repeat_jitter=0.01, jitter=0.05):
    """Seeded evaluation-request stream with uneven sizes and Poisson arrivals.

    Sizes are log-uniform on [min_atoms, max_atoms]; force fields alternate
    50/50 between HO.2015 (water clusters) and CHO.2008 (C/H/O clusters);
    ``periodic_fraction`` are cubic cells of 20-30 A; ``charged_fraction`` carry
    a net charge of +-1 e; ``repeat_fraction`` re-evaluate an earlier system with
    Gaussian jitter of ``repeat_jitter`` A (a relaxation step). New systems get
    ``jitter`` A of Gaussian noise on every atom, as the molecular workloads do
    (it also keeps linear CO2 away from exactly collinear torsions).
    """
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_requests))
    out = []
    for k in range(n_requests):
        if out and rng.random() < repeat_fraction:
            src = out[rng.integers(len(out))]
            base = src.system
            x = base.positions + rng.normal(0.0, repeat_jitter, base.positions.shape)
            sys = System(list(base.symbols), x, None if base.cell is None else base.cell.copy(), base.pbc,
                         base.total_charge, base.force_field)
            out.append(Request(k, float(arrivals[k]), sys, src.index if src.repeat_of is None else src.repeat_of))
            continue
        size = int(round(np.exp(rng.uniform(np.log(min_atoms), np.log(max_atoms)))))
        ff = "ffield.reax.HO.2015" if rng.random() < 0.5 else "ffield.reax.CHO.2008"
        mols = _cluster_of_size(rng, size, ff)
        n = sum(len(m[0]) for m in mols)
        periodic = rng.random() < periodic_fraction
        if periodic:
            box = rng.uniform(20.0, 30.0)
        else:
            box = max(4.0, (n * 10.0) ** (1.0 / 3.0))  # roughly liquid density
        symbols, x = _place(rng, mols, box, 2.4, periodic=periodic)
        if jitter:
            x = x + rng.normal(0.0, jitter, x.shape)
        charge = float(rng.choice([-1.0, 1.0])) if rng.random() < charged_fraction else 0.0
        cell = np.diag([box] * 3) if periodic else None
        out.append(Request(k, float(arrivals[k]), System(symbols, x, cell, periodic, charge, ff)))
    return out


def anatase_slab_water(nx=4, ny=4, a=3.785, c=9.514, u=0.2081, gap=15.0, n_water=32, seed=5,
                       displacement=0.0, min_dist=2.2):
    """Anatase TiO2 (001) slab of ``nx x ny x 1`` conventional cells plus water in a vacuum gap.

    Tetragonal anatase (I4_1/amd) with lattice constants ``a``, ``c`` and oxygen
    parameter ``u``: 4 Ti and 8 O per conventional cell, so 4x4x1 gives 192
    atoms. ``n_water`` rigid H2O are placed at random in the gap of height
    ``gap`` above the slab (oxygens at least ``min_dist`` from every heavy atom),
    and the cell is periodic in all three directions. ``displacement`` adds
    seeded Gaussian noise to every atom.
    """
    rng = np.random.default_rng(seed)
    ti_frac = [(0, 0, 0), (0, 0.5, 0.25), (0.5, 0.5, 0.5), (0.5, 0, 0.75)]
    o_frac = []
    for fx, fy, fz in ti_frac:
        o_frac += [(fx, fy, fz + u), (fx, fy, fz - u)]
    symbols, coords = [], []
    for ix in range(nx):
        for iy in range(ny):
            for s, fr in [("Ti", f) for f in ti_frac] + [("O", f) for f in o_frac]:
                fx, fy, fz = fr
                symbols.append(s)
                coords.append(((ix + fx) * a, (iy + fy) * a, (fz % 1.0) * c))
    x = np.array(coords, dtype=float)
    lx, ly, lz = nx * a, ny * a, c + gap
    heavy = x.copy()
    w_symbols, w_local = _water()
    placed = 0
    while placed < n_water:
        centre = np.array([rng.uniform(0, lx), rng.uniform(0, ly), rng.uniform(c + 1.0, c + gap - 1.0)])
        xyz = w_local @ _rotation(rng).T + centre
        d = xyz[0][None, :] - heavy
        d[:, :2] -= np.array([lx, ly]) * np.rint(d[:, :2] / np.array([lx, ly]))
        d[:, 2] -= lz * np.rint(d[:, 2] / lz)
        if np.min(np.einsum("ij,ij->i", d, d)) < min_dist * min_dist:
            continue
        symbols += w_symbols
        x = np.vstack((x, xyz))
        heavy = np.vstack((heavy, xyz[:1]))
        placed += 1
    if displacement:
        x = x + rng.normal(0.0, displacement, x.shape)
    return System(symbols, x, np.diag([lx, ly, lz]), True, 0.0, "ffield.reax.TiOH.Kim2013")


# The parameter groups the differentiation workload perturbs and differentiates: bond (bond energy,
# bond order, over-coordination weight), vdW, and valence-angle records.
BOND_PARAMETERS = ("De_s", "De_p", "De_pp", "p_be1", "p_be2", "p_ovun1", "p_bo1", "p_bo2", "p_bo3", "p_bo4", "p_bo5",
                   "p_bo6")
VDW_PARAMETERS = ("D", "alpha", "gamma_w", "r_vdW")


def perturbed_copies(n_copies=256, seed=5, displacement=0.05, relative=0.02):
    """The differentiation workload: ``n_copies`` copies of the anatase slab with water, each with
    seeded Gaussian displacements of ``displacement`` A and its own uniform +-``relative``
    perturbation of every bond, vdW and angle parameter of ffield.reax.TiOH.Kim2013.

    Yields ``(System, perturbed ForceField)``; the unperturbed force field is the reference.
    """
    import copy

    from .forcefield import ForceField

    base = anatase_slab_water()
    ff0 = ForceField.bundled(base.force_field)
    rng = np.random.default_rng(seed)
    for _ in range(n_copies):
        x = base.positions + rng.normal(0.0, displacement, base.positions.shape)
        ff = copy.deepcopy(ff0)
        seen = set()
        for key, prm in ff.pairs.items():
            if id(prm) in seen:
                continue
            seen.add(id(prm))
            for name in BOND_PARAMETERS + VDW_PARAMETERS:
                if name in prm and prm[name] != 0:
                    prm[name] *= 1.0 + rng.uniform(-relative, relative)
        for records in ff.angles.values():
            for rec in records:
                if id(rec) in seen:
                    continue
                seen.add(id(rec))
                rec *= 1.0 + rng.uniform(-relative, relative, rec.shape)
        yield System(list(base.symbols), x, base.cell.copy(), True, 0.0, base.force_field), ff


def hydrogen_peroxide():
    """H2O2 (O-O 1.475 A, O-H 0.95 A, O-O-H 94.8 deg, H-O-O-H dihedral 111.5 deg)."""
    th, ph = np.deg2rad(94.8), np.deg2rad(111.5)
    o1, o2 = np.array([0.0, 0, 0]), np.array([1.475, 0, 0])
    h1 = o1 + 0.95 * np.array([np.cos(th), np.sin(th), 0.0])
    h2 = o2 + 0.95 * np.array([-np.cos(th), np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph)])
    return System(["H", "O", "O", "H"], np.vstack((h1, o1, o2, h2)), None, False, 0.0, "ffield.reax.HO.2015")
