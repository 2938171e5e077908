"""Write golden fixtures by running the UNMODIFIED xreac reference (v0.10.0) in this container.

Usage (needs the reference checkout; not run by the test suite):

    python tests/golden/make_golden.py <path of the xreac v0.10.0 checkout> [case ...]

The reference depends on HIPS ``autograd``, which is not installed here, so the
torch-backed stand-in in ``tests/golden/shim`` goes first on ``sys.path``. With
it, ``xreac.Calculator.evaluate`` runs unchanged: energies and charges come from
numpy, forces from the reference's own derivative graph replayed by
``torch.autograd``.

For every case the script records the inputs, the reference's ``Evaluation``
fields, its canonical neighbour list ``(i, j, S)`` and its per-edge corrected
bond orders, into one compressed ``<case>.npz``. It also records the parsed
parameter dicts of the bundled force fields (``forcefields.json``) so the parser
can be checked without the reference present.

Cases: the reference's own test geometries (imported from its ``examples/`` and
``tests/``), small versions of the benchmark workloads generated with
``xreac_gb300.workloads`` (the 192-atom water cluster is the full-size cluster
workload), a few request-stream samples, and caller-supplied neighbour lists
(``supplied_*``: skin lists and thinned lists in shuffled order, whose lists are
stored as ``sup_i``, ``sup_j``, ``sup_S``).
"""

from __future__ import annotations

import hashlib
import json
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]


def _setup(reference):
    reference = Path(reference)
    for p in (REPO, reference / "tests", reference / "examples", reference / "src", HERE / "shim"):
        sys.path.insert(0, str(p))


def reference_cases():
    """Geometries of the reference's own tests (examples/*.py and tests/cases.py)."""
    from cases import CASES  # tests/cases.py
    from periodic_water import periodic_cases
    from small_cells import small_cell_cases
    from water_cluster import water_cases

    out = {}
    water = water_cases()
    for name, (s, x) in water.items():
        out["water_" + name] = ("ffield.reax.HO.2015", s, x, None, None, 0.0)
    for name, (s, x, cell, pbc) in periodic_cases(include_bulk=True).items():
        out["periodic_" + name] = ("ffield.reax.HO.2015", s, x, cell, pbc, 0.0)
    for name, (ff, s, x, cell, pbc) in small_cell_cases().items():
        out["small_" + name] = (ff, s, x, cell, pbc, 0.0)
    for name, (s, x) in CASES.items():
        out["zno_" + name] = ("ffield.reax.ZnOH.2010", s, np.asarray(x, dtype=float), None, None, 0.0)
    methane = np.vstack(([0, 0, 0], 0.63 * np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]])))
    out["carbon_methane"] = ("ffield.reax.CHO.2008", ["C"] + ["H"] * 4, methane, None, None, 0.0)
    out["carbon_monoxide"] = ("ffield.reax.CHO.2008", ["C", "O"], np.array([[0.0, 0, 0], [1.15, 0, 0]]), None, None, 0.0)
    out["carbon_dimer"] = ("ffield.reax.CHO.2008", ["C", "C"], np.array([[0.0, 0, 0], [1.2, 0, 0]]), None, None, 0.0)
    out["periodic_carbon_chain"] = (
        "ffield.reax.CHO.2008",
        ["C"] * 3,
        np.array([[0.0, 0, 0], [1.5, 0.4, 0.2], [3.0, -0.2, 0.8]]),
        np.diag([4.5, 12.0, 12.0]),
        [True, False, False],
        0.0,
    )
    s, x = water["monomer"]
    out["charged_hydroxide"] = ("ffield.reax.HO.2015", s[:2], x[:2].copy(), None, None, -1.0)
    out["charged_hydronium"] = ("ffield.reax.HO.2015", s + ["H"], np.vstack((x, [-0.3, -0.45, 0.85])), None, None, 1.0)
    ff, s, x, cell, pbc = small_cell_cases()["water_4A"]
    out["charged_water_4A"] = (ff, s, x, cell, pbc, -1.0)
    return out


def workload_cases():
    """Seeded systems shaped like the benchmark workloads."""
    from xreac_gb300 import workloads as w

    out = {}

    def add(name, sys_):
        out[name] = (sys_.force_field, list(sys_.symbols), sys_.positions, sys_.cell, sys_.pbc, sys_.total_charge)

    add("cluster_water_192", w.water_cluster())  # the full 64-H2O cluster workload
    add("box_water_192", w.water_box(n_mol=64, box=12.42, seed=2))
    # Periodic heights above twice the cutoff: only the nearest image of a pair can be in range.
    add("box_water_1536", w.water_box(n_mol=512, box=24.82, seed=2))
    add("box_cho_89", w.cho_mixture(counts=(8, 8, 8, 3), seed=3))
    add("peroxide", w.hydrogen_peroxide())
    add("anatase_water_288", w.anatase_slab_water(displacement=0.05))
    stream = w.request_stream(n_requests=48, seed=4, periodic_fraction=0.2, charged_fraction=0.1)
    picked = [r for r in stream if r.system.n <= 160][:8]
    for r in picked:
        add(f"stream_{r.index:02d}", r.system)
    # A 342-atom C/H/O cluster of the serving stream whose QEq matrix has one negative eigenvalue:
    # the reference's direct KKT solve accepts it, so an iterative solver must too.
    add("stream_indefinite_qeq", w.request_stream(n_requests=120)[39].system)
    return out


def supplied_cases(cases):
    """Caller-supplied neighbour lists, built with the reference's own replicated_neighbors at a larger
    cutoff (a skin list: the result must equal the replicated one) or thinned (a partial list: the
    result must follow the list, not the geometry), and handed over in a shuffled order."""
    from xreac.neighbors import replicated_neighbors

    rng = np.random.default_rng(8)
    out = {}

    def shuffled(i, j, S):
        order = rng.permutation(len(i))
        return i[order], j[order], S[order]

    def half_mask(i, j, S):
        neg = (S[:, 0] < 0) | ((S[:, 0] == 0) & ((S[:, 1] < 0) | ((S[:, 1] == 0) & (S[:, 2] < 0))))
        return (i < j) | ((i == j) & neg)

    def thinned(i, j, S, keep_half):
        """Keep the half edges where keep_half, and with each its reverse."""
        half = half_mask(i, j, S)
        kept = {(int(a), int(b), *map(int, s)) for a, b, s, h, k in zip(i, j, S, half, keep_half) if h and k}
        keep = np.array([((int(a), int(b), *map(int, s)) in kept) if h else
                         ((int(b), int(a), *(-int(v) for v in s)) in kept) for a, b, s, h in zip(i, j, S, half)])
        return i[keep], j[keep], S[keep]

    def distances(x, i, j, S, cell):
        lat = np.eye(3) if cell is None else np.asarray(cell, dtype=float)
        v = x[j] - x[i] + S @ lat
        return np.sqrt(np.sum(v * v, axis=1))

    for base in ("small_water_4A", "periodic_carbon_chain", "cluster_water_192"):
        ff_name, s, x, cell, pbc, charge = cases[base]
        x = np.asarray(x, dtype=float)
        from xreac import ForceField

        rc = float(ForceField.bundled(ff_name).general[12])
        (i, j, S), _ = replicated_neighbors(x, rc + 1.0, cell, pbc, max_expanded_atoms=100000)
        out[f"supplied_skin_{base}"] = (ff_name, s, x, cell, pbc, charge, shuffled(i, j, S))
        r = distances(x, i, j, S, cell)
        if base == "cluster_water_192":
            # drop about half of the pairs beyond 2.5 A (H-bond acceptors, vdW and Coulomb partners)
            keep = (r <= 2.5) | (rng.random(len(i)) < 0.5)
        else:
            keep = r <= 6.0  # only the pairs within 6 A
        out[f"supplied_partial_{base}"] = (ff_name, s, x, cell, pbc, charge, shuffled(*thinned(i, j, S, keep)))
    return out


def _ff_to_json(ff):
    def num(v):
        return [float(t) for t in np.asarray(v).ravel()]

    return dict(
        checksum=ff.checksum,
        citation=ff.citation,
        general=num(ff.general),
        atoms={s: {k: float(v) for k, v in a.items()} for s, a in ff.atoms.items()},
        pairs={f"{s}|{t}": {k: float(v) for k, v in p.items()} for (s, t), p in ff.pairs.items()},
        angles={"|".join(k): [num(r) for r in v] for k, v in ff.angles.items()},
        torsions={"|".join(k): num(v) for k, v in ff.torsions.items()},
        hydrogen_bonds={"|".join(k): num(v) for k, v in ff.hydrogen_bonds.items()},
        vdw_type=ff.vdw_type,
        elements=list(ff.elements),
    )


def run_case(name, ff_name, symbols, x, cell, pbc, charge, full_derivative=False, neighbors=None):
    import xreac
    from xreac.energy import EnergyModel
    from xreac.neighbors import replicated_neighbors

    ff = xreac.ForceField.bundled(ff_name)
    calc = xreac.Calculator(ff)
    t0 = time.time()
    res = calc.evaluate(symbols, x, cell=cell, pbc=pbc, total_charge=charge, full_derivative=full_derivative,
                        neighbors=neighbors)
    elapsed = time.time() - t0
    # Per-edge quantities from the pure-numpy forward pass of the same model.
    if neighbors is None:
        (nb, _) = replicated_neighbors(np.asarray(x, float), ff.general[12], cell, pbc)
    else:
        nb = neighbors
    model = EnergyModel(ff, symbols, nb, cell, pbc, total_charge=charge)
    _, r = model.edges.geometry(np.asarray(x, float))
    q = model.electrostatics(r)[0]
    comps, _, (bo, total, nlp) = model.components(np.asarray(x, float), q, return_bond_state=True)
    n = len(symbols)
    nz = np.flatnonzero(bo)
    canon = np.column_stack((model.edges.i, model.edges.j, model.edges.shifts)).astype(np.int32)
    data = dict(
        ff=np.array(ff_name),
        symbols=np.array(symbols),
        positions=np.asarray(x, dtype=float),
        cell=np.zeros((0, 3)) if cell is None else np.asarray(cell, dtype=float).reshape(-1, 3),
        pbc=np.broadcast_to(np.asarray(pbc if pbc is not None else cell is not None, dtype=bool), (3,)).copy(),
        total_charge=np.array(float(charge)),
        full_derivative=np.array(bool(full_derivative)),
        energy=np.array(res.energy),
        energy_numpy=np.array(float(np.sum(comps))),
        components=np.array([res.components[k] for k in xreac.energy.COMPONENTS]),
        forces=res.forces,
        charges=res.charges,
        total_bond_orders=res.total_bond_orders,
        lone_pairs=res.lone_pairs,
        bond_counts=res.bond_counts,
        dipole=res.dipole,
        cell_repetitions=np.array(res.cell_repetitions),
        edge_count=np.array(len(canon)),
        edge_sha256=np.array(hashlib.sha256(np.ascontiguousarray(canon).tobytes()).hexdigest()),
        bo_value=bo[nz],
        seconds=np.array(elapsed),
        neighbor_backend=np.array(res.neighbor_backend),
    )
    if neighbors is not None:  # the list as handed over (not canonical; edges beyond the cutoff included)
        data.update(sup_i=np.asarray(neighbors[0], dtype=np.int32), sup_j=np.asarray(neighbors[1], dtype=np.int32),
                    sup_S=np.asarray(neighbors[2], dtype=np.int32))
    if len(canon) <= 100_000:  # small lists are stored in full; large ones by count and hash
        data.update(edge_i=canon[:, 0], edge_j=canon[:, 1], edge_S=canon[:, 2:].astype(np.int8), bo_index=nz.astype(np.int32))
    else:
        data.update(bo_i=canon[nz, 0], bo_j=canon[nz, 1], bo_S=canon[nz, 2:].astype(np.int8))
    if n <= 200:
        data["bond_orders"] = res.bond_orders
    np.savez_compressed(HERE / f"{name}.npz", **data)
    return elapsed, len(model.edges.i)


def main(reference, only=None):
    _setup(reference)
    import xreac

    ffs = {}
    for name in ("ffield.reax.HO.2015", "ffield.reax.CHO.2008", "ffield.reax.ZnOH.2010", "ffield.reax.TiOH.Kim2013"):
        ffs[name] = _ff_to_json(xreac.ForceField.bundled(name))
    (HERE / "forcefields.json").write_text(json.dumps(ffs, sort_keys=True))
    cases = reference_cases()
    cases.update(workload_cases())
    for name, (ff_name, s, x, cell, pbc, charge) in cases.items():
        if only and name not in only:
            continue
        dt, m = run_case(name, ff_name, list(s), x, cell, pbc, charge)
        print(f"{name:28s} n={len(s):4d} edges={m:7d} {dt:6.2f} s", flush=True)
    for name, (ff_name, s, x, cell, pbc, charge, nb) in supplied_cases(cases).items():
        if only and name not in only:
            continue
        dt, m = run_case(name, ff_name, list(s), x, cell, pbc, charge, neighbors=nb)
        print(f"{name:28s} n={len(s):4d} edges={m:7d} {dt:6.2f} s (supplied list)", flush=True)
    for name in ("water_distorted_dimer", "zno_cluster20", "small_water_4A", "carbon_methane"):
        if only and name + "_full" not in only:
            continue
        ff_name, s, x, cell, pbc, charge = cases[name]
        run_case(name + "_full", ff_name, list(s), x, cell, pbc, charge, full_derivative=True)
        print(f"{name + '_full':28s} (charge-response forces)", flush=True)


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference checkout> [case ...]")
    main(sys.argv[1], set(sys.argv[2:]) or None)
