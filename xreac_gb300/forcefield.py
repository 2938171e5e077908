"""ReaxFF parameter files: parsing, mixing and packing into device tables.

The Python surface mirrors xreac's ``ForceField`` (``src/xreac/forcefield.py:27-341``):
``from_file``, ``bundled``, ``validate_model``, ``vdw_type``, ``elements`` and the
dict views ``general / atoms / pairs / angles / torsions / hydrogen_bonds`` with the
same keys, units and derived values (``eta`` doubled, ``r_vdW`` doubled,
``gamma = (gamma_i gamma_j)^-1.5``, NaN for sign-mismatched ``p_boc*`` mixing,
``0-i-j-0`` torsion wildcards with explicit entries taking precedence).

Beyond the dicts, :meth:`ForceField.tables` packs everything the CUDA kernels read
into flat float64/int32 arrays indexed by element number, so a force field is
uploaded once and shared by every system evaluated with it.
"""

from __future__ import annotations

from dataclasses import dataclass
from hashlib import sha256
from itertools import combinations_with_replacement
from pathlib import Path
import warnings

import numpy as np

# Column names of the 32 per-element values (four lines per element) and of the
# 16 per-bond values (two lines per bond) in the standard ReaxFF format.
# The names are part of the public dict interface and follow xreac's keys
# (src/xreac/forcefield.py:16-24).
ATOM_FIELDS = (
    "r_s valency mass r_vdw epsilon gamma r_pi valency_e "
    "alpha gamma_w valency_boc p_ovun5 unused12 chi eta p_hbond "
    "r_pi_pi p_lp2 heat b_o_131 b_o_132 b_o_133 bcut_acks2 unused23 "
    "p_ovun2 p_val3 unused26 valency_val p_val5 rcore ecore acore"
).split()
BOND_FIELDS = (
    "De_s De_p De_pp p_be1 p_bo5 v13cor p_bo6 p_ovun1 p_be2 p_bo3 p_bo4 unused11 p_bo1 p_bo2 ovc unused15"
).split()

# Pair values derived by mixing two elements' values (src/xreac/forcefield.py:217-244).
_MEAN_MIXED = (("r_s", "r_s"), ("r_p", "r_pi"), ("r_pp", "r_pi_pi"))
_GEOMETRIC_MIXED = (
    ("p_boc3", "b_o_132"),
    ("p_boc4", "b_o_131"),
    ("p_boc5", "b_o_133"),
    ("D", "epsilon"),
    ("alpha", "alpha"),
    ("gamma_w", "gamma_w"),
    ("r_vdW", "r_vdw"),
    ("rcore", "rcore"),
    ("ecore", "ecore"),
    ("acore", "acore"),
)
_OFF_DIAGONAL = ("D", "r_vdW", "alpha", "r_s", "r_p", "r_pp")

# Packed column order of the device pair table (one row per ordered element pair).
PAIR_COLUMNS = (
    "De_s De_p De_pp p_be1 p_be2 p_bo1 p_bo2 p_bo3 p_bo4 p_bo5 p_bo6 p_ovun1 ovc v13cor "
    "r_s r_p r_pp p_boc3 p_boc4 p_boc5 D alpha gamma_w r_vdW rcore ecore acore gamma"
).split()
# Packed column order of the device atom table (one row per element).
ATOM_COLUMNS = (
    "r_s valency mass r_vdw epsilon gamma r_pi valency_e alpha gamma_w valency_boc p_ovun5 chi eta "
    "p_hbond r_pi_pi p_lp2 p_ovun2 p_val3 valency_val p_val5 rcore ecore acore"
).split()


class _Lines:
    """Line cursor with the format's comment rules: text after ``!`` or ``#`` is ignored."""

    def __init__(self, lines):
        self._lines = lines
        self._pos = 0

    def raw(self):
        if self._pos >= len(self._lines):
            raise StopIteration
        self._pos += 1
        return self._lines[self._pos - 1]

    def tokens(self):
        while True:
            fields = self.raw().split("!")[0].split("#")[0].split()
            if fields:
                return fields

    def count(self):
        n = int(self.tokens()[0])
        if n < 0:
            raise ValueError("Negative section count")
        return n

    def remaining_tokens(self):
        return any(line.split("!")[0].split("#")[0].strip() for line in self._lines[self._pos :])


def _numbers(tokens, n):
    if len(tokens) != n:
        raise ValueError(f"Expected {n} parameters, received {len(tokens)}")
    values = np.array([float(t.replace("D", "E").replace("d", "e")) for t in tokens])
    if not np.isfinite(values).all():
        raise ValueError("Non-finite force-field parameters")
    return values


@dataclass(frozen=True)
class ForceField:
    """Parsed ReaxFF parameters; dict views match xreac's ``ForceField``."""

    path: Path
    checksum: str
    citation: str
    general: np.ndarray
    atoms: dict
    pairs: dict
    angles: dict
    torsions: dict
    hydrogen_bonds: dict

    # ------------------------------------------------------------------ loading
    @classmethod
    def bundled(cls, name):
        """Load a parameter file shipped in this package's ``data`` directory.

        Mirrors ``ForceField.bundled`` (src/xreac/forcefield.py:84-95).
        """
        if not isinstance(name, str) or Path(name).name != name or name in ("", ".", ".."):
            raise ValueError("A bundled parameter name must be a plain filename")
        return cls.from_file(Path(__file__).resolve().with_name("data") / name)

    @classmethod
    def from_file(cls, path):
        """Read a standard ReaxFF file (39 general parameters, four-line atoms).

        Semantics follow src/xreac/forcefield.py:120-315; malformed files raise
        ``ValueError`` and unreadable ones the operating system's error.
        """
        path = Path(path).resolve()
        raw = path.read_bytes()
        lines = raw.decode().splitlines()
        if not lines:
            raise ValueError(f"Empty ReaxFF parameter file: {path}")
        citation = lines[0]
        cur = _Lines(lines[1:])
        try:
            general = cls._read_general(cur)
            atoms, names = cls._read_atoms(cur)
            pairs = cls._read_bonds(cur, names)
            cls._mix_pairs(pairs, atoms, names)
            cls._read_off_diagonal(cur, pairs, names)
            angles = cls._read_angles(cur, names)
            torsions = cls._read_torsions(cur, names)
            hbonds = cls._read_hbonds(cur, names)
            if cur.remaining_tokens():
                raise ValueError("Unsupported trailing parameter section")
        except (StopIteration, IndexError, ValueError) as exc:
            raise ValueError(f"Invalid or unsupported ReaxFF file {path}: {exc}") from exc
        return cls(path, sha256(raw).hexdigest(), citation, general, atoms, pairs, angles, torsions, hbonds)

    @staticmethod
    def _index_labels(tokens, names, wildcard=False):
        labels = []
        for token in tokens:
            k = int(token)
            if wildcard and k == 0:
                labels.append("*")
            elif 1 <= k <= len(names):
                labels.append(names[k - 1])
            else:
                raise ValueError("Invalid element index")
        return tuple(labels)

    @staticmethod
    def _read_general(cur):
        if cur.count() != 39:
            raise ValueError("Only the standard 39-global-parameter format is supported")
        return np.array([_numbers(cur.tokens()[:1], 1)[0] for _ in range(39)])

    @staticmethod
    def _read_atoms(cur):
        n = cur.count()
        if n == 0:
            raise ValueError("A force field must define at least one atom type")
        for _ in range(3):  # three free-text header lines, read verbatim
            cur.raw()
        atoms, names = {}, []
        for _ in range(n):
            head = cur.tokens()
            name = head[0]
            if any(name.casefold() == other.casefold() for other in atoms):
                raise ValueError(f"Duplicate element {name}")
            values = _numbers(head[1:] + cur.tokens() + cur.tokens() + cur.tokens(), 32)
            entry = dict(zip(ATOM_FIELDS, values))
            entry["eta"] *= 2
            entry["p_hbond"] = int(entry["p_hbond"])
            if entry["mass"] < 21:
                entry["valency_val"] = entry["valency_boc"]
            atoms[name] = entry
            names.append(name)
        return atoms, names

    @classmethod
    def _read_bonds(cls, cur, names):
        n = cur.count()
        cur.raw()  # second free-text header line
        pairs = {}
        for _ in range(n):
            head = cur.tokens()
            key = cls._index_labels(head[:2], names)
            tail = cur.tokens()
            if len(tail) == 7:  # the trailing unused value may be omitted
                tail.append("0")
            entry = dict(zip(BOND_FIELDS, _numbers(head[2:] + tail, 16)))
            pairs[key] = pairs[key[::-1]] = entry
        return pairs

    @staticmethod
    def _mix_pairs(pairs, atoms, names):
        """Nonbonded and bond-order mixing for every element pair, bonded or not."""
        for s, t in combinations_with_replacement(names, 2):
            entry = pairs.get((s, t), dict.fromkeys(BOND_FIELDS, 0.0))
            a, b = atoms[s], atoms[t]
            for out, col in _MEAN_MIXED:
                entry[out] = (a[col] + b[col]) / 2
            for out, col in _GEOMETRIC_MIXED:
                product = a[col] * b[col]
                if product < 0:
                    if not out.startswith("p_boc"):
                        raise ValueError(f"Invalid mixing parameters for {s}/{t}: {col}")
                    entry[out] = np.nan  # checked where an active correction uses it
                else:
                    entry[out] = np.sqrt(product)
            entry["r_vdW"] *= 2
            if a["gamma"] * b["gamma"] <= 0:
                raise ValueError("Charge shielding parameters must be positive")
            entry["gamma"] = (a["gamma"] * b["gamma"]) ** -1.5
            pairs[(s, t)] = pairs[(t, s)] = entry

    @classmethod
    def _read_off_diagonal(cls, cur, pairs, names):
        for _ in range(cur.count()):
            tokens = cur.tokens()
            key = cls._index_labels(tokens[:2], names)
            values = _numbers(tokens[2:], 6)
            if key not in pairs:
                raise ValueError("Off-diagonal entry without bond parameters")
            for col, value in zip(_OFF_DIAGONAL, values):
                if value > 0:
                    pairs[key][col] = value * (2 if col == "r_vdW" else 1)

    @classmethod
    def _read_angles(cls, cur, names):
        angles = {}
        for _ in range(cur.count()):
            tokens = cur.tokens()
            key = cls._index_labels(tokens[:3], names)
            values = _numbers(tokens[3:], 7)
            for k in {key, key[::-1]}:
                angles.setdefault(k, []).append(values)
        return angles

    @classmethod
    def _read_torsions(cls, cur, names):
        torsions, explicit = {}, set()
        for _ in range(cur.count()):
            tokens = cur.tokens()
            key = cls._index_labels(tokens[:4], names, wildcard=True)
            if len(tokens) - 4 not in (5, 6, 7):
                raise ValueError("Expected 5 to 7 torsion parameters")
            values = _numbers(tokens[4:], len(tokens) - 4)[:5]
            if "*" not in key:
                torsions[key] = torsions[key[::-1]] = values
                explicit.update((key, key[::-1]))
                continue
            if key[0] != "*" or key[3] != "*" or "*" in key[1:3]:
                raise ValueError("Only terminal 0-i-j-0 torsion wildcards are supported")
            # Explicit rows always win; a later wildcard replaces an earlier one.
            for s in names:
                for t in names:
                    full = (s, key[1], key[2], t)
                    for k in (full, full[::-1]):
                        if k not in explicit:
                            torsions[k] = values
        return torsions

    @classmethod
    def _read_hbonds(cls, cur, names):
        try:
            n = cur.count()
        except StopIteration:
            return {}  # the final hydrogen-bond block may be omitted
        hbonds = {}
        for _ in range(n):
            tokens = cur.tokens()
            hbonds[cls._index_labels(tokens[:3], names)] = _numbers(tokens[3:], 4)
        return hbonds

    # ----------------------------------------------------------------- checking
    @property
    def elements(self):
        """Parameter-file atom labels in file order (dummy types included)."""
        return tuple(self.atoms)

    @property
    def vdw_type(self):
        """LAMMPS vdW variant: 1 shielded, 2 inner wall, 3 both (src/xreac/forcefield.py:102-118)."""
        kinds = []
        for a in self.atoms.values():
            shielded = a["gamma_w"] > 0.5
            core = a["rcore"] > 0.01 and a["acore"] > 0.01
            kinds.append(3 if shielded and core else 1 if shielded else 2 if core else 0)
        if not kinds or 0 in kinds:
            raise ValueError("Inconsistent or unsupported van der Waals method across atom types")
        if len(set(kinds)) != 1:
            warnings.warn(
                "Mixed van der Waals methods; using the first atom type's method, as LAMMPS does",
                RuntimeWarning,
                stacklevel=2,
            )
        return kinds[0]

    def validate_model(self, elements=None):
        """Reject models outside the implemented equations (src/xreac/forcefield.py:317-341)."""
        if elements is not None:
            key = frozenset(elements)
            validated = self.__dict__.setdefault("_validated_elements", set())
            if key in validated:
                return
            self.validate_model(None)
            self._validate_elements(key)
            validated.add(key)
            return
        self.vdw_type
        g = self.general
        if g[11] != 0 or g[12] <= 0:
            raise ValueError("Only zero lower taper radius and a positive upper cutoff are supported")
        if g[1] <= 0 or g[28] <= 0 or g[29] <= 0:
            raise ValueError("Invalid bond-order correction, vdW exponent, or bond-order cutoff")

    def _validate_elements(self, elements):
        missing = set(elements) - self.atoms.keys()
        if missing:
            raise ValueError(f"Atom types absent from the force field: {', '.join(sorted(missing))}")
        present = set(elements)
        for s in present:
            a = self.atoms[s]
            if a["eta"] <= 0 or a["gamma"] <= 0:
                raise ValueError("Invalid QEq hardness or shielding")
            if a["mass"] <= 0 or a["valency"] < 0:
                raise ValueError("Positive atomic masses and nonnegative valencies are required")
            for t in present:
                p = self.pairs[s, t]
                if p["r_vdW"] <= 0:
                    raise ValueError(f"Invalid van der Waals radius for {s}/{t}")
                for atom_radius, pair_radius in (("r_s", "r_s"), ("r_pi", "r_p"), ("r_pi_pi", "r_pp")):
                    if a[atom_radius] > 0 and self.atoms[t][atom_radius] > 0 and p[pair_radius] <= 0:
                        raise ValueError(f"Invalid {pair_radius} for {s}/{t}")

    # ------------------------------------------------------------------ packing
    def tables(self):
        """Flat arrays for the device, indexed by element number in file order.

        Returns a dict of contiguous numpy arrays:

        - ``general`` (39,) float64
        - ``atom`` (T, len(ATOM_COLUMNS)) float64
        - ``pair`` (T*T, len(PAIR_COLUMNS)) float64, row ``s*T+t``
        - ``angle_index`` (T**3, 2) int32 ``(first, count)`` into ``angle`` (R, 7)
        - ``torsion_index`` (T**4,) int32 row of ``torsion`` (Q, 5) or -1; only
          entries with a nonzero V1, V2, V3 or V_conj are kept (as
          src/xreac/energy.py:84-87 does)
        - ``hbond_index`` (T**3,) int32 row of ``hbond`` (H, 4) or -1
        """
        names = self.elements
        T = len(names)
        pos = {s: k for k, s in enumerate(names)}
        atom = np.array([[float(self.atoms[s][c]) for c in ATOM_COLUMNS] for s in names])
        pair = np.array([[float(self.pairs[s, t][c]) for c in PAIR_COLUMNS] for s in names for t in names])
        angle_index = np.zeros((T**3, 2), dtype=np.int32)
        angle_rows = []
        for (a, b, c), records in self.angles.items():
            k = (pos[a] * T + pos[b]) * T + pos[c]
            angle_index[k] = (len(angle_rows), len(records))
            angle_rows.extend(records)
        # torsion records in dict order; only those with a nonzero V1, V2, V3 or V_conj get a row
        torsion_index = np.full(T**4, -1, dtype=np.int32)
        torsion_rows = np.zeros((0, 5))
        if self.torsions:
            vals = np.array([np.asarray(v, dtype=np.float64).reshape(5) for v in self.torsions.values()])
            where = np.array([((pos[a] * T + pos[b]) * T + pos[c]) * T + pos[d] for a, b, c, d in self.torsions])
            keep = np.any(vals[:, [0, 1, 2, 4]] != 0, axis=1)
            torsion_index[where[keep]] = np.arange(int(keep.sum()), dtype=np.int32)
            torsion_rows = vals[keep]
        hbond_index = np.full(T**3, -1, dtype=np.int32)
        hbond_rows = np.zeros((0, 4))
        if self.hydrogen_bonds:
            hbond_rows = np.array([np.asarray(v, dtype=np.float64).reshape(4) for v in self.hydrogen_bonds.values()])
            where = np.array([(pos[a] * T + pos[b]) * T + pos[c] for a, b, c in self.hydrogen_bonds])
            hbond_index[where] = np.arange(len(where), dtype=np.int32)
        return dict(
            general=np.ascontiguousarray(self.general, dtype=np.float64),
            atom=np.ascontiguousarray(atom),
            pair=np.ascontiguousarray(pair),
            angle_index=angle_index,
            angle=np.ascontiguousarray(np.array(angle_rows, dtype=np.float64).reshape(-1, 7)),
            torsion_index=torsion_index,
            torsion=np.ascontiguousarray(np.array(torsion_rows, dtype=np.float64).reshape(-1, 5)),
            hbond_index=hbond_index,
            hbond=np.ascontiguousarray(np.array(hbond_rows, dtype=np.float64).reshape(-1, 4)),
            ntypes=T,
        )

    def angle_row_keys(self):
        """``(key, record index)`` of every row of ``tables()["angle"]``, in row order."""
        return [(key, q) for key, records in self.angles.items() for q in range(len(records))]

    def type_indices(self, symbols):
        """Element numbers (file order) of a sequence of labels, as int32."""
        pos = self.__dict__.get("_type_pos")
        if pos is None:
            pos = self.__dict__["_type_pos"] = {s: k for k, s in enumerate(self.elements)}
        return np.fromiter((pos[s] for s in symbols), dtype=np.int32, count=len(symbols))
