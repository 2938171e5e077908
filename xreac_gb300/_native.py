"""ctypes bindings of the C ABI declared in include/xreac_gb300.h.

The library is built in-tree (``python -m xreac_gb300.build``). There is no CPU fallback: when the
library or a GPU is missing, loading fails with an error that says so.
"""

from __future__ import annotations

import ctypes
from ctypes import POINTER, byref, c_char_p, c_double, c_int, c_longlong, c_uint, c_void_p
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libxreac_gb300.so"

XR_OK = 0
XR_EINPUT = 1
XR_ECOINCIDENT = 2
XR_ESINGULAR = 3
XR_ENONFINITE = 4
XR_ECHARGE = 5
XR_ECOLLINEAR = 6
XR_ECAPACITY = 7
XR_EBADPARAM = 8
XR_ECUDA = 9
XR_EUNSUPPORTED = 10
XR_ECG_NOCONV = 11
XR_EWAIT = 12

XR_FLAG_FULL_DERIVATIVE = 1
XR_FLAG_DEVICE_IO = 2
XR_FLAG_PARAM_GRADIENT = 4
XR_FLAG_QEQ_GRADIENT = 8

EXPORTED = (
    "xr_ff_create",
    "xr_ff_destroy",
    "xr_ff_update",
    "xr_ff_set_count",
    "xr_ff_set_count_of",
    "xr_ff_update_sets",
    "xr_ctx_create",
    "xr_ctx_destroy",
    "xr_last_error",
    "xr_ctx_set_qeq",
    "xr_ctx_reserve",
    "xr_ctx_set_wait_test",
    "xr_test_math",
    "xr_eval",
    "xr_eval_batch",
    "xr_eval_batch_sets",
    "xr_eval_neighbors",
    "xr_neighbors_check",
    "xr_ctx_set_skin",
    "xr_ctx_set_cell_list",
    "xr_ctx_set_graphs",
    "xr_last_graph",
    "xr_last_list_info",
    "xr_get_neighbors",
    "xr_get_bonds",
    "xr_last_launches",
    "xr_last_list_sizes",
    "xr_ctx_set_profiling",
    "xr_ctx_stage_times",
    "xr_last_transfer_bytes",
    "xr_last_qeq_iterations",
    "xr_last_qeq_work",
    "xr_get_param_gradient",
    "xr_get_param_gradient_system",
    "xr_get_param_gradient_blocks",
    "xr_get_param_gradient_atoms",
    "xr_ctx_memory",
    "xr_footprint_bytes",
    "xr_count_neighbors_static",
    "xr_static_last_error",
)

XR_STATIC_MAX_ATOMS = 16384
XR_MAX_PARAMETER_SETS = 65536


# Pointer members are declared as void* (the C layout is the same); assign addresses with addr().
class System(ctypes.Structure):
    _fields_ = [
        ("natoms", c_int),
        ("types", c_void_p),          # const int*
        ("positions", c_void_p),      # const double*, natoms x 3
        ("cell", c_void_p),           # const double*, 9 or NULL
        ("pbc", c_int * 3),
        ("total_charge", c_double),
        ("charges_guess", c_void_p),  # const double* or NULL
    ]


class Neighbors(ctypes.Structure):
    _fields_ = [
        ("count", c_longlong),
        ("i", c_void_p),  # const int*, count
        ("j", c_void_p),  # const int*, count
        ("S", c_void_p),  # const int*, count x 3
    ]


class Result(ctypes.Structure):
    _fields_ = [
        ("energy", c_void_p),             # double[15]
        ("forces", c_void_p),             # double[natoms * 3]
        ("charges", c_void_p),            # double[natoms]
        ("total_bond_orders", c_void_p),  # double[natoms]
        ("lone_pairs", c_void_p),         # double[natoms]
        ("bond_counts", c_void_p),        # int[natoms]
        ("dipole", c_void_p),             # double[3]
    ]


_LIB = None


def load():
    """Load the CUDA library; raises if it was not built (no CPU fallback exists)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not LIB_PATH.exists():
        raise RuntimeError(
            f"xreac_gb300 CUDA library not found at {LIB_PATH}; build it with `python -m xreac_gb300.build`"
        )
    lib = ctypes.CDLL(str(LIB_PATH))
    lib.xr_ff_create.argtypes = [
        POINTER(c_double), c_int, POINTER(c_double), POINTER(c_double), POINTER(c_int), c_int,
        POINTER(c_int), POINTER(c_double), c_int, POINTER(c_int), POINTER(c_double), c_int,
        POINTER(c_int), POINTER(c_double), c_int, POINTER(c_void_p),
    ]
    lib.xr_ff_create.restype = c_int
    lib.xr_ff_update.argtypes = [
        c_void_p, POINTER(c_double), POINTER(c_double), POINTER(c_double), POINTER(c_int), c_int, POINTER(c_int),
        POINTER(c_double), POINTER(c_int), POINTER(c_double), POINTER(c_int), POINTER(c_double),
    ]
    lib.xr_ff_update.restype = c_int
    lib.xr_ff_set_count.argtypes = [c_void_p, c_int]
    lib.xr_ff_set_count.restype = c_int
    lib.xr_ff_set_count_of.argtypes = [c_void_p]
    lib.xr_ff_set_count_of.restype = c_int
    lib.xr_ff_update_sets.argtypes = [c_void_p, c_int, c_int, POINTER(c_double), POINTER(c_double), POINTER(c_double),
                                      POINTER(c_double), POINTER(c_double)]
    lib.xr_ff_update_sets.restype = c_int
    lib.xr_ff_destroy.argtypes = [c_void_p]
    lib.xr_ff_destroy.restype = None
    lib.xr_ctx_create.argtypes = [c_int, c_void_p, POINTER(c_void_p)]
    lib.xr_ctx_create.restype = c_int
    lib.xr_ctx_destroy.argtypes = [c_void_p]
    lib.xr_ctx_destroy.restype = None
    lib.xr_last_error.argtypes = [c_void_p]
    lib.xr_last_error.restype = c_char_p
    lib.xr_ctx_set_qeq.argtypes = [c_void_p, c_double, c_int]
    lib.xr_ctx_set_qeq.restype = c_int
    lib.xr_ctx_reserve.argtypes = [c_void_p, c_int, c_int, c_longlong, c_longlong]
    lib.xr_ctx_reserve.restype = c_int
    lib.xr_ctx_set_wait_test.argtypes = [c_void_p, c_longlong, c_int]
    lib.xr_ctx_set_wait_test.restype = c_int
    lib.xr_test_math.argtypes = [c_int, c_void_p, c_void_p, c_int]
    lib.xr_test_math.restype = c_int
    lib.xr_eval.argtypes = [c_void_p, c_void_p, POINTER(System), c_uint, POINTER(Result)]
    lib.xr_eval.restype = c_int
    lib.xr_eval_batch.argtypes = [c_void_p, c_void_p, c_int, POINTER(System), c_uint, POINTER(Result)]
    lib.xr_eval_batch.restype = c_int
    lib.xr_eval_batch_sets.argtypes = [c_void_p, c_void_p, c_int, POINTER(System), POINTER(c_int), c_uint,
                                       POINTER(Result)]
    lib.xr_eval_batch_sets.restype = c_int
    lib.xr_eval_neighbors.argtypes = [c_void_p, c_void_p, POINTER(System), POINTER(Neighbors), c_uint, POINTER(Result)]
    lib.xr_eval_neighbors.restype = c_int
    lib.xr_neighbors_check.argtypes = [c_int, POINTER(c_int), POINTER(Neighbors), c_char_p, c_int]
    lib.xr_neighbors_check.restype = c_int
    lib.xr_ctx_set_skin.argtypes = [c_void_p, c_double]
    lib.xr_ctx_set_skin.restype = c_int
    lib.xr_ctx_set_cell_list.argtypes = [c_void_p, c_int]
    lib.xr_ctx_set_cell_list.restype = c_int
    lib.xr_ctx_set_graphs.argtypes = [c_void_p, c_int]
    lib.xr_ctx_set_graphs.restype = c_int
    lib.xr_last_graph.argtypes = [c_void_p]
    lib.xr_last_graph.restype = c_int
    lib.xr_last_list_info.argtypes = [c_void_p, POINTER(c_int), POINTER(c_longlong)]
    lib.xr_last_list_info.restype = c_int
    lib.xr_get_neighbors.argtypes = [c_void_p, c_int, POINTER(c_int), POINTER(c_int), POINTER(c_int), c_longlong,
                                     POINTER(c_longlong)]
    lib.xr_get_neighbors.restype = c_int
    lib.xr_get_bonds.argtypes = [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_longlong,
                                 POINTER(c_longlong)]  # i, j, S, bo: int*, int*, int*, double*
    lib.xr_get_bonds.restype = c_int
    lib.xr_last_launches.argtypes = [c_void_p]
    lib.xr_last_launches.restype = c_longlong
    lib.xr_last_list_sizes.argtypes = [c_void_p, POINTER(c_longlong), c_int]
    lib.xr_last_list_sizes.restype = c_int
    lib.xr_ctx_set_profiling.argtypes = [c_void_p, c_int]
    lib.xr_ctx_set_profiling.restype = c_int
    lib.xr_ctx_stage_times.argtypes = [c_void_p, POINTER(c_double), c_int, POINTER(c_longlong)]
    lib.xr_ctx_stage_times.restype = c_int
    lib.xr_last_transfer_bytes.argtypes = [c_void_p, POINTER(c_longlong), POINTER(c_longlong)]
    lib.xr_last_transfer_bytes.restype = c_int
    lib.xr_last_qeq_iterations.argtypes = [c_void_p]
    lib.xr_last_qeq_iterations.restype = c_int
    lib.xr_last_qeq_work.argtypes = [c_void_p, POINTER(c_longlong), POINTER(c_double)]
    lib.xr_last_qeq_work.restype = c_int
    lib.xr_get_param_gradient.argtypes = [c_void_p, POINTER(c_double), c_longlong, POINTER(c_double), c_longlong]
    lib.xr_get_param_gradient.restype = c_int
    lib.xr_get_param_gradient_system.argtypes = [c_void_p, c_int, POINTER(c_double), c_longlong, POINTER(c_double),
                                                 c_longlong]
    lib.xr_get_param_gradient_system.restype = c_int
    lib.xr_get_param_gradient_blocks.argtypes = [c_void_p, POINTER(c_double), c_longlong]
    lib.xr_get_param_gradient_blocks.restype = c_int
    lib.xr_get_param_gradient_atoms.argtypes = [c_void_p, c_int, POINTER(c_double), c_longlong]
    lib.xr_get_param_gradient_atoms.restype = c_int
    lib.xr_ctx_memory.argtypes = [c_void_p, POINTER(c_longlong), POINTER(c_longlong), c_int]
    lib.xr_ctx_memory.restype = c_int
    lib.xr_footprint_bytes.argtypes = [c_int, c_int, c_longlong, c_longlong]
    lib.xr_footprint_bytes.restype = c_longlong
    lib.xr_count_neighbors_static.argtypes = [POINTER(System), c_double, c_void_p, POINTER(c_int), POINTER(c_longlong)]
    lib.xr_count_neighbors_static.restype = c_int
    lib.xr_static_last_error.argtypes = []
    lib.xr_static_last_error.restype = c_char_p
    _LIB = lib
    return lib


def addr(a):
    """Address of a C-contiguous numpy array's data (None for None), for the void* struct members."""
    if a is None:
        return None
    return a.__array_interface__["data"][0]


def ptr(a, ctype):
    """Pointer to a C-contiguous numpy array (or NULL for None)."""
    if a is None:
        return None
    return a.ctypes.data_as(POINTER(ctype))


class ForceFieldHandle:
    """Device copy of a force field's packed tables (``xr_ff``)."""

    def __init__(self, tables, is_carbon, vdw_type):
        lib = load()
        self._lib = lib
        t = tables
        keep = dict(
            general=np.ascontiguousarray(t["general"], dtype=np.float64),
            atom=np.ascontiguousarray(t["atom"], dtype=np.float64),
            pair=np.ascontiguousarray(t["pair"], dtype=np.float64),
            is_carbon=np.ascontiguousarray(is_carbon, dtype=np.int32),
            angle_index=np.ascontiguousarray(t["angle_index"], dtype=np.int32),
            angle=np.ascontiguousarray(t["angle"], dtype=np.float64),
            torsion_index=np.ascontiguousarray(t["torsion_index"], dtype=np.int32),
            torsion=np.ascontiguousarray(t["torsion"], dtype=np.float64),
            hbond_index=np.ascontiguousarray(t["hbond_index"], dtype=np.int32),
            hbond=np.ascontiguousarray(t["hbond"], dtype=np.float64),
        )
        handle = c_void_p()
        code = lib.xr_ff_create(
            ptr(keep["general"], c_double), int(t["ntypes"]), ptr(keep["atom"], c_double), ptr(keep["pair"], c_double),
            ptr(keep["is_carbon"], c_int), int(vdw_type), ptr(keep["angle_index"], c_int), ptr(keep["angle"], c_double),
            len(keep["angle"]), ptr(keep["torsion_index"], c_int), ptr(keep["torsion"], c_double), len(keep["torsion"]),
            ptr(keep["hbond_index"], c_int), ptr(keep["hbond"], c_double), len(keep["hbond"]), byref(handle),
        )
        if code != XR_OK:
            raise RuntimeError(f"xr_ff_create failed with code {code}")
        self.handle = handle
        self._shape = {k: v.shape for k, v in keep.items()}
        self.nsets = 1

    def update(self, tables, is_carbon, vdw_type):
        """New values for the same table shapes (``xr_ff_update``), written into the device tables."""
        t = tables
        keep = dict(
            general=np.ascontiguousarray(t["general"], dtype=np.float64),
            atom=np.ascontiguousarray(t["atom"], dtype=np.float64),
            pair=np.ascontiguousarray(t["pair"], dtype=np.float64),
            is_carbon=np.ascontiguousarray(is_carbon, dtype=np.int32),
            angle_index=np.ascontiguousarray(t["angle_index"], dtype=np.int32),
            angle=np.ascontiguousarray(t["angle"], dtype=np.float64),
            torsion_index=np.ascontiguousarray(t["torsion_index"], dtype=np.int32),
            torsion=np.ascontiguousarray(t["torsion"], dtype=np.float64),
            hbond_index=np.ascontiguousarray(t["hbond_index"], dtype=np.int32),
            hbond=np.ascontiguousarray(t["hbond"], dtype=np.float64),
        )
        if {k: v.shape for k, v in keep.items()} != self._shape:
            raise ValueError("an updated force field must have the same elements and parameter records")
        code = self._lib.xr_ff_update(
            self.handle, ptr(keep["general"], c_double), ptr(keep["atom"], c_double), ptr(keep["pair"], c_double),
            ptr(keep["is_carbon"], c_int), int(vdw_type), ptr(keep["angle_index"], c_int), ptr(keep["angle"], c_double),
            ptr(keep["torsion_index"], c_int), ptr(keep["torsion"], c_double), ptr(keep["hbond_index"], c_int),
            ptr(keep["hbond"], c_double))
        if code != XR_OK:
            raise RuntimeError(f"xr_ff_update failed with code {code}")
        self.nsets = 1

    def set_count(self, nsets):
        """Resize to ``nsets`` parameter sets (``xr_ff_set_count``); new sets start as set 0."""
        code = self._lib.xr_ff_set_count(self.handle, int(nsets))
        if code != XR_OK:
            raise (ValueError if code == XR_EINPUT else RuntimeError)(f"xr_ff_set_count failed with code {code}")
        self.nsets = int(nsets)

    def update_sets(self, first, count, atom=None, pair=None, angle=None, torsion=None, hbond=None):
        """Values of sets ``first .. first + count - 1`` (``xr_ff_update_sets``): each table None (set
        0's values) or ``count`` stacked tables of the force field's shapes."""
        keep = {}
        for name, a in (("atom", atom), ("pair", pair), ("angle", angle), ("torsion", torsion), ("hbond", hbond)):
            if a is None:
                keep[name] = None
                continue
            a = np.ascontiguousarray(a, dtype=np.float64)
            if a.shape != (int(count),) + self._shape[name]:
                raise ValueError(f"{name} tables of the parameter sets must have shape (count,) + {self._shape[name]}")
            keep[name] = a
        code = self._lib.xr_ff_update_sets(self.handle, int(first), int(count), ptr(keep["atom"], c_double),
                                           ptr(keep["pair"], c_double), ptr(keep["angle"], c_double),
                                           ptr(keep["torsion"], c_double), ptr(keep["hbond"], c_double))
        if code != XR_OK:
            raise (ValueError if code == XR_EINPUT else RuntimeError)(f"xr_ff_update_sets failed with code {code}")

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            self._lib.xr_ff_destroy(h)
            self.handle = None


class Context:
    """Device work buffers and stream of one host thread (``xr_ctx``)."""

    def __init__(self, device=0, stream=None):
        lib = load()
        self._lib = lib
        handle = c_void_p()
        code = lib.xr_ctx_create(int(device), c_void_p(stream) if stream else None, byref(handle))
        if code != XR_OK:
            raise RuntimeError(f"xr_ctx_create failed with code {code} (is a CUDA GPU available?)")
        self.handle = handle

    def last_error(self):
        return self._lib.xr_last_error(self.handle).decode()

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            self._lib.xr_ctx_destroy(h)
            self.handle = None
