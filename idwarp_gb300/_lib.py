"""ctypes binding of ``libidwarp_gb300.so`` (the C ABI in include/idwarp_gb300.h).

The library is built in-tree by :func:`idwarp_gb300.build.build`.  Loading
fails loudly when it is missing: there is no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

from .build import LIB

IDW_HOST = 0
IDW_DEVICE = 1
IDW_EVAL_EXACT = 0
IDW_EVAL_FAST = 1
IDW_PREC_FP64 = 0
IDW_PREC_MIXED = 1
IDW_ADJ_PRECISE = 0
IDW_ADJ_FAST = 1
IDW_WALK_LISTS_AUTO = 0
IDW_WALK_LISTS_OFF = 1
IDW_TREE_KD = 0
IDW_TREE_MORTON = 1
IDW_OK = 0
IDW_ERR_ARG = -1
IDW_ERR_STATE = -2
IDW_ERR_CUDA = -3
IDW_ERR_NONFINITE = -4
IDW_ERR_LIMIT = -5
IDW_ERR_NOMEM = -6
IDW_ERR_RESTART = -7

_ERRNAMES = {
    -1: "IDW_ERR_ARG", -2: "IDW_ERR_STATE", -3: "IDW_ERR_CUDA", -4: "IDW_ERR_NONFINITE",
    -5: "IDW_ERR_LIMIT", -6: "IDW_ERR_NOMEM", -7: "IDW_ERR_RESTART",
}


class idw_options(C.Structure):
    _fields_ = [
        ("aExp", C.c_double), ("bExp", C.c_double), ("LdefFact", C.c_double), ("alpha", C.c_double),
        ("errTol", C.c_double), ("symmTol", C.c_double), ("cornerAngle", C.c_double),
        ("evalMode", C.c_int32), ("useRotations", C.c_int32), ("zeroCornerRotations", C.c_int32),
        ("bucketSize", C.c_int32), ("precision", C.c_int32), ("diagnostics", C.c_int32),
        ("mixedGate", C.c_double), ("exactSchedule", C.c_int32), ("adjointPrecision", C.c_int32),
        ("walkLists", C.c_int32), ("treeBuild", C.c_int32), ("deterministic", C.c_int32),
        ("reserved", C.c_int32 * 2),
    ]


class idw_stats(C.Structure):
    _fields_ = [
        ("leafPairs", C.c_int64), ("approx", C.c_int64), ("visited", C.c_int64), ("fp64Fallback", C.c_int64),
        ("nUnique", C.c_int64), ("nTreeNodes", C.c_int64), ("maxDepth", C.c_int64), ("nVol", C.c_int64),
        ("nSurfPts", C.c_int64), ("nLoop", C.c_int64), ("Ldef0", C.c_double), ("lastKernelMs", C.c_double),
        ("warpLeafSlots", C.c_int64), ("warpNodeSlots", C.c_int64), ("preciseTerms", C.c_int64),
        ("walkListEntries", C.c_int64), ("treeBuildMs", C.c_double),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved"}


class idw_tuning(C.Structure):
    _fields_ = [("batchGroup", C.c_int32), ("adjMaxGroup", C.c_int32), ("batchMs", C.c_double * 4),
                ("adjMs", C.c_double * 3), ("reserved", C.c_int32 * 4)]

    def as_dict(self):
        return {"batchGroup": self.batchGroup, "adjMaxGroup": self.adjMaxGroup, "batchMs": list(self.batchMs),
                "adjMs": dict(zip((16, 8, 4), list(self.adjMs)))}


class LibraryError(RuntimeError):
    pass


_lib = None
_VP = C.c_void_p
_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int32)

# (name, argtypes); every function returns int status unless listed in _VOID
_SIGS = {
    "idw_default_options": [C.POINTER(idw_options)],
    "idw_create": [C.POINTER(idw_options), C.POINTER(_VP)],
    "idw_destroy": [_VP],
    "idw_last_error": [_VP, C.c_char_p, C.c_int],
    "idw_set_stream": [_VP, _VP],
    "idw_synchronize": [_VP],
    "idw_set_options": [_VP, C.POINTER(idw_options)],
    "idw_create_common_grid": [_VP, _VP, C.c_int64, C.c_int],
    "idw_set_symmetry_planes": [_VP, _DP, _DP, C.c_int32],
    "idw_point_reduce": [_DP, C.c_int32, C.c_double, _DP, _IP, _IP],
    "idw_initialize_warping": [_VP, _DP, C.c_int32, _DP, C.c_int32, _IP, _IP, C.c_int32, _IP, C.c_int32],
    "idw_set_surface_coordinates": [_VP, _VP, C.c_int64, C.c_int],
    "idw_get_surface_coordinates": [_VP, _VP, C.c_int64, C.c_int],
    "idw_warp_mesh": [_VP],
    "idw_set_surface_coordinates_cs": [_VP, _VP, C.c_int64, C.c_int],
    "idw_warp_mesh_cs": [_VP],
    "idw_get_volume_coordinates_cs": [_VP, _VP, C.c_int64, C.c_int],
    "idw_warp_mesh_batch": [_VP, _VP, C.c_int32, _VP, C.c_int],
    "idw_get_volume_coordinates": [_VP, _VP, C.c_int64, C.c_int],
    "idw_get_common_volume_coordinates": [_VP, _VP, C.c_int64, C.c_int],
    "idw_get_volume_coordinates_async": [_VP, _VP, C.c_int64],
    "idw_set_volume_coordinates": [_VP, _VP, C.c_int64, C.c_int],
    "idw_set_external_mesh_indices": [_VP, _IP, C.c_int64],
    "idw_get_solver_mesh_dof": [_VP, C.POINTER(C.c_int64)],
    "idw_warp_to_solver_grid": [_VP, _VP, C.c_int64, _VP, C.c_int64, C.c_int],
    "idw_solver_to_warp_grid": [_VP, _VP, C.c_int64, _VP, C.c_int64, C.c_int],
    "idw_warp_deriv": [_VP, _VP, C.c_int64, C.c_int],
    "idw_get_dxs": [_VP, _VP, C.c_int64, C.c_int],
    "idw_warp_deriv_batch": [_VP, _VP, C.c_int32, _VP, C.c_int],
    "idw_warp_deriv_fwd": [_VP, _VP, C.c_int64, _VP, C.c_int64, C.c_int],
    "idw_warp_deriv_fwd_batch": [_VP, _VP, C.c_int32, _VP, C.c_int],
    "idw_warp_deriv_noalloc": [_VP, _VP, C.c_int64, _VP, C.c_int64],
    "idw_autotune": [_VP, C.c_int32, C.c_int32, C.POINTER(idw_tuning)],
    "idw_get_denominator0": [_VP, _VP, C.c_int64, C.c_int],
    "idw_compute_denominator0": [_VP],
    "idw_set_denominator0": [_VP, _VP, C.c_int64, C.c_int64, C.c_int],
    "idw_dry_run_costs": [_VP, _VP, C.c_int64, C.c_int],
    "idw_get_denominator": [_VP, _VP, C.c_int64, C.c_int],
    "idw_get_stats": [_VP, C.POINTER(idw_stats)],
    "idw_get_tree": [_VP, _IP, _DP, _DP, _DP],
    "idw_get_surface_state": [_VP, _DP, _DP, _DP, _IP, _IP],
    "idw_get_nodal_properties": [_VP, _DP, _DP],
}
_VOID = {"idw_default_options"}


def exported_symbols():
    """Names of the entry points the Python layer binds (all declared in the header)."""
    return sorted(_SIGS)


def load(path=None):
    """Load the shared library (must already be built) and bind its signatures."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB
    if not os.path.exists(p):
        raise LibraryError(
            "libidwarp_gb300.so not found at %s: build it first with "
            "`python -c 'import __graft_entry__ as g; g.build()'` or idwarp_gb300.build.build()" % p)
    L = C.CDLL(p)
    for name, args in _SIGS.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = None if name in _VOID else C.c_int
    if path is None:
        _lib = L
    return L


def dptr(a):
    return a.ctypes.data_as(_DP)


def iptr(a):
    return a.ctypes.data_as(_IP)


def vptr(a):
    """Host numpy array or CUDA tensor -> (void pointer, where-flag)."""
    if isinstance(a, np.ndarray):
        return C.c_void_p(a.ctypes.data), IDW_HOST
    # torch tensor
    if a.is_cuda:
        return C.c_void_p(a.data_ptr()), IDW_DEVICE
    return C.c_void_p(a.data_ptr()), IDW_HOST


def check(lib, ctx, rc, what):
    if rc != 0:
        msg = C.create_string_buffer(1024)
        if ctx:
            lib.idw_last_error(ctx, msg, 1024)
        raise LibraryError("%s failed (%s): %s" % (what, _ERRNAMES.get(rc, rc), msg.value.decode(errors="replace")))
