"""ctypes wrapper of the oracle library (test infrastructure only).

The oracle is a CPU FP64 restatement of IDWarp's warping path, used by the
tests and by bench.py's CPU-baseline leg to CHECK the GPU library.  Nothing in
the product package imports this module.
"""
import ctypes as C
import os

import numpy as np

from .build import build_oracle

_lib = None
_libs = {}

_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)
_LP = C.POINTER(C.c_longlong)


def _d(a):
    return a.ctypes.data_as(_DP)


def _i(a):
    return a.ctypes.data_as(_IP)


def use_library(path=None):
    """Load the oracle from another build of the same source (None: the default
    build).  Used to measure how sensitive a case is to rounding order."""
    global _lib
    _lib = None
    return lib(path)


def _bind(L):
    L.orc_new.restype = C.c_void_p
    L.orc_new.argtypes = [_DP]
    L.orc_free.argtypes = [C.c_void_p]
    L.orc_set_options.argtypes = [C.c_void_p, _DP]
    L.orc_set_symmetry.argtypes = [C.c_void_p, _DP, _DP, C.c_int]
    L.orc_set_volume.argtypes = [C.c_void_p, _DP, C.c_longlong]
    L.orc_point_reduce.argtypes = [_DP, C.c_int, C.c_double, _DP, _IP]
    L.orc_set_surface_definition.argtypes = [C.c_void_p, _DP, C.c_int, _IP, C.c_int, _IP, C.c_int]
    L.orc_set_surface_coords.argtypes = [C.c_void_p, _DP]
    L.orc_warp.argtypes = [C.c_void_p, _DP]
    L.orc_warp_range.argtypes = [C.c_void_p, C.c_longlong, C.c_longlong]
    L.orc_warp_complex.argtypes = [C.c_void_p, _DP, _DP, _DP, _DP]
    L.orc_warp_deriv.argtypes = [C.c_void_p, _DP, _DP]
    L.orc_warp_deriv_range.argtypes = [C.c_void_p, _DP, _DP, C.c_longlong, C.c_longlong]
    L.orc_warp_deriv_fwd.argtypes = [C.c_void_p, _DP, _DP]
    L.orc_sizes.argtypes = [C.c_void_p, _LP]
    L.orc_ldef0.restype = C.c_double
    L.orc_ldef0.argtypes = [C.c_void_p]
    L.orc_get_tree.argtypes = [C.c_void_p, _IP, _DP, _DP, _DP]
    L.orc_get_surface.argtypes = [C.c_void_p, _DP, _DP, _DP, _IP, _IP]
    L.orc_get_den0.argtypes = [C.c_void_p, _DP]
    L.orc_get_denom.argtypes = [C.c_void_p, _DP]
    L.orc_get_nodal.argtypes = [C.c_void_p, _DP, _DP]
    L.orc_stats.argtypes = [C.c_void_p, _LP]
    L.orc_dry_run.argtypes = [C.c_void_p, _DP]
    L.orc_set_threads.argtypes = [C.c_int]
    L.orc_max_threads.restype = C.c_int
    return L


def lib(path=None):
    """The oracle library (the checker build unless another build's path is
    given); each build is loaded once."""
    global _lib
    if path is None and _lib is not None:
        return _lib
    p = os.path.abspath(path or build_oracle())
    if p not in _libs:
        _libs[p] = _bind(C.CDLL(p))
    if path is None:
        _lib = _libs[p]
    return _libs[p]


def timing_library():
    """The timing build of the same source (-O3, tuned for the host CPU, FMA
    contraction allowed): the CPU baseline's speed, never the checker."""
    from .build import build_oracle_timing

    return lib(build_oracle_timing())


DEFAULT_OPTIONS = {
    "aExp": 3.0,
    "bExp": 5.0,
    "LdefFact": 1.0,
    "alpha": 0.25,
    "errTol": 0.0005,
    "evalMode": "fast",
    "useRotations": True,
    "zeroCornerRotations": True,
    "cornerAngle": 30.0,
    "bucketSize": 8,
    "treeBuild": "kd",
}


def pack_options(opts):
    o = dict(DEFAULT_OPTIONS)
    o.update(opts or {})
    return np.array(
        [
            o["aExp"], o["bExp"], o["LdefFact"], o["alpha"], o["errTol"],
            0.0 if o["evalMode"] == "exact" else 1.0,
            1.0 if o["useRotations"] else 0.0,
            1.0 if o["zeroCornerRotations"] else 0.0,
            o["cornerAngle"], float(o["bucketSize"]),
            1.0 if o["treeBuild"] == "morton" else 0.0,
        ],
        dtype=np.float64,
    )


def set_threads(n, library=None):
    (library or lib()).orc_set_threads(int(n))


def max_threads(library=None):
    return (library or lib()).orc_max_threads()


def point_reduce(pts, tol=1e-12):
    pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
    n = len(pts)
    uniq = np.zeros((max(n, 1), 3))
    link = np.zeros(max(n, 1), dtype=np.intc)
    nu = lib().orc_point_reduce(_d(pts), n, tol, _d(uniq), _i(link))
    return uniq[:nu].copy(), link[:n].copy(), nu


class OracleMesh:
    """One oracle instance: the reference's USMesh state restated on the CPU."""

    def __init__(self, options=None, library=None):
        self.L = library or lib()
        self.opts = dict(DEFAULT_OPTIONS)
        self.opts.update(options or {})
        self._ov = pack_options(self.opts)
        self.h = self.L.orc_new(_d(self._ov))
        self.nVol = 0
        self.nPts = 0

    def __del__(self):
        try:
            self.L.orc_free(self.h)
        except Exception:
            pass

    def set_options(self, **kw):
        self.opts.update(kw)
        self._ov = pack_options(self.opts)
        self.L.orc_set_options(self.h, _d(self._ov))

    def set_symmetry(self, pts, normals):
        pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
        normals = np.ascontiguousarray(normals, dtype=np.float64).reshape(-1, 3)
        rc = self.L.orc_set_symmetry(self.h, _d(pts), _d(normals), len(pts))
        assert rc == 0, rc

    def set_volume(self, xv0):
        xv0 = np.ascontiguousarray(xv0, dtype=np.float64).reshape(-1, 3)
        self.nVol = len(xv0)
        self.L.orc_set_volume(self.h, _d(xv0), self.nVol)

    def set_surface_definition(self, pts, conn, face_sizes):
        pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
        conn = np.ascontiguousarray(np.asarray(conn).ravel(), dtype=np.intc)
        fs = np.ascontiguousarray(np.asarray(face_sizes).ravel(), dtype=np.intc)
        self.nPts = len(pts)
        rc = self.L.orc_set_surface_definition(self.h, _d(pts), len(pts), _i(conn), len(conn), _i(fs), len(fs))
        assert rc == 0, rc

    def set_surface_coordinates(self, xs):
        xs = np.ascontiguousarray(xs, dtype=np.float64).reshape(-1, 3)
        assert len(xs) == self.nPts
        self.L.orc_set_surface_coords(self.h, _d(xs))

    def warp(self):
        out = np.zeros((self.nVol, 3))
        rc = self.L.orc_warp(self.h, _d(out))
        assert rc == 0, rc
        return out

    def warp_range(self, j0, j1):
        rc = self.L.orc_warp_range(self.h, int(j0), int(j1))
        assert rc == 0, rc

    def warp_complex(self, xs_complex):
        xs = np.asarray(xs_complex).reshape(-1, 3)
        xr = np.ascontiguousarray(xs.real, dtype=np.float64)
        xi = np.ascontiguousarray(xs.imag, dtype=np.float64)
        vr = np.zeros((self.nVol, 3))
        vi = np.zeros((self.nVol, 3))
        rc = self.L.orc_warp_complex(self.h, _d(xr), _d(xi), _d(vr), _d(vi))
        assert rc == 0, rc
        return vr + 1j * vi

    def warp_deriv(self, dxv):
        dxv = np.ascontiguousarray(dxv, dtype=np.float64).reshape(-1, 3)
        out = np.zeros((self.nPts, 3))
        rc = self.L.orc_warp_deriv(self.h, _d(dxv), _d(out))
        assert rc == 0, rc
        return out

    def warp_deriv_range(self, dxv, j0, j1):
        dxv = np.ascontiguousarray(dxv, dtype=np.float64).reshape(-1, 3)
        out = np.zeros((self.nPts, 3))
        rc = self.L.orc_warp_deriv_range(self.h, _d(dxv), _d(out), int(j0), int(j1))
        assert rc == 0, rc
        return out

    def warp_deriv_fwd(self, dxs):
        dxs = np.ascontiguousarray(dxs, dtype=np.float64).reshape(-1, 3)
        out = np.zeros((self.nVol, 3))
        rc = self.L.orc_warp_deriv_fwd(self.h, _d(dxs), _d(out))
        assert rc == 0, rc
        return out

    def sizes(self):
        out = np.zeros(8, dtype=np.int64)
        self.L.orc_sizes(self.h, out.ctypes.data_as(_LP))
        keys = ["nUnique", "nNodes", "maxDepth", "nVol", "nPts", "nLoop", "nFaces"]
        return dict(zip(keys, [int(v) for v in out[:7]]))

    def ldef0(self):
        return self.L.orc_ldef0(self.h)

    def tree(self):
        s = self.sizes()
        nn = s["nNodes"]
        lu = np.zeros((nn, 4), dtype=np.intc)
        geom = np.zeros((nn, 4))
        ai = np.zeros(nn)
        err = np.zeros((nn, 12))
        self.L.orc_get_tree(self.h, _i(lu), _d(geom), _d(ai), _d(err))
        return {"l": lu[:, 0].copy(), "u": lu[:, 1].copy(), "dnum": lu[:, 2].copy(), "escape": lu[:, 3].copy(),
                "X": geom[:, :3].copy(), "oradius": geom[:, 3].copy(), "Ai": ai, "err": err}

    def surface(self):
        n = self.sizes()["nUnique"]
        xu0 = np.zeros((n, 3))
        ai = np.zeros(n)
        n0 = np.zeros((n, 3))
        ic = np.zeros(n, dtype=np.intc)
        xi = np.zeros(n, dtype=np.intc)
        self.L.orc_get_surface(self.h, _d(xu0), _d(ai), _d(n0), _i(ic), _i(xi))
        return {"Xu0": xu0, "Ai": ai, "normals0": n0, "isCorner": ic, "XuInd": xi}

    def den0(self):
        out = np.zeros(self.nVol)
        self.L.orc_get_den0(self.h, _d(out))
        return out

    def denom(self):
        out = np.zeros(self.nVol)
        self.L.orc_get_denom(self.h, _d(out))
        return out

    def nodal(self):
        n = self.sizes()["nUnique"]
        Mi = np.zeros((n, 3, 3))
        Bi = np.zeros((n, 3))
        self.L.orc_get_nodal(self.h, _d(Mi), _d(Bi))
        return Mi, Bi

    def stats(self):
        out = np.zeros(3, dtype=np.int64)
        self.L.orc_stats(self.h, out.ctypes.data_as(_LP))
        return {"leafPairs": int(out[0]), "approx": int(out[1]), "visited": int(out[2])}

    def dry_run(self):
        out = np.zeros(self.nVol)
        self.L.orc_dry_run(self.h, _d(out))
        return out
