"""CPU tests of the host side: the C-ABI library loads and exports every
declared entry point, the options layer, point merging, PLOT3D I/O and the
synthetic generators.  No CUDA call is made here."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_functions():
    with open(os.path.join(ROOT, "include", "idwarp_gb300.h")) as f:
        src = f.read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|void)\s+(idw_\w+)\s*\(", src, flags=re.M)))


def test_library_exports_every_declared_symbol(built_lib):
    from idwarp_gb300 import _lib

    L = C.CDLL(built_lib)
    declared = _header_functions()
    assert len(declared) >= 30
    for name in declared:
        assert hasattr(L, name), name
    # and the Python binding binds only declared entry points
    assert set(_lib.exported_symbols()) <= set(declared)


def test_default_options_match_reference(built_lib):
    from idwarp_gb300 import _lib

    L = _lib.load()
    o = _lib.idw_options()
    L.idw_default_options(C.byref(o))
    assert (o.aExp, o.bExp, o.LdefFact, o.alpha, o.errTol) == (3.0, 5.0, 1.0, 0.25, 0.0005)
    assert (o.evalMode, o.useRotations, o.zeroCornerRotations, o.bucketSize) == (1, 1, 1, 8)
    assert o.cornerAngle == 30.0 and o.symmTol == 1e-6


def test_point_reduce_library_matches_oracle(built_lib, oracle_lib):
    from idwarp_gb300 import pointReduce
    from oracle.pyoracle import point_reduce
    from tests.meshes import sphere_small, wing_small

    rng = np.random.default_rng(5)
    for m in (sphere_small(), wing_small()):
        pts = m["pts"].copy()
        # sprinkle near-duplicates inside and outside the tolerance
        k = rng.choice(len(pts), 20, replace=False)
        extra = pts[k] + rng.choice([3e-13, 5e-12], size=(20, 1)) * rng.normal(size=(20, 3))
        pts = np.vstack([pts, extra])
        u1, l1, n1 = pointReduce(pts, 1e-12)
        u2, l2, n2 = point_reduce(pts, 1e-12)
        assert n1 == n2
        np.testing.assert_array_equal(l1, l2)
        np.testing.assert_array_equal(u1, u2)


def test_options_semantics():
    from idwarp_gb300.options import BaseSolver, Error

    defs = {"aExp": [float, 3.0], "evalMode": [str, ["fast", "exact"]], "gridFile": [(str, type(None)), None]}
    b = BaseSolver("IDWarp", "x", defaultOptions=defs, options={"AEXP": 4, "evalmode": "exact"})
    assert b.getOption("aexp") == 4.0 and isinstance(b.getOption("aExp"), float)
    assert b.getOption("EvalMode") == "exact"
    with pytest.raises(Error):
        b.setOption("evalMode", "slow")
    with pytest.raises(Error):
        b.setOption("nope", 1)
    with pytest.raises(Error):
        b.setOption("aExp", "three")


def test_usmesh_requires_options(built_lib):
    from idwarp_gb300 import Error, USMesh

    with pytest.raises(Error):
        USMesh()


def test_plot3d_roundtrip(tmp_path):
    from idwarp_gb300.plot3d import readPlot3D, readPlot3DSurface, writePlot3D, writePlot3DSurface

    rng = np.random.default_rng(0)
    nodes = rng.normal(size=(4 * 3 * 2 + 5 * 2 * 2, 3))
    sizes = np.array([[4, 3, 2], [5, 2, 2]])
    f = tmp_path / "g.xyz"
    writePlot3D(str(f), nodes, sizes)
    back, sz = readPlot3D(str(f), return_blocks=True)
    np.testing.assert_array_equal(back, nodes)
    np.testing.assert_array_equal(sz, sizes)
    blk = rng.normal(size=(3, 4, 3))
    fs = tmp_path / "s.xyz"
    writePlot3DSurface(str(fs), [blk])
    pts, conn = readPlot3DSurface(str(fs))
    np.testing.assert_array_equal(pts, blk.reshape(-1, 3))
    assert conn.shape == (2 * 3, 4) and conn.min() == 0 and conn.max() == 11
    np.testing.assert_array_equal(conn[0], [0, 1, 5, 4])


def test_synthetic_sizes():
    from idwarp_gb300 import synthetic as S

    s = S.sphere_ogrid()
    assert len(s["pts"]) == 6 * 19 * 19
    assert len(s["xv0"]) == 1946 * 49
    w = S.wing_shell(ni=41, nj=11, nk=6)
    assert w["xv0"].shape == (41 * 11 * 6, 3)
    assert np.all(w["xv0"][:, 1] >= -1e-12)
    xs = S.wing_perturbation(w["pts"], seed=2)
    assert np.isfinite(xs).all() and np.abs(xs - w["pts"]).max() < 0.3


def test_nonfinite_surface_coordinates_raise_error():
    # the library's non-finite status becomes the reference's Error, and the
    # call never counts as a new surface
    import math

    from idwarp_gb300 import Error, USMesh
    from idwarp_gb300 import _lib

    class FakeLib:
        def idw_set_surface_coordinates(self, ctx, ptr, n, where):
            import ctypes as C

            a = (C.c_double * n).from_address(ptr.value)
            return _lib.IDW_ERR_NONFINITE if any(not math.isfinite(v) for v in a) else 0

    m = USMesh.__new__(USMesh)
    m.nSurf, m.ctx, m.lib, m._surfVersion = 4, None, FakeLib(), 0
    m.setSurfaceCoordinates(np.ones((4, 3)))
    assert m._surfVersion == 1
    bad = np.ones((4, 3))
    bad[2, 1] = np.inf
    with pytest.raises(Error, match="Non-finite"):
        m.setSurfaceCoordinates(bad)
    assert m._surfVersion == 1


def test_complex_step_classes_errors():
    # USMesh_C runs the complex step in FP64 only; MultiUSMesh_C is not provided
    from idwarp_gb300 import Error, MultiUSMesh_C, USMesh_C

    with pytest.raises(Error, match="FP64"):
        USMesh_C(options={"precision": "mixed"})
    with pytest.raises(Error, match="USMesh_C"):
        MultiUSMesh_C(options={})
