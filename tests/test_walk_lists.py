"""Recorded decisions of the mixed fast walk (option walkLists "auto") against
the walk that decides as it goes (walkLists "off").

The fast walk's open/approximate decisions depend on the set-up state and
errTol only (kd_tree.F90:619-662: the distance from the initial volume point
to the cluster centroid of Xu0, the init-time error table, den0), so the
library records them once per warp of 32 volume nodes and replays them.  The
replay evaluates the same terms with the same device code in the same order:
positions and work counters agree bit for bit, for every weight law, bucket
size, symmetry-plane count and precision gate, across several surfaces, after
errTol changes, and for the tangent (warpDerivFwd)."""
import numpy as np
import pytest

from tests.meshes import build_gpu, sphere_small, wing_small

pytestmark = pytest.mark.gpu

CASES = [
    ("wing", {}, 0),
    ("sphere", {}, 0),
    ("sphere", {}, 1),
    ("sphere", {}, 3),
    ("sphere", {"bucketSize": 1}, 0),
    ("sphere", {"bucketSize": 64}, 0),
    ("sphere", {"aExp": 4.0, "bExp": 6.0}, 0),
    ("sphere", {"aExp": 2.5, "bExp": 4.5}, 0),
    ("wing", {"LdefFact": 100.0}, 0),
    ("wing", {"mixedGate": 1e-6}, 0),  # most terms in double-float
    ("wing", {"errTol": 1e-2}, 0),
    ("wing", {"errTol": 0.0}, 0),  # every cluster opened: leaves only
]

STATS = ("leafPairs", "approx", "visited", "fp64Fallback", "preciseTerms")


def _mesh(which, planes):
    m = dict(sphere_small() if which == "sphere" else wing_small())
    if planes:
        m["symmetryPlanes"] = [[[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]], [[0.0, 0.0, 0.0], [0.0, 1.0, 0.0]],
                               [[0.0, 0.0, 0.0], [0.0, 0.0, 1.0]]][:planes]
    return m


def _warps(m, opts, surfaces):
    g = build_gpu(m, opts, precision="mixed")
    out = []
    for xs in surfaces:
        g.setSurfaceCoordinates(xs)
        g.warpMesh()
        out.append((g.getWarpGrid().copy(), g.getStats()))
    return out


@pytest.mark.parametrize("which,opts,planes", CASES)
def test_replay_equals_decision_walk(which, opts, planes, built_lib):
    m = _mesh(which, planes)
    rng = np.random.default_rng(7)
    xs0 = m["xs"]
    xs1 = xs0 + 1e-3 * rng.standard_normal(xs0.shape)
    rep = _warps(m, dict(opts, walkLists="auto"), [xs0, xs1, xs0])
    ref = _warps(m, dict(opts, walkLists="off"), [xs0, xs1, xs0])
    for (xr, sr), (xw, sw) in zip(rep, ref):
        np.testing.assert_array_equal(xr, xw)
        for k in STATS:
            assert sr[k] == sw[k], k
    # the third warp repeats the first surface: same grid
    np.testing.assert_array_equal(rep[0][0], rep[2][0])


def test_errtol_change_rerecords(built_lib):
    # errTol changes between warps: the lists are recorded again (the
    # precision gate's denominator stays the first walk's on both sides)
    m = wing_small()
    res = []
    for wl in ("auto", "off"):
        g = build_gpu(m, {"walkLists": wl}, precision="mixed")
        g.setSurfaceCoordinates(m["xs"])
        g.warpMesh()
        s0 = g.getStats()
        g.setOption("errTol", 1e-3)
        g.warpMesh()
        res.append((g.getWarpGrid().copy(), g.getStats(), s0))
    np.testing.assert_array_equal(res[0][0], res[1][0])
    for k in STATS:
        assert res[0][1][k] == res[1][1][k], k
    assert res[0][1]["approx"] != res[0][2]["approx"]


def test_tangent_replay(built_lib):
    m = _mesh("sphere", 1)
    rng = np.random.default_rng(11)
    xsd = rng.standard_normal(m["xs"].shape)
    res = []
    for wl in ("auto", "off"):
        g = build_gpu(m, {"walkLists": wl}, precision="mixed")
        g.setSurfaceCoordinates(m["xs"])
        g.warpMesh()
        res.append(np.asarray(g.warpDerivFwd(xsd.ravel(), solverVec=False)).copy())
    np.testing.assert_array_equal(res[0], res[1])


def test_few_volume_nodes(built_lib):
    # a single partial warp of volume nodes
    m = dict(wing_small())
    m["xv0"] = m["xv0"][:19].copy()
    a = _warps(m, {"walkLists": "auto"}, [m["xs"]])[0]
    b = _warps(m, {"walkLists": "off"}, [m["xs"]])[0]
    np.testing.assert_array_equal(a[0], b[0])
    for k in STATS:
        assert a[1][k] == b[1][k], k


def test_batched_surfaces_replay(built_lib):
    # five surfaces: a group of four and one alone, each replayed
    m = _mesh("wing", 0)
    rng = np.random.default_rng(5)
    surfs = np.stack([m["xs"] + 1e-3 * rng.standard_normal(m["xs"].shape) for _ in range(5)])
    res = []
    for wl in ("auto", "off"):
        g = build_gpu(m, {"walkLists": wl}, precision="mixed")
        g.setSurfaceCoordinates(m["xs"])
        g.warpMesh()
        res.append((g.warpMeshBatch(surfs), g.getStats()))
    np.testing.assert_array_equal(res[0][0], res[1][0])
    for k in ("leafPairs", "approx", "visited"):
        assert res[0][1][k] == res[1][1][k], k


def test_batched_tangents_replay(built_lib):
    m = _mesh("sphere", 1)
    rng = np.random.default_rng(6)
    dirs = rng.standard_normal((3,) + m["xs"].shape)
    res = []
    for wl in ("auto", "off"):
        g = build_gpu(m, {"walkLists": wl}, precision="mixed")
        g.setSurfaceCoordinates(m["xs"])
        g.warpMesh()
        res.append(g.warpDerivFwdBatch(dirs))
    np.testing.assert_array_equal(res[0], res[1])


@pytest.mark.parametrize("prec", ["precise", "fast"])
@pytest.mark.parametrize("nseeds", [1, 21])
def test_reverse_product_replay(prec, nseeds, built_lib):
    # the adjoint lands warp sums with FP64 atomics, whose order varies from
    # run to run: the replayed and the deciding walk agree to that rounding
    m = _mesh("wing", 0)
    rng = np.random.default_rng(9)
    nvol = len(m["xv0"])
    dxv = rng.standard_normal((nseeds, nvol, 3))
    res = []
    for wl in ("auto", "off"):
        g = build_gpu(m, {"walkLists": wl, "adjointPrecision": prec}, precision="mixed")
        g.setSurfaceCoordinates(m["xs"])
        g.warpMesh()
        if nseeds == 1:
            g.warpDeriv(dxv[0].ravel(), solverVec=False)
            out = g.getdXs()[None]
        else:
            out = g.warpDerivBatch(dxv)
        res.append((out, g.getStats()))
    scale = np.abs(res[1][0]).max()
    assert np.abs(res[0][0] - res[1][0]).max() <= 1e-11 * scale
    for k in ("leafPairs", "approx", "visited", "fp64Fallback"):
        assert res[0][1][k] == res[1][1][k], k


def test_new_estimate_rerecords(built_lib):
    # a denominator estimate loaded after the first warp (as from a restart
    # file) moves every decision threshold: the lists are recorded again
    import ctypes as C

    from idwarp_gb300 import _lib

    m = wing_small()
    res = []
    for wl in ("auto", "off"):
        g = build_gpu(m, {"walkLists": wl}, precision="mixed")
        g.setSurfaceCoordinates(m["xs"])
        g.warpMesh()
        s0 = g.getStats()
        den = np.ascontiguousarray(g.getDenominator0() * 3.0)
        assert g.lib.idw_set_denominator0(g.ctx, den.ctypes.data_as(C.c_void_p), len(den), 0, _lib.IDW_HOST) == 0
        g.warpMesh()
        res.append((g.getWarpGrid().copy(), g.getStats(), s0))
    np.testing.assert_array_equal(res[0][0], res[1][0])
    for k in STATS:
        assert res[0][1][k] == res[1][1][k], k
    assert res[0][1]["approx"] != res[0][2]["approx"]
