"""The Morton surface tree (option treeBuild "morton") built on the GPU,
against the oracle's restatement of the same tree.

Integer state (point order, ranges, escape indices, leaf flags) is equal;
centroid and radius are formed in the same order on both sides (bottom-up
sums, the same distance formula) and are equal bit for bit.  With the tree
equal, every walk takes the oracle's decisions: FP64 results within the
FP64 parity bar of the kd tree, mixed within its mixed bar, and the replayed
walk equal to the deciding one.  Against the reference kd tree the fast-mode
error (max |fast - exact| / Ldef0) stays within a small factor of the kd
tree's at each errTol."""
import ctypes as C

import numpy as np
import pytest

from tests.meshes import build_gpu, build_oracle, sphere_small, wing_small

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12  # max |GPU - oracle| / Ldef0, FP64 form
TOL_MIXED = 1e-8  # max |mixed - oracle| / Ldef0, same tree and decisions
ERR_FACTOR = 8.0  # Morton tree's fast-mode error over the kd tree's, at most
MORTON = {"treeBuild": "morton"}


def _mesh(name, planes=0):
    m = dict(sphere_small() if name == "sphere" else wing_small())
    if planes:
        m["symmetryPlanes"] = [[[0.0, 0.0, 0.0], [0.0, 0.0, 1.0]], [[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]],
                               [[0.0, 0.0, 0.0], [0.0, 1.0, 0.0]]][:planes]
    return m


@pytest.mark.parametrize("bucket", [1, 8, 64])
@pytest.mark.parametrize("name", ["sphere", "wing"])
def test_device_tree_equals_oracle(name, bucket, built_lib, oracle_lib):
    m = _mesh(name)
    opts = dict(MORTON, bucketSize=bucket)
    om = build_oracle(m, opts)
    g = build_gpu(m, opts)
    to, tg = om.tree(), g.getTree()
    for k in ("l", "u", "escape"):
        np.testing.assert_array_equal(to[k], tg[k])
    np.testing.assert_array_equal(to["dnum"] == 0, tg["isLeaf"] == 1)
    np.testing.assert_array_equal(to["X"], tg["X"])
    np.testing.assert_array_equal(to["oradius"], tg["oradius"])
    np.testing.assert_allclose(tg["Ai"], to["Ai"], rtol=1e-12)
    so, sg = om.surface(), g.getSurfaceState()
    np.testing.assert_array_equal(so["Xu0"], sg["Xu0"])
    np.testing.assert_array_equal(so["XuInd"], sg["XuInd"])
    np.testing.assert_allclose(g.getDenominator0(), om.den0(), rtol=1e-12)
    st = g.getStats()
    assert st["nTreeNodes"] == len(to["l"]) and st["treeBuildMs"] > 0.0


@pytest.mark.parametrize("mode", ["fast", "exact"])
@pytest.mark.parametrize("name,planes", [("sphere", 0), ("wing", 0), ("sphere", 1)])
def test_warp_fp64_matches_oracle(name, planes, mode, built_lib, oracle_lib):
    m = _mesh(name, planes)
    opts = dict(MORTON, evalMode=mode)
    om = build_oracle(m, opts)
    g = build_gpu(m, opts, precision="fp64")
    om.set_surface_coordinates(m["xs"])
    g.setSurfaceCoordinates(m["xs"])
    xo = om.warp()
    g.warpMesh()
    L = om.ldef0()
    assert np.abs(g.getWarpGrid().reshape(-1, 3) - xo).max() / L < TOL_FP64
    so, sg = om.stats(), g.getStats()
    assert sg["leafPairs"] == so["leafPairs"] and sg["approx"] == so["approx"]


@pytest.mark.parametrize("walk_lists", ["auto", "off"])
@pytest.mark.parametrize("name", ["sphere", "wing"])
def test_warp_mixed_matches_oracle(name, walk_lists, built_lib, oracle_lib):
    m = _mesh(name)
    om = build_oracle(m, MORTON)
    g = build_gpu(m, dict(MORTON, walkLists=walk_lists), precision="mixed")
    om.set_surface_coordinates(m["xs"])
    g.setSurfaceCoordinates(m["xs"])
    xo = om.warp()
    g.warpMesh()
    g.warpMesh()  # the second warp replays the recorded decisions
    assert np.abs(g.getWarpGrid().reshape(-1, 3) - xo).max() / om.ldef0() < TOL_MIXED
    so, sg = om.stats(), g.getStats()
    assert sg["leafPairs"] == so["leafPairs"] and sg["approx"] == so["approx"]


def test_replay_equals_decision_walk(built_lib):
    m = _mesh("wing")
    rng = np.random.default_rng(3)
    xs1 = m["xs"] + 1e-3 * rng.standard_normal(m["xs"].shape)
    out = []
    for wl in ("auto", "off"):
        g = build_gpu(m, dict(MORTON, walkLists=wl), precision="mixed")
        res = []
        for xs in (m["xs"], xs1):
            g.setSurfaceCoordinates(xs)
            g.warpMesh()
            res.append(g.getWarpGrid().copy())
        out.append(res)
    for a, b in zip(*out):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-9)])
def test_warp_deriv_matches_oracle(precision, tol, built_lib, oracle_lib):
    m = _mesh("wing")
    om = build_oracle(m, MORTON)
    g = build_gpu(m, MORTON, precision=precision)
    om.set_surface_coordinates(m["xs"])
    g.setSurfaceCoordinates(m["xs"])
    om.warp()
    g.warpMesh()
    dxv = np.random.default_rng(1).normal(size=m["xv0"].shape)
    do = om.warp_deriv(dxv)
    g.warpDeriv(dxv.ravel(), solverVec=False)
    assert np.abs(g.getdXs() - do).max() <= tol * np.abs(do).max()


def test_warp_deriv_fwd_matches_oracle(built_lib, oracle_lib):
    m = _mesh("sphere", 1)
    om = build_oracle(m, MORTON)
    g = build_gpu(m, MORTON, precision="fp64")
    om.set_surface_coordinates(m["xs"])
    g.setSurfaceCoordinates(m["xs"])
    om.warp()
    g.warpMesh()
    dxs = np.random.default_rng(2).normal(size=m["xs"].shape)
    do = om.warp_deriv_fwd(dxs)
    dg = np.asarray(g.warpDerivFwd(dxs.ravel(), solverVec=False)).reshape(-1, 3)
    assert np.abs(dg - do).max() <= 1e-10 * np.abs(do).max()


def test_single_leaf_surface(built_lib, oracle_lib):
    # fewer unique points than bucketSize + 1: the tree is one leaf
    m = _mesh("wing")
    xs = m["xs"]
    keep = m["conn"][:8]  # the first two quads
    used = np.unique(keep)
    remap = -np.ones(len(m["pts"]), dtype=np.int64)
    remap[used] = np.arange(len(used))
    small = {"pts": m["pts"][used], "conn": remap[keep], "faceSizes": np.array([4, 4]), "xv0": m["xv0"][:500],
             "xs": xs[used]}
    om = build_oracle(small, MORTON)
    g = build_gpu(small, MORTON, precision="fp64")
    assert len(g.getTree()["l"]) == 1
    om.set_surface_coordinates(small["xs"])
    g.setSurfaceCoordinates(small["xs"])
    xo = om.warp()
    g.warpMesh()
    assert np.abs(g.getWarpGrid().reshape(-1, 3) - xo).max() / om.ldef0() < TOL_FP64


def test_invalid_tree_build_rejected(built_lib):
    from idwarp_gb300 import _lib

    g = build_gpu(_mesh("sphere"), MORTON)
    o = _lib.idw_options()
    g.lib.idw_default_options(C.byref(o))
    o.treeBuild = 7
    assert g.lib.idw_set_options(g.ctx, C.byref(o)) == _lib.IDW_ERR_ARG


@pytest.mark.parametrize("name", ["sphere", "wing"])
def test_fast_error_report(name, built_lib):
    # the error report: fast mode against exact mode with each tree, mixed
    m = _mesh(name)
    ge = build_gpu(m, {"evalMode": "exact"}, precision="mixed")
    ge.setSurfaceCoordinates(m["xs"])
    ge.warpMesh()
    xe = ge.getWarpGrid().copy()
    L = ge.getStats()["Ldef0"]
    ex_m = build_gpu(m, dict(MORTON, evalMode="exact"), precision="mixed")
    ex_m.setSurfaceCoordinates(m["xs"])
    ex_m.warpMesh()
    assert np.abs(ex_m.getWarpGrid() - xe).max() / L < TOL_MIXED  # same sums, other order
    for tol in (1e-3, 1e-4, 1e-5):
        err = {}
        for tb in ("kd", "morton"):
            g = build_gpu(m, {"treeBuild": tb, "errTol": tol}, precision="mixed")
            g.setSurfaceCoordinates(m["xs"])
            g.warpMesh()
            err[tb] = np.abs(g.getWarpGrid() - xe).max() / L
        assert err["morton"] <= ERR_FACTOR * err["kd"], (tol, err)


@pytest.mark.parametrize("opts,planes", [
    ({"aExp": 2.5, "bExp": 4.5}, 0),   # real-valued exponents: the third weight law
    ({"aExp": 4.0, "bExp": 6.0}, 1),
    ({"LdefFact": 100.0}, 0),
    ({}, 3),
])
@pytest.mark.parametrize("precision,tol", [("fp64", TOL_FP64), ("mixed", TOL_MIXED)])
def test_laws_and_planes(opts, planes, precision, tol, built_lib, oracle_lib):
    m = _mesh("sphere", planes)
    o = dict(MORTON, **opts)
    om = build_oracle(m, o)
    g = build_gpu(m, o, precision=precision)
    om.set_surface_coordinates(m["xs"])
    g.setSurfaceCoordinates(m["xs"])
    xo = om.warp()
    g.warpMesh()
    if precision == "mixed" and opts.get("aExp", 3.0) % 1.0:
        tol = 1e-7  # real-valued exponents: FP32 powers throughout, as with the kd tree
    assert np.abs(g.getWarpGrid().reshape(-1, 3) - xo).max() / om.ldef0() < tol
    so, sg = om.stats(), g.getStats()
    assert sg["leafPairs"] == so["leafPairs"] and sg["approx"] == so["approx"]


def test_deterministic_reverse_product(built_lib):
    # the deterministic mode on the Morton tree: bitwise repeatable, within
    # the atomics' rounding of the default
    m = _mesh("wing", 1)
    dxv = np.random.default_rng(8).standard_normal(m["xv0"].shape)
    out = []
    for det in (True, True, False):
        g = build_gpu(m, dict(MORTON, deterministic=det), precision="mixed")
        g.setSurfaceCoordinates(m["xs"])
        g.warpMesh()
        g.warpDeriv(dxv.ravel(), solverVec=False)
        out.append(g.getdXs().copy())
    np.testing.assert_array_equal(out[0], out[1])
    assert np.abs(out[0] - out[2]).max() <= 1e-12 * np.abs(out[2]).max()
