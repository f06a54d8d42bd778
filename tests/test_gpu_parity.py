"""GPU parity: the CUDA library through its C ABI against the oracle.

Integer/index state (tree, permutation, counts) must match exactly; floating
point results within the tolerances written in each test.  FP64 GPU vs FP64
oracle differs only by operation order/FMA contraction and by integer powers
computed by multiplication instead of pow(), so the bar is ~1e-12 relative.
"""
import numpy as np
import pytest

from tests.meshes import build_gpu, build_oracle, sphere_small, wing_small

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-12  # max |GPU - oracle| / Ldef for the FP64 form


@pytest.fixture(scope="module")
def sphere():
    return sphere_small()


@pytest.fixture(scope="module")
def wing():
    return wing_small()


def _ldef(om):
    return om.ldef0()


@pytest.mark.parametrize("case", ["sphere", "wing"])
def test_tree_matches_oracle(case, sphere, wing, built_lib, oracle_lib):
    m = sphere if case == "sphere" else wing
    om = build_oracle(m)
    g = build_gpu(m)
    to, tg = om.tree(), g.getTree()
    np.testing.assert_array_equal(to["l"], tg["l"])
    np.testing.assert_array_equal(to["u"], tg["u"])
    np.testing.assert_array_equal(to["escape"], tg["escape"])
    np.testing.assert_array_equal(to["dnum"] == 0, tg["isLeaf"] == 1)
    np.testing.assert_allclose(tg["X"], to["X"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(tg["oradius"], to["oradius"], rtol=1e-13)
    np.testing.assert_allclose(tg["Ai"], to["Ai"], rtol=1e-12)
    interior = to["dnum"] != 0
    # err_j = RMS(dExact - dApprox): at large radii dExact and dApprox agree to
    # many digits, so the summation order (chunked on the GPU) moves err by
    # ~1e-16 of dExact; dExact itself is bounded by the innermost error here.
    eo, eg = to["err"][interior], tg["err"][interior]
    scale = np.maximum(eo[:, :1], 1e-300)
    assert np.all(np.abs(eg - eo) <= 1e-10 * scale + 1e-9 * np.abs(eo)), np.max(np.abs(eg - eo) / scale)
    so, sg = om.surface(), g.getSurfaceState()
    np.testing.assert_array_equal(so["Xu0"], sg["Xu0"])
    np.testing.assert_array_equal(so["XuInd"], sg["XuInd"])
    np.testing.assert_array_equal(so["isCorner"], sg["isCorner"])
    np.testing.assert_allclose(sg["Ai"], so["Ai"], rtol=1e-12)
    np.testing.assert_allclose(sg["normals0"], so["normals0"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(g.getDenominator0(), om.den0(), rtol=1e-12)


@pytest.mark.parametrize("case", ["sphere", "wing"])
def test_nodal_properties_match_oracle(case, sphere, wing, built_lib, oracle_lib):
    m = sphere if case == "sphere" else wing
    om = build_oracle(m)
    g = build_gpu(m)
    om.set_surface_coordinates(m["xs"])
    g.setSurfaceCoordinates(m["xs"])
    Mo, Bo = om.nodal()
    Mg, Bg = g.getNodalProperties()
    np.testing.assert_allclose(Mg, Mo, atol=1e-13)
    np.testing.assert_allclose(Bg, Bo, atol=1e-12)


@pytest.mark.parametrize("mode", ["fast", "exact"])
@pytest.mark.parametrize("case", ["sphere", "wing"])
def test_warp_fp64_matches_oracle(case, mode, sphere, wing, built_lib, oracle_lib):
    m = sphere if case == "sphere" else wing
    om = build_oracle(m, {"evalMode": mode})
    g = build_gpu(m, {"evalMode": mode}, precision="fp64")
    om.set_surface_coordinates(m["xs"])
    g.setSurfaceCoordinates(m["xs"])
    xo = om.warp()
    g.warpMesh()
    xg = g.getWarpGrid().reshape(-1, 3)
    L = _ldef(om)
    assert np.abs(xg - xo).max() / L < TOL_FP64
    so, sg = om.stats(), g.getStats()
    # identical decisions -> identical work counts
    assert sg["leafPairs"] == so["leafPairs"]
    assert sg["approx"] == so["approx"]


@pytest.mark.parametrize("mode", ["fast", "exact"])
@pytest.mark.parametrize("case", ["sphere", "wing"])
def test_warp_deriv_fp64_matches_oracle(case, mode, sphere, wing, built_lib, oracle_lib):
    m = sphere if case == "sphere" else wing
    om = build_oracle(m, {"evalMode": mode})
    g = build_gpu(m, {"evalMode": mode}, precision="fp64")
    om.set_surface_coordinates(m["xs"])
    g.setSurfaceCoordinates(m["xs"])
    om.warp()
    g.warpMesh()
    rng = np.random.default_rng(1)
    dxv = rng.normal(size=m["xv0"].shape)
    do = om.warp_deriv(dxv)
    g.warpDeriv(dxv.ravel(), solverVec=False)
    dg = g.getdXs()
    scale = np.abs(do).max()
    assert np.abs(dg - do).max() <= 1e-10 * scale


def test_warp_deriv_batch_matches_single(wing, built_lib):
    g = build_gpu(wing, precision="fp64")
    g.setSurfaceCoordinates(wing["xs"])
    g.warpMesh()
    rng = np.random.default_rng(4)
    seeds = rng.normal(size=(5,) + wing["xv0"].shape)
    batch = g.warpDerivBatch(seeds)
    for s in range(5):
        g.warpDeriv(seeds[s].ravel(), solverVec=False)
        single = g.getdXs()
        np.testing.assert_allclose(batch[s], single, rtol=1e-12, atol=1e-12 * np.abs(single).max())


@pytest.mark.parametrize("precision,mode", [("fp64", "fast"), ("fp64", "exact"), ("mixed", "fast"),
                                            ("mixed", "exact")])
def test_rigid_rotation_gpu(precision, mode, built_lib):
    # an open tube turned about its axis: every node has M_i = R, b_i = 0, so
    # the volume turns by R (the mixed form carries R - I in its reference
    # motion, leaving nothing to round in FP32)
    from tests.meshes import open_cylinder, rotation_z

    m = open_cylinder()
    R = rotation_z(10.0)
    g = build_gpu(m, {"evalMode": mode}, sym=False, precision=precision)
    g.setSurfaceCoordinates(m["pts"] @ R.T)
    g.warpMesh()
    tol = 1e-12 if precision == "fp64" else 1e-10
    np.testing.assert_allclose(g.getWarpGrid().reshape(-1, 3), m["xv0"] @ R.T, rtol=0, atol=tol)


def test_rigid_translation_gpu(sphere, built_lib):
    g = build_gpu(sphere, precision="fp64")
    t = np.array([0.25, 0.5, -0.125])
    g.setSurfaceCoordinates(sphere["pts"] + t)
    g.warpMesh()
    xv = g.getWarpGrid().reshape(-1, 3)
    np.testing.assert_allclose(xv - sphere["xv0"], np.broadcast_to(t, xv.shape), atol=1e-12)


def test_options_take_effect_like_reference(wing, built_lib, oracle_lib):
    # LdefFact, alpha, useRotations act at the next warp; errTol too.
    opts = {"LdefFact": 2.0, "alpha": 0.5, "useRotations": False, "errTol": 5e-4}
    om = build_oracle(wing, opts)
    g = build_gpu(wing, opts, precision="fp64")
    om.set_surface_coordinates(wing["xs"])
    g.setSurfaceCoordinates(wing["xs"])
    xo = om.warp()
    g.warpMesh()
    assert np.abs(g.getWarpGrid().reshape(-1, 3) - xo).max() / om.ldef0() < TOL_FP64


def test_solver_ordering_roundtrip(wing, built_lib):
    g = build_gpu(wing, precision="fp64")
    n = 3 * len(wing["xv0"])
    rng = np.random.default_rng(8)
    ind = rng.permutation(n)[: n // 2]
    g.setExternalMeshIndices(ind)
    g.setSurfaceCoordinates(wing["xs"])
    g.warpMesh()
    np.testing.assert_array_equal(g.getSolverGrid(), g.getWarpGrid()[ind])
    # the reverse of a gather is a scatter-add
    v = rng.normal(size=len(ind))
    w = g._solverToWarp(v)
    ref = np.zeros(n)
    np.add.at(ref, ind, v)
    np.testing.assert_allclose(w, ref, atol=0)


def test_errors_are_raised(sphere, built_lib):
    from idwarp_gb300 import Error
    from idwarp_gb300._lib import LibraryError

    g = build_gpu(sphere, precision="fp64")
    with pytest.raises(Error):
        g.setSurfaceCoordinates(sphere["pts"][:-1])
    bad = sphere["pts"].copy()
    bad[3, 1] = np.nan
    with pytest.raises(Error):
        g.setSurfaceCoordinates(bad)
    with pytest.raises(LibraryError):
        g.warpDeriv(np.zeros(3 * len(sphere["xv0"])), solverVec=False)  # before warpMesh


TOL_MIXED = 1e-8  # max |mixed - FP64| / Ldef (precision error on the same tree and decisions)
# warpDeriv, max |mixed - FP64| / max |dXs|: the double-float adjoint (the
# default) and the FP32 one (adjointPrecision "fast")
TOL_DERIV = {"precise": 1e-9, "fast": 1e-6}


@pytest.mark.parametrize("mode", ["fast", "exact"])
@pytest.mark.parametrize("case", ["sphere", "wing"])
def test_mixed_matches_fp64_same_decisions(case, mode, sphere, wing, built_lib):
    m = sphere if case == "sphere" else wing
    g64 = build_gpu(m, {"evalMode": mode}, precision="fp64")
    g32 = build_gpu(m, {"evalMode": mode}, precision="mixed")
    for g in (g64, g32):
        g.setSurfaceCoordinates(m["xs"])
        g.warpMesh()
    x64 = g64.getWarpGrid().reshape(-1, 3)
    x32 = g32.getWarpGrid().reshape(-1, 3)
    s64, s32 = g64.getStats(), g32.getStats()
    assert s32["leafPairs"] == s64["leafPairs"]
    assert s32["approx"] == s64["approx"]
    err = np.abs(x32 - x64).max() / s64["Ldef0"]
    assert err < TOL_MIXED, err


def test_mixed_matches_oracle_fast(wing, built_lib, oracle_lib):
    om = build_oracle(wing)
    g = build_gpu(wing, precision="mixed")
    om.set_surface_coordinates(wing["xs"])
    g.setSurfaceCoordinates(wing["xs"])
    xo = om.warp()
    g.warpMesh()
    err = np.abs(g.getWarpGrid().reshape(-1, 3) - xo).max() / om.ldef0()
    assert err < TOL_MIXED, err


def test_mixed_general_exponents(sphere, built_lib, oracle_lib):
    # non-(3,5) integer exponents and real exponents take the other weight paths
    for a, b in ((4.0, 6.0), (2.5, 4.5)):
        opts = {"aExp": a, "bExp": b}
        om = build_oracle(sphere, opts)
        g64 = build_gpu(sphere, opts, precision="fp64")
        g32 = build_gpu(sphere, opts, precision="mixed")
        om.set_surface_coordinates(sphere["xs"])
        xo = om.warp()
        for g, tol in ((g64, TOL_FP64), (g32, 1e-7)):
            g.setSurfaceCoordinates(sphere["xs"])
            g.warpMesh()
            err = np.abs(g.getWarpGrid().reshape(-1, 3) - xo).max() / om.ldef0()
            assert err < tol, (a, b, err)


@pytest.mark.parametrize("adj", ["precise", "fast"])
def test_mixed_deriv_matches_oracle(adj, wing, built_lib, oracle_lib):
    # the mixed warpDeriv against the oracle: the fast form divides by the
    # mixed warp's denominator (FP32 weights, ~1e-7 relative per node), the
    # precise form by its own double-float denominator
    om = build_oracle(wing)
    g = build_gpu(wing, {"adjointPrecision": adj}, precision="mixed")
    om.set_surface_coordinates(wing["xs"])
    g.setSurfaceCoordinates(wing["xs"])
    om.warp()
    g.warpMesh()
    rng = np.random.default_rng(2)
    dxv = rng.normal(size=wing["xv0"].shape)
    do = om.warp_deriv(dxv)
    g.warpDeriv(dxv.ravel(), solverVec=False)
    err = np.abs(g.getdXs() - do).max() / np.abs(do).max()
    assert err <= TOL_DERIV[adj], err


@pytest.mark.parametrize("adj", ["precise", "fast"])
def test_mixed_deriv_every_seed_group(adj, wing, built_lib):
    # 29 seeds = groups of 16, 8, 4 and 1 (fast) or 16, 4, 4, 4, 1 (precise):
    # every form of the mixed adjoint's warp reduction against the FP64 adjoint
    g64 = build_gpu(wing, precision="fp64")
    g32 = build_gpu(wing, {"adjointPrecision": adj}, precision="mixed")
    seeds = np.random.default_rng(19).normal(size=(29,) + wing["xv0"].shape)
    out = []
    for g in (g64, g32):
        g.setSurfaceCoordinates(wing["xs"])
        g.warpMesh()
        out.append(g.warpDerivBatch(seeds))
    for lo, hi in ((0, 16), (16, 24), (24, 28), (28, 29)):
        ref = out[0][lo:hi]
        assert np.abs(out[1][lo:hi] - ref).max() <= TOL_DERIV[adj] * np.abs(ref).max(), (lo, hi)


@pytest.mark.parametrize("adj", ["precise", "fast"])
@pytest.mark.parametrize("mode", ["fast", "exact"])
def test_mixed_deriv_batch_matches_fp64(mode, adj, wing, built_lib):
    # the mixed adjoint (S seeds sharing one walk) against the FP64 adjoint
    g64 = build_gpu(wing, {"evalMode": mode}, precision="fp64")
    g32 = build_gpu(wing, {"evalMode": mode, "adjointPrecision": adj}, precision="mixed")
    rng = np.random.default_rng(9)
    seeds = rng.normal(size=(6,) + wing["xv0"].shape)
    out = []
    for g in (g64, g32):
        g.setSurfaceCoordinates(wing["xs"])
        g.warpMesh()
        out.append(g.warpDerivBatch(seeds))
    scale = np.abs(out[0]).max()
    assert np.abs(out[1] - out[0]).max() <= TOL_DERIV[adj] * scale, np.abs(out[1] - out[0]).max() / scale


@pytest.mark.parametrize("mode", ["fast", "exact"])
@pytest.mark.parametrize("case", ["sphere", "wing"])
def test_warp_deriv_fwd_fp64_matches_oracle(case, mode, sphere, wing, built_lib, oracle_lib):
    # warpDerivFwd against the oracle's complex-step tangent (exact to rounding)
    m = sphere if case == "sphere" else wing
    om = build_oracle(m, {"evalMode": mode})
    g = build_gpu(m, {"evalMode": mode}, precision="fp64")
    om.set_surface_coordinates(m["xs"])
    g.setSurfaceCoordinates(m["xs"])
    om.warp()
    rng = np.random.default_rng(11)
    dxs = rng.normal(size=m["pts"].shape)
    do = om.warp_deriv_fwd(dxs)
    dg = g.warpDerivFwd(dxs, solverVec=False).reshape(-1, 3)
    assert np.abs(dg - do).max() <= 1e-10 * np.abs(do).max()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("mixed", 1e-6)])
def test_warp_deriv_dot_product(precision, tol, wing, built_lib):
    # <dXv, J dXs> = <J^T dXv, dXs> between warpDerivFwd and warpDeriv
    g = build_gpu(wing, precision=precision)
    g.setSurfaceCoordinates(wing["xs"])
    g.warpMesh()
    rng = np.random.default_rng(12)
    dxs = rng.normal(size=wing["pts"].shape)
    dxv = rng.normal(size=3 * len(wing["xv0"]))
    fwd = g.warpDerivFwd(dxs, solverVec=False)
    g.warpDeriv(dxv, solverVec=False)
    rev = g.getdXs()
    a, b = float(np.dot(dxv, fwd)), float(np.sum(rev * dxs))
    # relative to the sums of |terms| (the products cancel to ~1% of them)
    scale = max(float(np.sum(np.abs(dxv * fwd))), float(np.sum(np.abs(rev * dxs))))
    assert abs(a - b) <= tol * scale, (a, b, scale)


@pytest.mark.parametrize("mode", ["fast", "exact"])
def test_warp_deriv_fwd_mixed_matches_fp64(mode, sphere, built_lib):
    g64 = build_gpu(sphere, {"evalMode": mode}, precision="fp64")
    g32 = build_gpu(sphere, {"evalMode": mode}, precision="mixed")
    rng = np.random.default_rng(13)
    dxs = rng.normal(size=sphere["pts"].shape)
    out = []
    for g in (g64, g32):
        g.setSurfaceCoordinates(sphere["xs"])
        out.append(g.warpDerivFwd(dxs, solverVec=False))
    assert np.abs(out[1] - out[0]).max() <= 1e-6 * np.abs(out[0]).max()
    # the mixed tangent walk leaves the mesh state ready for the next warp
    g32.warpMesh()
    g64.warpMesh()
    err = np.abs(g32.getWarpGrid() - g64.getWarpGrid()).max() / g64.getStats()["Ldef0"]
    assert err < TOL_MIXED


@pytest.mark.parametrize("mode", ["fast", "exact"])
@pytest.mark.parametrize("case", ["sphere", "wing"])
def test_mixed_batch_walk_matches_fp64(case, mode, sphere, wing, built_lib):
    # five surfaces: one shared walk of four, then one of one
    from idwarp_gb300 import synthetic as S

    m = sphere if case == "sphere" else wing
    pert = S.sphere_perturbation if case == "sphere" else S.wing_perturbation
    surfaces = np.stack([pert(m["pts"], seed=200 + i) for i in range(5)])
    g64 = build_gpu(m, {"evalMode": mode}, precision="fp64")
    g32 = build_gpu(m, {"evalMode": mode}, precision="mixed")
    out = g32.warpMeshBatch(surfaces)
    st = g32.getStats()
    L = g64.getStats()["Ldef0"]
    for b in range(5):
        g64.setSurfaceCoordinates(surfaces[b])
        g64.warpMesh()
        err = np.abs(out[b] - g64.getWarpGrid().reshape(-1, 3)).max() / L
        assert err < TOL_MIXED, (b, err)
    # the stored surface and grid of the mesh are left alone
    g32.setSurfaceCoordinates(m["xs"])
    g32.warpMesh()
    g64.setSurfaceCoordinates(m["xs"])
    g64.warpMesh()
    assert np.abs(g32.getWarpGrid() - g64.getWarpGrid()).max() / L < TOL_MIXED
    # decisions are those of one walk per group
    s64 = g64.getStats()
    assert st["leafPairs"] == 2 * s64["leafPairs"]
    assert st["approx"] == 2 * s64["approx"]


def test_autotune_keeps_results(wing, built_lib):
    from idwarp_gb300 import synthetic as S

    g = build_gpu(wing, precision="mixed")
    g.setSurfaceCoordinates(wing["xs"])
    g.warpMesh()
    surfaces = np.stack([S.wing_perturbation(wing["pts"], seed=60 + i) for i in range(3)])
    seeds = np.random.default_rng(61).normal(size=(5,) + wing["xv0"].shape)
    before = (g.warpMeshBatch(surfaces), g.warpDerivBatch(seeds))
    t = g.autotune(nSurfaces=3, nSeeds=5)
    assert t["batchGroup"] in (1, 2, 3, 4) and t["adjMaxGroup"] in (16, 8, 4)
    assert all(ms > 0 for ms in t["batchMs"][:3])
    g.setSurfaceCoordinates(wing["xs"])
    g.warpMesh()
    after = (g.warpMeshBatch(surfaces), g.warpDerivBatch(seeds))
    L = g.getStats()["Ldef0"]
    assert np.abs(after[0] - before[0]).max() / L < 1e-9
    assert np.abs(after[1] - before[1]).max() <= 1e-6 * np.abs(before[1]).max()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-13), ("mixed", 1e-7)])
def test_tangent_batch_matches_single(precision, tol, wing, built_lib):
    # five directions: one shared walk of four, then one of one (mixed)
    g = build_gpu(wing, precision=precision)
    g.setSurfaceCoordinates(wing["xs"])
    g.warpMesh()
    rng = np.random.default_rng(71)
    dirs = rng.normal(size=(5,) + wing["pts"].shape)
    batch = g.warpDerivFwdBatch(dirs)
    for d in range(5):
        single = g.warpDerivFwd(dirs[d], solverVec=False).reshape(-1, 3)
        assert np.abs(batch[d] - single).max() <= tol * np.abs(single).max(), d
    # the warp itself is untouched
    x = g.getWarpGrid()
    g.warpMesh()
    np.testing.assert_array_equal(g.getWarpGrid(), x)
