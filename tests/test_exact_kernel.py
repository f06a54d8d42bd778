"""Exact mode (evalMode = exact) through the tiled N-body kernel against the
mixed tree walk's exact mode (option exactSchedule "tiled" / "walk"): the two
schedules evaluate the same terms with the same arithmetic in the same order,
so positions and counters agree bit for bit.
Leaves larger than a shared-memory tile, one-point leaves, several mirrors,
other weight laws and the double-float leaf gate are covered; agreement with
the oracle's exact sum is in test_gpu_parity."""
import numpy as np
import pytest

from tests.meshes import build_gpu, build_oracle, sphere_small, wing_small

pytestmark = pytest.mark.gpu

CASES = [
    ("wing", {}, 0),
    ("sphere", {}, 0),
    ("sphere", {"bucketSize": 1}, 0),
    ("sphere", {"bucketSize": 300}, 0),  # leaves above the 256-point tile
    ("sphere", {}, 3),
    ("sphere", {"aExp": 4.0, "bExp": 6.0}, 0),
    ("sphere", {"aExp": 2.5, "bExp": 4.5}, 0),
    ("wing", {"LdefFact": 100.0}, 0),
    ("wing", {"mixedGate": 1e-6}, 0),  # most leaves re-summed in double-float
]


def _mesh(which, planes):
    m = dict(sphere_small() if which == "sphere" else wing_small())
    if planes:
        m["symmetryPlanes"] = [[[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]], [[0.0, 0.0, 0.0], [0.0, 1.0, 0.0]],
                               [[0.0, 0.0, 0.0], [0.0, 0.0, 1.0]]][:planes]
    return m


def _warp(m, opts):
    g = build_gpu(m, dict(opts, evalMode="exact"), precision="mixed")
    g.setSurfaceCoordinates(m["xs"])
    g.warpMesh()
    return g.getWarpGrid(), g.getStats()


@pytest.mark.parametrize("which,opts,planes", CASES)
def test_tiled_exact_equals_walk(which, opts, planes, built_lib):
    m = _mesh(which, planes)
    x_tiled, st_tiled = _warp(m, dict(opts, exactSchedule="tiled"))
    x_walk, st_walk = _warp(m, dict(opts, exactSchedule="walk"))
    np.testing.assert_array_equal(x_tiled, x_walk)
    for k in ("leafPairs", "visited", "preciseTerms"):
        assert st_tiled[k] == st_walk[k], k
    assert st_tiled["approx"] == 0
    assert st_tiled["leafPairs"] == st_tiled["nVol"] * st_tiled["nLoop"] * st_tiled["nUnique"]


def test_four_nodes_per_thread_on_a_larger_mesh(built_lib):
    # 245k volume nodes: a full wave of 512-node blocks, so the tiled kernel
    # carries four nodes per thread
    from idwarp_gb300 import synthetic as S

    m = S.wing_shell(ni=201, nj=61, nk=20, first=1e-5, far=25.0)
    m["xs"] = S.wing_perturbation(m["pts"], seed=2)
    x_tiled, st_tiled = _warp(m, {"exactSchedule": "tiled"})
    x_walk, st_walk = _warp(m, {"exactSchedule": "walk"})
    np.testing.assert_array_equal(x_tiled, x_walk)
    assert st_tiled["leafPairs"] == st_walk["leafPairs"]
    assert st_tiled["preciseTerms"] == st_walk["preciseTerms"]


def test_diagnostics_use_the_walk(built_lib):
    # the slot counts exist only in the walk: diagnostics select it
    m = wing_small()
    x_tiled, _ = _warp(m, {"exactSchedule": "tiled"})
    x_diag, st = _warp(m, {"exactSchedule": "tiled", "diagnostics": 1})
    np.testing.assert_array_equal(x_tiled, x_diag)
    assert st["warpLeafSlots"] > 0


def test_tiled_exact_matches_oracle_with_gate_forced(built_lib, oracle_lib):
    # every leaf through the double-float path still matches the FP64 exact sum
    m = wing_small()
    om = build_oracle(m, {"evalMode": "exact"})
    om.set_surface_coordinates(m["xs"])
    xo = om.warp()
    x, st = _warp(m, {"mixedGate": 1e-6, "exactSchedule": "tiled"})
    assert st["preciseTerms"] > 0
    assert np.abs(x.reshape(-1, 3) - xo).max() / om.ldef0() < 1e-9


def test_tiled_exact_tangent_equals_walk(built_lib):
    # warpDerivFwd in exact mode runs the same evaluation with the tangent
    # nodal properties: the tiled schedule gives the walk's bits
    m = wing_small()
    dxs = np.random.default_rng(61).normal(size=m["pts"].shape)
    out = {}
    for sched in ("tiled", "walk"):
        g = build_gpu(m, {"evalMode": "exact", "exactSchedule": sched}, precision="mixed")
        g.setSurfaceCoordinates(m["xs"])
        out[sched] = g.warpDerivFwd(dxs, solverVec=False)
    np.testing.assert_array_equal(out["tiled"], out["walk"])


def _deriv(m, opts, precision, dxv):
    g = build_gpu(m, dict(opts, evalMode="exact"), precision=precision)
    g.setSurfaceCoordinates(m["xs"])
    g.warpMesh()
    if dxv.ndim == 1:
        g.warpDeriv(dxv, solverVec=False)
        return g.getdXs()
    return g.warpDerivBatch(dxv)


@pytest.mark.parametrize("which,planes", [("wing", 0), ("sphere", 3)])
def test_tiled_exact_adjoint(which, planes, built_lib):
    # the reverse product in exact mode (the FP32 form, whose one-seed calls
    # the tiled kernel serves): tiled (per-warp moment reduction) against the
    # walk and against the FP64 form; sums in another order, so within the
    # FP32 form's tolerance rather than bitwise
    m = _mesh(which, planes)
    dxv = np.random.default_rng(71).normal(size=3 * len(m["xv0"]))
    ref = _deriv(m, {}, "fp64", dxv)
    tiled = _deriv(m, {"exactSchedule": "tiled", "adjointPrecision": "fast"}, "mixed", dxv)
    walk = _deriv(m, {"exactSchedule": "walk", "adjointPrecision": "fast"}, "mixed", dxv)
    scale = np.abs(ref).max()
    assert np.abs(tiled - walk).max() <= 1e-6 * scale
    assert np.abs(tiled - ref).max() <= 1e-6 * scale


def test_tiled_exact_adjoint_several_seeds(built_lib):
    m = wing_small()
    dxv = np.random.default_rng(72).normal(size=(3, len(m["xv0"]), 3))
    tiled = _deriv(m, {"exactSchedule": "tiled", "adjointPrecision": "fast"}, "mixed", dxv)
    walk = _deriv(m, {"exactSchedule": "walk", "adjointPrecision": "fast"}, "mixed", dxv)
    assert tiled.shape == walk.shape
    assert np.abs(tiled - walk).max() <= 1e-6 * np.abs(walk).max()


def test_tiled_exact_batch_equals_single_warps(built_lib):
    # warpMeshBatch in exact mode runs the tiled kernel once per surface: the
    # same bits as one warpMesh per surface
    from idwarp_gb300 import synthetic as S

    m = wing_small()
    surf = np.stack([S.wing_perturbation(m["pts"], seed=300 + i) for i in range(3)])
    g = build_gpu(m, {"evalMode": "exact", "exactSchedule": "tiled"}, precision="mixed")
    batch = g.warpMeshBatch(surf)
    for i in range(3):
        g.setSurfaceCoordinates(surf[i])
        g.warpMesh()
        np.testing.assert_array_equal(batch[i].ravel(), g.getWarpGrid())
