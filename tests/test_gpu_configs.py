"""GPU against the oracle at the sizes of the measured configurations.

* S1: the whole cubed-sphere O-grid (6 x 18 x 18 quad cells, 48 stretched
  radial layers out to r = 20: 95,354 volume nodes, 2,166 surface points),
  5 deg rotation about z plus four Gaussian bumps (seed 0), errTol 1e-4,
  fast and exact mode, and one warpDeriv seed dXv ~ N(0, 1) (seed 1).
* W: the 2M-node NACA0012 half-wing shell (401 x 101 x 50, one symmetry
  plane), twist + FFD perturbation (seed 2), warped whole on the GPU and
  compared with the oracle on a seeded sample of 20,000 volume nodes (the
  volume nodes are independent given the surface, so the sample's oracle
  result is the full mesh's at those nodes); GPU meshes of just the sampled
  nodes give the decision counts for the same nodes.
* Both with the reference's kd tree and with the GPU-built Morton tree
  (option treeBuild "morton", against the oracle's restatement of it).

Bars: FP64 1e-12 Ldef, mixed 1e-8 Ldef (max over nodes of the largest
coordinate error), widened to 4x the case's rounding sensitivity where that
is larger (the oracle's timing build, with FMA contraction, against its
checker build, without).  Fast-mode decision counts (leaf pairs, cluster
approximations) must be equal.  The procedure follows the reference's
regression test (tests/test_USMesh.py:24-102: warp, then warpDeriv of a
seed, per mesh).
"""
import numpy as np
import pytest

from tests.meshes import build_gpu, build_oracle

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "mixed": 1e-8}
# warpDeriv, relative to max |dXs|: FP64 against the oracle, mixed against
# the FP64 adjoint of the same mesh
TOL_DERIV = {"fp64": 1e-10, "mixed": 1e-9}
W_SAMPLE = 20000


def _sensitivity(m, opts, idx=None):
    """max |timing build - checker build| / Ldef of the oracle on (a sample of) m."""
    from oracle.pyoracle import OracleMesh, timing_library

    sub = dict(m)
    if idx is not None:
        sub["xv0"] = m["xv0"][idx]
    om = build_oracle(sub, opts)
    om.set_surface_coordinates(m["xs"])
    xo = om.warp()
    L = om.ldef0()
    ot = OracleMesh(dict(om.opts), library=timing_library())
    ot.set_volume(sub["xv0"])
    planes = m.get("symmetryPlanes")
    if planes:
        ot.set_symmetry(np.array([p[0] for p in planes]), np.array([p[1] for p in planes]))
    else:
        ot.set_symmetry(np.zeros((0, 3)), np.zeros((0, 3)))
    ot.set_surface_definition(m["pts"], m["conn"], m["faceSizes"])
    ot.set_surface_coordinates(m["xs"])
    return om, xo, L, float(np.abs(ot.warp() - xo).max() / L)


@pytest.fixture(scope="module")
def s1():
    from idwarp_gb300 import synthetic as S

    m = S.sphere_ogrid(n=18, layers=48)
    m["xs"] = S.sphere_perturbation(m["pts"], seed=0)
    return m


@pytest.fixture(scope="module")
def w():
    from idwarp_gb300 import synthetic as S

    m = S.wing_shell(401, 101, 50, first=1e-5, far=25.0)
    m["xs"] = S.wing_perturbation(m["pts"], seed=2)
    m["idx"] = np.sort(np.random.default_rng(12).choice(len(m["xv0"]), W_SAMPLE, replace=False))
    return m


@pytest.mark.parametrize("tree", ["kd", "morton"])
@pytest.mark.parametrize("mode", ["fast", "exact"])
def test_s1_warp_matches_oracle(mode, tree, s1, built_lib, oracle_lib):
    # tree "morton": the GPU-built tree against the oracle's restatement of it
    assert len(s1["xv0"]) == 95354 and len(s1["pts"]) == 2166
    opts = {"evalMode": mode, "treeBuild": tree}
    om, xo, L, sens = _sensitivity(s1, opts)
    so = om.stats()
    for prec in ("fp64", "mixed"):
        g = build_gpu(s1, opts, precision=prec)
        g.setSurfaceCoordinates(s1["xs"])
        g.warpMesh()
        err = np.abs(g.getWarpGrid().reshape(-1, 3) - xo).max() / L
        assert err <= max(TOL[prec], 4 * sens), (prec, err, sens)
        sg = g.getStats()
        assert (sg["leafPairs"], sg["approx"]) == (so["leafPairs"], so["approx"]), prec


@pytest.mark.parametrize("mode", ["fast", "exact"])
def test_s1_warp_deriv(mode, s1, built_lib, oracle_lib):
    om = build_oracle(s1, {"evalMode": mode})
    om.set_surface_coordinates(s1["xs"])
    om.warp()
    dxv = np.random.default_rng(1).normal(size=s1["xv0"].shape)
    do = om.warp_deriv(dxv)
    out = {}
    for prec in ("fp64", "mixed"):
        g = build_gpu(s1, {"evalMode": mode}, precision=prec)
        g.setSurfaceCoordinates(s1["xs"])
        g.warpMesh()
        g.warpDeriv(dxv.ravel(), solverVec=False)
        out[prec] = g.getdXs()
    scale = np.abs(do).max()
    assert np.abs(out["fp64"] - do).max() <= TOL_DERIV["fp64"] * scale
    assert np.abs(out["mixed"] - out["fp64"]).max() <= TOL_DERIV["mixed"] * scale


@pytest.mark.parametrize("mode,tree", [("fast", "kd"), ("exact", "kd"), ("fast", "morton")])
def test_w_sample_matches_oracle(mode, tree, w, built_lib, oracle_lib):
    idx = w["idx"]
    opts = {"evalMode": mode, "treeBuild": tree}
    om, xo, L, sens = _sensitivity(w, opts, idx)
    so = om.stats()
    sub = dict(w)
    sub["xv0"] = w["xv0"][idx]
    for prec in ("fp64", "mixed"):
        bar = max(TOL[prec], 4 * sens)
        # the sampled nodes alone: errors and decision counts for those nodes
        g = build_gpu(sub, opts, precision=prec)
        g.setSurfaceCoordinates(w["xs"])
        g.warpMesh()
        err = np.abs(g.getWarpGrid().reshape(-1, 3) - xo).max() / L
        assert err <= bar, (prec, "sample mesh", err, sens)
        sg = g.getStats()
        assert (sg["leafPairs"], sg["approx"]) == (so["leafPairs"], so["approx"]), prec
        del g
        # the whole 2M-node mesh (FP64 exact mode on the sample only: minutes
        # of FP64 pairs otherwise), read at the sampled nodes
        if prec == "fp64" and mode == "exact":
            continue
        g = build_gpu(w, opts, precision=prec)
        g.setSurfaceCoordinates(w["xs"])
        g.warpMesh()
        err = np.abs(g.getWarpGrid().reshape(-1, 3)[idx] - xo).max() / L
        assert err <= bar, (prec, "whole mesh", err, sens)
        del g
