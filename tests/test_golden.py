"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py).

The fixtures follow the reference test procedure (tests/test_USMesh.py of
mdolab/idwarp: shear-sweep and inflate perturbations, sums of the warped grid
and of dXs for dXv = linspace(0, 1, ndof), the complex-step identity) on small
seeded synthetic meshes, with values from the oracle.  The CPU tests pin the
oracle to them; the GPU tests compare the library, through its C ABI, with
them.
"""
import glob
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(HERE, "golden", "*.npz")))
REF_OPTS = {"aExp": 3.0, "bExp": 5.0, "LdefFact": 1.0, "alpha": 0.25, "errTol": 5e-4, "bucketSize": 8,
            "useRotations": True, "zeroCornerRotations": True, "cornerAngle": 30.0}


def load(name):
    with np.load(os.path.join(HERE, "golden", name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def sym_of(g):
    s = g["symmetry"]
    return [[s[i, 0].tolist(), s[i, 1].tolist()] for i in range(len(s))] or None


def test_fixtures_present():
    assert CASES == ["sphere_inflate", "sphere_shear", "wing_sym_shear"]


@pytest.mark.parametrize("name", CASES)
def test_fixture_identities(name):
    g = load(name)
    # complex step and reverse product agree (test_USMesh.py:70-91 pattern)
    assert abs(g["sum_complex_step"] - g["sum_dxs"]) <= 1e-10 * abs(g["sum_dxs"])
    assert abs(np.sum(g["xv_fast"]) - g["sum_warped"]) <= 1e-9 * np.abs(g["xv_fast"]).sum()
    # fast mode stays within its error control of the exact sum
    assert np.abs(g["xv_fast"] - g["xv_exact"]).max() < 1e-2 * g["ldef0"]
    if len(g["symmetry"]) == 0:
        # a uniform translation of every surface coordinate moves every volume
        # node by the same amount, so sum(dXs) = sum(dXv)
        n = g["xv0"].size
        assert abs(g["sum_dxs"] - n / 2.0) <= 1e-9 * n


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_fixture(name, oracle_lib):
    from oracle.pyoracle import OracleMesh

    g = load(name)
    for mode in ("fast", "exact"):
        om = OracleMesh(dict(REF_OPTS, evalMode=mode))
        om.set_volume(g["xv0"])
        if len(g["symmetry"]):
            om.set_symmetry(g["symmetry"][:, 0], g["symmetry"][:, 1])
        om.set_surface_definition(g["pts"], g["conn"], g["faceSizes"])
        om.set_surface_coordinates(g["xs"])
        xv = om.warp()
        np.testing.assert_allclose(xv, g["xv_" + mode], rtol=0, atol=1e-13 * g["ldef0"])
        assert om.stats()["leafPairs"] == int(g["leafPairs_" + mode])
        if mode == "fast":
            dxs = om.warp_deriv(np.linspace(0.0, 1.0, g["xv0"].size).reshape(-1, 3))
            np.testing.assert_allclose(dxs, g["dxs"], rtol=0, atol=1e-11 * np.abs(g["dxs"]).max())


def _gpu_mesh(g, mode, precision):
    import contextlib
    import io

    from idwarp_gb300 import USMesh

    opts = dict(REF_OPTS, evalMode=mode, precision=precision, fileType="NPY", symmetryPlanes=sym_of(g))
    with contextlib.redirect_stdout(io.StringIO()):
        mesh = USMesh(options=opts)
        mesh.createCommonGrid(g["xv0"])
        mesh.setSurfaceDefinition(g["pts"], g["conn"], g["faceSizes"])
    return mesh


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-8)])
@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_fixture(name, precision, tol, built_lib):
    # Bars: 1e-12 (FP64) / 1e-8 (mixed) of Ldef, widened to 4x the case's
    # rounding sensitivity (sens_*: the oracle source compiled with FMA
    # contraction against the fixture), which is 5.5e-11 Ldef and 3e-5 of
    # max|dXs| on the sheared wing, where most rotation angles are below 1e-3.
    g = load(name)
    for mode in ("fast", "exact"):
        mesh = _gpu_mesh(g, mode, precision)
        mesh.setSurfaceCoordinates(g["xs"])
        mesh.warpMesh()
        xv = mesh.getWarpGrid().reshape(-1, 3)
        err = np.abs(xv - g["xv_" + mode]).max() / g["ldef0"]
        assert err < max(tol, 4 * float(g["sens_xv_" + mode])), (mode, err)
        st = mesh.getStats()
        assert st["leafPairs"] == int(g["leafPairs_" + mode])
        assert st["approx"] == int(g["approx_" + mode])
        if mode == "fast":
            np.testing.assert_allclose(mesh.getDenominator0(), g["den0"], rtol=1e-12)
            dxv = np.linspace(0.0, 1.0, g["xv0"].size)
            mesh.warpDeriv(dxv, solverVec=False)
            dxs = mesh.getdXs()
            dtol = max(1e-10 if precision == "fp64" else 1e-9, 4 * float(g["sens_dxs"]))
            assert np.abs(dxs - g["dxs"]).max() <= dtol * np.abs(g["dxs"]).max()
            assert abs(np.sum(dxs) - g["sum_dxs"]) <= dtol * np.abs(g["dxs"]).sum()
