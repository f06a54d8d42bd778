"""Complex step through USMesh_C on the GPU's FP64 path, following the
reference's procedure (tests/test_USMesh.py:88-100): warp a perturbed
surface, add i*h (h = 1e-40) to every surface coordinate, warp again, and
compare Im(Xv)/h dotted with dXv = linspace(0, 1, ndof) against sum(dXs) of
warpDeriv with that dXv.  Also Im(Xv)/h against warpDerivFwd along the
all-ones direction, against the oracle's complex step, and the real part
against the FP64 USMesh warp."""
import contextlib
import io

import numpy as np
import pytest

from tests.meshes import OPTS, build_gpu, build_oracle, wing_small

pytestmark = pytest.mark.gpu

H = 1e-40


def _usmesh_c(m, opts):
    from idwarp_gb300 import USMesh_C

    o = dict(OPTS)
    o.update(opts)
    o["fileType"] = "NPY"
    if m.get("symmetryPlanes"):
        o["symmetryPlanes"] = m["symmetryPlanes"]
    with contextlib.redirect_stdout(io.StringIO()):
        g = USMesh_C(options=o)
        g.createCommonGrid(m["xv0"])
        g.setSurfaceDefinition(m["pts"], m["conn"], m["faceSizes"])
    return g


@pytest.fixture(scope="module")
def s1():
    from idwarp_gb300 import synthetic as S

    m = S.sphere_ogrid(n=18, layers=48)
    m["xs"] = S.sphere_perturbation(m["pts"], seed=0)
    return m


@pytest.mark.parametrize("case,mode,tree", [("s1", "fast", "kd"), ("wing", "fast", "kd"), ("wing", "exact", "kd"),
                                             ("wing", "fast", "morton")])
def test_complex_step_matches_derivatives(case, mode, tree, s1, built_lib, oracle_lib):
    # tree "morton": the same checks on the GPU-built tree (the oracle builds it too)
    m = s1 if case == "s1" else wing_small()
    opts = {"evalMode": mode, "treeBuild": tree}
    gc = _usmesh_c(m, opts)
    coords0 = gc.getSurfaceCoordinates()
    assert coords0.dtype == np.complex128
    gc.setSurfaceCoordinates(m["xs"])
    gc.warpMesh()
    xr = gc.getWarpGrid()
    gc.setSurfaceCoordinates(m["xs"] + 1j * H)
    gc.warpMesh()
    xc = gc.getWarpGrid()
    deriv = xc.imag / H

    g = build_gpu(m, opts, precision="fp64")
    g.setSurfaceCoordinates(m["xs"])
    g.warpMesh()
    x64 = g.getWarpGrid()
    L = g.getStats()["Ldef0"]
    # the real part is the ordinary FP64 warp
    assert np.abs(xc.real - x64).max() <= 1e-14 * L
    assert np.abs(xr.real - x64).max() <= 1e-14 * L and np.all(xr.imag == 0.0)

    # reverse product (the reference's check): dot(dXv, Im Xv / h) = sum(dXs)
    dxv = np.linspace(0.0, 1.0, 3 * len(m["xv0"]))
    g.warpDeriv(dxv, solverVec=False)
    dxs = g.getdXs()
    a, b = float(np.dot(dxv, deriv)), float(np.sum(dxs))
    assert abs(a - b) <= 1e-10 * float(np.sum(np.abs(dxv * deriv))), (a, b)

    # forward product along the same (all-ones) direction
    fwd = g.warpDerivFwd(np.ones(m["pts"].shape), solverVec=False)
    assert np.abs(deriv - fwd).max() <= 1e-10 * np.abs(fwd).max()

    # the oracle's complex step (CPU restatement in std::complex)
    om = build_oracle(m, opts)
    om.set_surface_coordinates(m["xs"])
    om.warp()
    xo = om.warp_complex(m["xs"] + 1j * H)
    do = xo.imag.ravel() / H
    assert np.abs(deriv - do).max() <= 1e-10 * np.abs(do).max()


def test_complex_step_rejects_mixed(built_lib):
    from idwarp_gb300 import Error, USMesh_C

    with pytest.raises(Error):
        USMesh_C(options={"precision": "mixed"})


def test_complex_step_without_imaginary_part(built_lib):
    # real coordinates through USMesh_C: a zero imaginary part everywhere
    m = wing_small()
    gc = _usmesh_c(m, {})
    gc.setSurfaceCoordinates(m["xs"])
    gc.warpMesh()
    xc = gc.getWarpGrid()
    assert xc.dtype == np.complex128 and np.all(xc.imag == 0.0)
