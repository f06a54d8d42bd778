"""Differentiation through the warp on a two-body mesh (wing + sphere): FFD
coefficients -> surface -> warp -> cell volumes -> sum(1/max(V, eps)), with
the gradient from the adjoint walk checked against central differences and
against the oracle's warpDeriv (the reference's reverse product)."""
import numpy as np
import pytest

from tests.meshes import OPTS

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def body():
    from idwarp_gb300 import synthetic as S

    return S.multibody(wing=(33, 13, 10), sphere=(8, 6))


def _mesh(m, precision, rotations=True):
    import contextlib
    import io

    from idwarp_gb300 import USMesh

    o = dict(OPTS, fileType="NPY", precision=precision, useRotations=rotations, symmetryPlanes=m["symmetryPlanes"])
    with contextlib.redirect_stdout(io.StringIO()):
        g = USMesh(options=o)
        g.createCommonGrid(m["xv0"])
        g.setSurfaceDefinition(m["pts"], m["conn"], m["faceSizes"])
    return g


def test_gradient_matches_oracle_reverse_product(body, built_lib, oracle_lib):
    import torch

    from idwarp_gb300.autograd import warp
    from idwarp_gb300.ffd import FFDBox, inverse_volume_objective
    from oracle.pyoracle import OracleMesh

    m = body
    g = _mesh(m, "fp64")
    ffd = FFDBox(m["pts"], select=np.arange(m["nWingPts"]))
    B, sel = ffd.torch_operator("cuda")
    xs0 = torch.tensor(m["pts"], device="cuda")
    cells = torch.tensor(m["cells"], device="cuda")
    coef = torch.tensor(np.random.default_rng(5).normal(scale=0.01, size=ffd.nVars), device="cuda", requires_grad=True)
    xs = ffd.apply(xs0, coef, B, sel)
    xv = warp(xs, g)
    xv.retain_grad()
    inverse_volume_objective(xv, cells, 1e-12).backward()
    # the same reverse product by the oracle: dXs = oracle.warpDeriv(dL/dXv)
    om = OracleMesh(dict(OPTS))
    om.set_volume(m["xv0"])
    om.set_symmetry(np.array([p[0] for p in m["symmetryPlanes"]]), np.array([p[1] for p in m["symmetryPlanes"]]))
    om.set_surface_definition(m["pts"], m["conn"], m["faceSizes"])
    om.set_surface_coordinates(xs.detach().cpu().numpy())
    om.warp()
    dxs = om.warp_deriv(xv.grad.cpu().numpy())
    g_oracle = ffd.B.T @ dxs[ffd.sel, 2]
    g_gpu = coef.grad.cpu().numpy()
    assert np.abs(g_gpu - g_oracle).max() <= 1e-10 * np.abs(g_oracle).max()


def test_ffd_loop_gradient_check_and_descent(body, built_lib):
    # Rotations off: the derivative is then the exact one.  With rotations the
    # reference's derivative drops the rotation of every node whose normal has
    # not turned (degenerate axis) -- at the undeformed surface, all of them --
    # so central differences differ from it by design (by 3-15% here); the
    # oracle comparison above covers that case.
    import torch

    from idwarp_gb300.ffd import FFDBox, ffd_loop

    m = body
    g = _mesh(m, "fp64", rotations=False)
    ffd = FFDBox(m["pts"], select=np.arange(m["nWingPts"]))
    xs0 = torch.tensor(m["pts"], device="cuda")
    cells = torch.tensor(m["cells"], device="cuda")
    out = ffd_loop(g, xs0, cells, ffd, steps=5, lr=2e-3, check_directions=3)
    for c in out["gradient_check"]:
        assert c["rel"] < 1e-6, out["gradient_check"]
    assert out["objective"][-1] < out["initial"]


def test_mixed_gradient_matches_fp64(body, built_lib):
    # central differences of the mixed objective are dominated by its rounding
    # (1/V of cells 1e-7 in size); compare the mixed gradient with the FP64 one.
    # dL/dXv = -dV/dXv / V^2 magnifies the mixed positions' 1e-9 Ldef error by
    # Ldef / (first spacing 1e-4) on the wall cells: about 2e-5 relative here.
    import torch

    from idwarp_gb300.autograd import warp
    from idwarp_gb300.ffd import FFDBox, inverse_volume_objective

    m = body
    ffd = FFDBox(m["pts"], select=np.arange(m["nWingPts"]))
    B, sel = ffd.torch_operator("cuda")
    xs0 = torch.tensor(m["pts"], device="cuda")
    cells = torch.tensor(m["cells"], device="cuda")
    c0 = np.random.default_rng(6).normal(scale=0.01, size=ffd.nVars)
    grads = []
    for precision in ("fp64", "mixed"):
        g = _mesh(m, precision)
        coef = torch.tensor(c0, device="cuda", requires_grad=True)
        inverse_volume_objective(warp(ffd.apply(xs0, coef, B, sel), g), cells, 1e-12).backward()
        grads.append(coef.grad.cpu().numpy())
    assert np.abs(grads[1] - grads[0]).max() <= 1e-4 * np.abs(grads[0]).max()
