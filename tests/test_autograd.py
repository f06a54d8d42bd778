"""torch.autograd bridge (idwarp_gb300.autograd): forward = warpMesh, backward =
warpDeriv, forward-mode = warpDerivFwd; checked against each other and against
central differences (the verifyWarpDeriv pattern, src/warp/verifyWarpDeriv.F90)."""
import numpy as np
import pytest

from tests.meshes import build_gpu, wing_small

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def wing():
    return wing_small()


def test_forward_backward_match_library(wing, built_lib):
    import torch

    from idwarp_gb300.autograd import warp

    g = build_gpu(wing, precision="fp64")
    xs = torch.tensor(wing["xs"], device="cuda", requires_grad=True)
    xv = warp(xs, g)
    np.testing.assert_array_equal(xv.detach().cpu().numpy().ravel(), g.getWarpGrid())
    rng = np.random.default_rng(21)
    w = rng.normal(size=xv.shape)
    (xv * torch.tensor(w, device="cuda")).sum().backward()
    g.warpDeriv(w.ravel(), solverVec=False)
    np.testing.assert_allclose(xs.grad.cpu().numpy(), g.getdXs(), rtol=0, atol=1e-13 * np.abs(g.getdXs()).max())


def test_gradient_against_central_differences(wing, built_lib):
    # Rotations off: with rotations the reference's derivative of the Rodrigues
    # matrix is defined as zero for degenerate axes and clamped angles
    # (vectorUtils_b.f90), which central differences do not see.
    import torch

    from idwarp_gb300.autograd import warp

    g = build_gpu(wing, {"useRotations": False}, precision="fp64")
    rng = np.random.default_rng(22)
    w = torch.tensor(rng.normal(size=wing["xv0"].shape), device="cuda")
    v = torch.tensor(rng.normal(size=wing["pts"].shape), device="cuda")
    xs0 = torch.tensor(wing["xs"], device="cuda")
    xs = xs0.clone().requires_grad_(True)
    (warp(xs, g) * w).sum().backward()
    ad = float((xs.grad * v).sum())
    h = 1e-6
    with torch.no_grad():
        fp = float((warp(xs0 + h * v, g) * w).sum())
        fm = float((warp(xs0 - h * v, g) * w).sum())
    fd = (fp - fm) / (2 * h)
    assert abs(ad - fd) <= 1e-6 * abs(fd), (ad, fd)


def test_forward_mode_matches_reverse(wing, built_lib):
    import torch
    import torch.autograd.forward_ad as fwAD

    from idwarp_gb300.autograd import warp

    g = build_gpu(wing, precision="fp64")
    rng = np.random.default_rng(23)
    v = torch.tensor(rng.normal(size=wing["pts"].shape), device="cuda")
    w = torch.tensor(rng.normal(size=wing["xv0"].shape), device="cuda")
    xs0 = torch.tensor(wing["xs"], device="cuda")
    with fwAD.dual_level():
        xv = warp(fwAD.make_dual(xs0, v), g)
        tangent = fwAD.unpack_dual(xv).tangent
    xs = xs0.clone().requires_grad_(True)
    (warp(xs, g) * w).sum().backward()
    a, b = float((tangent * w).sum()), float((xs.grad * v).sum())
    assert abs(a - b) <= 1e-11 * abs(b), (a, b)
