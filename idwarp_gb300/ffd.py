"""Shape-optimisation helpers around the differentiable warp.

``FFDBox`` moves surface points with a trivariate Bernstein lattice (control
point displacements along z, as a pyGeo FFD with z-only design variables
would), ``hex_volumes`` computes cell volumes of the warped grid with torch,
and ``ffd_loop`` runs gradient steps on the FFD coefficients minimising
sum(1 / max(V_cell, eps)) through ``idwarp_gb300.autograd.warp`` (backward =
the adjoint tree walk).
"""
import math
import time

import numpy as np
import torch

from .autograd import warp
from .synthetic import HEX_TETS


def _bernstein(t, n):
    """Bernstein basis of degree n at t in [0,1]; shape (len(t), n+1)."""
    t = np.clip(np.asarray(t, dtype=np.float64), 0.0, 1.0)
    k = np.arange(n + 1)
    binom = np.array([math.comb(n, j) for j in k], dtype=np.float64)
    return binom[None, :] * t[:, None] ** k[None, :] * (1.0 - t[:, None]) ** (n - k)[None, :]


class FFDBox:
    """Bernstein lattice of shape (nx, ny, nz) over the bounding box of the
    selected points (padded by ``pad`` of its size); the design variables are
    the z displacements of the lattice control points."""

    def __init__(self, pts, select=None, shape=(4, 4, 3), pad=0.05):
        pts = np.asarray(pts, dtype=np.float64)
        sel = np.arange(len(pts)) if select is None else np.asarray(select)
        p = pts[sel]
        lo, hi = p.min(axis=0), p.max(axis=0)
        size = np.maximum(hi - lo, 1e-12)
        lo, hi = lo - pad * size, hi + pad * size
        u = (p - lo) / (hi - lo)
        nx, ny, nz = shape
        bx, by, bz = _bernstein(u[:, 0], nx - 1), _bernstein(u[:, 1], ny - 1), _bernstein(u[:, 2], nz - 1)
        self.B = np.einsum("pi,pj,pk->pijk", bx, by, bz).reshape(len(sel), nx * ny * nz)
        self.sel = sel
        self.nPts = len(pts)
        self.nVars = nx * ny * nz

    def torch_operator(self, device):
        return torch.tensor(self.B, device=device), torch.tensor(self.sel, device=device, dtype=torch.long)

    def apply(self, xs0, coef, B=None, sel=None):
        """Surface coordinates for coefficients ``coef`` (torch, differentiable)."""
        if B is None:
            B, sel = self.torch_operator(coef.device)
        dz = B @ coef
        disp = torch.zeros_like(xs0)
        disp[sel, 2] = dz
        return xs0 + disp


def hex_volumes(xv, cells):
    """Signed volumes of hexahedra ``cells`` (M, 8) of the grid ``xv`` (N, 3), torch."""
    x = xv[cells]
    v = 0.0
    for a, b, c, d in HEX_TETS:
        v = v + torch.sum(torch.cross(x[:, b] - x[:, a], x[:, c] - x[:, a], dim=1) * (x[:, d] - x[:, a]), dim=1) / 6.0
    return v


def inverse_volume_objective(xv, cells, eps):
    return torch.sum(1.0 / torch.clamp(hex_volumes(xv, cells), min=eps))


def ffd_loop(mesh, xs0, cells, ffd, steps=50, lr=1e-3, eps=1e-12, check_directions=5, fd_step=1e-6, seed=300,
             coef0=None, fd_mesh=None):
    """Gradient steps (Adam) on the FFD coefficients minimising
    sum(1 / max(V_cell, eps)) of the warped grid, from ``coef0`` (zero by
    default: the undeformed surface).  Before the loop the gradient is
    checked against central differences on ``check_directions`` random
    directions; the differences are taken with ``fd_mesh`` when given (an
    FP64 mesh of the same grid: a step of 1e-6 is below the resolution of
    the mixed forward's own rounding), else with ``mesh``.  Returns a dict
    with the objective history, the gradient check and timings."""
    dev = xs0.device
    B, sel = ffd.torch_operator(dev)
    if coef0 is None:
        coef = torch.zeros(ffd.nVars, dtype=torch.float64, device=dev, requires_grad=True)
    else:
        coef = torch.as_tensor(coef0, dtype=torch.float64, device=dev).clone().requires_grad_(True)

    def objective(c, m=mesh):
        return inverse_volume_objective(warp(ffd.apply(xs0, c, B, sel), m), cells, eps)

    fdm = fd_mesh if fd_mesh is not None else mesh

    f0 = objective(coef)
    f0.backward()
    g0 = coef.grad.detach().clone()
    rng = np.random.default_rng(seed)
    check = []
    with torch.no_grad():
        for _ in range(check_directions):
            d = torch.tensor(rng.normal(size=ffd.nVars), device=dev)
            fp = objective(coef + fd_step * d, fdm).item()
            fm = objective(coef - fd_step * d, fdm).item()
            fd = (fp - fm) / (2 * fd_step)
            ad = float(torch.dot(g0, d))
            check.append({"ad": ad, "fd": fd, "rel": abs(ad - fd) / max(abs(fd), 1e-300)})
    coef.grad = None
    opt = torch.optim.Adam([coef], lr=lr)
    hist = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        opt.zero_grad()
        f = objective(coef)
        f.backward()
        opt.step()
        hist.append(f.item())
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    return {"objective": hist, "initial": f0.item(), "gradient_check": check, "seconds": dt,
            "seconds_per_step": dt / max(steps, 1), "coef": coef.detach().cpu().numpy()}
