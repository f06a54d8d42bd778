"""torch.autograd bridge: Xv = warp(Xs) with the reverse product as backward.

``IDWarpFn.apply(xs, mesh)`` sets the surface coordinates of a
:class:`~idwarp_gb300.USMesh`, warps, and returns the volume coordinates as a
(nVol, 3) float64 tensor in warp (common) order on the device of ``xs``.  Its
backward is ``warpDeriv`` (the reverse product (dXv/dXs)^T g, computed by the
adjoint tree walk), and its forward-mode rule is ``warpDerivFwd``.

The library runs on the caller's current CUDA stream, so tensors made by torch
are ordered with the library's kernels without extra synchronisation.
"""
import ctypes as C

import torch

from . import _lib


def _bind_stream(mesh, device):
    if device.type == "cuda":
        s = torch.cuda.current_stream(device)
        mesh.lib.idw_set_stream(mesh.ctx, C.c_void_p(s.cuda_stream))


def _ptr(t):
    return C.c_void_p(t.data_ptr()), (_lib.IDW_DEVICE if t.is_cuda else _lib.IDW_HOST)


def _relinearise(mesh, xs_c, version):
    """Make the mesh's surface the forward call's again, if it changed since."""
    if mesh._surfVersion != version:
        mesh.setSurfaceCoordinates(xs_c)


class IDWarpFn(torch.autograd.Function):
    """Differentiable warpMesh: (nSurf, 3) surface coordinates -> (nVol, 3) volume coordinates."""

    @staticmethod
    def forward(ctx, xs, mesh):
        xs_c = xs.detach().to(torch.float64).contiguous()
        _bind_stream(mesh, xs_c.device)
        mesh.setSurfaceCoordinates(xs_c)
        mesh.warpMesh()
        xv = torch.empty((mesh.nVol, 3), dtype=torch.float64, device=xs_c.device)
        p, where = _ptr(xv)
        mesh._chk(mesh.lib.idw_get_volume_coordinates(mesh.ctx, p, xv.numel(), where), "getWarpGrid")
        ctx.mesh = mesh
        ctx.xs_c = xs_c
        ctx.version = mesh._surfVersion
        return xv

    @staticmethod
    def backward(ctx, gxv):
        mesh = ctx.mesh
        g = gxv.detach().to(device=ctx.xs_c.device, dtype=torch.float64).contiguous()
        _bind_stream(mesh, g.device)
        # the reverse product linearises at the forward call's surface; the
        # denominator depends on Xu0 only and stays valid
        _relinearise(mesh, ctx.xs_c, ctx.version)
        dxs = torch.empty((mesh.nSurf, 3), dtype=torch.float64, device=g.device)
        pg, where = _ptr(g)
        pd, _ = _ptr(dxs)
        mesh._chk(mesh.lib.idw_warp_deriv_batch(mesh.ctx, pg, 1, pd, where), "warpDeriv")
        return dxs, None

    @staticmethod
    def jvp(ctx, dxs, _mesh_tangent):
        mesh = ctx.mesh
        d = dxs.detach().to(device=ctx.xs_c.device, dtype=torch.float64).contiguous()
        _bind_stream(mesh, d.device)
        _relinearise(mesh, ctx.xs_c, ctx.version)
        out = torch.empty((mesh.nVol, 3), dtype=torch.float64, device=d.device)
        pi, where = _ptr(d)
        po, _ = _ptr(out)
        mesh._chk(mesh.lib.idw_warp_deriv_fwd(mesh.ctx, pi, d.numel(), po, out.numel(), where), "warpDerivFwd")
        return out


def warp(xs, mesh):
    """Differentiable warp of ``mesh`` to surface ``xs`` (see :class:`IDWarpFn`)."""
    return IDWarpFn.apply(xs, mesh)
