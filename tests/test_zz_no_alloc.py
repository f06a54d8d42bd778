"""idw_warp_deriv_noalloc: warpDeriv for one seed with scratch in a static
device array instead of per-call allocations.  Collected last; passes alone
and after the other GPU tests."""
import ctypes as C

import numpy as np
import pytest

from tests.meshes import build_gpu, wing_small

pytestmark = pytest.mark.gpu


def _noalloc(g, dxv, dxs):
    return g.lib.idw_warp_deriv_noalloc(g.ctx, C.c_void_p(dxv.data_ptr()), dxv.numel(), C.c_void_p(dxs.data_ptr()),
                                        dxs.numel())


@pytest.mark.parametrize("mode", ["fast", "exact"])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-12)])
def test_noalloc_matches_warp_deriv(precision, tol, mode, built_lib):
    import torch

    m = wing_small()
    # the entry point computes the FP32 form of the mixed adjoint (its
    # scratch has no room for the double-float form's denominator)
    g = build_gpu(m, {"evalMode": mode, "adjointPrecision": "fast"}, precision=precision)
    g.setSurfaceCoordinates(m["xs"])
    g.warpMesh()
    rng = np.random.default_rng(31)
    seed = rng.normal(size=3 * len(m["xv0"]))
    g.warpDeriv(seed, solverVec=False)
    ref = g.getdXs()
    dxv = torch.tensor(seed, device="cuda")
    dxs = torch.full((len(m["pts"]), 3), np.nan, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    g.lib.idw_set_stream(g.ctx, C.c_void_p(stream.cuda_stream))
    for _ in range(2):
        assert _noalloc(g, dxv, dxs) == 0
        torch.cuda.synchronize()
        out = dxs.cpu().numpy()
        assert np.all(np.isfinite(out))
        # same kernels as warpDeriv; only the order of the atomic sums differs
        assert np.abs(out - ref).max() <= tol * np.abs(ref).max()
    # no device memory is taken by a call (after the first, which may load code)
    free0 = torch.cuda.mem_get_info()[0]
    assert _noalloc(g, dxv, dxs) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_two_contexts_in_turn(built_lib):
    # two meshes (two contexts) share the one static scratch; calls made one
    # after the other, each finished before the next starts, must each give
    # their own mesh's warpDeriv
    import torch

    from tests.meshes import sphere_small

    stream = torch.cuda.current_stream()
    cases = []
    for m, prec in ((wing_small(), "mixed"), (sphere_small(), "fp64")):
        g = build_gpu(m, {"adjointPrecision": "fast"}, precision=prec)
        g.lib.idw_set_stream(g.ctx, C.c_void_p(stream.cuda_stream))
        g.setSurfaceCoordinates(m["xs"])
        g.warpMesh()
        seed = np.random.default_rng(len(m["pts"])).normal(size=3 * len(m["xv0"]))
        g.warpDeriv(seed, solverVec=False)
        dxv = torch.tensor(seed, device="cuda")
        dxs = torch.full((len(m["pts"]), 3), np.nan, dtype=torch.float64, device="cuda")
        cases.append((g, g.getdXs(), dxv, dxs))
    for rep in range(2):
        for g, ref, dxv, dxs in (cases if rep == 0 else cases[::-1]):
            dxs.fill_(np.nan)
            assert _noalloc(g, dxv, dxs) == 0
            torch.cuda.synchronize()
            out = dxs.cpu().numpy()
            assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max(), rep


def test_noalloc_rejects_bad_arguments(built_lib):
    import torch

    from idwarp_gb300._lib import IDW_ERR_ARG, IDW_ERR_STATE

    m = wing_small()
    g = build_gpu(m, precision="mixed")
    dxv = torch.zeros(3 * len(m["xv0"]), dtype=torch.float64, device="cuda")
    dxs = torch.zeros(3 * len(m["pts"]), dtype=torch.float64, device="cuda")
    assert _noalloc(g, dxv, dxs) == IDW_ERR_STATE  # before warpMesh
    g.setSurfaceCoordinates(m["xs"])
    g.warpMesh()
    assert _noalloc(g, dxv[:-3], dxs) == IDW_ERR_ARG
    assert _noalloc(g, dxv, dxs[:-3]) == IDW_ERR_ARG
    assert _noalloc(g, dxv, dxs) == 0


def test_noalloc_rejects_oversize_surface(built_lib):
    import torch

    from idwarp_gb300 import synthetic as S
    from idwarp_gb300._lib import IDW_ERR_LIMIT

    # ~240k unique surface nodes: beyond the static scratch in mixed precision
    m = S.sphere_ogrid(n=200, layers=2)
    m["xs"] = m["pts"]
    g = build_gpu(m, precision="mixed")
    g.setSurfaceCoordinates(m["xs"])
    g.warpMesh()
    dxv = torch.zeros(3 * len(m["xv0"]), dtype=torch.float64, device="cuda")
    dxs = torch.zeros(3 * len(m["pts"]), dtype=torch.float64, device="cuda")
    assert _noalloc(g, dxv, dxs) == IDW_ERR_LIMIT
    msg = C.create_string_buffer(512)
    g.lib.idw_last_error(g.ctx, msg, 512)
    assert b"static scratch" in msg.value
