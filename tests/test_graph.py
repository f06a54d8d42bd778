"""Forward + adjoint captured in one CUDA graph.

After one eager call with the same sizes (which builds the gate denominators
and grows the adjoint accumulators), the device-pointer calls
set_surface_coordinates -> warp_mesh -> get_volume_coordinates ->
warp_deriv_batch allocate nothing and do not synchronise, so torch can capture
them in a CUDA graph and replay it for new surfaces and seeds."""
import ctypes as C

import numpy as np
import pytest

from tests.meshes import build_gpu, wing_small

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_forward_adjoint_graph_replay(precision, built_lib):
    import torch

    from idwarp_gb300 import _lib
    from idwarp_gb300 import synthetic as S

    m = wing_small()
    g = build_gpu(m, precision=precision)
    L = g.lib
    nv, ns = len(m["xv0"]), len(m["pts"])
    xs = torch.tensor(m["xs"], device="cuda")
    seeds = torch.zeros((2, nv, 3), dtype=torch.float64, device="cuda")
    xv = torch.empty((nv, 3), dtype=torch.float64, device="cuda")
    dxs = torch.empty((2, ns, 3), dtype=torch.float64, device="cuda")
    D = _lib.IDW_DEVICE

    def step():
        assert L.idw_set_surface_coordinates(g.ctx, C.c_void_p(xs.data_ptr()), xs.numel(), D) == 0
        assert L.idw_warp_mesh(g.ctx) == 0
        assert L.idw_get_volume_coordinates(g.ctx, C.c_void_p(xv.data_ptr()), xv.numel(), D) == 0
        assert L.idw_warp_deriv_batch(g.ctx, C.c_void_p(seeds.data_ptr()), 2, C.c_void_p(dxs.data_ptr()), D) == 0

    s = torch.cuda.Stream()
    L.idw_set_stream(g.ctx, C.c_void_p(s.cuda_stream))
    with torch.cuda.stream(s):
        step()  # warm-up outside capture
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s):
        step()
    torch.cuda.synchronize()

    rng = np.random.default_rng(41)
    ref = build_gpu(m, precision=precision)
    for k in range(2):
        surf = S.wing_perturbation(m["pts"], seed=300 + k)
        sd = rng.normal(size=(2, nv, 3))
        xs.copy_(torch.tensor(surf))
        seeds.copy_(torch.tensor(sd))
        graph.replay()
        torch.cuda.synchronize()
        ref.setSurfaceCoordinates(surf)
        ref.warpMesh()
        np.testing.assert_allclose(xv.cpu().numpy().ravel(), ref.getWarpGrid(), rtol=0, atol=1e-13)
        want = ref.warpDerivBatch(sd)
        got = dxs.cpu().numpy()
        assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
