"""Option deterministic: reverse products whose sums land order-independently
(192-bit fixed-point sums with integer atomics, after a pass that finds each
target's exponent), so dXs is the same bit for bit on every run.

Every form of the reverse product is covered: FP64 (fast and exact), the
double-float mixed form, the FP32 mixed form, the tiled exact kernel, several
seeds per walk, one and three symmetry planes, rotations on and off.  Against
the default FP64 atomics the results differ by the rounding of the sums only
(relative to max |dXs|: 1e-12 here)."""
import numpy as np
import pytest

from tests.meshes import build_gpu, sphere_small, wing_small

pytestmark = pytest.mark.gpu

FORMS = [
    ("fp64", {}),
    ("fp64", {"evalMode": "exact"}),
    ("mixed", {}),
    ("mixed", {"adjointPrecision": "fast"}),
    ("mixed", {"evalMode": "exact", "exactSchedule": "tiled", "adjointPrecision": "fast"}),
    ("mixed", {"evalMode": "exact"}),
    ("mixed", {"useRotations": False}),
]


def _deriv(g, dxv, nseeds):
    if nseeds == 1:
        g.warpDeriv(dxv[0].ravel(), solverVec=False)
        return g.getdXs().copy()[None]
    return np.asarray(g.warpDerivBatch(dxv)).copy()


@pytest.mark.parametrize("nseeds", [1, 5, 17])
@pytest.mark.parametrize("precision,opts", FORMS)
def test_repeatable_and_close_to_atomics(precision, opts, nseeds, built_lib):
    if nseeds > 1 and opts.get("exactSchedule") == "tiled":
        pytest.skip("the tiled exact kernel takes one seed at a time; groups walk")
    m = wing_small()
    rng = np.random.default_rng(3)
    dxv = rng.standard_normal((nseeds,) + m["xv0"].shape)
    gd = build_gpu(m, dict(opts, deterministic=True), precision=precision)
    ga = build_gpu(m, opts, precision=precision)
    for g in (gd, ga):
        g.setSurfaceCoordinates(m["xs"])
        g.warpMesh()
    first = _deriv(gd, dxv, nseeds)
    for _ in range(3):
        np.testing.assert_array_equal(_deriv(gd, dxv, nseeds), first)
    ref = _deriv(ga, dxv, nseeds)
    scale = np.abs(ref).max()
    assert np.abs(first - ref).max() <= 1e-12 * scale, np.abs(first - ref).max() / scale


@pytest.mark.parametrize("planes", [1, 3])
def test_symmetry_planes(planes, built_lib):
    m = dict(sphere_small())
    m["symmetryPlanes"] = [[[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]], [[0.0, 0.0, 0.0], [0.0, 1.0, 0.0]],
                           [[0.0, 0.0, 0.0], [0.0, 0.0, 1.0]]][:planes]
    dxv = np.random.default_rng(4).standard_normal((1,) + m["xv0"].shape)
    out = []
    for det in (True, True, False):
        g = build_gpu(m, {"deterministic": det}, precision="mixed")
        g.setSurfaceCoordinates(m["xs"])
        g.warpMesh()
        out.append(_deriv(g, dxv, 1))
    np.testing.assert_array_equal(out[0], out[1])
    assert np.abs(out[0] - out[2]).max() <= 1e-12 * np.abs(out[2]).max()


def test_state_cleared_for_other_contexts(built_lib):
    # a deterministic call leaves nothing behind: a context with atomics gives
    # the same products before and after it (to their own run-to-run rounding)
    m = wing_small()
    dxv = np.random.default_rng(5).standard_normal((1,) + m["xv0"].shape)
    ga = build_gpu(m, precision="mixed")
    gd = build_gpu(m, {"deterministic": True}, precision="mixed")
    for g in (ga, gd):
        g.setSurfaceCoordinates(m["xs"])
        g.warpMesh()
    before = _deriv(ga, dxv, 1)
    _deriv(gd, dxv, 1)
    after = _deriv(ga, dxv, 1)
    assert np.abs(after - before).max() <= 1e-12 * np.abs(before).max()


def test_option_switches_at_run_time(built_lib):
    # like every option, it reaches the library at the next warpMesh
    # (idwarp/UnstructuredMesh.py:1051-1069) and holds for the reverse
    # products after it
    m = wing_small()
    dxv = np.random.default_rng(6).standard_normal((1,) + m["xv0"].shape)
    g = build_gpu(m, precision="fp64")
    g.setSurfaceCoordinates(m["xs"])
    g.warpMesh()
    a = _deriv(g, dxv, 1)
    g.setOption("deterministic", True)
    g.warpMesh()
    d1 = _deriv(g, dxv, 1)
    d2 = _deriv(g, dxv, 1)
    np.testing.assert_array_equal(d1, d2)
    assert np.abs(d1 - a).max() <= 1e-12 * np.abs(a).max()


def test_capture_refused(built_lib):
    # the passes wait for the stream: a deterministic call inside a CUDA graph
    # capture returns IDW_ERR_STATE before it enqueues anything
    import ctypes as C

    import torch

    from idwarp_gb300 import _lib

    m = wing_small()
    g = build_gpu(m, {"deterministic": True}, precision="mixed")
    g.setSurfaceCoordinates(m["xs"])
    g.warpMesh()
    nv, ns = len(m["xv0"]), len(m["pts"])
    seeds = torch.zeros((1, nv, 3), dtype=torch.float64, device="cuda")
    dxs = torch.empty((1, ns, 3), dtype=torch.float64, device="cuda")
    s = torch.cuda.Stream()
    g.lib.idw_set_stream(g.ctx, C.c_void_p(s.cuda_stream))
    graph = torch.cuda.CUDAGraph()
    rc = None
    with torch.cuda.graph(graph, stream=s):
        rc = g.lib.idw_warp_deriv_batch(g.ctx, C.c_void_p(seeds.data_ptr()), 1, C.c_void_p(dxs.data_ptr()),
                                        _lib.IDW_DEVICE)
        torch.zeros(1, device="cuda")  # the graph holds one node of its own
    assert rc == _lib.IDW_ERR_STATE
    torch.cuda.synchronize()


def test_concurrent_contexts(built_lib):
    # two host threads with their own contexts: deterministic reverse products
    # in one (serialised in the process, state in constant memory) and the
    # default ones in the other (their kernels never read that state)
    import ctypes as C
    import threading

    import torch

    m = wing_small()
    dxv = np.random.default_rng(7).standard_normal(m["xv0"].shape).ravel()
    gd = build_gpu(m, {"deterministic": True}, precision="mixed")
    ga = build_gpu(m, precision="mixed")
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]  # kernels of the two contexts may overlap
    for g, st in zip((gd, ga), streams):
        g.lib.idw_set_stream(g.ctx, C.c_void_p(st.cuda_stream))
    refs = {}
    for name, g in (("det", gd), ("atomic", ga)):
        g.setSurfaceCoordinates(m["xs"])
        g.warpMesh()
        g.warpDeriv(dxv, solverVec=False)
        refs[name] = g.getdXs().copy()
    errors = []

    def run(name, g, n):
        try:
            for _ in range(n):
                g.warpDeriv(dxv, solverVec=False)
                out = g.getdXs()
                if name == "det":
                    if not np.array_equal(out, refs[name]):
                        errors.append((name, "not bitwise"))
                elif np.abs(out - refs[name]).max() > 1e-12 * np.abs(refs[name]).max():
                    errors.append((name, float(np.abs(out - refs[name]).max())))
        except Exception as e:  # the thread's failure is the test's
            errors.append((name, repr(e)))

    threads = [threading.Thread(target=run, args=("det", gd, 4)), threading.Thread(target=run, args=("atomic", ga, 8))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
