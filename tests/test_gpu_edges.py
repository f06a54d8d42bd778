"""Edge cases of the warping path on the GPU against the oracle: extreme
options (LdefFact 100, exponents 4/6 overflow FP32 without scaling), several
symmetry planes, bucket sizes, errTol 0, a one-leaf tree, rotations and corner
handling switched off, non-finite and mismatched input."""
import numpy as np
import pytest

from tests.meshes import OPTS, build_gpu, build_oracle, sphere_small, wing_small

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sphere():
    return sphere_small()


def _cmp(m, opts, sym=True, tol64=1e-12, tol32=1e-8, counts=True):
    om = build_oracle(m, opts, sym=sym)
    om.set_surface_coordinates(m["xs"])
    xo = om.warp()
    L = om.ldef0()
    so = om.stats()
    for precision, tol in (("fp64", tol64), ("mixed", tol32)):
        g = build_gpu(m, opts, sym=sym, precision=precision)
        g.setSurfaceCoordinates(m["xs"])
        g.warpMesh()
        err = np.abs(g.getWarpGrid().reshape(-1, 3) - xo).max() / L
        assert err < tol, (precision, opts, err)
        if counts:
            st = g.getStats()
            assert st["leafPairs"] == so["leafPairs"], (precision, opts)
            assert st["approx"] == so["approx"], (precision, opts)


@pytest.mark.parametrize("opts", [{"LdefFact": 100.0}, {"LdefFact": 0.01}, {"aExp": 4.0, "bExp": 6.0},
                                  {"alpha": 2.0}, {"alpha": 0.0}])
def test_extreme_weight_laws(sphere, opts, built_lib, oracle_lib):
    _cmp(sphere, opts)


@pytest.mark.parametrize("bucket", [1, 4, 16, 64])
def test_bucket_sizes(sphere, bucket, built_lib, oracle_lib):
    _cmp(sphere, {"bucketSize": bucket})


def test_errtol_zero_is_exact(sphere, built_lib, oracle_lib):
    om = build_oracle(sphere, {"evalMode": "exact"})
    om.set_surface_coordinates(sphere["xs"])
    xe = om.warp()
    g = build_gpu(sphere, {"errTol": 0.0}, precision="mixed")
    g.setSurfaceCoordinates(sphere["xs"])
    g.warpMesh()
    assert g.getStats()["approx"] == 0
    assert np.abs(g.getWarpGrid().reshape(-1, 3) - xe).max() / om.ldef0() < 1e-8


def test_rotations_and_corners_off(built_lib, oracle_lib):
    m = wing_small()
    _cmp(m, {"useRotations": False})
    _cmp(m, {"zeroCornerRotations": False})
    _cmp(m, {"cornerAngle": 80.0})


@pytest.mark.parametrize("nplanes", [2, 3])
def test_several_symmetry_planes(nplanes, built_lib, oracle_lib):
    # the sphere cut by planes through its centre: x = 0, y = 0, z = 0
    m = dict(sphere_small())
    planes = [[[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]], [[0.0, 0.0, 0.0], [0.0, 1.0, 0.0]],
              [[0.0, 0.0, 0.0], [0.0, 0.0, 1.0]]][:nplanes]
    m["symmetryPlanes"] = planes
    _cmp(m, {})


def test_single_leaf_tree(built_lib, oracle_lib):
    # a surface small enough that the root is a leaf: exact sums only
    from idwarp_gb300 import synthetic as S

    m = S.sphere_ogrid(n=1, layers=4)
    m["xs"] = S.sphere_perturbation(m["pts"], seed=0)
    _cmp(m, {"bucketSize": 64})


def test_bad_input_raises(sphere, built_lib):
    from idwarp_gb300 import Error
    from idwarp_gb300._lib import LibraryError

    g = build_gpu(sphere, precision="mixed")
    with pytest.raises(Error):
        g.setSurfaceCoordinates(np.full_like(sphere["xs"], np.inf))
    with pytest.raises(Error):
        g.setSurfaceCoordinates(sphere["xs"][:-2])
    g.setSurfaceCoordinates(sphere["xs"])
    g.warpMesh()
    with pytest.raises(LibraryError):
        g.warpDeriv(np.zeros(5), solverVec=False)
    with pytest.raises(Error):
        g.warpDerivFwd(np.zeros((3, 3)), solverVec=False)


@pytest.mark.parametrize("opts,planes", [({"LdefFact": 100.0}, 0), ({}, 2)])
def test_mixed_derivatives_extreme_cases(opts, planes, built_lib):
    # reverse and tangent products of the mixed form against FP64 where the
    # forward needed care (large LdefFact, several mirrors)
    m = dict(sphere_small())
    if planes:
        m["symmetryPlanes"] = [[[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]], [[0.0, 0.0, 0.0], [0.0, 1.0, 0.0]]][:planes]
    rng = np.random.default_rng(51)
    dxv = rng.normal(size=3 * len(m["xv0"]))
    dxs = rng.normal(size=m["pts"].shape)
    out = {}
    for precision in ("fp64", "mixed"):
        g = build_gpu(m, opts, precision=precision)
        g.setSurfaceCoordinates(m["xs"])
        g.warpMesh()
        g.warpDeriv(dxv, solverVec=False)
        out[precision] = (g.getdXs(), g.warpDerivFwd(dxs, solverVec=False))
    # reverse product: the double-float adjoint; tangent: the FP32 walk
    for k, tol in ((0, 1e-9), (1, 1e-6)):
        ref = out["fp64"][k]
        assert np.abs(out["mixed"][k] - ref).max() <= tol * np.abs(ref).max(), k


def test_nonfinite_volume_grid_raises(sphere, built_lib):
    # the volume grid's finiteness is checked on the device with its bounding box
    import contextlib
    import io

    from idwarp_gb300 import USMesh
    from idwarp_gb300._lib import LibraryError

    x = np.array(sphere["xv0"], dtype=np.float64)
    x[len(x) // 2, 1] = np.nan
    with contextlib.redirect_stdout(io.StringIO()):
        g = USMesh(options=dict(OPTS, fileType="NPY", precision="mixed"))
    with pytest.raises(LibraryError, match="IDW_ERR_NONFINITE"):
        g.createCommonGrid(x)


def test_empty_volume_mesh(sphere, built_lib):
    import contextlib
    import io

    from idwarp_gb300 import USMesh

    o = dict(OPTS, fileType="NPY", precision="mixed")
    with contextlib.redirect_stdout(io.StringIO()):
        g = USMesh(options=o)
        g.createCommonGrid(np.zeros((0, 3)))
        g.setSurfaceDefinition(sphere["pts"], sphere["conn"], sphere["faceSizes"])
    g.setSurfaceCoordinates(sphere["xs"])
    g.warpMesh()
    assert g.getWarpGrid().size == 0
    g.warpDeriv(np.zeros(0), solverVec=False)
    assert np.all(g.getdXs() == 0.0)


def test_plot3d_grid_file_roundtrip(tmp_path, built_lib):
    # a two-block PLOT3D volume grid in, warped grid out with the same blocks
    import contextlib
    import io

    from idwarp_gb300 import USMesh
    from idwarp_gb300 import synthetic as S
    from idwarp_gb300.plot3d import readPlot3D, writePlot3D

    m = S.wing_shell(ni=17, nj=7, nk=6, first=1e-3, far=5.0)
    n = len(m["xv0"])
    half = (n // 2) // (17 * 7) * (17 * 7)
    sizes = np.array([[17, 7, half // (17 * 7)], [17, 7, (n - half) // (17 * 7)]])
    f = tmp_path / "vol.xyz"
    writePlot3D(str(f), m["xv0"], sizes)
    o = dict(OPTS, fileType="PLOT3D", gridFile=str(f), precision="mixed", symmetryPlanes=m["symmetryPlanes"])
    with contextlib.redirect_stdout(io.StringIO()):
        g = USMesh(options=o)
        g.setSurfaceDefinition(m["pts"], m["conn"], m["faceSizes"])
    xs = S.wing_perturbation(m["pts"], seed=2)
    g.setSurfaceCoordinates(xs)
    g.warpMesh()
    out = tmp_path / "warped.xyz"
    g.writeGrid(str(out))
    back, sz = readPlot3D(str(out), return_blocks=True)
    np.testing.assert_array_equal(sz, sizes)
    np.testing.assert_array_equal(back, g.getCommonGrid().reshape(-1, 3))


def test_async_grid_reads(sphere, built_lib):
    # getWarpGrid(wait=False): reads queued behind each warp, while the next
    # warp writes the other device buffer; every read must hold its own warp
    import torch

    from idwarp_gb300 import synthetic as S

    g = build_gpu(sphere, precision="mixed")
    surfaces = [S.sphere_perturbation(sphere["pts"], seed=k) for k in range(5)]
    want = []
    for xs in surfaces:
        g.setSurfaceCoordinates(xs)
        g.warpMesh()
        want.append(g.getWarpGrid().copy())
    n = 3 * len(sphere["xv0"])
    bufs = [torch.empty(n, dtype=torch.float64, pin_memory=True).numpy() for _ in range(3)]
    got = []
    for k, xs in enumerate(surfaces):
        g.setSurfaceCoordinates(xs)
        g.warpMesh()
        g.getWarpGrid(out=bufs[k % 3], wait=False)
        if k % 3 == 2:
            g.synchronize()
            got += [b.copy() for b in bufs]
    g.synchronize()
    got += [bufs[k % 3].copy() for k in range(len(got), len(surfaces))]
    for k in range(len(surfaces)):
        np.testing.assert_array_equal(got[k], want[k])
    # the synchronous read still sees the latest warp
    np.testing.assert_array_equal(g.getWarpGrid(), want[-1])

