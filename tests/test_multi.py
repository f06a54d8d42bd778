"""MultiUSMesh: two warped groups (wing, sphere) and a fixed background group
behind one solver ordering, against one USMesh per group."""
import numpy as np
import pytest

from tests.meshes import OPTS


def _parts():
    from idwarp_gb300 import synthetic as S

    w = S.wing_shell(ni=25, nj=9, nk=6, first=1e-3, far=5.0)
    s = S.sphere_ogrid(n=6, layers=5, r_out=8.0)
    c = np.array([0.5, 4.5, 0.0])
    s = dict(s, xv0=0.5 * s["xv0"] + c, pts=0.5 * s["pts"] + c)
    bg = np.random.default_rng(3).uniform(-10, 10, size=(500, 3))
    return w, s, bg


class _FakeMesh:
    """Stands in for USMesh to test MultiUSMesh's host logic on the CPU."""

    def __init__(self, options=None, comm=None, debug=False):
        self.options = options

    def createCommonGrid(self, x):
        self.x = np.asarray(x).ravel().copy()

    def setExternalMeshIndices(self, ind):
        self.ind = np.asarray(ind)

    def getSolverGrid(self):
        return self.x[self.ind] + 1.0  # "warped": shifted by one

    def setSurfaceDefinition(self, pts, conn, faceSizes):
        self.pts, self.conn, self.faceSizes = np.array(pts), np.array(conn), np.array(faceSizes)

    def getSurfaceCoordinates(self):
        return self.pts


def test_routing_and_solver_order_on_cpu(monkeypatch):
    import idwarp_gb300.MultiUnstructuredMesh as MM

    monkeypatch.setattr(MM, "USMesh", _FakeMesh)
    w, s, bg = _parts()
    grids = [("wing", w["xv0"], 1), ("background", bg, 1), ("sphere", s["xv0"], 2)]
    mm = MM.MultiUSMesh(grids, {"wing": {}, "sphere": {}})
    ncoord = 3 * (len(w["xv0"]) + len(bg) + len(s["xv0"]))
    ind = np.random.default_rng(4).permutation(ncoord)[: ncoord // 3]
    mm.setExternalMeshIndices(ind)
    full = np.concatenate([w["xv0"], bg, s["xv0"]]).ravel()
    nw3 = 3 * len(w["xv0"])
    shift = np.where((ind < nw3) | (ind >= nw3 + bg.size), 1.0, 0.0)  # background stays put
    np.testing.assert_array_equal(mm.getSolverGrid(), full[ind] + shift)
    nwp = len(w["pts"])
    pts = np.concatenate([w["pts"], s["pts"]])
    conn = np.concatenate([w["conn"], s["conn"] + nwp])
    fs = np.concatenate([w["faceSizes"], s["faceSizes"]])
    blk = np.concatenate([np.zeros(len(w["faceSizes"]), int), 2 + (np.arange(len(s["faceSizes"])) % 2)])
    mm.setSurfaceDefinition(pts, conn, fs, blk)
    wing, sph = mm.meshes
    np.testing.assert_array_equal(wing.pts, w["pts"])
    np.testing.assert_array_equal(wing.conn, w["conn"])
    np.testing.assert_array_equal(sph.pts, s["pts"])
    np.testing.assert_array_equal(sph.conn, s["conn"])
    np.testing.assert_array_equal(mm.getSurfaceCoordinates(), pts)


@pytest.mark.gpu
def test_multi_matches_single_instances(built_lib):
    from idwarp_gb300 import MultiUSMesh, USMesh
    from idwarp_gb300 import synthetic as S
    import contextlib
    import io

    w, s, bg = _parts()
    wopts = dict(OPTS, fileType="NPY", precision="fp64", symmetryPlanes=w["symmetryPlanes"])
    sopts = dict(OPTS, fileType="NPY", precision="fp64")
    grids = [("wing", w["xv0"], 1), ("background", bg, 1), ("sphere", s["xv0"], 2)]
    with contextlib.redirect_stdout(io.StringIO()):
        mm = MultiUSMesh(grids, {"wing": wopts, "sphere": sopts})
    ncoord = 3 * (len(w["xv0"]) + len(bg) + len(s["xv0"]))
    ind = np.random.default_rng(4).permutation(ncoord)[: ncoord // 2]
    mm.setExternalMeshIndices(ind)
    nwp = len(w["pts"])
    pts = np.concatenate([w["pts"], s["pts"]])
    conn = np.concatenate([w["conn"], s["conn"] + nwp])
    fs = np.concatenate([w["faceSizes"], s["faceSizes"]])
    blk = np.concatenate([np.zeros(len(w["faceSizes"]), int), 2 + (np.arange(len(s["faceSizes"])) % 2)])
    with contextlib.redirect_stdout(io.StringIO()):
        mm.setSurfaceDefinition(pts, conn, fs, blk)
    np.testing.assert_array_equal(mm.getSurfaceCoordinates(), pts)
    xs = np.concatenate([S.wing_perturbation(w["pts"], seed=2), S.sphere_perturbation(s["pts"], seed=0)])
    mm.setSurfaceCoordinates(xs)
    mm.warpMesh()
    got = mm.getSolverGrid()
    # reference: one USMesh per group on the full combined grid order
    full = np.concatenate([w["xv0"], bg, s["xv0"]]).ravel().copy()
    with contextlib.redirect_stdout(io.StringIO()):
        gw = USMesh(options=wopts)
        gw.createCommonGrid(w["xv0"])
        gw.setSurfaceDefinition(w["pts"], w["conn"], w["faceSizes"])
        gs = USMesh(options=sopts)
        gs.createCommonGrid(s["xv0"])
        gs.setSurfaceDefinition(s["pts"], s["conn"], s["faceSizes"])
    gw.setSurfaceCoordinates(xs[:nwp])
    gw.warpMesh()
    gs.setSurfaceCoordinates(xs[nwp:])
    gs.warpMesh()
    full[: 3 * len(w["xv0"])] = gw.getWarpGrid()
    full[3 * (len(w["xv0"]) + len(bg)):] = gs.getWarpGrid()
    np.testing.assert_allclose(got, full[ind], rtol=0, atol=1e-12)
    # reverse and forward products per group
    rng = np.random.default_rng(5)
    dxv = rng.normal(size=len(ind))
    dxs = mm.warpDeriv(dxv)
    dfull = np.zeros(ncoord)
    np.add.at(dfull, ind, dxv)
    gw.warpDeriv(dfull[: 3 * len(w["xv0"])], solverVec=False)
    gs.warpDeriv(dfull[3 * (len(w["xv0"]) + len(bg)):], solverVec=False)
    want = np.concatenate([gw.getdXs(), gs.getdXs()])
    np.testing.assert_allclose(dxs, want, rtol=0, atol=1e-11 * np.abs(want).max())
    tan = rng.normal(size=pts.shape)
    dv = mm.warpDerivFwd(tan)
    vfull = np.zeros(ncoord)
    vfull[: 3 * len(w["xv0"])] = gw.warpDerivFwd(tan[:nwp], solverVec=False)
    vfull[3 * (len(w["xv0"]) + len(bg)):] = gs.warpDerivFwd(tan[nwp:], solverVec=False)
    np.testing.assert_allclose(dv, vfull[ind], rtol=0, atol=1e-11 * np.abs(vfull).max())


def test_constructor_from_plot3d_file(monkeypatch, tmp_path):
    # MultiUSMesh(gridFile, optionsDict): a multi-block PLOT3D combined grid
    # with cgns_utils-style block names; blocks of one zone form one group
    import idwarp_gb300.MultiUnstructuredMesh as MM
    from idwarp_gb300 import Error
    from idwarp_gb300.plot3d import writePlot3D

    monkeypatch.setattr(MM, "USMesh", _FakeMesh)
    w, s, bg = _parts()
    half = len(s["xv0"]) // 2
    blocks = [w["xv0"], bg, s["xv0"][:half], s["xv0"][half:]]
    sizes = [[len(b), 1, 1] for b in blocks]
    f = tmp_path / "combined.xyz"
    writePlot3D(str(f), np.concatenate(blocks), sizes)
    names = ["wing.00000", "background.00000", "sphere.00000", "sphere.00001"]
    with pytest.raises(Error, match="block names"):
        MM.MultiUSMesh(str(f), {"wing": {}})
    (tmp_path / "combined.xyz.names").write_text("\n".join(names) + "\n")
    mm = MM.MultiUSMesh(str(f), {"wing": {}, "sphere": {}})
    assert mm.names == ["wing", "sphere"]
    assert mm.cgnsBlockIntervals == [[0, 1], [2, 4]]
    nw, nb = 3 * len(w["xv0"]), bg.size
    assert mm.cgnsVolNodeIntervals == [[0, nw], [nw + nb, nw + nb + s["xv0"].size]]
    np.testing.assert_array_equal(mm.meshes[1].x, s["xv0"].ravel())
    np.testing.assert_array_equal(mm.backgroundNodes[0], bg.ravel())
    # explicit names win over the file; scattered blocks of a zone are refused
    mm2 = MM.MultiUSMesh(f, {"wing": {}}, blockNames=["wing.0", "wing.1", "bg.0", "bg.1"])
    assert mm2.cgnsBlockIntervals == [[0, 2]]
    with pytest.raises(Error, match="not consecutive"):
        MM.MultiUSMesh(str(f), {"wing": {}}, blockNames=["wing.0", "bg.0", "wing.1", "bg.1"])
