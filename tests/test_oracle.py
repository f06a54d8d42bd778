"""CPU tests of the oracle (the FP64 restatement of the reference path).

The reference (Fortran + PETSc/MPI) cannot be built here and its regression
meshes are not available, so the oracle is checked against the identities the
reference's own tests and examples use: the adjoint/forward dot product
(examples/structured/dotprod.py:38-49), central differences
(src/warp/verifyWarpDeriv.F90), complex step (tests/test_USMesh.py:88-100),
and analytic invariants of the method.
"""
import numpy as np
import pytest

from tests.meshes import OPTS, build_oracle, sphere_small, wing_small


@pytest.fixture(scope="module")
def sphere():
    return sphere_small()


@pytest.fixture(scope="module")
def wing():
    return wing_small()


def test_point_reduce_semantics(oracle_lib):
    from oracle.pyoracle import point_reduce

    pts = np.array([[0, 0, 0], [1, 0, 0], [0, 0, 0], [1, 0, 1e-13], [2, 0, 0], [1, 0, 0]], dtype=float)
    uniq, link, nu = point_reduce(pts, 1e-12)
    assert nu == 3
    assert list(link) == [1, 2, 1, 2, 3, 2]
    np.testing.assert_array_equal(uniq[1], [1, 0, 0])


def test_point_reduce_sphere_counts(sphere, oracle_lib):
    from oracle.pyoracle import point_reduce

    _, link, nu = point_reduce(sphere["pts"])
    assert nu == 6 * 10 * 10 + 2
    assert link.min() == 1 and link.max() == nu


@pytest.mark.parametrize("mode", ["fast", "exact"])
def test_rigid_translation(sphere, mode, oracle_lib):
    om = build_oracle(sphere, {"evalMode": mode})
    t = np.array([0.3, -0.2, 0.1])
    om.set_surface_coordinates(sphere["pts"] + t)
    xv = om.warp()
    np.testing.assert_allclose(xv - sphere["xv0"], np.broadcast_to(t, xv.shape), atol=1e-13)


@pytest.mark.parametrize("mode", ["fast", "exact"])
def test_rigid_rotation_about_the_normals_plane(mode, oracle_lib):
    # every normal of an open tube is perpendicular to its axis: turning the
    # tube about the axis gives every node M_i = R and b_i = 0, so the warped
    # volume is the same rotation of the initial one
    from tests.meshes import open_cylinder, rotation_z

    m = open_cylinder()
    R = rotation_z(10.0)
    om = build_oracle(m, {"evalMode": mode}, sym=False)
    om.set_surface_coordinates(m["pts"] @ R.T)
    xv = om.warp()
    np.testing.assert_allclose(xv, m["xv0"] @ R.T, rtol=0, atol=1e-12)


def test_identity_surface_gives_identity_volume(sphere, oracle_lib):
    om = build_oracle(sphere)
    om.set_surface_coordinates(sphere["pts"])
    xv = om.warp()
    np.testing.assert_allclose(xv, sphere["xv0"], atol=1e-13)


@pytest.mark.parametrize("mode", ["fast", "exact"])
def test_wall_nodes_follow_surface(sphere, mode, oracle_lib):
    # A volume node on a surface node has d^2 = eps, so that node's weight
    # dominates and S_i(Xu0_i) = Xu_i - Xu0_i: the wall nodes move with the wall.
    om = build_oracle(sphere, {"evalMode": mode})
    om.set_surface_coordinates(sphere["xs"])
    xv = om.warp()
    from oracle.pyoracle import point_reduce

    uniq, link, nu = point_reduce(sphere["pts"])
    # first shell of the O-grid is the unique surface points in first-seen order
    first = np.zeros(nu, dtype=int)
    seen = np.zeros(nu, dtype=bool)
    for i, l in enumerate(link):
        if not seen[l - 1]:
            first[l - 1] = i
            seen[l - 1] = True
    np.testing.assert_allclose(xv[:nu], sphere["xs"][first], atol=1e-12)


@pytest.mark.parametrize("mode", ["fast", "exact"])
@pytest.mark.parametrize("case", ["sphere", "wing"])
def test_dot_product(case, mode, sphere, wing, oracle_lib):
    m = sphere if case == "sphere" else wing
    om = build_oracle(m, {"evalMode": mode})
    om.set_surface_coordinates(m["xs"])
    om.warp()
    rng = np.random.default_rng(7)
    dxv = rng.normal(size=m["xv0"].shape)
    dxs_in = rng.normal(size=m["pts"].shape)
    dxs = om.warp_deriv(dxv)
    fwd = om.warp_deriv_fwd(dxs_in)
    a, b = np.sum(dxv * fwd), np.sum(dxs * dxs_in)
    assert abs(a - b) <= 1e-10 * (abs(a) + abs(b))


def test_central_difference(wing, oracle_lib):
    om = build_oracle(wing)
    om.set_surface_coordinates(wing["xs"])
    om.warp()
    rng = np.random.default_rng(3)
    dxv = rng.normal(size=wing["xv0"].shape)
    dxs = om.warp_deriv(dxv).ravel()
    h = 1e-6
    for dof in [0, 31, 200, 401]:
        x = wing["xs"].ravel().copy()
        x[dof] += h
        om.set_surface_coordinates(x.reshape(-1, 3))
        xp = om.warp()
        x[dof] -= 2 * h
        om.set_surface_coordinates(x.reshape(-1, 3))
        xm = om.warp()
        fd = np.sum(dxv * (xp - xm)) / (2 * h)
        assert abs(fd - dxs[dof]) <= 1e-5 * max(1.0, abs(fd)), (dof, fd, dxs[dof])
    om.set_surface_coordinates(wing["xs"])


def test_complex_step_matches_adjoint_columns(sphere, oracle_lib):
    om = build_oracle(sphere, {"evalMode": "fast"})
    om.set_surface_coordinates(sphere["xs"])
    om.warp()
    rng = np.random.default_rng(11)
    dxv = rng.normal(size=sphere["xv0"].shape)
    dxs = om.warp_deriv(dxv).ravel()
    h = 1e-40
    for dof in [3, 77, 500]:
        x = sphere["xs"].astype(complex).ravel()
        x[dof] += 1j * h
        xv = om.warp_complex(x.reshape(-1, 3))
        cs = np.sum(dxv * xv.imag) / h
        assert abs(cs - dxs[dof]) <= 1e-10 * max(1.0, abs(cs))


def test_symmetry_plane_mirror_consistency(wing, oracle_lib):
    # Mirrored volume nodes of a symmetric configuration stay on their side and
    # the symmetry-plane nodes keep y == 0 to rounding.
    om = build_oracle(wing)
    om.set_surface_coordinates(wing["xs"])
    xv = om.warp()
    on_plane = np.abs(wing["xv0"][:, 1]) < 1e-14
    assert np.abs(xv[on_plane, 1]).max() < 1e-12
    assert om.sizes()["nLoop"] == 2


def test_fast_converges_to_exact(wing, oracle_lib):
    errs = []
    ex = build_oracle(wing, {"evalMode": "exact"})
    ex.set_surface_coordinates(wing["xs"])
    xe = ex.warp()
    for tol in [1e-2, 1e-4, 1e-6, 0.0]:
        om = build_oracle(wing, {"errTol": tol})
        om.set_surface_coordinates(wing["xs"])
        errs.append(np.abs(om.warp() - xe).max())
    assert errs[0] >= errs[1] >= errs[2]
    # errTol = 0 never approximates: the walk then visits every leaf in tree
    # order, which is the exact loop's order, so the results are identical.
    assert errs[3] == 0.0


def test_tree_invariants(wing, oracle_lib):
    om = build_oracle(wing)
    t = om.tree()
    s = om.sizes()
    n = s["nUnique"]
    assert t["l"][0] == 0 and t["u"][0] == n - 1
    leaf = t["dnum"] == 0
    assert np.all(t["u"][leaf] - t["l"][leaf] <= OPTS["bucketSize"])
    # preorder: escape of the root is the node count, leaves cover [0,n) in order
    assert t["escape"][0] == s["nNodes"]
    cover = np.concatenate([np.arange(a, b + 1) for a, b in zip(t["l"][leaf], t["u"][leaf])])
    np.testing.assert_array_equal(cover, np.arange(n))
    # interior node area = sum of member areas
    surf = om.surface()
    csum = np.concatenate([[0.0], np.cumsum(surf["Ai"])])
    np.testing.assert_allclose(t["Ai"], csum[t["u"] + 1] - csum[t["l"]], rtol=1e-12)


def test_dry_run_costs_closed_form_at_errtol_zero(oracle_lib):
    # kd_tree.F90:789-830 with errTol 0: no approximation is accepted, so each
    # mirror walk visits every interior node (0.5) and every point (1), and the
    # cost of a node is nLoop (0.5 nInterior + n) / n
    from tests.meshes import wing_small

    m = wing_small()
    om = build_oracle(m, {"errTol": 0.0})
    t = om.tree()
    n = om.sizes()["nUnique"]
    nloop = om.sizes()["nLoop"]
    want = nloop * (0.5 * int(np.sum(t["dnum"] != 0)) + n) / n
    np.testing.assert_allclose(om.dry_run(), want, rtol=1e-14)
