"""Seeded synthetic meshes and surface perturbations.

The reference's benchmark meshes are CGNS files downloaded at test time; no
CGNS library exists here, so these generators build the same kinds of
geometry in memory:

* ``sphere_ogrid``  — a cubed-sphere quad surface (6 patches, duplicated patch
  edges) inside a hexahedral O-grid shell with geometric radial stretching.
* ``wing_shell``    — a NACA0012 rectangular half-wing (semi-span 3c, root on
  the symmetry plane y=0, closed trailing edge, elliptical tip cap) inside a
  structured shell grid extruded along the wall normals, first spacing
  ``first`` (chords) stretched geometrically to ``far`` chords.

Each returns a dict with ``xv0`` (N_v, 3) volume nodes, ``pts`` (n_pts, 3)
surface points in the caller's (patch) order with duplicates, ``conn`` (flat,
0-based), ``faceSizes`` and ``symmetryPlanes`` in the reference's option form.
"""
import numpy as np


def _geometric(n, first, total):
    """n+1 distances 0=h_0<h_1<...<h_n=total with h_1=first, geometric growth."""
    if n == 1:
        return np.array([0.0, total])
    lo, hi = 1.0 + 1e-12, 4.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        s = first * (mid ** n - 1.0) / (mid - 1.0)
        if s > total:
            hi = mid
        else:
            lo = mid
    ratio = 0.5 * (lo + hi)
    h = first * (ratio ** np.arange(n + 1) - 1.0) / (ratio - 1.0)
    h *= total / h[-1]
    return h


def sphere_ogrid(n=18, layers=48, ratio=1.12, r_out=20.0):
    """Cubed-sphere O-grid: 6*(n+1)^2 surface pts (6n^2+2 unique), ~unique*(layers+1) volume nodes."""
    xi = np.tan(np.pi / 4 * np.linspace(-1.0, 1.0, n + 1))
    U, V = np.meshgrid(xi, xi, indexing="ij")
    one = np.ones_like(U)
    faces = [
        (one, U, V), (-one, V, U), (U, one, V), (V, -one, U), (U, V, one), (V, U, -one)
    ]
    pts = []
    conn = []
    off = 0
    for (a, b, c) in faces:
        p = np.stack([a, b, c], axis=-1).reshape(-1, 3)
        p /= np.linalg.norm(p, axis=1, keepdims=True)
        pts.append(p)
        idx = np.arange((n + 1) ** 2).reshape(n + 1, n + 1)
        q = np.stack([idx[:-1, :-1], idx[1:, :-1], idx[1:, 1:], idx[:-1, 1:]], axis=-1).reshape(-1, 4)
        conn.append(q + off)
        off += (n + 1) ** 2
    pts = np.concatenate(pts)
    conn = np.concatenate(conn).ravel().astype(np.intc)
    face_sizes = np.full(len(conn) // 4, 4, dtype=np.intc)
    # unique directions for the volume shell (exact duplicates on patch edges)
    key = np.round(pts * 1e12).astype(np.int64)
    _, first_idx = np.unique(key, axis=0, return_index=True)
    dirs = pts[np.sort(first_idx)]
    h = (ratio ** np.arange(layers + 1) - 1.0) / (ratio ** layers - 1.0)
    radii = 1.0 + (r_out - 1.0) * h
    xv0 = (radii[:, None, None] * dirs[None, :, :]).reshape(-1, 3)
    return {"xv0": xv0, "pts": pts, "conn": conn, "faceSizes": face_sizes, "symmetryPlanes": None,
            "name": "sphere_ogrid_n%d_l%d" % (n, layers)}


def _naca0012_closed(x):
    return 0.6 * (0.2969 * np.sqrt(x) - 0.1260 * x - 0.3516 * x ** 2 + 0.2843 * x ** 3 - 0.1036 * x ** 4)


def wing_shell(ni=401, nj=101, nk=50, first=1e-5, far=25.0, semispan=3.0, cap=0.05):
    """NACA0012 half-wing shell mesh: ni*nj surface pts, ni*nj*nk volume nodes."""
    th = np.linspace(0.0, 2.0 * np.pi, ni)
    x = 0.5 * (1.0 + np.cos(th))
    sgn = np.where(th < np.pi, -1.0, 1.0)
    s = np.linspace(-1.0, 1.0, nj)
    y = semispan * 0.5 * (1.0 + np.tanh(1.6 * s) / np.tanh(1.6))
    tfac = np.ones(nj)
    cap0 = semispan - cap
    m = y > cap0
    tfac[m] = np.sqrt(np.maximum(0.0, 1.0 - ((y[m] - cap0) / cap) ** 2))
    tfac[-1] = 0.0
    X = np.broadcast_to(x[None, :], (nj, ni))
    Y = np.broadcast_to(y[:, None], (nj, ni))
    Z = sgn[None, :] * _naca0012_closed(x)[None, :] * tfac[:, None]
    Z[:, 0] = 0.0
    Z[:, -1] = 0.0
    W = np.stack([X, Y, Z], axis=-1).astype(np.float64)  # (nj, ni, 3)
    # quad connectivity on the (j, i) grid
    idx = np.arange(nj * ni).reshape(nj, ni)
    q = np.stack([idx[:-1, :-1], idx[:-1, 1:], idx[1:, 1:], idx[1:, :-1]], axis=-1).reshape(-1, 4)
    # node normals: average of adjacent quad (diagonal cross product) normals
    P = W.reshape(-1, 3)
    d1 = P[q[:, 2]] - P[q[:, 0]]
    d2 = P[q[:, 3]] - P[q[:, 1]]
    fn = np.cross(d1, d2)
    fn /= np.linalg.norm(fn, axis=1, keepdims=True) + 1e-300
    N = np.zeros_like(P)
    for c in range(4):
        np.add.at(N, q[:, c], fn)
    N /= np.linalg.norm(N, axis=1, keepdims=True) + 1e-300
    # orient outward: at the root mid-chord upper surface the normal is +z
    probe = idx[nj // 2, (3 * ni) // 4]
    if N[probe, 2] < 0:
        N = -N
        q = q[:, ::-1].copy()
    # keep root nodes on the symmetry plane
    N[idx[0, :], 1] = 0.0
    N /= np.linalg.norm(N, axis=1, keepdims=True) + 1e-300
    h = _geometric(nk - 1, first, far)
    xv0 = (P[None, :, :] + h[:, None, None] * N[None, :, :]).reshape(-1, 3)
    conn = q.ravel().astype(np.intc)
    face_sizes = np.full(len(q), 4, dtype=np.intc)
    return {"xv0": xv0, "pts": P.copy(), "conn": conn, "faceSizes": face_sizes,
            "symmetryPlanes": [[[0.0, 0.0, 0.0], [0.0, 1.0, 0.0]]],
            "name": "wing_shell_%dx%dx%d" % (ni, nj, nk), "shape": (nk, nj, ni)}


def sphere_perturbation(pts, seed=0, angle_deg=5.0, n_bumps=4, amp=0.01, width=0.3):
    """5 deg rigid rotation about z plus Gaussian radial bumps (centres uniform on the sphere)."""
    rng = np.random.default_rng(seed)
    c = rng.normal(size=(n_bumps, 3))
    c /= np.linalg.norm(c, axis=1, keepdims=True)
    p = np.array(pts, dtype=np.float64)
    rad = p / np.linalg.norm(p, axis=1, keepdims=True)
    disp = np.zeros_like(p)
    for b in range(n_bumps):
        d2 = np.sum((p - c[b]) ** 2, axis=1)
        disp += amp * np.exp(-d2 / (2 * width ** 2))[:, None] * rad
    p = p + disp
    a = np.deg2rad(angle_deg)
    R = np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])
    return p @ R.T


def _bspline_basis(t, n_ctrl, degree=3):
    """Clamped uniform B-spline basis values at t in [0,1]; shape (len(t), n_ctrl)."""
    k = degree
    n_knots = n_ctrl + k + 1
    inner = np.linspace(0.0, 1.0, n_ctrl - k + 1)
    knots = np.concatenate([np.zeros(k), inner, np.ones(k)])
    assert len(knots) == n_knots
    t = np.clip(np.asarray(t, dtype=np.float64), 0.0, 1.0 - 1e-14)
    B = np.zeros((len(t), n_knots - 1))
    for i in range(n_knots - 1):
        B[:, i] = (knots[i] <= t) & (t < knots[i + 1])
    for d in range(1, k + 1):
        Bn = np.zeros((len(t), n_knots - 1 - d))
        for i in range(n_knots - 1 - d):
            den1 = knots[i + d] - knots[i]
            den2 = knots[i + d + 1] - knots[i + 1]
            a = (t - knots[i]) / den1 * B[:, i] if den1 > 0 else 0.0
            b = (knots[i + d + 1] - t) / den2 * B[:, i + 1] if den2 > 0 else 0.0
            Bn[:, i] = a + b
        B = Bn
    return B


def wing_perturbation(pts, seed=2, twist_tip_deg=-4.0, semispan=3.0, ffd=(8, 6, 2), sigma=0.005):
    """Linear twist 0 -> twist_tip about the quarter chord plus a cubic B-spline FFD z-field."""
    rng = np.random.default_rng(seed)
    p = np.array(pts, dtype=np.float64)
    ang = np.deg2rad(twist_tip_deg) * np.clip(p[:, 1] / semispan, 0.0, 1.0)
    xr = p[:, 0] - 0.25
    zr = p[:, 2]
    # rotation about the y axis through (0.25, y, 0); nose-down for negative angles
    xn = 0.25 + np.cos(ang) * xr + np.sin(ang) * zr
    zn = -np.sin(ang) * xr + np.cos(ang) * zr
    p[:, 0] = xn
    p[:, 2] = zn
    nx, ny, nz = ffd
    ctrl = rng.normal(0.0, sigma, size=(nx, ny, nz))
    lo = np.array([-0.05, 0.0, -0.1])
    hi = np.array([1.05, semispan + 0.05, 0.1])
    u = (np.asarray(pts)[:, 0] - lo[0]) / (hi[0] - lo[0])
    v = (np.asarray(pts)[:, 1] - lo[1]) / (hi[1] - lo[1])
    w = (np.asarray(pts)[:, 2] - lo[2]) / (hi[2] - lo[2])
    Bu = _bspline_basis(u, nx, min(3, nx - 1))
    Bv = _bspline_basis(v, ny, min(3, ny - 1))
    Bw = _bspline_basis(w, nz, min(3, nz - 1))
    dz = np.einsum("pi,pj,pk,ijk->p", Bu, Bv, Bw, ctrl)
    p[:, 2] += dz
    return p


def sphere_cells(n, layers):
    """Hexahedral cells (N, 8) of ``sphere_ogrid(n, layers)`` (volume node indices)."""
    xi = np.tan(np.pi / 4 * np.linspace(-1.0, 1.0, n + 1))
    m = sphere_ogrid(n=n, layers=1)
    pts = m["pts"]
    key = np.round(pts * 1e12).astype(np.int64)
    _, first_idx, inv = np.unique(key, axis=0, return_index=True, return_inverse=True)
    # volume nodes use the unique directions in order of first appearance
    order = np.argsort(np.argsort(first_idx))
    dir_of_pt = order[inv.ravel()]
    nd = len(first_idx)
    q = dir_of_pt[m["conn"].reshape(-1, 4)]
    cells = []
    for k in range(layers):
        cells.append(np.concatenate([q + k * nd, q + (k + 1) * nd], axis=1))
    del xi
    return np.concatenate(cells).astype(np.int64)


def wing_cells(ni, nj, nk):
    """Hexahedral cells (N, 8) of ``wing_shell(ni, nj, nk)`` (volume node indices)."""
    idx = np.arange(nk * nj * ni).reshape(nk, nj, ni)
    a = idx[:-1, :-1, :-1]
    b = idx[:-1, :-1, 1:]
    c = idx[:-1, 1:, 1:]
    d = idx[:-1, 1:, :-1]
    e = idx[1:, :-1, :-1]
    f = idx[1:, :-1, 1:]
    g = idx[1:, 1:, 1:]
    h = idx[1:, 1:, :-1]
    return np.stack([a, b, c, d, e, f, g, h], axis=-1).reshape(-1, 8).astype(np.int64)


def multibody(wing=(577, 261, 53), sphere=(158, 79), sphere_radius=0.5, sphere_center=(0.5, 4.5, 0.0),
              sphere_far=10.0):
    """Two bodies in one warp: the NACA0012 half-wing shell and a sphere O-grid
    (radius ``sphere_radius`` at ``sphere_center``, beside the wing tip), one
    surface definition and one volume point set (the two blocks overlap; IDW
    needs no connectivity).  ``cells`` lists the hexahedra of both blocks.
    Default sizes: 7.98M + 11.98M = 19.96M volume nodes, 150,597 + 151,686
    surface points."""
    ni, nj, nk = wing
    n, layers = sphere
    w = wing_shell(ni, nj, nk)
    s = sphere_ogrid(n=n, layers=layers, r_out=sphere_far / sphere_radius)
    c = np.asarray(sphere_center, dtype=np.float64)
    s_xv0 = s["xv0"] * sphere_radius + c
    s_pts = s["pts"] * sphere_radius + c
    nwv, nwp = len(w["xv0"]), len(w["pts"])
    cells = np.concatenate([wing_cells(ni, nj, nk), sphere_cells(n, layers) + nwv])
    xv0 = np.concatenate([w["xv0"], s_xv0])
    # orient every hexahedron so that its initial volume is positive
    flip = hex_volumes_np(xv0, cells) < 0
    cells[flip] = cells[flip][:, [4, 5, 6, 7, 0, 1, 2, 3]]
    return {"xv0": xv0, "pts": np.concatenate([w["pts"], s_pts]),
            "conn": np.concatenate([w["conn"], s["conn"] + nwp]).astype(np.intc),
            "faceSizes": np.concatenate([w["faceSizes"], s["faceSizes"]]).astype(np.intc),
            "symmetryPlanes": w["symmetryPlanes"], "cells": cells, "nWingPts": nwp,
            "name": "multibody_wing%dx%dx%d_sphere%dx%d" % (ni, nj, nk, n, layers)}


# six tetrahedra around the diagonal 0-6 of a hexahedron (corners 0-3 bottom,
# 4-7 top, both counter-clockwise seen from below)
HEX_TETS = ((0, 1, 2, 6), (0, 2, 3, 6), (0, 3, 7, 6), (0, 7, 4, 6), (0, 4, 5, 6), (0, 5, 1, 6))


def hex_volumes_np(xv, cells, chunk=1 << 20):
    """Signed volumes of hexahedra (sum of six tetrahedra), numpy."""
    out = np.empty(len(cells))
    for s0 in range(0, len(cells), chunk):
        x = xv[cells[s0:s0 + chunk]]
        v = 0.0
        for a, b, c, d in HEX_TETS:
            v = v + np.einsum("ij,ij->i", np.cross(x[:, b] - x[:, a], x[:, c] - x[:, a]), x[:, d] - x[:, a]) / 6.0
        out[s0:s0 + chunk] = v
    return out
