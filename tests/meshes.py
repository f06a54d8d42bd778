"""Small seeded test meshes shared by the CPU and GPU tests."""
import numpy as np

from idwarp_gb300 import synthetic as S

OPTS = {
    "aExp": 3.0,
    "bExp": 5.0,
    "LdefFact": 1.0,
    "alpha": 0.25,
    "errTol": 1e-4,
    "evalMode": "fast",
    "useRotations": True,
    "bucketSize": 8,
}


def sphere_small():
    m = S.sphere_ogrid(n=10, layers=12)
    m["xs"] = S.sphere_perturbation(m["pts"], seed=0)
    return m


def wing_small():
    m = S.wing_shell(ni=41, nj=17, nk=10, first=1e-4, far=10.0)
    m["xs"] = S.wing_perturbation(m["pts"], seed=2)
    return m


def build_oracle(m, opts=None, sym=True):
    from oracle.pyoracle import OracleMesh

    o = dict(OPTS)
    o.update(opts or {})
    om = OracleMesh(o)
    om.set_volume(m["xv0"])
    planes = m.get("symmetryPlanes") if sym else None
    if planes:
        om.set_symmetry(np.array([p[0] for p in planes]), np.array([p[1] for p in planes]))
    else:
        om.set_symmetry(np.zeros((0, 3)), np.zeros((0, 3)))
    om.set_surface_definition(m["pts"], m["conn"], m["faceSizes"])
    return om


def build_gpu(m, opts=None, sym=True, precision="fp64"):
    import contextlib
    import io

    from idwarp_gb300 import USMesh

    o = dict(OPTS)
    o.update(opts or {})
    o["fileType"] = "NPY"
    o["precision"] = precision
    planes = m.get("symmetryPlanes") if sym else None
    if planes:
        o["symmetryPlanes"] = planes
    with contextlib.redirect_stdout(io.StringIO()):
        mesh = USMesh(options=o)
        mesh.createCommonGrid(m["xv0"])
        mesh.setSurfaceDefinition(m["pts"], m["conn"], m["faceSizes"])
    return mesh


def open_cylinder(n_around=24, n_along=8, radius=1.0, length=3.0, n_vol=3000, seed=3):
    """An open tube (radius, axis z, no end caps) of quads and seeded volume
    points around it.  Every surface normal is perpendicular to z, so a
    rotation about z is what each node's Rodrigues rotation reproduces."""
    th = np.linspace(0.0, 2 * np.pi, n_around, endpoint=False)
    z = np.linspace(0.0, length, n_along + 1)
    pts = np.array([[radius * np.cos(t), radius * np.sin(t), zz] for zz in z for t in th])
    conn = []
    for j in range(n_along):
        for i in range(n_around):
            a = j * n_around + i
            b = j * n_around + (i + 1) % n_around
            conn += [a, b, b + n_around, a + n_around]
    rng = np.random.default_rng(seed)
    r = rng.uniform(1.2, 6.0, n_vol)
    t = rng.uniform(0.0, 2 * np.pi, n_vol)
    xv0 = np.stack([r * np.cos(t), r * np.sin(t), rng.uniform(-1.0, length + 1.0, n_vol)], axis=1)
    return {"pts": pts, "conn": np.array(conn, dtype=np.int32), "faceSizes": np.full(n_along * n_around, 4, np.int32),
            "xv0": xv0}


def rotation_z(deg):
    c, s = np.cos(np.radians(deg)), np.sin(np.radians(deg))
    return np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])
