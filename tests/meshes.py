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
