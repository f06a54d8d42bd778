"""Generate the golden fixtures of the warping path with the oracle.

The reference's own regression values (tests/ref/*.ref of mdolab/idwarp) are
sums over CGNS meshes that are not distributed with it, and the reference
(Fortran + PETSc + CGNS) cannot be built in this environment, so these
fixtures are produced by the oracle (oracle/idw_oracle.cpp, the CPU FP64
restatement of the reference algorithm) on small seeded synthetic meshes.
They follow the reference test procedure of tests/test_USMesh.py:
  * options of tests/test_USMesh.py:129-141 (aExp 3, bExp 5, LdefFact 1,
    alpha 0.25, errTol 5e-4, fast mode, bucketSize 8, rotations on);
  * the "shearing sweep" perturbation x += 0.05 z (test_USMesh.py:55-58) and
    the "inflate" perturbation x *= 1.1, y *= 1.2, z *= 1.3 (:50-54);
  * sums of the initial and warped grids (:44-46, :64-67);
  * warpDeriv with dXv = linspace(0, 1, ndof) and the sum of dXs (:70-76);
  * the complex-step check: a complex perturbation i*h on every surface
    coordinate, sum(dXv . Im(Xv)/h) (:80-91), which must equal sum(dXs).

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from idwarp_gb300 import synthetic as S  # noqa: E402
from oracle.pyoracle import OracleMesh  # noqa: E402

REF_OPTS = {"aExp": 3.0, "bExp": 5.0, "LdefFact": 1.0, "alpha": 0.25, "errTol": 5e-4, "evalMode": "fast",
            "useRotations": True, "zeroCornerRotations": True, "cornerAngle": 30.0, "bucketSize": 8}


def cases():
    sph = S.sphere_ogrid(n=8, layers=10)
    wing = S.wing_shell(ni=33, nj=13, nk=10, first=1e-4, far=10.0)
    return {
        "sphere_shear": (sph, "shear"),
        "sphere_inflate": (sph, "inflate"),
        "wing_sym_shear": (wing, "shear"),
    }


def perturb(pts, kind):
    x = np.array(pts, dtype=np.float64)
    if kind == "shear":
        x[:, 0] += 0.05 * x[:, 2]
    else:
        x[:, 0] *= 1.1
        x[:, 1] *= 1.2
        x[:, 2] *= 1.3
    return x


def oracle_mesh(m, mode):
    o = dict(REF_OPTS)
    o["evalMode"] = mode
    om = OracleMesh(o)
    om.set_volume(m["xv0"])
    if m.get("symmetryPlanes"):
        om.set_symmetry(np.array([p[0] for p in m["symmetryPlanes"]]), np.array([p[1] for p in m["symmetryPlanes"]]))
    om.set_surface_definition(m["pts"], m["conn"], m["faceSizes"])
    return om


def make(m, kind):
    xs = perturb(m["pts"], kind)
    out = {"xv0": m["xv0"], "pts": m["pts"], "conn": m["conn"], "faceSizes": m["faceSizes"], "xs": xs,
           "symmetry": np.array(m["symmetryPlanes"] if m.get("symmetryPlanes") else np.zeros((0, 2, 3)),
                                dtype=np.float64).reshape(-1, 2, 3)}
    for mode in ("fast", "exact"):
        om = oracle_mesh(m, mode)
        om.set_surface_coordinates(xs)
        xv = om.warp()
        out["xv_" + mode] = xv
        st = om.stats()
        out["leafPairs_" + mode] = np.int64(st["leafPairs"])
        out["approx_" + mode] = np.int64(st["approx"])
        if mode == "fast":
            out["ldef0"] = np.float64(om.ldef0())
            out["den0"] = om.den0()
            out["sum_initial"] = np.float64(np.sum(m["xv0"]))
            out["sum_warped"] = np.float64(np.sum(xv))
            dxv = np.linspace(0.0, 1.0, 3 * len(m["xv0"]))
            dxs = om.warp_deriv(dxv.reshape(-1, 3))
            out["dxs"] = dxs
            out["sum_dxs"] = np.float64(np.sum(dxs))
            h = 1e-40
            xvi = om.warp_complex(xs + 1j * h).imag
            out["sum_complex_step"] = np.float64(np.dot(dxv, (xvi / h).ravel()))
    return out


def sensitivity(m, kind, data):
    """How far the same oracle source compiled with FMA contraction moves the
    results: the rounding sensitivity of the reference formulas on this case
    (small rotation angles make the Rodrigues angle acos(n0 . n) ill-conditioned).
    A correct implementation can differ from the fixture by this much."""
    from oracle.build import build_oracle_contracted
    from oracle.pyoracle import use_library

    use_library(build_oracle_contracted())
    try:
        other = make(m, kind)
    finally:
        use_library(None)
    out = {}
    for mode in ("fast", "exact"):
        out["sens_xv_" + mode] = np.float64(np.abs(other["xv_" + mode] - data["xv_" + mode]).max() / data["ldef0"])
    out["sens_dxs"] = np.float64(np.abs(other["dxs"] - data["dxs"]).max() / np.abs(data["dxs"]).max())
    return out


def main():
    for name, (m, kind) in cases().items():
        data = make(m, kind)
        data.update(sensitivity(m, kind, data))
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **data)
        print(name, os.path.getsize(path), "bytes", "sum_warped %.15g sum_dxs %.15g cs %.15g" % (
            data["sum_warped"], data["sum_dxs"], data["sum_complex_step"]),
            "sensitivity xv %.1e/%.1e dxs %.1e" % (data["sens_xv_fast"], data["sens_xv_exact"], data["sens_dxs"]))


if __name__ == "__main__":
    main()
