"""The host kd-tree build (idwarp_gb300/csrc/idw_host.cpp, threaded above 4096
points) against the oracle's build_tree restatement, on the CPU: a small
driver compiled with g++ dumps the tree of the same merged, lexsorted surface
points the library builds from."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def kd_dump(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("kd") / "kd_dump")
    src = os.path.join(ROOT, "idwarp_gb300", "csrc")
    cmd = ["g++", "-O2", "-std=c++17", "-pthread", "-I", src, os.path.join(src, "idw_host.cpp"),
           os.path.join(ROOT, "tests", "host", "kd_dump.cpp"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _host_tree(exe, upts, bucket, tmp_path):
    fin, fout = tmp_path / "pts.bin", tmp_path / "tree.bin"
    np.ascontiguousarray(upts, dtype=np.float64).tofile(fin)
    r = subprocess.run([exe, str(fin), str(bucket), str(fout)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = fout.read_bytes()
    nn = int(np.frombuffer(raw, np.int32, 1)[0])
    ints = np.frombuffer(raw, np.int32, 4 * nn, 4).reshape(4, nn)
    dbl = np.frombuffer(raw, np.float64, 4 * nn, 4 + 16 * nn)
    return {"l": ints[0], "u": ints[1], "escape": ints[2], "leaf": ints[3], "X": dbl[:3 * nn].reshape(nn, 3),
            "oradius": dbl[3 * nn:]}


@pytest.mark.parametrize("which,bucket", [("sphere", 8), ("wing", 8), ("wing", 1), ("wing_12k", 8),
                                          ("wing_12k", 18)])
def test_host_tree_matches_oracle(which, bucket, kd_dump, tmp_path, oracle_lib):
    from oracle.pyoracle import point_reduce
    from idwarp_gb300 import synthetic as S
    from tests.meshes import build_oracle, sphere_small, wing_small

    if which == "sphere":
        m = sphere_small()
    elif which == "wing":
        m = wing_small()
    else:
        m = S.wing_shell(ni=201, nj=61, nk=3, first=1e-5, far=25.0)
    # the unique points as USMesh.setSurfaceDefinition makes them
    u, _, n = point_reduce(m["pts"], 1e-12)
    u = u[:n]
    u = u[np.lexsort(u.T)]
    host = _host_tree(kd_dump, u, bucket, tmp_path)
    to = build_oracle(m, {"bucketSize": bucket}).tree()
    np.testing.assert_array_equal(host["l"], to["l"])
    np.testing.assert_array_equal(host["u"], to["u"])
    np.testing.assert_array_equal(host["escape"], to["escape"])
    np.testing.assert_array_equal(host["leaf"] == 1, to["dnum"] == 0)
    np.testing.assert_allclose(host["X"], to["X"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(host["oradius"], to["oradius"], rtol=1e-13)
