"""The Morton surface tree (option treeBuild "morton") on the CPU: the oracle's
restatement against the tree's definition, and its fast-mode error against
the reference kd tree's.

The tree has no counterpart in the reference (which builds the kd tree of
src/modules/kd_tree.F90:123-300); what is checked here is its definition:
points in Morton-code order (21 bits per axis over the bounding cube, ties
in point order), every interior node split where the highest differing bit
of its first and last key flips, leaves of at most bucketSize+1 points, the
kd tree's aggregates (setCenters, kd_tree.F90:558-593)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from tests.meshes import build_oracle, sphere_small, wing_small


def _codes(pts):
    # an independent restatement of the code: cell floor((x - lo) 2^21 / extent)
    # per axis (extent = largest side), bits x, y, z from the top of each triple
    lo, hi = pts.min(0), pts.max(0)
    ext = max(hi - lo)
    inv = 2097152.0 / ext if ext > 0 else 0.0
    q = np.minimum(np.floor((pts - lo) * inv), 2097151).astype(np.uint64)
    code = np.zeros(len(pts), dtype=np.uint64)
    for b in range(21):
        for c in range(3):
            code |= ((q[:, c] >> np.uint64(b)) & np.uint64(1)) << np.uint64(3 * b + 2 - c)
    return code


def _mesh(name):
    return sphere_small() if name == "sphere" else wing_small()


@pytest.mark.parametrize("bucket", [1, 8, 64])
@pytest.mark.parametrize("name", ["sphere", "wing"])
def test_oracle_tree_definition(name, bucket, oracle_lib):
    m = _mesh(name)
    om = build_oracle(m, {"treeBuild": "morton", "bucketSize": bucket})
    t = om.tree()
    xu0 = om.surface()["Xu0"]
    n = len(xu0)
    code = _codes(xu0)
    assert np.all(code[1:] >= code[:-1])
    keys = [(int(c) << 32) | i for i, c in enumerate(code)]  # ties keep the point order
    l, u, esc, leaf = t["l"], t["u"], t["escape"], t["dnum"] == 0
    nn = len(l)
    assert l[0] == 0 and u[0] == n - 1 and esc[0] == nn
    lv = np.flatnonzero(leaf)
    assert l[lv[0]] == 0 and u[lv[-1]] == n - 1 and np.all(l[lv[1:]] == u[lv[:-1]] + 1)
    assert np.all((u - l)[leaf] <= bucket) and np.all((u - l)[~leaf] > bucket)
    for k in np.flatnonzero(~leaf):
        a, b = k + 1, esc[k + 1]  # left child, right child
        assert l[a] == l[k] and u[b] == u[k] and l[b] == u[a] + 1 and esc[b] == esc[k]
        hb = (keys[l[k]] ^ keys[u[k]]).bit_length() - 1
        assert all((keys[i] >> hb) & 1 == 0 for i in range(l[a], u[a] + 1))
        assert all((keys[i] >> hb) & 1 == 1 for i in range(l[b], u[b] + 1))
    for k in range(nn):
        p = xu0[l[k]:u[k] + 1]
        # the sums are formed bottom-up: a few roundings per level from numpy's mean
        np.testing.assert_allclose(t["X"][k], p.mean(0), rtol=0, atol=1e-13 * np.abs(p).max())
        r = np.sqrt(((p - t["X"][k]) ** 2).sum(1)).max()
        if r > 0:
            assert abs(1.0 / t["oradius"][k] - r) <= 1e-14 * r


@pytest.mark.parametrize("name", ["sphere", "wing"])
def test_oracle_exact_mode_same_sum(name, oracle_lib):
    # exact mode sums every pair: the tree only changes the order
    m = _mesh(name)
    res = []
    for tb in ("kd", "morton"):
        om = build_oracle(m, {"evalMode": "exact", "treeBuild": tb})
        om.set_surface_coordinates(m["xs"])
        res.append(om.warp().copy())
    assert np.abs(res[0] - res[1]).max() / om.ldef0() < 1e-13


# max |fast - exact| / Ldef0 over the volume of the Morton tree, at most this
# factor times the kd tree's, at each errTol (the oracle measures 0.9 to 5.1)
ERR_FACTOR = 8.0


@pytest.mark.parametrize("name", ["sphere", "wing"])
def test_oracle_fast_error_report(name, oracle_lib):
    m = _mesh(name)
    ex = build_oracle(m, {"evalMode": "exact"})
    ex.set_surface_coordinates(m["xs"])
    xe = ex.warp().copy()
    L = ex.ldef0()
    prev = None
    for tol in (1e-3, 1e-4, 1e-5):
        err = {}
        for tb in ("kd", "morton"):
            om = build_oracle(m, {"treeBuild": tb, "errTol": tol})
            om.set_surface_coordinates(m["xs"])
            err[tb] = np.abs(om.warp() - xe).max() / L
        assert err["morton"] <= ERR_FACTOR * err["kd"], (tol, err)
        prev = err["morton"] if prev is None else prev
    assert err["morton"] < prev  # errTol 1e-5 against 1e-3


def test_struct_sizes_match_header(tmp_path):
    # the ctypes mirrors of the C structs have the header's layout
    from idwarp_gb300 import _lib

    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "idwarp_gb300.h"\n'
                   'int main(void) { printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(idw_options), sizeof(idw_stats), '
                   'sizeof(idw_tuning), offsetof(idw_options, treeBuild), offsetof(idw_stats, treeBuildMs), '
                   'offsetof(idw_options, deterministic)); return 0; }\n')
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-I", inc, str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert got == [C.sizeof(_lib.idw_options), C.sizeof(_lib.idw_stats), C.sizeof(_lib.idw_tuning),
                   _lib.idw_options.treeBuild.offset, _lib.idw_stats.treeBuildMs.offset,
                   _lib.idw_options.deterministic.offset]
