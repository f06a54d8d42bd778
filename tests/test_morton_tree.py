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


def _parallel_build(pts, bucket):
    """The device build's index arithmetic (idw_tree.cu: k_tree_radix,
    k_tree_keep, k_tree_nodes), one interior node at a time: direction and
    range from the common-prefix lengths with the neighbours, the split by
    binary search, the cut at bucket-size nodes, preorder by sorting the kept
    ranges on (first ascending, last descending), escapes by binary search."""
    import bisect

    n = len(pts)
    code = [int(c) for c in _codes(pts)]
    perm = sorted(range(n), key=lambda i: code[i])  # stable: ties keep the point order
    k = [code[i] for i in perm]

    def prefix(i, j):
        if j < 0 or j >= n:
            return -1
        if k[i] != k[j]:
            return 64 - (k[i] ^ k[j]).bit_length()
        return 64 + 32 - (i ^ j).bit_length()

    nr = 2 * n - 1
    parent = [-1] * nr
    rng = [None] * max(n - 1, 1)
    for i in range(n - 1):
        d = 1 if prefix(i, i + 1) > prefix(i, i - 1) else -1
        dmin = prefix(i, i - d)
        lmax = 2
        while prefix(i, i + lmax * d) > dmin:
            lmax *= 2
        ln, t = 0, lmax // 2
        while t >= 1:
            if prefix(i, i + (ln + t) * d) > dmin:
                ln += t
            t //= 2
        j = i + ln * d
        dnode = prefix(i, j)
        s, div = 0, 2
        while True:
            t = (ln + div - 1) // div
            if prefix(i, i + (s + t) * d) > dnode:
                s += t
            if t <= 1:
                break
            div *= 2
        gamma = i + s * d + (-1 if d < 0 else 0)
        lo, hi = min(i, j), max(i, j)
        left = n - 1 + gamma if lo == gamma else gamma
        right = n - 1 + gamma + 1 if hi == gamma + 1 else gamma + 1
        rng[i] = (lo, hi)
        assert parent[left] == -1 and parent[right] == -1  # every node has one parent
        parent[left] = parent[right] = i
    keys = []
    for r in range(nr):
        g = rng[r] if r < n - 1 else (r - (n - 1), r - (n - 1))
        p = parent[r]
        if p < 0 or rng[p][1] - rng[p][0] > bucket:
            keys.append((g[0] << 32) | (0xFFFFFFFF - g[1]))
    keys.sort()
    nodes = []
    for kk, key in enumerate(keys):
        lo, hi = key >> 32, 0xFFFFFFFF - (key & 0xFFFFFFFF)
        esc = bisect.bisect_left(keys, (hi + 1) << 32, kk + 1)
        nodes.append((lo, hi, esc, hi - lo <= bucket))
    return perm, nodes


@pytest.mark.parametrize("bucket", [1, 8])
@pytest.mark.parametrize("name", ["sphere", "wing"])
def test_parallel_construction_equals_oracle(name, bucket, oracle_lib):
    from oracle.pyoracle import point_reduce

    m = _mesh(name)
    om = build_oracle(m, {"treeBuild": "morton", "bucketSize": bucket})
    t = om.tree()
    uniq, _, _ = point_reduce(m["pts"])
    srt = uniq[np.lexsort(uniq.T)]  # the unique points in the order the tree receives them
    perm, nodes = _parallel_build(srt, bucket)
    np.testing.assert_array_equal(srt[perm], om.surface()["Xu0"])
    nodes = np.array(nodes)
    np.testing.assert_array_equal(nodes[:, 0], t["l"])
    np.testing.assert_array_equal(nodes[:, 1], t["u"])
    np.testing.assert_array_equal(nodes[:, 2], t["escape"])
    np.testing.assert_array_equal(nodes[:, 3] == 1, t["dnum"] == 0)


@pytest.mark.parametrize("n", [1, 2, 3, 9, 100, 700])
def test_parallel_construction_random_clouds(n):
    # tied codes (points 1e-12 apart) and tiny clouds; the radius pass's
    # 256-point tasks (k_tree_radius) cover every (node, point) pair once
    rng = np.random.default_rng(n)
    pts = rng.standard_normal((n, 3))
    if n > 10:
        pts[n // 2:n // 2 + 5] = pts[n // 2] + 1e-12 * np.arange(5)[:, None]
    for bucket in (1, 2, 8):
        _, nodes = _parallel_build(pts, bucket)
        nodes = np.array(nodes)
        leaf = nodes[:, 3] == 1
        lv = nodes[leaf]
        assert lv[0, 0] == 0 and lv[-1, 1] == n - 1 and np.all(lv[1:, 0] == lv[:-1, 1] + 1)
        for kk in np.flatnonzero(~leaf):
            a = kk + 1
            b = nodes[a, 2]
            assert nodes[a, 0] == nodes[kk, 0] and nodes[b, 1] == nodes[kk, 1] and nodes[b, 0] == nodes[a, 1] + 1
        for task in (256, 4):
            chunks = (nodes[:, 1] - nodes[:, 0] + task) // task
            incl = np.cumsum(chunks)
            seen = set()
            for c in range(int(incl[-1])):
                a = int(np.searchsorted(incl, c, side="right"))
                first = incl[a] - chunks[a]
                i0 = nodes[a, 0] + (c - first) * task
                i1 = min(nodes[a, 1], i0 + task - 1)
                assert nodes[a, 0] <= i0 <= i1 <= nodes[a, 1]
                for i in range(i0, i1 + 1):
                    assert (a, i) not in seen
                    seen.add((a, i))
            assert len(seen) == int((nodes[:, 1] - nodes[:, 0] + 1).sum())
