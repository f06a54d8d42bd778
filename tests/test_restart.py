"""Restart file of the denominator estimate (initializeWarping.F90:98-312):
the byte layout and the load/check/recompute decisions on the CPU; on the GPU
the dryRun load-balancing costs against the oracle, the estimate check and the
round trip through USMesh(restartFile=...)."""
import numpy as np
import pytest

from idwarp_gb300.restart import load_or_compute, read_restart, write_restart
from tests.meshes import build_gpu, build_oracle, sphere_small, wing_small


# ---------------------------------------------------------------- CPU
def test_layout_matches_reference_bytes(tmp_path):
    # int32 count, then the float64 estimate, then the float64 costs, native order
    den0 = np.array([1.5, 2.25, 3.0])
    costs = np.array([0.125, 0.5, 0.75])
    f = tmp_path / "r.bin"
    write_restart(str(f), den0, costs)
    raw = f.read_bytes()
    assert len(raw) == 4 + 16 * 3
    assert np.frombuffer(raw[:4], np.int32)[0] == 3
    np.testing.assert_array_equal(np.frombuffer(raw[4:28], np.float64), den0)
    np.testing.assert_array_equal(np.frombuffer(raw[28:], np.float64), costs)
    n, d, c = read_restart(str(f))
    assert n == 3
    np.testing.assert_array_equal(d, den0)
    np.testing.assert_array_equal(c, costs)


def test_truncated_and_missing_files(tmp_path):
    assert read_restart(str(tmp_path / "none.bin")) is None
    f = tmp_path / "short.bin"
    f.write_bytes(np.int32(10).tobytes() + np.zeros(5).tobytes())
    n, d, c = read_restart(str(f))
    assert n == 10 and d is None and c is None


class _Fake:
    """Stand-in for the device: the estimate is 1..n, the check accepts a
    loaded estimate when no checked node (every 100th) is above the truth by
    more than 1e-15 relative, as the reference's one-sided check."""

    def __init__(self, n):
        self.n = n
        self.truth = np.arange(1.0, n + 1.0)
        self.calls = []
        self.den0 = None

    def load(self, den0):
        self.calls.append("load")
        chk = np.arange(0, self.n, 100)
        if np.any(1.0 - self.truth[chk] / den0[chk] > 1e-15):
            return False
        self.den0 = den0
        return True

    def compute(self):
        self.calls.append("compute")
        self.den0 = self.truth.copy()

    def save(self):
        self.calls.append("save")
        return self.den0, np.full(self.n, 0.5)


def _run(path, fake):
    return load_or_compute(str(path), fake.n, fake.load, fake.compute, fake.save, log=lambda *a: None)


def test_restart_decisions(tmp_path):
    f = tmp_path / "r.bin"
    fake = _Fake(250)
    assert _run(f, fake) == "computed" and fake.calls == ["compute", "save"]
    assert read_restart(str(f))[0] == 250
    fake = _Fake(250)
    assert _run(f, fake) == "loaded" and fake.calls == ["load"]
    # a checked node above the truth: not accurate -> deleted, recomputed, saved
    n, d, c = read_restart(str(f))
    d[100] *= 2.0
    write_restart(str(f), d, c)
    fake = _Fake(250)
    assert _run(f, fake) == "computed" and fake.calls == ["load", "compute", "save"]
    np.testing.assert_array_equal(read_restart(str(f))[1], fake.truth)
    # an unchecked node, or a checked one below the truth, passes the check
    d = fake.truth.copy()
    d[101] *= 2.0
    d[200] *= 0.5
    write_restart(str(f), d, c)
    fake = _Fake(250)
    assert _run(f, fake) == "loaded"
    # another node count: recomputed and saved with the new count
    fake = _Fake(300)
    assert _run(f, fake) == "computed" and fake.calls == ["compute", "save"]
    assert read_restart(str(f))[0] == 300


# ---------------------------------------------------------------- GPU
@pytest.mark.gpu
@pytest.mark.parametrize("which", ["sphere", "wing"])
def test_dry_run_costs_match_oracle(which, built_lib, oracle_lib):
    m = sphere_small() if which == "sphere" else wing_small()
    om = build_oracle(m)
    ref = om.dry_run()
    g = build_gpu(m, precision="mixed")
    got = g.getLoadBalancingCosts()
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.gpu
def test_dry_run_costs_errtol_zero(built_lib):
    # no approximation is ever accepted: every interior node is visited (0.5)
    # and every point summed (1), on every mirror
    m = wing_small()
    g = build_gpu(m, {"errTol": 0.0}, precision="mixed")
    st = g.getStats()
    nInterior = int(np.sum(g.getTree()["isLeaf"] == 0))
    n = st["nUnique"]
    want = st["nLoop"] * (0.5 * nInterior + n) / n
    np.testing.assert_allclose(g.getLoadBalancingCosts(), want, rtol=1e-14)


@pytest.mark.gpu
def test_restart_file_roundtrip(tmp_path, built_lib):
    m = wing_small()
    f = tmp_path / "wing.restart"
    a = build_gpu(m, {"restartFile": str(f)}, precision="mixed")
    assert a.restartStatus == "computed"
    n, d, c = read_restart(str(f))
    assert n == len(m["xv0"])
    np.testing.assert_array_equal(d, a.getDenominator0())
    np.testing.assert_array_equal(c, a.getLoadBalancingCosts())
    a.setSurfaceCoordinates(m["xs"])
    a.warpMesh()
    xa = a.getWarpGrid()
    # a second instance loads the file and warps to the same bits
    b = build_gpu(m, {"restartFile": str(f)}, precision="mixed")
    assert b.restartStatus == "loaded"
    b.setSurfaceCoordinates(m["xs"])
    b.warpMesh()
    np.testing.assert_array_equal(b.getWarpGrid(), xa)
    # and so does one without a restart file
    c0 = build_gpu(m, precision="mixed")
    c0.setSurfaceCoordinates(m["xs"])
    c0.warpMesh()
    np.testing.assert_array_equal(c0.getWarpGrid(), xa)


@pytest.mark.gpu
def test_restart_file_rejected_cases(tmp_path, built_lib):
    m = sphere_small()
    f = tmp_path / "sphere.restart"
    build_gpu(m, {"restartFile": str(f)}, precision="fp64")
    n, d0, c0 = read_restart(str(f))
    # a checked node (every 100th from 0) above its estimate: recomputed and rewritten
    d = d0.copy()
    d[300] *= 1.0 + 1e-12
    write_restart(str(f), d, c0)
    g = build_gpu(m, {"restartFile": str(f)}, precision="fp64")
    assert g.restartStatus == "computed"
    np.testing.assert_array_equal(read_restart(str(f))[1], d0)
    # the reference's check is one-sided and sparse: a smaller checked value or
    # a changed unchecked one loads
    d = d0.copy()
    d[300] *= 0.5
    d[301] *= 2.0
    write_restart(str(f), d, c0)
    g = build_gpu(m, {"restartFile": str(f)}, precision="fp64")
    assert g.restartStatus == "loaded"
    # non-finite values or another node count: recomputed
    d = d0.copy()
    d[7] = np.nan
    write_restart(str(f), d, c0)
    assert build_gpu(m, {"restartFile": str(f)}, precision="fp64").restartStatus == "computed"
    write_restart(str(f), d0[:-1], c0[:-1])
    assert build_gpu(m, {"restartFile": str(f)}, precision="fp64").restartStatus == "computed"
    assert read_restart(str(f))[0] == n
