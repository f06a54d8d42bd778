"""The complex type of the GPU's complex-step build (idw_cplx.cuh), compiled
as host C++ and checked against numpy's complex functions and the
real-valued derivatives: sqrt and division exactly as complex functions;
acos, sin, cos as the analytic continuation a complex step resolves
(imaginary parts of 1e-40 and of order one)."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "idwarp_gb300", "csrc")


@pytest.fixture(scope="module")
def cplx_bin(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("cplx") / "cplx_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", CSRC, os.path.join(ROOT, "tests", "host", "cplx_check.cpp"),
                    "-o", out], check=True)
    return out


def _run(binary, z):
    inp = "".join("%.17g %.17g\n" % (v.real, v.imag) for v in z)
    r = subprocess.run([binary], input=inp, capture_output=True, text=True, check=True)
    v = np.array([[float(t) for t in ln.split()] for ln in r.stdout.strip().splitlines()])
    return v[:, 0::2] + 1j * v[:, 1::2]


def test_complex_step_derivatives(cplx_bin):
    h = 1e-40
    x = np.array([0.3, 0.9, 1.7, 4.0, 1e-3, 123.0])
    out = _run(cplx_bin, x + 1j * h)
    sq, _, sn, cs, _ = out.T
    np.testing.assert_allclose(sq.real, np.sqrt(x), rtol=1e-15)
    np.testing.assert_allclose(sq.imag / h, 0.5 / np.sqrt(x), rtol=1e-14)
    np.testing.assert_allclose(sn.real, np.sin(x), rtol=1e-15)
    np.testing.assert_allclose(sn.imag / h, np.cos(x), rtol=1e-14)
    np.testing.assert_allclose(cs.real, np.cos(x), rtol=1e-15)
    np.testing.assert_allclose(cs.imag / h, -np.sin(x), rtol=1e-14)
    xa = np.array([-0.99, -0.5, 0.0, 0.3, 0.999999, 0.9999999999])
    ac = _run(cplx_bin, xa + 1j * h)[:, 1]
    np.testing.assert_allclose(ac.real, np.arccos(xa), rtol=1e-15)
    np.testing.assert_allclose(ac.imag / h, -1.0 / np.sqrt(1.0 - xa * xa), rtol=1e-12)
    # at the clamp (x = 1) the reference derivative is zero
    assert _run(cplx_bin, np.array([1.0 + 1j * h]))[0, 1].imag == 0.0


def test_complex_functions(cplx_bin):
    rng = np.random.default_rng(5)
    z = rng.normal(size=40) * 3 + 1j * rng.normal(size=40)
    z = np.concatenate([z, [-4.0 + 0j, -4.0 + 1e-30j, -4.0 - 1e-30j, 2j, 0j + 1e-300]])
    out = _run(cplx_bin, z)
    np.testing.assert_allclose(out[:, 0], np.sqrt(z), rtol=1e-15, atol=1e-300)
    np.testing.assert_allclose(out[:, 2], np.sin(z), rtol=1e-14)
    np.testing.assert_allclose(out[:, 3], np.cos(z), rtol=1e-14)
    w = z.imag + 1j * z.real
    ok = w != 0
    np.testing.assert_allclose(out[ok, 4], z[ok] / w[ok], rtol=1e-15)
