"""GPU test of the device build of the double-float arithmetic of the DF_STAGE
mode (csrc/perthread/dfloat.cuh through mpgos_probe_df_math): every operation
gives the same two floats as the host build of the same header (the CPU
checker tests/dfloat_check.cpp in its "eval" mode, compiled here with g++),
and exp / log / pow / sin / cos keep the accuracy the CPU test asserts, now
measured on the device results against long double."""
import struct
import subprocess

import numpy as np
import pytest

from mpgos_gb300 import capi
from tests.conftest import REPO

pytestmark = pytest.mark.gpu

HEADER_DIR = REPO / "massively-parallel-gpu-ode-solver_gb300" / "csrc" / "perthread"


@pytest.fixture(scope="module")
def host_eval(tmp_path_factory):
    exe = tmp_path_factory.mktemp("dfloat_eval") / "dfloat_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{HEADER_DIR}",
                    str(REPO / "tests" / "dfloat_check.cpp"), "-o", str(exe)], check=True)

    def run(op, a, b):
        data = struct.pack("<iq", capi.DF_OPS[op], a.size) + a.tobytes() + b.tobytes()
        out = np.frombuffer(subprocess.run([str(exe), "eval"], input=data, capture_output=True, check=True).stdout,
                            dtype=np.float64)
        return out[0::2], out[1::2]
    return run


def _df(v):
    """The double-float a double converts to, as long double (hi + lo)."""
    hi = v.astype(np.float32)
    lo = (v - hi.astype(np.float64)).astype(np.float32)
    return hi.astype(np.longdouble) + lo.astype(np.longdouble)


def _inputs(op, rng, n=50000):
    u = rng.uniform
    if op == "exp":
        return np.where(np.arange(n) % 2 == 0, u(-69.0, 80.0, n), u(-1.0, 1.0, n)), np.zeros(n)
    if op == "log":
        return np.exp(u(-30.0, 30.0, n)), np.zeros(n)
    if op == "pow":
        return np.exp(u(-3.0, 3.0, n)), u(-6.0, 6.0, n)
    if op in ("sin", "cos", "sinpi", "cospi"):
        return np.where(np.arange(n) % 2 == 0, u(-2000.0, 2000.0, n), u(-1.0, 1.0, n)), np.zeros(n)
    if op == "sqrt":
        return np.exp(u(-20.0, 20.0, n)), np.zeros(n)
    if op == "pow_int":
        return u(0.5, 1.5, n), rng.integers(-6, 7, n).astype(np.float64)
    if op == "split":   # doubles across float's range, both signs, plus the fallback's ranges
        v = rng.choice([-1.0, 1.0], n) * (1.0 + u(0.0, 1.0, n)) * 2.0 ** rng.integers(-140, 140, n)
        v[:8] = [0.0, -0.0, 1.0, 10.0, 1e-30, 3e38, 1e300, 1e-300]
        return v, np.zeros(n)
    signs = rng.choice([-1.0, 1.0], (2, n))
    return signs[0] * u(0.5, 1.0, n) * 2.0 ** rng.integers(-8, 8, n), signs[1] * u(0.5, 1.0, n) * 2.0 ** rng.integers(-8, 8, n)


@pytest.mark.parametrize("op", sorted(k for k in capi.DF_OPS if not k.startswith("root")))
def test_device_build_equals_host_build(op, host_eval, native_libs):
    a, b = _inputs(op, np.random.default_rng(7))
    dh, dl = capi.df_math(op, a, b)
    hh, hl = host_eval(op, a, b)
    np.testing.assert_array_equal(dh.view(np.uint64), hh.view(np.uint64), err_msg=f"{op}: hi")
    np.testing.assert_array_equal(dl.view(np.uint64), hl.view(np.uint64), err_msg=f"{op}: lo")


def test_device_exp_log_pow_sin_cos_accuracy(native_libs):
    """Bars of the CPU test: exp, log, pow within a few units of
    2^-48 (|argument| + 1) relative; sin, cos within a few times the argument's
    own double-float precision."""
    rng = np.random.default_rng(11)
    ulp48 = np.longdouble(2.0) ** -48

    def value(op, a, b=None):
        h, l = capi.df_math(op, a, b)
        return h.astype(np.longdouble) + l.astype(np.longdouble)

    x, _ = _inputs("exp", rng)
    X = _df(x)
    assert np.max(np.abs(value("exp", x) - np.exp(X)) / np.exp(X) / (ulp48 * (np.abs(X) + 1))) < 2.5
    a, _ = _inputs("log", rng)
    A = _df(a)
    assert np.max(np.abs(value("log", a) - np.log(A)) / (ulp48 * (np.abs(np.log(A)) + 1))) < 3.0
    a, b = _inputs("pow", rng)
    A, B = _df(a), _df(b)
    P = np.exp(B * np.log(A))
    assert np.max(np.abs(value("pow", a, b) - P) / P / (ulp48 * (np.abs(B * np.log(A)) + 1))) < 10.0
    x, _ = _inputs("sin", rng)
    X = _df(x)
    bound = np.abs(X) * ulp48 + np.longdouble(2.0) ** -50
    for op, f in (("sin", np.sin), ("cos", np.cos)):
        assert np.max(np.abs(value(op, x) - f(X)) / bound) < 4.0, op


def test_device_split_step_factor_is_fp64_accurate(native_libs):
    """The split controller's R^(1/5) and R^(1/4) on the device (FP32 log2 /
    exp2 estimate on the MUFU unit, FP64 correction): within 4 ulp of the
    exact root for ratios over twelve decades and errors over 60 binades."""
    rng = np.random.default_rng(13)
    n = 50000
    err = (1.0 + rng.uniform(0.0, 1.0, n)) * 2.0 ** -rng.integers(0, 60, n)
    tol = err * 10.0 ** rng.uniform(-6.0, 6.0, n)
    for op, p in (("root5", 5), ("root4", 4)):
        y, lo = capi.df_math(op, tol, err)
        exact = (tol.astype(np.longdouble) / err.astype(np.longdouble)) ** (np.longdouble(1) / p)
        ulp = np.spacing(exact.astype(np.float64)).astype(np.longdouble)
        assert np.all(lo == 0.0)
        bad = ~np.isfinite(y)
        assert not bad.any(), (op, int(bad.sum()), tol[bad][:4].tolist(), err[bad][:4].tolist(), y[bad][:4].tolist())
        assert np.all(np.isfinite(exact.astype(np.float64)))
        ratio = (np.abs(y.astype(np.longdouble) - exact) / ulp).astype(np.float64)
        worst = int(np.argmax(ratio))
        assert ratio[worst] <= 4.0, (op, float(ratio[worst]), float(tol[worst]), float(err[worst]), float(y[worst]))
