"""CPU tests of the oracle: pinned against the reference's own solver.

The golden fixtures in tests/golden/ were produced by the reference's
per-thread kernel compiled for the CPU (tests/golden/make_golden.py). The
oracle restates that algorithm with the same floating-point expression
grouping, so on the machine and compiler flags the fixtures were made with
(x86-64, -ffp-contract=off) the two agree bit for bit; elsewhere the host math
library may round differently and the comparison falls back to 1e-9 relative.
"""
import platform

import numpy as np
import pytest

from tests.conftest import golden_files
from mpgos_gb300 import workloads as W
from oracle import build_oracle, oracle as O
from tests.golden.make_golden import load

BITWISE = platform.machine() in ("x86_64", "AMD64")
FLOAT_KEYS = ("td", "x", "t", "cp", "acc", "dtime", "dstate")
INT_KEYS = ("acci", "didx")


def assert_same(res, ref, bitwise):
    for k in FLOAT_KEYS:
        if k not in ref:
            continue
        a = np.asarray(res[k], dtype=np.float64).ravel()
        b = np.asarray(ref[k], dtype=np.float64).ravel()
        if bitwise:
            assert np.array_equal(a.view(np.uint64), b.view(np.uint64)), f"{k} differs bitwise"
        else:
            np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-12, err_msg=k)
    for k in INT_KEYS:
        if k in ref:
            np.testing.assert_array_equal(np.asarray(res[k]).ravel(), np.asarray(ref[k]).ravel(), err_msg=k)


@pytest.mark.parametrize("path", golden_files(), ids=lambda p: p.stem)
def test_oracle_matches_reference_golden(path, oracle_libs):
    case, ref = load(path)
    res = O.run_oracle(case)
    assert_same(res, ref, BITWISE)


def _random_cases():
    rng = np.random.default_rng(123)
    c = W.lorenz_case(nt=64, tol=1e-8, rho=(20.0, 28.0))
    c.arrays["x"][:] = rng.uniform(-5, 5, (3, 64))
    yield "lorenz_chaotic_window", c
    c = W.duffing_param_case(nt=256, periods=2, tol=1e-7, seed=5)
    yield "duffing_param_loose", c
    c = W.duffing_events_case(nt=64, periods=2, ndo=16, seed=3)
    c.options["dense_freq"] = 3
    c.options["dense_min_dt"] = 0.0
    yield "duffing_events_freq3", c
    c = W.keller_miksis_case(n_amp=4, n_freq=16, periods=1, amp=(1.0, 1.5), freq=(20.0, 60.0))
    yield "keller_miksis_strong", c


@pytest.mark.skipif(not build_oracle.reference_available(), reason="reference checkout not present")
@pytest.mark.parametrize("name,case", list(_random_cases()), ids=lambda v: v if isinstance(v, str) else "")
def test_oracle_matches_reference_cpu_build(name, case, oracle_libs):
    res = O.run_oracle(case)
    ref = O.run_ref_cpu(case)
    assert_same(res, ref, True)


def test_oracle_inactive_instances_untouched(oracle_libs):
    c = W.lorenz_case(nt=64)
    c.n_active = 40
    res = O.run_oracle(c)
    np.testing.assert_array_equal(res["x"][:, 40:], c.arrays["x"][:, 40:])
    assert np.all(res["t"][:40] == 10.0)
    assert np.all(res["t"][40:] == 0.0)


def test_oracle_zero_length_interval(oracle_libs):
    c = W.lorenz_case(nt=8)
    c.arrays["t"][:] = 10.0  # already at TD1: one zero-length step, accepted
    res = O.run_oracle(c)
    np.testing.assert_array_equal(res["x"], c.arrays["x"])
    assert np.all(res["nacc"] == 1)


def test_oracle_attempt_limit_flag(oracle_libs):
    c = W.lorenz_case(nt=8)
    c.options["max_attempts"] = 10
    res = O.run_oracle(c)
    assert np.all(res["status"] & 8)
    assert np.all(res["nacc"] + res["nrej"] == 10)


def test_oracle_nonfinite_state_stops(oracle_libs):
    c = W.lorenz_case(nt=4)
    c.arrays["x"][0, 1] = np.inf
    res = O.run_oracle(c)
    assert res["status"][1] & 1
    assert res["status"][0] == 0
