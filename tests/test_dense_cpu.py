"""CPU checks of the dense-output interpolation oracle (the statement the GPU
kernel csrc/perthread/dense_interp.cuh is compared with on the GPU).

Cubic Hermite interpolation between consecutive accepted steps, slopes from
the right-hand side: it reproduces every stored point exactly, gives NaN
outside the stored range, and between the points it agrees with an
independent integration to the requested time within the interpolant's
O(h^4) error (measured ~2e-8 median, 7.5e-8 max at tol 1e-10 for this case).
"""
import numpy as np
import pytest

from mpgos_gb300 import workloads as W
from oracle import oracle as O


@pytest.fixture(scope="module")
def dense_run(oracle_libs):
    case = W.duffing_param_case(nt=64, periods=2, tol=1e-10, ndo=2048)
    return case, O.run_oracle(case)


def test_stored_points_are_reproduced_and_outside_is_nan(dense_run):
    case, ref = dense_run
    for i in (0, 17, 63):
        k = ref["didx"][i]
        assert 0 < k < case.ndo
        ts = ref["dtime"][:k, i]
        out = O.dense_interpolate(case, ref["didx"], ref["dtime"], ref["dstate"], ts)
        np.testing.assert_array_equal(out[:, :, i], ref["dstate"][:k, :, i])
    T = case.arrays["td"][1][0]
    out = O.dense_interpolate(case, ref["didx"], ref["dtime"], ref["dstate"], [-1e-9, T + 1e-9])
    assert np.isnan(out).all()


def test_interpolation_error_between_steps(dense_run):
    case, ref = dense_run
    T = case.arrays["td"][1][0]
    times = np.linspace(0.05, T - 0.05, 13)
    out = O.dense_interpolate(case, ref["didx"], ref["dtime"], ref["dstate"], times)
    worst = 0.0
    for j, tau in enumerate(times):
        c = W.duffing_param_case(nt=64, periods=2, tol=1e-13)
        c.arrays["td"][1][:] = tau
        x = O.run_oracle(c)["x"]
        worst = max(worst, float(np.max(np.abs(out[j] - x))))
    assert worst < 3e-7, worst


def test_empty_dense_output_gives_nan(oracle_libs):
    case = W.duffing_param_case(nt=8, periods=1, ndo=4)
    didx = np.zeros(8, np.int32)
    out = O.dense_interpolate(case, didx, np.zeros((4, 8)), np.zeros((4, 2, 8)), [0.0, 1.0])
    assert np.isnan(out).all()
