"""Edge cases of the launch: no active instance or system (Solve is a
no-op), a one-instance ensemble, and an empty time domain (t0 == t1): the
reference's loop takes one accepted step of size 0 (below the minimum step:
accepted with the minimum-step warning, which the oracle reports too) and
stops, leaving the state unchanged, in every mode."""
import numpy as np
import pytest

from mpgos_gb300 import capi, coupled_workloads as CW, workloads as W
from mpgos_gb300.capi import CbOption, CbVariable
from mpgos_gb300.solver import Option, Variable
from oracle import oracle as O

pytestmark = pytest.mark.gpu

MODES = [capi.MODE_PLAIN, capi.MODE_CHOSEN, capi.MODE_DF_STAGE | capi.MODE_PERSISTENT]


@pytest.mark.parametrize("mode", MODES)
def test_no_active_instance_is_a_no_op(mode, native_libs):
    case = W.lorenz_case(nt=256)
    with W.load_solver(case, mode=mode) as s:
        before = W.read_results(s)
        s.SolverOption(Option.ActiveNumberOfThreads, 0)
        s.Solve()
        after = W.read_results(s)
    for k in ("x", "t", "acci", "td"):
        np.testing.assert_array_equal(before[k], after[k])


def test_no_active_system_is_a_no_op(native_libs):
    case = CW.ring_case("ring16_full", ns=32, periods=1)
    with CW.load_coupled_solver(case, mode=capi.MODE_PERSISTENT) as s:
        before = CW.read_coupled_results(s)
        s.SolverOption(CbOption.ActiveSystems, 0)
        s.Solve()
        after = CW.read_coupled_results(s)
    for k in ("x", "t", "iuacc", "isacc"):
        np.testing.assert_array_equal(before[k], after[k])


@pytest.mark.parametrize("mode", MODES)
def test_single_instance_ensemble(mode, native_libs, oracle_libs):
    case = W.lorenz_case(nt=1, rho=(10.0, 10.0))
    res = W.run_gpu(case, mode=mode, block=32)
    ref = O.run_oracle(case)
    assert res["status"][0] == 0 and res["t"][0] == 10.0
    assert np.max(np.abs(res["x"] - ref["x"]) / np.abs(ref["x"])) < 1e-9
    assert abs(int(res["nacc"][0]) - int(ref["nacc"][0])) <= 1


@pytest.mark.parametrize("mode", MODES)
def test_empty_time_domain(mode, native_libs, oracle_libs):
    case = W.lorenz_case(nt=64)
    case.arrays["td"][1] = case.arrays["td"][0]
    res = W.run_gpu(case, mode=mode)
    ref = O.run_oracle(case)
    np.testing.assert_array_equal(res["x"], case.arrays["x"])
    np.testing.assert_array_equal(res["t"], case.arrays["td"][0])
    np.testing.assert_array_equal(res["nacc"], ref["nacc"])
    np.testing.assert_array_equal(res["status"], ref["status"])
    assert np.all(res["status"] == capi.INSTANCE_MINIMUM_STEP)


@pytest.mark.parametrize("mode", [0, capi.MODE_PERSISTENT, capi.MODE_DF_STAGE | capi.MODE_PERSISTENT])
def test_coupled_single_system_and_empty_time_domain(mode, native_libs, oracle_libs):
    """One coupled system (a warp integrates it alone) against the oracle, and
    an empty time domain leaving every unit unchanged."""
    case = CW.ring_case("ring16_full", ns=1, periods=1, seed=3)
    res = CW.run_coupled_gpu(case, mode=mode, warps=1)
    ref = O.run_oracle_coupled(case)
    scale = np.max(np.abs(case.arrays["x"]), axis=1, keepdims=True)
    assert np.all(np.abs(res["x"] - ref["x"]) <= 1e-9 * (np.abs(ref["x"]) + scale))
    np.testing.assert_array_equal(res["iuacc"], ref["iuacc"])
    empty = CW.ring_case("ring16_full", ns=8, periods=1, seed=4)
    empty.arrays["td"][1] = empty.arrays["td"][0]
    res = CW.run_coupled_gpu(empty, mode=mode, warps=2)
    np.testing.assert_array_equal(res["x"], empty.arrays["x"])
    np.testing.assert_array_equal(res["t"], empty.arrays["td"][0])


def test_df_stage_leaves_untouched_inputs_bit_exact(native_libs):
    """DF_STAGE holds values as double-floats (48 of 53 bits); data a run does
    not change (the 21 Keller-Miksis coefficients here) is written back with
    its original FP64 bits, not as a rounded round trip."""
    case = W.keller_miksis_case(n_amp=4, n_freq=8, periods=1)
    res = W.run_gpu(case, mode=capi.MODE_DF_STAGE | capi.MODE_PERSISTENT)
    np.testing.assert_array_equal(res["cp"], case.arrays["cp"])
    assert np.all(res["t"] == case.arrays["td"][1])
