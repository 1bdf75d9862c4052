"""GPU parity tests of the per-thread solver (sm_103a kernels through the C-ABI).

Bar: against the reference's own CUDA solver built for
sm_103a, event counts and integer accessories bit-exact and FP64 end states
within 1e-9 relative. The PLAIN kernels meet it with margin: they are
bit-identical to the reference kernel (oracle/_ref cubins, launched on the
same device buffers). The CHOSEN form changes the step-size factor by ~1e-7
relative, so it is held to the 1e-9 bar on every instance that is not
chaotic (see parity.sensitive_instances). Against the CPU (oracle, golden
fixtures of the reference CPU build) see tests/parity.py for the bars.
"""
import math

import numpy as np
import pytest

from tests.conftest import golden_files
from tests.golden.make_golden import load
from tests.parity import (assert_bitwise, assert_close, assert_cpu_parity, assert_ints_equal, perturbation_spread,
                          scaled_close, sensitive_instances)
from mpgos_gb300 import capi, workloads as W
from mpgos_gb300.solver import Option, Variable
from oracle import oracle as O, ref_gpu as R

pytestmark = pytest.mark.gpu

MODES = {"plain": 0, "fast": 1, "persistent": 2, "chosen": 3, "df": 16, "df_persistent": 18, "split": 128,
         "split_persistent": 130}
# modes whose stage arithmetic is double-float (DF_STAGE, and SPLIT: double-float
# right-hand side and stage sums, FP64 state, error norm and control)
DF_STAGES = capi.MODE_DF_STAGE | capi.MODE_SPLIT


def _ref_available(case):
    return R.available(case.system, case.algorithm, case.nt, case.ndo)


def _random_cases():
    rng = np.random.default_rng(2026)
    c = W.lorenz_case(nt=1000, rho=(0.5, 24.0))
    c.arrays["x"][:] = rng.uniform(-15.0, 15.0, (3, 1000))
    c.arrays["x"][2] += 20.0
    c.options["initial_dt"] = 1e-3
    c.arrays["td"][1] = 2.0
    yield "lorenz_random_ic_1000", c
    yield "duffing_param_1000", W.duffing_param_case(nt=1000, periods=2, seed=3)
    yield "duffing_events_udt_512", W.duffing_events_case(nt=512, periods=2, ndo=16, seed=21, stop_after=5)
    yield "bouncing_ball_300", W.bouncing_ball_case(nt=300, impacts=9, seed=5)
    yield "keller_miksis_16x16", W.keller_miksis_case(n_amp=16, n_freq=16, periods=2)
    c = W.duffing_rk4_case(nt=300, periods=3)
    c.n_active = 250
    yield "duffing_rk4_partial", c


RANDOM = list(_random_cases())
GOLDEN = [(p.stem, *load(p)) for p in golden_files()]


# ---- bit-level parity with the reference kernel ----------------------------
@pytest.mark.parametrize("name,case", [(n, c) for n, c, _ in GOLDEN] + RANDOM, ids=lambda v: v if isinstance(v, str) else "")
def test_plain_is_bitwise_identical_to_reference_kernel(name, case, native_libs):
    if not _ref_available(case):
        pytest.skip("no reference cubin for this case (see oracle/build_oracle.REF_GPU_KERNELS)")
    ref = R.run_ref_gpu(case)  # one warp per block, the reference's default
    for mode in (0, 2):  # static and persistent mapping
        assert_bitwise(W.run_gpu(case, mode=mode, block=64), ref,
                       keys=["td", "x", "t", "cp", "acc", "acci", "didx"] + (["dtime", "dstate"] if case.ndo else []))


# ---- parity with the reference CPU build (golden fixtures) ------------------
def _perturbation(mode):
    """Input perturbation whose effect on the CPU reference bounds the
    legitimate GPU/CPU difference: one ulp of the initial state for the
    reference arithmetic, 1e-9 relative for FAST_CONTROL and DF_STAGE (whose
    step sizes differ by ~1e-7 relative, i.e. ~1e-11 of the local error, and
    whose double-float stages round at ~4e-15; SPLIT's as well)."""
    return 1e-9 if MODES[mode] & (capi.MODE_FAST_CONTROL | DF_STAGES) else 0.0


def _tol_perturbation(mode):
    """FAST_CONTROL and DF_STAGE round the step-size factor in FP32 (~1e-7
    relative): the same step-grid shift as moving the tolerances by ~1e-6
    relative. SPLIT forms the factor to FP64 accuracy, but its error estimate
    carries the stages' double-float rounding, ~1e-6 of it at tol 1e-10: the
    same shift."""
    return 1e-6 if MODES[mode] & (capi.MODE_FAST_CONTROL | DF_STAGES) else 0.0


def _int_slack(mode):
    """DF_STAGE's error estimate carries double-float rounding on top of the
    FP32 step factor: the estimate dt |sum_j e_j k_j| cancels down to ~tol of
    terms of size |k| dt, so its ~4e-15 |k| dt rounding is ~1e-6 of the
    estimate at tol 1e-10 (FP64: ~5e-8). Accept/reject decisions within that
    band of the threshold flip; over thousands of steps per instance a step
    count may differ by one on a few percent of the instances (see
    parity.assert_ints_equal), never by more. SPLIT's estimate carries the
    same rounding."""
    return 0.02 if MODES[mode] & DF_STAGES else 0.0


def _skip_unsupported(case, mode):
    """Every mode runs every scheme here (FAST_CONTROL and FP32_STAGE are
    no-ops for the fixed-step RK4, DF_STAGE runs its stages in double-float on
    the reference's FP64 time grid)."""


@pytest.mark.parametrize("mode", list(MODES), ids=str)
@pytest.mark.parametrize("name,case,ref", GOLDEN, ids=lambda v: v if isinstance(v, str) else "")
def test_gpu_matches_reference_golden(name, case, ref, mode, native_libs, oracle_libs):
    _skip_unsupported(case, mode)
    res = W.run_gpu(case, mode=MODES[mode], block=64)
    assert_cpu_parity(res, ref, case, key=name, rel=_perturbation(mode), tol_rel=_tol_perturbation(mode),
                      int_slack=_int_slack(mode))
    assert np.all(res["status"] & (capi.INSTANCE_NONFINITE | capi.INSTANCE_ATTEMPT_LIMIT) == 0)


# ---- parity with the oracle ----------------------------------------------
@pytest.mark.parametrize("mode", ["plain", "chosen", "df_persistent", "split_persistent"], ids=str)
@pytest.mark.parametrize("name,case", RANDOM, ids=lambda v: v if isinstance(v, str) else "")
def test_gpu_matches_oracle(name, case, mode, native_libs, oracle_libs):
    _skip_unsupported(case, mode)
    ref = O.run_oracle(case)
    res = W.run_gpu(case, mode=MODES[mode], block=96)
    assert_cpu_parity(res, ref, case, key=name, rel=_perturbation(mode), tol_rel=_tol_perturbation(mode),
                      int_slack=_int_slack(mode))
    _, stable = perturbation_spread(case, _perturbation(mode), name, _tol_perturbation(mode))
    assert_ints_equal(res, ref, ("nacc", "nrej", "status"), stable, _int_slack(mode),
                      fraction=_rejection_fraction(case, mode))


def _rejection_fraction(case, mode):
    """With events, most rejected steps are the secant refinements that land
    each event inside its tolerance band, and whether one landing takes an
    iteration more or fewer turns on the last bits of the event function
    there. Double-float stages round those values differently from FP64, so
    (Keller-Miksis, ~20 landings and 30-80 rejections per instance and two
    periods, accepted steps and event counts equal) a rejection count moves
    by a few: 5 % of it per instance, accepted steps and status at the
    default bar."""
    if MODES[mode] & DF_STAGES and W.SHAPES[case.system][4] > 0:
        return {"nrej": 0.05}
    return None


@pytest.mark.parametrize("fast", [0, 1, 16, 128])
def test_mapping_and_block_size_do_not_change_results(fast, native_libs):
    case = W.keller_miksis_case(n_amp=8, n_freq=32, periods=2)
    base = W.run_gpu(case, mode=fast, block=32)
    for block in (64, 128, 256):
        assert_bitwise(base, W.run_gpu(case, mode=fast, block=block))
    assert_bitwise(base, W.run_gpu(case, mode=fast | capi.MODE_PERSISTENT, block=128))


@pytest.mark.parametrize("mode", [0, 3, capi.MODE_SPLIT])
def test_graph_phases_equal_individual_solves(mode, native_libs):
    case = W.duffing_rk4_case(nt=1024, periods=16)
    a = W.run_gpu(case, mode=mode, graph=False)
    b = W.run_gpu(case, mode=mode, graph=True)
    assert_bitwise(a, b)
    assert np.all(b["acci"][0] == 16 * 401)


def test_graph_streams_accessory_per_phase(native_libs, oracle_libs):
    case = W.keller_miksis_case(n_amp=4, n_freq=8, periods=5)
    import torch  # device memory for the per-phase output only
    out = torch.zeros((case.phases, case.nt), dtype=torch.float64, device="cuda")
    with W.load_solver(case, mode=3) as s:
        s.SolvePhases(case.phases, stream_accessory=0, phase_output_ptr=out.data_ptr())
        res = W.read_results(s)
    per_period = out.cpu().numpy()
    np.testing.assert_array_equal(per_period[-1], res["acc"][0])
    c = case.copy()
    c.phases = 1
    for p in range(case.phases):
        r = O.run_oracle(c)
        assert scaled_close(per_period[p], r["acc"][0], 1e-9).all(), f"period {p}"
        for k in ("x", "t", "acc", "acci", "td", "didx"):
            c.arrays[k] = r[k]


# ---- the headline workload at full size -----------------------------------
def test_lorenz_full_size(native_libs, oracle_libs):
    """2^20-instance Lorenz at 1e-10. PLAIN: bit-identical to the reference
    kernel over the whole ensemble. CHOSEN: 512 instances spread over the rho
    range replayed through the oracle; non-chaotic ones within 1e-9 with equal
    step counts."""
    case = W.lorenz_case(nt=1 << 20)
    chosen = W.run_gpu(case, mode=3, block=128)
    assert np.all(chosen["t"] == 10.0) and np.all(chosen["status"] == 0)
    assert chosen["acci"][0].sum() == chosen["nacc"].sum()
    if _ref_available(case):
        plain = W.run_gpu(case, mode=0, block=64)
        assert_bitwise(plain, R.run_ref_gpu(case), keys=["x", "t", "acci"])
    idx = np.unique(np.concatenate([np.linspace(0, case.nt - 1, 448).astype(np.int64),
                                    np.random.default_rng(1).integers(0, case.nt, 64)]))
    sub = case.subset(idx)
    ref = O.run_oracle(sub)
    chaotic = sensitive_instances(sub)
    assert chaotic.sum() < 0.05 * idx.size, chaotic.sum()
    calm = ~chaotic
    got = {k: v[..., idx] for k, v in chosen.items() if np.ndim(v) and np.shape(v)[-1] == case.nt}
    assert_close(got, ref, mask=calm, keys=("x", "t"))
    np.testing.assert_array_equal(got["nacc"][calm], ref["nacc"][calm])


def test_lorenz_full_size_df_stage(native_libs, oracle_libs):
    """2^20-instance Lorenz at 1e-10 in DF_STAGE (the headline chosen form).
    512 instances replayed through the oracle: every instance whose end state
    the oracle itself keeps within 1e-10 under a 1e-13 relative perturbation
    of the initial state (not chaotic at the double-float rounding level of
    ~4e-15 per operation) is within 1e-9 of the FP64 oracle with the same
    step count."""
    case = W.lorenz_case(nt=1 << 20)
    df = W.run_gpu(case, mode=capi.MODE_DF_STAGE | capi.MODE_PERSISTENT, block=128)
    assert np.all(df["t"] == 10.0) and np.all(df["status"] == 0)
    assert df["acci"][0].sum() == df["nacc"].sum()
    idx = np.unique(np.concatenate([np.linspace(0, case.nt - 1, 448).astype(np.int64),
                                    np.random.default_rng(1).integers(0, case.nt, 64)]))
    sub = case.subset(idx)
    ref = O.run_oracle(sub)
    pert = sub.copy()
    pert.arrays["x"] = pert.arrays["x"] * (1.0 + 1e-13)
    moved = O.run_oracle(pert)
    calm = scaled_close(moved["x"], ref["x"], 1e-10).all(axis=0)
    assert calm.mean() > 0.95, calm.mean()
    got = {k: v[..., idx] for k, v in df.items() if np.ndim(v) and np.shape(v)[-1] == case.nt}
    assert_close(got, ref, mask=calm, keys=("x", "t"), ints=False)
    assert_ints_equal(got, ref, ("nacc", "acci"), calm, _int_slack("df"))


def test_lorenz_full_size_split(native_libs, oracle_libs):
    """2^20-instance Lorenz at 1e-10 in SPLIT (double-float right-hand side and
    stage sums; FP64 state update, time, error norm, step-size control): the
    headline form. 512 instances replayed through the FP64 oracle: every
    instance whose end state the oracle itself keeps within 1e-10 under a
    1e-13 relative perturbation of the initial state is within 1e-9 of it,
    step counts equal up to the bounded accept/reject flips of the stages'
    double-float rounding (_int_slack)."""
    case = W.lorenz_case(nt=1 << 20)
    sp = W.run_gpu(case, mode=capi.MODE_SPLIT | capi.MODE_PERSISTENT, block=128)
    assert np.all(sp["t"] == 10.0) and np.all(sp["status"] == 0)
    assert sp["acci"][0].sum() == sp["nacc"].sum()
    idx = np.unique(np.concatenate([np.linspace(0, case.nt - 1, 448).astype(np.int64),
                                    np.random.default_rng(1).integers(0, case.nt, 64)]))
    sub = case.subset(idx)
    ref = O.run_oracle(sub)
    pert = sub.copy()
    pert.arrays["x"] = pert.arrays["x"] * (1.0 + 1e-13)
    moved = O.run_oracle(pert)
    calm = scaled_close(moved["x"], ref["x"], 1e-10).all(axis=0)
    assert calm.mean() > 0.95, calm.mean()
    got = {k: v[..., idx] for k, v in sp.items() if np.ndim(v) and np.shape(v)[-1] == case.nt}
    assert_close(got, ref, mask=calm, keys=("x", "t"), ints=False)
    assert_ints_equal(got, ref, ("nacc", "acci"), calm, _int_slack("split"))


@pytest.mark.parametrize("mode", [capi.MODE_DF_STAGE, capi.MODE_SPLIT])
def test_double_float_modes_flag_values_outside_float_range(mode, native_libs):
    """DF_STAGE and SPLIT compute with float's exponent range: an instance
    that starts from a value outside it (a parameter of 1e40, a state
    component of 1e-40) gets MPGOS_INSTANCE_RANGE, the others do not; the FP64
    modes never set it."""
    case = W.lorenz_case(nt=64, rho=(0.0, 13.9))
    case.arrays["cp"][0, 3] = 1e40
    case.arrays["x"][1, 7] = 1e-40
    res = W.run_gpu(case, mode=mode)
    flagged = (res["status"] & capi.INSTANCE_RANGE) != 0
    assert flagged[3] and flagged[7]
    assert not flagged[np.setdiff1d(np.arange(64), [3, 7])].any()
    plain = W.run_gpu(case, mode=capi.MODE_PLAIN)
    assert not np.any(plain["status"] & capi.INSTANCE_RANGE)


@pytest.mark.parametrize("mode", [capi.MODE_DF_STAGE, capi.MODE_SPLIT])
def test_double_float_static_and_persistent_agree(mode, native_libs):
    case = W.keller_miksis_case(n_amp=8, n_freq=16, periods=2)
    a = W.run_gpu(case, mode=mode, block=64)
    b = W.run_gpu(case, mode=mode | capi.MODE_PERSISTENT, block=128)
    assert_bitwise(a, b)


def test_split_rk4_keeps_the_reference_time_grid(native_libs):
    """SPLIT with the fixed-step RK4: stages in double-float, the state update
    x + (dt/6)(k1 + 2 k2 + 2 k3 + k4) and the time in FP64 on the reference's
    grid: step counts and end times are the reference kernel's exactly (PLAIN
    is bit-identical to it), the states agree to ~1e-13."""
    case = W.duffing_rk4_case(nt=1024, periods=8)
    ref = W.run_gpu(case, mode=capi.MODE_PLAIN, graph=True)
    res = W.run_gpu(case, mode=capi.MODE_SPLIT | capi.MODE_PERSISTENT, graph=True)
    np.testing.assert_array_equal(res["acci"], ref["acci"])
    np.testing.assert_array_equal(res["t"], ref["t"])
    assert np.max(np.abs(res["x"] - ref["x"])) < 1e-11
    assert np.max(np.abs(res["acc"] - ref["acc"])) < 1e-11


def test_df_stage_static_and_persistent_agree(native_libs):
    case = W.keller_miksis_case(n_amp=8, n_freq=16, periods=2)
    a = W.run_gpu(case, mode=capi.MODE_DF_STAGE, block=64)
    b = W.run_gpu(case, mode=capi.MODE_DF_STAGE | capi.MODE_PERSISTENT, block=128)
    assert_bitwise(a, b)


def test_fp32_stage_mode_error_is_bounded(native_libs, oracle_libs):
    """FP32 stages at rtol = atol = 1e-6 on the non-chaotic Lorenz range:
    end-state error against the FP64 oracle of the same tolerance."""
    case = W.lorenz_case(nt=4096, tol=1e-6, rho=(0.0, 13.9))
    ref = O.run_oracle(case)
    res = W.run_gpu(case, mode=capi.MODE_FP32_STAGE | capi.MODE_CHOSEN, block=128)
    assert np.all(np.isfinite(res["x"])) and np.all(res["t"] == 10.0)
    assert np.quantile(scaled_rel(res["x"], ref["x"]), 0.99) < 1e-4


def test_float_precision_table(native_libs, oracle_libs):
    """Precision = float (the reference's float build) at 1e-5."""
    case = W.lorenz_case(nt=512, tol=1e-5, rho=(0.0, 13.9))
    ref = O.run_oracle(case)
    res = W.run_gpu(case, mode=0, precision="float")
    assert np.all(res["t"] == np.float32(10.0))
    assert np.quantile(scaled_rel(res["x"], ref["x"]), 0.99) < 1e-3


def scaled_rel(a, b):
    scale = np.max(np.abs(b), axis=1, keepdims=True)
    return np.max(np.abs(a - b) / (np.abs(b) + 1e-3 * scale), axis=0)


@pytest.mark.parametrize("mode", [0, 3, capi.MODE_SPLIT])
def test_status_flags_and_attempt_limit(mode, native_libs, oracle_libs):
    case = W.lorenz_case(nt=64)
    case.arrays["x"][0, 5] = np.nan
    res = W.run_gpu(case, mode=mode)
    ref = O.run_oracle(case)
    assert res["status"][5] == capi.INSTANCE_NONFINITE      # shrinks to the minimum step, then stops
    np.testing.assert_array_equal(res["status"], ref["status"])
    case.options["max_attempts"] = 10
    res = W.run_gpu(case, mode=mode)
    assert np.all(res["status"] & capi.INSTANCE_ATTEMPT_LIMIT)
    assert np.all(res["nacc"] + res["nrej"] == 10)


@pytest.mark.parametrize("mode", [capi.MODE_SPLIT, capi.MODE_DF_STAGE], ids=["split", "df_stage"])
def test_bounded_trig_reports_arguments_beyond_its_bound(mode, native_libs):
    """The Duffing plugin is built with MPGOS_DF_TRIG_BOUNDED (branch-free
    double-float cos for |t| < 2^14): one forcing period moved to start at
    2^14 gives NaN forcing in the double-float modes, and every instance stops
    with MPGOS_INSTANCE_NONFINITE instead of integrating a wrong cosine; the
    FP64 kernel integrates the same period normally, and inside the bound the
    modes agree with it."""
    case = W.duffing_rk4_case(nt=256, periods=1)
    res = W.run_gpu(case, mode=mode)
    ref = W.run_gpu(case, mode=capi.MODE_PLAIN)
    assert not np.any(res["status"]) and not np.any(ref["status"])
    assert np.max(np.abs(res["x"] - ref["x"])) < 1e-12
    far = case.copy()
    far.arrays["td"][0] = 2.0 ** 14
    far.arrays["td"][1] = 2.0 ** 14 + 2.0 * math.pi
    res = W.run_gpu(far, mode=mode)
    assert np.all(res["status"] & capi.INSTANCE_NONFINITE)
    ref = W.run_gpu(far, mode=capi.MODE_PLAIN)
    assert not np.any(ref["status"])


def test_two_solver_objects_alternate(native_libs):
    """Two objects on one device, interleaved as T7_DoubleBuffering does."""
    c1 = W.duffing_rk4_case(nt=512, periods=4)
    c2 = W.duffing_rk4_case(nt=512, periods=4, B=0.35)
    with W.load_solver(c1, mode=0) as s1, W.load_solver(c2, mode=2) as s2:
        for _ in range(4):
            s1.Solve()
            s1.InsertSynchronisationPoint()
            s2.Solve()
            s2.InsertSynchronisationPoint()
            s1.SynchroniseSolver()
            s2.SynchroniseSolver()
        r1, r2 = W.read_results(s1), W.read_results(s2)
    assert_bitwise(r1, W.run_gpu(c1, mode=0))
    assert_bitwise(r2, W.run_gpu(c2, mode=0))


def test_checkpoint_restore_replays_bitwise(native_libs):
    case = W.duffing_param_case(nt=2048, periods=2)
    with W.load_solver(case, mode=3) as s:
        s.checkpoint_save()
        s.Solve()
        a = W.read_results(s)
        s.checkpoint_restore()
        s.Solve()
        b = W.read_results(s)
    assert_bitwise(a, b)


def test_autotune_keeps_state(native_libs, tmp_path):
    case = W.keller_miksis_case(n_amp=8, n_freq=16, periods=1)
    base = W.run_gpu(case, mode=1)
    cache = tmp_path / "tune.jsonl"
    with W.load_solver(case, mode=1) as s:
        grid, block, mode = s.autotune(fast_control=True, cache_path=str(cache))
        assert block in (32, 64, 96, 128, 192, 256) and mode & capi.MODE_FAST_CONTROL
        s.Solve()
        res = W.read_results(s)
    assert_bitwise(base, res)
    assert cache.read_text().count("keller_miksis") == 1
    with W.load_solver(case, mode=1) as s:
        assert s.autotune(True, str(cache))[1:] == (block, mode)


def test_host_api_bounds_and_scalar_access(native_libs):
    from mpgos_gb300 import ProblemSolver, MpgosError
    from mpgos_gb300.solver import (ActualState, ControlParameters, DenseIndex, DenseState, RelativeTolerance,
                                    SharedParameters, TimeDomain)
    with ProblemSolver("duffing_events", 8, ndo=4) as s:
        s.SetHost(3, ActualState, 1, 0.25)
        assert s.GetHost(3, ActualState, 1) == 0.25
        s.SetHost(SharedParameters, 0, 0.3)
        assert s.GetHost(SharedParameters, 0) == 0.3
        s.SetHost(2, DenseState, 1, 3, 7.0)
        assert s.host(DenseState)[3, 1, 2] == 7.0
        with pytest.raises(MpgosError):
            s.SetHost(8, ActualState, 0, 1.0)
        with pytest.raises(MpgosError):
            s.SetHost(0, ControlParameters, 1, 1.0)
        with pytest.raises(MpgosError):
            s.SetHost(0, DenseIndex, 4)
        with pytest.raises(MpgosError):
            s.SolverOption(RelativeTolerance, 2, 1e-9)
        with pytest.raises(MpgosError):
            s.SolverOption(RelativeTolerance, 0, -1.0)
        with pytest.raises(MpgosError):
            s.SolverOption(Option.ThreadsPerBlock, 1024)
        s.SetHost(0, TimeDomain, 1, math.pi)
        assert s.host(Variable.TimeDomain)[1, 0] == math.pi


@pytest.mark.parametrize("ipt", [2, 3])
def test_instances_per_thread_is_a_mapping_only(ipt, native_libs):
    """InstancesPerThread > 1 shrinks the static grid; each lane integrates
    its instances in turn (grid stride). Results are bit-identical to one
    instance per lane, for the reference arithmetic and for DF_STAGE."""
    from mpgos_gb300.capi import Option
    case = W.keller_miksis_case(n_amp=8, n_freq=16, periods=2)
    for mode in (capi.MODE_PLAIN, capi.MODE_DF_STAGE, capi.MODE_SPLIT):
        a = W.run_gpu(case, mode=mode, block=32)
        with W.load_solver(case, mode=mode, block=32) as s:
            s.SolverOption(Option.InstancesPerThread, ipt)
            grid, block, _ = s.launch_config()
            assert grid == -(-case.nt // (32 * ipt))
            for _ in range(case.phases):
                s.Solve()
            b = W.read_results(s)
        assert_bitwise(a, b)


def test_autotuner_explores_mapping_and_placement(native_libs, tmp_path):
    from mpgos_gb300.capi import Option
    case = W.duffing_rk4_case(nt=4096, periods=2)
    cache = tmp_path / "tune.json"
    with W.load_solver(case, mode=0) as s:
        s.autotune(fast_control=False, cache_path=str(cache))
        n = int(s.GetOption(Option.InstancesPerThread))
        ps = int(s.GetOption(Option.PreferSharedMemory))
        assert n in (1, 2, 4) and ps in (0, 1)
        ref = W.read_results(s)
    line = cache.read_text()
    assert '"instances_per_thread"' in line and '"prefer_shared"' in line
    with W.load_solver(case, mode=0) as s:   # cached choice restored
        s.autotune(fast_control=False, cache_path=str(cache))
        assert int(s.GetOption(Option.InstancesPerThread)) == n
        assert int(s.GetOption(Option.PreferSharedMemory)) == ps
    # the tuned launch integrates the same ensemble bit for bit
    res = W.run_gpu(case, mode=0)
    with W.load_solver(case, mode=0) as s:
        s.SolverOption(Option.InstancesPerThread, n)
        s.SolverOption(Option.PreferSharedMemory, ps)
        for _ in range(case.phases):
            s.Solve()
        tuned = W.read_results(s)
    assert_bitwise(res, tuned)


def test_autotuner_double_float_tries_outlined_right_hand_side(native_libs, tmp_path):
    """For double-float kernels the autotuner also times the out-of-line
    right-hand side; its choice is cached and restored, and the tuned launch
    integrates the ensemble exactly as the inlined default does."""
    from mpgos_gb300.capi import Option
    case = W.keller_miksis_case(n_amp=16, n_freq=16, periods=2)
    cache = tmp_path / "tune_df.json"
    with W.load_solver(case, mode=capi.MODE_DF_STAGE) as s:
        s.autotune(arithmetic=capi.MODE_DF_STAGE, cache_path=str(cache))
        ol = int(s.GetOption(Option.OutlineRhs))
        assert ol in (0, 1)
        _, _, m = s.launch_config()
        assert m & capi.MODE_DF_STAGE and bool(m & 64) == bool(ol)
    assert '"outline_rhs"' in cache.read_text()
    with W.load_solver(case, mode=capi.MODE_DF_STAGE) as s:
        s.autotune(arithmetic=capi.MODE_DF_STAGE, cache_path=str(cache))
        assert int(s.GetOption(Option.OutlineRhs)) == ol
        for _ in range(case.phases):
            s.Solve()
        tuned = W.read_results(s)
    assert_bitwise(W.run_gpu(case, mode=capi.MODE_DF_STAGE), tuned)


def test_warp_reconvergence_is_scheduling_only(native_libs):
    """The per-attempt warp ballot only changes how lanes are scheduled:
    results are bit-identical with it on and off (events make lanes diverge
    on this system, so both code paths run divergent warps)."""
    from mpgos_gb300.capi import Option
    case = W.keller_miksis_case(n_amp=8, n_freq=16, periods=2)
    for mode in (capi.MODE_PLAIN, capi.MODE_CHOSEN, capi.MODE_DF_STAGE | capi.MODE_PERSISTENT,
                 capi.MODE_SPLIT | capi.MODE_PERSISTENT):
        out = []
        for rv in (0, 1):
            with W.load_solver(case, mode=mode, block=64) as s:
                s.SolverOption(Option.WarpReconverge, rv)
                assert int(s.GetOption(Option.WarpReconverge)) == rv
                for _ in range(case.phases):
                    s.Solve()
                out.append(W.read_results(s))
        assert_bitwise(out[0], out[1])


@pytest.mark.parametrize("graph", [False, True], ids=["solves", "graph"])
def test_work_order_is_scheduling_only(graph, native_libs):
    """WorkOrder (every launch takes the instances longest first by the
    previous launch's step attempts, sorted on the device) changes only which
    lane integrates which instance and when: over three periods, as separate
    solves and as one graph of phases (the second and third launches run in
    the sorted order), every output of every instance is bit-identical to
    index order, in FP64, SPLIT and DF_STAGE, static and persistent. Values
    other than 0 and 1 are refused."""
    from mpgos_gb300.capi import MpgosError, Option
    case = W.keller_miksis_case(n_amp=24, n_freq=40, periods=3)
    for mode in (capi.MODE_PLAIN, capi.MODE_CHOSEN, capi.MODE_SPLIT, capi.MODE_SPLIT | capi.MODE_PERSISTENT,
                 capi.MODE_DF_STAGE | capi.MODE_PERSISTENT):
        out = []
        for order in (0, 1):
            with W.load_solver(case, mode=mode, block=64) as s:
                s.SolverOption(Option.WorkOrder, order)
                assert int(s.GetOption(Option.WorkOrder)) == order
                if graph:
                    s.SolvePhases(case.phases)
                else:
                    for _ in range(case.phases):
                        s.Solve()
                out.append(W.read_results(s))
        assert_bitwise(out[0], out[1])
        n = np.asarray(out[0]["nacc"]) + np.asarray(out[0]["nrej"])
        assert n.max() > 2 * n.min()   # uneven: the order is not the identity
    with W.load_solver(case, mode=capi.MODE_PLAIN) as s:
        with pytest.raises(MpgosError):
            s.SolverOption(Option.WorkOrder, 2)


@pytest.mark.parametrize("system", ["keller_miksis", "lorenz", "duffing_rk4"])
def test_outlined_right_hand_side_is_code_layout_only(system, native_libs):
    """OutlineRhs (double-float kernels: the right-hand side as one
    out-of-line function) changes only where the code sits: results are
    bit-identical to the inlined kernels, static and persistent, with and
    without the warp reconvergence ballot, RKCK45 and RK4."""
    from mpgos_gb300.capi import Option
    case = {"keller_miksis": lambda: W.keller_miksis_case(n_amp=8, n_freq=16, periods=2),
            "lorenz": lambda: W.lorenz_case(nt=512),
            "duffing_rk4": lambda: W.duffing_rk4_case(nt=256, periods=4)}[system]()
    for mode in (capi.MODE_DF_STAGE, capi.MODE_DF_STAGE | capi.MODE_PERSISTENT, capi.MODE_SPLIT,
                 capi.MODE_SPLIT | capi.MODE_PERSISTENT):
        for rv in (0, 1):
            out = []
            for ol in (0, 1):
                with W.load_solver(case, mode=mode, block=64) as s:
                    s.SolverOption(Option.WarpReconverge, rv)
                    s.SolverOption(Option.OutlineRhs, ol)
                    assert int(s.GetOption(Option.OutlineRhs)) == ol
                    _, _, m = s.launch_config()
                    assert bool(m & 64) == bool(ol)
                    for _ in range(case.phases):
                        s.Solve()
                    out.append(W.read_results(s))
            assert_bitwise(out[0], out[1])


def test_config1_duffing_rk4_full_size(native_libs):
    """The plain small configuration at full size: forced Duffing, 8192
    instances, fixed-step RK4 with dt = 2 pi / 400 over 1024 forcing periods
    (1024 phases replayed from one CUDA graph), running maximum of x as an
    accessory. PLAIN (and the persistent mapping) are bit-identical to the
    reference's kernel launched once per period; every instance takes
    1024 x 401 steps (400 plus the clamped end step of each period)."""
    case = W.duffing_rk4_case(nt=8192, periods=1024)
    if not R.available(case.system, case.algorithm, case.nt, case.ndo):
        pytest.skip("reference cubin for Duffing RK4 at 8192 instances not built")
    ref = R.run_ref_gpu(case)
    for mode in (capi.MODE_PLAIN, capi.MODE_PERSISTENT):
        res = W.run_gpu(case, mode=mode, graph=True)
        assert_bitwise(res, ref, keys=["x", "t", "acc", "acci"])
    assert np.all(res["acci"][0] == 1024 * 401)


def test_df_stage_rk4_keeps_the_reference_time_grid(native_libs):
    """DF_STAGE with the fixed-step RK4: stages in double-float, time on the
    FP64 grid of the reference, so the step counts (the 400 steps and the
    clamped end step of every period) and the end times are those of the
    reference kernel exactly and the states agree to ~1e-13."""
    case = W.duffing_rk4_case(nt=1024, periods=8)
    ref = W.run_gpu(case, mode=capi.MODE_PLAIN, graph=True)
    res = W.run_gpu(case, mode=capi.MODE_DF_STAGE | capi.MODE_PERSISTENT, graph=True)
    np.testing.assert_array_equal(res["acci"], ref["acci"])
    np.testing.assert_array_equal(res["t"], ref["t"])
    assert np.max(np.abs(res["x"] - ref["x"])) < 1e-11
    assert np.max(np.abs(res["acc"] - ref["acc"])) < 1e-11
