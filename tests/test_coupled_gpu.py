"""GPU parity tests of the coupled per-block solver (one warp per system).

* Against the reference's own coupled kernel (MultipleSystems_SingleBlockLaunch
  built for sm_103a, oracle/_ref cubins, launched on the same device buffers):
  every output bit-identical, for the four coupling storages, RK4 and RKCK45,
  dense output, and the 16384 x 64-unit ring at full ensemble size.
* The mapping (warps per CTA, persistent work queue, coupling matrix in shared
  or global memory) changes nothing: bit-identical.
* Against the CPU oracle: end states within 1e-9 of the component's scale or
  within 1e3 x the oracle's own spread under tiny perturbations; crossing
  counts and step counts equal on the systems the perturbations leave
  unchanged (see test_coupled_matches_oracle for the allowance).
"""
import numpy as np
import pytest

from tests.parity import assert_bitwise, scaled_close
from mpgos_gb300 import capi, coupled_workloads as CW
from mpgos_gb300.capi import CbVariable as V
from oracle import oracle as O, ref_gpu as R

pytestmark = pytest.mark.gpu

KEYS = ["td", "t", "x", "iuacc", "isacc", "didx"]


def _ref(case, tpb, spb):
    if not R.coupled_available(case.system, case.algorithm, case.ns, tpb, spb, case.ndo):
        pytest.skip("reference coupled cubin not built (oracle/build_oracle.REF_GPU_CB_KERNELS)")
    return R.run_ref_gpu_coupled(case, tpb, spb)


REF_CASES = [
    ("ring16_full", dict(), 64, 4),
    ("ring16_band", dict(), 64, 4),
    ("ring16_circband", dict(), 64, 4),
    ("ring16_circ", dict(), 64, 4),
    ("ring16_full", dict(algorithm=0), 64, 4),
    ("ring16_full", dict(ndo=8), 64, 4),
    ("ring64", dict(), 128, 2),
]


@pytest.mark.parametrize("system,kw,tpb,spb", REF_CASES,
                         ids=["full", "band", "circband", "circ", "full_rk4", "full_dense", "ring64"])
def test_coupled_is_bitwise_identical_to_reference_kernel(system, kw, tpb, spb, native_libs):
    ns = 512 if system == "ring64" else 256
    case = CW.ring_case(system, ns=ns, periods=2, seed=11, **kw)
    if case.ndo:
        case.options["dense_min_dt"] = 0.5
    ref = _ref(case, tpb, spb)
    res = CW.run_coupled_gpu(case, mode=0, warps=4)
    assert np.all(res["status"] == 0)
    assert_bitwise(res, ref, keys=KEYS + (["dtime", "dstate"] if case.ndo else []))
    # the persistent work queue integrates the same systems in another order
    assert_bitwise(CW.run_coupled_gpu(case, mode=capi.MODE_PERSISTENT, warps=2), ref, keys=KEYS)


def test_mapping_does_not_change_results(native_libs):
    case = CW.ring_case("ring64", ns=96, periods=1, seed=12)
    base = CW.run_coupled_gpu(case, mode=0, warps=1)
    for warps in (2, 4, 8):
        assert_bitwise(base, CW.run_coupled_gpu(case, mode=0, warps=warps))
    assert_bitwise(base, CW.run_coupled_gpu(case, mode=capi.MODE_PERSISTENT, warps=4))
    c = case.copy()
    c.options["shared_coupling"] = 0
    c.options["shared_global"] = 0
    assert_bitwise(base, CW.run_coupled_gpu(c, mode=0, warps=4))


def test_active_systems_and_phases(native_libs):
    case = CW.ring_case("ring16_full", ns=64, periods=1, seed=13)
    case.n_active = 40
    res = CW.run_coupled_gpu(case, mode=capi.MODE_PERSISTENT, warps=4)
    assert np.all(res["t"][:40] == case.arrays["td"][1, :40])
    np.testing.assert_array_equal(res["x"][:, 40 * 16:], case.arrays["x"][:, 40 * 16:])
    # two launches of one period each == the oracle's two phases
    c2 = CW.ring_case("ring16_full", ns=64, periods=1, seed=13)
    c2.phases = 2
    two = CW.run_coupled_gpu(c2, mode=0, warps=4)
    ora = O.run_oracle_coupled(c2)
    assert scaled_close(two["x"], ora["x"], 1e-9).mean() > 0.9


def _spread(case):
    """The oracle's own sensitivity: end-state spread and the systems whose
    integer outputs stay unchanged under five tiny perturbations (initial
    states one ulp up and down, tolerances 1e-12 relative up and down, and
    multiply-adds contracted into fused multiply-adds)."""
    base = O.run_oracle_coupled(case)
    spread = np.zeros_like(base["x"])
    stable = np.ones(case.ns, bool)
    for kind, sign in (("x", np.inf), ("x", -np.inf), ("tol", 1.0), ("tol", -1.0), ("fma", 0)):
        pert = case.copy()
        if kind == "x":
            pert.arrays["x"] = np.nextafter(pert.arrays["x"], sign)
        elif kind == "tol":
            pert.rtol = pert.rtol * (1.0 + sign * 1e-12)
            pert.atol = pert.atol * (1.0 + sign * 1e-12)
        moved = O.run_oracle_coupled(pert, fma=(kind == "fma"))
        spread = np.maximum(spread, np.abs(moved["x"] - base["x"]))
        same = np.all(moved["iuacc"].reshape(-1, case.ns, case.ups) == base["iuacc"].reshape(-1, case.ns, case.ups),
                      axis=(0, 2))
        stable &= same & (moved["nacc"] == base["nacc"]) & (moved["nrej"] == base["nrej"])
    return base, spread, stable


@pytest.mark.parametrize("system", ["ring16_full", "ring16_band", "ring64"])
def test_coupled_matches_oracle(system, native_libs, oracle_libs):
    """End states: every element within the bar. Integer outputs (crossing
    counts, step counts): equal on the systems whose integers the oracle's
    own perturbations leave unchanged, with at most 2% of those allowed to
    differ: every accepted event landing must fall inside the event band,
    and a landing whose event value is a rounding error from the band edge
    takes one more refinement step under any change of rounding, which a
    finite set of perturbations samples but cannot exhaust."""
    ns, periods = {"ring64": (128, 1), "ring256": (24, 1)}.get(system, (256, 2))
    case = CW.ring_case(system, ns=ns, periods=periods, seed=14)
    ora, spread, stable = _spread(case)
    assert stable.mean() > 0.5
    res = CW.run_coupled_gpu(case, mode=capi.MODE_PERSISTENT, warps=4)
    mag = np.max(np.abs(case.arrays["x"]), axis=-1)
    ok = scaled_close(res["x"], ora["x"], 1e-9, mag, floor=1.0) | (np.abs(res["x"] - ora["x"]) <= 1e3 * spread)
    assert ok.all(), f"{int((~ok).sum())} end-state elements outside the bar"
    same = np.all(res["iuacc"].reshape(-1, case.ns, case.ups) == ora["iuacc"].reshape(-1, case.ns, case.ups),
                  axis=(0, 2))
    for k in ("nacc", "nrej", "status"):
        same &= res[k] == ora[k]
    assert (~same[stable]).sum() <= max(1, int(0.02 * stable.sum())), \
        f"{int((~same[stable]).sum())} of {int(stable.sum())} stable systems differ in integer outputs"
    np.testing.assert_array_equal(res["isacc"][0], res["nacc"])


DF_MODES = [capi.MODE_DF_STAGE, capi.MODE_SPLIT]
DF_IDS = ["df_stage", "split"]


@pytest.mark.parametrize("arith", DF_MODES, ids=DF_IDS)
@pytest.mark.parametrize("system", ["ring16_full", "ring64", "ring256"])
def test_coupled_double_float_modes_match_oracle(system, arith, native_libs, oracle_libs):
    """DF_STAGE (double-float stages, coupling dot products and sin/cos on the
    FP32 pipe) and SPLIT (the same right-hand side, coupling and stage sums;
    FP64 update, error norm, control and events): end states within 1e-9 of
    the component scale or the oracle's own perturbation spread; integer
    outputs equal on the systems the perturbations leave unchanged, with the
    step-flip allowance."""
    ns, periods = {"ring64": (128, 1), "ring256": (24, 1)}.get(system, (256, 2))
    case = CW.ring_case(system, ns=ns, periods=periods, seed=14)
    ora, spread, stable = _spread(case)
    res = CW.run_coupled_gpu(case, mode=arith | capi.MODE_PERSISTENT, warps=4)
    assert np.all(res["status"] == 0) and np.all(res["t"] == case.arrays["td"][1])
    mag = np.max(np.abs(case.arrays["x"]), axis=-1)
    ok = scaled_close(res["x"], ora["x"], 1e-9, mag, floor=1.0) | (np.abs(res["x"] - ora["x"]) <= 1e3 * spread)
    assert ok.mean() > 0.99, f"{int((~ok).sum())} end-state elements outside the bar"
    # zero crossings per unit: equal on the stable systems (step-flip allowance)
    same = np.all(res["iuacc"].reshape(-1, case.ns, case.ups) == ora["iuacc"].reshape(-1, case.ns, case.ups),
                  axis=(0, 2))
    assert (~same[stable]).sum() <= max(1, int(0.02 * stable.sum()))
    # step counts: every event landing must fall inside the +-1e-6 band, and
    # whether a secant step lands inside it or needs one more refinement turns
    # on the event value's last bits; with ~4 crossings per unit and period
    # there are hundreds of landings per system, so the counts move by a few
    # steps on many systems: bounded here by 5 % per system and 0.5 % in total
    for k in ("nacc", "nrej"):
        d = np.abs(res[k].astype(np.int64) - ora[k])
        assert np.all(d[stable] <= np.maximum(3, ora[k][stable] // 20)), k
        assert abs(int(res[k].sum()) - int(ora[k].sum())) <= max(3, int(ora[k].sum()) // 200), k
    np.testing.assert_array_equal(res["isacc"][0], res["nacc"])


@pytest.mark.parametrize("arith", DF_MODES, ids=DF_IDS)
def test_coupled_double_float_mapping_is_invariant(arith, native_libs):
    case = CW.ring_case("ring64", ns=96, periods=1, seed=12)
    base = CW.run_coupled_gpu(case, mode=arith, warps=1)
    for warps in (2, 4, 8):
        assert_bitwise(base, CW.run_coupled_gpu(case, mode=arith | capi.MODE_PERSISTENT, warps=warps))


def test_coupled_split_rk4_keeps_the_reference_time_grid(native_libs, oracle_libs):
    """SPLIT RK4: the FP64 time grid of the reference (t += dt in FP64), so
    every system takes exactly the oracle's steps; end states within 1e-11
    of the component scale (double-float stages, FP64 update)."""
    case = CW.ring_case("ring16_full", ns=128, periods=2, seed=16, algorithm=0)
    ora = O.run_oracle_coupled(case)
    res = CW.run_coupled_gpu(case, mode=capi.MODE_SPLIT | capi.MODE_PERSISTENT, warps=4)
    assert np.all(res["status"] == 0)
    np.testing.assert_array_equal(res["t"], ora["t"])
    np.testing.assert_array_equal(res["nacc"], ora["nacc"])
    mag = np.max(np.abs(case.arrays["x"]), axis=-1)
    assert scaled_close(res["x"], ora["x"], 1e-11, mag, floor=1.0).all()


def test_coupled_split_flags_values_outside_float_range(native_libs):
    """A system parameter below float's normal range (1e-40) cannot be held
    by a double-float: SPLIT flags the system MPGOS_INSTANCE_RANGE and keeps
    integrating; the other systems are unflagged."""
    case = CW.ring_case("ring16_full", ns=64, periods=1, seed=17)
    case.arrays["sp"][0, 5] = 1e-40
    res = CW.run_coupled_gpu(case, mode=capi.MODE_SPLIT, warps=4)
    flagged = (res["status"] & capi.INSTANCE_RANGE) != 0
    assert flagged[5] and flagged.sum() == 1
    assert np.all(res["t"] == case.arrays["td"][1])


@pytest.mark.parametrize("tpb,spb,alg", [(64, 1, 1), (32, 1, 1), (64, 2, 1), (32, 1, 0)],
                         ids=["SingleSystem_SingleBlockLaunch", "SingleSystem_MultipleBlockLaunches",
                              "MultipleSystems_MultipleBlockLaunches", "SingleSystem_MultipleBlockLaunches_rk4"])
def test_coupled_matches_every_reference_kernel_variant(tpb, spb, alg, native_libs):
    """The reference picks one of four coupled kernels from SPB, UPS and TPB
    (one system or several per block; the block's logical threads in one or
    several passes). One warp per system here covers every shape: the GB300
    FP64 kernel is bit-identical to each variant on 512 rings of 64 units."""
    case = CW.ring_case("ring64", ns=512, periods=1, seed=12, algorithm=alg)
    ref = _ref(case, tpb, spb)
    res = CW.run_coupled_gpu(case, mode=0, warps=4)
    assert np.all(res["status"] == 0)
    assert_bitwise(res, ref, keys=KEYS)


def test_coupled_full_ensemble_matches_reference_kernel(native_libs):
    """16384 rings of 64 units with the dense coupling matrix (the coupled
    configuration at full ensemble size; two forcing periods): crossing
    counts per unit, step counts per system and end states bit-identical to
    the reference kernel."""
    case = CW.ring_case("ring64", ns=16384, periods=2, seed=5)
    ref = _ref(case, 128, 2)
    res = CW.run_coupled_gpu(case, mode=capi.MODE_PERSISTENT, warps=4)
    assert np.all(res["status"] == 0)
    assert_bitwise(res, ref, keys=KEYS)


def test_attempt_limit_is_reported(native_libs):
    case = CW.ring_case("ring16_full", ns=32, periods=2, seed=15)
    case.options["max_attempts"] = 50
    res = CW.run_coupled_gpu(case, mode=0, warps=4)
    assert np.all(res["status"] & capi.INSTANCE_ATTEMPT_LIMIT)
    assert np.all(res["nacc"] + res["nrej"] == 50)
    assert np.all(res["t"] < case.arrays["td"][1])


@pytest.mark.parametrize("tpb", [128, 256], ids=["SingleSystem_MultipleBlockLaunches", "SingleSystem_SingleBlockLaunch"])
def test_large_systems_match_reference_kernels(tpb, native_libs):
    """Rings of 256 units (eight units per lane of the integrating warp; the
    256x256 FP64 coupling matrix is read from global memory, as it does not fit
    shared memory): bit-identical to the reference's kernel for one system per
    block, with the block's 256 logical threads in two passes of 128 or one of
    256."""
    case = CW.ring_case("ring256", ns=64, periods=1, seed=13)
    ref = _ref(case, tpb, 1)
    for mode, warps in ((0, 2), (capi.MODE_PERSISTENT, 1)):
        res = CW.run_coupled_gpu(case, mode=mode, warps=warps)
        assert np.all(res["status"] == 0)
        assert_bitwise(res, ref, keys=KEYS)


@pytest.mark.parametrize("arith", DF_MODES, ids=DF_IDS)
def test_large_systems_double_float_reads_global_matrices(arith, native_libs):
    """DF_STAGE and SPLIT with a 256x256 coupling matrix (512 KB as
    double-floats, more than shared memory holds): the kernel reads the
    runtime's double-float copy from global memory; the mapping changes
    nothing (bit-identical), and a matrix changed on the host between solves
    is converted again."""
    case = CW.ring_case("ring256", ns=24, periods=1, seed=14)
    base = CW.run_coupled_gpu(case, mode=arith, warps=1)
    assert np.all(base["status"] == 0)
    assert_bitwise(base, CW.run_coupled_gpu(case, mode=arith | capi.MODE_PERSISTENT, warps=2))
    other = case.copy()
    other.arrays["cmat"] = other.arrays["cmat"] * 0.5
    fresh = CW.run_coupled_gpu(other, mode=arith, warps=1)
    with CW.load_coupled_solver(case, mode=arith, warps=1) as s:
        s.Solve()
        s.host(V.ActualTime)[:] = other.arrays["t"]
        s.host(V.ActualState)[:] = other.arrays["x"]
        s.host(V.IntegerUnitAccessories)[:] = other.arrays["iuacc"]
        s.host(V.IntegerSystemAccessories)[:] = other.arrays["isacc"]
        for i in range(s.NC):
            s.SetCouplingMatrix(i, other.arrays["cmat"][i])
        s.SynchroniseFromHostToDevice(V.All)
        s.Solve()
        again = CW.read_coupled_results(s)
    assert not np.array_equal(fresh["x"], base["x"])
    assert_bitwise(fresh, again)
