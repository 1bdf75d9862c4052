"""GPU tests of the discrete adjoint (forced Duffing with per-instance k, B).

For the terminal loss L_i = |x_i(T) - target_i|^2 (one loss per instance):
  * against FP64 central finite differences of the same discrete map: the
    oracle replays the recorded step sequence with perturbed inputs, so the
    differences carry no step-selection noise; bar 1e-6 relative;
  * against the forward-sensitivity equations (duffing_param_sens.cuh)
    integrated as an augmented system at rtol = atol = 1e-12: the adjoint
    differentiates the 1e-9 discretisation and the sensitivities the exact
    flow, so they agree to the integration tolerance;
  * the PLAIN and persistent mappings and any checkpoint spacing give the
    same gradient up to rounding;
  * through the torch.autograd harness;
  * a tape too short for the step count is reported, not silently used.
"""
import numpy as np
import pytest

from mpgos_gb300 import capi, workloads as W
from mpgos_gb300.solver import Variable
from oracle import oracle as O, ref_gpu as R

pytestmark = pytest.mark.gpu

MAX_STEPS = 4096


def forward_adjoint(case, target, mode=0, segment=32, want_tape=False):
    """Recorded forward pass + adjoint through the C-ABI. Returns x(T),
    dL/dx0 [2][NT], dL/dcp [2][NT] and, optionally, the step tape."""
    import torch
    from mpgos_gb300.autograd import AdjointRunner
    runner = AdjointRunner(case, mode=mode, max_steps=MAX_STEPS, segment=segment)
    x0 = torch.tensor(case.arrays["x"], dtype=torch.float64, device="cuda")
    cp = torch.tensor(case.arrays["cp"], dtype=torch.float64, device="cuda")
    xT = runner.forward(x0, cp)
    tape = None
    if want_tape:
        t = runner.solver.tape_info()
        n = R.device_to_host(t.n_steps, (case.nt,), np.int32)
        dt = R.device_to_host(t.dt, (t.max_steps, case.nt), np.float64)
        tape = (dt, n)
    gx0, gcp = runner.backward(2.0 * (xT - torch.tensor(target, device="cuda")))
    runner.close()
    return xT.cpu().numpy(), gx0.cpu().numpy(), gcp.cpu().numpy(), tape


def rel_err(a, b):
    scale = np.max(np.abs(b), axis=0)
    return np.max(np.abs(a - b), axis=0) / scale


@pytest.fixture(scope="module")
def duffing_case():
    return W.duffing_param_case(nt=512, periods=4, tol=1e-9, seed=11), W.duffing_param_targets(512, seed=11)


def test_adjoint_matches_central_differences_of_the_discrete_map(duffing_case, native_libs, oracle_libs):
    case, target = duffing_case
    xT, gx0, gcp, (dt, n) = forward_adjoint(case, target, want_tape=True)
    assert np.all(n > 0) and np.all(n <= MAX_STEPS)
    # the replayed map reproduces the GPU forward pass
    base = O.replay(case, dt, n)
    assert np.max(np.abs(base - xT) / (np.abs(xT) + 1e-3)) < 1e-12
    grad = np.concatenate([gx0, gcp], axis=0)
    fd = np.zeros_like(grad)
    for j in range(4):
        x0, cp = case.arrays["x"].copy(), case.arrays["cp"].copy()
        arr = x0 if j < 2 else cp
        row = j % 2
        h = 1e-6 * np.maximum(np.abs(arr[row]), 1.0)
        lp, lm = [], []
        for sgn, out in ((+1, lp), (-1, lm)):
            x0s, cps = x0.copy(), cp.copy()
            (x0s if j < 2 else cps)[row] += sgn * h
            xe = O.replay(case, dt, n, x0=x0s, cp=cps)
            out.append(np.sum((xe - target) ** 2, axis=0))
        fd[j] = (lp[0] - lm[0]) / (2.0 * h)
    rel = rel_err(grad, fd)
    assert np.max(rel) < 1e-6, np.max(rel)


DF_PERSISTENT = capi.MODE_DF_STAGE | capi.MODE_PERSISTENT


def test_df_adjoint_matches_central_differences_of_the_discrete_map(duffing_case, native_libs, oracle_libs):
    """DF_STAGE records its double-float step sequence and differentiates in
    double-float: same 1e-6 bar against FP64 central differences of the
    replayed map."""
    case, target = duffing_case
    xT, gx0, gcp, (dt, n) = forward_adjoint(case, target, mode=DF_PERSISTENT, want_tape=True)
    assert np.all(n > 0) and np.all(n <= MAX_STEPS)
    # the FP64 replay of the double-float forward pass: same map, ~48-bit stages
    base = O.replay(case, dt, n)
    assert np.max(np.abs(base - xT) / (np.abs(xT) + 1e-3)) < 1e-9
    grad = np.concatenate([gx0, gcp], axis=0)
    fd = np.zeros_like(grad)
    for j in range(4):
        x0, cp = case.arrays["x"].copy(), case.arrays["cp"].copy()
        arr = x0 if j < 2 else cp
        row = j % 2
        h = 1e-6 * np.maximum(np.abs(arr[row]), 1.0)
        out = []
        for sgn in (+1, -1):
            x0s, cps = x0.copy(), cp.copy()
            (x0s if j < 2 else cps)[row] += sgn * h
            out.append(np.sum((O.replay(case, dt, n, x0=x0s, cp=cps) - target) ** 2, axis=0))
        fd[j] = (out[0] - out[1]) / (2.0 * h)
    rel = rel_err(grad, fd)
    assert np.max(rel) < 1e-6, np.max(rel)


@pytest.mark.parametrize("record_mode", [DF_PERSISTENT, capi.MODE_CHOSEN])
def test_df_and_fp64_reverse_passes_agree_on_one_tape(record_mode, duffing_case, native_libs):
    """One recorded tape (double-float or FP64 forward), reversed once in
    double-float and once in FP64 (KERNEL_MODE switched between the calls):
    the two gradients differ only by the double-float rounding of the
    reverse pass."""
    import torch
    from mpgos_gb300.autograd import AdjointRunner
    case, target = duffing_case
    runner = AdjointRunner(case, mode=record_mode, max_steps=MAX_STEPS)
    x0 = torch.tensor(case.arrays["x"], dtype=torch.float64, device="cuda")
    cp = torch.tensor(case.arrays["cp"], dtype=torch.float64, device="cuda")
    xT = runner.forward(x0, cp)
    g = 2.0 * (xT - torch.tensor(target, device="cuda"))
    runner.solver.set_mode(DF_PERSISTENT)
    gx_df, gc_df = runner.backward(g)
    runner.solver.set_mode(capi.MODE_PERSISTENT)
    gx_64, gc_64 = runner.backward(g)
    runner.close()
    a = np.concatenate([gx_df.cpu().numpy(), gc_df.cpu().numpy()])
    b = np.concatenate([gx_64.cpu().numpy(), gc_64.cpu().numpy()])
    assert not np.array_equal(a, b)       # two different reverse kernels ran
    assert np.max(rel_err(a, b)) < 1e-9, np.max(rel_err(a, b))


def test_adjoint_matches_forward_sensitivities(duffing_case, native_libs, oracle_libs):
    case, target = duffing_case
    xT, gx0, gcp, _ = forward_adjoint(case, target)
    sens = O.run_oracle(W.duffing_param_sens_case(case, tol=1e-12))
    S = sens["x"][2:].reshape(4, 2, case.nt)          # S[j, r, i] = d x_r(T) / d theta_j
    lam = 2.0 * (xT - target)
    grad_sens = np.einsum("jri,ri->ji", S, lam)        # theta = (x0, v0, k, B)
    rel = rel_err(np.concatenate([gx0, gcp], axis=0), grad_sens)
    assert np.median(rel) < 1e-6, np.median(rel)
    assert np.max(rel) < 1e-4, np.max(rel)


def test_adjoint_converges_to_forward_sensitivities(duffing_case, native_libs, oracle_libs):
    """The comparison above with the recorded forward pass at rtol = atol =
    1e-12 instead of 1e-9: the discrete gradient of the finer discretisation
    and the sensitivities of the exact flow then differ by the integration
    errors of both, and every gradient component of every instance is within
    1e-6 relative of the forward sensitivities (the bar of the adjoint
    against finite differences)."""
    case, target = duffing_case
    fine = case.copy()
    fine.rtol = np.full_like(case.rtol, 1e-12)
    fine.atol = np.full_like(case.atol, 1e-12)
    xT, gx0, gcp, _ = forward_adjoint(fine, target)
    sens = O.run_oracle(W.duffing_param_sens_case(fine, tol=1e-12))
    S = sens["x"][2:].reshape(4, 2, case.nt)
    lam = 2.0 * (xT - target)
    grad_sens = np.einsum("jri,ri->ji", S, lam)
    rel = rel_err(np.concatenate([gx0, gcp], axis=0), grad_sens)
    assert np.max(rel) < 1e-6, np.max(rel)


def test_adjoint_mapping_and_segments_agree(duffing_case, native_libs):
    case, target = duffing_case
    _, a0, c0, _ = forward_adjoint(case, target, mode=0, segment=32)
    _, a1, c1, _ = forward_adjoint(case, target, mode=2, segment=7)
    # the forward passes are bit-identical; the reverse pass re-advances the
    # state within a segment in tableau form, so checkpoint spacing changes
    # the gradient only by rounding
    # FAST_CONTROL takes a slightly different step sequence: same gradient to
    # the integration tolerance
    _, a2, c2, _ = forward_adjoint(case, target, mode=3, segment=64)
    assert np.max(rel_err(np.concatenate([a1, c1]), np.concatenate([a0, c0]))) < 1e-10
    assert np.max(rel_err(np.concatenate([a2, c2]), np.concatenate([a0, c0]))) < 1e-5


def test_autograd_harness(duffing_case, native_libs):
    import torch
    from mpgos_gb300.autograd import AdjointRunner, terminal_state
    case, target = duffing_case
    runner = AdjointRunner(case, mode=3, max_steps=MAX_STEPS)
    x0 = torch.tensor(case.arrays["x"], dtype=torch.float64, device="cuda", requires_grad=True)
    cp = torch.tensor(case.arrays["cp"], dtype=torch.float64, device="cuda", requires_grad=True)
    xT = terminal_state(x0, cp, runner)
    ((xT - torch.tensor(target, device="cuda")) ** 2).sum().backward()
    runner.close()
    _, gx0, gcp, _ = forward_adjoint(case, target, mode=3)
    np.testing.assert_array_equal(x0.grad.cpu().numpy(), gx0)
    np.testing.assert_array_equal(cp.grad.cpu().numpy(), gcp)


def test_tape_overflow_is_reported(native_libs):
    import torch
    from mpgos_gb300.autograd import AdjointRunner
    case = W.duffing_param_case(nt=64, periods=4, seed=2)
    runner = AdjointRunner(case, mode=0, max_steps=16)
    xT = runner.forward(torch.tensor(case.arrays["x"], device="cuda"), torch.tensor(case.arrays["cp"], device="cuda"))
    with pytest.raises(RuntimeError, match="tape"):
        runner.backward(torch.ones_like(xT))
    runner.close()


@pytest.mark.parametrize("mode", [capi.MODE_PLAIN, DF_PERSISTENT], ids=["fp64", "df"])
def test_rk4_adjoint_matches_central_differences(mode, native_libs, oracle_libs):
    """Fixed-step RK4 (Lorenz, rho per instance, dt = 1e-3 over t in [0, 1]):
    gradient of |x(T)|^2 with respect to x0 and rho, FP64 and double-float
    reverse passes, against FP64 central differences of the replayed map
    (bar 1e-6)."""
    import torch
    from mpgos_gb300.autograd import AdjointRunner
    case = W.lorenz_case(nt=256, t_end=1.0, rho=(0.0, 13.9))
    case.algorithm = 0
    case.options["initial_dt"] = 1e-3
    runner = AdjointRunner(case, mode=mode, max_steps=1100, segment=16)
    x0 = torch.tensor(case.arrays["x"], dtype=torch.float64, device="cuda")
    cp = torch.tensor(case.arrays["cp"], dtype=torch.float64, device="cuda")
    xT = runner.forward(x0, cp)
    t = runner.solver.tape_info()
    n = R.device_to_host(t.n_steps, (case.nt,), np.int32)
    dt = R.device_to_host(t.dt, (t.max_steps, case.nt), np.float64)
    assert np.all((n >= 1000) & (n <= 1001))
    gx0, gcp = runner.backward(2.0 * xT)
    runner.close()
    grad = np.concatenate([gx0.cpu().numpy(), gcp.cpu().numpy()])
    fd = np.zeros_like(grad)
    for j in range(4):
        arr, row = (case.arrays["x"], j) if j < 3 else (case.arrays["cp"], 0)
        h = 1e-6 * np.maximum(np.abs(arr[row]), 1.0)
        out = []
        for sgn in (+1, -1):
            xa, ca = case.arrays["x"].copy(), case.arrays["cp"].copy()
            (xa if j < 3 else ca)[row] += sgn * h
            out.append(np.sum(O.replay(case, dt, n, x0=xa, cp=ca) ** 2, axis=0))
        fd[j] = (out[0] - out[1]) / (2.0 * h)
    rel = rel_err(grad, fd)
    assert np.max(rel) < 1e-6, np.max(rel)
