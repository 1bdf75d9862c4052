"""GPU dense-output interpolation (mpgos_pt_dense_interpolate) against the CPU
statement of the same interpolant (oracle.dense_interpolate) on the GPU's own
dense output: the only differences are the right-hand side evaluations (CUDA
vs host cos), so the bar is 1e-13 relative to the state's scale."""
import numpy as np
import pytest

from mpgos_gb300 import capi, workloads as W
from mpgos_gb300.solver import Variable
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def gpu_dense(case, times, mode=0):
    import torch
    with W.load_solver(case, mode=mode) as s:
        s.Solve()
        t = torch.tensor(times, dtype=torch.float64, device="cuda")
        out = torch.full((len(times), s.SD, case.nt), -7.0, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        s.DenseInterpolate(t.data_ptr(), len(times), out.data_ptr())
        s.SynchroniseDevice()
        res = W.read_results(s)
        return res, out.cpu().numpy()


@pytest.mark.parametrize("mode", [0, capi.MODE_DF_STAGE | capi.MODE_PERSISTENT])
def test_gpu_interpolation_matches_cpu_statement(mode, native_libs, oracle_libs):
    case = W.duffing_param_case(nt=1024, periods=2, tol=1e-10, ndo=2048)
    T = case.arrays["td"][1][0]
    rng = np.random.default_rng(3)
    times = np.concatenate([rng.uniform(0.0, T, 40), [0.0, T, -1.0, T + 1.0]])
    res, out = gpu_dense(case, times, mode)
    assert np.all(res["didx"] < case.ndo)
    ref = O.dense_interpolate(case, res["didx"], res["dtime"], res["dstate"], times)
    nan = np.isnan(ref)
    np.testing.assert_array_equal(np.isnan(out), nan)
    assert nan[-2:].all() and not nan[:-2].any()
    scale = np.max(np.abs(res["dstate"]))
    assert np.max(np.abs(out[~nan] - ref[~nan])) < 1e-13 * scale


def test_gpu_interpolation_rejects_bad_calls(native_libs):
    import torch
    case = W.duffing_param_case(nt=64, periods=1)
    with W.load_solver(case) as s:
        t = torch.zeros(4, dtype=torch.float64, device="cuda")
        o = torch.zeros((4, 2, 64), dtype=torch.float64, device="cuda")
        with pytest.raises(RuntimeError, match="NDO"):
            s.DenseInterpolate(t.data_ptr(), 4, o.data_ptr())
