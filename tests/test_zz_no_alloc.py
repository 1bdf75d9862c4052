"""GPU test of mpgos_pt_solve_record_static, the recording entry point that
keeps the adjoint tape in the runtime's static device scratch instead of
cudaMalloc'd buffers.

Collected last (file name) so that it runs both alone and after every other
GPU test in one process. Two recordings in a row through each entry point,
each followed by the reverse pass: tapes, end states and gradients must be
bit-identical between the static-scratch and the allocating entry point, the
second static recording and its reverse pass (after the first call has
loaded the kernels) must leave the device's free memory unchanged, and an
oversized tape must be refused with a clear error.
"""
import numpy as np
import pytest

from mpgos_gb300 import capi, workloads as W
from mpgos_gb300.solver import Variable
from oracle import ref_gpu as R

pytestmark = pytest.mark.gpu

MAX_STEPS, SEGMENT = 4096, 32


def _two_calls(case, target, static: bool):
    import torch
    out = []
    free = []   # device free bytes before and after each recording + reverse pass
    with W.load_solver(case, mode=0) as s:
        a = case.arrays
        g = torch.empty((s.SD, s.NT), dtype=torch.float64, device="cuda")
        gx0 = torch.empty_like(g)
        gcp = torch.empty((s.NCP, s.NT), dtype=torch.float64, device="cuda")
        for _ in range(2):
            s.host(Variable.ActualState)[:] = a["x"]
            s.host(Variable.ActualTime)[0, :] = a["t"]
            s.host(Variable.TimeDomain)[:] = a["td"]
            s.host(Variable.IntegerAccessories)[:] = a["acci"]
            s.SynchroniseFromHostToDevice(Variable.All)
            s.SynchroniseDevice()
            before = torch.cuda.mem_get_info()[0]
            (s.SolveRecordStatic if static else s.SolveRecord)(MAX_STEPS, SEGMENT)
            s.SynchroniseFromDeviceToHost(Variable.ActualState)
            s.SynchroniseDevice()
            xT = s.host(Variable.ActualState).copy()
            g.copy_(torch.from_numpy(2.0 * (xT - target)))
            torch.cuda.synchronize()
            s.Adjoint(g.data_ptr(), gx0.data_ptr(), gcp.data_ptr())
            s.SynchroniseDevice()
            free.append((before, torch.cuda.mem_get_info()[0]))
            t = s.tape_info()
            n = R.device_to_host(t.n_steps, (case.nt,), np.int32)
            dt = R.device_to_host(t.dt, (t.max_steps, case.nt), np.float64)
            out.append(dict(xT=xT, gx0=gx0.cpu().numpy(), gcp=gcp.cpu().numpy(), n=n, dt=dt,
                            status=s.host(Variable.Status).copy(), free=free[-1]))
    return out


def test_static_scratch_recording_matches_allocating_entry_point(native_libs):
    case = W.duffing_param_case(nt=256, periods=4, tol=1e-9, seed=11)
    target = W.duffing_param_targets(256, seed=11)
    heap = _two_calls(case, target, static=False)
    stat = _two_calls(case, target, static=True)
    for h, st in zip(heap, stat):
        assert np.all(h["n"] > 0) and np.all(h["n"] <= MAX_STEPS)
        for k in ("xT", "gx0", "gcp", "n"):
            assert np.array_equal(h[k].view(np.uint8), st[k].view(np.uint8)), k
        used = np.arange(MAX_STEPS)[:, None] < h["n"][None, :]
        assert np.array_equal(h["dt"][used], st["dt"][used])
    # the second call repeats the first
    for k in ("xT", "gx0", "gcp", "n"):
        assert np.array_equal(stat[0][k], stat[1][k]), k
    # the second static recording and reverse pass took no device memory
    before, after = stat[1]["free"]
    assert before == after, f"free device memory changed by {before - after} bytes"


def test_static_scratch_rejects_an_oversized_tape(native_libs):
    case = W.duffing_param_case(nt=256, periods=1, tol=1e-9, seed=12)
    with W.load_solver(case, mode=0) as s:
        too_many = capi.STATIC_TAPE_BYTES // (8 * case.nt) + 1
        with pytest.raises(capi.MpgosError) as e:
            s.SolveRecordStatic(too_many, SEGMENT)
        assert e.value.code == 1 and "static tape" in str(e.value)
        s.SolveRecordStatic(64, SEGMENT)        # a fitting tape still records
        s.SynchroniseDevice()
