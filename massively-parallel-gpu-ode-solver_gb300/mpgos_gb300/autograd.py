"""torch.autograd binding of the discrete adjoint (a test harness).

``terminal_state(x0, cp, runner)`` integrates an ensemble from initial states
``x0`` [SD][NT] with control parameters ``cp`` [NCP][NT] and returns the end
states x(T) [SD][NT]; its backward pass is the GPU discrete adjoint
(mpgos_pt_solve_record / mpgos_pt_adjoint of the C-ABI). Any scalar loss built
from x(T) in torch therefore gets d loss / d x0 and d loss / d cp with the
frozen step sequence of the forward pass. torch only moves tensors here; the
integration and its adjoint are the sm_103a kernels.
"""
from __future__ import annotations

import numpy as np
import torch

from . import capi, workloads as W
from .solver import Variable


class AdjointRunner:
    """A solver loaded with ``case`` whose forward pass records the adjoint tape."""

    def __init__(self, case: W.Case, mode: int = 0, max_steps: int = 20000, segment: int = 32, device: int = 0):
        self.case = case
        self.max_steps, self.segment = max_steps, segment
        self.solver = W.load_solver(case, mode=mode, device=device)
        self.device = torch.device("cuda", device)

    def close(self):
        self.solver.close()

    def forward(self, x0: torch.Tensor, cp: torch.Tensor) -> torch.Tensor:
        s, a = self.solver, self.case.arrays
        s.host(Variable.ActualState)[:] = x0.detach().double().cpu().numpy()
        if s.NCP:
            s.host(Variable.ControlParameters)[:] = cp.detach().double().cpu().numpy()
        s.host(Variable.TimeDomain)[:] = a["td"]
        s.host(Variable.ActualTime)[0, :] = a["t"]
        if s.NIA:
            s.host(Variable.IntegerAccessories)[:] = a["acci"]
        if s.NA:
            s.host(Variable.Accessories)[:] = a["acc"]
        s.SynchroniseFromHostToDevice(Variable.All)
        s.SolveRecord(self.max_steps, self.segment)
        s.SynchroniseFromDeviceToHost(Variable.ActualState)
        s.InsertSynchronisationPoint()
        s.SynchroniseSolver()
        return torch.from_numpy(s.host(Variable.ActualState).copy()).to(self.device)

    def backward(self, grad_xT: torch.Tensor):
        s = self.solver
        g = grad_xT.detach().to(device=self.device, dtype=torch.float64).contiguous()
        gx0 = torch.empty_like(g)
        gcp = torch.empty((max(s.NCP, 1), s.NT), dtype=torch.float64, device=self.device)
        torch.cuda.synchronize(self.device)
        s.Adjoint(g.data_ptr(), gx0.data_ptr(), gcp.data_ptr())
        s.SynchroniseFromDeviceToHost(Variable.Status)
        s.InsertSynchronisationPoint()
        s.SynchroniseSolver()
        bad = int(np.count_nonzero(s.host(Variable.Status) & capi.INSTANCE_TAPE_OVERFLOW))
        if bad:
            raise RuntimeError(f"{bad} instances took more accepted steps than the tape holds ({self.max_steps})")
        return gx0, gcp[: s.NCP]


class _TerminalState(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x0, cp, runner):
        ctx.runner = runner
        return runner.forward(x0, cp)

    @staticmethod
    def backward(ctx, grad_xT):
        gx0, gcp = ctx.runner.backward(grad_xT)
        return gx0, gcp, None


def terminal_state(x0: torch.Tensor, cp: torch.Tensor, runner: AdjointRunner) -> torch.Tensor:
    return _TerminalState.apply(x0, cp, runner)
