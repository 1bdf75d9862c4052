"""Synthetic coupled ensembles (rings of forced Duffing units) and a GPU runner.

A ``CbCase`` holds every input of one coupled ensemble in the layout of the
coupled solver (unit scope [field][NS*UPS], system scope [field][NS]) with the
coupling matrices in full [NC][UPS][UPS] form; the same ``CbCase`` is fed to
the GPU solver (``run_coupled_gpu``), to the CPU oracle and to the
reference's own coupled kernel, so all integrate identical inputs.

``ring_case``: systems of UPS Duffing units
  x_i'' + k x_i' + x_i + x_i^3 = B cos(t) + sum_j C_ij x_j
(systems/ring_duffing.cuh), k = 0.25, B ~ U[0.2, 0.4] per system, initial
(x_i, v_i) ~ U[-1, 1]^2 per unit, adaptive RKCK45, an event on every x_i = 0
crossing counted per unit, the accepted steps counted per system. Coupling
``dense``: nearest ring neighbours 0.1, every other entry N(0, 0.01^2);
``circulant``: the circulant ring (0.1 on both neighbours, 0 elsewhere),
which every storage (full, banded, circular-banded, full circular) holds.
At full size (the coupled configuration): 16384 systems x 64 units, dense
coupling, rtol = atol = 1e-9, 256 forcing periods.
"""
from __future__ import annotations

import copy
import math
from dataclasses import dataclass, field

import numpy as np

from .coupled import matrix_entries, store_matrices

CB_SHAPES = {  # UPS, UD, NC, CBW, CCI, NUP, NSP, NGP, NIGP, NUA, NIUA, NSA, NISA, NE
    "ring64": (64, 2, 1, 0, 0, 0, 1, 1, 0, 0, 1, 0, 1, 1),
    "ring16_full": (16, 2, 1, 0, 0, 0, 1, 1, 0, 0, 1, 0, 1, 1),
    "ring16_band": (16, 2, 1, 1, 0, 0, 1, 1, 0, 0, 1, 0, 1, 1),
    "ring16_circband": (16, 2, 1, 1, 1, 0, 1, 1, 0, 0, 1, 0, 1, 1),
    "ring16_circ": (16, 2, 1, 0, 1, 0, 1, 1, 0, 0, 1, 0, 1, 1),
    "ring256": (256, 2, 1, 0, 0, 0, 1, 1, 0, 0, 1, 0, 1, 1),
}

CB_DEFAULT_OPTIONS = dict(initial_dt=1e-2, max_dt=1e6, min_dt=1e-12, grow=5.0, shrink=0.1, dense_min_dt=0.0,
                          dense_freq=1, max_attempts=10_000_000, shared_global=1, shared_coupling=1)


@dataclass
class CbCase:
    system: str
    algorithm: int                 # 0 RK4, 1 RKCK45
    ns: int
    ndo: int = 0
    phases: int = 1
    n_active: int | None = None
    arrays: dict = field(default_factory=dict)
    rtol: np.ndarray | None = None
    atol: np.ndarray | None = None
    etol: np.ndarray | None = None
    edir: np.ndarray | None = None
    options: dict = field(default_factory=lambda: dict(CB_DEFAULT_OPTIONS))

    @property
    def shape(self):
        return CB_SHAPES[self.system]

    @property
    def ups(self) -> int:
        return self.shape[0]

    def copy(self) -> "CbCase":
        return copy.deepcopy(self)

    def stored_matrix(self) -> np.ndarray:
        ups, _, nc, cbw, cci = self.shape[:5]
        return store_matrices(self.arrays["cmat"], cbw, cci)


def ring_matrix(ups: int, kind: str, rng) -> np.ndarray:
    if kind == "dense":
        C = rng.normal(0.0, 0.01, (ups, ups))
    elif kind == "circulant":
        C = np.zeros((ups, ups))
    else:
        raise ValueError(kind)
    for i in range(ups):
        C[i, (i + 1) % ups] = 0.1
        C[i, (i - 1) % ups] = 0.1
    return C


def ring_case(system: str = "ring64", ns: int = 16384, periods: float = 256, tol: float = 1e-9, seed: int = 5,
              ndo: int = 0, coupling: str | None = None, algorithm: int = 1, dt_rk4: float | None = None) -> CbCase:
    ups, ud, nc, cbw, cci, nup, nsp, ngp, nigp, nua, niua, nsa, nisa, ne = CB_SHAPES[system]
    rng = np.random.default_rng(seed)
    nu = ns * ups
    c = CbCase(system=system, algorithm=algorithm, ns=ns, ndo=ndo)
    if coupling is None:
        coupling = "dense" if (cbw == 0 and cci == 0) else "circulant"
    a = c.arrays
    a["td"] = np.vstack([np.zeros(ns), np.full(ns, 2.0 * math.pi * periods)])
    a["t"] = np.zeros(ns)
    a["x"] = rng.uniform(-1.0, 1.0, (ud, nu))
    a["up"] = np.zeros((nup, nu))
    a["uacc"] = np.zeros((nua, nu))
    a["iuacc"] = np.zeros((niua, nu), dtype=np.int32)
    a["sp"] = rng.uniform(0.2, 0.4, (nsp, ns))
    a["sacc"] = np.zeros((nsa, ns))
    a["isacc"] = np.zeros((nisa, ns), dtype=np.int32)
    a["cstr"] = np.ones((nc, ns))
    a["didx"] = np.zeros(ns, dtype=np.int32)
    a["dtime"] = np.zeros((ndo, ns))
    a["dstate"] = np.zeros((ndo, ud, nu))
    a["gp"] = np.array([0.25])
    a["igp"] = np.zeros(nigp, dtype=np.int32)
    a["cidx"] = np.array([1], dtype=np.int32)
    a["cmat"] = np.stack([ring_matrix(ups, coupling, rng) for _ in range(nc)])
    c.rtol = np.full(ud, tol)
    c.atol = np.full(ud, tol)
    c.etol = np.full(ne, 1e-6)
    c.edir = np.zeros(ne, dtype=np.int32)
    if algorithm == 0:
        c.options["initial_dt"] = dt_rk4 or 2.0 * math.pi / 400.0
    return c


def load_coupled_solver(case: CbCase, mode: int = 0, warps: int | None = None, device: int = 0):
    from .capi import CbOption as O, CbVariable as V
    from .coupled import CoupledProblemSolver

    s = CoupledProblemSolver(case.system, case.ns, case.ndo, algorithm=case.algorithm, device=device)
    a = case.arrays
    s.host(V.TimeDomain)[:] = a["td"]
    s.host(V.ActualTime)[:] = a["t"]
    s.host(V.ActualState)[:] = a["x"]
    for var, key, n in ((V.UnitParameters, "up", s.NUP), (V.UnitAccessories, "uacc", s.NUA),
                        (V.IntegerUnitAccessories, "iuacc", s.NiUA), (V.SystemParameters, "sp", s.NSP),
                        (V.SystemAccessories, "sacc", s.NSA), (V.IntegerSystemAccessories, "isacc", s.NiSA),
                        (V.CouplingStrength, "cstr", s.NC)):
        if n:
            s.host(var)[:] = a[key]
    s.host(V.DenseIndex)[:] = a["didx"]
    if case.ndo:
        s.host(V.DenseTime)[:] = a["dtime"]
        s.host(V.DenseState)[:] = a["dstate"]
    if s.NGP:
        s.host(V.GlobalParameters)[:] = a["gp"]
    if s.NiGP:
        s.host(V.IntegerGlobalParameters)[:] = a["igp"]
    s.host(V.CouplingIndex)[:] = a["cidx"]
    for i in range(s.NC):
        s.SetCouplingMatrix(i, a["cmat"][i])
    o = case.options
    s.SolverOption(O.InitialTimeStep, o["initial_dt"])
    s.SolverOption(O.MaximumTimeStep, o["max_dt"])
    s.SolverOption(O.MinimumTimeStep, o["min_dt"])
    s.SolverOption(O.TimeStepGrowLimit, o["grow"])
    s.SolverOption(O.TimeStepShrinkLimit, o["shrink"])
    s.SolverOption(O.DenseOutputMinimumTimeStep, o["dense_min_dt"])
    s.SolverOption(O.DenseOutputSaveFrequency, o["dense_freq"])
    s.SolverOption(O.MaximumAttempts, o["max_attempts"])
    s.SolverOption(O.SharedGlobalVariables, o["shared_global"])
    s.SolverOption(O.SharedCouplingMatrices, o["shared_coupling"])
    if case.n_active is not None:
        s.SolverOption(O.ActiveSystems, case.n_active)
    if case.algorithm == 1:
        for i in range(s.UD):
            s.SolverOption(O.RelativeTolerance, i, case.rtol[i])
            s.SolverOption(O.AbsoluteTolerance, i, case.atol[i])
    for i in range(s.NE):
        s.SolverOption(O.EventTolerance, i, case.etol[i])
        s.SolverOption(O.EventDirection, i, int(case.edir[i]))
    s.SolverOption(O.KernelMode, mode)
    if warps is not None:
        s.SolverOption(O.WarpsPerBlock, warps)
    s.SynchroniseFromHostToDevice(V.All)
    return s


def read_coupled_results(s) -> dict:
    from .capi import CbVariable as V

    s.SynchroniseFromDeviceToHost(V.All)
    for v in (V.Status, V.AcceptedSteps, V.RejectedSteps):
        s.SynchroniseFromDeviceToHost(v)
    s.SynchroniseDevice()
    out = dict(td=s.host(V.TimeDomain).copy(), t=s.host(V.ActualTime).copy(), x=s.host(V.ActualState).copy(),
               didx=s.host(V.DenseIndex).copy(), status=s.host(V.Status).copy(),
               nacc=s.host(V.AcceptedSteps).copy(), nrej=s.host(V.RejectedSteps).copy())
    out["iuacc"] = s.host(V.IntegerUnitAccessories).copy() if s.NiUA else np.zeros((0, s.NU), np.int32)
    out["uacc"] = s.host(V.UnitAccessories).copy() if s.NUA else np.zeros((0, s.NU))
    out["isacc"] = s.host(V.IntegerSystemAccessories).copy() if s.NiSA else np.zeros((0, s.NS), np.int32)
    out["sacc"] = s.host(V.SystemAccessories).copy() if s.NSA else np.zeros((0, s.NS))
    if s.NDO:
        out["dtime"] = s.host(V.DenseTime).copy()
        out["dstate"] = s.host(V.DenseState).copy()
    return out


def run_coupled_gpu(case: CbCase, mode: int = 0, warps: int | None = None, device: int = 0) -> dict:
    """Integrate ``case`` on the GPU: ``case.phases`` launches, then read back."""
    with load_coupled_solver(case, mode=mode, warps=warps, device=device) as s:
        for _ in range(case.phases):
            s.Solve()
        return read_coupled_results(s)


def stored_entries(system: str) -> int:
    ups, _, nc, cbw, cci = CB_SHAPES[system][:5]
    return nc * matrix_entries(ups, cbw, cci)


def _main(argv=None) -> int:
    """Integrate one ring ensemble on the GPU and print a summary line:
    ``python -m mpgos_gb300.coupled_workloads --system ring64 --ns 2048
    --periods 2 --mode 18 --warps 2 --launches 2`` (the command the coupled
    kernel profiles are taken with)."""
    import argparse
    import json
    import time

    ap = argparse.ArgumentParser(prog="python -m mpgos_gb300.coupled_workloads")
    ap.add_argument("--system", default="ring64", choices=sorted(CB_SHAPES))
    ap.add_argument("--ns", type=int, default=2048)
    ap.add_argument("--periods", type=float, default=2)
    ap.add_argument("--mode", type=int, default=0, help="MPGOS_MODE_* bits (PERSISTENT 2, DF_STAGE 16, SPLIT 128)")
    ap.add_argument("--warps", type=int, default=4)
    ap.add_argument("--launches", type=int, default=1)
    ap.add_argument("--adjoint", type=int, default=0, metavar="SEG",
                    help="after the launches: one recording pass and one reverse pass (gradient of the summed "
                         "terminal energy) with checkpoints every SEG steps, in --adjoint-mode")
    ap.add_argument("--adjoint-mode", type=int, default=None, help="MPGOS_MODE_* bits of the reverse pass")
    a = ap.parse_args(argv)
    case = ring_case(a.system, ns=a.ns, periods=a.periods)
    from .capi import CbVariable as V
    with load_coupled_solver(case, mode=a.mode, warps=a.warps) as s:
        s.checkpoint_save()
        for _ in range(a.launches):
            s.checkpoint_restore()
            s.SynchroniseDevice()
            t0 = time.perf_counter()
            s.Solve()
            s.SynchroniseDevice()
            wall = time.perf_counter() - t0
        res = read_coupled_results(s)
        adj = None
        if a.adjoint:
            import numpy as np
            import torch
            s.checkpoint_restore()
            s.SolveRecord(int(res["nacc"].max()) + 64, a.adjoint)
            s.SynchroniseFromDeviceToHost(V.ActualState)
            s.SynchroniseDevice()
            xT = s.host(V.ActualState)
            g = torch.tensor(np.stack([xT[0] + xT[0] ** 3, xT[1]]), device="cuda")
            gx0 = torch.empty_like(g)
            gsp = torch.empty((max(s.NSP, 1), case.ns), dtype=torch.float64, device="cuda")
            if a.adjoint_mode is not None:
                s.set_mode(a.adjoint_mode)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.Adjoint(g.data_ptr(), gx0.data_ptr(), gsp.data_ptr())
            s.SynchroniseDevice()
            adj = time.perf_counter() - t0
    print(json.dumps({"system": a.system, "ns": a.ns, "periods": a.periods, "mode": a.mode, "warps": a.warps,
                      "accepted": int(res["nacc"].sum()), "rejected": int(res["nrej"].sum()),
                      "status_max": int(res["status"].max()), "wall_s_last": wall, "adjoint_wall_s": adj}))
    return 0


if __name__ == "__main__":
    raise SystemExit(_main())
