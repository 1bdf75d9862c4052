"""Synthetic ensembles of the benchmark configurations, and a GPU runner.

A ``Case`` holds every input of one ensemble in the reference's SoA layout
(SingleSystem_PerThread_Interface.cuh:355-366: ``[field][NT]`` arrays,
dense state ``[NDO][SD][NT]``) plus the solver options. The same ``Case`` is
fed to the GPU solver (``run_gpu``) and to the CPU oracle, so both integrate
identical inputs.

Configurations (all inputs synthetic; seeds fixed):
  * ``duffing_rk4``   forced hardening Duffing, fixed-step RK4, dt = 2 pi/400,
                      one forcing period per launch (8192 instances at full size)
  * ``lorenz``        Lorenz ensemble, rho = linspace(0, 21), RKCK45 1e-10,
                      t in [0, 10] (2^20 instances at full size)
  * ``duffing_param`` Duffing with per-instance (k, B) and random initial
                      states, RKCK45 1e-9 (adjoint workload, 2^18 at full size)
  * ``keller_miksis`` Keller-Miksis bubble, 512 x 512 grid of pressure
                      amplitude x frequency, RKCK45 1e-10, one acoustic
                      period per launch, radius-maximum event
  * ``duffing_events`` / ``bouncing_ball`` event, dense-output and
                      user-termination coverage cases
"""
from __future__ import annotations

import copy
import math
from dataclasses import dataclass, field

import numpy as np

SHAPES = {  # SD, NCP, NSP, NISP, NE, NA, NIA of the hook files in systems/
    "lorenz": (3, 1, 0, 0, 0, 0, 1),
    "duffing": (2, 1, 1, 0, 0, 1, 1),
    "duffing_param": (2, 2, 0, 0, 0, 0, 1),
    "duffing_param_sens": (10, 2, 0, 0, 0, 0, 1),
    "duffing_events": (2, 1, 1, 1, 2, 2, 2),
    "bouncing_ball": (2, 1, 1, 1, 2, 1, 2),
    "keller_miksis": (2, 21, 0, 0, 1, 1, 2),
}

DEFAULT_OPTIONS = dict(initial_dt=1e-2, max_dt=1e6, min_dt=1e-12, grow=5.0, shrink=0.1, dense_min_dt=0.0,
                       dense_freq=1, max_attempts=1_000_000)


@dataclass
class Case:
    system: str
    algorithm: int                 # 0 RK4, 1 RKCK45
    nt: int
    ndo: int = 0
    phases: int = 1                # launches (Solve() calls) per run
    n_active: int | None = None
    arrays: dict = field(default_factory=dict)
    rtol: np.ndarray | None = None
    atol: np.ndarray | None = None
    etol: np.ndarray | None = None
    edir: np.ndarray | None = None
    options: dict = field(default_factory=lambda: dict(DEFAULT_OPTIONS))

    @property
    def shape(self):
        return SHAPES[self.system]

    def copy(self) -> "Case":
        return copy.deepcopy(self)

    def subset(self, idx) -> "Case":
        """The instances ``idx`` as a stand-alone ensemble (same options)."""
        idx = np.asarray(idx)
        c = self.copy()
        c.nt = int(idx.size)
        c.n_active = None
        for k, v in self.arrays.items():
            if k in ("sp", "spi"):
                continue
            c.arrays[k] = np.ascontiguousarray(v[..., idx])
        return c


def empty_case(system: str, algorithm: int, nt: int, ndo: int = 0) -> Case:
    sd, ncp, nsp, nisp, ne, na, nia = SHAPES[system]
    c = Case(system=system, algorithm=algorithm, nt=nt, ndo=ndo)
    c.arrays = dict(
        td=np.zeros((2, nt)), x=np.zeros((sd, nt)), t=np.zeros(nt), cp=np.zeros((ncp, nt)), sp=np.zeros(nsp),
        spi=np.zeros(nisp, dtype=np.int32), acc=np.zeros((na, nt)), acci=np.zeros((nia, nt), dtype=np.int32),
        didx=np.zeros(nt, dtype=np.int32), dtime=np.zeros((ndo, nt)), dstate=np.zeros((ndo, sd, nt)),
    )
    c.rtol = np.full(sd, 1e-8)
    c.atol = np.full(sd, 1e-8)
    c.etol = np.full(ne, 1e-6)
    c.edir = np.zeros(ne, dtype=np.int32)
    return c


def linspace(b: float, e: float, n: int) -> np.ndarray:
    """Linspace of the reference tutorials (T1_Reference/Reference.cu:134-150)."""
    x = np.empty(n)
    x[0] = b
    if n > 1:
        x[n - 1] = e
        inc = (e - b) / (n - 1)
        for i in range(1, n - 1):
            x[i] = b + i * inc
    return x


def logspace(b: float, e: float, n: int) -> np.ndarray:
    """Logspace of the reference tutorials (T4_QuasiperiodicForcing/QuasiperiodicForcing.cu Logspace)."""
    x = np.empty(n)
    x[0] = b
    if n > 1:
        x[n - 1] = e
        eb, ee = math.log10(b), math.log10(e)
        inc = (ee - eb) / (n - 1)
        for i in range(1, n - 1):
            x[i] = math.pow(10.0, eb + i * inc)
    return x


# ---------------------------------------------------------------------------
# configurations
# ---------------------------------------------------------------------------
def lorenz_case(nt: int = 1 << 20, t_end: float = 10.0, tol: float = 1e-10, rho=(0.0, 21.0)) -> Case:
    c = empty_case("lorenz", 1, nt)
    a = c.arrays
    a["td"][1] = t_end
    a["x"][:] = 10.0
    a["cp"][0] = linspace(rho[0], rho[1], nt)
    c.rtol[:] = tol
    c.atol[:] = tol
    c.options["initial_dt"] = 1e-2
    return c


def duffing_rk4_case(nt: int = 8192, periods: int = 1024, B: float = 0.3) -> Case:
    c = empty_case("duffing", 0, nt)
    a = c.arrays
    a["td"][0] = 0.0
    a["td"][1] = 2.0 * math.pi
    a["x"][0] = -0.5
    a["x"][1] = 0.1
    a["cp"][0] = linspace(0.2, 0.3, nt)
    a["sp"][0] = B
    a["acc"][0] = -0.5
    c.options["initial_dt"] = 2.0 * math.pi / 400.0
    c.phases = periods
    return c


def duffing_param_case(nt: int = 1 << 18, periods: int = 64, tol: float = 1e-9, seed: int = 20261203,
                       ndo: int = 0) -> Case:
    rng = np.random.default_rng(seed)
    c = empty_case("duffing_param", 1, nt, ndo)
    a = c.arrays
    a["td"][1] = 2.0 * math.pi * periods
    a["cp"][0] = rng.uniform(0.2, 0.3, nt)
    a["cp"][1] = rng.uniform(0.2, 0.4, nt)
    a["x"][:] = rng.uniform(-1.0, 1.0, (2, nt))
    c.rtol[:] = tol
    c.atol[:] = tol
    return c


def duffing_param_targets(nt: int, seed: int = 20261203) -> np.ndarray:
    """Per-instance terminal targets ~ N(0, 0.5^2) of the adjoint loss."""
    rng = np.random.default_rng(seed + 1)
    return rng.normal(0.0, 0.5, (2, nt))


def duffing_param_sens_case(base: Case, tol: float = 1e-12) -> Case:
    """The forward-sensitivity system of ``base`` (a duffing_param case):
    state plus d(state)/d(x0, v0, k, B), starting from the identity block."""
    c = empty_case("duffing_param_sens", 1, base.nt)
    for k in ("td", "t", "cp"):
        c.arrays[k] = base.arrays[k].copy()
    c.arrays["x"][:2] = base.arrays["x"]
    c.arrays["x"][2] = 1.0   # dx0/dx0(0)
    c.arrays["x"][5] = 1.0   # dx1/dx1(0)
    c.rtol[:] = tol
    c.atol[:] = tol
    c.options = dict(base.options)
    return c


def duffing_events_case(nt: int = 256, periods: int = 4, ndo: int = 16, seed: int = 7, stop_after: int = 0,
                        tol: float = 1e-9) -> Case:
    rng = np.random.default_rng(seed)
    c = empty_case("duffing_events", 1, nt, ndo)
    a = c.arrays
    a["td"][1] = 2.0 * math.pi
    a["x"][0] = rng.uniform(-1.0, 1.0, nt)
    a["x"][1] = rng.uniform(-1.0, 1.0, nt)
    a["cp"][0] = linspace(0.2, 0.3, nt)
    a["sp"][0] = 0.3
    a["spi"][0] = stop_after
    c.rtol[:] = tol
    c.atol[:] = tol
    c.etol[:] = 1e-6
    c.edir[:] = [-1, 0]
    c.options.update(dense_min_dt=2.0 * math.pi / 64, dense_freq=1, max_dt=1e3, min_dt=1e-14, grow=10.0, shrink=0.2)
    c.phases = periods
    return c


def bouncing_ball_case(nt: int = 128, impacts: int = 6, seed: int = 11) -> Case:
    rng = np.random.default_rng(seed)
    c = empty_case("bouncing_ball", 1, nt)
    a = c.arrays
    a["td"][1] = 1e3
    a["x"][0] = rng.uniform(0.5, 2.0, nt)
    a["x"][1] = rng.uniform(-1.0, 1.0, nt)
    a["cp"][0] = rng.uniform(0.5, 0.9, nt)
    a["sp"][0] = 9.81
    a["spi"][0] = impacts
    c.rtol[:] = 1e-10
    c.atol[:] = 1e-10
    c.etol[:] = 1e-8
    c.edir[:] = [-1, -1]
    return c


# Water at 25 C and the bubble constants of the reference Keller-Miksis
# tutorials (T4_QuasiperiodicForcing/QuasiperiodicForcing.cu, FillSolverObject).
KM_WATER = dict(Pv=3.166775638952003e+03, Rho=9.970639504998557e+02, ST=0.071977583160056,
                Vis=8.902125058209557e-04, CL=1.497251785455527e+03)


def keller_miksis_coefficients(pa1_bar: float, f1_khz: float, pa2_bar: float = 0.0, f2_khz: float = 0.0,
                               phase: float = 0.0, re_um: float = 10.0, pinf_bar: float = 1.0,
                               kappa: float = 1.4) -> list:
    """The 21 control parameters of one bubble (coefficient formulas of
    T4_QuasiperiodicForcing/QuasiperiodicForcing.cu FillSolverObject)."""
    w = KM_WATER
    PI = math.pi
    Pinf = pinf_bar * 1.0e5
    PA1 = pa1_bar * 1.0e5
    PA2 = pa2_bar * 1.0e5
    RE = re_um / 1.0e6
    f1 = 2.0 * PI * (f1_khz * 1000)
    f2 = 2.0 * PI * (f2_khz * 1000)
    s = 2.0 * PI / RE / f1
    cp = [
        (2.0 * w["ST"] / RE + Pinf - w["Pv"]) * math.pow(s, 2.0) / w["Rho"],
        (1.0 - 3.0 * kappa) * (2 * w["ST"] / RE + Pinf - w["Pv"]) * s / w["CL"] / w["Rho"],
        (Pinf - w["Pv"]) * math.pow(s, 2.0) / w["Rho"],
        (2.0 * w["ST"] / RE / w["Rho"]) * math.pow(s, 2.0),
        (4.0 * w["Vis"] / w["Rho"] / math.pow(RE, 2.0)) * (2.0 * PI / f1),
        PA1 * math.pow(s, 2.0) / w["Rho"],
        PA2 * math.pow(s, 2.0) / w["Rho"],
        (RE * f1 * PA1 / w["Rho"] / w["CL"]) * math.pow(s, 2.0),
        (RE * f2 * PA2 / w["Rho"] / w["CL"]) * math.pow(s, 2.0),
        RE * f1 / (2.0 * PI) / w["CL"],
        3.0 * kappa,
        (f2_khz / f1_khz),
        phase,
        2.0 * PI / f1,
        RE,
        pa1_bar, f1_khz, pa2_bar, f2_khz, phase, re_um,
    ]
    return cp


def keller_miksis_case(n_amp: int = 512, n_freq: int = 512, periods: int = 1024, tol: float = 1e-10,
                       amp=(0.5, 1.5), freq=(20.0, 1000.0)) -> Case:
    nt = n_amp * n_freq
    c = empty_case("keller_miksis", 1, nt)
    a = c.arrays
    amps = linspace(amp[0], amp[1], n_amp)
    freqs = logspace(freq[0], freq[1], n_freq)
    cp = np.empty((21, nt))
    i = 0
    for pa in amps:
        for f in freqs:
            cp[:, i] = keller_miksis_coefficients(pa, f)
            i += 1
    a["cp"][:] = cp
    a["td"][1] = 1.0
    a["x"][0] = 1.0
    a["x"][1] = 0.0
    c.rtol[:] = tol
    c.atol[:] = tol
    c.edir[:] = -1
    c.phases = periods
    return c


# ---------------------------------------------------------------------------
# GPU runner
# ---------------------------------------------------------------------------
def load_solver(case: Case, mode: int = 0, block: int | None = None, device: int = 0, precision: str = "double"):
    """A ProblemSolver holding ``case`` on the device (inputs uploaded)."""
    from .solver import ProblemSolver, Option, Variable

    s = ProblemSolver(case.system, case.nt, case.ndo, algorithm=case.algorithm, precision=precision, device=device)
    a = case.arrays
    s.host(Variable.TimeDomain)[:] = a["td"]
    s.host(Variable.ActualState)[:] = a["x"]
    s.host(Variable.ActualTime)[0, :] = a["t"]
    if s.NCP:
        s.host(Variable.ControlParameters)[:] = a["cp"]
    if s.NSP:
        s.host(Variable.SharedParameters)[:] = a["sp"]
    if s.NISP:
        s.host(Variable.IntegerSharedParameters)[:] = a["spi"]
    if s.NA:
        s.host(Variable.Accessories)[:] = a["acc"]
    if s.NIA:
        s.host(Variable.IntegerAccessories)[:] = a["acci"]
    s.host(Variable.DenseIndex)[0, :] = a["didx"]
    if case.ndo:
        s.host(Variable.DenseTime)[:] = a["dtime"]
        s.host(Variable.DenseState)[:] = a["dstate"]
    o = case.options
    s.SolverOption(Option.InitialTimeStep, o["initial_dt"])
    s.SolverOption(Option.MaximumTimeStep, o["max_dt"])
    s.SolverOption(Option.MinimumTimeStep, o["min_dt"])
    s.SolverOption(Option.TimeStepGrowLimit, o["grow"])
    s.SolverOption(Option.TimeStepShrinkLimit, o["shrink"])
    s.SolverOption(Option.DenseOutputMinimumTimeStep, o["dense_min_dt"])
    s.SolverOption(Option.DenseOutputSaveFrequency, o["dense_freq"])
    s.SolverOption(Option.MaximumAttempts, o["max_attempts"])
    if case.n_active is not None:
        s.SolverOption(Option.ActiveNumberOfThreads, case.n_active)
    if case.algorithm == 1:
        for i in range(s.SD):
            s.SolverOption(Option.RelativeTolerance, i, case.rtol[i])
            s.SolverOption(Option.AbsoluteTolerance, i, case.atol[i])
    for i in range(s.NE):
        s.SolverOption(Option.EventTolerance, i, case.etol[i])
        s.SolverOption(Option.EventDirection, i, int(case.edir[i]))
    s.SolverOption(Option.KernelMode, mode)
    if block is not None:
        s.SolverOption(Option.ThreadsPerBlock, block)
    s.SynchroniseFromHostToDevice(Variable.All)
    return s


def read_results(s) -> dict:
    from .solver import Variable

    s.SynchroniseFromDeviceToHost(Variable.All)
    for v in (Variable.Status, Variable.AcceptedSteps, Variable.RejectedSteps):
        s.SynchroniseFromDeviceToHost(v)
    s.InsertSynchronisationPoint()
    s.SynchroniseSolver()
    out = dict(
        td=s.host(Variable.TimeDomain).copy(), x=s.host(Variable.ActualState).copy(),
        t=s.host(Variable.ActualTime)[0].copy(), didx=s.host(Variable.DenseIndex)[0].copy(),
        status=s.host(Variable.Status)[0].copy(), nacc=s.host(Variable.AcceptedSteps)[0].copy(),
        nrej=s.host(Variable.RejectedSteps)[0].copy(),
    )
    out["cp"] = s.host(Variable.ControlParameters).copy() if s.NCP else np.zeros((0, s.NT))
    out["acc"] = s.host(Variable.Accessories).copy() if s.NA else np.zeros((0, s.NT))
    out["acci"] = s.host(Variable.IntegerAccessories).copy() if s.NIA else np.zeros((0, s.NT), dtype=np.int32)
    if s.NDO:
        out["dtime"] = s.host(Variable.DenseTime).copy()
        out["dstate"] = s.host(Variable.DenseState).copy()
    return out


def run_gpu(case: Case, mode: int = 0, block: int | None = None, graph: bool = False, device: int = 0,
            precision: str = "double") -> dict:
    """Integrate ``case`` on the GPU: ``case.phases`` launches, then read back."""
    with load_solver(case, mode=mode, block=block, device=device, precision=precision) as s:
        if graph:
            s.SolvePhases(case.phases)
        else:
            for _ in range(case.phases):
                s.Solve()
        return read_results(s)


def _main(argv=None) -> int:
    """Integrate one synthetic ensemble on the GPU and print a summary line:
    ``python -m mpgos_gb300.workloads --case lorenz --nt 262144 --mode 18
    --block 128 --launches 2`` (the command the kernel profiles are taken
    with: every launch is a full integration from the initial state)."""
    import argparse
    import json
    import time

    ap = argparse.ArgumentParser(prog="python -m mpgos_gb300.workloads")
    ap.add_argument("--case", default="lorenz", choices=["lorenz", "keller_miksis", "duffing_param", "duffing_rk4"])
    ap.add_argument("--nt", type=int, default=1 << 18)
    ap.add_argument("--mode", type=int, default=0, help="MPGOS_MODE_* bits")
    ap.add_argument("--block", type=int, default=128)
    ap.add_argument("--launches", type=int, default=1)
    ap.add_argument("--outline", action="store_true",
                    help="double-float kernels: the right-hand side out of line (MPGOS_OUTLINE_RHS)")
    ap.add_argument("--periods", type=int, default=None, help="forcing periods (duffing_param, duffing_rk4)")
    ap.add_argument("--work-order", action="store_true",
                    help="every launch takes the instances longest first by the previous launch's attempts "
                         "(MPGOS_WORK_ORDER; the first launch in index order)")
    ap.add_argument("--adjoint", type=int, default=0, metavar="SEG",
                    help="after the launches: one recording pass and one reverse pass with checkpoints every SEG steps")
    a = ap.parse_args(argv)
    if a.case == "lorenz":
        case = lorenz_case(nt=a.nt)
    elif a.case == "keller_miksis":
        side = max(1, int(round(math.sqrt(a.nt))))
        case = keller_miksis_case(n_amp=side, n_freq=max(1, a.nt // side))
    elif a.case == "duffing_param":
        case = duffing_param_case(nt=a.nt, **({"periods": a.periods} if a.periods else {}))
    else:
        case = duffing_rk4_case(nt=a.nt, **({"periods": a.periods} if a.periods else {}))
    from .solver import Variable
    with load_solver(case, mode=a.mode, block=a.block) as s:
        if a.outline:
            from .capi import Option
            s.SolverOption(Option.OutlineRhs, 1)
        if a.work_order:
            from .capi import Option
            s.SolverOption(Option.WorkOrder, 1)
        s.checkpoint_save()
        times = []
        for _ in range(a.launches):
            s.checkpoint_restore()
            s.SynchroniseDevice()
            t0 = time.perf_counter()
            s.Solve()
            s.SynchroniseDevice()
            times.append(time.perf_counter() - t0)
        res = read_results(s)
        adj = None
        if a.adjoint:
            import torch
            s.checkpoint_restore()
            s.SolveRecord(int(res["nacc"].max()) + 64, a.adjoint)
            g = torch.ones((s.SD, case.nt), dtype=torch.float64, device="cuda")
            gx0, gp = torch.empty_like(g), torch.empty((max(s.NCP, 1), case.nt), dtype=torch.float64, device="cuda")
            s.SynchroniseDevice()
            t0 = time.perf_counter()
            s.Adjoint(g.data_ptr(), gx0.data_ptr(), gp.data_ptr())
            s.SynchroniseDevice()
            adj = time.perf_counter() - t0
    print(json.dumps({"case": a.case, "nt": case.nt, "mode": a.mode, "block": a.block, "launches": a.launches,
                      "accepted": int(res["nacc"].sum()), "rejected": int(res["nrej"].sum()),
                      "status_max": int(res["status"].max()), "wall_s_last": times[-1], "adjoint_wall_s": adj}))
    return 0


if __name__ == "__main__":
    raise SystemExit(_main())
