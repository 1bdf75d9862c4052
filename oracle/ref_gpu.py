"""Launch the reference's own per-thread kernel (sm_103a cubin) on the GPU.

TEST INFRASTRUCTURE ONLY: the reference kernels for bit-level parity of the GB300
kernels and the reference-kernel timing in bench.py. Never used by the
product.

The cubins (oracle/_ref/ref_gpu_*.cubin, see build_oracle.py) hold one
instantiation of the reference kernel SingleSystem_PerThread<NT,...>
(SourceCodes/SingleSystem_PerThread_Solver.cuh:11-437) each. They are loaded
with the CUDA driver API and launched exactly as the reference's Solve()
does (SingleSystem_PerThread_Interface.cuh:1279-1285: grid ceil(NT/block),
dynamic shared memory PreferSharedMemory * (NSP*8 + NISP*4), by-value
argument structs) on the device buffers of a GB300 ``ProblemSolver``, whose
SoA layout is the reference's. Tolerance and event arrays are separate device
copies padded to max(SD, NE) entries, because the reference kernel reads the
event options for every index below SD (SingleSystem_PerThread_Solver.cuh:60).

Launches use one warp per block (the reference's default BlockSize, the warp
size, SingleSystem_PerThread_Interface.cuh:343): the reference kernel stages
tolerances and event options into shared memory from threads 0..SD-1 and
reads them from every thread without a barrier
(SingleSystem_PerThread_Solver.cuh:37-65), so with several warps per block the
later warps can read the shared arrays before they are written. Larger blocks
are launched only with the ``sync`` cubins, built with one barrier added
after that staging (build_oracle.REF_GPU_SYNC_KERNELS).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build_oracle as _b

_cuda = None


class ThreadConfiguration(C.Structure):
    _fields_ = [("GridSize", C.c_int), ("BlockSize", C.c_int), ("NumberOfActiveThreads", C.c_int)]


class GlobalVariables(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in (
        "d_TimeDomain", "d_ActualState", "d_ActualTime", "d_ControlParameters", "d_SharedParameters",
        "d_IntegerSharedParameters", "d_Accessories", "d_IntegerAccessories", "d_RelativeTolerance",
        "d_AbsoluteTolerance", "d_EventTolerance", "d_EventDirection", "d_DenseOutputIndex",
        "d_DenseOutputTimeInstances", "d_DenseOutputStates")]


class SharedMemoryUsage(C.Structure):
    _fields_ = [("PreferSharedMemory", C.c_int), ("IsAdaptive", C.c_int)]


class SolverOptions(C.Structure):
    _fields_ = [("InitialTimeStep", C.c_double), ("MaximumTimeStep", C.c_double), ("MinimumTimeStep", C.c_double),
                ("TimeStepGrowLimit", C.c_double), ("TimeStepShrinkLimit", C.c_double),
                ("DenseOutputSaveFrequency", C.c_int), ("DenseOutputMinimumTimeStep", C.c_double)]


def _driver():
    global _cuda
    if _cuda is None:
        lib = C.CDLL("libcuda.so.1")
        P = C.c_void_p
        for name, args in {
            "cuModuleLoad": [C.POINTER(P), C.c_char_p],
            "cuModuleUnload": [P],
            "cuModuleGetFunctionCount": [C.POINTER(C.c_uint), P],
            "cuModuleEnumerateFunctions": [C.POINTER(P), C.c_uint, P],
            "cuLaunchKernel": [P, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, P,
                               C.POINTER(P), C.POINTER(P)],
            "cuMemAlloc_v2": [C.POINTER(C.c_uint64), C.c_size_t],
            "cuMemFree_v2": [C.c_uint64],
            "cuMemcpyHtoD_v2": [C.c_uint64, P, C.c_size_t],
            "cuMemcpyDtoH_v2": [P, C.c_uint64, C.c_size_t],
            "cuCtxGetCurrent": [C.POINTER(P)],
            "cuGetErrorString": [C.c_int, C.POINTER(C.c_char_p)],
        }.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = C.c_int
        _cuda = lib
    return _cuda


def _ck(rc, what):
    if rc != 0:
        s = C.c_char_p()
        _driver().cuGetErrorString(rc, C.byref(s))
        raise RuntimeError(f"{what}: CUDA driver error {rc} ({s.value.decode() if s.value else '?'})")


def available(system: str, algorithm: int, nt: int, ndo: int, rreg: int | None = None, sync: bool = False) -> bool:
    return _b.ref_cubin(system, algorithm, nt, ndo, rreg, sync).exists()


class ReferenceKernel:
    """One loaded reference kernel (system, algorithm, NT, NDO)."""

    def __init__(self, system: str, algorithm: int, nt: int, ndo: int = 0, rreg: int | None = None,
                 sync: bool = False):
        path = _b.ref_cubin(system, algorithm, nt, ndo, rreg, sync)
        self.sync = sync
        if not path.exists():
            raise FileNotFoundError(f"{path} not built (needs the reference checkout at build time)")
        cu = _driver()
        ctx = C.c_void_p()
        _ck(cu.cuCtxGetCurrent(C.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context: create a ProblemSolver on the device first")
        self.mod = C.c_void_p()
        _ck(cu.cuModuleLoad(C.byref(self.mod), str(path).encode()), f"cuModuleLoad({path.name})")
        n = C.c_uint()
        _ck(cu.cuModuleGetFunctionCount(C.byref(n), self.mod), "cuModuleGetFunctionCount")
        if n.value != 1:
            raise RuntimeError(f"{path.name}: expected one kernel, found {n.value}")
        funcs = (C.c_void_p * 1)()
        _ck(cu.cuModuleEnumerateFunctions(funcs, 1, self.mod), "cuModuleEnumerateFunctions")
        self.fn = C.c_void_p(funcs[0])
        self.system, self.algorithm, self.nt, self.ndo = system, algorithm, nt, ndo
        self._dev = []

    def close(self):
        cu = _driver()
        for p in self._dev:
            cu.cuMemFree_v2(p)
        self._dev = []
        if self.mod.value:
            cu.cuModuleUnload(self.mod)
            self.mod = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _upload(self, arr: np.ndarray) -> int:
        cu = _driver()
        arr = np.ascontiguousarray(arr)
        p = C.c_uint64()
        _ck(cu.cuMemAlloc_v2(C.byref(p), max(arr.nbytes, 16)), "cuMemAlloc")
        self._dev.append(p.value)
        if arr.nbytes:
            _ck(cu.cuMemcpyHtoD_v2(p.value, arr.ctypes.data, arr.nbytes), "cuMemcpyHtoD")
        return p.value

    def bind(self, solver, case, block: int = 64, prefer_shared: int = 1):
        """Prepare a launch on the device buffers of ``solver`` (holding ``case``)."""
        from mpgos_gb300.solver import Variable as V
        if solver.NT != self.nt or solver.NDO != self.ndo:
            raise ValueError("solver size does not match the compiled reference kernel")
        if block > 32 and not self.sync:
            raise ValueError("blocks of more than one warp need the cubin with the staging barrier (sync=True)")
        sd, ne = solver.SD, solver.NE
        pad = max(sd, ne, 1)
        tol = lambda v, dt: np.concatenate([np.asarray(v, dt), np.zeros(pad, dt)])[:pad]
        g = GlobalVariables(
            solver.device_ptr(V.TimeDomain), solver.device_ptr(V.ActualState), solver.device_ptr(V.ActualTime),
            solver.device_ptr(V.ControlParameters), solver.device_ptr(V.SharedParameters),
            solver.device_ptr(V.IntegerSharedParameters), solver.device_ptr(V.Accessories),
            solver.device_ptr(V.IntegerAccessories),
            self._upload(tol(case.rtol, np.float64)), self._upload(tol(case.atol, np.float64)),
            self._upload(tol(case.etol, np.float64)), self._upload(tol(case.edir, np.int32)),
            solver.device_ptr(V.DenseIndex), solver.device_ptr(V.DenseTime), solver.device_ptr(V.DenseState))
        n_active = case.n_active if case.n_active is not None else case.nt
        grid = (self.nt + block - 1) // block
        self.tc = ThreadConfiguration(grid, block, n_active)
        self.gv = g
        self.smu = SharedMemoryUsage(prefer_shared, 1 if self.algorithm == 1 else 0)
        o = case.options
        self.so = SolverOptions(o["initial_dt"], o["max_dt"], o["min_dt"], o["grow"], o["shrink"],
                                int(o["dense_freq"]), o["dense_min_dt"])
        self.grid, self.block = grid, block
        self.smem = prefer_shared * (solver.NSP * 8 + solver.NISP * 4)
        self.stream = solver.stream()
        self.params = (C.c_void_p * 4)(C.addressof(self.tc), C.addressof(self.gv), C.addressof(self.smu),
                                      C.addressof(self.so))

    def launch(self):
        _ck(_driver().cuLaunchKernel(self.fn, self.grid, 1, 1, self.block, 1, 1, self.smem, C.c_void_p(self.stream),
                                     self.params, None), "cuLaunchKernel")


def run_ref_gpu(case, block: int = 32, rreg: int | None = None, device: int = 0) -> dict:
    """Integrate ``case`` (all phases) with the reference kernel on the GPU."""
    from mpgos_gb300 import workloads as W
    with W.load_solver(case, mode=0, device=device) as s:
        s.SynchroniseDevice()
        with ReferenceKernel(case.system, case.algorithm, case.nt, case.ndo, rreg) as k:
            k.bind(s, case, block=block)
            for _ in range(case.phases):
                k.launch()
            s.SynchroniseDevice()
        return W.read_results(s)


def device_to_host(ptr: int, shape, dtype) -> np.ndarray:
    """Copy a device array (raw pointer) to a new host array (test helper)."""
    out = np.empty(shape, dtype=dtype)
    if out.nbytes:
        _ck(_driver().cuMemcpyDtoH_v2(out.ctypes.data, int(ptr), out.nbytes), "cuMemcpyDtoH")
    return out


# ---- coupled per-block solver -----------------------------------------------------
class CbThreadConfiguration(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("LogicalThreadsPerBlock", "NumberOfBlockLaunches", "ThreadPaddingPerBlock",
                                       "BlockSize", "GridSize", "TotalLogicalThreads")]


class CbGlobalVariables(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in (
        "d_TimeDomain", "d_ActualState", "d_ActualTime", "d_UnitParameters", "d_SystemParameters",
        "d_GlobalParameters", "d_IntegerGlobalParameters", "d_UnitAccessories", "d_IntegerUnitAccessories",
        "d_SystemAccessories", "d_IntegerSystemAccessories", "d_CouplingMatrix", "d_CouplingStrength",
        "d_CouplingIndex", "d_DenseOutputIndex", "d_DenseOutputTimeInstances", "d_DenseOutputStates",
        "d_RelativeTolerance", "d_AbsoluteTolerance", "d_EventTolerance", "d_EventDirection")]


class CbSharedMemoryUsage(C.Structure):
    _fields_ = [("GlobalVariables", C.c_bool), ("CouplingMatrices", C.c_bool), ("SingleCouplingMatrixSize", C.c_int),
                ("IsAdaptive", C.c_int)]


class CbSolverOptions(C.Structure):
    _fields_ = [("InitialTimeStep", C.c_double), ("ActiveSystems", C.c_int), ("MaximumTimeStep", C.c_double),
                ("MinimumTimeStep", C.c_double), ("TimeStepGrowLimit", C.c_double),
                ("TimeStepShrinkLimit", C.c_double), ("DenseOutputSaveFrequency", C.c_int),
                ("DenseOutputMinimumTimeStep", C.c_double)]


def coupled_available(system: str, algorithm: int, ns: int, tpb: int, spb: int, ndo: int) -> bool:
    return _b.ref_cb_cubin(system, algorithm, ns, tpb, spb, ndo).exists()


class CoupledReferenceKernel(ReferenceKernel):
    """The reference's coupled kernel for one (system, algorithm, NS, TPB,
    SPB, NDO): MultipleSystems_SingleBlockLaunch
    (CoupledSystmes_PerBlock_Solver.cuh:1507-2211), or the SingleSystem /
    MultipleBlockLaunches variants (:10, :786, :2214) where SPB and UPS > TPB
    select them, launched as the reference's Solve() does
    (CoupledSystems_PerBlock_Interface.cuh:1947-1966: grid ceil(NS/SPB),
    block TPB, thread configuration of :385-390, dynamic shared memory for the
    global parameters and, when shared, the coupling matrices, :540-544) on
    the device buffers of a GB300 ``CoupledProblemSolver``. Layouts without
    thread padding only (SPB*UPS a multiple of TPB, or SPB*UPS == TPB), where
    the reference's unit layout is the GB300 one."""

    def __init__(self, system: str, algorithm: int, ns: int, tpb: int, spb: int, ndo: int = 0):
        path = _b.ref_cb_cubin(system, algorithm, ns, tpb, spb, ndo)
        if not path.exists():
            raise FileNotFoundError(f"{path} not built (needs the reference checkout at build time)")
        cu = _driver()
        ctx = C.c_void_p()
        _ck(cu.cuCtxGetCurrent(C.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context: create a solver on the device first")
        self.mod = C.c_void_p()
        _ck(cu.cuModuleLoad(C.byref(self.mod), str(path).encode()), f"cuModuleLoad({path.name})")
        n = C.c_uint()
        _ck(cu.cuModuleGetFunctionCount(C.byref(n), self.mod), "cuModuleGetFunctionCount")
        if n.value != 1:
            raise RuntimeError(f"{path.name}: expected one kernel, found {n.value}")
        funcs = (C.c_void_p * 1)()
        _ck(cu.cuModuleEnumerateFunctions(funcs, 1, self.mod), "cuModuleEnumerateFunctions")
        self.fn = C.c_void_p(funcs[0])
        self.system, self.algorithm, self.ns, self.tpb, self.spb, self.ndo = system, algorithm, ns, tpb, spb, ndo
        self._dev = []

    def bind(self, solver, case, shared_global: int = 1, shared_coupling: int = 0):
        """Prepare a launch on the buffers of ``solver`` (holding ``case``);
        the defaults are the reference's (SharedGlobalVariables on,
        SharedCouplingMatrices off unless circular)."""
        from mpgos_gb300.capi import CbVariable as V
        ups = solver.UPS
        logical = self.spb * ups
        if solver.NS != self.ns or solver.NDO != self.ndo or logical % self.tpb or self.ns % self.spb:
            raise ValueError("solver shape does not match the compiled reference kernel (or needs thread padding)")
        if solver.CCI == 1:
            shared_coupling = 1  # the reference forces it (CoupledSystems_PerBlock_Interface.cuh:524-527)
        d = solver.device_ptr
        self.gv = CbGlobalVariables(
            d(V.TimeDomain), d(V.ActualState), d(V.ActualTime), d(V.UnitParameters), d(V.SystemParameters),
            d(V.GlobalParameters), d(V.IntegerGlobalParameters), d(V.UnitAccessories), d(V.IntegerUnitAccessories),
            d(V.SystemAccessories), d(V.IntegerSystemAccessories), d(V.CouplingMatrix), d(V.CouplingStrength),
            d(V.CouplingIndex), d(V.DenseIndex), d(V.DenseTime), d(V.DenseState),
            self._upload(np.asarray(case.rtol, np.float64)), self._upload(np.asarray(case.atol, np.float64)),
            self._upload(np.asarray(case.etol, np.float64)), self._upload(np.asarray(case.edir, np.int32)))
        grid = self.ns // self.spb
        self.tc = CbThreadConfiguration(logical, logical // self.tpb, 0, self.tpb, grid, self.ns * ups)
        self.smu = CbSharedMemoryUsage(bool(shared_global), bool(shared_coupling), solver.MAT,
                                       1 if self.algorithm == 1 else 0)
        o = case.options
        n_active = case.n_active if case.n_active is not None else case.ns
        self.so = CbSolverOptions(o["initial_dt"], n_active, o["max_dt"], o["min_dt"], o["grow"], o["shrink"],
                                  int(o["dense_freq"]), o["dense_min_dt"])
        self.grid, self.block = grid, self.tpb
        self.smem = shared_global * (solver.NGP * 8 + solver.NiGP * 4) + shared_coupling * solver.NC * solver.MAT * 8
        self.stream = solver.stream()
        self.params = (C.c_void_p * 4)(C.addressof(self.tc), C.addressof(self.gv), C.addressof(self.smu),
                                      C.addressof(self.so))


def run_ref_gpu_coupled(case, tpb: int, spb: int, device: int = 0, shared_coupling: int = 0) -> dict:
    """Integrate a ``CbCase`` (all phases) with the reference coupled kernel."""
    from mpgos_gb300 import coupled_workloads as CW
    with CW.load_coupled_solver(case, device=device) as s:
        s.SynchroniseDevice()
        with CoupledReferenceKernel(case.system, case.algorithm, case.ns, tpb, spb, case.ndo) as k:
            k.bind(s, case, shared_global=1, shared_coupling=shared_coupling)
            for _ in range(case.phases):
                k.launch()
            s.SynchroniseDevice()
        return CW.read_coupled_results(s)
