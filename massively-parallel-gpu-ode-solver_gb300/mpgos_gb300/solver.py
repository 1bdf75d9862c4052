"""Host-side mirror of the reference's per-thread solver object.

``ProblemSolver`` keeps the method names, argument meaning and index layout
of ``class ProblemSolver`` in
SourceCodes/SingleSystem_PerThread_Interface.cuh:117-208 (SolverOption,
SetHost, GetHost, SynchroniseFromHostToDevice, SynchroniseFromDeviceToHost,
Solve, InsertSynchronisationPoint, SynchroniseSolver, SynchroniseDevice,
Print), on top of the C-ABI of ``include/mpgos.h``. Where the reference calls
exit(1) on a bad index or option, this raises ``MpgosError``. The compile-time
template arguments of the reference (SD, NCP, ... come from the system plugin;
NT and NDO are constructor arguments here.

Beyond the reference: numpy views of the pinned host buffers (``host``), the
device pointers (``device_ptr``), CUDA-graph phase runs (``SolvePhases``),
event timing, status/step statistics and the autotuner.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import Algorithm, MpgosError, Option, Variable

# Reference enumerator names (SingleSystem_PerThread_Interface.cuh:33-62).
RK4, RKCK45 = Algorithm.RK4, Algorithm.RKCK45
(All, TimeDomain, ActualState, ActualTime, ControlParameters, SharedParameters, IntegerSharedParameters,
 Accessories, IntegerAccessories, DenseOutput, DenseIndex, DenseTime, DenseState) = (
    Variable.All, Variable.TimeDomain, Variable.ActualState, Variable.ActualTime, Variable.ControlParameters,
    Variable.SharedParameters, Variable.IntegerSharedParameters, Variable.Accessories, Variable.IntegerAccessories,
    Variable.DenseOutput, Variable.DenseIndex, Variable.DenseTime, Variable.DenseState)
(ThreadsPerBlock, InitialTimeStep, ActiveNumberOfThreads, MaximumTimeStep, MinimumTimeStep, TimeStepGrowLimit,
 TimeStepShrinkLimit, RelativeTolerance, AbsoluteTolerance, EventTolerance, EventDirection,
 DenseOutputMinimumTimeStep, DenseOutputSaveFrequency, PreferSharedMemory) = (
    Option.ThreadsPerBlock, Option.InitialTimeStep, Option.ActiveNumberOfThreads, Option.MaximumTimeStep,
    Option.MinimumTimeStep, Option.TimeStepGrowLimit, Option.TimeStepShrinkLimit, Option.RelativeTolerance,
    Option.AbsoluteTolerance, Option.EventTolerance, Option.EventDirection, Option.DenseOutputMinimumTimeStep,
    Option.DenseOutputSaveFrequency, Option.PreferSharedMemory)
KernelMode, MaximumAttempts = Option.KernelMode, Option.MaximumAttempts

_INDEXED_OPTIONS = {Option.RelativeTolerance, Option.AbsoluteTolerance, Option.EventTolerance, Option.EventDirection}
_INT_VARIABLES = {Variable.IntegerSharedParameters, Variable.IntegerAccessories, Variable.DenseIndex,
                  Variable.Status, Variable.AcceptedSteps, Variable.RejectedSteps}


class ProblemSolver:
    """One ensemble of NT instances of a compiled system on one GPU.

    ``system``    name of a system plugin (``libmpgos_<system>.so``)
    ``nt``        number of instances (the reference's NT template argument)
    ``ndo``       dense-output slots per instance (NDO)
    ``algorithm`` RK4 or RKCK45; ``precision`` "double" or "float"
    """

    def __init__(self, system: str, nt: int, ndo: int = 0, algorithm=RKCK45, precision: str = "double",
                 device: int = 0):
        self._lib = capi.runtime()
        pbytes = {"double": 8, "float": 4}[precision]
        self._table = capi.kernel_table(system, int(algorithm), pbytes)
        h = C.c_void_p()
        capi.check(self._lib.mpgos_pt_create(self._table, int(nt), int(ndo), int(device), C.byref(h)))
        self._h = h
        shp = capi.Shape()
        capi.check(self._lib.mpgos_pt_get_shape(h, C.byref(shp), None, None))
        self.system = system
        self.NT, self.NDO = int(nt), int(ndo)
        self.SD, self.NCP, self.NSP, self.NISP = shp.sd, shp.ncp, shp.nsp, shp.nisp
        self.NE, self.NA, self.NIA = shp.ne, shp.na, shp.nia
        self.algorithm = Algorithm(shp.algorithm)
        self.modes = shp.modes
        self.dtype = np.float64 if pbytes == 8 else np.float32
        self._views = {}

    # ---- lifetime -------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._views.clear()
            self._lib.mpgos_pt_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- SolverOption (:611-703) -------------------------------------------
    def SolverOption(self, option, *args):
        option = Option(option)
        if option in _INDEXED_OPTIONS:
            if len(args) != 2:
                raise MpgosError(1, f"SolverOption {option.name} needs (index, value)")
            index, value = args
        else:
            if len(args) != 1:
                raise MpgosError(1, f"SolverOption {option.name} needs exactly one value")
            index, value = 0, args[0]
        capi.check(self._lib.mpgos_pt_set_option(self._h, int(option), int(index), float(value)))

    def GetOption(self, option, index: int = 0) -> float:
        v = C.c_double()
        capi.check(self._lib.mpgos_pt_get_option(self._h, int(Option(option)), int(index), C.byref(v)))
        return v.value

    # ---- host buffers ------------------------------------------------------
    def _fields(self, var: Variable) -> int:
        return {
            Variable.TimeDomain: 2, Variable.ActualState: self.SD, Variable.ActualTime: 1,
            Variable.ControlParameters: self.NCP, Variable.Accessories: self.NA,
            Variable.IntegerAccessories: self.NIA, Variable.DenseIndex: 1, Variable.DenseTime: self.NDO,
            Variable.DenseState: self.NDO * self.SD, Variable.Status: 1, Variable.AcceptedSteps: 1,
            Variable.RejectedSteps: 1,
        }.get(var, 0)

    def host(self, var) -> np.ndarray:
        """numpy view of the pinned host buffer of ``var``.

        Per-instance arrays are shaped [fields, NT] (dense state [NDO, SD, NT]);
        shared parameters are 1-D.
        """
        var = Variable(var)
        if var in self._views:
            return self._views[var]
        ptr, cnt = C.c_void_p(), C.c_int64()
        capi.check(self._lib.mpgos_pt_host_buffer(self._h, int(var), C.byref(ptr), C.byref(cnt)))
        dt = np.int32 if var in _INT_VARIABLES else self.dtype
        n = int(cnt.value)
        ctype = C.c_int32 if dt == np.int32 else (C.c_double if dt == np.float64 else C.c_float)
        if n == 0:
            arr = np.zeros(0, dtype=dt)
        else:
            arr = np.ctypeslib.as_array((ctype * n).from_address(ptr.value))
        if var in (Variable.SharedParameters, Variable.IntegerSharedParameters):
            view = arr
        elif var == Variable.DenseState:
            view = arr.reshape(self.NDO, self.SD, self.NT)
        else:
            view = arr.reshape(self._fields(var), self.NT)
        self._views[var] = view
        return view

    def device_ptr(self, var) -> int:
        ptr, cnt = C.c_void_p(), C.c_int64()
        capi.check(self._lib.mpgos_pt_device_buffer(self._h, int(Variable(var)), C.byref(ptr), C.byref(cnt)))
        return int(ptr.value or 0)

    # ---- SetHost / GetHost (:706-1080) ---------------------------------------
    def _bound(self, fn, what, value, lo, hi):
        if value < lo or value > hi:
            raise MpgosError(1, f"{fn}: {what} index {value} outside {lo}..{hi}")

    def _locate(self, fn, args):
        """Resolve the four overloads of SetHost/GetHost to (array, flat index)."""
        if len(args) >= 1 and isinstance(args[0], Variable):
            var, serial = args[0], int(args[1])                    # global scope
            if var == Variable.SharedParameters:
                self._bound(fn, "SharedParameters", serial, 0, self.NSP - 1)
            elif var == Variable.IntegerSharedParameters:
                self._bound(fn, "IntegerSharedParameters", serial, 0, self.NISP - 1)
            else:
                raise MpgosError(1, f"{fn}: variable {var.name} needs a different argument configuration")
            return self.host(var), serial, 2
        pid, var = int(args[0]), Variable(args[1])
        self._bound(fn, "ProblemNumber", pid, 0, self.NT - 1)
        rest = args[2:]
        if var == Variable.DenseState:                                # (pid, var, comp, step[, value])
            comp, step = int(rest[0]), int(rest[1])
            self._bound(fn, "DenseState/ComponentNumber", comp, 0, self.SD - 1)
            self._bound(fn, "DenseState/TimeStepNumber", step, 0, self.NDO - 1)
            return self.host(var).reshape(-1), pid + comp * self.NT + step * self.NT * self.SD, 4
        if var in (Variable.ActualTime, Variable.DenseIndex):       # system scope
            return self.host(var).reshape(-1), pid, 2
        limits = {Variable.TimeDomain: 2, Variable.ActualState: self.SD, Variable.ControlParameters: self.NCP,
                  Variable.Accessories: self.NA, Variable.IntegerAccessories: self.NIA, Variable.DenseTime: self.NDO}
        if var not in limits:
            raise MpgosError(1, f"{fn}: variable {var.name} needs a different argument configuration")
        serial = int(rest[0])
        self._bound(fn, var.name, serial, 0, limits[var] - 1)
        return self.host(var).reshape(-1), pid + serial * self.NT, 3

    def SetHost(self, *args):
        arr, idx, nidx = self._locate("SetHost", args)
        if len(args) != nidx + 1:
            raise MpgosError(1, "SetHost: wrong number of arguments")
        value = args[-1]
        if len(args) == 3 and not isinstance(args[0], Variable) and Variable(args[1]) == Variable.DenseIndex:
            self._bound("SetHost", "DenseIndex-Value", int(value), 0, self.NDO - 1)
        arr[idx] = value

    def GetHost(self, *args):
        arr, idx, nidx = self._locate("GetHost", args)
        if len(args) != nidx:
            raise MpgosError(1, "GetHost: wrong number of arguments")
        return arr[idx].item()

    # ---- synchronisation / solve (:833-965, :1279-1312) --------------------
    def SynchroniseFromHostToDevice(self, var=Variable.All):
        capi.check(self._lib.mpgos_pt_sync_h2d(self._h, int(Variable(var))))

    def SynchroniseFromDeviceToHost(self, var=Variable.All):
        capi.check(self._lib.mpgos_pt_sync_d2h(self._h, int(Variable(var))))

    def Solve(self):
        capi.check(self._lib.mpgos_pt_solve(self._h))

    def SolvePhases(self, n_phases: int, stream_accessory: int = -1, phase_output_ptr: int = 0):
        """n_phases Solve() calls captured once into a CUDA graph and replayed."""
        capi.check(self._lib.mpgos_pt_solve_phases(self._h, int(n_phases), int(stream_accessory),
                                                   C.c_void_p(phase_output_ptr or None)))

    def InsertSynchronisationPoint(self):
        capi.check(self._lib.mpgos_pt_insert_sync_point(self._h))

    def SynchroniseSolver(self):
        capi.check(self._lib.mpgos_pt_sync_solver(self._h))

    def SynchroniseDevice(self):
        capi.check(self._lib.mpgos_pt_sync_device(self._h))

    # ---- extensions ----------------------------------------------------------
    def stream(self) -> int:
        s = C.c_void_p()
        capi.check(self._lib.mpgos_pt_stream(self._h, C.byref(s)))
        return int(s.value or 0)

    def launch_config(self):
        g, b, m = C.c_int(), C.c_int(), C.c_int32()
        capi.check(self._lib.mpgos_pt_launch_config(self._h, C.byref(g), C.byref(b), C.byref(m)))
        return g.value, b.value, m.value

    def timer_start(self):
        capi.check(self._lib.mpgos_pt_timer_start(self._h))

    def timer_stop(self) -> float:
        ms = C.c_float()
        capi.check(self._lib.mpgos_pt_timer_stop(self._h, C.byref(ms)))
        return float(ms.value)

    def autotune(self, fast_control: bool = True, cache_path: str | None = None, arithmetic: int | None = None):
        """Pick block size and mapping by timing; ``arithmetic`` (a MPGOS_MODE_*
        value: 0, MODE_FAST_CONTROL, MODE_DF_STAGE or MODE_SPLIT) overrides
        ``fast_control``."""
        arith = int(bool(fast_control)) if arithmetic is None else int(arithmetic)
        capi.check(self._lib.mpgos_pt_autotune(self._h, arith, cache_path.encode() if cache_path else None))
        return self.launch_config()

    def checkpoint_save(self):
        capi.check(self._lib.mpgos_pt_checkpoint_save(self._h))

    def checkpoint_restore(self):
        capi.check(self._lib.mpgos_pt_checkpoint_restore(self._h))

    def SolveRecord(self, max_steps: int, segment: int = 32):
        """One Solve() that records the adjoint tape (frozen step sizes and a
        checkpoint every ``segment`` accepted steps)."""
        capi.check(self._lib.mpgos_pt_solve_record(self._h, int(max_steps), int(segment)))

    def SolveRecordStatic(self, max_steps: int, segment: int = 32):
        """SolveRecord into the runtime's static device scratch
        (mpgos_pt_solve_record_static): no device allocation; at most
        MPGOS_STATIC_TAPE_BYTES of tape; one scratch per device and process,
        so concurrent recordings race."""
        capi.check(self._lib.mpgos_pt_solve_record_static(self._h, int(max_steps), int(segment)))

    def Adjoint(self, dLdxT_ptr: int, dLdx0_ptr: int, dLdp_ptr: int):
        """Reverse pass over the recorded tape; device pointers, FP64,
        [SD][NT] in, [SD][NT] and [NCP][NT] out."""
        capi.check(self._lib.mpgos_pt_adjoint(self._h, C.c_void_p(dLdxT_ptr), C.c_void_p(dLdx0_ptr),
                                              C.c_void_p(dLdp_ptr or None)))

    def DenseInterpolate(self, times_ptr: int, n_times: int, out_ptr: int):
        """Cubic Hermite interpolation of the device dense output at n_times
        requested times (device pointers, FP64): out [n_times][SD][NT]."""
        capi.check(self._lib.mpgos_pt_dense_interpolate(self._h, C.c_void_p(times_ptr), int(n_times),
                                                        C.c_void_p(out_ptr)))

    def tape_info(self):
        t = capi.Tape()
        capi.check(self._lib.mpgos_pt_tape_info(self._h, C.byref(t)))
        return t

    def set_mode(self, mode: int):
        self.SolverOption(Option.KernelMode, mode)

    # ---- Print (:1083-1276): same file names and number format ---------------
    def Print(self, var, thread_id: int | None = None, directory: str = "."):
        """Write a variable to the reference's file (SingleSystem_PerThread_Interface.cuh:1083-1276):
        <Variable>InSolverObject.txt, or DenseOutput_<thread>.txt."""
        import os
        from . import textout as T
        var = Variable(var)
        if thread_id is None:
            names = {Variable.TimeDomain: "TimeDomain", Variable.ActualState: "ActualState",
                     Variable.ActualTime: "ActualTime", Variable.ControlParameters: "ControlParameters",
                     Variable.SharedParameters: "SharedParameters",
                     Variable.IntegerSharedParameters: "IntegerSharedParameters",
                     Variable.Accessories: "Accessories", Variable.IntegerAccessories: "IntegerAccessories"}
            if var not in names:
                raise MpgosError(1, f"Print: variable {var.name} needs a different argument configuration")
            T.general(os.path.join(directory, f"{names[var]}InSolverObject.txt"), np.atleast_2d(self.host(var)))
            return
        if var != Variable.DenseOutput:
            raise MpgosError(1, f"Print: variable {var.name} needs a different argument configuration")
        self._bound("Print", "Thread", thread_id, 0, self.NT - 1)
        tid = int(thread_id)
        z = lambda n, v: self.host(v) if n else np.zeros((0, self.NT))
        T.perthread_dense(os.path.join(directory, f"DenseOutput_{tid}.txt"), tid, z(self.NCP, ControlParameters),
                          self.host(SharedParameters).ravel() if self.NSP else [],
                          self.host(IntegerSharedParameters).ravel() if self.NISP else [],
                          z(self.NA, Accessories), z(self.NIA, IntegerAccessories),
                          int(self.host(DenseIndex)[0, tid]) if self.NDO else 0,
                          self.host(DenseTime) if self.NDO else np.zeros((0, self.NT)),
                          self.host(DenseState) if self.NDO else np.zeros((0, self.SD, self.NT)))
