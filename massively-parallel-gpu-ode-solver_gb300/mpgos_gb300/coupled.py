"""Host-side mirror of the reference's coupled per-block solver object.

``CoupledProblemSolver`` keeps the method names, argument meaning and index
layout of ``class ProblemSolver`` in
SourceCodes/CoupledSystems_PerBlock_Interface.cuh:135-248 (SolverOption,
the six SetHost/GetHost overloads, SynchroniseFromHostToDevice,
SynchroniseFromDeviceToHost, Solve, InsertSynchronisationPoint,
SynchroniseSolver, SynchroniseDevice, Print) on top of the ``mpgos_cb_*``
C-ABI of ``include/mpgos.h``. The reference's compile-time arguments UPS,
UD, NC, CBW, CCI, NUP, NSP, NGP, NiGP, NUA, NiUA, NSA, NiSA, NE come from the
coupled-system plugin; NS and NDO are constructor arguments. TPB and SPB
(threads and systems per block) have no meaning here: one warp integrates
one system, ``WarpsPerBlock`` systems share a CTA.

Unit-scope arrays are laid out [field][NS*UPS] with unit u of system s at
s*UPS + u, which is the reference's layout whenever its thread padding is
zero (SPB*UPS a multiple of TPB, NS a multiple of SPB); system-scope arrays
are [field][NS]. The coupling matrix is set element by element in full
(row, col) form and stored in the plugin's compressed storage (full,
banded, circular-banded or full circular) exactly as the reference's
SetHost does (CoupledSystems_PerBlock_Interface.cuh:993-1080); the full form
is kept on the host for GetHost and Print.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import Algorithm, CbOption, CbVariable, MpgosError

_INDEXED = {CbOption.RelativeTolerance, CbOption.AbsoluteTolerance, CbOption.EventTolerance, CbOption.EventDirection}
_INT_VARS = {CbVariable.IntegerGlobalParameters, CbVariable.IntegerUnitAccessories,
             CbVariable.IntegerSystemAccessories, CbVariable.CouplingIndex, CbVariable.DenseIndex,
             CbVariable.Status, CbVariable.AcceptedSteps, CbVariable.RejectedSteps}
_UNIT = {CbVariable.ActualState: "UD", CbVariable.UnitParameters: "NUP", CbVariable.UnitAccessories: "NUA",
         CbVariable.IntegerUnitAccessories: "NiUA"}
_SYSTEM = {CbVariable.TimeDomain: "TWO", CbVariable.SystemParameters: "NSP", CbVariable.SystemAccessories: "NSA",
           CbVariable.IntegerSystemAccessories: "NiSA", CbVariable.CouplingStrength: "NC",
           CbVariable.DenseTime: "NDO"}
_GLOBAL = {CbVariable.GlobalParameters: "NGP", CbVariable.IntegerGlobalParameters: "NiGP",
           CbVariable.CouplingIndex: "NC"}


def matrix_entries(ups: int, cbw: int, cci: int) -> int:
    """Stored entries of one coupling matrix
    (CoupledSystems_PerBlock_Interface.cuh:426-438)."""
    if cci == 0:
        return ups * ups if cbw == 0 else ups * (2 * cbw + 1)
    return ups if cbw == 0 else 2 * cbw + 1


def matrix_slot(ups: int, cbw: int, cci: int, coupling: int, row: int, col: int) -> int:
    """Index of entry (row, col) of coupling matrix ``coupling`` in the stored
    form (CoupledSystems_PerBlock_Interface.cuh:1003-1064): full matrices
    column-major, banded ones by shifted diagonal (column col - row + CBW,
    wrapped into 0..UPS-1), circular ones without the row. Raises
    ``MpgosError`` for an entry the storage cannot hold."""
    if cci == 0 and cbw == 0:
        return row + col * ups + coupling * ups * ups
    mcol = col - row + cbw
    if mcol >= ups:
        mcol -= ups
    if mcol < 0:
        mcol += ups
    width = 2 * cbw + 1 if cbw > 0 else ups
    if mcol < 0 or mcol >= width:
        raise MpgosError(1, f"SetHost: Coupling Matrix Shifted Diagonal index {mcol} outside 0..{width - 1}")
    if cci == 0:
        return row + mcol * ups + coupling * ups * width
    return mcol + coupling * width


def store_matrices(full: np.ndarray, cbw: int, cci: int) -> np.ndarray:
    """Stored form of full coupling matrices ``full`` [NC][UPS][UPS]: every
    non-zero (row, col) placed by ``matrix_slot``; for circular storages the
    last row written wins, as with element-wise SetHost in row order."""
    full = np.asarray(full, dtype=np.float64)
    nc, ups, _ = full.shape
    out = np.zeros(nc * matrix_entries(ups, cbw, cci))
    if cci == 0 and cbw == 0:
        return np.ascontiguousarray(full.transpose(0, 2, 1).reshape(-1))
    for c in range(nc):
        for r, col in zip(*np.nonzero(full[c])):
            out[matrix_slot(ups, cbw, cci, c, int(r), int(col))] = full[c, r, col]
    return out


class CoupledProblemSolver:
    """NS coupled systems of UPS units each, on one GPU.

    ``system``    coupled-system plugin name (``libmpgos_<system>.so``)
    ``ns``        number of systems (the reference's NS)
    ``ndo``       dense-output slots per system (NDO)
    """

    def __init__(self, system: str, ns: int, ndo: int = 0, algorithm=Algorithm.RKCK45, precision: str = "double",
                 device: int = 0, tpb: int | None = None, spb: int | None = None):
        # tpb / spb: the reference's launch shape; used only to lay out the
        # unit-scope files of Print in its padded rows (one warp integrates
        # one system here whatever the shape)
        self.print_tpb, self.print_spb = tpb, spb
        self._lib = capi.runtime()
        pbytes = {"double": 8, "float": 4}[precision]
        self._table = capi.coupled_kernel_table(system, int(algorithm), pbytes)
        h = C.c_void_p()
        capi.check(self._lib.mpgos_cb_create(self._table, int(ns), int(ndo), int(device), C.byref(h)))
        self._h = h
        s = capi.CbShape()
        capi.check(self._lib.mpgos_cb_get_shape(h, C.byref(s), None, None))
        self.system = system
        self.NS, self.NDO = int(ns), int(ndo)
        self.UPS, self.UD, self.NC, self.CBW, self.CCI = s.ups, s.ud, s.nc, s.cbw, s.cci
        self.NUP, self.NSP, self.NGP, self.NiGP = s.nup, s.nsp, s.ngp, s.nigp
        self.NUA, self.NiUA, self.NSA, self.NiSA, self.NE = s.nua, s.niua, s.nsa, s.nisa, s.ne
        self.MAT = s.matrix_entries
        self.algorithm = Algorithm(s.algorithm)
        self.dtype = np.float64 if pbytes == 8 else np.float32
        self.NU = self.NS * self.UPS
        self._views = {}
        self._full_matrix = np.zeros((max(self.NC, 1), self.UPS, self.UPS), dtype=self.dtype)

    # ---- lifetime -------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._views.clear()
            self._lib.mpgos_cb_destroy(self._h)
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

    # ---- SolverOption (:760-860) ---------------------------------------------
    def SolverOption(self, option, *args):
        option = CbOption(option)
        if option in _INDEXED:
            if len(args) != 2:
                raise MpgosError(1, f"SolverOption {option.name} needs (index, value)")
            index, value = args
        else:
            if len(args) != 1:
                raise MpgosError(1, f"SolverOption {option.name} needs exactly one value")
            index, value = 0, args[0]
        capi.check(self._lib.mpgos_cb_set_option(self._h, int(option), int(index), float(value)))

    # ---- host buffers ------------------------------------------------------
    def _limit(self, name: str) -> int:
        return {"TWO": 2, "UD": self.UD, "NUP": self.NUP, "NUA": self.NUA, "NiUA": self.NiUA, "NSP": self.NSP,
                "NSA": self.NSA, "NiSA": self.NiSA, "NC": self.NC, "NDO": self.NDO, "NGP": self.NGP,
                "NiGP": self.NiGP}[name]

    def host(self, var) -> np.ndarray:
        """numpy view of the pinned host buffer of ``var``: unit scope
        [fields, NS*UPS], system scope [fields, NS], dense state
        [NDO, UD, NS*UPS], global scope and the stored coupling matrices 1-D."""
        var = CbVariable(var)
        if var in self._views:
            return self._views[var]
        ptr, cnt = C.c_void_p(), C.c_int64()
        capi.check(self._lib.mpgos_cb_host_buffer(self._h, int(var), C.byref(ptr), C.byref(cnt)))
        dt = np.int32 if var in _INT_VARS else self.dtype
        n = int(cnt.value)
        ctype = C.c_int32 if dt == np.int32 else (C.c_double if dt == np.float64 else C.c_float)
        arr = np.zeros(0, dtype=dt) if n == 0 else np.ctypeslib.as_array((ctype * n).from_address(ptr.value))
        if var in _UNIT:
            view = arr.reshape(self._limit(_UNIT[var]), self.NU)
        elif var in _SYSTEM:
            view = arr.reshape(self._limit(_SYSTEM[var]), self.NS)
        elif var == CbVariable.DenseState:
            view = arr.reshape(self.NDO, self.UD, self.NU)
        elif var in (CbVariable.ActualTime, CbVariable.DenseIndex, CbVariable.Status, CbVariable.AcceptedSteps,
                     CbVariable.RejectedSteps):
            view = arr.reshape(self.NS)
        else:
            view = arr
        self._views[var] = view
        return view

    def device_ptr(self, var) -> int:
        ptr, cnt = C.c_void_p(), C.c_int64()
        capi.check(self._lib.mpgos_cb_device_buffer(self._h, int(CbVariable(var)), C.byref(ptr), C.byref(cnt)))
        return int(ptr.value or 0)

    # ---- SetHost / GetHost (:870-1145, :1280-1530) ------------------------
    @staticmethod
    def _bound(fn, what, value, lo, hi):
        if value < lo or value > hi:
            raise MpgosError(1, f"{fn}: {what} index {value} outside {lo}..{hi}")

    def _locate(self, fn, args):
        """Resolve the six overloads to (flat array, index, arguments used)."""
        V = CbVariable
        if isinstance(args[0], V):                                           # global scope
            var, serial = args[0], int(args[1])
            if var not in _GLOBAL:
                raise MpgosError(1, f"{fn}: variable {var.name} needs a different argument configuration")
            self._bound(fn, var.name, serial, 0, self._limit(_GLOBAL[var]) - 1)
            return self.host(var).reshape(-1), serial, 2
        if isinstance(args[1], V):
            a0, var = int(args[0]), args[1]
            if var == V.CouplingMatrix:                                        # (coupling, var, row, col)
                row, col = int(args[2]), int(args[3])
                self._bound(fn, "CouplingNumber", a0, 0, self.NC - 1)
                self._bound(fn, "Coupling Matrix Row", row, 0, self.UPS - 1)
                self._bound(fn, "Coupling Matrix Col", col, 0, self.UPS - 1)
                return ("matrix", a0, row, col), matrix_slot(self.UPS, self.CBW, self.CCI, a0, row, col), 4
            self._bound(fn, "SystemNumber", a0, 0, self.NS - 1)
            if var in (V.DenseIndex, V.ActualTime):                            # (system, var)
                return self.host(var).reshape(-1), a0, 2
            if var not in _SYSTEM:
                raise MpgosError(1, f"{fn}: variable {var.name} needs a different argument configuration")
            serial = int(args[2])                                              # (system, var, serial)
            self._bound(fn, var.name, serial, 0, self._limit(_SYSTEM[var]) - 1)
            return self.host(var).reshape(-1), a0 + serial * self.NS, 3
        sysn, unit, var = int(args[0]), int(args[1]), V(args[2])
        self._bound(fn, "SystemNumber", sysn, 0, self.NS - 1)
        self._bound(fn, "UnitNumber", unit, 0, self.UPS - 1)
        g = sysn * self.UPS + unit
        if var == V.DenseState:                                                # (system, unit, var, comp, slot)
            comp, slot = int(args[3]), int(args[4])
            self._bound(fn, "ComponentNumber in dense state", comp, 0, self.UD - 1)
            self._bound(fn, "DenseState", slot, 0, self.NDO - 1)
            return self.host(var).reshape(-1), g + comp * self.NU + slot * self.NU * self.UD, 5
        if var not in _UNIT:
            raise MpgosError(1, f"{fn}: variable {var.name} needs a different argument configuration")
        serial = int(args[3])                                                  # (system, unit, var, serial)
        self._bound(fn, var.name, serial, 0, self._limit(_UNIT[var]) - 1)
        return self.host(var).reshape(-1), g + serial * self.NU, 4

    def SetHost(self, *args):
        arr, idx, nargs = self._locate("SetHost", args)
        if len(args) != nargs + 1:
            raise MpgosError(1, "SetHost: wrong number of arguments")
        value = args[-1]
        if isinstance(arr, tuple):
            _, cpl, row, col = arr
            self._full_matrix[cpl, row, col] = value
            self.host(CbVariable.CouplingMatrix)[idx] = value
            return
        arr[idx] = value

    def GetHost(self, *args):
        arr, idx, nargs = self._locate("GetHost", args)
        if len(args) != nargs:
            raise MpgosError(1, "GetHost: wrong number of arguments")
        if isinstance(arr, tuple):
            _, cpl, row, col = arr
            return self._full_matrix[cpl, row, col].item()
        return arr[idx].item()

    def SetCouplingMatrix(self, coupling: int, full: np.ndarray):
        """Whole-matrix form of SetHost(coupling, CouplingMatrix, row, col, v)
        over every non-zero (row, col) of the full UPS x UPS matrix; a
        non-zero entry outside a banded storage is an error, as in SetHost."""
        full = np.asarray(full, dtype=self.dtype)
        if full.shape != (self.UPS, self.UPS):
            raise MpgosError(1, f"coupling matrix must be {self.UPS}x{self.UPS}")
        self._bound("SetCouplingMatrix", "CouplingNumber", coupling, 0, self.NC - 1)
        n = self.MAT
        stored = store_matrices(full[None], self.CBW, self.CCI)
        self.host(CbVariable.CouplingMatrix)[coupling * n:(coupling + 1) * n] = stored
        self._full_matrix[coupling] = full

    # ---- synchronisation and solve ------------------------------------------
    def SynchroniseFromHostToDevice(self, var):
        capi.check(self._lib.mpgos_cb_sync_h2d(self._h, int(CbVariable(var))))

    def SynchroniseFromDeviceToHost(self, var):
        capi.check(self._lib.mpgos_cb_sync_d2h(self._h, int(CbVariable(var))))

    def Solve(self):
        capi.check(self._lib.mpgos_cb_solve(self._h))

    def InsertSynchronisationPoint(self):
        capi.check(self._lib.mpgos_cb_insert_sync_point(self._h))

    def SynchroniseSolver(self):
        capi.check(self._lib.mpgos_cb_sync_solver(self._h))

    def SynchroniseDevice(self):
        self.InsertSynchronisationPoint()
        self.SynchroniseSolver()

    def timer_start(self):
        capi.check(self._lib.mpgos_cb_timer_start(self._h))

    def timer_stop(self) -> float:
        ms = C.c_float()
        capi.check(self._lib.mpgos_cb_timer_stop(self._h, C.byref(ms)))
        return float(ms.value)

    def stream(self) -> int:
        p = C.c_void_p()
        capi.check(self._lib.mpgos_cb_stream(self._h, C.byref(p)))
        return int(p.value or 0)

    def checkpoint_save(self):
        capi.check(self._lib.mpgos_cb_checkpoint_save(self._h))

    def checkpoint_restore(self):
        capi.check(self._lib.mpgos_cb_checkpoint_restore(self._h))

    def SolveRecord(self, max_steps: int, segment: int = 32):
        """One Solve() that records the adjoint tape (frozen step sizes and a
        checkpoint of every unit every ``segment`` accepted steps)."""
        capi.check(self._lib.mpgos_cb_solve_record(self._h, int(max_steps), int(segment)))

    def Adjoint(self, dLdxT_ptr: int, dLdx0_ptr: int, dLdsp_ptr: int):
        """Reverse pass over the recorded tape; device pointers, FP64:
        [UD][NS*UPS] in, [UD][NS*UPS] and [NSP][NS] out."""
        capi.check(self._lib.mpgos_cb_adjoint(self._h, C.c_void_p(dLdxT_ptr), C.c_void_p(dLdx0_ptr),
                                              C.c_void_p(dLdsp_ptr or None)))

    def tape_info(self):
        t = capi.Tape()
        capi.check(self._lib.mpgos_cb_tape_info(self._h, C.byref(t)))
        return t

    def set_mode(self, mode: int):
        self.SolverOption(CbOption.KernelMode, int(mode))

    def Print(self, var, serial: int | None = None, directory: str = "."):
        """Write a variable to the reference's file (CoupledSystems_PerBlock_Interface.cuh:1808-1945):
        <Variable>InSolverObject.txt for the unit, system and global scope,
        CouplingMatrixInSolverObject_<serial>.txt, DenseOutput_<serial>.txt."""
        import os
        from . import textout as T
        V = CbVariable
        var = V(var)
        path = lambda name: os.path.join(directory, name)
        if serial is not None:
            if var == V.CouplingMatrix:
                self._bound("Print", "CouplingMatrix", serial, 0, self.NC - 1)
                T.system_scope(path(f"CouplingMatrixInSolverObject_{serial}.txt"), self._full_matrix[serial].T)
            elif var == V.DenseOutput:
                self._bound("Print", "DenseOutput", serial, 0, self.NS - 1)
                h = lambda x, n: self.host(x) if n else np.zeros((0, self.NS * self.UPS))
                hs = lambda x, n: self.host(x) if n else np.zeros((0, self.NS))
                T.coupled_dense(path(f"DenseOutput_{serial}.txt"), serial, self.UPS, h(V.UnitParameters, self.NUP),
                                h(V.UnitAccessories, self.NUA), h(V.IntegerUnitAccessories, self.NiUA),
                                hs(V.SystemParameters, self.NSP), hs(V.SystemAccessories, self.NSA),
                                hs(V.IntegerSystemAccessories, self.NiSA),
                                self.host(V.GlobalParameters) if self.NGP else [],
                                self.host(V.IntegerGlobalParameters) if self.NiGP else [],
                                int(self.host(V.DenseIndex)[serial]) if self.NDO else 0,
                                self.host(V.DenseTime) if self.NDO else np.zeros((0, self.NS)),
                                self.host(V.DenseState) if self.NDO else np.zeros((0, self.UD, self.NS * self.UPS)))
            else:
                raise MpgosError(1, f"Print: variable {var.name} needs a different argument configuration")
            return
        names = {V.TimeDomain: "TimeDomain", V.ActualTime: "ActualTime", V.ActualState: "ActualState",
                 V.UnitParameters: "UnitParameters", V.SystemParameters: "SystemParameters",
                 V.GlobalParameters: "GlobalParameters", V.IntegerGlobalParameters: "IntegerGlobalParameters",
                 V.UnitAccessories: "UnitAccessories", V.IntegerUnitAccessories: "IntegerUnitAccessories",
                 V.SystemAccessories: "SystemAccessories", V.IntegerSystemAccessories: "IntegerSystemAccessories",
                 V.CouplingStrength: "CouplingStrength", V.CouplingIndex: "CouplingIndex"}
        if var not in names:
            raise MpgosError(1, f"Print: variable {var.name} needs a different argument configuration")
        f = path(f"{names[var]}InSolverObject.txt")
        data = np.atleast_2d(self.host(var))
        if var in _UNIT:
            T.unit_scope(f, data, self.NS, self.UPS, self.print_tpb, self.print_spb)
        else:
            T.system_scope(f, data)
