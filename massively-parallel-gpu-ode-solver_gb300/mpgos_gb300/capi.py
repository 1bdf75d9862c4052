"""ctypes binding of the C-ABI declared in ``include/mpgos.h``.

The runtime library and the system plugins are loaded from the in-tree build
directory; there is no fallback of any kind: if a library is missing or a call
fails, an exception is raised.
"""
from __future__ import annotations

import ctypes as C
from enum import IntEnum
from pathlib import Path

from . import build as _build


class MpgosError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"[mpgos status {code}] {message}")
        self.code = code


# ---- enums of include/mpgos.h (reference names in solver.py) ---------------
class Algorithm(IntEnum):
    RK4 = 0
    RKCK45 = 1


class Variable(IntEnum):
    All = 0
    TimeDomain = 1
    ActualState = 2
    ActualTime = 3
    ControlParameters = 4
    SharedParameters = 5
    IntegerSharedParameters = 6
    Accessories = 7
    IntegerAccessories = 8
    DenseOutput = 9
    DenseIndex = 10
    DenseTime = 11
    DenseState = 12
    Status = 32
    AcceptedSteps = 33
    RejectedSteps = 34


class Option(IntEnum):
    ThreadsPerBlock = 0
    InitialTimeStep = 1
    ActiveNumberOfThreads = 2
    MaximumTimeStep = 3
    MinimumTimeStep = 4
    TimeStepGrowLimit = 5
    TimeStepShrinkLimit = 6
    RelativeTolerance = 7
    AbsoluteTolerance = 8
    EventTolerance = 9
    EventDirection = 10
    DenseOutputMinimumTimeStep = 11
    DenseOutputSaveFrequency = 12
    PreferSharedMemory = 13
    KernelMode = 32
    MaximumAttempts = 33
    InstancesPerThread = 34
    WarpReconverge = 35
    OutlineRhs = 36
    WorkOrder = 37


MODE_PLAIN = 0
MODE_FAST_CONTROL = 1
MODE_PERSISTENT = 2
MODE_FP32_STAGE = 4
MODE_DF_STAGE = 16
MODE_SPLIT = 128
MODE_CHOSEN = MODE_FAST_CONTROL | MODE_PERSISTENT

INSTANCE_OK = 0
INSTANCE_NONFINITE = 1
INSTANCE_MINIMUM_STEP = 2
INSTANCE_EVENT_OMITTED = 4
INSTANCE_ATTEMPT_LIMIT = 8
INSTANCE_TAPE_OVERFLOW = 16
INSTANCE_RANGE = 32

ABI_VERSION = 2
STATIC_TAPE_BYTES = 16 * 1024 * 1024  # MPGOS_STATIC_TAPE_BYTES of mpgos.h


# Coupled per-block solver (CoupledSystems_PerBlock_Interface.cuh:33-66).
class CbVariable(IntEnum):
    All = 0
    TimeDomain = 1
    ActualTime = 2
    ActualState = 3
    UnitParameters = 4
    SystemParameters = 5
    GlobalParameters = 6
    IntegerGlobalParameters = 7
    UnitAccessories = 8
    IntegerUnitAccessories = 9
    SystemAccessories = 10
    IntegerSystemAccessories = 11
    CouplingMatrix = 12
    CouplingStrength = 13
    CouplingIndex = 14
    DenseOutput = 15
    DenseIndex = 16
    DenseTime = 17
    DenseState = 18
    Status = 32
    AcceptedSteps = 33
    RejectedSteps = 34


class CbOption(IntEnum):
    InitialTimeStep = 0
    ActiveSystems = 1
    MaximumTimeStep = 2
    MinimumTimeStep = 3
    TimeStepGrowLimit = 4
    TimeStepShrinkLimit = 5
    RelativeTolerance = 6
    AbsoluteTolerance = 7
    EventTolerance = 8
    EventDirection = 9
    DenseOutputSaveFrequency = 10
    DenseOutputMinimumTimeStep = 11
    SharedGlobalVariables = 12
    SharedCouplingMatrices = 13
    KernelMode = 32
    MaximumAttempts = 33
    WarpsPerBlock = 34


class CbShape(C.Structure):
    _fields_ = [(n, C.c_int32) for n in
                ("ups", "ud", "nc", "cbw", "cci", "nup", "nsp", "ngp", "nigp", "nua", "niua", "nsa", "nisa", "ne",
                 "algorithm", "precision_bytes", "matrix_entries")]


class CbKernelTable(C.Structure):
    _fields_ = [
        ("abi_version", C.c_int32),
        ("shape", CbShape),
        ("name", C.c_char_p),
        ("launch", C.c_void_p),
        ("occupancy", C.c_void_p),
        ("dynamic_smem", C.c_void_p),
        ("launch_record", C.c_void_p),
        ("launch_adjoint", C.c_void_p),
        ("adjoint_smem", C.c_void_p),
        ("adjoint_occupancy", C.c_void_p),
    ]


class Shape(C.Structure):
    _fields_ = [(n, C.c_int32) for n in
                ("sd", "ncp", "nsp", "nisp", "ne", "na", "nia", "algorithm", "precision_bytes", "modes")]


class Tape(C.Structure):
    _fields_ = [("segment", C.c_int32), ("max_steps", C.c_int32), ("dt", C.c_void_p), ("ckpt_x", C.c_void_p),
                ("ckpt_t", C.c_void_p), ("n_steps", C.c_void_p)]


class KernelTable(C.Structure):
    _fields_ = [
        ("abi_version", C.c_int32),
        ("shape", Shape),
        ("name", C.c_char_p),
        ("launch", C.c_void_p),
        ("occupancy", C.c_void_p),
        ("launch_record", C.c_void_p),
        ("launch_adjoint", C.c_void_p),
        ("dense_interpolate", C.c_void_p),
    ]


_runtime = None
_plugins: dict = {}


def _declare(lib):
    P = C.c_void_p
    i32, i64 = C.c_int32, C.c_int64
    sigs = {
        "mpgos_last_error": (C.c_char_p, []),
        "mpgos_abi_version": (C.c_int, []),
        "mpgos_pt_create": (C.c_int, [P, i64, i32, C.c_int, C.POINTER(P)]),
        "mpgos_pt_destroy": (C.c_int, [P]),
        "mpgos_pt_get_shape": (C.c_int, [P, C.POINTER(Shape), C.POINTER(i64), C.POINTER(i32)]),
        "mpgos_pt_set_option": (C.c_int, [P, i32, i32, C.c_double]),
        "mpgos_pt_get_option": (C.c_int, [P, i32, i32, C.POINTER(C.c_double)]),
        "mpgos_pt_host_buffer": (C.c_int, [P, i32, C.POINTER(P), C.POINTER(i64)]),
        "mpgos_pt_device_buffer": (C.c_int, [P, i32, C.POINTER(P), C.POINTER(i64)]),
        "mpgos_pt_sync_h2d": (C.c_int, [P, i32]),
        "mpgos_pt_sync_d2h": (C.c_int, [P, i32]),
        "mpgos_pt_solve": (C.c_int, [P]),
        "mpgos_pt_solve_phases": (C.c_int, [P, i32, i32, P]),
        "mpgos_pt_insert_sync_point": (C.c_int, [P]),
        "mpgos_pt_sync_solver": (C.c_int, [P]),
        "mpgos_pt_sync_device": (C.c_int, [P]),
        "mpgos_pt_stream": (C.c_int, [P, C.POINTER(P)]),
        "mpgos_pt_launch_config": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(i32)]),
        "mpgos_pt_timer_start": (C.c_int, [P]),
        "mpgos_pt_timer_stop": (C.c_int, [P, C.POINTER(C.c_float)]),
        "mpgos_pt_autotune": (C.c_int, [P, i32, C.c_char_p]),
        "mpgos_pt_checkpoint_save": (C.c_int, [P]),
        "mpgos_pt_checkpoint_restore": (C.c_int, [P]),
        "mpgos_probe_fma_peak": (C.c_int, [C.c_int, i32, C.POINTER(C.c_double)]),
        "mpgos_probe_df_math": (C.c_int, [C.c_int, i32, i64, P, P, P]),
        "mpgos_pt_solve_record": (C.c_int, [P, i32, i32]),
        "mpgos_pt_adjoint": (C.c_int, [P, P, P, P]),
        "mpgos_pt_tape_info": (C.c_int, [P, C.POINTER(Tape)]),
        "mpgos_pt_dense_interpolate": (C.c_int, [P, P, C.c_int32, P]),
        "mpgos_pt_solve_record_static": (C.c_int, [P, i32, i32]),
        "mpgos_cb_create": (C.c_int, [P, i64, i32, C.c_int, C.POINTER(P)]),
        "mpgos_cb_destroy": (C.c_int, [P]),
        "mpgos_cb_get_shape": (C.c_int, [P, C.POINTER(CbShape), C.POINTER(i64), C.POINTER(i32)]),
        "mpgos_cb_set_option": (C.c_int, [P, i32, i32, C.c_double]),
        "mpgos_cb_host_buffer": (C.c_int, [P, i32, C.POINTER(P), C.POINTER(i64)]),
        "mpgos_cb_device_buffer": (C.c_int, [P, i32, C.POINTER(P), C.POINTER(i64)]),
        "mpgos_cb_sync_h2d": (C.c_int, [P, i32]),
        "mpgos_cb_sync_d2h": (C.c_int, [P, i32]),
        "mpgos_cb_solve": (C.c_int, [P]),
        "mpgos_cb_insert_sync_point": (C.c_int, [P]),
        "mpgos_cb_sync_solver": (C.c_int, [P]),
        "mpgos_cb_timer_start": (C.c_int, [P]),
        "mpgos_cb_timer_stop": (C.c_int, [P, C.POINTER(C.c_float)]),
        "mpgos_cb_stream": (C.c_int, [P, C.POINTER(P)]),
        "mpgos_cb_checkpoint_save": (C.c_int, [P]),
        "mpgos_cb_checkpoint_restore": (C.c_int, [P]),
        "mpgos_cb_solve_record": (C.c_int, [P, i32, i32]),
        "mpgos_cb_adjoint": (C.c_int, [P, P, P, P]),
        "mpgos_cb_tape_info": (C.c_int, [P, C.POINTER(Tape)]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


# Exported symbol names of the runtime (everything mpgos.h declares for it).
RUNTIME_SYMBOLS = (
    "mpgos_last_error", "mpgos_abi_version", "mpgos_pt_create", "mpgos_pt_destroy", "mpgos_pt_get_shape",
    "mpgos_pt_set_option", "mpgos_pt_get_option", "mpgos_pt_host_buffer", "mpgos_pt_device_buffer",
    "mpgos_pt_sync_h2d", "mpgos_pt_sync_d2h", "mpgos_pt_solve", "mpgos_pt_solve_phases",
    "mpgos_pt_insert_sync_point", "mpgos_pt_sync_solver", "mpgos_pt_sync_device", "mpgos_pt_stream",
    "mpgos_pt_launch_config", "mpgos_pt_timer_start", "mpgos_pt_timer_stop", "mpgos_pt_autotune",
    "mpgos_pt_checkpoint_save", "mpgos_pt_checkpoint_restore", "mpgos_probe_fma_peak", "mpgos_probe_df_math",
    "mpgos_pt_solve_record", "mpgos_pt_adjoint", "mpgos_pt_tape_info", "mpgos_pt_solve_record_static",
    "mpgos_pt_dense_interpolate",
    "mpgos_cb_create", "mpgos_cb_destroy", "mpgos_cb_get_shape", "mpgos_cb_set_option", "mpgos_cb_host_buffer",
    "mpgos_cb_device_buffer", "mpgos_cb_sync_h2d", "mpgos_cb_sync_d2h", "mpgos_cb_solve",
    "mpgos_cb_insert_sync_point", "mpgos_cb_sync_solver", "mpgos_cb_timer_start", "mpgos_cb_timer_stop",
    "mpgos_cb_stream", "mpgos_cb_checkpoint_save", "mpgos_cb_checkpoint_restore",
    "mpgos_cb_solve_record", "mpgos_cb_adjoint", "mpgos_cb_tape_info",
)
# mpgos_pt_system_kernels: per-thread system plugins; mpgos_cb_system_kernels:
# coupled-system plugins.
PLUGIN_SYMBOLS = ("mpgos_pt_system_kernels", "mpgos_cb_system_kernels")


def runtime():
    """Load (once) libmpgos_runtime.so from the in-tree build directory."""
    global _runtime
    if _runtime is None:
        path = _build.runtime_lib()
        if not path.exists():
            raise FileNotFoundError(f"{path} is missing: run __graft_entry__.build() (or mpgos_gb300.build.build_all())")
        lib = C.CDLL(str(path), mode=C.RTLD_GLOBAL)
        _runtime = _declare(lib)
        if _runtime.mpgos_abi_version() != ABI_VERSION:
            raise MpgosError(4, "runtime ABI version mismatch")
    return _runtime


def plugin(name: str):
    """Load (once) the system plugin libmpgos_<name>.so (per-thread or
    coupled: whichever of the two entry points it exports is declared)."""
    if name not in _plugins:
        path = _build.system_lib(name)
        if not path.exists():
            raise FileNotFoundError(f"{path} is missing: run __graft_entry__.build()")
        lib = C.CDLL(str(path))
        for sym in PLUGIN_SYMBOLS:
            if hasattr(lib, sym):
                fn = getattr(lib, sym)
                fn.restype = C.c_void_p
                fn.argtypes = [C.c_int32, C.c_int32]
        _plugins[name] = lib
    return _plugins[name]


def coupled_kernel_table(system: str, algorithm: int, precision_bytes: int) -> int:
    lib = plugin(system)
    if not hasattr(lib, "mpgos_cb_system_kernels"):
        raise MpgosError(5, f"{system!r} is not a coupled-system plugin")
    ptr = lib.mpgos_cb_system_kernels(int(algorithm), int(precision_bytes))
    if not ptr:
        raise MpgosError(5, f"coupled system {system!r} has no kernels for algorithm {algorithm}, "
                            f"{precision_bytes}-byte precision")
    return ptr


def coupled_kernel_table_info(ptr: int) -> CbKernelTable:
    return CbKernelTable.from_address(ptr)


def kernel_table(system: str, algorithm: int, precision_bytes: int) -> int:
    lib = plugin(system)
    if not hasattr(lib, "mpgos_pt_system_kernels"):
        raise MpgosError(5, f"{system!r} is not a per-thread system plugin")
    ptr = lib.mpgos_pt_system_kernels(int(algorithm), int(precision_bytes))
    if not ptr:
        raise MpgosError(5, f"system {system!r} has no kernels for algorithm {algorithm}, {precision_bytes}-byte precision")
    return ptr


def kernel_table_info(ptr: int) -> KernelTable:
    return KernelTable.from_address(ptr)


def check(rc: int) -> None:
    if rc != 0:
        msg = runtime().mpgos_last_error()
        raise MpgosError(rc, msg.decode() if msg else "")


def loaded_library_paths() -> list:
    """Paths of the native libraries this module has loaded."""
    out = []
    if _runtime is not None:
        out.append(str(_build.runtime_lib()))
    out.extend(str(_build.system_lib(n)) for n in _plugins)
    return out


DF_OPS = {"exp": 0, "log": 1, "pow": 2, "sin": 3, "cos": 4, "sqrt": 5, "div": 6, "mul": 7, "add": 8, "pow_int": 9,
          "sinpi": 10, "cospi": 11, "split": 12, "root5": 13, "root4": 14}


def df_math(op: str, a, b=None, device: int = 0):
    """Device double-float evaluation (mpgos_probe_df_math): (hi, lo) arrays of
    op(a, b) with a, b converted to double-float."""
    import numpy as np
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(np.zeros_like(a) if b is None else b, dtype=np.float64)
    out = np.empty(2 * a.size, dtype=np.float64)
    check(runtime().mpgos_probe_df_math(int(device), DF_OPS[op], a.size, a.ctypes.data, b.ctypes.data,
                                        out.ctypes.data))
    return out[0::2].copy(), out[1::2].copy()


def fma_peak(device: int = 0, precision_bytes: int = 8) -> float:
    """Measured FMA throughput of the device in FLOP/s (mpgos_probe_fma_peak)."""
    v = C.c_double()
    check(runtime().mpgos_probe_fma_peak(int(device), int(precision_bytes), C.byref(v)))
    return float(v.value)
