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


MODE_PLAIN = 0
MODE_FAST_CONTROL = 1
MODE_PERSISTENT = 2
MODE_FP32_STAGE = 4
MODE_CHOSEN = MODE_FAST_CONTROL | MODE_PERSISTENT

INSTANCE_OK = 0
INSTANCE_NONFINITE = 1
INSTANCE_MINIMUM_STEP = 2
INSTANCE_EVENT_OMITTED = 4
INSTANCE_ATTEMPT_LIMIT = 8
INSTANCE_TAPE_OVERFLOW = 16

ABI_VERSION = 1


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
        "mpgos_pt_solve_record": (C.c_int, [P, i32, i32]),
        "mpgos_pt_adjoint": (C.c_int, [P, P, P, P]),
        "mpgos_pt_tape_info": (C.c_int, [P, C.POINTER(Tape)]),
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
    "mpgos_pt_checkpoint_save", "mpgos_pt_checkpoint_restore", "mpgos_probe_fma_peak",
    "mpgos_pt_solve_record", "mpgos_pt_adjoint", "mpgos_pt_tape_info",
)
PLUGIN_SYMBOLS = ("mpgos_pt_system_kernels",)


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
    """Load (once) the system plugin libmpgos_<name>.so."""
    if name not in _plugins:
        path = _build.system_lib(name)
        if not path.exists():
            raise FileNotFoundError(f"{path} is missing: run __graft_entry__.build()")
        lib = C.CDLL(str(path))
        fn = lib.mpgos_pt_system_kernels
        fn.restype = C.c_void_p
        fn.argtypes = [C.c_int32, C.c_int32]
        _plugins[name] = lib
    return _plugins[name]


def kernel_table(system: str, algorithm: int, precision_bytes: int) -> int:
    ptr = plugin(system).mpgos_pt_system_kernels(int(algorithm), int(precision_bytes))
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


def fma_peak(device: int = 0, precision_bytes: int = 8) -> float:
    """Measured FMA throughput of the device in FLOP/s (mpgos_probe_fma_peak)."""
    v = C.c_double()
    check(runtime().mpgos_probe_fma_peak(int(device), int(precision_bytes), C.byref(v)))
    return float(v.value)
