"""Python front end of the CPU oracle (and of the pinned reference CPU build).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline leg, as the reference results to compare with. The
product never imports it.

``run_oracle(case)`` integrates a ``mpgos_gb300.workloads.Case`` with the
oracle (oracle_perthread.cpp), ``run_ref_cpu(case)`` with the reference's own
solver kernel compiled for the CPU (only where the reference checkout exists).
Both return the same result dictionary as ``workloads.run_gpu``.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import build_oracle as _b

_libs: dict = {}
_ref_libs: dict = {}

_D = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_I = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def _oracle(system: str, fma: bool = False):
    key = (system, fma)
    if key not in _libs:
        path = _b.build_oracle(system, fma=fma)
        lib = C.CDLL(str(path))
        lib.oracle_pt_solve.restype = C.c_int
        lib.oracle_pt_solve.argtypes = [
            C.c_int, C.c_longlong, C.c_longlong, C.c_longlong, C.c_int,
            _D, _D, _D, _D, _D, _I, _D, _I, _D, _D, _D, _I, _I, _D, _D, _I, _I, _I, _D, C.c_int, C.c_longlong, C.c_int]
        lib.oracle_pt_threads.restype = C.c_int
        _libs[key] = lib
    return _libs[key]


def _ref(system: str):
    if system not in _ref_libs:
        path = _b.build_ref(system)
        if path is None:
            raise FileNotFoundError("reference checkout not available: reference CPU build cannot be made")
        lib = C.CDLL(str(path))
        lib.ref_cpu_solve.restype = C.c_int
        lib.ref_cpu_solve.argtypes = [
            C.c_int, C.c_longlong, C.c_longlong, C.c_int,
            _D, _D, _D, _D, _D, _I, _D, _I, _D, _D, _D, _I, _I, _D, _D, _D, C.c_int]
        lib.ref_cpu_set_threads.restype = C.c_int
        lib.ref_cpu_set_threads.argtypes = [C.c_int]
        _ref_libs[system] = lib
    return _ref_libs[system]


def replay(case, dt_tape: np.ndarray, n_steps: np.ndarray, x0=None, cp=None, threads: int = 0) -> np.ndarray:
    """End states of ``case`` integrated with a frozen step sequence
    (``dt_tape`` [max_steps][NT], ``n_steps`` [NT]); optional replacement
    initial states / control parameters. Returns x(T) [SD][NT]."""
    lib = _oracle(case.system)
    if not hasattr(lib.oracle_pt_replay, "_typed"):
        lib.oracle_pt_replay.restype = C.c_int
        lib.oracle_pt_replay.argtypes = [C.c_int, C.c_longlong, C.c_longlong, C.c_longlong, _D, _D, _D, _D, _I, _D,
                                         _I, _D, _I, C.c_int]
        lib.oracle_pt_replay._typed = True
    a, tol, _ = _prepare(case)
    x = np.ascontiguousarray((a["x"] if x0 is None else np.asarray(x0, np.float64)).copy())
    cpa = a["cp"] if cp is None else np.ascontiguousarray(np.asarray(cp, np.float64))
    t = np.ascontiguousarray(a["t"].copy())
    rc = lib.oracle_pt_replay(case.algorithm, case.nt, 0, case.nt, x, t, cpa, tol["sp"], tol["spi"], a["acc"],
                              a["acci"], np.ascontiguousarray(dt_tape, dtype=np.float64),
                              np.ascontiguousarray(n_steps, dtype=np.int32), int(threads))
    if rc != 0:
        raise RuntimeError(f"oracle_pt_replay failed with {rc}")
    return x


def dense_interpolate(case, didx, dtime, dstate, times, acc=None, acci=None) -> np.ndarray:
    """CPU cubic Hermite interpolation of a dense output (``didx`` [NT],
    ``dtime`` [NDO][NT], ``dstate`` [NDO][SD][NT], e.g. read back from the GPU)
    at ``times``, with the right-hand side of ``case``'s hooks as slopes.
    Returns [n_times][SD][NT]."""
    lib = _oracle(case.system)
    if not hasattr(lib.oracle_pt_dense_interpolate, "_typed"):
        lib.oracle_pt_dense_interpolate.restype = C.c_int
        lib.oracle_pt_dense_interpolate.argtypes = [C.c_longlong, C.c_int, _I, _D, _D, _D, _D, _I, _D, _I, _D,
                                                    C.c_int, _D]
        lib.oracle_pt_dense_interpolate._typed = True
    a, tol, _ = _prepare(case)
    times = np.ascontiguousarray(np.asarray(times, np.float64))
    sd = np.asarray(dstate).shape[1] if np.asarray(dstate).ndim == 3 else a["x"].shape[0]
    out = np.empty((len(times), sd, case.nt))
    rc = lib.oracle_pt_dense_interpolate(
        case.nt, case.ndo, np.ascontiguousarray(didx, dtype=np.int32), np.ascontiguousarray(dtime, dtype=np.float64),
        np.ascontiguousarray(dstate, dtype=np.float64), a["cp"], tol["sp"], tol["spi"],
        np.ascontiguousarray(a["acc"] if acc is None else acc, dtype=np.float64),
        np.ascontiguousarray(a["acci"] if acci is None else acci, dtype=np.int32), times, len(times), out)
    if rc != 0:
        raise RuntimeError(f"oracle_pt_dense_interpolate failed with {rc}")
    return out


def max_threads(system: str = "lorenz") -> int:
    return int(_oracle(system).oracle_pt_threads())


def _prepare(case):
    a = {k: np.ascontiguousarray(v.copy()) for k, v in case.arrays.items()}
    for k in ("acci", "didx", "spi"):
        a[k] = np.ascontiguousarray(a[k].astype(np.int32))
    pad = lambda v, dt: np.ascontiguousarray(np.concatenate([np.asarray(v, dtype=dt), np.zeros(1, dt)]))
    tol = dict(rtol=pad(case.rtol, np.float64), atol=pad(case.atol, np.float64), etol=pad(case.etol, np.float64),
               edir=pad(case.edir, np.int32), sp=pad(a["sp"], np.float64), spi=pad(a["spi"], np.int32))
    for k in ("cp", "acc", "acci", "dtime", "dstate"):
        if a[k].size == 0:   # zero-sized fields still need a valid pointer
            a[k] = np.zeros(1, dtype=a[k].dtype)
    o = case.options
    opt6 = np.array([o["initial_dt"], o["max_dt"], o["min_dt"], o["grow"], o["shrink"], o["dense_min_dt"]])
    return a, tol, opt6


def _results(case, a, status, nacc, nrej):
    sd, ncp, nsp, nisp, ne, na, nia = case.shape
    nt = case.nt
    out = dict(td=a["td"], x=a["x"], t=a["t"], didx=a["didx"], status=status, nacc=nacc, nrej=nrej,
               cp=a["cp"].reshape(ncp, nt) if ncp else np.zeros((0, nt)),
               acc=a["acc"].reshape(na, nt) if na else np.zeros((0, nt)),
               acci=a["acci"].reshape(nia, nt) if nia else np.zeros((0, nt), dtype=np.int32))
    if case.ndo:
        out["dtime"] = a["dtime"]
        out["dstate"] = a["dstate"]
    return out


def run_oracle(case, threads: int = 0, first: int = 0, count: int | None = None, fma: bool = False) -> dict:
    """Integrate ``case`` (all its phases) with the CPU oracle; ``fma``: the
    build with contracted multiply-adds (a rounding perturbation, not a
    reference)."""
    lib = _oracle(case.system, fma)
    a, tol, opt6 = _prepare(case)
    nt = case.nt
    n_active = case.n_active if case.n_active is not None else nt
    count = n_active - first if count is None else count
    status = np.zeros(nt, np.int32)
    nacc = np.zeros(nt, np.int32)
    nrej = np.zeros(nt, np.int32)
    o = case.options
    for _ in range(case.phases):
        rc = lib.oracle_pt_solve(case.algorithm, nt, first, count, case.ndo, a["td"], a["x"], a["t"], a["cp"],
                                 tol["sp"], tol["spi"], a["acc"], a["acci"], tol["rtol"], tol["atol"], tol["etol"],
                                 tol["edir"], a["didx"], a["dtime"], a["dstate"], status, nacc, nrej, opt6,
                                 int(o["dense_freq"]), int(o["max_attempts"]), int(threads))
        if rc != 0:
            raise RuntimeError(f"oracle_pt_solve failed with {rc}")
    return _results(case, a, status, nacc, nrej)


def time_oracle(case, threads: int = 0) -> float:
    """Wall-clock seconds of one oracle run of ``case``."""
    t0 = time.perf_counter()
    run_oracle(case, threads=threads)
    return time.perf_counter() - t0


def ref_cpu_available(system: str) -> bool:
    """The reference's CPU build can be made (checkout or staged headers)."""
    return _b.reference_available()


def run_ref_cpu(case, threads: int = 1) -> dict:
    """Integrate ``case`` with the reference's own kernel compiled for the CPU
    (nt in {64, 256, 1024}, ndo in {0, 16}; Lorenz RKCK45 also 65536 and
    131072), instances spread over ``threads`` host threads (0: all)."""
    lib = _ref(case.system)
    lib.ref_cpu_set_threads(int(threads))
    a, tol, opt6 = _prepare(case)
    nt = case.nt
    n_active = case.n_active if case.n_active is not None else nt
    # The reference kernel reads the event options for every component index
    # below SD (SingleSystem_PerThread_Solver.cuh:60); pad them to SD entries.
    sd = case.shape[0]
    etol = np.ascontiguousarray(np.concatenate([tol["etol"], np.zeros(sd)]))
    edir = np.ascontiguousarray(np.concatenate([tol["edir"], np.zeros(sd, np.int32)]))
    for _ in range(case.phases):
        rc = lib.ref_cpu_solve(case.algorithm, nt, n_active, case.ndo, a["td"], a["x"], a["t"], a["cp"], tol["sp"],
                               tol["spi"], a["acc"], a["acci"], tol["rtol"], tol["atol"], etol, edir, a["didx"],
                               a["dtime"], a["dstate"], opt6, int(case.options["dense_freq"]))
        if rc != 0:
            raise RuntimeError(f"ref_cpu_solve: (nt={nt}, ndo={case.ndo}) not compiled")
    z = np.zeros(nt, np.int32)
    return _results(case, a, z, z.copy(), z.copy())


# ---- coupled per-block solver -------------------------------------------------
class _CbArrays(C.Structure):
    _fields_ = [("ns", C.c_longlong)] + [(n, C.c_void_p) for n in (
        "td", "t", "sp", "sacc", "cstr", "dtime", "x", "up", "uacc", "dstate", "isacc", "didx", "iuacc", "gp", "cmat",
        "rtol", "atol", "etol", "igp", "cidx", "edir", "status", "nacc", "nrej")]


class _CbOpts(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("initial_dt", "max_dt", "min_dt", "grow", "shrink", "dense_min_dt")] + [
        ("dense_freq", C.c_int), ("ndo", C.c_int), ("max_attempts", C.c_longlong)]


_cb_libs: dict = {}


def _oracle_cb(system: str, fma: bool = False):
    key = (system, fma)
    if key not in _cb_libs:
        lib = C.CDLL(str(_b.build_oracle_coupled(system, fma=fma)))
        lib.oracle_cb_solve.restype = C.c_int
        lib.oracle_cb_solve.argtypes = [C.POINTER(_CbArrays), C.POINTER(_CbOpts), C.c_int, C.c_longlong, C.c_longlong,
                                        C.c_int]
        lib.oracle_cb_shape.restype = None
        lib.oracle_cb_shape.argtypes = [C.POINTER(C.c_int)]
        _cb_libs[key] = lib
    return _cb_libs[key]


def oracle_cb_shape(system: str) -> tuple:
    """(UPS, UD, NC, CBW, CCI, NUP, NSP, NGP, NIGP, NUA, NIUA, NSA, NISA, NE, MAT)."""
    out = (C.c_int * 15)()
    _oracle_cb(system).oracle_cb_shape(out)
    return tuple(out)


def run_oracle_coupled(case, threads: int = 0, first: int = 0, count: int | None = None, fma: bool = False) -> dict:
    """Integrate a ``coupled_workloads.CbCase`` (all phases) with the coupled
    oracle; systems [first, first + count) only when given (the others keep
    their inputs); ``fma``: the contracted build. Returns the dictionary of
    ``run_coupled_gpu``."""
    lib = _oracle_cb(case.system, fma)
    a = case.arrays
    f64 = lambda v: np.ascontiguousarray(np.array(v, dtype=np.float64, copy=True))
    i32 = lambda v: np.ascontiguousarray(np.array(v, dtype=np.int32, copy=True))
    ns = case.ns
    st = dict(td=f64(a["td"]), t=f64(a["t"]), sp=f64(a["sp"]), sacc=f64(a["sacc"]), cstr=f64(a["cstr"]),
              dtime=f64(a["dtime"]), x=f64(a["x"]), up=f64(a["up"]), uacc=f64(a["uacc"]), dstate=f64(a["dstate"]),
              isacc=i32(a["isacc"]), didx=i32(a["didx"]), iuacc=i32(a["iuacc"]), gp=f64(a["gp"]),
              cmat=f64(case.stored_matrix()), rtol=f64(case.rtol), atol=f64(case.atol), etol=f64(case.etol),
              igp=i32(a["igp"]), cidx=i32(a["cidx"]), edir=i32(case.edir), status=np.zeros(ns, np.int32),
              nacc=np.zeros(ns, np.int32), nrej=np.zeros(ns, np.int32))
    pad = {k: (v if v.size else np.zeros(2, v.dtype)) for k, v in st.items()}
    arr = _CbArrays(ns, *[pad[n].ctypes.data for n, _ in _CbArrays._fields_[1:]])
    o = case.options
    opts = _CbOpts(o["initial_dt"], o["max_dt"], o["min_dt"], o["grow"], o["shrink"], o["dense_min_dt"],
                   int(o["dense_freq"]), int(case.ndo), int(o["max_attempts"]))
    n_active = case.n_active if case.n_active is not None else ns
    count = n_active - first if count is None else count
    for _ in range(case.phases):
        rc = lib.oracle_cb_solve(C.byref(arr), C.byref(opts), int(case.algorithm), int(first), int(count), int(threads))
        if rc != 0:
            raise RuntimeError(f"oracle_cb_solve failed with {rc}")
    out = {k: st[k] for k in ("td", "t", "x", "didx", "status", "nacc", "nrej", "iuacc", "uacc", "isacc", "sacc")}
    if case.ndo:
        out["dtime"], out["dstate"] = st["dtime"], st["dstate"]
    return out


def replay_coupled(case, dt_tape: np.ndarray, n_steps: np.ndarray, x0=None, sp=None, threads: int = 0) -> np.ndarray:
    """End states of a ``CbCase`` integrated with a frozen step sequence
    (``dt_tape`` [max_steps][NS], ``n_steps`` [NS]); optional replacement
    initial states [UD][NS*UPS] / system parameters [NSP][NS]. Returns x(T)."""
    lib = _oracle_cb(case.system)
    if not hasattr(lib.oracle_cb_replay, "_typed"):
        lib.oracle_cb_replay.restype = C.c_int
        lib.oracle_cb_replay.argtypes = [C.POINTER(_CbArrays), C.POINTER(_CbOpts), C.c_int, _D, _I, C.c_int,
                                         C.c_longlong, C.c_longlong, C.c_int]
        lib.oracle_cb_replay._typed = True
    a = case.arrays
    f64 = lambda v: np.ascontiguousarray(np.array(v, dtype=np.float64, copy=True))
    i32 = lambda v: np.ascontiguousarray(np.array(v, dtype=np.int32, copy=True))
    st = dict(td=f64(a["td"]), t=f64(a["t"]), sp=f64(a["sp"] if sp is None else sp), sacc=f64(a["sacc"]),
              cstr=f64(a["cstr"]), dtime=f64(a["dtime"]), x=f64(a["x"] if x0 is None else x0), up=f64(a["up"]),
              uacc=f64(a["uacc"]), dstate=f64(a["dstate"]), isacc=i32(a["isacc"]), didx=i32(a["didx"]),
              iuacc=i32(a["iuacc"]), gp=f64(a["gp"]), cmat=f64(case.stored_matrix()), rtol=f64(case.rtol),
              atol=f64(case.atol), etol=f64(case.etol), igp=i32(a["igp"]), cidx=i32(a["cidx"]), edir=i32(case.edir),
              status=np.zeros(case.ns, np.int32), nacc=np.zeros(case.ns, np.int32), nrej=np.zeros(case.ns, np.int32))
    pad = {k: (v if v.size else np.zeros(2, v.dtype)) for k, v in st.items()}
    arr = _CbArrays(case.ns, *[pad[n].ctypes.data for n, _ in _CbArrays._fields_[1:]])
    o = case.options
    opts = _CbOpts(o["initial_dt"], o["max_dt"], o["min_dt"], o["grow"], o["shrink"], o["dense_min_dt"],
                   int(o["dense_freq"]), int(case.ndo), int(o["max_attempts"]))
    dt = np.ascontiguousarray(dt_tape, dtype=np.float64)
    rc = lib.oracle_cb_replay(C.byref(arr), C.byref(opts), int(case.algorithm), dt,
                              np.ascontiguousarray(n_steps, dtype=np.int32), int(dt.shape[0]), 0, int(case.ns),
                              int(threads))
    if rc != 0:
        raise RuntimeError(f"oracle_cb_replay failed with {rc}")
    return st["x"]


def time_oracle_coupled(case, threads: int = 0, count: int | None = None) -> tuple:
    """Wall time of the coupled oracle on the first ``count`` systems; returns
    (seconds, accepted system-steps)."""
    t0 = time.perf_counter()
    r = run_oracle_coupled(case, threads=threads, first=0, count=count)
    dt = time.perf_counter() - t0
    n = case.ns if count is None else count
    return dt, int(r["nacc"][:n].sum())
