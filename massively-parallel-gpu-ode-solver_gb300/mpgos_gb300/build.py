"""In-tree build of the native libraries (no pip install, no cmake).

Outputs, all under ``massively-parallel-gpu-ode-solver_gb300/_build/``:

* ``libmpgos_runtime.so``   host runtime implementing the C-ABI of ``include/mpgos.h``
* ``libmpgos_<system>.so``  one system plugin per hook file in ``systems/``
  (sm_103a kernels for that system's user hooks)
* ``libmpgos_<ring>.so``    coupled-system plugins (one warp per system),
  one per ``systems/<ring>.cu`` in ``COUPLED``

Every CUDA translation unit is compiled with
``-gencode arch=compute_103a,code=sm_103a`` only. Units are compiled in
parallel and skipped when their output is newer than every input.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent          # massively-parallel-gpu-ode-solver_gb300/
REPO_ROOT = PKG_ROOT.parent
BUILD_DIR = PKG_ROOT / "_build"
INCLUDE_DIR = REPO_ROOT / "include"
CSRC = PKG_ROOT / "csrc"
SYSTEMS_DIR = PKG_ROOT / "systems"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# System plugins built by default: name -> source file (hook file + plugin export).
SYSTEMS = ["lorenz", "duffing", "duffing_param", "duffing_param_sens", "duffing_events", "bouncing_ball",
           "keller_miksis"]
# Coupled-system plugins: the ring of Duffing oscillators with 64 units and,
# at 16 units, each of the four coupling-matrix storages.
COUPLED = ["ring64", "ring16_full", "ring16_band", "ring16_circband", "ring16_circ", "ring256"]


def nvcc_path() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def cuda_home() -> Path:
    return Path(nvcc_path()).resolve().parent.parent


def _newer(out: Path, deps) -> bool:
    if not out.exists():
        return False
    t = out.stat().st_mtime
    return all(Path(d).stat().st_mtime <= t for d in deps)


def _deps_glob(*dirs) -> list:
    out = []
    for d in dirs:
        for ext in ("*.cuh", "*.h", "*.cu", "*.cpp", "*.hpp"):
            out.extend(Path(d).rglob(ext))
    return out


def _run(cmd: list, what: str) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build of {what} failed (exit {proc.returncode}):\n{' '.join(cmd)}\n{proc.stdout}")


def _common_flags() -> list:
    lib = cuda_home() / "lib64"
    return [
        "-O3", "-std=c++17", "-lineinfo", "-shared", "-Xcompiler", "-fPIC",
        "-Xcompiler", "-fvisibility=hidden", "-cudart", "shared",
        f"-I{INCLUDE_DIR}", f"-I{CSRC / 'perthread'}", f"-I{CSRC / 'coupled'}", f"-I{SYSTEMS_DIR}",
        "-Xlinker", f"-rpath,{lib}", "-Xlinker", "-rpath,$ORIGIN",
    ]


def runtime_lib() -> Path:
    return BUILD_DIR / "libmpgos_runtime.so"


def system_lib(name: str) -> Path:
    return BUILD_DIR / f"libmpgos_{name}.so"


def build_runtime(force: bool = False) -> Path:
    out = runtime_lib()
    srcs = [CSRC / "runtime" / "runtime.cpp", CSRC / "runtime" / "runtime_coupled.cpp", CSRC / "runtime" / "probes.cu",
            CSRC / "runtime" / "work_order.cu"]
    deps = [*srcs, INCLUDE_DIR / "mpgos.h"]
    if not force and _newer(out, deps):
        return out
    cmd = [nvcc_path(), *ARCH, *_common_flags(), "-x", "cu", *map(str, srcs), "-o", str(out)]
    _run(cmd, "libmpgos_runtime.so")
    return out


# Per-thread system plugins are compiled as several translation units in
# parallel (plugin_export.cuh, MPGOS_PLUGIN_PARTS): the main unit (tables, FP64
# and float kernels, adjoint) and one unit per double-float kernel set,
# (arithmetic, scheme) = DF_STAGE or SPLIT x RK4 or RKCK45, then linked.
PART_SETS = [(16, 0), (16, 1), (128, 0), (128, 1)]

_COMPILE_POOL = cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 4))


def build_system(name: str, force: bool = False, extra: list | None = None) -> Path:
    out = system_lib(name)
    src = SYSTEMS_DIR / f"{name}.cu"
    deps = [src, INCLUDE_DIR / "mpgos.h", *_deps_glob(CSRC / "perthread", CSRC / "coupled"),
            *SYSTEMS_DIR.glob("*.cuh")]
    if not force and _newer(out, deps):
        return out
    if "coupled_plugin_export.cuh" in src.read_text():
        cmd = [nvcc_path(), *ARCH, *_common_flags(), *(extra or []), str(src), "-o", str(out)]
        _run(cmd, f"libmpgos_{name}.so")
        return out
    objdir = BUILD_DIR / "obj"
    objdir.mkdir(parents=True, exist_ok=True)
    flags = [f for f in _common_flags() if f != "-shared"]
    units = [("main", ["-DMPGOS_PLUGIN_PARTS"])] + [
        (f"part{a}_{g}", ["-DMPGOS_PLUGIN_PARTS", f"-DMPGOS_PART_ARITH={a}", f"-DMPGOS_PART_ALG={g}"])
        for a, g in PART_SETS]
    futs, objs = [], []
    for tag, defs in units:
        obj = objdir / f"{name}.{tag}.o"
        objs.append(obj)
        cmd = [nvcc_path(), *ARCH, *flags, *defs, *(extra or []), "-c", str(src), "-o", str(obj)]
        futs.append(_COMPILE_POOL.submit(_run, cmd, f"libmpgos_{name}.so ({tag})"))
    for f in futs:
        f.result()
    cmd = [nvcc_path(), *ARCH, *_common_flags(), *(extra or []), *map(str, objs), "-o", str(out)]
    _run(cmd, f"libmpgos_{name}.so (link)")
    return out


def build_all(force: bool = False, systems=None, jobs: int | None = None) -> dict:
    """Build the runtime and every system plugin; returns {name: path}."""
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    systems = list(systems or (SYSTEMS + COUPLED))
    jobs = jobs or max(1, min(len(systems) + 1, os.cpu_count() or 4))
    results = {}
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = {ex.submit(build_runtime, force): "runtime"}
        for s in systems:
            futs[ex.submit(build_system, s, force)] = s
        errors = []
        for f in cf.as_completed(futs):
            try:
                results[futs[f]] = f.result()
            except Exception as e:  # collect all failures, then raise once
                errors.append(str(e))
        if errors:
            raise RuntimeError("\n\n".join(errors))
    return results


if __name__ == "__main__":
    import sys
    r = build_all(force="--force" in sys.argv)
    for k, v in sorted(r.items()):
        print(f"{k}: {v}")
