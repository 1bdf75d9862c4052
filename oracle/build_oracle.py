"""Build recipe of the CPU oracle and of the pinned reference CPU build.

TEST INFRASTRUCTURE ONLY.

* ``oracle/_build/liboracle_<system>.so`` - the oracle (oracle_perthread.cpp)
  compiled once per hook file, with OpenMP. Built everywhere, including the
  GPU machine.
* ``oracle/_ref/libref_cpu_<system>.so`` - the reference's own
  SourceCodes/SingleSystem_PerThread_Solver.cuh compiled for the CPU through
  ref_cpu_entry.cpp, straight from the reference checkout (MPGOS_REFERENCE_ROOT,
  default /root/reference). Built only where that checkout exists; used to
  pin the oracle and to generate tests/golden fixtures.

Both use ``-ffp-contract=off`` so that no multiply-add is fused: built with the
same flags on the same machine, the two agree bit for bit.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
REPO_ROOT = ORACLE_DIR.parent
SYSTEMS_DIR = REPO_ROOT / "massively-parallel-gpu-ode-solver_gb300" / "systems"
BUILD_DIR = ORACLE_DIR / "_build"
REF_DIR = ORACLE_DIR / "_ref"
REFERENCE_ROOT = Path(os.environ.get("MPGOS_REFERENCE_ROOT", "/root/reference"))

SYSTEMS = ["lorenz", "duffing", "duffing_param", "duffing_events", "bouncing_ball", "keller_miksis"]
FLAGS = ["-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math"]


def oracle_lib(system: str) -> Path:
    return BUILD_DIR / f"liboracle_{system}.so"


def ref_lib(system: str) -> Path:
    return REF_DIR / f"libref_cpu_{system}.so"


def reference_available() -> bool:
    return (REFERENCE_ROOT / "SourceCodes" / "SingleSystem_PerThread_Solver.cuh").exists()


def _newer(out: Path, deps) -> bool:
    if not out.exists():
        return False
    t = out.stat().st_mtime
    return all(Path(d).stat().st_mtime <= t for d in deps)


def _run(cmd, what):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"build of {what} failed:\n{' '.join(map(str, cmd))}\n{p.stdout}")


def build_oracle(system: str, force: bool = False) -> Path:
    out = oracle_lib(system)
    src = ORACLE_DIR / "oracle_perthread.cpp"
    hdr = SYSTEMS_DIR / f"{system}.cuh"
    if not force and _newer(out, [src, hdr, ORACLE_DIR / "host_shim.hpp", Path(__file__)]):
        return out
    cmd = ["g++", *FLAGS, "-fopenmp", f"-I{ORACLE_DIR}", f"-I{SYSTEMS_DIR}",
           f'-DMPGOS_SYSTEM_HEADER="{system}.cuh"', str(src), "-o", str(out)]
    _run(cmd, out.name)
    return out


def build_ref(system: str, force: bool = False) -> Path | None:
    if not reference_available():
        return None
    out = ref_lib(system)
    src = ORACLE_DIR / "ref_cpu_entry.cpp"
    hdr = SYSTEMS_DIR / f"{system}.cuh"
    if not force and _newer(out, [src, hdr, ORACLE_DIR / "host_shim.hpp", Path(__file__)]):
        return out
    cmd = ["g++", *FLAGS, "-w", f"-I{ORACLE_DIR}", f"-I{SYSTEMS_DIR}", f"-I{REFERENCE_ROOT / 'SourceCodes'}",
           f'-DMPGOS_SYSTEM_HEADER="{system}.cuh"', str(src), "-o", str(out)]
    _run(cmd, out.name)
    return out


def build_all(force: bool = False) -> dict:
    BUILD_DIR.mkdir(exist_ok=True)
    REF_DIR.mkdir(exist_ok=True)
    res = {}
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        futs = {}
        for s in SYSTEMS:
            futs[ex.submit(build_oracle, s, force)] = ("oracle", s)
            futs[ex.submit(build_ref, s, force)] = ("ref", s)
        errors = []
        for f in cf.as_completed(futs):
            try:
                res[futs[f]] = f.result()
            except Exception as e:
                errors.append(str(e))
        if errors:
            raise RuntimeError("\n".join(errors))
    return res


if __name__ == "__main__":
    import sys
    for k, v in sorted(build_all(force="--force" in sys.argv).items()):
        print(k, v)
