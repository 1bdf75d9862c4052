"""Build recipe of the CPU oracle and of the pinned reference CPU build.

TEST INFRASTRUCTURE ONLY.

* ``oracle/_build/liboracle_<system>.so`` - the oracle (oracle_perthread.cpp)
  compiled once per hook file, with OpenMP. Built everywhere, including the
  GPU machine.
* ``oracle/_ref/ref_gpu_<system>_<alg>_nt<NT>_ndo<NDO>.cubin`` - the
  reference's own per-thread kernel built for sm_103a (ref_gpu_entry.cu),
  device code only; built where the reference checkout exists and shipped to
  the GPU machine with the working tree.
* ``oracle/_build/liboracle_fma_<system>.so`` / ``liboracle_cb_fma_<system>.so``
  - the same oracles with multiply-adds contracted into fused multiply-adds
  (``-ffp-contract=fast``, plus ``-mfma`` on x86-64 where FMA is not in the
  base instruction set). Not a reference: the tests measure how far the
  oracle's own results move when only the rounding of multiply-adds changes,
  which is the difference between the GPU and the host arithmetic.
* ``oracle/_build/liboracle_cb_<system>.so`` - the coupled-solver oracle
  (oracle_coupled.cpp) compiled once per coupled-system plugin source
  ``systems/<system>.cu`` (its hook file and coupling storage).
* ``oracle/_ref/ref_gpu_cb_<system>_<alg>_ns<NS>_tpb<TPB>_spb<SPB>_ndo<NDO>.cubin``
  - the reference's own coupled kernels (all four variants, picked from
  SPB, UPS and TPB as its Solve() does) built for sm_103a
  (ref_gpu_coupled_entry.cu).
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

SYSTEMS = ["lorenz", "duffing", "duffing_param", "duffing_param_sens", "duffing_events", "bouncing_ball",
           "keller_miksis"]
FLAGS = ["-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math"]
# Coupled-system plugins (the product's build list): the oracle and the
# reference cubins read hook file, UPS, CBW and CCI from systems/<name>.cu.
COUPLED = ["ring64", "ring16_full", "ring16_band", "ring16_circband", "ring16_circ", "ring256"]


def coupled_defs(system: str) -> dict:
    """{"header": hook file, "UPS": .., "CBW": .., "CCI": ..} of a coupled plugin."""
    import re
    text = (SYSTEMS_DIR / f"{system}.cu").read_text()
    out = {"header": re.search(r'#include\s+"([^"/]+\.cuh)"', text).group(1)}
    for k in ("UPS", "CBW", "CCI"):
        out[k] = int(re.search(rf"#define\s+MPGOS_SYS_{k}\s+(\d+)", text).group(1))
    return out


def _coupled_macros(system: str) -> list:
    d = coupled_defs(system)
    return [f'-DMPGOS_SYSTEM_HEADER="{d["header"]}"', f"-DMPGOS_SYS_UPS={d['UPS']}", f"-DMPGOS_SYS_CBW={d['CBW']}",
            f"-DMPGOS_SYS_CCI={d['CCI']}"]


def oracle_cb_lib(system: str, fma: bool = False) -> Path:
    return BUILD_DIR / f"liboracle_cb_{'fma_' if fma else ''}{system}.so"


def build_oracle_coupled(system: str, force: bool = False, fma: bool = False) -> Path:
    out = oracle_cb_lib(system, fma)
    src = ORACLE_DIR / "oracle_coupled.cpp"
    d = coupled_defs(system)
    deps = [src, SYSTEMS_DIR / d["header"], SYSTEMS_DIR / f"{system}.cu", ORACLE_DIR / "host_shim.hpp", Path(__file__)]
    if not force and _newer(out, deps):
        return out
    cmd = ["g++", *(_fma_flags() if fma else FLAGS), "-fopenmp", f"-I{ORACLE_DIR}", f"-I{SYSTEMS_DIR}",
           *_coupled_macros(system), str(src), "-o", str(out)]
    _run(cmd, out.name)
    return out


# Reference coupled kernels built as cubins: (system, algorithm, NS, TPB, SPB,
# NDO), all with SPB * UPS == TPB and NS a multiple of SPB, so that the
# reference's unit layout has no thread padding and coincides with the GB300
# layout. The 16384-system ring64 cubins serve the full-size parity test and
# the reference-kernel timing (two launch shapes: 2 and 4 systems per block).
REF_GPU_CB_KERNELS = [
    ("ring16_full", 1, 256, 64, 4, 0), ("ring16_band", 1, 256, 64, 4, 0), ("ring16_circband", 1, 256, 64, 4, 0),
    ("ring16_circ", 1, 256, 64, 4, 0), ("ring16_full", 0, 256, 64, 4, 0), ("ring16_full", 1, 256, 64, 4, 8),
    ("ring64", 1, 512, 128, 2, 0), ("ring64", 1, 16384, 128, 2, 0), ("ring64", 1, 16384, 256, 4, 0),
    # the reference's three other coupled kernels (variant chosen from SPB, UPS, TPB as its Solve() does):
    # SingleSystem_SingleBlockLaunch, SingleSystem_MultipleBlockLaunches, MultipleSystems_MultipleBlockLaunches
    ("ring64", 1, 512, 64, 1, 0), ("ring64", 1, 512, 32, 1, 0), ("ring64", 1, 512, 64, 2, 0),
    ("ring64", 0, 512, 32, 1, 0),
    # 256 units per system: more units than threads per block (SingleSystem_MultipleBlockLaunches)
    # and one 256-thread block per system (SingleSystem_SingleBlockLaunch)
    ("ring256", 1, 64, 128, 1, 0), ("ring256", 1, 64, 256, 1, 0),
]


def ref_cb_cubin(system: str, algorithm: int, ns: int, tpb: int, spb: int, ndo: int) -> Path:
    alg = "rkck45" if algorithm else "rk4"
    return REF_DIR / f"ref_gpu_cb_{system}_{alg}_ns{ns}_tpb{tpb}_spb{spb}_ndo{ndo}.cubin"


def build_ref_gpu_coupled(system: str, algorithm: int, ns: int, tpb: int, spb: int, ndo: int,
                          force: bool = False) -> Path | None:
    if not (REFERENCE_ROOT / "SourceCodes" / "CoupledSystmes_PerBlock_Solver.cuh").exists():
        return None
    out = ref_cb_cubin(system, algorithm, ns, tpb, spb, ndo)
    src = ORACLE_DIR / "ref_gpu_coupled_entry.cu"
    d = coupled_defs(system)
    deps = [src, SYSTEMS_DIR / d["header"], SYSTEMS_DIR / f"{system}.cu", ORACLE_DIR / "ref_types_coupled.hpp",
            Path(__file__)]
    if not force and _newer(out, deps):
        return out
    cmd = ["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-lineinfo", "-w",
           f"-I{ORACLE_DIR}", f"-I{SYSTEMS_DIR}", f"-I{REFERENCE_ROOT / 'SourceCodes'}", *_coupled_macros(system),
           f"-DREF_NS={ns}", f"-DREF_TPB={tpb}", f"-DREF_SPB={spb}", f"-DREF_NDO={ndo}",
           f"-DREF_ALG={'RKCK45' if algorithm else 'RK4'}", str(src), "-o", str(out)]
    _run(cmd, out.name)
    return out


def oracle_lib(system: str, fma: bool = False) -> Path:
    return BUILD_DIR / f"liboracle_{'fma_' if fma else ''}{system}.so"


def _fma_flags() -> list:
    import platform
    flags = [f for f in FLAGS if f != "-ffp-contract=off"] + ["-ffp-contract=fast"]
    if platform.machine() in ("x86_64", "AMD64"):
        flags.append("-mfma")
    return flags


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


def build_oracle(system: str, force: bool = False, fma: bool = False) -> Path:
    out = oracle_lib(system, fma)
    src = ORACLE_DIR / "oracle_perthread.cpp"
    hdr = SYSTEMS_DIR / f"{system}.cuh"
    if not force and _newer(out, [src, hdr, ORACLE_DIR / "host_shim.hpp", Path(__file__)]):
        return out
    cmd = ["g++", *(_fma_flags() if fma else FLAGS), "-fopenmp", f"-I{ORACLE_DIR}", f"-I{SYSTEMS_DIR}",
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


# Reference GPU kernels built as cubins: (system, algorithm, NT, NDO). The
# reference's NT and NDO are template arguments, so every ensemble size the
# tests and the bench compare against is listed. For keller_miksis (SD = 2 >
# NE = 1) the unmodified reference kernel indexes its event-option arrays by
# component (SingleSystem_PerThread_Solver.cuh:60: `ltid < SD`), which reads
# past the NE-entry device array and writes past the NE-entry shared array;
# it is never built. Systems listed in REF_GPU_EVENT_FIX are built instead
# from a temporary copy of the reference sources (outside this repository)
# in which only that condition reads `ltid < NE`.
REF_GPU_EVENT_FIX = {"keller_miksis"}
REF_GPU_KERNELS = [
    ("keller_miksis", 1, 64, 0), ("keller_miksis", 1, 256, 0), ("keller_miksis", 1, 65536, 0),
    ("lorenz", 1, 256, 0), ("lorenz", 1, 1000, 0), ("lorenz", 0, 64, 0), ("lorenz", 1, 1 << 20, 0),
    ("duffing", 0, 64, 0), ("duffing", 0, 8192, 0),
    ("duffing_param", 1, 256, 0), ("duffing_param", 1, 1000, 0),
    ("duffing_events", 1, 64, 16), ("duffing_events", 1, 512, 16),
    ("bouncing_ball", 1, 64, 0), ("bouncing_ball", 1, 300, 0),
]
# Register caps of the reference's own makefiles (T2_Lorenz/makefile: 64).
REF_GPU_RREG = {"lorenz": 64}


def ref_cubin(system: str, algorithm: int, nt: int, ndo: int, rreg: int | None = None) -> Path:
    tag = f"_rr{rreg}" if rreg else ""
    return REF_DIR / f"ref_gpu_{system}_{'rkck45' if algorithm else 'rk4'}_nt{nt}_ndo{ndo}{tag}.cubin"


def build_ref_gpu(system: str, algorithm: int, nt: int, ndo: int, rreg: int | None = None,
                  force: bool = False) -> Path | None:
    if not reference_available():
        return None
    out = ref_cubin(system, algorithm, nt, ndo, rreg)
    src = ORACLE_DIR / "ref_gpu_entry.cu"
    hdr = SYSTEMS_DIR / f"{system}.cuh"
    if not force and _newer(out, [src, hdr, ORACLE_DIR / "ref_types.hpp", Path(__file__)]):
        return out
    src_dir, tmp = REFERENCE_ROOT / "SourceCodes", None
    if system in REF_GPU_EVENT_FIX:
        tmp, src_dir = _event_fixed_sources()
        if src_dir is None:
            return None
    cmd = ["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-lineinfo", "-w",
           f"-I{ORACLE_DIR}", f"-I{SYSTEMS_DIR}", f"-I{src_dir}",
           f'-DMPGOS_SYSTEM_HEADER="{system}.cuh"', f"-DREF_NT={nt}", f"-DREF_ALG={'RKCK45' if algorithm else 'RK4'}",
           f"-DREF_NDO={ndo}"]
    if rreg:
        cmd.append(f"-maxrregcount={rreg}")
    cmd += [str(src), "-o", str(out)]
    try:
        _run(cmd, out.name)
    finally:
        if tmp is not None:
            import shutil
            shutil.rmtree(tmp, ignore_errors=True)
    return out


def _event_fixed_sources():
    """Copy the reference's SourceCodes to a temporary directory and change the
    event-option staging condition of SingleSystem_PerThread_Solver.cuh from
    `ltid < SD` to `ltid < NE` (the only change). Returns (temporary
    directory, patched SourceCodes path), or (None, None) if the line is not
    found as expected."""
    import shutil
    import tempfile
    tmp = Path(tempfile.mkdtemp(prefix="mpgos_ref_evfix_"))
    dst = tmp / "SourceCodes"
    shutil.copytree(REFERENCE_ROOT / "SourceCodes", dst)
    f = dst / "SingleSystem_PerThread_Solver.cuh"
    lines = f.read_text().split("\n")
    hits = [i for i, l in enumerate(lines) if l.strip() == "if ( ltid < SD)" and "EventTolerance" in "".join(lines[i:i + 4])]
    if len(hits) != 1:
        shutil.rmtree(tmp, ignore_errors=True)
        return None, None
    lines[hits[0]] = lines[hits[0]].replace("ltid < SD", "ltid < NE")
    f.write_text("\n".join(lines))
    return tmp, dst


def build_all(force: bool = False) -> dict:
    BUILD_DIR.mkdir(exist_ok=True)
    REF_DIR.mkdir(exist_ok=True)
    res = {}
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        futs = {}
        for s in SYSTEMS:
            futs[ex.submit(build_oracle, s, force)] = ("oracle", s)
            futs[ex.submit(build_oracle, s, force, True)] = ("oracle_fma", s)
            futs[ex.submit(build_ref, s, force)] = ("ref", s)
        for s in COUPLED:
            futs[ex.submit(build_oracle_coupled, s, force)] = ("oracle_cb", s)
            futs[ex.submit(build_oracle_coupled, s, force, True)] = ("oracle_cb_fma", s)
        for k in REF_GPU_CB_KERNELS:
            futs[ex.submit(build_ref_gpu_coupled, *k, force)] = ("ref_gpu_cb", *k)
        for (s, alg, nt, ndo) in REF_GPU_KERNELS:
            futs[ex.submit(build_ref_gpu, s, alg, nt, ndo, None, force)] = ("ref_gpu", s, alg, nt, ndo)
            if s in REF_GPU_RREG:
                rr = REF_GPU_RREG[s]
                futs[ex.submit(build_ref_gpu, s, alg, nt, ndo, rr, force)] = ("ref_gpu", s, alg, nt, ndo, rr)
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
