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
* ``oracle/_ref/ref_print_check`` - the reference's own Print /
  WriteToFileGeneral (SingleSystem_PerThread_Interface.cuh:1083-1276) built
  for the host (ref_print_entry.cpp), for the byte comparison of the text
  files (tests/test_textout_cpu.py).
* ``oracle/_ref/libref_cpu_<system>.so`` - the reference's own
  SourceCodes/SingleSystem_PerThread_Solver.cuh compiled for the CPU through
  ref_cpu_entry.cpp, straight from the reference checkout (MPGOS_REFERENCE_ROOT,
  else a checkout named ``reference`` beside this repository; elsewhere the
  staged copy of its per-thread headers in the git-ignored baseline/_ref),
  with OpenMP. Built only where those sources exist; used to
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
# The reference's per-thread solver headers, staged by stage_reference_sources()
# from a checkout into this git-ignored directory, which travels with the
# working tree to machines without the checkout (the GPU host), so the
# reference's CPU build can be made there for the CPU baseline.
STAGED_ROOT = REPO_ROOT / "baseline" / "_ref"
STAGED_HEADERS = ["MPGOS_Overloaded_MathFunction.cuh", "SingleSystem_PerThread_Solver.cuh",
                  "SingleSystem_PerThread_DenseOutput.cuh", "SingleSystem_PerThread_ExplicitRungeKutta_Steppers.cuh",
                  "SingleSystem_PerThread_ExplicitRungeKutta_ErrorControllers.cuh",
                  "SingleSystem_PerThread_EventHandling.cuh", "SingleSystem_PerThread_Interface.cuh"]
CHECKOUT_ROOT = Path(os.environ.get("MPGOS_REFERENCE_ROOT", str(REPO_ROOT.parent / "reference")))


def _solver_header(root: Path) -> Path:
    return root / "SourceCodes" / "SingleSystem_PerThread_Solver.cuh"


# the checkout where it exists, else the staged headers (CPU builds only)
REFERENCE_ROOT = CHECKOUT_ROOT if _solver_header(CHECKOUT_ROOT).exists() else STAGED_ROOT


def full_checkout() -> bool:
    """The reference checkout itself (not the staged copy) is present: the
    GPU cubins and the coupled builds need it."""
    return _solver_header(CHECKOUT_ROOT).exists()


def stage_reference_sources() -> Path | None:
    """Copy the reference's per-thread solver headers from the checkout into
    baseline/_ref/SourceCodes (git-ignored), where they differ."""
    if not full_checkout():
        return None
    import shutil
    dst = STAGED_ROOT / "SourceCodes"
    dst.mkdir(parents=True, exist_ok=True)
    for name in STAGED_HEADERS:
        src = CHECKOUT_ROOT / "SourceCodes" / name
        out = dst / name
        if not out.exists() or out.read_bytes() != src.read_bytes():
            shutil.copyfile(src, out)
    return dst

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
    if not full_checkout():
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
    return _solver_header(REFERENCE_ROOT).exists()


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
    # -fno-extern-tls-init: the kernel's `extern __shared__` (thread_local here)
    # array is statically initialised; no TLS init wrapper is needed or emitted
    cmd = ["g++", *FLAGS, "-fopenmp", "-fno-extern-tls-init", "-w", f"-I{ORACLE_DIR}", f"-I{SYSTEMS_DIR}",
           f"-I{REFERENCE_ROOT / 'SourceCodes'}", f'-DMPGOS_SYSTEM_HEADER="{system}.cuh"',
           *([f"-DMPGOS_REF_NT_EXTRA={REF_CPU_NT_EXTRA[system]}"] if system in REF_CPU_NT_EXTRA else []),
           str(src), "-o", str(out)]
    _run(cmd, out.name)
    return out


# Extra ensemble sizes of the reference CPU build (RKCK45, no dense output):
# the CPU-baseline samples of the 2^20 Lorenz ensemble (every 16th and every
# 8th instance).
REF_CPU_NT_EXTRA = {"lorenz": "X(65536) X(131072)"}


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
    ("keller_miksis", 1, 1 << 18, 0),
    ("lorenz", 1, 256, 0), ("lorenz", 1, 1000, 0), ("lorenz", 0, 64, 0), ("lorenz", 1, 1 << 20, 0),
    ("duffing", 0, 64, 0), ("duffing", 0, 8192, 0),
    ("duffing_param", 1, 256, 0), ("duffing_param", 1, 1000, 0),
    ("duffing_events", 1, 64, 16), ("duffing_events", 1, 512, 16),
    ("bouncing_ball", 1, 64, 0), ("bouncing_ball", 1, 300, 0),
]
# Register caps of the reference's own makefiles (T2_Lorenz/makefile: 64).
REF_GPU_RREG = {"lorenz": 64}
# Launch-shape sweep of the reference kernel (the timing baselines): the
# reference stages its tolerances and event options into shared memory with
# no barrier before other warps read them (SingleSystem_PerThread_Solver.cuh:
# 37-88), which is harmless only with one warp per block, its default. These
# cubins are built from a temporary copy of the reference sources with one
# __syncthreads() added after that staging (nothing else changed), so that
# blocks of 64..256 threads read defined tolerances; (system, algorithm, NT,
# NDO, register cap or None).
REF_GPU_SYNC_KERNELS = [
    ("lorenz", 1, 1 << 20, 0, None), ("lorenz", 1, 1 << 20, 0, 64),
    ("keller_miksis", 1, 1 << 18, 0, None), ("duffing", 0, 8192, 0, None),
]


def ref_cubin(system: str, algorithm: int, nt: int, ndo: int, rreg: int | None = None, sync: bool = False) -> Path:
    tag = (f"_rr{rreg}" if rreg else "") + ("_sync" if sync else "")
    return REF_DIR / f"ref_gpu_{system}_{'rkck45' if algorithm else 'rk4'}_nt{nt}_ndo{ndo}{tag}.cubin"


def build_ref_gpu(system: str, algorithm: int, nt: int, ndo: int, rreg: int | None = None,
                  force: bool = False, sync: bool = False) -> Path | None:
    if not full_checkout():
        return None
    out = ref_cubin(system, algorithm, nt, ndo, rreg, sync)
    src = ORACLE_DIR / "ref_gpu_entry.cu"
    hdr = SYSTEMS_DIR / f"{system}.cuh"
    if not force and _newer(out, [src, hdr, ORACLE_DIR / "ref_types.hpp", Path(__file__)]):
        return out
    src_dir, tmp = REFERENCE_ROOT / "SourceCodes", None
    if system in REF_GPU_EVENT_FIX or sync:
        tmp, src_dir = _patched_sources(event_fix=system in REF_GPU_EVENT_FIX, barrier=sync)
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


def _patched_sources(event_fix: bool, barrier: bool):
    """Copy the reference's SourceCodes to a temporary directory and patch
    SingleSystem_PerThread_Solver.cuh there: with ``event_fix`` the
    event-option staging condition reads `ltid < NE` instead of `ltid < SD`;
    with ``barrier`` one `__syncthreads();` goes in front of the per-instance
    part of the kernel (`if (tid < ThreadConfiguration.NumberOfActiveThreads)`),
    after the shared-memory staging, which every thread of a block reaches.
    Nothing else changes. Returns (temporary directory, patched SourceCodes
    path), or (None, None) if a line is not found exactly once."""
    import shutil
    import tempfile
    tmp = Path(tempfile.mkdtemp(prefix="mpgos_ref_patch_"))
    dst = tmp / "SourceCodes"
    shutil.copytree(REFERENCE_ROOT / "SourceCodes", dst)
    f = dst / "SingleSystem_PerThread_Solver.cuh"
    lines = f.read_text().split("\n")
    if event_fix:
        hits = [i for i, l in enumerate(lines)
                if l.strip() == "if ( ltid < SD)" and "EventTolerance" in "".join(lines[i:i + 4])]
        if len(hits) != 1:
            shutil.rmtree(tmp, ignore_errors=True)
            return None, None
        lines[hits[0]] = lines[hits[0]].replace("ltid < SD", "ltid < NE")
    if barrier:
        hits = [i for i, l in enumerate(lines) if l.strip() == "if (tid < ThreadConfiguration.NumberOfActiveThreads)"]
        if len(hits) != 1:
            shutil.rmtree(tmp, ignore_errors=True)
            return None, None
        lines.insert(hits[0], "\t__syncthreads();")
    f.write_text("\n".join(lines))
    return tmp, dst


def ref_print_exe() -> Path:
    return REF_DIR / "ref_print_check"


def build_ref_print(force: bool = False) -> Path | None:
    """The reference's WriteToFileGeneral and Print member definitions
    (SingleSystem_PerThread_Interface.cuh:1083-1276), copied unchanged from
    its header into oracle/_ref/ref_print_members.inc, compiled on the host
    with ref_print_entry.cpp (which declares the class they belong to)."""
    hdr = REFERENCE_ROOT / "SourceCodes" / "SingleSystem_PerThread_Interface.cuh"
    if not hdr.exists():
        return None
    out = ref_print_exe()
    src = ORACLE_DIR / "ref_print_entry.cpp"
    if not force and _newer(out, [src, hdr, Path(__file__)]):
        return out
    lines = hdr.read_text().split("\n")
    start = [i for i, l in enumerate(lines) if "::WriteToFileGeneral(std::string FileName" in l]
    if len(start) != 1:
        return None
    first = start[0] - 2   # the two template lines of the definition
    end = [i for i in range(first, len(lines)) if lines[i].strip().startswith("// SOLVE")]
    if not end or not lines[first].startswith("template <int NT"):
        return None
    frag = "\n".join(lines[first:end[0]])
    if "::Print(ListOfVariables Variable, int ThreadID)" not in frag:
        return None
    REF_DIR.mkdir(exist_ok=True)
    (REF_DIR / "ref_print_members.inc").write_text(frag + "\n")
    _run(["g++", "-O1", "-std=c++17", "-w", f"-I{REF_DIR}", str(src), "-o", str(out)], out.name)
    return out


def build_all(force: bool = False) -> dict:
    BUILD_DIR.mkdir(exist_ok=True)
    REF_DIR.mkdir(exist_ok=True)
    stage_reference_sources()
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
        futs[ex.submit(build_ref_print, force)] = ("ref_print",)
        for (s, alg, nt, ndo, rr) in REF_GPU_SYNC_KERNELS:
            futs[ex.submit(build_ref_gpu, s, alg, nt, ndo, rr, force, True)] = ("ref_gpu_sync", s, alg, nt, ndo, rr)
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
