"""The C++ drop-in interface: reference user programs compile unchanged, and
a reference-style program runs through it on the GPU.

The reference ships no tests; its tutorials are its user programs. Every
per-thread tutorial (Tutorials_SingleSystem_PerThread/T1..T8) is compiled,
unmodified, against include/mpgos/SingleSystem_PerThread_Interface.cuh
wherever the reference checkout is present.
"""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from tests.conftest import REPO
from mpgos_gb300 import build
from oracle import build_oracle

TUTORIALS = ["T1_Reference/Reference.cu", "T2_Lorenz/Lorenz.cu", "T3_PoincareSection/Poincare.cu",
             "T4_QuasiperiodicForcing/QuasiperiodicForcing.cu", "T5_LargeTimeScaleDifferences/KellerMiksis.cu",
             "T6_ImpactDynamics/ImpactDynamics.cu", "T7_DoubleBuffering/DoubleBuffering.cu",
             "T8_MultiGPUSingleNode/MultiGPUSingleNode.cu"]
FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O3",
         f"-I{REPO / 'include' / 'mpgos'}", f"-I{REPO / 'include'}"]


def nvcc(args, cwd):
    p = subprocess.run([build.nvcc_path(), *args], cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True, timeout=600)
    assert p.returncode == 0, p.stdout[-4000:]


@pytest.mark.skipif(not build_oracle.reference_available(), reason="reference checkout not present")
@pytest.mark.parametrize("tutorial", TUTORIALS, ids=lambda t: t.split("/")[0])
def test_reference_tutorial_compiles_unchanged(tutorial, tmp_path):
    src = build_oracle.REFERENCE_ROOT / "Tutorials_SingleSystem_PerThread" / tutorial
    nvcc([*FLAGS, f"-I{src.parent}", "-c", str(src), "-o", str(tmp_path / "t.o")], tmp_path)


def build_dropin_program(tmp_path: Path) -> Path:
    build.build_runtime()
    exe = tmp_path / "lorenz_dropin"
    nvcc([*FLAGS, f"-I{build.SYSTEMS_DIR}", str(REPO / "tests" / "dropin" / "lorenz_dropin.cu"),
          f"-L{build.BUILD_DIR}", "-lmpgos_runtime", "-Xlinker", f"-rpath,{build.BUILD_DIR}", "-o", str(exe)],
         tmp_path)
    return exe


def test_dropin_program_builds_and_links(tmp_path):
    assert build_dropin_program(tmp_path).exists()


@pytest.mark.gpu
def test_dropin_program_matches_oracle(tmp_path, oracle_libs):
    from mpgos_gb300 import workloads as W
    from oracle import oracle as O
    exe = build_dropin_program(tmp_path)
    p = subprocess.run([str(exe)], cwd=tmp_path, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=300)
    assert p.returncode == 0, p.stdout[-3000:]
    rows = [l.split() for l in p.stdout.splitlines() if l and l[0].isdigit() and len(l.split()) == 5]
    assert len(rows) == 256
    x = np.array([[float(r[1]), float(r[2]), float(r[3])] for r in rows]).T
    steps = np.array([int(r[4]) for r in rows])
    ref = O.run_oracle(W.lorenz_case(nt=256))
    np.testing.assert_allclose(x, ref["x"], rtol=1e-9, atol=1e-12)
    np.testing.assert_array_equal(steps, ref["acci"][0])
