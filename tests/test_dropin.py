"""The C++ drop-in interface: reference user programs compile unchanged, and
a reference-style program runs through it on the GPU.

The reference ships no tests; its tutorials are its user programs. Every
per-thread tutorial (Tutorials_SingleSystem_PerThread/T1..T8) is compiled,
unmodified, against include/mpgos/SingleSystem_PerThread_Interface.cuh, and
both coupled tutorials (Tutorials_CoupledSystems_PerBlock/T1, T2) against
include/mpgos/CoupledSystems_PerBlock_Interface.cuh, wherever the reference
checkout is present.
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
COUPLED_TUTORIALS = ["T1_RingOfDuffingOscillators/RingOfDuffingOscillators.cu", "T2_BubbleEnsemble/BubbleEnsemble.cu"]
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


@pytest.mark.skipif(not build_oracle.reference_available(), reason="reference checkout not present")
@pytest.mark.parametrize("tutorial", COUPLED_TUTORIALS, ids=lambda t: t.split("/")[0])
def test_reference_coupled_tutorial_compiles_unchanged(tutorial, tmp_path):
    src = build_oracle.REFERENCE_ROOT / "Tutorials_CoupledSystems_PerBlock" / tutorial
    nvcc([*FLAGS, f"-I{src.parent}", "-c", str(src), "-o", str(tmp_path / "t.o")], tmp_path)


def build_dropin_program(tmp_path: Path, name: str = "lorenz_dropin") -> Path:
    build.build_runtime()
    exe = tmp_path / name
    nvcc([*FLAGS, f"-I{build.SYSTEMS_DIR}", str(REPO / "tests" / "dropin" / f"{name}.cu"),
          f"-L{build.BUILD_DIR}", "-lmpgos_runtime", "-Xlinker", f"-rpath,{build.BUILD_DIR}", "-o", str(exe)],
         tmp_path)
    return exe


def test_dropin_program_builds_and_links(tmp_path):
    assert build_dropin_program(tmp_path).exists()


def test_coupled_dropin_program_builds_and_links(tmp_path):
    assert build_dropin_program(tmp_path, "ring_dropin").exists()


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


@pytest.mark.gpu
def test_coupled_dropin_program_matches_the_c_abi_path(tmp_path, oracle_libs):
    """The coupled drop-in class (kernels instantiated in the user's
    translation unit) gives the same bits as the same inputs through the
    plugin and the Python mirror, and matches the oracle."""
    from mpgos_gb300 import coupled_workloads as CW
    from oracle import oracle as O
    exe = build_dropin_program(tmp_path, "ring_dropin")
    case = CW.ring_case("ring16_full", ns=64, periods=1, seed=31)
    with open(tmp_path / "ring_input.bin", "wb") as f:
        f.write(np.array([0.0, case.arrays["td"][1, 0]]).tobytes())
        f.write(np.ascontiguousarray(case.arrays["x"]).tobytes())
        f.write(np.ascontiguousarray(case.arrays["sp"][0]).tobytes())
        f.write(np.ascontiguousarray(case.arrays["cmat"][0]).tobytes())
    p = subprocess.run([str(exe)], cwd=tmp_path, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=300)
    assert p.returncode == 0, p.stdout[-3000:]
    rows = [l.split() for l in p.stdout.splitlines() if l and l[0].isdigit() and len(l.split()) == 6]
    assert len(rows) == 64 * 16
    x = np.array([[float(r[2]) for r in rows], [float(r[3]) for r in rows]])
    crossings = np.array([int(r[4]) for r in rows])
    steps = np.array([int(r[5]) for r in rows]).reshape(64, 16)[:, 0]
    res = CW.run_coupled_gpu(case, mode=0, warps=4)
    assert np.array_equal(x.view(np.uint8), res["x"].view(np.uint8))
    np.testing.assert_array_equal(crossings, res["iuacc"][0])
    np.testing.assert_array_equal(steps, res["isacc"][0])
    ora = O.run_oracle_coupled(case)
    mag = np.max(np.abs(case.arrays["x"]), axis=1, keepdims=True)
    assert np.mean(np.abs(x - ora["x"]) <= 1e-9 * (np.abs(ora["x"]) + mag)) > 0.95
