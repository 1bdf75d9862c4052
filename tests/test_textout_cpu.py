"""The Print text formats: the C++ writers of the drop-in headers
(include/mpgos/dropin_print.h, compiled here with g++) and the Python ones
(mpgos_gb300.textout) produce byte-identical files for the same arrays; the
per-thread files are byte-identical to the ones the reference's own Print
writes (its member functions compiled for the host from its header,
oracle/ref_print_entry.cpp); and spot checks of the reference's layout
(width 18, precision 10, scientific; trailing commas in the coupled files;
PADDING rows of a padded launch)."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from mpgos_gb300 import textout as T

REPO = Path(__file__).resolve().parent.parent


def val(k):
    return (k % 7 - 3) * 1.2345678901234 * 10.0 ** (k % 9 - 4)


def dv(n, off):
    return np.array([val(i + off) for i in range(n)])


def iv(n, off):
    return np.array([(i + off) * 37 % 101 - 50 for i in range(n)], dtype=np.int32)


@pytest.fixture(scope="module")
def cpp_files(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("textout_cpp")
    exe = d / "textout_check"
    subprocess.run([gxx, "-O1", "-std=c++17", f"-I{REPO / 'include' / 'mpgos'}", str(REPO / "tests" / "textout_check.cpp"),
                    "-o", str(exe)], check=True)
    subprocess.run([str(exe), str(d)], check=True)
    return d


def test_python_and_cpp_writers_agree(cpp_files, tmp_path):
    nt, sd = 4, 3
    x = dv(sd * nt, 1).reshape(sd, nt)
    ia = iv(2 * nt, 3).reshape(2, nt)
    T.general(tmp_path / "general_double.txt", x)
    T.general(tmp_path / "general_int.txt", ia)
    cp, sp, acc = dv(2 * nt, 20).reshape(2, nt), dv(2, 30), dv(nt, 40).reshape(1, nt)
    dt, ds = dv(5 * nt, 50).reshape(5, nt), dv(5 * sd * nt, 80).reshape(5, sd, nt)
    T.perthread_dense(tmp_path / "pt_dense.txt", 2, cp, sp, iv(1, 7), acc, ia, 3, dt, ds)
    ns, ups, ud = 5, 3, 2
    nu = ns * ups
    xs = dv(ud * nu, 200).reshape(ud, nu)
    iua = iv(nu, 11).reshape(1, nu)
    T.system_scope(tmp_path / "system_double.txt", dv(2 * ns, 300).reshape(2, ns))
    T.system_scope(tmp_path / "system_int.txt", iv(ns, 5).reshape(1, ns))
    T.unit_scope(tmp_path / "unit_double.txt", xs, ns, ups, 4, 2)
    T.unit_scope(tmp_path / "unit_int.txt", iua, ns, ups, 4, 2)
    T.unit_scope(tmp_path / "unit_unpadded.txt", xs, ns, ups)
    T.coupled_dense(tmp_path / "cb_dense.txt", 1, ups, dv(2 * nu, 400).reshape(2, nu), dv(nu, 450).reshape(1, nu),
                    iua, dv(ns, 500).reshape(1, ns), dv(2 * ns, 520).reshape(2, ns), iv(ns, 9).reshape(1, ns),
                    dv(2, 540), iv(1, 13), 4, dv(4 * ns, 600).reshape(4, ns), dv(4 * ud * nu, 700).reshape(4, ud, nu))
    names = sorted(p.name for p in cpp_files.glob("*.txt"))
    assert len(names) == 9
    for n in names:
        assert (tmp_path / n).read_bytes() == (cpp_files / n).read_bytes(), n


def test_reference_layout_spot_checks(cpp_files):
    lines = (cpp_files / "general_double.txt").read_text().splitlines()
    assert lines[0] == ",".join(f"{val(1 + 0 + j * 4):18.10e}" for j in range(3))
    assert len(lines[0].split(",")[0]) == 18
    sys_lines = (cpp_files / "system_int.txt").read_text().splitlines()
    assert all(l.endswith(",") for l in sys_lines)
    # 5 systems of 3 units, 2 systems per block, 4 threads: blocks of 6 logical
    # threads padded to 8, 3 blocks = 24 rows; the last block holds one system
    unit = (cpp_files / "unit_double.txt").read_text().splitlines()
    assert len(unit) == 24
    pad = [i for i, l in enumerate(unit) if "PADDING" in l]
    assert pad == [6, 7, 14, 15] + list(range(19, 24))
    assert len((cpp_files / "unit_unpadded.txt").read_text().splitlines()) == 15
    dense = (cpp_files / "cb_dense.txt").read_text().splitlines()
    assert dense[0] == "UnitParameters:" and "Time series:" in dense
    t = dense.index("Time series:")
    assert len(dense) - t - 2 == 4      # header line + 4 stored points of system 1


def test_per_thread_files_match_the_reference_print(cpp_files, tmp_path):
    """SingleSystem_PerThread_Interface.cuh:1083-1276 (the reference's
    WriteToFileGeneral and Print, built for the host) against the drop-in
    writers on the same arrays: the general layout for a double and an int
    variable, and the dense-output file of one thread, byte for byte."""
    import sys
    sys.path.insert(0, str(REPO))
    from oracle import build_oracle
    exe = build_oracle.build_ref_print()
    if exe is None:
        pytest.skip("the reference's SingleSystem_PerThread_Interface.cuh is not available here")
    subprocess.run([str(exe), str(tmp_path)], check=True)
    pairs = {"ActualStateInSolverObject.txt": "general_double.txt",
             "IntegerAccessoriesInSolverObject.txt": "general_int.txt", "DenseOutput_2.txt": "pt_dense.txt"}
    for ref_name, ours in pairs.items():
        assert (tmp_path / ref_name).read_bytes() == (cpp_files / ours).read_bytes(), ref_name
