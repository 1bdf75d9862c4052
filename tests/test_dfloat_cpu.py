"""CPU test of the double-float arithmetic of the DF_STAGE mode
(csrc/perthread/dfloat.cuh), built for the host from the same header."""
import subprocess

import pytest

from tests.conftest import REPO

HEADER_DIR = REPO / "massively-parallel-gpu-ode-solver_gb300" / "csrc" / "perthread"


@pytest.fixture(scope="module")
def errors(tmp_path_factory):
    exe = tmp_path_factory.mktemp("dfloat") / "dfloat_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{HEADER_DIR}",
                    str(REPO / "tests" / "dfloat_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {k: float(v) for k, v in (line.split() for line in out.strip().splitlines())}


def test_double_float_precision(errors):
    # ~48 significant bits: 2^-46 = 1.4e-14 covers every operation's bound
    for op in ("add", "mul", "div", "sqrt", "fma"):
        assert errors[op] < 1.5e-14, (op, errors[op])
    assert errors["dot2"] < 2.5e-14, errors["dot2"]   # two products' tails, relative to |ab| + |cd|
    # five-term unnormalised product sums, relative to the sum of the terms' magnitudes
    assert errors["prod_sum"] < 5e-14, errors["prod_sum"]
    assert errors["prod_sum_axpy"] < 7e-14, errors["prod_sum_axpy"]
    assert errors["cvt"] < 4e-15          # double -> double-float keeps 48 bits (2^-48)


def test_double_float_sine_cosine(errors):
    # FP32-pipe sin/cos: within a few times the argument's own double-float
    # precision (|x| 2^-48 + 2^-50) up to |x| = 2000, ~1e-14 absolute for |x| < 1
    assert errors["trig"] < 4.0, errors["trig"]
    assert errors["trig_small"] < 2e-14, errors["trig_small"]
    # sincospi reduces by halves exactly: absolute error of the kernels alone, any |x| <= 2000
    assert errors["trigpi"] < 2e-14, errors["trigpi"]


def test_double_float_exp_log_pow(errors):
    # FP32-pipe exp / log / pow: within a few units of 2^-48 (|x| + 1), the
    # precision the argument carries (x = the exponent, log a, b log a)
    assert errors["exp"] < 2.5, errors["exp"]
    assert errors["log"] < 3.0, errors["log"]
    assert errors["pow"] < 10.0, errors["pow"]
    assert errors["pow_int"] < 1e-13, errors["pow_int"]    # repeated squaring, |n| <= 6
    assert errors["fallback"] == 0                           # out-of-range arguments: the FP64 functions


def test_double_float_invariants(errors):
    assert errors["cmp"] == 0             # comparisons order like the exact values
    assert errors["norm"] <= 0.5          # |lo| <= ulp(hi) / 2 after every operation


@pytest.fixture(scope="module")
def conversions(tmp_path_factory):
    exe = tmp_path_factory.mktemp("df_convert") / "df_convert_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{HEADER_DIR}",
                    str(REPO / "tests" / "df_convert_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {k: float(v) for k, v in (line.split() for line in out.strip().splitlines())}


def test_integer_pipe_conversions(conversions):
    """FP64 <-> double-float conversions of the precision split
    (df_convert.cuh): widen is the exact float->double conversion, to_double
    the nearest double to hi + lo, split keeps 47+ bits and normalises."""
    assert conversions["widen_mismatches"] == 0
    assert conversions["to_double_mismatches"] == 0
    assert conversions["split_bound_violations"] == 0
    assert conversions["split_max_rel_err"] <= 2.0 ** -47
    assert conversions["split_unnormalised"] == 0
    assert conversions["range_mismatches"] == 0


def test_split_step_factor_is_fp64_accurate(conversions):
    """0.9 R^(1/5) / R^(1/4) of the split controller: the FP32 estimate
    corrected in FP64 lands within a few ulp of the exact root (CUDA's FP64
    pow is specified to 2 ulp)."""
    assert conversions["root_max_ulp"] <= 4.0, conversions["root_max_ulp"]


def _trig_table():
    """The committed table of sin / cos (j pi/128) as numbers: {name: [64 x k] floats}."""
    import re
    text = (HEADER_DIR / "dfloat_trig_table.h").read_text()
    out = {}
    for name in ("MAIN", "TAIL"):
        body = text.split(f"#define MPGOS_DF_TRIG_TABLE_{name}")[1].split("#define")[0]
        rows = re.findall(r"\{([^}]*)\}", body)
        out[name] = [[float.fromhex(v.strip()[:-1]) for v in r.split(",")] for r in rows]
    return out


def test_trig_table_entries_are_triple_float_sines_and_cosines():
    """sin(j pi/128) and cos(j pi/128), j = 0..63: hi + lo + lo2 within 4e-19 of
    the long double values (the table carries ~72 bits; an x86 long double
    angle and sine carry 64, a few 1e-20 here), every part a float and |lo| at
    most half an ulp of hi."""
    import numpy as np
    t = _trig_table()
    assert len(t["MAIN"]) == 64 and len(t["TAIL"]) == 64
    pi = np.longdouble("3.14159265358979323846264338327950288")
    for j, (m, tail) in enumerate(zip(t["MAIN"], t["TAIL"])):
        a = pi * j / np.longdouble(128)
        for (hi, lo, lo2), f in (((m[0], m[1], tail[0]), np.sin), ((m[2], m[3], tail[1]), np.cos)):
            exact = f(a)
            got = np.longdouble(hi) + np.longdouble(lo) + np.longdouble(lo2)
            assert abs(got - exact) <= 4e-19, (j, float(got - exact))
            assert np.float32(hi) == hi and np.float32(lo) == lo and np.float32(lo2) == lo2
            if hi != 0.0:
                assert abs(lo) <= np.spacing(np.float32(abs(hi))) / 2, (j, hi, lo)


def test_trig_table_is_what_the_generator_writes():
    pytest.importorskip("mpmath")
    gen = HEADER_DIR / "gen_dfloat_trig_table.py"
    out = subprocess.run(["python3", str(gen)], check=True, capture_output=True, text=True).stdout
    assert out == (HEADER_DIR / "dfloat_trig_table.h").read_text()


@pytest.mark.parametrize("bounded", [False, True], ids=["default", "bounded"])
def test_bounded_trig_is_the_table_path_or_nan(tmp_path, bounded):
    """MPGOS_DF_TRIG_BOUNDED: inside the bounds (|x| < 2^14 for sin/cos,
    2^16 for sincospi) the branch-free forms give the table path's bits, outside
    (and for infinities and NaN) NaN in both parts; with the macro defined the
    public sin, cos, sincos and sincospi are those forms."""
    exe = tmp_path / "dfloat_bounded_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{HEADER_DIR}",
                    *(["-DMPGOS_DF_TRIG_BOUNDED"] if bounded else []),
                    str(REPO / "tests" / "dfloat_bounded_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = {k: int(v) for k, v in (line.split() for line in out.strip().splitlines())}
    assert got["bounded_in_differs"] == 0
    assert got["bounded_out_not_nan"] == 0
    assert got["public_differs"] == 0
    assert got["inside"] > 100000 and got["outside"] > 10000
