"""Writes dfloat_trig_table.h: sin(j pi/128) and cos(j pi/128), j = 0..63, as
double-float pairs (hi = the float nearest the value, lo = the float nearest
the remainder) and a third float each (the float nearest what hi + lo
leaves), computed with mpmath at 60 decimal digits.

    python gen_dfloat_trig_table.py > dfloat_trig_table.h
"""
import mpmath
import numpy as np

mpmath.mp.dps = 60


def split(v) -> tuple:
    hi = np.float32(float(v))
    lo = np.float32(float(v - mpmath.mpf(float(hi))))
    lo2 = np.float32(float(v - mpmath.mpf(float(hi)) - mpmath.mpf(float(lo))))
    return float(hi), float(lo), float(lo2)


def hexf(x: float) -> str:
    if x == 0.0:
        return "0.0f"
    mant, exp = float.hex(x).split("p")
    return mant.rstrip("0").rstrip(".") + "p" + exp + "f"


def main() -> None:
    print("// sin(j pi/128), cos(j pi/128) for j = 0..63: double-float pairs")
    print("// {sin hi, sin lo, cos hi, cos lo} and the third floats {sin lo2, cos lo2};")
    print("// written by gen_dfloat_trig_table.py.")
    main, tail = [], []
    for j in range(64):
        a = mpmath.pi * j / 128
        sh, sl, s2 = split(mpmath.sin(a))
        ch, cl, c2 = split(mpmath.cos(a))
        main.append("    {" + ", ".join(hexf(v) for v in (sh, sl, ch, cl)) + "}")
        tail.append("    {" + ", ".join(hexf(v) for v in (s2, c2)) + "}")
    for name, rows in (("MAIN", main), ("TAIL", tail)):
        print(f"#define MPGOS_DF_TRIG_TABLE_{name} \\")
        print(", \\\n".join(rows))


if __name__ == "__main__":
    main()
