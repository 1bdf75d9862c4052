"""Text files of Print in the reference's formats (the Python side of
include/mpgos/dropin_print.h; both write byte-identical files).

Every value as an ofstream with width 18, precision 10 and std::scientific
writes it (integers unaffected by the floating-point flags); arrays are given
as numpy arrays [column][row].
  general        per-thread Print(variable): values separated by ','
                 (SingleSystem_PerThread_Interface.cuh:1083-1108);
  system_scope   coupled system/global scope: every value followed by ','
                 (CoupledSystems_PerBlock_Interface.cuh:1571-1596);
  unit_scope     coupled unit scope in the reference's padded logical-thread
                 rows for a TPB / SPB launch shape, padding as "PADDING"
                 (:1529-1569);
  perthread_dense, coupled_dense   Print(DenseOutput, serial).
"""
from __future__ import annotations

import numpy as np


def value(v) -> str:
    if isinstance(v, (int, np.integer)):
        return f"{int(v):18d}"
    if isinstance(v, str):
        return f"{v:>18}"
    return f"{float(v):18.10e}"


def _rows(data) -> np.ndarray:
    a = np.asarray(data)
    return a.reshape(1, -1) if a.ndim == 1 else a


def general(path: str, data) -> None:
    cols = _rows(data)
    with open(path, "w") as f:
        for i in range(cols.shape[1]):
            f.write(",".join(value(c[i]) for c in cols) + "\n")


def system_scope(path: str, data) -> None:
    cols = _rows(data)
    with open(path, "w") as f:
        for i in range(cols.shape[1]):
            f.write("".join(value(c[i]) + "," for c in cols) + "\n")


def layout(ns: int, ups: int, tpb: int, spb: int):
    """Padded logical-thread rows of the reference
    (CoupledSystems_PerBlock_Interface.cuh:385-390): for every row, the index
    in the unpadded unit layout or -1 for padding."""
    logical = spb * ups
    launches = logical // tpb + (0 if logical % tpb == 0 else 1)
    padding = launches * tpb - logical
    grid = ns // spb + (0 if ns % spb == 0 else 1)
    per = logical + padding
    total = per * grid
    limit = (ns // spb) * per + (ns % spb) * ups
    r = np.arange(total)
    b, l = r // per, r % per
    return np.where((l < logical) & (r < limit), b * spb * ups + l, -1)


def unit_scope(path: str, data, ns: int, ups: int, tpb: int | None = None, spb: int | None = None) -> None:
    cols = _rows(data)
    if tpb is None or spb is None:
        tpb, spb = ups, 1
    rows = layout(ns, ups, tpb, spb)
    with open(path, "w") as f:
        for u in rows:
            if u < 0:
                f.write("".join(value("PADDING") + "," for _ in cols) + "\n")
            else:
                f.write("".join(value(c[u]) + "," for c in cols) + "\n")


def perthread_dense(path: str, tid: int, cp, sp, spi, acc, acci, didx: int, dtime, dstate) -> None:
    """cp [NCP][NT], sp [NSP], spi [NISP], acc [NA][NT], acci [NIA][NT],
    dtime [NDO][NT], dstate [NDO][SD][NT]."""
    def row(title, vals):
        return [title, ",".join(value(v) for v in vals)]
    lines = (row("ControlParameters:", np.asarray(cp)[:, tid]) + row("SharedParameters:", sp) +
             row("IntegerSharedParameters:", spi) + row("Accessories:", np.asarray(acc)[:, tid]) +
             row("IntegerAccessories:", np.asarray(acci)[:, tid]) + ["", "Time series:"])
    dtime, dstate = np.asarray(dtime), np.asarray(dstate)
    for i in range(min(int(didx), dtime.shape[0])):
        lines.append(value(dtime[i, tid]) + "," + ",".join(value(v) for v in dstate[i, :, tid]))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def coupled_dense(path: str, sid: int, ups: int, up, uacc, iuacc, sp, sacc, isacc, gp, igp, didx: int, dtime,
                  dstate) -> None:
    """Unit arrays [field][NS*UPS], system arrays [field][NS], gp [NGP],
    igp [NiGP], dtime [NDO][NS], dstate [NDO][UD][NS*UPS]."""
    base = sid * ups
    out = []

    def units(title, data):
        data = np.asarray(data)
        out.append(title)
        out.append(value("Serial No.") + "," + ",".join(value(f"U{u}") for u in range(ups)))
        for k in range(data.shape[0]):
            out.append(value(k) + "," + ",".join(value(v) for v in data[k, base:base + ups]))
        out.append("")

    def plain(title, vals):
        out.append(title)
        out.append(",".join(value(v) for v in vals))
        out.append("")

    units("UnitParameters:", up)
    units("UnitAccessories:", uacc)
    units("IntegerUnitAccessories:", iuacc)
    plain("SystemParameters:", np.asarray(sp)[:, sid])
    plain("SystemAccessories:", np.asarray(sacc)[:, sid])
    plain("IntegerSystemAccessories:", np.asarray(isacc)[:, sid])
    plain("GlobalParameters:", gp)
    plain("IntegerGlobalParameters:", igp)
    dtime, dstate = np.asarray(dtime), np.asarray(dstate)
    ud = dstate.shape[1]
    out.append("Time series:")
    out.append(value("t") + "," + ",".join(value(f"U{u}/C{c}") for u in range(ups) for c in range(ud)))
    for i in range(min(int(didx), dtime.shape[0])):
        out.append(value(dtime[i, sid]) + "," + ",".join(value(dstate[i, c, base + u]) for u in range(ups)
                                                         for c in range(ud)))
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
