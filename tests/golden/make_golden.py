"""Generate the golden fixtures of tests/golden/ from the reference itself.

Each fixture is the reference's own per-thread solver kernel
(SourceCodes/SingleSystem_PerThread_Solver.cuh and the headers it includes,
compiled for the CPU by oracle/build_oracle.py into oracle/_ref/) run on a
small seeded ensemble of one of the hook files in systems/. The file stores
the complete inputs (SoA arrays, tolerances, options, number of launches)
and the complete outputs, so tests can replay the inputs through the oracle
or the GPU solver without depending on the case builders.

Run from the repository root, where the reference checkout is present:
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "massively-parallel-gpu-ode-solver_gb300"))

from mpgos_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402


def cases():
    c = W.lorenz_case(nt=256)
    yield "lorenz_rkck45_256", c
    c = W.lorenz_case(nt=64, tol=1e-6)
    c.algorithm = 0
    c.options["initial_dt"] = 1e-3
    yield "lorenz_rk4_64", c
    yield "duffing_rk4_64x8", W.duffing_rk4_case(nt=64, periods=8)
    yield "duffing_param_rkck45_256", W.duffing_param_case(nt=256, periods=4)
    yield "duffing_events_dense_64x3", W.duffing_events_case(nt=64, periods=3, ndo=16)
    yield "duffing_events_stop_64", W.duffing_events_case(nt=64, periods=2, ndo=16, stop_after=3, seed=9)
    yield "bouncing_ball_64", W.bouncing_ball_case(nt=64)
    yield "keller_miksis_8x8x2", W.keller_miksis_case(n_amp=8, n_freq=8, periods=2)


def save(name: str, case, out: dict) -> None:
    meta = dict(system=case.system, algorithm=case.algorithm, nt=case.nt, ndo=case.ndo, phases=case.phases,
                n_active=case.n_active, options=case.options)
    arrays = {f"in_{k}": v for k, v in case.arrays.items()}
    arrays.update(rtol=case.rtol, atol=case.atol, etol=case.etol, edir=case.edir)
    arrays.update({f"out_{k}": np.asarray(v) for k, v in out.items() if k not in ("status", "nacc", "nrej")})
    np.savez_compressed(HERE / f"{name}.npz", meta=np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8),
                        **arrays)


def load(path: Path):
    """(case, outputs) of a fixture."""
    z = np.load(path)
    meta = json.loads(bytes(z["meta"]).decode())
    c = W.empty_case(meta["system"], meta["algorithm"], meta["nt"], meta["ndo"])
    c.phases = meta["phases"]
    c.n_active = meta["n_active"]
    c.options = meta["options"]
    for k in list(c.arrays):
        c.arrays[k] = z[f"in_{k}"]
    c.rtol, c.atol, c.etol, c.edir = z["rtol"], z["atol"], z["etol"], z["edir"]
    out = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
    return c, out


def main():
    for name, case in cases():
        out = O.run_ref_cpu(case)
        save(name, case, out)
        print(f"{name}: {case.system} nt={case.nt} phases={case.phases} "
              f"accepted(sum of counters)={int(np.asarray(out['acci'])[-1].sum())}")


if __name__ == "__main__":
    main()
