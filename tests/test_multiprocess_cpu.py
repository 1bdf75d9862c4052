"""The multi-GPU path on CPU ranks (torch.distributed gloo, world size 2):
contiguous sharding of the ensemble with a host gather of the per-instance
results reproduces the single-process ensemble exactly (instances are
independent: no data-path exchange), and bench.py's max/sum reductions of
the timing scalars work on a gloo group. Each rank integrates its shard with
the CPU oracle (the GPU solver object per rank is the same host code on a
device)."""
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

from mpgos_gb300 import sharding

REPO = Path(__file__).resolve().parent.parent


def test_shard_range_covers_everything_once():
    for n in (0, 1, 7, 64, 1000):
        for world in (1, 2, 3, 8):
            spans = [sharding.shard_range(n, r, world) for r in range(world)]
            idx = np.concatenate([np.arange(f, f + c) for f, c in spans]) if n else np.zeros(0)
            np.testing.assert_array_equal(idx, np.arange(n))
            counts = [c for _, c in spans]
            assert max(counts) - min(counts) <= 1
    with pytest.raises(ValueError):
        sharding.shard_range(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    sys.path[:0] = [str(REPO), str(REPO / "massively-parallel-gpu-ode-solver_gb300")]
    import torch.distributed as dist
    from mpgos_gb300 import sharding as S, workloads as W
    from oracle import oracle as O
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        case = W.lorenz_case(nt=203)
        part = S.shard_case(case, rank, world)
        res = O.run_oracle(part, threads=1)
        full = S.gather(res)
        mx = bench.dist_max(world, float(rank + 1))
        sm = bench.dist_sum(world, float(rank + 1))
        if rank == 0:
            ref = O.run_oracle(case, threads=1)
            for k in ("x", "t", "nacc", "nrej", "status", "acci"):
                np.testing.assert_array_equal(full[k], ref[k], err_msg=k)
            assert mx == float(world) and sm == float(world * (world + 1) // 2)
            Path(out_dir, "ok").write_text("ok")
        else:
            assert full is None
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_gloo_sharded_ensemble_matches_single_process(oracle_libs, tmp_path):
    import torch.multiprocessing as mp
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    mp.spawn(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    assert (tmp_path / "ok").read_text() == "ok"
