"""Benchmark of the per-thread ensemble solver (the hot path) on GB300.

Workload (headline): Lorenz ensemble, 2^20 instances, rho = linspace(0, 21),
initial state (10, 10, 10), adaptive Cash-Karp 4(5) at rtol = atol = 1e-10
over t in [0, 10], FP64. One step = one integration of the whole ensemble
from the initial state (one Solve() launch, after a device-side restore of
the initial state). Metric: accepted instance-steps per second.

Arms:
  default           the GB300 kernels through the C-ABI, chosen form:
                    DF_STAGE (double-float stage arithmetic on the FP32 pipe,
                    log-domain step control) on the persistent work queue,
                    launch shape autotuned. Measured in the same run and
                    reported beside it: the FP64 FAST_CONTROL form ("fast_fp64"),
                    the PLAIN form (reference arithmetic, static mapping,
                    "plain") and the reference's own kernel built for sm_103a
                    ("reference_gpu"); and the coupled configuration (rings of
                    64 Duffing units) in DF_STAGE and FP64 beside the
                    reference's coupled kernel ("coupled"), and the
                    adjoint configuration's adjoint/forward time ratio
                    ("adjoint").
  --impl reference  the reference's CPU implementation of the path: the
                    reference solver compiled for this host where its build
                    exists (oracle/_ref), else the oracle port
                    (oracle/oracle_perthread.cpp), OpenMP on all host cores,
                    each step a bounded sample of the workload.

Timing: W untimed warm-up steps, then exactly K steps, each timed with CUDA
events on the solver's stream; L2 (129 MB) is flushed before every step by
writing a 512 MB buffer, outside the timed event pair. Under torchrun every
rank integrates its own full ensemble (weak scaling, no data-path
collective); the time is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
PKG = REPO / "massively-parallel-gpu-ode-solver_gb300"
for p in (str(REPO), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)

WORKLOAD = "lorenz_rkck45_tol1e-10_t0-10_2^20"
CHOSEN_MODE = 16 | 2   # MPGOS_MODE_DF_STAGE | MPGOS_MODE_PERSISTENT (the autotuner may drop persistence)
METRIC = "accepted instance-steps/s (Lorenz RKCK45, rtol=atol=1e-10, 2^20 instances)"
UNIT = "instance-steps/s"
NT = 1 << 20

# Algorithmic FP64 FLOP per RKCK45 step attempt of the Lorenz system
# (1 add/sub/mul/div = 1 FLOP, an FMA = 2): six right-hand sides of 9 FLOP,
# stage sums, solution and embedded error 55 FLOP per component
# (3+5+7+9+11 stage sums, 9 solution, 11 error), and 2 FLOP per component in
# the controller (tolerance scale and ratio). pow / exp2 are counted as one
# special-function evaluation, not as FLOP.
FLOP_PER_ATTEMPT = 6 * 9 + 3 * 55 + 3 * 2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nt", type=int, default=NT, help="instances per GPU (default 2^20)")
    ap.add_argument("--no-plain", action="store_true", help="skip the PLAIN-form measurement")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--no-coupled", action="store_true", help="skip the coupled-configuration leg")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint-configuration leg")
    ap.add_argument("--no-uneven", action="store_true", help="skip the uneven (Keller-Miksis) leg")
    ap.add_argument("--no-rk4", action="store_true", help="skip the fixed-step (Duffing RK4) leg")
    return ap.parse_args()


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        import tempfile
        self.path = Path(tempfile.gettempdir()) / f"mpgos_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self) -> dict:
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return world, rank, local


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _reduce(world, value: float, op: str) -> float:
    """All-reduce of one scalar over the ranks (timing and step counts only;
    no data-path collective). The tensor lives where the backend wants it:
    the GPU for nccl, the host for gloo."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def dist_max(world, value: float) -> float:
    return _reduce(world, value, "max")


def dist_sum(world, value: float) -> float:
    return _reduce(world, value, "sum")


def load_peaks() -> dict:
    p = REPO / "MEASURED_PEAKS.json"
    return json.loads(p.read_text()) if p.exists() else {}


def load_traffic() -> dict:
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu summary."""
    p = REPO / "profiles" / "roofline_traffic.json"
    return json.loads(p.read_text()) if p.exists() else {}


def cpu_sample_case(nt: int, stride: int):
    from mpgos_gb300 import workloads as W
    full = W.lorenz_case(nt=nt)
    return full.subset(np.arange(0, nt, stride))


def cpu_baseline(nt: int, stride: int = 8):
    """Oracle port (OpenMP, all host cores) on every stride-th instance; the
    baseline line, the oracle's results and the sampled case."""
    from oracle import oracle as O
    case = cpu_sample_case(nt, stride)
    threads = O.max_threads("lorenz")
    O.run_oracle(cpu_sample_case(nt, nt // 64))  # load + warm
    t0 = time.perf_counter()
    res = O.run_oracle(case, threads=threads)
    dt = time.perf_counter() - t0
    steps = float(res["nacc"].sum())
    return {"value": steps / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{case.nt} of {nt} instances (every {stride}th, same rho distribution), "
                      f"{int(steps)} accepted steps in {dt:.2f} s"}, res, case


def end_state_errors(results: dict, oracle_res: dict, sample: "W.Case", stride: int) -> dict:
    """End-state error of each GPU mode against the FP64 oracle (the CPU
    restatement of the reference solver) on the oracle's sample instances:
    per instance the largest component error scaled by |oracle| + 1e-3 x the
    component's ensemble scale; quantiles over all sampled instances and over
    the non-chaotic ones (rho < 13.9: the Lorenz system from (10, 10, 10) shows
    transient chaos above, where rounding differences are amplified)."""
    ref = oracle_res["x"]
    scale = np.max(np.abs(ref), axis=1, keepdims=True)
    calm = sample.arrays["cp"][0] < 13.9
    out = {"sample": f"every {stride}th instance ({ref.shape[1]}), oracle rtol = atol = 1e-10",
           "non_chaotic_instances": int(calm.sum())}
    for name, res in results.items():
        if res is None:
            continue
        x = res["x"][:, ::stride]
        per = np.max(np.abs(x - ref) / (np.abs(ref) + 1e-3 * scale), axis=0)
        out[name] = {"median": float(np.median(per)), "q99_non_chaotic": float(np.quantile(per[calm], 0.99)),
                     "max_non_chaotic": float(per[calm].max()), "max_all": float(per.max()),
                     "within_1e-9_non_chaotic": float(np.mean(per[calm] <= 1e-9)),
                     "accepted_steps_vs_oracle": float(res["nacc"][::stride].sum() / oracle_res["nacc"].sum())}
    return out


def run_reference(args):
    """--impl reference: the reference's CPU implementation on the host cores."""
    world, rank, local = dist_setup()
    if rank != 0:
        return
    from oracle import oracle as O
    stride = 16
    case = cpu_sample_case(args.nt, stride)
    # The oracle port (OpenMP over instances): the CPU restatement of the
    # reference's per-thread solver, pinned bit for bit to the reference's own
    # kernel compiled for the CPU (tests/test_oracle.py). That reference build
    # runs one instance at a time through static thread indices, so it cannot
    # use more than one core, and it only exists where the reference checkout
    # was present at build time; the port is what runs here.
    kind = "port"
    runner = lambda c: O.run_oracle(c, threads=0)
    threads = O.max_threads("lorenz")
    for _ in range(args.warmup):
        runner(cpu_sample_case(args.nt, args.nt // 256))
    times, steps = [], 0.0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        res = runner(case)
        times.append(time.perf_counter() - t0)
        steps += float(res["nacc"].sum())
    total = sum(times)
    value = steps / total
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": WORKLOAD, "instances": args.nt, "sample_stride": stride},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                             "sample": f"{case.nt} of {args.nt} instances (every {stride}th) per step"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def flush_l2(buf):
    buf.fill_(1)


def adjoint_leg(local: int, flush) -> dict:
    """Adjoint configuration: forced Duffing ensemble of 2^18 instances with
    per-instance (k, B), RKCK45 1e-9 over 64 forcing periods, loss = squared
    distance of the terminal state to per-instance targets; gradients with
    respect to (x0, v0, k, B) by the discrete adjoint with a checkpoint every
    32 accepted steps. On the same inputs, persistent mapping, three forms:
      fp64                 FP64 (FAST_CONTROL) forward, recording and reverse;
      fp64_fwd_df_reverse  the same FP64 forward and recording, reverse pass
                           in double-float (KERNEL_MODE switched to DF_STAGE
                           between SolveRecord and Adjoint);
      df_stage             double-float forward, recording and reverse.
    Each times the forward pass alone, the recording forward pass and the
    reverse pass; adjoint/forward = (recording + reverse) / forward of the
    same forward arithmetic. The headline is the FP64-forward form with the
    double-float reverse pass (the configuration integrates in FP64)."""
    import torch
    from mpgos_gb300 import capi, workloads as W
    from mpgos_gb300.solver import Variable
    nt, seg = 1 << 18, 32
    case = W.duffing_param_case(nt=nt, periods=64, tol=1e-9)
    target = torch.tensor(W.duffing_param_targets(nt), device=f"cuda:{local}")
    out = {"workload": "duffing_param_2^18_rkck45_tol1e-9_64periods_seg32", "unit": "ms",
           "gradients_per_instance": 4}
    FP64 = capi.MODE_FAST_CONTROL | capi.MODE_PERSISTENT
    DF = capi.MODE_DF_STAGE | capi.MODE_PERSISTENT

    def run(mode, reverse_modes):
        """Forward and recording in `mode`; one reverse pass per entry of
        `reverse_modes` on the same tape."""
        with W.load_solver(case, mode=mode, block=128, device=local) as s:
            s.checkpoint_save()
            # tape capacity: the largest accepted-step count of a plain forward pass
            s.Solve()
            s.SynchroniseFromDeviceToHost(Variable.AcceptedSteps)
            s.SynchroniseDevice()
            max_steps = int(s.host(Variable.AcceptedSteps).max()) + 64
            g = torch.empty((2, nt), dtype=torch.float64, device=f"cuda:{local}")
            gx0, gcp = torch.empty_like(g), torch.empty_like(g)
            x_dev = torch.empty_like(g)
            fwd, rec, rev = [], [], {m: [] for m in reverse_modes}
            grads = {}
            for i in range(3):
                s.set_mode(mode)
                flush_l2(flush)
                torch.cuda.synchronize()
                s.checkpoint_restore()
                s.timer_start()
                s.Solve()
                t_f = s.timer_stop()
                flush_l2(flush)
                torch.cuda.synchronize()
                s.checkpoint_restore()
                s.timer_start()
                s.SolveRecord(max_steps, seg)
                t_r = s.timer_stop()
                s.SynchroniseFromDeviceToHost(Variable.ActualState)
                s.SynchroniseDevice()
                x_dev.copy_(torch.from_numpy(s.host(Variable.ActualState)))
                g.copy_(2.0 * (x_dev - target))
                for m in reverse_modes:
                    s.set_mode(m)
                    torch.cuda.synchronize()
                    s.timer_start()
                    s.Adjoint(g.data_ptr(), gx0.data_ptr(), gcp.data_ptr())
                    t_b = s.timer_stop()
                    grads[m] = torch.cat([gx0, gcp]).cpu().numpy()
                    if i:
                        rev[m].append(t_b)
                if i:
                    fwd.append(t_f)
                    rec.append(t_r)
            s.SynchroniseFromDeviceToHost(Variable.Status)
            s.SynchroniseDevice()
            overflow = int(np.count_nonzero(s.host(Variable.Status) & capi.INSTANCE_TAPE_OVERFLOW))
        f, r = statistics.median(fwd), statistics.median(rec)
        res = {}
        for m in reverse_modes:
            b = statistics.median(rev[m])
            res[m] = {"forward_ms": f, "recording_forward_ms": r, "reverse_ms": b,
                      "adjoint_over_forward": (r + b) / f, "tape_overflow_instances": overflow,
                      "tape_steps": max_steps}
        return res, grads

    def rel(a, b):
        return float(np.max(np.abs(a - b) / np.maximum(np.max(np.abs(b), axis=1, keepdims=True), 1e-300)))

    r64, g64 = run(FP64, (FP64, DF))
    rdf, gdf = run(DF, (DF,))
    head = r64[DF]
    out.update({"fp64": r64[FP64], "fp64_fwd_df_reverse": head, "df_stage": rdf[DF],
                "adjoint_over_forward": head["adjoint_over_forward"],
                "headline_form": "FP64 forward + recording, double-float reverse",
                # one FP64 tape reversed in FP64 and in double-float: the reverse arithmetic's own error
                "gradient_max_rel_diff_df_vs_fp64_reverse_same_tape": rel(g64[DF], g64[FP64]),
                # different (both 1e-9-controlled) step sequences
                "gradient_max_rel_diff_df_stage_vs_fp64": rel(gdf[DF], g64[FP64])})
    return out


def rk4_leg(local: int, flush) -> dict:
    """Fixed-step configuration: forced Duffing oscillator, 8192 instances,
    RK4 with dt = 2 pi / 400 over 1024 forcing periods (1024 phases replayed
    from one CUDA graph), running maximum of x as an accessory. Times PLAIN
    (bit-identical to the reference kernel, checked), the double-float form
    (same step counts on the same FP64 time grid) and the reference's kernel
    launched once per period; one warm-up and two timed runs each."""
    import torch
    from mpgos_gb300 import capi, workloads as W
    from oracle import ref_gpu as R
    case = W.duffing_rk4_case(nt=8192, periods=1024)
    out = {"workload": "duffing_rk4_8192_dt2pi/400_1024periods", "unit": "accepted instance-steps/s"}

    def run(mode, reference=False, tune=False):
        with W.load_solver(case, mode=mode, block=64, device=local) as s:
            s.checkpoint_save()
            kern = None
            if reference:
                kern = R.ReferenceKernel("duffing", 0, case.nt, 0)
                kern.bind(s, case, block=32)
            if tune:
                s.autotune(arithmetic=mode & capi.MODE_DF_STAGE)
            cfg = {}
            if not reference:
                grid, blk, m = s.launch_config()
                cfg = {"grid": grid, "block": blk, "mode": m,
                       "outline_rhs": int(s.GetOption(capi.Option.OutlineRhs))}
            times = []
            for i in range(3):
                flush_l2(flush)
                torch.cuda.synchronize()
                s.checkpoint_restore()
                s.timer_start()
                if reference:
                    for _ in range(case.phases):
                        kern.launch()
                else:
                    s.SolvePhases(case.phases)
                ms = s.timer_stop()
                if i:
                    times.append(ms)
            res = W.read_results(s)
            if kern is not None:
                kern.close()
        steps = float(res["acci"][0].sum())
        return {"ms": statistics.median(times), "value": steps / (statistics.median(times) / 1e3), **cfg}, res

    out["plain"], rp = run(capi.MODE_PLAIN)
    out["df_stage_autotuned"], rd = run(capi.MODE_DF_STAGE, tune=True)
    out["df_steps_equal_plain"] = bool(np.array_equal(rd["acci"], rp["acci"]))
    out["df_max_abs_diff_vs_plain"] = float(np.max(np.abs(rd["x"] - rp["x"])))
    if R.available("duffing", 0, case.nt, 0):
        ref, rr = run(capi.MODE_PLAIN, reference=True)
        out["reference_gpu"] = ref
        out["speedup_df_vs_reference_gpu"] = out["df_stage_autotuned"]["value"] / ref["value"]
        out["plain_bitwise_equal_to_reference_kernel"] = bool(all(
            np.array_equal(np.asarray(rp[k]).view(np.uint8), np.asarray(rr[k]).view(np.uint8))
            for k in ("x", "t", "acc", "acci")))
    return out


def uneven_leg(local: int, flush) -> dict:
    """Uneven configuration at reduced size: Keller-Miksis bubbles on a
    256 x 256 grid of driving amplitude x frequency (2^16 instances; the
    configuration's 512 x 512 grid and 1024 periods scaled down to keep the
    bench short), RKCK45 1e-10, 4 acoustic periods as 4 phases captured in
    one CUDA graph, the per-period maximum radius streamed out after every
    phase. Step counts per instance differ by two orders of magnitude. Times
    the static and persistent mappings of the FP64 (FAST_CONTROL) and
    double-float forms and the reference's kernel (sm_103a cubin, event
    options fixed, one launch per period) on the same inputs; checks PLAIN
    against the reference kernel bit for bit."""
    import torch
    from mpgos_gb300 import capi, workloads as W
    from mpgos_gb300.solver import Variable
    from oracle import ref_gpu as R
    case = W.keller_miksis_case(n_amp=256, n_freq=256, periods=4)
    nt, phases = case.nt, case.phases
    out = {"workload": "keller_miksis_256x256_rkck45_tol1e-10_4periods", "unit": "accepted instance-steps/s",
           "phases": phases}
    per_phase = torch.empty((phases, nt), dtype=torch.float64, device=f"cuda:{local}")

    def run(mode, block=128, reference=False, tune=False):
        with W.load_solver(case, mode=mode, block=block, device=local) as s:
            s.checkpoint_save()
            kern = None
            if reference:
                kern = R.ReferenceKernel("keller_miksis", 1, nt, 0)
                kern.bind(s, case, block=32)
            if tune:
                s.autotune(arithmetic=mode & (capi.MODE_FAST_CONTROL | capi.MODE_DF_STAGE))
            grid, blk, m = s.launch_config() if not reference else (kern.grid, kern.block, -1)
            outline = int(s.GetOption(capi.Option.OutlineRhs)) if not reference else 0
            times = []
            for i in range(3):
                flush_l2(flush)
                torch.cuda.synchronize()
                s.checkpoint_restore()
                s.timer_start()
                if reference:
                    for _ in range(phases):
                        kern.launch()
                else:
                    s.SolvePhases(phases, 0, per_phase.data_ptr())
                ms = s.timer_stop()
                if i:
                    times.append(ms)
            res = W.read_results(s)
            if kern is not None:
                kern.close()
        # accepted steps of all phases, counted by the system's own hook (integer accessory 1)
        steps = float(res["acci"][1].sum())
        return {"ms": statistics.median(times), "value": steps / (statistics.median(times) / 1e3),
                "grid": grid, "block": blk, "mode": m, "outline_rhs": outline}, res

    FAST, DF, P = capi.MODE_FAST_CONTROL, capi.MODE_DF_STAGE, capi.MODE_PERSISTENT
    # static mappings with the reference's one-warp blocks (the best static shape for uneven
    # work: a finished warp frees its block), persistent with 128-thread blocks, and the
    # autotuned double-float choice
    forms = {"fp64_static_b32": (FAST, 32), "fp64_persistent": (FAST | P, 128), "df_static_b32": (DF, 32),
             "df_persistent": (DF | P, 128)}
    results = {}
    for name, (mode, block) in forms.items():
        out[name], results[name] = run(mode, block)
    out["df_autotuned"], _ = run(DF, tune=True)
    plain, rplain = run(capi.MODE_PLAIN, 32)
    out["plain_static_b32"] = plain
    n = results["fp64_static_b32"]["acci"][1]
    out["steps_per_instance_min_max"] = [int(n.min()), int(n.max())]
    out["persistent_over_static_fp64"] = out["fp64_static_b32"]["ms"] / out["fp64_persistent"]["ms"]
    out["persistent_over_static_df"] = out["df_static_b32"]["ms"] / out["df_persistent"]["ms"]
    if R.available("keller_miksis", 1, nt, 0):
        ref, rref = run(capi.MODE_PLAIN, reference=True)
        out["reference_gpu"] = ref
        best = max(out[k]["value"] for k in ("df_persistent", "df_autotuned", "df_static_b32"))
        out["speedup_best_df_vs_reference_gpu"] = best / ref["value"]
        out["speedup_fp64_persistent_vs_reference_gpu"] = out["fp64_persistent"]["value"] / ref["value"]
        out["plain_bitwise_equal_to_reference_kernel"] = bool(all(
            np.array_equal(np.asarray(rplain[k]).view(np.uint8), np.asarray(rref[k]).view(np.uint8))
            for k in ("x", "t", "acc", "acci")))
        # double-float form against the reference kernel over the whole ensemble: end states
        # and per-period maximum radii relative to each component's scale, integer outputs
        # (event count, accepted steps) per instance
        # (the FP64 FAST_CONTROL form beside it: what a different rounding of the step-size
        # factor alone does on this ensemble)
        def versus_reference(r):
            rel = {}
            for k in ("x", "acc"):
                a, b = np.asarray(r[k], np.float64), np.asarray(rref[k], np.float64)
                scale = np.max(np.abs(b), axis=1, keepdims=True)
                rel[k] = (np.abs(a - b) / (np.abs(b) + 1e-3 * scale)).max(axis=0)
            steps, ref_steps = float(r["acci"][1].sum()), float(rref["acci"][1].sum())
            return {"instances_within_1e-9_end_state": float(np.mean(rel["x"] <= 1e-9)),
                    "instances_within_1e-9_max_radius": float(np.mean(rel["acc"] <= 1e-9)),
                    "event_count_equal_fraction": float(np.mean(r["acci"][0] == rref["acci"][0])),
                    "accepted_steps_equal_fraction": float(np.mean(r["acci"][1] == rref["acci"][1])),
                    "accepted_steps_total_rel_diff": abs(steps - ref_steps) / ref_steps}
        out["df_vs_reference_gpu"] = versus_reference(results["df_static_b32"])
        out["fp64_fast_vs_reference_gpu"] = versus_reference(results["fp64_static_b32"])
    return out


def coupled_leg(local: int, flush) -> dict:
    """Coupled configuration beside the headline: 16384 rings of 64 Duffing
    units (dense coupling, RKCK45 1e-9, crossing events), two forcing periods
    per launch. Times the DF_STAGE and FP64 warp-per-system kernels and the
    reference's own coupled kernel (sm_103a cubin, TPB 256 / SPB 4) on the same
    inputs; one warm-up and two timed launches each, L2 flushed before each."""
    import torch
    from mpgos_gb300 import capi, coupled_workloads as CW
    from mpgos_gb300.capi import CbVariable as V
    case = CW.ring_case("ring64", ns=16384, periods=2, seed=5)

    def run(mode=None, warps=4, ref=None):
        with CW.load_coupled_solver(case, mode=mode or 0, warps=warps, device=local) as s:
            s.checkpoint_save()
            kern = None
            if ref is not None:
                from oracle import ref_gpu
                kern = ref_gpu.CoupledReferenceKernel("ring64", 1, case.ns, ref[0], ref[1], 0)
                kern.bind(s, case, shared_global=1, shared_coupling=0)
            launch = kern.launch if kern is not None else s.Solve
            times = []
            for i in range(3):
                flush_l2(flush)
                torch.cuda.synchronize()
                s.checkpoint_restore()
                s.timer_start()
                launch()
                ms = s.timer_stop()
                if i:
                    times.append(ms)
            res = CW.read_coupled_results(s)
            if kern is not None:
                kern.close()
        steps = float(res["isacc"][0].sum())  # accepted steps, counted by the systems' own hook
        return {"ms": statistics.median(times), "value": steps / (statistics.median(times) / 1e3)}, res

    def adjoint(mode, reverse_modes, warps, seg=32):
        """Recording forward pass in `mode` and one reverse pass per entry of
        `reverse_modes` on that tape, for the gradient of the summed terminal
        energy E = sum_i (v_i^2/2 + x_i^2/2 + x_i^4/4) with respect to B (and
        the initial states); median of two timed rounds after one warm-up,
        L2 flushed before each pass."""
        with CW.load_coupled_solver(case, mode=mode, warps=warps, device=local) as s:
            s.checkpoint_save()
            s.Solve()
            res = CW.read_coupled_results(s)
            max_steps = int(max(res["nacc"].max(), res["isacc"][0].max() if len(res["isacc"]) else 0)) + 64
            nu = case.ns * case.ups
            dev = f"cuda:{local}"
            gx0 = torch.empty((2, nu), dtype=torch.float64, device=dev)
            gsp = torch.empty((max(s.NSP, 1), case.ns), dtype=torch.float64, device=dev)
            rec, rev = [], {m: [] for m in reverse_modes}
            for i in range(3):
                s.set_mode(mode)
                flush_l2(flush)
                torch.cuda.synchronize()
                s.checkpoint_restore()
                s.timer_start()
                s.SolveRecord(max_steps, seg)
                t_r = s.timer_stop()
                s.SynchroniseFromDeviceToHost(V.ActualState)
                s.SynchroniseDevice()
                xT = s.host(V.ActualState)
                gT = torch.tensor(np.stack([xT[0] + xT[0] ** 3, xT[1]]), device=dev)
                for m in reverse_modes:
                    s.set_mode(m)
                    flush_l2(flush)
                    torch.cuda.synchronize()
                    s.timer_start()
                    s.Adjoint(gT.data_ptr(), gx0.data_ptr(), gsp.data_ptr())
                    t_b = s.timer_stop()
                    if i:
                        rev[m].append(t_b)
                if i:
                    rec.append(t_r)
            s.SynchroniseFromDeviceToHost(V.Status)
            s.SynchroniseDevice()
            overflow = int(np.count_nonzero(s.host(V.Status) & capi.INSTANCE_TAPE_OVERFLOW))
        return {m: {"recording_forward_ms": statistics.median(rec), "reverse_ms": statistics.median(rev[m]),
                    "tape_steps": max_steps, "segment": seg, "tape_overflow_systems": overflow}
                for m in reverse_modes}

    out = {"workload": "ring64_16384x64_dense_rkck45_tol1e-9_2periods", "unit": "accepted system-steps/s"}
    df, rdf = run(capi.MODE_DF_STAGE | capi.MODE_PERSISTENT, warps=2)
    fp, rfp = run(capi.MODE_PERSISTENT, warps=4)
    out["df_stage"], out["fp64"] = df, fp
    FP, DFM = capi.MODE_PERSISTENT, capi.MODE_DF_STAGE | capi.MODE_PERSISTENT
    a64 = adjoint(FP, (FP, DFM), warps=4)
    adf = adjoint(DFM, (DFM,), warps=2)
    forms = {"fp64": (a64[FP], fp), "fp64_fwd_df_reverse": (a64[DFM], fp), "df_stage": (adf[DFM], df)}
    adj = {}
    for name, (r, f) in forms.items():
        r["forward_ms"] = f["ms"]
        r["adjoint_over_forward"] = (r["recording_forward_ms"] + r["reverse_ms"]) / f["ms"]
        adj[name] = r
    adj["adjoint_over_forward"] = adj["fp64_fwd_df_reverse"]["adjoint_over_forward"]
    adj["headline_form"] = "FP64 forward + recording, double-float reverse"
    out["adjoint_wrt_B"] = adj
    from oracle import ref_gpu as R
    if R.coupled_available("ring64", 1, case.ns, 256, 4, 0):
        ref, rref = run(ref=(256, 4))
        out["reference_gpu"] = ref
        out["speedup_df_vs_reference_gpu"] = df["value"] / ref["value"]
        out["fp64_bitwise_equal_to_reference_kernel"] = bool(
            all(np.array_equal(rfp[k], rref[k]) for k in ("x", "iuacc", "isacc")))
        mag = np.max(np.abs(rref["x"]), axis=1, keepdims=True)
        err = (np.abs(rdf["x"] - rref["x"]) / mag).max(axis=0).reshape(case.ns, -1).max(axis=1)
        out["df_systems_within_1e-9_of_reference"] = float(np.mean(err <= 1e-9))
        out["df_crossing_counts_equal_fraction"] = float(np.mean(np.all(
            rdf["iuacc"].reshape(case.ns, -1) == rref["iuacc"].reshape(case.ns, -1), axis=1)))
    return out


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)

    world, rank, local = dist_setup()
    import torch
    torch.cuda.set_device(local)
    from mpgos_gb300 import build, capi, workloads as W
    from mpgos_gb300.solver import Variable

    build.build_all()
    case = W.lorenz_case(nt=args.nt)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    def measure(mode, steps, warmup, clocks=None, tune=False, reference=False):
        """Time ``steps`` integrations of the whole ensemble: our kernels in
        ``mode`` (autotuned launch shape if ``tune``) or, with ``reference``,
        the reference's own kernel (sm_103a cubin) on the same buffers."""
        s = W.load_solver(case, mode=mode, block=128, device=local)
        s.checkpoint_save()
        kern = None
        if reference:
            from oracle import ref_gpu
            kern = ref_gpu.ReferenceKernel("lorenz", 1, args.nt, 0)
            kern.bind(s, case, block=32)   # reference default: one warp per block
            launch = kern.launch
        else:
            if tune:
                s.autotune(arithmetic=mode & (capi.MODE_FAST_CONTROL | capi.MODE_DF_STAGE))
            launch = s.Solve
        for _ in range(warmup):
            s.checkpoint_restore()
            launch()
        s.SynchroniseDevice()
        grid, block, m = s.launch_config() if not reference else (kern.grid, kern.block, -1)
        kernel_ms, step_ms = [], []
        dist_barrier(world)
        torch.cuda.synchronize()
        ctx = clocks if clocks is not None else _Null()
        accepted = attempts = 0.0
        with ctx:
            for _ in range(steps):
                flush_l2(flush)
                torch.cuda.synchronize()
                s.timer_start()
                s.checkpoint_restore()
                launch()
                step_ms.append(s.timer_stop())
                if reference:
                    s.SynchroniseFromDeviceToHost(Variable.IntegerAccessories)
                    s.InsertSynchronisationPoint()
                    s.SynchroniseSolver()
                    accepted += float(s.host(Variable.IntegerAccessories)[0].sum())
                else:
                    for v in (Variable.AcceptedSteps, Variable.RejectedSteps):
                        s.SynchroniseFromDeviceToHost(v)
                    s.InsertSynchronisationPoint()
                    s.SynchroniseSolver()
                    na = float(s.host(Variable.AcceptedSteps).sum())
                    accepted += na
                    attempts += na + float(s.host(Variable.RejectedSteps).sum())
            torch.cuda.synchronize()
        # kernel-only time of the dominant kernel (events on its stream around the launch)
        for _ in range(min(steps, 3)):
            flush_l2(flush)
            torch.cuda.synchronize()
            s.checkpoint_restore()
            s.timer_start()
            launch()
            kernel_ms.append(s.timer_stop())
        dist_barrier(world)
        res = W.read_results(s)
        if kern is not None:
            kern.close()
        s.close()
        return dict(step_ms=step_ms, kernel_ms=kernel_ms, accepted=accepted, attempts=attempts, grid=grid,
                    block=block, mode=m, res=res)

    clocks = Clocks(local)
    chosen = measure(CHOSEN_MODE, args.steps, args.warmup, clocks, tune=True)
    t_step = dist_max(world, sum(chosen["step_ms"]) / 1e3)
    acc_all = dist_sum(world, chosen["accepted"])
    value = acc_all / t_step
    ms_per_step = 1e3 * t_step / args.steps

    # e2e through the public API with host buffers: H2D of the step's inputs,
    # Solve, D2H of the end states and step counters, every step.
    with W.load_solver(case, mode=chosen["mode"], block=chosen["block"], device=local) as s:
        host_x0 = s.host(Variable.ActualState).copy()
        host_t0 = s.host(Variable.ActualTime).copy()
        host_c0 = s.host(Variable.IntegerAccessories).copy()
        h2d = [Variable.ActualState, Variable.ActualTime, Variable.IntegerAccessories]
        d2h = [Variable.ActualState, Variable.IntegerAccessories]
        s.Solve()
        s.SynchroniseDevice()
        e2e_steps = max(1, min(args.steps, 3))
        dist_barrier(world)
        acc = 0.0
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            s.host(Variable.ActualState)[:] = host_x0
            s.host(Variable.ActualTime)[:] = host_t0
            s.host(Variable.IntegerAccessories)[:] = host_c0
            for v in h2d:
                s.SynchroniseFromHostToDevice(v)
            s.Solve()
            for v in d2h:
                s.SynchroniseFromDeviceToHost(v)
            s.InsertSynchronisationPoint()
            s.SynchroniseSolver()
            acc += float(s.host(Variable.IntegerAccessories)[0].sum())
        dt = dist_max(world, time.perf_counter() - t0)
        e2e = {"value": dist_sum(world, acc) / dt, "unit": UNIT,
               "h2d_bytes_per_step": int(sum(s.host(v).nbytes for v in h2d)),
               "d2h_bytes_per_step": int(sum(s.host(v).nbytes for v in d2h)), "steps": e2e_steps}

    def summarize(r):
        tp = dist_max(world, sum(r["step_ms"]) / 1e3)
        return {"value": dist_sum(world, r["accepted"]) / tp, "ms_per_step": 1e3 * tp / len(r["step_ms"]),
                "kernel_ms": statistics.median(r["kernel_ms"]), "grid": r["grid"], "block": r["block"],
                "mode": r["mode"]}

    fast_r = measure(capi.MODE_CHOSEN, max(1, min(args.steps, 3)), 1, tune=True)
    fast = summarize(fast_r)
    # the FP32-stage form on the same inputs (end-state error reported below)
    f32_r = measure(capi.MODE_FP32_STAGE | capi.MODE_CHOSEN, 1, 1)
    fp32_stage = summarize(f32_r)
    coupled = None if args.no_coupled else coupled_leg(local, flush)
    adjoint = None if args.no_adjoint else adjoint_leg(local, flush)
    uneven = None if args.no_uneven else uneven_leg(local, flush)
    rk4 = None if args.no_rk4 else rk4_leg(local, flush)
    plain = ref_gpu = p = None
    parity = {}
    if not args.no_plain:
        p = measure(capi.MODE_PLAIN, max(1, min(args.steps, 3)), 1)
        plain = summarize(p)
        from oracle import ref_gpu as R
        if R.available("lorenz", 1, args.nt, 0):
            r = measure(capi.MODE_PLAIN, max(1, min(args.steps, 3)), 1, reference=True)
            ref_gpu = summarize(r)
            ref_gpu["kernel"] = "reference SingleSystem_PerThread built for sm_103a (oracle/_ref cubin), block 32"
            same = all(np.array_equal(np.asarray(p["res"][k]).view(np.uint8), np.asarray(r["res"][k]).view(np.uint8))
                       for k in ("x", "t", "acci"))
            parity["plain_bitwise_equal_to_reference_kernel"] = bool(same)
            ref_res = r["res"]
        else:
            ref_res = p["res"]
        a, b = chosen["res"]["x"], ref_res["x"]
        scale = np.max(np.abs(b), axis=1, keepdims=True)
        rel = np.abs(a - b) / (np.abs(b) + 1e-3 * scale)
        per_inst = rel.max(axis=0)
        parity.update({"chosen_vs_reference_max_scaled_rel": float(per_inst.max()),
                       "chosen_instances_within_1e-9": float(np.mean(per_inst <= 1e-9)),
                       "chosen_step_count_equal_fraction": float(np.mean(chosen["res"]["acci"][0] == ref_res["acci"][0]))})

    if rank != 0:
        return

    peak_fp64 = capi.fma_peak(local, 8)
    peak_fp32_ops = capi.fma_peak(local, 4) / 2.0   # FP32 FMA instructions per second
    kernel_s = statistics.median(chosen["kernel_ms"]) / 1e3
    attempts_per_launch = chosen["attempts"] / args.steps
    prof = load_traffic()
    instr = prof.get("lorenz_df_thread_instr_per_attempt")
    traffic = prof.get("lorenz_df_dram_bytes_per_launch")
    achieved = (instr * attempts_per_launch / kernel_s) if instr else None
    peaks = load_peaks()
    # per instance: x (3), t, td (2), rho read and x, t written in FP64; the
    # step-counter accessory read and written, status and the two step
    # counters written, as int32
    hbm_bytes = args.nt * ((3 + 1 + 2 + 1) * 8 + (3 + 1) * 8 + 2 * 4 + 3 * 4)
    cpu = errors = None
    if not args.no_cpu:
        stride = 8
        cpu, oracle_res, sample = cpu_baseline(args.nt, stride)
        errors = end_state_errors({"plain": p["res"] if p else None, "fast_fp64": fast_r["res"],
                                   "df_stage": chosen["res"], "fp32_stage": f32_r["res"]}, oracle_res, sample, stride)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "df64 (float pairs, ~48-bit) stages; f64 state in HBM", "data": "synthetic",
        "config": {"workload": WORKLOAD, "instances": args.nt, "form": "chosen: DF_STAGE + persistent",
                   "mode": chosen["mode"], "grid": chosen["grid"], "block": chosen["block"],
                   "l2": "flushed before every step (512 MB write), outside the timed events",
                   "accepted_steps_per_launch": chosen["accepted"] / args.steps,
                   "attempts_per_launch": attempts_per_launch},
        "e2e": e2e,
        "fast_fp64": fast,
        "fp32_stage": fp32_stage,
        "end_state_error_vs_fp64_oracle": errors,
        "coupled": coupled,
        "adjoint": adjoint,
        "uneven": uneven,
        "rk4": rk4,
        "plain": plain,
        "reference_gpu": ref_gpu,
        "speedup_vs_reference_gpu": (value / ref_gpu["value"]) if ref_gpu else None,
        "parity": parity,
        "roofline": {"bound": "instruction issue (FP32 pipe)",
                     "achieved": achieved / 1e12 if achieved else None,
                     "peak": peak_fp32_ops / 1e12, "unit": "T thread-instructions/s",
                     "frac": achieved / peak_fp32_ops if achieved else None, "traffic": traffic,
                     "thread_instructions_per_attempt": instr,
                     "instructions_source": "smsp__inst_executed x thread/inst per step attempt, ncu capture "
                                            "of the same kernel on 2^18 instances (profiles/roofline_traffic.json)",
                     "kernel_ms": kernel_s * 1e3,
                     "peak_source": "measured FFMA instruction rate (mpgos_probe_fma_peak, precision 4), same GPU, "
                                    "same run: the issue ceiling every instruction shares",
                     "algorithmic_fp64_equivalent_tflops": FLOP_PER_ATTEMPT * attempts_per_launch / kernel_s / 1e12,
                     "fp64_fma_peak_tflops": peak_fp64 / 1e12,
                     "hbm_peak_gbs_measured": peaks.get("hbm_gbs"),
                     # the HBM side of the same launch: algorithmic bytes (state, time, time
                     # domain and rho read; state, time, step counter and status words written)
                     "hbm": {"algorithmic_bytes": hbm_bytes, "achieved_gbs": hbm_bytes / kernel_s / 1e9,
                             "frac_of_measured": (hbm_bytes / kernel_s / 1e9 / peaks["hbm_gbs"])
                             if peaks.get("hbm_gbs") else None}},
        "cpu_baseline": cpu,
        "clocks": clocks.summary(),
        "gpu_launches": args.steps,
    }
    print(json.dumps(line))


class _Null:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


if __name__ == "__main__":
    main()
