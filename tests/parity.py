"""Comparison helpers shared by the GPU parity tests.

Three kinds of comparison, each with the bar it can meet:

* GPU vs the reference's own kernel on the same GPU (``bitwise``): the PLAIN
  kernels keep the reference's operation order, so every output, including
  values sampled on the step grid (dense output, extrema over accepted
  steps), must agree bit for bit.
* GPU vs CPU (oracle or golden fixtures from the reference's CPU build)
  (``close``): fused multiply-adds and CUDA's math library round differently
  from the host, so FP64 end states agree to ~1e-13 relative. The bar of
  ``assert_cpu_parity`` is 1e-9 relative to the component's scale (the larger
  of the value and the largest initial or final magnitude of that component
  over the ensemble): a state that ends next to zero at an event carries the
  rounding of the whole trajectory, not of its own size. Elements may also
  differ by up to 1e3 times the CPU reference's own spread under tiny input
  perturbations (chaotic members). Integer outputs must be equal on every
  instance the perturbations leave unchanged.
* Values sampled on the step grid (accessories recording extrema over
  accepted steps, dense-output times and states) move with the grid, which
  moves when an event-refinement step lands a rounding error away from the
  tolerance band; these are compared at 1e-4 (``grid``).
"""
import numpy as np

END_STATE_KEYS = ("td", "x", "t", "cp")
GRID_KEYS = ("acc", "dtime", "dstate")
INT_KEYS = ("acci", "didx")


def scaled_close(a, b, rtol, magnitude=None, floor=1e-3):
    """|a - b| <= rtol * (|b| + floor * magnitude of the row), the magnitude
    being the largest |b| of the row or, where larger, ``magnitude`` (e.g.
    the largest initial value of the component: a state that ends next to
    zero at an event still moved on the scale of its trajectory)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if b.size == 0:
        return np.ones(b.shape, bool)
    if b.ndim == 1:
        scale = np.max(np.abs(b))
    else:
        scale = np.max(np.abs(b), axis=-1, keepdims=True)
    if magnitude is not None:
        scale = np.maximum(scale, np.asarray(magnitude, np.float64).reshape(np.shape(scale)))
    return np.abs(a - b) <= rtol * (np.abs(b) + floor * scale)


def assert_close(res, ref, rtol=1e-9, grid_rtol=1e-4, ints=True, mask=None, keys=None):
    """``mask``: instances to compare (default all)."""
    for k in keys or (END_STATE_KEYS + GRID_KEYS):
        if k not in ref or np.asarray(ref[k]).size == 0:
            continue
        a, b = np.asarray(res[k]), np.asarray(ref[k])
        if mask is not None:
            a, b = a[..., mask], b[..., mask]
        ok = scaled_close(a, b, grid_rtol if k in GRID_KEYS else rtol)
        if not ok.all():
            bad = np.argwhere(~ok)[:5]
            raise AssertionError(f"{k}: {int((~ok).sum())} elements differ, e.g. at {bad.tolist()}: "
                                 f"{a[tuple(bad[0])]!r} vs {b[tuple(bad[0])]!r}")
    if ints:
        for k in INT_KEYS:
            if k in ref:
                a, b = np.asarray(res[k]), np.asarray(ref[k])
                if mask is not None:
                    a, b = a[..., mask], b[..., mask]
                np.testing.assert_array_equal(a, b, err_msg=k)


def assert_bitwise(a, b, keys=None):
    for k in keys or sorted(set(a) & set(b)):
        x, y = np.asarray(a[k]), np.asarray(b[k])
        assert x.shape == y.shape, k
        assert np.array_equal(x.view(np.uint8), y.view(np.uint8)), f"{k} differs bitwise"


_SPREAD_CACHE = {}


def perturbation_spread(case, rel=0.0, key=None, tol_rel=0.0):
    """What tiny changes do to the CPU reference itself. The oracle is run on
    ``case`` and on three variants: every initial state moved by one unit in
    the last place (``rel`` = 0) or by ``rel`` relative; the same inputs with
    multiply-adds contracted into fused multiply-adds (the rounding change
    between host and GPU arithmetic, which event refinements and impacts can
    amplify far beyond one ulp); and, with ``tol_rel`` > 0, the tolerances
    moved up and down by ``tol_rel`` relative (which moves every step size by
    about tol_rel / 5, the step-grid shift of a step-size factor rounded
    differently, and flips every accept/reject decision within that margin). Returns (|difference| per float output, the largest over
    the variants; mask of instances whose integer outputs no variant changed).
    Cached under ``key``."""
    from oracle import oracle as O
    ck = (key, rel, tol_rel)
    if key is not None and ck in _SPREAD_CACHE:
        return _SPREAD_CACHE[ck]
    base = O.run_oracle(case)
    pert = case.copy()
    x = pert.arrays["x"]
    pert.arrays["x"] = np.nextafter(x, np.inf) if rel == 0.0 else x * (1.0 + rel) + (x == 0) * rel
    runs = [O.run_oracle(pert), O.run_oracle(case, fma=True)]
    if tol_rel > 0.0:
        for sign in (1.0, -1.0):
            pt = case.copy()
            pt.rtol = pt.rtol * (1.0 + sign * tol_rel)
            pt.atol = pt.atol * (1.0 + sign * tol_rel)
            runs.append(O.run_oracle(pt))
    spread = {k: np.max([np.abs(np.asarray(m[k], np.float64) - np.asarray(base[k], np.float64)) for m in runs], axis=0)
              for k in END_STATE_KEYS + GRID_KEYS if k in base}
    stable = np.ones(case.nt, bool)
    for moved in runs:
        for k in INT_KEYS:
            if k in base:
                diff = np.asarray(moved[k]) != np.asarray(base[k])
                stable &= ~(diff.any(axis=0) if diff.ndim > 1 else diff)
    out = (spread, stable)
    if key is not None:
        _SPREAD_CACHE[ck] = out
    return out


def assert_ints_equal(res, ref, keys, mask, slack=0.0, fraction=None):
    """Integer outputs equal on the instances of ``mask``. With ``slack`` > 0
    (a fraction), up to max(1, slack x #mask) instances may differ, each by
    at most max(2, 1 % of the count): a mode whose step-size factor is
    rounded differently from the reference's (FAST_CONTROL, DF_STAGE) takes
    one step more or fewer where an error estimate lands within that
    rounding of the tolerance (and the steps after it shift, so a rejection
    count can move by two), which no finite set of perturbations of the CPU
    reference catches every time. ``fraction`` overrides the 1 % per key."""
    bad = np.zeros(np.shape(mask), bool)
    for k in keys:
        if k not in ref:
            continue
        a, b = np.asarray(res[k]), np.asarray(ref[k])
        d = np.abs(a.astype(np.int64) - b.astype(np.int64))
        d = d.reshape(-1, d.shape[-1]).max(axis=0) if d.ndim > 1 else d
        if slack <= 0.0:
            np.testing.assert_array_equal(a[..., mask], b[..., mask], err_msg=k)
            continue
        ref_abs = np.abs(b.astype(np.int64))
        ref_abs = ref_abs.reshape(-1, ref_abs.shape[-1]).max(axis=0) if ref_abs.ndim > 1 else ref_abs
        frac = (fraction or {}).get(k, 0.01)
        allowed = np.maximum(2, (ref_abs * frac).astype(np.int64))
        assert np.all(d[mask] <= allowed[mask]), f"{k}: integer outputs differ by more than the step-flip allowance"
        bad |= (d > 0) & mask
    if slack > 0.0:
        limit = max(1, int(slack * int(np.sum(mask))))
        assert int(bad.sum()) <= limit, f"{int(bad.sum())} stable instances differ in integer outputs (limit {limit})"


def assert_cpu_parity(res, ref, case, key, rel=0.0, rtol=1e-9, grid_rtol=1e-4, factor=1e3, min_stable=0.5,
                      tol_rel=0.0, int_slack=0.0):
    """GPU result vs a CPU reference result of the same inputs.

    Every float element must agree within the bar of ``scaled_close`` or
    within ``factor`` times the CPU reference's own spread under the input
    perturbation of ``perturbation_spread`` (chaotic members and states that
    end inside an event band); integer outputs must be equal on every instance
    whose integers the perturbation leaves unchanged."""
    spread, stable = perturbation_spread(case, rel, key, tol_rel)
    assert stable.mean() >= min_stable, f"only {stable.mean():.2f} of the instances are stable"
    for k in END_STATE_KEYS + GRID_KEYS:
        if k not in ref or np.asarray(ref[k]).size == 0:
            continue
        a, b = np.asarray(res[k], np.float64), np.asarray(ref[k], np.float64)
        mag = np.max(np.abs(case.arrays["x"]), axis=-1) if k == "x" and a.ndim == 2 else None
        ok = (scaled_close(a, b, grid_rtol if k in GRID_KEYS else rtol, mag, floor=1.0) |
              (np.abs(a - b) <= factor * spread[k]))
        if not ok.all():
            bad = np.argwhere(~ok)[:3]
            raise AssertionError(f"{k}: {int((~ok).sum())} elements outside the bar, e.g. at {bad.tolist()}: "
                                 f"{a[tuple(bad[0])]!r} vs {b[tuple(bad[0])]!r} (spread {spread[k][tuple(bad[0])]!r})")
    assert_ints_equal(res, ref, INT_KEYS, stable, int_slack)


def sensitive_instances(case, rtol=1e-10):
    """Instances whose end state moves by more than ``rtol`` (scaled) when the
    initial state is perturbed by one unit in the last place: the chaotic or
    near-bifurcation members of the ensemble, where rounding differences
    between two correct implementations are amplified beyond any fixed
    tolerance. Computed with the oracle."""
    from oracle import oracle as O
    base = O.run_oracle(case)
    pert = case.copy()
    pert.arrays["x"] = np.nextafter(pert.arrays["x"], np.inf)
    moved = O.run_oracle(pert)
    ok = scaled_close(moved["x"], base["x"], rtol).all(axis=0)
    return ~ok
