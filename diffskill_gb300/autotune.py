"""Start-up autotuner of the substep's launch shapes and particle re-sort cadence.

The reference leaves launch shapes to Taichi.  Here two families of choices
depend on the workload and are picked by measurement on the batch itself:

* launch shapes (``MpmTuning`` of the C ABI): the CTAs-per-SM targets (register
  budgets) the FP32 p2g, g2p.grad and p2g.grad kernels are compiled for, and
  the stride width of the grid kernels.  The best occupancy trades latency
  hiding against register spills and depends on particles per cell, active
  grid blocks and scene count;
* the re-sort cadence (``Horizon.resort_every``): re-sorting particles by cell
  costs a radix sort and a gather of the state, and restores the locality that
  the scatter and gather kernels lose as the dough deforms.

``tune`` times every candidate with CUDA events (kernel launch shapes by the
library's per-kernel profiler on a one-action horizon, coordinate descent
from the defaults; the re-sort cadence by whole forward+backward iterations)
and keeps the fastest.  A candidate replaces the current choice only when it
is faster by more than ``margin`` (timing noise does not move the defaults).
Results are cached per device and workload shape in a JSON file
(``DIFFSKILL_GB300_TUNE_CACHE``, default ``~/.cache/diffskill_gb300/tuning.json``).
"""
from __future__ import annotations

import ctypes
import json
import os
from dataclasses import asdict, dataclass, field
from typing import Callable, Dict, List, Optional, Sequence

import numpy as np

# candidates per launch-shape field, the default first
CANDIDATES: Dict[str, Sequence[int]] = {
    "p2g_ctas": (7, 6, 8),
    "g2p_adj_ctas": (6, 5, 7, 8),
    "p2g_adj_ctas": (5, 4, 6),
    "grid_ctas_per_sm": (16, 8, 32),
    "g2p_ctas": (8, 10, 12),
    "grid_op_adj_ctas": (6, 12, 16),
}
# the profiler kinds (diffskill_gb300._lib.KERNEL_KINDS) whose times decide each field
KINDS: Dict[str, Sequence[str]] = {
    "p2g_ctas": ("p2g",),
    "g2p_adj_ctas": ("g2p_adj",),
    "p2g_adj_ctas": ("p2g_adj",),
    "grid_ctas_per_sm": ("grid_op", "grid_op_adj"),
    "g2p_ctas": ("g2p",),
    "grid_op_adj_ctas": ("grid_op_adj",),
}
FP32_ONLY = ("p2g_ctas", "g2p_adj_ctas", "p2g_adj_ctas", "g2p_ctas", "grid_op_adj_ctas")


@dataclass
class Tuning:
    p2g_ctas: int = 7
    g2p_adj_ctas: int = 6
    p2g_adj_ctas: int = 5
    grid_ctas_per_sm: int = 16
    g2p_ctas: int = 8
    grid_op_adj_ctas: int = 6
    resort_every: Optional[int] = None  # substeps; None = the Horizon's default (one action)
    measured: Dict[str, Dict[str, float]] = field(default_factory=dict)  # candidate -> median ms

    def shapes(self) -> Dict[str, int]:
        return {k: getattr(self, k) for k in CANDIDATES}


def pick(times: Dict[int, Sequence[float]], order: Sequence[int], margin: float = 0.01) -> int:
    """The candidate with the smallest median time.  ``order[0]`` (the current
    choice) is kept unless another candidate's median is below it by more than
    ``margin`` (relative); among those, the fastest wins."""
    med = {c: float(np.median(times[c])) for c in order if times.get(c)}
    if not med:
        raise ValueError("no timings")
    best = order[0] if order[0] in med else min(med, key=med.get)
    fastest = min(med, key=med.get)
    if med[fastest] < med[best] * (1.0 - margin):
        best = fastest
    return best


def coordinate_descent(measure: Callable[[Dict[str, int]], Dict[str, float]], start: Dict[str, int],
                       candidates: Dict[str, Sequence[int]] = CANDIDATES,
                       kinds: Dict[str, Sequence[str]] = KINDS, reps: int = 3, margin: float = 0.01):
    """Tune each field in turn with the others held at their current best.

    ``measure(shapes)`` runs the workload once with those launch shapes and
    returns milliseconds per kernel kind (per launch).  Returns the chosen
    shapes and the median times seen per field and candidate."""
    cur = dict(start)
    seen: Dict[str, Dict[str, float]] = {}
    for name, cands in candidates.items():
        order = [cur[name]] + [c for c in cands if c != cur[name]]
        times: Dict[int, List[float]] = {c: [] for c in order}
        for _ in range(reps):
            for c in order:
                ms = measure(dict(cur, **{name: c}))
                times[c].append(sum(ms.get(k, 0.0) for k in kinds[name]))
        cur[name] = pick(times, order, margin)
        seen[name] = {str(c): float(np.median(v)) for c, v in times.items()}
    return cur, seen


def resort_candidates(n_sub: int, k: int, F: int) -> List[int]:
    """Re-sort intervals (substeps) worth timing: one action (the default), two
    and five actions, half and a fifth of an action, and never (0); each a
    multiple of the checkpoint interval ``k`` and shorter than the horizon ``F``."""
    out = []
    for R in (n_sub, 2 * n_sub, 5 * n_sub, n_sub // 2, n_sub // 5):
        R = k * max(1, -(-R // k))
        if 0 < R < F and R not in out:
            out.append(R)
    out.append(0)
    return out


def workload_key(bt) -> str:
    import torch
    eng, hz = bt.eng, bt.hz
    P = eng.P
    p2 = int(round(float(np.log2(max(P, 1))) * 4))  # particle count to a quarter octave
    return (f"{torch.cuda.get_device_name(eng.device)}|grid={eng.n_grid}|prec={eng.prec}|S={eng.S}|"
            f"P~2^{p2 / 4:.2f}|F={hz.F}|k={hz.k}")


def _cache_path() -> str:
    return os.environ.get("DIFFSKILL_GB300_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "diffskill_gb300", "tuning.json"))


def _load_cache(path: str) -> dict:
    try:
        with open(path) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _store_cache(path: str, key: str, t: Tuning) -> None:
    data = _load_cache(path)
    data[key] = asdict(t)
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as fh:
            json.dump(data, fh, indent=1)
        os.replace(tmp, path)
    except OSError:
        pass  # a read-only home: tuning still applies to this process


def apply(eng, t: Tuning) -> None:
    """Sets the launch shapes of ``t`` on the engine's library handle."""
    from . import _lib
    s = _lib.MpmTuning(*[int(v) for v in t.shapes().values()])
    _lib.check(eng.lib.mpm_set_tuning(eng.h, ctypes.byref(s)), eng.h, "mpm_set_tuning")


def _measure_shapes(bt, shapes: Dict[str, int]) -> Dict[str, float]:
    """One forward + loss + adjoint of a one-action horizon with ``shapes``;
    per-launch milliseconds per kernel kind from the library's profiler."""
    import torch
    eng, hz = bt.eng, bt._tune_hz
    apply(eng, Tuning(**shapes))
    eng.profile(True)
    hz.forward(bt.state0, bt.actions[:1])
    hz.loss(bt.targets, bt.density_weight, bt.contact_weight)
    hz.backward()
    torch.cuda.synchronize()
    prof = eng.profile_read()
    eng.profile(False)
    return {k: ms / cnt for k, (ms, cnt) in prof.items() if cnt}


def _time_iteration(bt, reps: int) -> List[float]:
    import torch
    out = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        bt.forward_backward()
        e1.record()
        torch.cuda.synchronize()
        out.append(e0.elapsed_time(e1))
    return out


def tune(bt, reps: int = 3, use_cache: bool = True, margin: float = 0.01, resort: bool = True) -> Tuning:
    """Tune the launch shapes and the re-sort cadence of a ``BatchedTrajectory``
    (on its own batch, before any CUDA-graph capture), apply them and return them."""
    import torch
    from .engine import Horizon
    eng, hz = bt.eng, bt.hz
    key = workload_key(bt)
    path = _cache_path()
    if use_cache:
        hit = _load_cache(path).get(key)
        if hit:
            t = Tuning(**hit)
            apply(eng, t)
            if t.resort_every is not None:
                hz.set_resort_every(t.resort_every)
            return t
    t = Tuning()
    fields = dict(CANDIDATES)
    if eng.prec != 0:  # the per-kernel variants exist for FP32 only
        for f in FP32_ONLY:
            fields.pop(f)
    # launch shapes on a one-action horizon (checkpoint interval <= 10)
    n = eng.n_sub
    k_short = max(d for d in range(1, min(n, 10) + 1) if n % d == 0)
    bt._tune_hz = Horizon(eng, 1, ckpt_every=k_short, resort_every=0)
    try:
        _measure_shapes(bt, t.shapes())  # warm-up
        shapes, seen = coordinate_descent(lambda s: _measure_shapes(bt, s), t.shapes(), fields, KINDS, reps, margin)
    finally:
        del bt._tune_hz
        torch.cuda.empty_cache()
    for k2, v in shapes.items():
        setattr(t, k2, v)
    t.measured.update(seen)
    apply(eng, t)
    # re-sort cadence on whole iterations
    if resort and hz.F > n:
        cands = resort_candidates(n, hz.k, hz.F)
        times: Dict[int, List[float]] = {}
        default = hz.R
        order = [default] + [c for c in cands if c != default]
        for R in order:
            hz.set_resort_every(R)
            times[R] = _time_iteration(bt, max(2, reps - 1))
        best = pick(times, order, margin)
        hz.set_resort_every(best)
        t.resort_every = best
        t.measured["resort_every"] = {str(c): float(np.median(v)) for c, v in times.items()}
    if use_cache:
        _store_cache(path, key, t)
    return t
