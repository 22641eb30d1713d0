"""Benchmark: fwd+bwd particle-substeps/s of the differentiable MPM substep.

Default workload (N=1): the batched FP32 configuration -- 64 independent
scenes, particle counts log-uniform in [5k, 40k] (seeded), 1-4 dough spheres
and 1-3 tools per scene, 64^3 grid each, 20 actions x 50 substeps, forward +
density-L1 loss + checkpointed adjoint + Adam step on the actions, the whole
iteration captured as one CUDA graph.  One "step" = one such iteration.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload config3|config3-small|config1|config2|config4|config5]
                  [--no-graph] [--no-extras]

For N>1 (torchrun) 64*N scenes are drawn from the same seeded generator and
sharded over the ranks by particle count (diffskill_gb300.sharding): weak
scaling, no collective on the data path; rank 0 prints one JSON line.
``--impl reference`` times the FP64 CPU restatement of the reference substep
(the oracle; the reference's own Taichi runtime does not install here) on the
host cores instead, over a multi-scene sample of the same workload.

The other workloads (config1, 2, 4, 5) print the same line for their own
configuration plus its accuracy report (FP32 / FP32_SVD64 against FP64, the
CPU oracle and central differences, as each configuration asks).
"""
from __future__ import annotations

import argparse
import copy
from dataclasses import asdict
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "fwd+bwd particle-substeps/s: batched FP32 vs plain FP64, action-grad err ≤1e-3"
UNIT = "particle-substeps/s"
WORKLOADS = ["config3", "config3-small", "config1", "config2", "config4", "config5"]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=WORKLOADS, default="config3")
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the plain-FP64 / accuracy / CPU legs")
    ap.add_argument("--ckpt", type=int, default=0, help="checkpoint interval (0 = choose by memory budget)")
    ap.add_argument("--no-tune", action="store_true", help="default launch shapes and re-sort cadence")
    return ap.parse_args()


# ----------------------------------------------------------------------------
# workloads
# ----------------------------------------------------------------------------
def make_workload(name: str, rank: int = 0, world: int = 1, precision: str = "fp32"):
    from diffskill_gb300 import scenes
    from diffskill_gb300.sharding import shard_scenes
    if name == "config3":
        # weak scaling: 64 scenes per rank drawn from one seeded stream, sharded by particle count
        every = scenes.config3(n_scenes=64 * world, seed=1003, precision=precision)
        mine = shard_scenes([s.n_particles for s in every], world, rank)
        scs = [every[i] for i in mine]
        desc = {"workload": "config3: 64 batched scenes per GPU, 5k-40k particles each (log-uniform, seeded), "
                            "1-4 dough spheres + 1-3 tools per scene, 64^3 grid, 20 actions x 50 substeps, "
                            "dt=1e-4, FP32, fwd+loss+adjoint+Adam per step",
                "scenes": len(scs)}
    elif name == "config3-small":  # profiling case: a few GB on the device
        scs = scenes.config3(seed=1003, precision=precision)[:16]
        for sc in scs:
            sc.actions = sc.actions[:2]
        desc = {"workload": "config3-small: the first 16 scenes of config3, 2 actions x 50 substeps, FP32 "
                            "(profiling case)", "scenes": len(scs)}
    elif name == "config2":
        scs = [scenes.config2(precision=precision)]
        desc = {"workload": "config2: single scene, 30k particles, box spatula + capsule, 64^3, "
                            "50 actions x 50 substeps, dt=1e-4, checkpoint every 10", "scenes": 1}
    elif name == "config4":
        scs = [scenes.config4(precision=precision)]
        desc = {"workload": "config4: single scene, 100k particles, knife (box ∩ prism) + two-finger gripper, "
                            "128^3, 30 actions x 50 substeps, density L1 to two piles + soft contact term",
                "scenes": 1}
    elif name == "config5":
        scs = scenes.config5(precision=precision)
        desc = {"workload": "config5: 16 batched scenes, 100k-500k particles each (log-uniform, seeded), "
                            "128^3 grids, 3 tools each, 100 actions x 50 substeps, checkpoint interval planned "
                            "to fit HBM", "scenes": len(scs)}
    else:
        sc = scenes.config1(dt=1e-4)
        sc.sim.precision = precision
        scs = [sc]
        desc = {"workload": "config1: single scene, 10k particles, capsule, 64^3, 10 actions x 50 substeps, "
                            "dt=1e-4 (the stated 5e-4 is unstable), FP64 plain method", "scenes": 1}
    return scs, desc


def choose_checkpoint(scs, budget_frac: float = 0.5) -> int:
    """Smallest checkpoint interval (dividing the horizon) whose stored frames fit the budget."""
    import torch
    from diffskill_gb300.engine import plan_checkpoint_interval
    P = sum(sc.n_particles for sc in scs)
    F = scs[0].n_actions * scs[0].sim.n_substeps
    w = 8 if scs[0].sim.precision_code == 2 else 4
    frame = 24 * (-(-P // 32) * 32) * w
    free, _ = torch.cuda.mem_get_info()
    try:
        return plan_checkpoint_interval(F, frame, int(budget_frac * free))
    except MemoryError:
        return scs[0].sim.n_substeps


def with_precision(scs, precision: str):
    out = [copy.deepcopy(s) for s in scs]
    for s in out:
        s.sim.precision = precision
    return out


# ----------------------------------------------------------------------------
# clocks sampled during the timed region
# ----------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.dev)], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ----------------------------------------------------------------------------
# roofline bookkeeping
# ----------------------------------------------------------------------------
# Algorithmic bytes per unit (words; particle units for particle kernels,
# grid-node units for grid kernels) of the compulsory-traffic model.  The
# adjoint's p2g recompute is not listed: with the grid store holding the
# substep (every substep at checkpoint interval 1) it returns at once and
# moves no bytes of its own.
ALGO_WORDS = {"p2g": ("particle", 33), "g2p": ("particle", 18), "g2p_adj": ("particle", 21),
              "p2g_adj": ("particle", 60), "grid_op": ("node", 8), "grid_op_adj": ("node", 12)}


def active_blocks(xs, n_grid: int) -> int:
    """Number of 4^3-node grid blocks the particle stencils touch (summed over
    scenes), the unit count of the sparse grid kernels."""
    nb = n_grid // 4
    tot = 0
    for x in xs:
        base = np.clip((np.asarray(x) * n_grid - 0.5).astype(np.int64), 0, n_grid - 3)
        keys = set()
        for o in (0, 2):
            for q in (0, 2):
                for r in (0, 2):
                    b = (base + np.array([o, q, r])) >> 2
                    keys.update(((b[:, 0] * nb + b[:, 1]) * nb + b[:, 2]).tolist())
        tot += len(keys)
    return tot


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel: str, workload: str):
    """DRAM bytes per launch of ``kernel`` from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "roofline_traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 3 and parts[0] == workload and parts[1] == kernel:
            try:
                return float(parts[2])
            except ValueError:
                return None
    return None


def kernel_table(eng, prof, final_state, w):
    fin = final_state[0:3, :eng.P].double().cpu().numpy().T
    xs = [fin[int(eng.offsets[i]):int(eng.offsets[i + 1])] for i in range(eng.S)]
    nblk = active_blocks(xs, eng.n_grid)
    units = {"particle": eng.P, "node": nblk * 64}
    kern = {}
    for kname, (tot_ms, cnt) in prof.items():
        if cnt == 0:
            continue
        entry = {"launches": cnt, "total_ms": round(tot_ms, 4), "avg_us": round(1e3 * tot_ms / cnt, 3)}
        if kname in ALGO_WORDS:
            unit, words = ALGO_WORDS[kname]
            b = units[unit] * words * w
            entry["algo_bytes_per_launch"] = b
            entry["achieved_gbs"] = round(b / (tot_ms / cnt * 1e-3) / 1e9, 1)
        kern[kname] = entry
    total_prof = sum(v["total_ms"] for v in kern.values())
    for v in kern.values():
        v["share"] = round(v["total_ms"] / total_prof, 4)
    return kern, nblk


def roofline_of(kern, workload):
    dom = max((k2 for k2 in kern if k2 in ALGO_WORDS), key=lambda k2: kern[k2]["total_ms"])
    peak, peak_kind = measured_peaks()
    d = kern[dom]
    return {"bound": "hbm", "kernel": dom, "achieved": d["achieved_gbs"], "peak": peak, "unit": "GB/s",
            "frac": round(d["achieved_gbs"] / peak, 4), "peak_source": f"{peak_kind} hbm_gbs (of {peak_kind})",
            "algo_bytes_per_launch": d["algo_bytes_per_launch"], "avg_launch_us": d["avg_us"],
            "traffic": ncu_traffic(dom, workload), "share_of_step": d["share"]}


# ----------------------------------------------------------------------------
# timing helpers
# ----------------------------------------------------------------------------
def timed(fn, steps: int, warmup: int, dist=None):
    """Device-timed milliseconds per call of ``fn`` (CUDA events on the current
    stream, barrier + synchronize on both sides)."""
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    return e0.elapsed_time(e1) / steps


def grad_errors(g_test, g_ref, rel_floor: float = 1e-6):
    """Per-scene relative action-gradient errors, L2 and max norms.  Scenes whose
    reference gradient is below ``rel_floor`` of the median norm (tools not
    acting on the dough) have no defined relative error and are listed as excluded."""
    norms = [float(np.linalg.norm(b)) for b in g_ref]
    med = float(np.median(norms)) if norms else 0.0
    l2, mx, excl = [], [], []
    for i, (a, b) in enumerate(zip(g_test, g_ref)):
        if norms[i] <= rel_floor * med:
            excl.append(i)
            continue
        l2.append(float(np.linalg.norm(a - b) / norms[i]))
        mx.append(float(np.abs(a - b).max() / np.abs(b).max()))
    return {"action_grad_rel_err_l2_median": float(np.median(l2)) if l2 else None,
            "action_grad_rel_err_l2_max": max(l2) if l2 else None,
            "action_grad_rel_err_maxnorm_median": float(np.median(mx)) if mx else None,
            "action_grad_rel_err_maxnorm_max": max(mx) if mx else None,
            "scenes_within_1e-3_l2": int(sum(e <= 1e-3 for e in l2)), "scenes_compared": len(l2),
            "excluded_zero_gradient": excl, "per_scene_l2": [round(e, 7) for e in l2]}


def loss_errors(l_test, l_ref):
    l_test, l_ref = np.asarray(l_test, dtype=np.float64), np.asarray(l_ref, dtype=np.float64)
    rel = np.abs(l_test - l_ref) / np.maximum(np.abs(l_ref), 1e-300)
    return {"loss_rel_err_median": float(np.median(rel)), "loss_rel_err_max": float(rel.max())}


def run_trajectory(scs, k, grads=True):
    """Eager forward (+ adjoint) of a batch; returns (per-scene loss, per-scene action grads)."""
    import torch
    from diffskill_gb300.trajectory import BatchedTrajectory
    bt = BatchedTrajectory(scs, ckpt_every=k)
    if grads:
        bt.forward_backward()
    else:
        bt.forward_only()
    torch.cuda.synchronize()
    bt.eng.check_status()
    loss = bt.loss.cpu().numpy().copy()
    g = [x.detach().cpu().numpy().copy() for x in bt.action_grads()] if grads else None
    del bt
    torch.cuda.empty_cache()
    return loss, g


def throughput_pair(scs, k, steps, warmup, graph=True, tune=True):
    """fwd+bwd (+Adam) and forward-only particle-substeps/s of a batch, graph-captured."""
    import torch
    from diffskill_gb300.trajectory import BatchedTrajectory
    bt = BatchedTrajectory(scs, ckpt_every=k, autotune=tune)
    ps = bt.particle_substeps
    if graph:
        bt.capture()
    ms = timed(bt.step, steps, warmup)
    if graph:
        bt.graph = None
        gf = bt.capture_forward()
        ms_f = timed(gf.replay, steps, warmup)
        del gf
    else:
        ms_f = timed(bt.forward_only, steps, warmup)
    bt.eng.check_status()
    del bt
    torch.cuda.empty_cache()
    return {"fwd_bwd": ps / (ms * 1e-3), "fwd_only": ps / (ms_f * 1e-3), "ms_fwd_bwd": ms, "ms_fwd_only": ms_f,
            "particle_substeps": ps, "checkpoint_every": k, "cuda_graph": graph}


# ----------------------------------------------------------------------------
# our arm, config 3 (the headline line)
# ----------------------------------------------------------------------------
def run_ours(args, rank, world, dist):
    import torch
    from diffskill_gb300.trajectory import BatchedTrajectory

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    scs, desc = make_workload(args.workload, rank, world)
    k = args.ckpt or (10 if args.workload == "config3-small" else choose_checkpoint(scs))
    # launch shapes and re-sort cadence picked by measurement on this batch (diffskill_gb300.autotune)
    bt = BatchedTrajectory(scs, ckpt_every=k, autotune=not args.no_tune)
    eng = bt.eng
    ps = bt.particle_substeps  # per iteration on this rank

    # reference point for accuracy: grads at the initial actions (eager)
    bt.forward_backward()
    torch.cuda.synchronize()
    eng.check_status()
    grad0 = [g.detach().cpu().numpy() for g in bt.action_grads()]
    loss0 = bt.loss.cpu().numpy().copy()
    launches0 = eng.launches
    bt.forward_backward()
    bt.adam()
    torch.cuda.synchronize()
    launches_per_step = eng.launches - launches0
    use_graph = not args.no_graph
    if use_graph:
        bt.reset_optimizer([sc.actions for sc in scs])
        bt.capture()

    # ---- device-resident timed region
    stream = torch.cuda.current_stream()
    with ClockSampler(dev) as clk:
        ms = timed(bt.step, args.steps, args.warmup, dist)
    clocks = clk.summary()
    eng.check_status()

    # ---- end to end: host inputs in, host results out, through the public API
    # the caller's positions in the caller's particle order; the library sorts them by cell on the device
    x_host = torch.from_numpy(np.ascontiguousarray(np.concatenate([sc.x0 for sc in scs]).T.astype(np.float32)))
    x_host = x_host.pin_memory()
    a_host = bt.actions.detach().cpu().pin_memory()
    loss_host = torch.empty(bt.loss.shape, dtype=bt.loss.dtype).pin_memory()
    grad_host = torch.empty(bt.grad.shape, dtype=bt.grad.dtype).pin_memory()
    xdev = torch.empty(x_host.shape, dtype=torch.float32, device=eng.device)
    h2d = x_host.numel() * x_host.element_size() + a_host.numel() * a_host.element_size()
    d2h = loss_host.numel() * loss_host.element_size() + grad_host.numel() * grad_host.element_size()

    def e2e_step():
        xdev.copy_(x_host, non_blocking=True)
        bt.set_initial_positions(xdev)
        bt.actions.copy_(a_host, non_blocking=True)
        bt.step()
        loss_host.copy_(bt.loss, non_blocking=True)
        grad_host.copy_(bt.grad, non_blocking=True)

    t0 = time.perf_counter()
    e2e_ms = timed(e2e_step, args.steps, 0, dist)
    e2e_wall = (time.perf_counter() - t0) / args.steps
    e2e_ms = max(e2e_ms, e2e_wall * 1e3)

    # ---- forward only (forward + loss, no adjoint), graph-captured
    if use_graph:
        bt.graph = None
        gf = bt.capture_forward()
        ms_fwd = timed(gf.replay, args.steps, args.warmup, dist)
        del gf
    else:
        ms_fwd = timed(bt.forward_only, args.steps, args.warmup, dist)

    # ---- instrumented pass (outside the timed regions): per-kernel CUDA events
    # (an NVTX range, so that a profiler can capture exactly this iteration:
    # ncu --nvtx --nvtx-include "mpm_iteration/")
    eng.profile(True)
    torch.cuda.nvtx.range_push("mpm_iteration")
    bt.forward_backward()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    prof = eng.profile_read()
    eng.profile(False)
    w = 4 if eng.dtype == torch.float32 else 8
    kern, nblk = kernel_table(eng, prof, bt.hz.final, w)
    roofline = roofline_of(kern, args.workload)
    P, S, G = eng.P, eng.S, eng.G
    F = bt.hz.F
    tuning = None
    if bt.tuning is not None:
        tuning = {k2: v for k2, v in asdict(bt.tuning).items() if k2 != "measured"}
        tuning["resort_every"] = bt.hz.R
    del bt, eng
    torch.cuda.empty_cache()

    # ---- aggregate over ranks
    tot_ps = ps * world
    if dist is not None:
        t = torch.tensor([ms, e2e_ms, ms_fwd], dtype=torch.float64, device=f"cuda:{dev}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms, e2e_ms, ms_fwd = float(t[0]), float(t[1]), float(t[2])
    if rank != 0:
        return None

    out = {
        "metric": METRIC, "value": tot_ps / (ms * 1e-3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded; reference datasets not shipped)",
        "config": dict(desc, particles_per_rank=P, substeps_per_step=F, checkpoint_every=k,
                       active_grid_blocks_final=nblk, grid_blocks_total=S * G // 64,
                       cuda_graph=use_graph, parallelism=f"scene-sharded x{world}" if world > 1 else "single GPU",
                       tuning=tuning,
                       l2="working set per step far above the 129 MB L2 (state frames + 4 grids)"),
        "e2e": {"value": tot_ps / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": h2d * world,
                "d2h_bytes_per_step": d2h * world},
        "fwd_only": {"value": tot_ps / (ms_fwd * 1e-3), "unit": UNIT, "ms_per_step": ms_fwd,
                     "what": "forward of all actions + density loss, no adjoint, no grid store, CUDA graph"},
        "gpu_launches": launches_per_step * args.steps,
        "roofline": roofline, "kernels": kern, "clocks": clocks,
    }
    if not args.no_extras:
        out.update(extras(args, scs, grad0, loss0, k))
    return out


def extras(args, scs, grad0, loss0, k):
    """Plain FP64 single-scene GPU path, FP32 gradient error vs FP64, the
    spec precision mode (FP32 state, FP64 SVD), CPU baseline."""
    from diffskill_gb300 import scenes
    res = {}
    # plain reference method on the GPU: config 1 in full, FP64, every frame stored, eager and graph-captured
    sc = scenes.config1(dt=1e-4)
    eager = throughput_pair([sc], 1, steps=2, warmup=1, graph=False, tune=False)
    graph = throughput_pair([sc], 1, steps=3, warmup=1, graph=True, tune=False)
    res["plain_fp64"] = {"value": eager["fwd_bwd"], "unit": UNIT, "graph_value": graph["fwd_bwd"],
                         "fwd_only_eager": eager["fwd_only"], "fwd_only_graph": graph["fwd_only"],
                         "workload": "config1: single scene FP64, 10k particles, capsule, 10 actions x 50 substeps, "
                                     "all frames stored (the reference's store-all tape)",
                         "batched_fp32_over_plain_fp64": None, "batched_fp32_over_plain_fp64_graph": None}
    # FP32 action gradients vs the FP64 GPU path on the same scenes (first 16)
    sub = scs[:16]
    l64, g64 = run_trajectory(with_precision(sub, "fp64"), 10)
    acc = grad_errors(grad0[:len(g64)], g64)
    acc.update(loss_errors(loss0[:len(l64)], l64))
    acc["scenes_checked"] = len(g64)
    acc["reference"] = "FP64 GPU path on the same scenes and actions (itself within 1e-9 of the FP64 CPU oracle)"
    res["accuracy"] = acc
    # the spec precision design: FP32 state and grid, FP64 SVD / return map / stress and their adjoints
    s64 = with_precision(scs, "fp32_svd64")
    # (no autotuning here: the tuned launch shapes are the FP32 kernels'; the re-sort
    # candidates would each cost a 6-second iteration)
    tp = throughput_pair(s64, k, steps=2, warmup=1, graph=not args.no_graph, tune=False)
    l_m, g_m = run_trajectory(with_precision(sub, "fp32_svd64"), 10)
    acc_m = grad_errors(g_m, g64)
    acc_m.update(loss_errors(l_m, l64))
    res["fp32_svd64"] = {"value": tp["fwd_bwd"], "unit": UNIT, "fwd_only": tp["fwd_only"],
                         "ms_per_step": tp["ms_fwd_bwd"], "accuracy_first16": acc_m,
                         "what": "same workload and iteration in MPM_PREC_FP32_SVD64 (CUDA graph)"}
    # CPU baseline: the FP64 oracle on the host cores, bounded multi-scene sample of the same workload
    res["cpu_baseline"] = cpu_baseline(scs)
    return res


def cpu_sample_scenes(scs, n: int = 8):
    """``n`` scenes spread over the particle-count range of the batch."""
    order = sorted(range(len(scs)), key=lambda i: scs[i].n_particles)
    pick = sorted({order[int(round(j * (len(order) - 1) / max(n - 1, 1)))] for j in range(n)})
    return [scs[i] for i in pick]


def cpu_baseline(scs, threads: int = 0):
    """FP64 oracle fwd+bwd on the host cores: 8 scenes across the size range,
    one action each (50 substeps), after a one-action warm-up; median of 3
    throughputs.  The first scene of config 1 in full is reported beside it."""
    from diffskill_gb300 import scenes
    from oracle import oracle as O
    threads = threads or os.cpu_count() or 1
    O.set_num_threads(threads)
    sample = cpu_sample_scenes(scs)
    O.time_fwd_bwd(sample[0], 1, threads)  # warm-up: one action
    vals = []
    for _ in range(3):
        t_tot, ps_tot = 0.0, 0
        for sc in sample:
            dt, ps = O.time_fwd_bwd(sc, 1, threads)
            t_tot += dt
            ps_tot += ps
        vals.append(ps_tot / t_tot)
    c1 = scenes.config1(dt=1e-4)
    O.time_fwd_bwd(c1, 1, threads)
    c1_vals = []
    for _ in range(3):
        dt, ps = O.time_fwd_bwd(c1, c1.n_actions, threads)
        c1_vals.append(ps / dt)
    ns = [s.n_particles for s in sample]
    return {"value": float(np.median(vals)), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"FP64 oracle fwd+bwd (store-all), {len(sample)} scenes of the workload spread over its "
                      f"size range ({min(ns)}-{max(ns)} particles), 1 action x 50 substeps each, median of 3 "
                      f"after a 1-action warm-up",
            "config1_full": {"value": float(np.median(c1_vals)), "unit": UNIT,
                             "sample": "config1 in full: 10k particles, 10 actions x 50 substeps, median of 3"}}


# ----------------------------------------------------------------------------
# the other configurations: throughput + accuracy reports
# ----------------------------------------------------------------------------
def central_differences(sc, coords, eps: float, k: int):
    """FP64 central differences of the loss along action coordinates (action, dim)."""
    out = []
    for (a, d) in coords:
        vals = []
        for sgn in (1.0, -1.0):
            s2 = copy.deepcopy(sc)
            s2.sim.precision = "fp64"
            s2.actions = s2.actions.copy()
            s2.actions[a, d] += sgn * eps
            l, _ = run_trajectory([s2], k, grads=False)
            vals.append(float(l[0]))
        out.append((vals[0] - vals[1]) / (2 * eps))
    return np.array(out)


def run_config(args, rank, world, dist):
    import torch
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    name = args.workload
    if name == "config1":
        prec_main = "fp64"
    elif name == "config4":
        prec_main = "fp32_svd64"
    else:
        prec_main = "fp32"
    scs, desc = make_workload(name, rank, world, prec_main)

    def k_for(batch):
        # the configuration's own interval, or the one the planner fits into HBM for this precision
        ce = batch[0].checkpoint_every
        return args.ckpt or (ce if ce != "auto" else 0) or choose_checkpoint(batch, 0.55)

    k = k_for(scs)
    rep = {"precision": prec_main}
    with ClockSampler(dev) as clk:
        tp = throughput_pair(scs, k, args.steps, args.warmup, graph=not args.no_graph)
    clocks = clk.summary()
    rep["throughput"] = tp
    # accuracy: the main mode against FP64 (and the other FP32 mode against both for configs 2, 4, 5)
    l_main, g_main = run_trajectory(scs, k)
    s64 = with_precision(scs, "fp64")
    if prec_main == "fp64":
        l64, g64 = l_main, g_main
    else:
        k64 = k_for(s64)
        t0 = time.perf_counter()
        l64, g64 = run_trajectory(s64, k64)
        rep["fp64"] = {"checkpoint_every": k64, "eager_fwd_bwd_s": time.perf_counter() - t0}
        rep[f"{prec_main}_vs_fp64"] = dict(grad_errors(g_main, g64), **loss_errors(l_main, l64))
    if name in ("config4", "config5", "config2"):
        other = "fp32" if prec_main != "fp32" else "fp32_svd64"
        so = with_precision(scs, other)
        ko = k_for(so)
        if name == "config5":
            # FP64 SVD at GB300's FP64 rate: one eager iteration, timed, serves both throughput and accuracy
            t0 = time.perf_counter()
            l_o, g_o = run_trajectory(so, ko)
            dt_o = time.perf_counter() - t0
            tp_o = {"fwd_bwd": tp["particle_substeps"] / dt_o, "checkpoint_every": ko, "cuda_graph": False,
                    "what": "one eager forward+loss+adjoint, wall time"}
        else:
            tp_o = throughput_pair(so, ko, max(1, args.steps // 2), 1, graph=not args.no_graph)
            l_o, g_o = run_trajectory(so, ko)
        rep[other] = {"throughput": tp_o, "vs_fp64": dict(grad_errors(g_o, g64), **loss_errors(l_o, l64)),
                      f"vs_{prec_main}": grad_errors(g_o, g_main)}
    if name == "config1":
        from oracle.oracle import Oracle
        sc = scs[0]
        o_loss, o_grad = Oracle(sc.sim, sc.tools).loss_and_grad(sc.x0, sc.actions, sc.target)
        coords = [(a, d) for a in range(sc.n_actions) for d in range(3)]
        fd = central_differences(sc, coords, 1e-3, k)
        g = g64[0].reshape(-1)
        rep["vs_cpu_oracle"] = {"loss": float(l64[0]), "oracle_loss": float(o_loss),
                                "loss_rel_err": abs(float(l64[0]) - o_loss) / abs(o_loss),
                                "grad_rel_err_l2": float(np.linalg.norm(g - o_grad.reshape(-1)) /
                                                         np.linalg.norm(o_grad)),
                                "grad_rel_err_max": float(np.abs(g - o_grad.reshape(-1)).max() /
                                                          np.abs(o_grad).max())}
        rep["vs_central_differences"] = {"eps": 1e-3, "coords": "all 30 action scalars",
                                         "rel_err_l2": float(np.linalg.norm(g - fd) / np.linalg.norm(fd)),
                                         "per_coord_rel_err_median": float(np.median(
                                             np.abs(g - fd) / np.maximum(np.abs(fd), 1e-12)))}
        rep["action_grad"] = [round(float(x), 9) for x in g]
    if name == "config2":
        sc = scs[0]
        rng = np.random.default_rng(2002)
        flat = rng.choice(sc.actions.size, size=8, replace=False)
        coords = [(int(i) // sc.actions.shape[1], int(i) % sc.actions.shape[1]) for i in flat]
        fd = central_differences(sc, coords, 1e-3, k)
        g32 = np.array([g_main[0][a, d] for a, d in coords])
        g64c = np.array([g64[0][a, d] for a, d in coords])
        rep["vs_central_differences"] = {
            "eps": 1e-3, "coords": coords, "fd_fp64": fd.tolist(), "fp32_adjoint": g32.tolist(),
            "fp64_adjoint": g64c.tolist(),
            "fp32_rel_err_l2": float(np.linalg.norm(g32 - fd) / np.linalg.norm(fd)),
            "fp64_rel_err_l2": float(np.linalg.norm(g64c - fd) / np.linalg.norm(fd))}
    if rank != 0:
        return None
    ps = tp["particle_substeps"]
    return {"metric": METRIC, "value": tp["fwd_bwd"] * world, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": tp["ms_fwd_bwd"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": {"fp64": "f64", "fp32": "f32"}.get(prec_main, "f32+f64svd"),
            "data": "synthetic (seeded)", "config": dict(desc, particle_substeps_per_step=ps, checkpoint_every=k),
            "fwd_only": {"value": tp["fwd_only"] * world, "unit": UNIT, "ms_per_step": tp["ms_fwd_only"]},
            "clocks": clocks, "report": rep}


# ----------------------------------------------------------------------------
# reference arm: the reference's CPU path, restated (taichi is not installable)
# ----------------------------------------------------------------------------
def run_reference(args, rank, world):
    if rank != 0:
        return None
    from oracle import oracle as O
    scs, desc = make_workload(args.workload, 0, 1)
    sample = cpu_sample_scenes(scs) if len(scs) > 1 else scs
    threads = os.cpu_count() or 1
    O.set_num_threads(threads)
    # one step = the next scene of the sample, fwd+bwd over one action (50 substeps)
    times, pss = [], []
    for i in range(args.warmup + args.steps):
        sc = sample[i % len(sample)]
        dt, ps = O.time_fwd_bwd(sc, 1, threads)
        if i >= args.warmup:
            times.append(dt)
            pss.append(ps)
    ms = 1e3 * float(np.mean(times))
    val = float(np.sum(pss)) / float(np.sum(times))
    ns = [s.n_particles for s in sample]
    sample_txt = (f"FP64 CPU restatement of the reference substep (oracle), store-all fwd+bwd; each step one "
                  f"action (50 substeps) of the next of {len(sample)} scenes of the workload spread over its size "
                  f"range ({min(ns)}-{max(ns)} particles)")
    return {"metric": METRIC, "value": val, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "config": desc, "impl": "reference",
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample_txt},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "taichi==0.7.26 (the reference runtime) does not install on Python 3.12; the reference arm "
                    "times the line-by-line FP64 C++/OpenMP restatement of its substep"}


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as tdist
        backend = "nccl" if (args.impl == "ours" and torch.cuda.is_available()) else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        tdist.init_process_group(backend=backend)
        dist = tdist
    if args.impl == "reference":
        out = run_reference(args, rank, world)
    elif args.workload in ("config3", "config3-small"):
        out = run_ours(args, rank, world, dist)
        if out is not None and "plain_fp64" in out:
            per_gpu = out["value"] / world
            out["plain_fp64"]["batched_fp32_over_plain_fp64"] = per_gpu / out["plain_fp64"]["value"]
            out["plain_fp64"]["batched_fp32_over_plain_fp64_graph"] = per_gpu / out["plain_fp64"]["graph_value"]
    else:
        out = run_config(args, rank, world, dist)
    if out is not None:
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
