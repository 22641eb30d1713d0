"""Benchmark: fwd+bwd particle-substeps/s of the differentiable MPM substep.

Default workload (N=1): the batched FP32 configuration -- 64 independent
scenes, particle counts log-uniform in [5k, 40k] (seeded), 1-4 dough spheres
and 1-3 tools per scene, 64^3 grid each, 20 actions x 50 substeps, forward +
density-L1 loss + checkpointed adjoint + Adam step on the actions, the whole
iteration captured as one CUDA graph.  One "step" = one such iteration.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload config3|config2|config1] [--no-graph]

For N>1 (torchrun) every rank runs its own seeded batch of scenes (weak
scaling, no collective on the data path); rank 0 prints one JSON line.
``--impl reference`` times the FP64 CPU restatement of the reference substep
(the oracle; the reference's own Taichi runtime does not install here) on the
host cores instead.
"""
from __future__ import annotations

import argparse
import copy
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "fwd+bwd particle-substeps/s: batched FP32 vs plain FP64, action-grad err ≤1e-3"
UNIT = "particle-substeps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["config3", "config3-small", "config2", "config1"], default="config3")
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip plain-FP64 / accuracy / CPU legs")
    ap.add_argument("--ckpt", type=int, default=0, help="checkpoint interval (0 = choose by memory budget)")
    return ap.parse_args()


# ----------------------------------------------------------------------------
# workloads
# ----------------------------------------------------------------------------
def make_workload(name: str, rank: int, precision: str = "fp32"):
    from diffskill_gb300 import scenes
    if name == "config3":
        scs = scenes.config3(seed=1003 + 7919 * rank, precision=precision)
        desc = {"workload": "config3: 64 batched scenes, 5k-40k particles each (log-uniform, seeded), "
                            "1-4 dough spheres + 1-3 tools per scene, 64^3 grid, 20 actions x 50 substeps, "
                            "dt=1e-4, FP32, fwd+loss+adjoint+Adam per step",
                "scenes": len(scs)}
    elif name == "config3-small":  # profiling case: a few GB on the device
        scs = scenes.config3(seed=1003 + 7919 * rank, precision=precision)[:16]
        for sc in scs:
            sc.actions = sc.actions[:2]
        desc = {"workload": "config3-small: the first 16 scenes of config3, 2 actions x 50 substeps, FP32 "
                            "(profiling case)", "scenes": len(scs)}
    elif name == "config2":
        scs = [scenes.config2(seed=1002 + 7919 * rank, precision=precision)]
        desc = {"workload": "config2: single scene, 30k particles, box spatula + capsule, 64^3, "
                            "50 actions x 50 substeps, dt=1e-4, FP32, checkpoint every 10", "scenes": 1}
    else:
        sc = scenes.config1(dt=1e-4, seed=1001 + 7919 * rank)
        sc.sim.precision = precision
        scs = [sc]
        desc = {"workload": "config1: single scene, 10k particles, capsule, 64^3, 10 actions x 50 substeps, "
                            "dt=1e-4 (the stated 5e-4 is unstable)", "scenes": 1}
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
# our arm
# ----------------------------------------------------------------------------
# algorithmic bytes per unit (words; particle units for particle kernels,
# grid-node units for grid kernels) of the compulsory-traffic model
ALGO_WORDS = {"p2g": ("particle", 33), "p2g_recompute": ("particle", 24), "g2p": ("particle", 18),
              "g2p_adj": ("particle", 21), "p2g_adj": ("particle", 60), "grid_op": ("node", 8),
              "grid_op_adj": ("node", 12)}


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


def run_ours(args, rank, world, dist):
    import torch
    from diffskill_gb300.trajectory import BatchedTrajectory

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    scs, desc = make_workload(args.workload, rank)
    k = args.ckpt or (10 if args.workload == "config3-small" else choose_checkpoint(scs))
    bt = BatchedTrajectory(scs, ckpt_every=k)
    eng = bt.eng
    ps = bt.particle_substeps  # per iteration on this rank

    # reference point for accuracy: grads at the initial actions (eager)
    bt.forward_backward()
    torch.cuda.synchronize()
    eng.check_status()
    grad0 = [g.detach().cpu().numpy() for g in bt.action_grads()]
    launches0 = eng.launches
    bt.forward_backward()
    bt.adam()
    torch.cuda.synchronize()
    launches_per_step = eng.launches - launches0
    use_graph = not args.no_graph
    if use_graph:
        bt.reset_optimizer([sc.actions for sc in scs])
        bt.capture()
    for _ in range(args.warmup):
        bt.step()
    torch.cuda.synchronize()

    def barrier():
        if dist is not None:
            dist.barrier()

    # ---- device-resident timed region
    barrier()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            bt.step()
        e1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = e0.elapsed_time(e1) / args.steps
    clocks = clk.summary()
    eng.check_status()

    # ---- end to end: host inputs in, host results out, through the public API
    x_host = torch.from_numpy(np.concatenate([sc.x0 for sc in scs]).T.astype(np.float32)).pin_memory()
    a_host = bt.actions.detach().cpu().pin_memory()
    loss_host = torch.empty(bt.loss.shape, dtype=bt.loss.dtype).pin_memory()
    grad_host = torch.empty(bt.grad.shape, dtype=bt.grad.dtype).pin_memory()
    xdev = torch.empty(x_host.shape, dtype=torch.float32, device=eng.device)
    h2d = x_host.numel() * x_host.element_size() + a_host.numel() * a_host.element_size()
    d2h = loss_host.numel() * loss_host.element_size() + grad_host.numel() * grad_host.element_size()
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(args.steps):
        xdev.copy_(x_host, non_blocking=True)
        bt.state0[0:3, :eng.P].copy_(xdev.to(bt.state0.dtype))
        bt.actions.copy_(a_host, non_blocking=True)
        bt.step()
        loss_host.copy_(bt.loss, non_blocking=True)
        grad_host.copy_(bt.grad, non_blocking=True)
    f1.record(stream)
    torch.cuda.synchronize()
    e2e_wall = (time.perf_counter() - t0) / args.steps
    e2e_ms = max(f0.elapsed_time(f1) / args.steps, e2e_wall * 1e3)
    barrier()

    # ---- instrumented pass (outside the timed region): per-kernel CUDA events
    # (an NVTX range, so that a profiler can capture exactly this iteration:
    # ncu --nvtx --nvtx-include "mpm_iteration/")
    eng.profile(True)
    torch.cuda.nvtx.range_push("mpm_iteration")
    bt.forward_backward()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    prof = eng.profile_read()
    eng.profile(False)

    # ---- aggregate over ranks
    tot_ps = ps * world
    if dist is not None:
        t = torch.tensor([ms, e2e_ms], dtype=torch.float64, device=eng.device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms, e2e_ms = float(t[0]), float(t[1])
    if rank != 0:
        return None

    w = 4 if eng.dtype == torch.float32 else 8
    fin = bt.hz.final[0:3, :eng.P].double().cpu().numpy().T
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
    dom = max((k2 for k2 in kern if k2 in ALGO_WORDS), key=lambda k2: kern[k2]["total_ms"])
    peak, peak_kind = measured_peaks()
    d = kern[dom]
    traffic = ncu_traffic(dom, args.workload)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": d["achieved_gbs"], "peak": peak, "unit": "GB/s",
                "frac": round(d["achieved_gbs"] / peak, 4), "peak_source": f"{peak_kind} hbm_gbs",
                "algo_bytes_per_launch": d["algo_bytes_per_launch"], "avg_launch_us": d["avg_us"],
                "traffic": traffic, "share_of_step": d["share"]}

    out = {
        "metric": METRIC, "value": tot_ps / (ms * 1e-3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded; reference datasets not shipped)",
        "config": dict(desc, particles_per_rank=eng.P, substeps_per_step=bt.hz.F, checkpoint_every=k,
                       active_grid_blocks_final=nblk, grid_blocks_total=eng.S * eng.G // 64,
                       cuda_graph=use_graph, parallelism=f"scene-sharded x{world}" if world > 1 else "single GPU",
                       l2="working set per step far above the 129 MB L2 (state frames + 4 grids)"),
        "e2e": {"value": tot_ps / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": h2d * world,
                "d2h_bytes_per_step": d2h * world},
        "gpu_launches": launches_per_step * args.steps,
        "roofline": roofline, "kernels": kern, "clocks": clocks,
    }
    if not args.no_extras:
        out.update(extras(args, scs, grad0, bt))
    return out


def extras(args, scs, grad0, bt):
    """Plain FP64 single-scene GPU path, FP32 gradient error vs FP64, CPU baseline."""
    import torch
    from diffskill_gb300 import scenes
    from diffskill_gb300.trajectory import BatchedTrajectory
    res = {}
    # plain reference method on the GPU: one scene, FP64, every frame stored, no graph
    sc = scenes.config1(dt=1e-4)
    sc.actions = sc.actions[:4]
    p64 = BatchedTrajectory([sc], ckpt_every=1)
    p64.forward_backward()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    reps = 2
    for _ in range(reps):
        p64.forward_backward()
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / reps
    plain = p64.particle_substeps / dt
    res["plain_fp64"] = {"value": plain, "unit": UNIT,
                         "workload": "single scene FP64, 10k particles, capsule, 4 actions x 50 substeps, "
                                     "all frames stored, eager launches",
                         "batched_fp32_over_plain_fp64": None}
    del p64
    # FP32 action gradients vs the FP64 GPU path on the same scenes (first 16, checkpointed)
    sub = [copy.deepcopy(s) for s in scs[:16]]
    for s in sub:
        s.sim.precision = "fp64"
    r64 = BatchedTrajectory(sub, ckpt_every=10)
    r64.forward_backward()
    torch.cuda.synchronize()
    g64 = [g.detach().cpu().numpy() for g in r64.action_grads()]
    del r64
    torch.cuda.empty_cache()
    res["accuracy"] = grad_errors(grad0[:len(g64)], g64)
    res["accuracy"]["scenes_checked"] = len(g64)
    # CPU baseline: the FP64 oracle on the host cores, bounded sample of the same workload
    res["cpu_baseline"] = cpu_baseline(scs[0], target_s=12.0)
    return res


def grad_errors(g32, g64):
    """Per-scene relative action-gradient errors, L2 and max norms.  Scenes whose
    FP64 gradient is below 1e-6 of the median norm (tools not acting on the
    dough) have no defined relative error and are listed as excluded."""
    norms = [float(np.linalg.norm(b)) for b in g64]
    med = float(np.median(norms)) if norms else 0.0
    l2, mx, excl = [], [], []
    for i, (a, b) in enumerate(zip(g32, g64)):
        if norms[i] <= 1e-6 * med:
            excl.append(i)
            continue
        l2.append(float(np.linalg.norm(a - b) / norms[i]))
        mx.append(float(np.abs(a - b).max() / np.abs(b).max()))
    return {"action_grad_rel_err_l2_median": float(np.median(l2)) if l2 else None,
            "action_grad_rel_err_l2_max": max(l2) if l2 else None,
            "action_grad_rel_err_maxnorm_median": float(np.median(mx)) if mx else None,
            "action_grad_rel_err_maxnorm_max": max(mx) if mx else None,
            "scenes_within_1e-3_l2": int(sum(e <= 1e-3 for e in l2)), "scenes_compared": len(l2),
            "excluded_zero_gradient": excl, "reference": "FP64 GPU path on the same scenes and actions"}


def cpu_baseline(sc, target_s: float = 12.0, threads: int = 0):
    from oracle import oracle as O
    threads = threads or os.cpu_count() or 1
    O.set_num_threads(threads)
    dt, ps = O.time_fwd_bwd(sc, 1, threads)
    n_act = max(1, min(sc.n_actions, int(target_s / max(dt, 1e-3))))
    if n_act > 1:
        dt, ps = O.time_fwd_bwd(sc, n_act, threads)
    return {"value": ps / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"FP64 oracle fwd+bwd (store-all), scene 0 of the workload ({sc.n_particles} particles, "
                      f"{len(sc.tools)} tools), {n_act} action(s) x {sc.sim.n_substeps} substeps, {dt:.1f} s"}


# ----------------------------------------------------------------------------
# reference arm: the reference's CPU path, restated (taichi is not installable)
# ----------------------------------------------------------------------------
def run_reference(args, rank, world):
    if rank != 0:
        return None
    from oracle import oracle as O
    scs, desc = make_workload(args.workload, 0)
    sc = scs[0]
    threads = os.cpu_count() or 1
    O.set_num_threads(threads)
    dt1, _ = O.time_fwd_bwd(sc, 1, threads)
    n_act = max(1, min(sc.n_actions, int(15.0 / max(dt1, 1e-3))))
    times, ps = [], 0
    for i in range(args.warmup + args.steps):
        dt, ps = O.time_fwd_bwd(sc, n_act, threads)
        if i >= args.warmup:
            times.append(dt)
    ms = 1e3 * float(np.mean(times))
    val = ps / (ms * 1e-3)
    sample = (f"FP64 CPU restatement of the reference substep (oracle), scene 0 of the workload "
              f"({sc.n_particles} particles), {n_act} action(s) x {sc.sim.n_substeps} substeps fwd+bwd per step")
    return {"metric": METRIC, "value": val, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "config": desc, "impl": "reference",
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
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
    else:
        out = run_ours(args, rank, world, dist)
        if out is not None and "plain_fp64" in out:
            out["plain_fp64"]["batched_fp32_over_plain_fp64"] = out["value"] / world / out["plain_fp64"]["value"]
    if out is not None:
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
