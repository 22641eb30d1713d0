"""GPU parity of the loss kernels of plb/engine/losses/loss.py against the
oracle: target-SDF propagation (bit-exact), SDF loss, IoU, hard contact
distance and its adjoint, and the ``Loss`` class mirror end to end."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from _util import all_tools, perturbed_state, rel_err, small_scene
from diffskill_gb300.config import ActionConfig, PrimitiveConfig, SimulatorConfig
from diffskill_gb300.engine import MpmEngine
from oracle import oracle as O
from oracle.oracle import Oracle, init_state

pytestmark = pytest.mark.gpu


def to_soa(eng, aos):
    st = eng.new_state()
    st[:, :aos.shape[0]] = torch.as_tensor(aos.T, dtype=eng.dtype, device=eng.device)
    return st


def blob_density(n: int, seed: int, empty: bool = False) -> np.ndarray:
    """A few dense boxes plus isolated nodes below the 1e-4 density threshold."""
    rng = np.random.default_rng(seed)
    d = np.zeros((n, n, n))
    if not empty:
        for _ in range(3):
            c = rng.integers(5, n - 5, size=3)
            r = rng.integers(1, 5, size=3)
            d[c[0] - r[0]:c[0] + r[0], c[1] - r[1]:c[1] + r[1], c[2] - r[2]:c[2] + r[2]] = rng.uniform(1e-3, 1e-2)
    d[rng.random((n, n, n)) < 0.002] = 5e-5
    return d


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("n_iters", [1, 3, None])
def test_target_sdf_bit_exact(gpu_lib, prec, n_iters):
    """40^3 grid (partial 8^3 tiles, dx not a power of two), three scenes, one
    of them without any dense node; None = the reference's 2 * n_grid sweeps,
    which also exercises the converged-early exit."""
    n = 40
    sim = SimulatorConfig(n_grid=n, dt=1e-4, substeps=10, precision=prec)
    dens = [blob_density(n, 1), blob_density(n, 2), blob_density(n, 3, empty=True)]
    eng = MpmEngine(sim, [[], [], []], [1, 1, 1])
    it = 2 * n if n_iters is None else n_iters
    sdf, near = eng.target_sdf(torch.as_tensor(np.stack([d.ravel() for d in dens])), it)
    torch.cuda.synchronize()
    for s, d in enumerate(dens):
        ref_s, ref_n = O.target_sdf(d, sim.dx, it, single=(prec == "fp32"))
        got_s = sdf[s].cpu().numpy().reshape(n, n, n)
        got_n = near[s].cpu().numpy().reshape(n, n, n, 3)
        assert np.array_equal(got_s, ref_s), (s, np.abs(got_s - ref_s).max())
        assert np.array_equal(got_n, ref_n), s
    if n_iters is None:
        assert (sdf[0] < 1000).all() and (sdf[2] == 1000).all()


def test_target_sdf_zero_iterations_leaves_zeros(gpu_lib):
    sim = SimulatorConfig(n_grid=16, dt=1e-4, substeps=10, precision="fp32")
    eng = MpmEngine(sim, [[]], [1])
    sdf, near = eng.target_sdf(torch.ones((1, 16 ** 3)), 0)
    assert float(sdf.abs().sum()) == 0.0 and float(near.abs().sum()) == 0.0


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_sdf_loss_and_iou_match_oracle(gpu_lib, prec):
    sc = small_scene(n=5000, precision=prec)
    eng = MpmEngine(sc.sim, [sc.tools], [sc.n_particles])
    o = Oracle(sc.sim, sc.tools)
    st = perturbed_state(sc.x0, seed=4)
    gm_ref = o.grid_mass(st)
    s = to_soa(eng, st)
    gm = eng.grid_mass(s)
    tgt = eng.targets([sc.target])
    tsdf, _ = eng.target_sdf(tgt)
    n = sc.sim.grid
    ref_sdf, _ = O.target_sdf(sc.target.reshape(n, n, n), sc.sim.dx, 2 * n, single=(prec == "fp32"))
    assert np.array_equal(tsdf[0].cpu().numpy(), ref_sdf.ravel())
    g = torch.full_like(gm, 0.5)
    loss = eng.sdf_loss(gm, tsdf, 2.5, g)
    iou = eng.iou(gm, tgt)
    torch.cuda.synchronize()
    ref_loss, _ = O.sdf_loss(gm_ref, ref_sdf.ravel())
    tol = 1e-12 if prec == "fp64" else 1e-5
    assert abs(float(loss[0]) - 2.5 * ref_loss) <= tol * abs(2.5 * ref_loss)
    # the gradient is added: 0.5 + 2.5 * sdf (the device may fuse it into one FMA)
    want = 0.5 + 2.5 * tsdf[0].double()
    assert rel_err(g[0].double().cpu().numpy(), want.cpu().numpy()) < (1e-15 if prec == "fp64" else 1e-7)
    ref_iou = O.iou(gm_ref, sc.target)
    assert abs(float(iou[0]) - ref_iou) <= tol * abs(ref_iou)
    # iou of the target with itself, as load_target_density records it
    t_dev = tgt[0].double().cpu().numpy()  # the target as the device holds it (FP32-rounded in fp32)
    assert abs(float(eng.iou(tgt, tgt)[0]) - O.iou(t_dev, t_dev)) < 1e-12


def test_contact_min_dist_matches_oracle(gpu_lib):
    tools = all_tools()
    sc = small_scene(n=3000, tools=tools, precision="fp64")
    eng = MpmEngine(sc.sim, [tools], [sc.n_particles])
    o = Oracle(sc.sim, tools)
    st = perturbed_state(sc.x0, seed=2)
    pose = o.pose0()
    s = to_soa(eng, st)
    pz = torch.as_tensor(pose, device=eng.device).contiguous()
    md, am = eng.contact_min_dist(s, pz)
    g_md = torch.arange(1, o.T + 1, dtype=torch.float64, device=eng.device)
    gs = eng.new_state()
    gp = torch.zeros((o.T, 8), dtype=torch.float64, device=eng.device)
    eng.contact_min_dist_bwd(s, pz, am, g_md, gs, gp)
    torch.cuda.synchronize()
    g_ref, gp_ref = np.zeros_like(st), np.zeros((o.T, 8))
    for t in range(o.T):
        gpt = np.zeros(8)
        ref_md, ref_am = o.contact_min(t, pose[t], st, float(t + 1), g_ref, gpt)
        gp_ref[t] = gpt
        assert int(am[t]) == ref_am, t
        assert abs(float(md[t]) - ref_md) <= 1e-12 * max(ref_md, 1e-12), t
    got = gs[0:3, :sc.n_particles].cpu().numpy().T
    assert rel_err(got, g_ref[:, 0:3]) < 1e-9
    assert rel_err(gp.cpu().numpy(), gp_ref) < 1e-9
    assert float(gs[3:].abs().sum()) == 0.0


def test_contact_min_dist_static_tool_and_far_particles(gpu_lib):
    """A tool with action_dim 0 reports 0 / -1; a tool far from every particle
    reports the smallest positive distance."""
    sc = small_scene(n=500, precision="fp64")
    far = PrimitiveConfig(shape="Sphere", init_pos=(0.5, 0.8, 0.5), radius=0.03,
                          action=ActionConfig(dim=3, scale=(0.01, 0.01, 0.01)))
    static = PrimitiveConfig(shape="Sphere", init_pos=(0.5, 0.15, 0.5), radius=0.03, action=ActionConfig(dim=0))
    tools = [far, static]
    eng = MpmEngine(sc.sim, [tools], [sc.n_particles])
    o = Oracle(sc.sim, tools)
    st = init_state(sc.x0)
    md, am = eng.contact_min_dist(to_soa(eng, st), torch.as_tensor(o.pose0(), device=eng.device).contiguous())
    torch.cuda.synchronize()
    ref_md, ref_am = o.contact_min(0, o.pose0()[0], st)
    assert int(am[0]) == ref_am and abs(float(md[0]) - ref_md) < 1e-12 * ref_md
    assert float(md[1]) == 0.0 and int(am[1]) == -1


@pytest.mark.parametrize("soft", [False, True])
def test_loss_class_matches_oracle(gpu_lib, soft):
    """``Loss.compute_loss_kernel`` and ``.grad`` on the MPMSimulator mirror
    against the oracle's terms: density L1, SDF loss and contact."""
    from diffskill_gb300.function import SimEnv
    from diffskill_gb300.loss import Loss, LossConfig

    tool = all_tools()[1]
    sc = small_scene(n=3000, tools=[tool], precision="fp64")
    env = SimEnv(sc.sim, sc.tools, sc.x0)
    sim = env.simulator
    n = sc.sim.grid
    L = Loss(LossConfig(soft_contact=soft), sim)
    L.load_target_density(grids=sc.target.reshape(n, n, n))
    L.compute_loss_kernel(0)
    o = Oracle(sc.sim, sc.tools)
    st = init_state(sc.x0)
    pose = o.pose0()
    gm = o.grid_mass(st)
    tsdf, _ = O.target_sdf(sc.target.reshape(n, n, n), sc.sim.dx, 2 * n)
    dens = float(np.abs(gm - sc.target).sum())
    sdfl = float(np.sum(tsdf.ravel() * gm))
    md = o.soft_contact(0, pose[0], st) if soft else o.contact_min(0, pose[0], st)[0]
    ref = md ** 2 + 10 * dens + 10 * sdfl
    assert abs(L.loss - ref) <= 1e-10 * abs(ref)
    assert abs(L.density_loss - dens) <= 1e-10 * dens and abs(L.sdf_loss - sdfl) <= 1e-10 * abs(sdfl)

    sim.zero_grad()
    L.compute_loss_kernel.grad(0)
    torch.cuda.synchronize()
    g_ref = np.zeros_like(st)
    o.grid_mass_bwd(st, 10 * np.sign(gm - sc.target) + 10 * tsdf.ravel(), g_ref)
    gp_ref = np.zeros(8)
    if soft:
        o.soft_contact(0, pose[0], st, 2 * md, g_ref, gp_ref)
    else:
        o.contact_min(0, pose[0], st, 2 * md, g_ref, gp_ref)
    got = sim._gframes[0][0:3, :sc.n_particles].cpu().numpy().T
    assert rel_err(got, g_ref[:, 0:3]) < 1e-9
    assert rel_err(sim._g_pose[0, 0].cpu().numpy(), gp_ref) < 1e-9

    # reward bookkeeping of reset / compute_loss (loss.py:335-351): reset leaves
    # loss = L(0) accumulated, so the next compute_loss(0) reports 2 L(0) as the
    # step loss and -L(0) as the reward
    L.reset()
    info = L.compute_loss(0)
    assert abs(L._start_loss - ref) <= 1e-10 * abs(ref)
    assert abs(info["loss"] - 2 * ref) <= 1e-10 * abs(ref) and abs(info["reward"] + ref) <= 1e-10 * abs(ref)
    # the same frame twice: the IoU moves only by the atomic summation order of the grid mass
    assert abs(info["incremental_iou"]) < 1e-12
