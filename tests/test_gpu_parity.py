"""GPU (sm_103a) parity against the FP64 CPU oracle, through the C ABI.

Tolerances (stated per test): the FP64 GPU path must match the oracle to
near round-off (1e-9 relative per row group); FP32 paths to what single
precision allows: one substep 1e-4 (forward) and 2e-4 (adjoint) relative to
the row-group magnitude, trajectory action gradients 1e-3 (the bound the
benchmark's accuracy claim states), positions after one action 1e-4.
"""
import numpy as np
import pytest
import torch

from _util import all_tools, collision_tools, group_errors, more_tools, perturbed_state, rel_err, small_scene
from diffskill_gb300.config import PrimitiveConfig
from diffskill_gb300.engine import Horizon, MpmEngine
from oracle.oracle import Oracle, init_state

pytestmark = pytest.mark.gpu

FWD_TOL = {"fp64": 1e-9, "fp32_svd64": 1e-4, "fp32": 1e-4}


def to_soa(eng, aos):
    st = eng.new_state()
    st[:, :aos.shape[0]] = torch.as_tensor(aos.T, dtype=eng.dtype, device=eng.device)
    return st


def to_aos(eng, st, n=None):
    n = eng.P if n is None else n
    return st[:, :n].double().cpu().numpy().T.copy()


def make_engine(sc, tools=None):
    tools = sc.tools if tools is None else tools
    return MpmEngine(sc.sim, [tools], [sc.n_particles])


@pytest.mark.parametrize("prec", ["fp64", "fp32_svd64", "fp32"])
def test_substep_forward_matches_oracle(gpu_lib, prec):
    tools = all_tools()
    sc = small_scene(n=3000, tools=tools, precision=prec)
    eng = make_engine(sc)
    o = Oracle(sc.sim, tools)
    st0 = perturbed_state(sc.x0, seed=3)
    act = o.expand_action(sc.actions[0])
    _, _, pseq = o.tools_action(o.pose0(), sc.actions[0])
    ref = o.substep(pseq[0], pseq[1], st0)
    pose = torch.as_tensor(pseq[:2], device=eng.device).contiguous()
    s0, s1 = to_soa(eng, st0), eng.new_state()
    eng.substep(s0, s1, pose[0], pose[1])
    torch.cuda.synchronize()
    assert eng.status() == 0
    errs = group_errors(to_aos(eng, s1), ref)
    assert max(errs.values()) < FWD_TOL[prec], errs
    del act


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-8), ("fp32_svd64", 2e-4), ("fp32", 2e-4)])
def test_substep_adjoint_matches_oracle(gpu_lib, prec, tol):
    tools = all_tools()
    sc = small_scene(n=3000, tools=tools, precision=prec)
    eng = make_engine(sc)
    o = Oracle(sc.sim, tools)
    st0 = perturbed_state(sc.x0, seed=4)
    _, _, pseq = o.tools_action(o.pose0(), sc.actions[0])
    g1 = np.random.default_rng(5).normal(size=st0.shape)
    gp_f, gp_f1 = np.zeros((o.T, 8)), np.zeros((o.T, 8))
    ref = o.substep_bwd(pseq[0], pseq[1], st0, g1, gp_f, gp_f1)
    pose = torch.as_tensor(pseq[:2], device=eng.device).contiguous()
    gpose = torch.zeros((2, o.T, 8), dtype=torch.float64, device=eng.device)
    s0, gg1, gg0 = to_soa(eng, st0), to_soa(eng, g1), eng.new_state()
    eng.substep_bwd(s0, gg1, gg0, pose[0], pose[1], gpose[0], gpose[1])
    torch.cuda.synchronize()
    errs = group_errors(to_aos(eng, gg0), ref)
    assert max(errs.values()) < tol, errs
    gp = gpose.cpu().numpy()
    assert rel_err(gp[0], gp_f) < tol * 10, (gp[0], gp_f)
    assert rel_err(gp[1], gp_f1) < tol * 10, (gp[1], gp_f1)
    # with frame f+1 from the forward, g2p.grad reads v' instead of re-gathering it
    s1 = eng.new_state()
    eng.substep(s0, s1, pose[0], pose[1])
    gg0b = eng.new_state()
    gpose2 = torch.zeros_like(gpose)
    eng.substep_bwd(s0, gg1, gg0b, pose[0], pose[1], gpose2[0], gpose2[1], st1=s1)
    torch.cuda.synchronize()
    errs_b = group_errors(to_aos(eng, gg0b), to_aos(eng, gg0))
    # the two calls rebuild the grid with different FP32 atomic orders (~1e-7 in v),
    # which the stress adjoint amplifies in the C and F rows
    assert max(errs_b.values()) < (1e-12 if prec == "fp64" else 1e-4), errs_b


def test_tools_action_matches_oracle(gpu_lib):
    tools = all_tools()
    sc = small_scene(n=100, tools=tools, precision="fp64", substeps=20)
    eng = make_engine(sc)
    o = Oracle(sc.sim, tools)
    acts, vel, pseq = o.tools_action(o.pose0(), sc.actions[0])
    n = sc.sim.n_substeps
    a = torch.zeros((o.T, 8), dtype=torch.float64, device=eng.device)
    a[:, :7] = torch.as_tensor(acts, device=eng.device)
    v = torch.zeros((n, o.T, 8), dtype=torch.float64, device=eng.device)
    p = torch.zeros((n + 1, o.T, 8), dtype=torch.float64, device=eng.device)
    p[0] = eng.pose0
    eng.tools_action(a, v, p)
    torch.cuda.synchronize()
    assert rel_err(p.cpu().numpy(), pseq) < 1e-13
    assert rel_err(v.cpu().numpy(), vel) < 1e-13
    # adjoint
    from oracle.oracle import lib, ptr
    gps = np.random.default_rng(1).normal(size=pseq.shape)
    g_ref, ga_ref = gps.copy(), np.zeros((o.T, 7))
    o.tools_action_bwd(acts, vel, pseq, o.last_coll, g_ref, ga_ref)
    g = torch.as_tensor(gps, device=eng.device).contiguous()
    ga = torch.zeros((o.T, 8), dtype=torch.float64, device=eng.device)
    eng.tools_action_bwd(v, p, g, ga)
    torch.cuda.synchronize()
    assert rel_err(g.cpu().numpy(), g_ref) < 1e-12
    assert rel_err(ga.cpu().numpy()[:, :7], ga_ref) < 1e-12


def _traj(eng, sc, k):
    hz = Horizon(eng, sc.n_actions, ckpt_every=k)
    st0 = eng.init_state([sc.x0])
    acts = eng.expand_actions([sc.actions])
    hz.forward(st0, acts)
    tgt = eng.targets([sc.target])
    loss = hz.loss(tgt, sc.density_weight, sc.contact_weight)
    g = hz.backward()
    torch.cuda.synchronize()
    return float(loss.sum()), eng.collapse_action_grad(g)[0].cpu().numpy(), hz


@pytest.mark.parametrize("prec,loss_tol,grad_tol", [("fp64", 1e-9, 1e-6), ("fp32_svd64", 1e-5, 1e-3),
                                                    ("fp32", 1e-5, 1e-3)])
def test_trajectory_loss_and_action_grad(gpu_lib, prec, loss_tol, grad_tol):
    """Config-1 shape (capsule, density L1 to the +0.1-shifted dough), 2 actions x 50 substeps."""
    sc = small_scene(n=4000, n_actions=2, substeps=50, precision=prec)
    o = Oracle(sc.sim, sc.tools)
    ref_loss, ref_grad = o.loss_and_grad(sc.x0, sc.actions, sc.target)
    eng = make_engine(sc)
    loss, grad, _ = _traj(eng, sc, k=10)
    assert eng.status() == 0
    assert abs(loss - ref_loss) / abs(ref_loss) < loss_tol, (loss, ref_loss)
    assert rel_err(grad, ref_grad) < grad_tol, (grad, ref_grad)


@pytest.mark.parametrize("prec", ["fp32", "fp32_svd64"])
def test_positions_after_one_action_match_oracle(gpu_lib, prec):
    """The FP32 state after one action (50 substeps) of config 1 (10k particles
    in a 0.2 x 0.1 x 0.2 box, capsule): every particle position within 1e-4
    relative (to the largest coordinate) of the FP64 oracle's."""
    from diffskill_gb300 import scenes
    sc = scenes.config1(n_actions=1, dt=1e-4)
    sc.sim.precision = prec
    ro = Oracle(sc.sim, sc.tools).rollout(sc.x0, sc.actions, keep_frames=False)
    eng = make_engine(sc)
    hz = Horizon(eng, 1, ckpt_every=50)
    hz.forward(eng.init_state([sc.x0]), eng.expand_actions([sc.actions]))
    torch.cuda.synchronize()
    assert eng.status() == 0
    x = hz.final[0:3, :eng.P].double().cpu().numpy().T
    xr = ro["final"][:, 0:3]
    assert np.abs(xr - sc.x0).max() > 1e-3  # the dough moved
    assert rel_err(x, xr) < 1e-4, rel_err(x, xr)


def test_checkpoint_recompute_equals_store_all(gpu_lib):
    """Analogue of long_term_gradient.ipynb cell 4: checkpointed grad == full-tape grad."""
    sc = small_scene(n=4000, n_actions=2, substeps=50, precision="fp64")
    eng = make_engine(sc)
    l1, g1, _ = _traj(eng, sc, k=1)
    l2, g2, _ = _traj(eng, sc, k=10)
    l3, g3, _ = _traj(eng, sc, k=50)
    assert abs(l1 - l2) <= 1e-12 * abs(l1) and abs(l1 - l3) <= 1e-12 * abs(l1)
    assert np.abs(g1 - g2).max() < 1e-4 and np.abs(g1 - g3).max() < 1e-4
    assert rel_err(g2, g1) < 1e-9 and rel_err(g3, g1) < 1e-9


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 1e-4)])
def test_pipelined_adjoint_equals_serial(gpu_lib, monkeypatch, prec, tol):
    """Every frame kept (k=1): the adjoint substeps run pipelined (each one's
    grid preparation beside the previous one's p2g.grad); loss, action and
    initial-state gradients equal the serial adjoint's.  FP64 to 1e-12; FP32
    to 1e-4, the run-to-run spread of its scatter's atomic summation order
    over 40 substeps (measured 2e-5 on the initial-state gradient)."""
    sc = small_scene(n=4000, n_actions=2, substeps=20, tools=[all_tools()[0], all_tools()[2]], precision=prec)
    eng = make_engine(sc)
    runs = []
    for pipelined in (True, False):
        if not pipelined:
            real = eng.set_pipelined_adjoint
            monkeypatch.setattr(eng, "set_pipelined_adjoint", lambda on: real(False))
        l, g, hz = _traj(eng, sc, k=1)
        runs.append((l, g, hz.g_state0[:, :sc.n_particles].clone()))
    (l0, g0, s0), (l1, g1, s1) = runs
    assert abs(l1 - l0) <= tol * abs(l0)
    assert rel_err(g1, g0) < tol
    assert rel_err(s1.cpu().numpy(), s0.cpu().numpy()) < tol


def test_auto_checkpoint_interval_fits_the_budget_and_keeps_gradients(gpu_lib):
    """ckpt_every="auto" under a frame budget of 16 frames: 40 substeps need 43
    frames at k=1, so the planner takes k=4 (11 checkpoints + a 4-frame
    segment); loss and action gradients equal the store-all run."""
    sc = small_scene(n=3000, n_actions=2, substeps=20, precision="fp64")
    eng = make_engine(sc)
    l1, g1, _ = _traj(eng, sc, k=1)
    frame_bytes = 24 * eng.ld * 8
    hz = Horizon(eng, sc.n_actions, ckpt_every="auto", frame_budget_bytes=16 * frame_bytes)
    assert hz.k == 4 and hz.n_ckpt == 11
    hz.forward(eng.init_state([sc.x0]), eng.expand_actions([sc.actions]))
    l2 = float(hz.loss(eng.targets([sc.target]), sc.density_weight, sc.contact_weight).sum())
    g2 = eng.collapse_action_grad(hz.backward())[0].cpu().numpy()
    assert abs(l2 - l1) <= 1e-12 * abs(l1)
    assert rel_err(g2, g1) < 1e-9


def test_batched_scenes_equal_single_scenes(gpu_lib):
    """Three scenes with different particle counts and tool sets in one launch
    give the same loss and action gradients as three separate runs."""
    base = small_scene(n=1500, n_actions=1, substeps=20, precision="fp64")
    scs = [small_scene(n=1000 + 500 * i, n_actions=1, substeps=20, precision="fp64", seed=2000 + i)
           for i in range(3)]
    at = all_tools()
    tools = [[at[1]], [at[2]], [at[0], at[4]]]  # every tool touches the dough
    for sc, tl in zip(scs, tools):
        sc.tools = tl
        sc.actions = np.random.default_rng(len(tl)).uniform(-1, 1, size=(1, sum(t.action.dim for t in tl)))
    eng = MpmEngine(base.sim, tools, [sc.n_particles for sc in scs])
    hz = Horizon(eng, 1, ckpt_every=10)
    hz.forward(eng.init_state([sc.x0 for sc in scs]), eng.expand_actions([sc.actions for sc in scs]))
    loss = hz.loss(eng.targets([sc.target for sc in scs]))
    g = eng.collapse_action_grad(hz.backward())
    torch.cuda.synchronize()
    for i, sc in enumerate(scs):
        e1 = MpmEngine(sc.sim, [tools[i]], [sc.n_particles])
        l1, g1, _ = _traj(e1, sc, k=10)
        assert abs(float(loss[i]) - l1) <= 1e-12 * abs(l1)
        gi = g[i].cpu().numpy()
        assert np.abs(g1).max() > 1e-6  # the tools act on the dough
        assert np.abs(gi - g1).max() <= 1e-9 * np.abs(g1).max(), (gi, g1)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_grid_mass_and_density_l1(gpu_lib, prec):
    sc = small_scene(n=5000, precision=prec)
    eng = make_engine(sc)
    o = Oracle(sc.sim, sc.tools)
    st = perturbed_state(sc.x0, seed=9)
    gm_ref = o.grid_mass(st)
    s = to_soa(eng, st)
    gm = eng.grid_mass(s)
    tgt = eng.targets([sc.target])
    g_gm = torch.empty_like(gm)
    loss = eng.density_l1(gm, tgt, 1.0, g_gm)
    torch.cuda.synchronize()
    tol = 1e-12 if prec == "fp64" else 1e-5
    assert rel_err(gm.cpu().numpy()[0], gm_ref) < tol
    assert abs(gm.double().sum().item() - sc.n_particles * sc.sim.p_mass) < 1e-6 * sc.n_particles * sc.sim.p_mass
    ref_loss = float(np.abs(gm_ref - sc.target).sum())
    assert abs(float(loss[0]) - ref_loss) < (1e-10 if prec == "fp64" else 1e-4) * ref_loss
    g_ref = np.zeros_like(st)
    o.grid_mass_bwd(st, np.sign(gm_ref - sc.target), g_ref)
    gs = eng.new_state()
    eng.grid_mass_bwd(s, g_gm, gs)
    torch.cuda.synchronize()
    got = to_aos(eng, gs)[:, 0:3]
    if prec == "fp64":
        assert rel_err(got, g_ref[:, 0:3]) < 1e-9
    else:  # sign flips where |m - target| ~ FP32 rounding change a few nodes
        assert np.mean(np.abs(got - g_ref[:, 0:3]) < 1e-3 * np.abs(g_ref[:, 0:3]).max()) > 0.99


def test_soft_contact_matches_oracle(gpu_lib):
    tools = all_tools()
    sc = small_scene(n=3000, tools=tools, precision="fp64")
    eng = make_engine(sc)
    o = Oracle(sc.sim, tools)
    st = perturbed_state(sc.x0, seed=2)
    pose = o.pose0()
    s = to_soa(eng, st)
    pz = torch.as_tensor(pose, device=eng.device).contiguous()
    md, sums = eng.soft_contact(s, pz)
    g_md = torch.arange(1, o.T + 1, dtype=torch.float64, device=eng.device)
    gs = eng.new_state()
    gp = torch.zeros((o.T, 8), dtype=torch.float64, device=eng.device)
    eng.soft_contact_bwd(s, pz, sums, g_md, gs, gp)
    torch.cuda.synchronize()
    g_ref, gp_ref = np.zeros_like(st), np.zeros((o.T, 8))
    for t in range(o.T):
        ref = o.soft_contact(t, pose[t], st)
        assert abs(float(md[t]) - ref) < 1e-10 * max(abs(ref), 1e-12)
        gpt = np.zeros(8)
        o.soft_contact(t, pose[t], st, float(t + 1), g_ref, gpt)
        gp_ref[t] = gpt
    assert rel_err(to_aos(eng, gs)[:, 0:3], g_ref[:, 0:3]) < 1e-9
    assert rel_err(gp.cpu().numpy(), gp_ref) < 1e-9


def test_out_of_grid_particle_sets_status_and_is_skipped(gpu_lib):
    """A particle outside [0, 1-3dx] is bounds-checked on the device: its
    scatter is skipped, the sticky status bit is set, nothing faults."""
    sc = small_scene(n=500, precision="fp32")
    eng = make_engine(sc)
    x = sc.x0.copy()
    x[7] = [1.5, 0.5, 0.5]
    s0 = eng.init_state([x])
    s1 = eng.new_state()
    pose = eng.pose0.unsqueeze(0).repeat(2, 1, 1).contiguous()
    eng.substep(s0, s1, pose[0], pose[1])
    st = eng.status(clear=True)
    assert st & 1
    assert eng.status(clear=True) == 0
    got = s1[:3, 7].cpu().numpy()
    assert np.allclose(got, [1.5, 0.5, 0.5])


@pytest.mark.gpu
def test_nonfinite_state_sets_status_and_raises(gpu_lib):
    """A NaN in one particle's deformation gradient is reported through the
    sticky status word (the kernels bound every loop and index, so nothing
    faults), and check_status raises like the reference's NaN check."""
    sc = small_scene(n=500, precision="fp32")
    eng = make_engine(sc)
    s0 = eng.init_state([sc.x0])
    s0[15, 11] = float("nan")
    s1 = eng.new_state()
    pose = eng.pose0.unsqueeze(0).repeat(2, 1, 1).contiguous()
    eng.substep(s0, s1, pose[0], pose[1])
    torch.cuda.synchronize()
    assert eng.status(clear=False) & 2
    with pytest.raises(FloatingPointError):
        eng.check_status()
    assert eng.status(clear=True) == 0


def test_invalid_arguments_raise(gpu_lib):
    from diffskill_gb300 import _lib
    sc = small_scene(n=100, precision="fp32")
    eng = make_engine(sc)
    s0 = eng.new_state()
    with pytest.raises(_lib.MpmError, match="must differ"):
        eng.substep(s0, s0, eng.pose0, eng.pose0)
    bad = PrimitiveConfig(shape="Box")
    bad_sim = sc.sim
    bad_sim.n_grid = 60
    with pytest.raises(_lib.MpmError, match="multiple of 8"):
        MpmEngine(bad_sim, [[bad]], [10])


@pytest.mark.parametrize("prec,loss_tol,grad_tol", [("fp64", 1e-9, 1e-6), ("fp32", 1e-5, 1e-3)])
def test_sorted_particles_warp_aggregated_scatter_matches_oracle(gpu_lib, prec, loss_tol, grad_tol):
    """BatchedTrajectory sorts particles by cell, so the p2g and g2p.grad scatters
    take the warp-segmented reduction path; results must still match the oracle."""
    from diffskill_gb300.trajectory import BatchedTrajectory, spatial_order
    sc = small_scene(n=6000, n_actions=2, substeps=25, precision=prec)
    order = spatial_order(sc.x0, sc.sim.grid)
    assert not np.array_equal(order, np.arange(sc.n_particles))
    bt = BatchedTrajectory([sc], ckpt_every=5)
    bt.forward_backward()
    torch.cuda.synchronize()
    assert bt.eng.status() == 0
    loss = float(bt.loss[0])
    grad = bt.action_grads()[0].cpu().numpy()
    ref_loss, ref_grad = Oracle(sc.sim, sc.tools).loss_and_grad(sc.x0, sc.actions, sc.target)
    assert abs(loss - ref_loss) / abs(ref_loss) < loss_tol, (loss, ref_loss)
    assert rel_err(grad, ref_grad) < grad_tol, (grad, ref_grad)


@pytest.mark.parametrize("k", [1, 10])
def test_grid_store_restore_equals_recompute(gpu_lib, k):
    """Restoring the stored forward grids (p2g grid and grid_op output) in the
    adjoint gives the recompute path's loss and gradients, also when the store
    fills up part way."""
    sc = small_scene(n=4000, n_actions=2, substeps=50, tools=[all_tools()[1], all_tools()[2]], precision="fp64")
    eng = make_engine(sc)
    out = []
    for store, budget in ((False, None), (True, None), (True, 2 * 64 * 1037 * 3)):  # ~97 FP64 blocks
        hz = Horizon(eng, sc.n_actions, ckpt_every=k, store_grids=store, store_budget_bytes=budget)
        hz.forward(eng.init_state([sc.x0]), eng.expand_actions([sc.actions]))
        loss = float(hz.loss(eng.targets([sc.target])).sum())
        g = eng.collapse_action_grad(hz.backward())[0].cpu().numpy()
        torch.cuda.synchronize()
        if store:
            n_stored = hz.store.stored_slots()
            assert n_stored > 0
            if budget is not None:
                assert n_stored < hz.store.slot_start.numel()  # partly stored, partly recomputed
        out.append((loss, g))
    (l0, g0) = out[0]
    for l, g in out[1:]:
        assert abs(l - l0) <= 1e-12 * abs(l0)
        assert rel_err(g, g0) < 1e-9


@pytest.mark.parametrize("k", [1, 10])
def test_resorting_particles_keeps_loss_and_gradients(gpu_lib, k):
    """Re-sorting particles by cell at every action boundary (and unsorting the
    frame gradient in the adjoint) leaves the loss and action gradients as they are."""
    sc = small_scene(n=5000, n_actions=3, substeps=20, tools=[all_tools()[0], all_tools()[2]], precision="fp64")
    eng = make_engine(sc)
    res = []
    for R in (0, 20):
        hz = Horizon(eng, sc.n_actions, ckpt_every=k, resort_every=R)
        assert hz.R == R
        hz.forward(eng.init_state([sc.x0]), eng.expand_actions([sc.actions]))
        loss = float(hz.loss(eng.targets([sc.target])).sum())
        g = eng.collapse_action_grad(hz.backward())[0].cpu().numpy()
        torch.cuda.synchronize()
        res.append((loss, g, hz.g_state0[:, :sc.n_particles].clone()))
        if R:
            assert not torch.equal(hz.perms[0][:sc.n_particles].cpu(), torch.arange(sc.n_particles))
    (l0, g0, s0), (l1, g1, s1) = res
    assert abs(l1 - l0) <= 1e-12 * abs(l0)
    assert rel_err(g1, g0) < 1e-9
    # the gradient w.r.t. the initial state comes back in the original particle order
    assert rel_err(s1.cpu().numpy(), s0.cpu().numpy()) < 1e-9



# ----------------------------------------------------------------------------
# RollingPin(Ext), Chopsticks, Cylinder, Torus, Gripper2 and the tool-tool
# collision projection
# ----------------------------------------------------------------------------
@pytest.mark.parametrize("prec,fwd_tol,bwd_tol", [("fp64", 1e-9, 1e-8), ("fp32", 1e-4, 1e-3)])
def test_more_tools_substep_matches_oracle(gpu_lib, prec, fwd_tol, bwd_tol):
    tools = more_tools()
    sc = small_scene(n=3000, tools=tools, precision=prec)
    eng = make_engine(sc)
    o = Oracle(sc.sim, tools)
    st0 = perturbed_state(sc.x0, seed=13)
    _, _, pseq = o.tools_action(o.pose0(), sc.actions[0])
    pose = torch.as_tensor(pseq[:2], device=eng.device).contiguous()
    ref = o.substep(pseq[0], pseq[1], st0)
    s0, s1 = to_soa(eng, st0), eng.new_state()
    eng.substep(s0, s1, pose[0], pose[1])
    torch.cuda.synchronize()
    assert eng.status() == 0
    errs = group_errors(to_aos(eng, s1), ref)
    assert max(errs.values()) < fwd_tol, errs
    g1 = np.random.default_rng(14).normal(size=st0.shape)
    gp_f, gp_f1 = np.zeros((o.T, 8)), np.zeros((o.T, 8))
    gref = o.substep_bwd(pseq[0], pseq[1], st0, g1, gp_f, gp_f1)
    gpose = torch.zeros((2, o.T, 8), dtype=torch.float64, device=eng.device)
    gg0 = eng.new_state()
    eng.substep_bwd(s0, to_soa(eng, g1), gg0, pose[0], pose[1], gpose[0], gpose[1])
    torch.cuda.synchronize()
    errs = group_errors(to_aos(eng, gg0), gref)
    assert max(errs.values()) < bwd_tol, errs
    gp = gpose.cpu().numpy()
    assert np.abs(gp_f).max() > 0 and np.abs(gp_f1).max() > 0  # every tool touches the dough
    assert rel_err(gp[0], gp_f) < bwd_tol * 10 and rel_err(gp[1], gp_f1) < bwd_tol * 10


@pytest.mark.parametrize("which", ["more", "collision"])
def test_kinematics_and_collision_projection_match_oracle(gpu_lib, which):
    """mpm_tools_action(_bwd) for the remaining tools' kinematics and for tools
    projected out of an obstacle box (oracle: the reference's sequential
    set_collision_idx loop and its autodiff semantics)."""
    tools = more_tools() if which == "more" else collision_tools()
    sc = small_scene(n=100, tools=tools, precision="fp64", substeps=20, n_actions=2)
    eng = make_engine(sc)
    o = Oracle(sc.sim, tools)
    assert eng.n_pairs == o.n_pairs == (2 if which == "collision" else 0)
    n = sc.sim.n_substeps
    pose_o = o.pose0()
    p0 = eng.pose0.clone()
    for s in range(sc.n_actions):
        acts, vel, pseq = o.tools_action(pose_o, sc.actions[s])
        a = torch.zeros((o.T, 8), dtype=torch.float64, device=eng.device)
        a[:, :7] = torch.as_tensor(acts, device=eng.device)
        v = torch.zeros((n, o.T, 8), dtype=torch.float64, device=eng.device)
        p = torch.zeros((n + 1, o.T, 8), dtype=torch.float64, device=eng.device)
        p[0] = p0
        coll = eng.new_coll(1)
        eng.tools_action(a, v, p, None if coll is None else coll[0])
        torch.cuda.synchronize()
        assert rel_err(p.cpu().numpy(), pseq) < 1e-12, s
        if which == "collision":
            c = coll[0].cpu().numpy()
            assert (c[..., 0] >= 0).any()
            assert np.array_equal(c[..., 0] >= 0, o.last_coll[..., 0] >= 0)
        gps = np.random.default_rng(s).normal(size=pseq.shape)
        g_ref, ga_ref = gps.copy(), np.zeros((o.T, 7))
        o.tools_action_bwd(acts, vel, pseq, o.last_coll, g_ref, ga_ref)
        g = torch.as_tensor(gps, device=eng.device).contiguous()
        ga = torch.zeros((o.T, 8), dtype=torch.float64, device=eng.device)
        eng.tools_action_bwd(v, p, g, ga, None if coll is None else coll[0])
        torch.cuda.synchronize()
        assert rel_err(g.cpu().numpy(), g_ref) < 1e-10, s
        assert rel_err(ga.cpu().numpy()[:, :7], ga_ref) < 1e-10, s
        pose_o, p0 = pseq[-1], p[-1].clone()


def test_collision_trajectory_loss_and_grad(gpu_lib):
    """Horizon over actions with tool-tool projections against the oracle's
    store-all rollout and reverse sweep."""
    tools = collision_tools()
    sc = small_scene(n=3000, tools=tools, precision="fp64", substeps=10, n_actions=2)
    eng = make_engine(sc)
    o = Oracle(sc.sim, tools)
    loss_ref, grad_ref = o.loss_and_grad(sc.x0, sc.actions, sc.target)
    hz = Horizon(eng, sc.n_actions, ckpt_every=5)
    hz.forward(eng.init_state([sc.x0]), eng.expand_actions([sc.actions]))
    loss = float(hz.loss(eng.targets([sc.target])).sum())
    g = eng.collapse_action_grad(hz.backward())[0].cpu().numpy()
    torch.cuda.synchronize()
    assert abs(loss - loss_ref) < 1e-12 * abs(loss_ref)
    assert rel_err(g, grad_ref) < 1e-8


@pytest.mark.parametrize("prec,loss_tol,grad_tol", [("fp64", 1e-9, 1e-6), ("fp32_svd64", 1e-5, 1e-3),
                                                    ("fp32", 1e-5, 1e-3)])
def test_config4_grid128_knife_gripper_trajectory(gpu_lib, prec, loss_tol, grad_tol):
    """Config-4 shape on the 128^3 grid: knife (box ∩ prism) and gripper, density
    L1 to the two half piles plus the soft contact term, against the oracle."""
    from diffskill_gb300 import scenes
    sc = scenes.config4(n_actions=2, n_particles=12000, substeps=10, precision=prec)
    assert sc.sim.grid == 128
    o = Oracle(sc.sim, sc.tools)
    ref_loss, ref_grad = o.loss_and_grad(sc.x0, sc.actions, sc.target, density_weight=sc.density_weight,
                                         contact_weight=sc.contact_weight)
    eng = make_engine(sc)
    loss, grad, _ = _traj(eng, sc, k=5)
    assert eng.status() == 0
    assert abs(loss - ref_loss) / abs(ref_loss) < loss_tol, (loss, ref_loss)
    assert np.abs(ref_grad).max() > 0
    assert rel_err(grad, ref_grad) < grad_tol, (grad, ref_grad)


@pytest.mark.gpu
def test_chained_forward_equals_unchained(gpu_lib):
    """Chained forward substeps (g2p flags the next substep's blocks, the
    marking pass is skipped) give the frames of unchained substeps."""
    sc = small_scene(n=4000, n_actions=2, substeps=30, tools=[all_tools()[1], all_tools()[2]], precision="fp64")
    eng = make_engine(sc)
    hz = Horizon(eng, sc.n_actions, ckpt_every=1, resort_every=0)  # keep the particle order
    st0 = eng.init_state([sc.x0])
    acts = eng.expand_actions([sc.actions])
    hz.forward(st0, acts)  # chained inside
    chained = hz.final.clone()
    frames = [st0.clone(), eng.new_state()]
    eng.set_chained(False)
    for f in range(hz.F):
        eng.substep(frames[f % 2], frames[(f + 1) % 2], hz.pose[f], hz.pose[f + 1])
    plain = frames[hz.F % 2]
    torch.cuda.synchronize()
    P = eng.P
    assert hz.R == 0
    assert rel_err(chained[:, :P].cpu().numpy(), plain[:, :P].cpu().numpy()) < 1e-12
