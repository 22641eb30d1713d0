"""The reference-shaped API (MPMSimulator / Primitives / GradModel) on the GPU,
checked against the FP64 oracle through the same observation functionals the
reference's optimiser uses (plb/engine/function.py, plb/optimizer/solver.py)."""
import numpy as np
import pytest
import torch

from _util import all_tools, small_scene
from diffskill_gb300.function import GradModel, SimEnv
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def oracle_obs_grad(o, x0, actions, Wx, Wc, Wd=None):
    """d/d actions of sum_s <Wx[s], x||v(s+1)> + <Wc[s], tools(s+1)> [+ <Wd[s], dists(s+1)>]."""
    ro = o.rollout(x0, actions, keep_frames=True)
    frames, poses = ro["frames"], ro["poses"]
    n, A = o.n_sub, len(actions)
    F = A * n
    g = np.zeros_like(frames[0])
    gp = np.zeros((F + 1, o.T, 8))
    loss = 0.0
    for f in range(F - 1, -1, -1):
        if (f + 1) % n == 0:
            s = (f + 1) // n - 1
            st = frames[f + 1]
            loss += float((Wx[s] * st[:, 0:6]).sum()) + float((Wc[s][:, :8] * poses[f + 1]).sum())
            g[:, 0:6] += Wx[s]
            gp[f + 1] += Wc[s][:, :8]
            if Wd is not None:
                col = 0
                x = np.ascontiguousarray(st[:, 0:3])
                for t in range(o.T):
                    nc = O.lib().oracle_tool_distance_cols(O.ctypes.byref(o.tools[t]))
                    pz = np.ascontiguousarray(poses[f + 1, t])
                    d = np.zeros((st.shape[0], nc))
                    O.lib().oracle_tool_distance(O.ctypes.byref(o.tools[t]), O.ptr(pz), st.shape[0], O.ptr(x),
                                                 O.ptr(d))
                    w = np.ascontiguousarray(Wd[s][:, col:col + nc])
                    loss += float((w * d).sum())
                    gx = np.zeros((st.shape[0], 3))
                    gpt = np.zeros(8)
                    O.lib().oracle_tool_distance_vjp(O.ctypes.byref(o.tools[t]), O.ptr(pz), st.shape[0], O.ptr(x),
                                                     O.ptr(w), O.ptr(gx), O.ptr(gpt))
                    g[:, 0:3] += gx
                    gp[f + 1, t] += gpt
                    col += nc
        g = o.substep_bwd(poses[f], poses[f + 1], frames[f], g, gp[f], gp[f + 1])
    g_act = np.zeros((A, o.T, 7))
    for s in range(A - 1, -1, -1):
        sl = gp[s * n:(s + 1) * n + 1]
        o.tools_action_bwd(ro["acts"][s], ro["vels"][s], poses[s * n:(s + 1) * n + 1], ro["colls"][s], sl, g_act[s])
    flat = np.concatenate([g_act[:, i, :o.dims[i + 1] - o.dims[i]] for i in range(o.T)], axis=1)
    return loss, flat


def _weights(rng, A, n, T, k=0):
    f32 = lambda a: a.astype(np.float32).astype(np.float64)  # exactly representable in the FP32 observations
    Wx = [f32(rng.normal(size=(n, 6))) for _ in range(A)]
    Wc = [f32(rng.normal(size=(T, 8))) for _ in range(A)]
    Wd = [f32(rng.normal(size=(n, k))) for _ in range(A)] if k else None
    return Wx, Wc, Wd


@pytest.mark.parametrize("return_dist", [False, True])
def test_gradmodel_matches_oracle(gpu_lib, return_dist):
    tools = [all_tools()[1], all_tools()[4]]  # capsule + gripper (two distance columns)
    sc = small_scene(n=1500, n_actions=3, substeps=10, tools=tools, precision="fp64")
    env = SimEnv(sc.sim, sc.tools, sc.x0)
    gm = GradModel(env, return_dist=return_dist)
    rng = np.random.default_rng(11)
    k = 3 if return_dist else 0
    Wx, Wc, Wd = _weights(rng, sc.n_actions, sc.n_particles, len(tools), k)
    acts = torch.tensor(sc.actions, dtype=torch.float32, device="cuda", requires_grad=True)
    obs = gm.reset()
    loss = 0
    for s in range(sc.n_actions):
        obs = gm.forward(s, acts[s], *obs)
        x = obs[0]
        loss = loss + (torch.as_tensor(Wx[s], device="cuda").float() * x[:, :6]).sum()
        loss = loss + (torch.as_tensor(Wc[s], device="cuda").float() * obs[1]).sum()
        if return_dist:
            loss = loss + (torch.as_tensor(Wd[s], device="cuda").float() * x[:, 6:]).sum()
    loss.backward()
    o = O.Oracle(sc.sim, tools)
    ref_loss, ref_grad = oracle_obs_grad(o, sc.x0, sc.actions.astype(np.float32).astype(np.float64), Wx, Wc, Wd)
    got = acts.grad.double().cpu().numpy()
    assert abs(loss.item() - ref_loss) < 1e-4 * abs(ref_loss)
    assert np.abs(got - ref_grad).max() < 1e-5 * np.abs(ref_grad).max(), (got, ref_grad)


def test_gradmodel_output_grid_density_loss_matches_oracle(gpu_lib):
    """Density L1 on the grid_m observation (output_grid, function.py:122-126, 147-152)."""
    sc = small_scene(n=2000, n_actions=2, substeps=25, precision="fp64")
    env = SimEnv(sc.sim, sc.tools, sc.x0)
    gm = GradModel(env, output_grid=(1,))
    acts = torch.tensor(sc.actions, dtype=torch.float64, device="cuda", requires_grad=True)
    obs = gm.reset()
    for s in range(sc.n_actions):
        obs = gm.forward(s, acts[s], *obs)
    tgt = torch.as_tensor(sc.target.reshape(64, 64, 64), device="cuda").float()
    loss = (obs[2] - tgt).abs().sum()
    loss.backward()
    ref_loss, ref_grad = O.Oracle(sc.sim, sc.tools).loss_and_grad(sc.x0, sc.actions, sc.target)
    assert abs(loss.item() - ref_loss) < 1e-5 * ref_loss
    got = acts.grad.double().cpu().numpy()
    assert np.abs(got - ref_grad).max() < 1e-3 * np.abs(ref_grad).max(), (got, ref_grad)


def test_simulator_state_io_and_step(gpu_lib):
    """get_state/set_state round trip; step(is_copy=True) == oracle rollout of one action."""
    sc = small_scene(n=1200, n_actions=1, substeps=10, precision="fp64")
    env = SimEnv(sc.sim, sc.tools, sc.x0)
    sim = env.simulator
    st = sim.get_state(0)
    assert st[0].shape == (1200, 3) and st[2].shape == (1200, 3, 3) and len(st) == 5
    assert np.allclose(st[2], np.eye(3)) and np.allclose(st[1], 0) and np.allclose(st[0], sc.x0)
    env.step(sc.actions[0])
    got = sim.get_state(0)
    ref = O.Oracle(sc.sim, sc.tools).rollout(sc.x0, sc.actions, keep_frames=False)
    fin = ref["final"]
    assert np.abs(got[0] - fin[:, 0:3]).max() < 1e-12
    assert np.abs(got[1] - fin[:, 3:6]).max() < 1e-9 * max(1, np.abs(fin[:, 3:6]).max())
    assert np.abs(got[4] - ref["poses"][-1][0][:7]).max() < 1e-12
    sim.set_state(0, st)
    back = sim.get_state(0)
    for a, b in zip(st, back):
        assert np.array_equal(np.asarray(a), np.asarray(b))
    # grid mass of frame 0 conserves mass (mpm_simulator.py:456-471)
    sim.compute_grid_m_kernel(0)
    assert abs(sim.get_m().sum() - 1200 * sc.sim.p_mass) < 1e-12


def test_primitives_api(gpu_lib):
    sc = small_scene(n=500, n_actions=2, substeps=5, tools=all_tools(), precision="fp32")
    env = SimEnv(sc.sim, sc.tools, sc.x0)
    prims = env.primitives
    assert prims.action_dims == [0, 3, 9, 15, 21, 28]
    assert prims.state_dim == 7 * 4 + 8
    assert prims[4].get_state(0).shape == (8,)
    with pytest.raises(ValueError):
        prims.set_action(0, env.simulator.substeps, np.zeros(5))
    prims.set_action(0, env.simulator.substeps, np.full(28, 3.0))  # clipped to [-1, 1]
    assert np.allclose(env.simulator._act[0, 0, :3].cpu().numpy(), 1.0)
    g = prims.get_grad(1)
    assert g.shape == (1, 28)
