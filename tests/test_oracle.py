"""CPU tests of the FP64 oracle: golden vectors from the reference, SVD,
SDF/normal property, and the hand adjoint against central differences."""
import json
import os

import numpy as np
import pytest

from _util import all_tools, collision_tools, more_tools, perturbed_state, small_scene
from diffskill_gb300 import scenes
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "density_assets.json")


@pytest.fixture(scope="module")
def golden():
    with open(GOLDEN) as fh:
        return json.load(fh)


# --------------------------------------------------------------------------
# golden vectors: the reference's density assets (plb/envs/assets/*.npy)
# --------------------------------------------------------------------------
def test_assets_pin_particle_mass(golden):
    """Every asset holds 10000 particles of p_mass=(dx/2)^2 (mpm_simulator.py:28-29)."""
    sim = scenes.config1().sim
    assert sim.p_mass == (0.5 / 64) ** 2
    for name, g in golden["grids"].items():
        assert g["n_grid"] == 64
        assert abs(g["total_mass"] - 10000 * sim.p_mass) < 1e-12, name


def test_oracle_grid_mass_reproduces_move3d_asset(golden):
    """Oracle compute_grid_m of a seeded sphere sample, placed like the
    Move3D-v1 target, matches the asset's mass, support and moments."""
    g = golden["grids"]["Move3D-v1.npy"]
    r = golden["move3d_v1_sphere_radius"]
    sc = scenes.config1(n_particles=10)
    rng = np.random.default_rng(77)
    x = scenes.sample_sphere(rng, 10000, (0, 0, 0), r)
    x = x - x.mean(0) + np.array(g["centroid"])  # same centroid as the asset
    o = O.Oracle(sc.sim, [])
    gm = o.grid_mass(O.init_state(x)).reshape(64, 64, 64)
    dx = 1 / 64
    idx = np.indices(gm.shape).reshape(3, -1).T * dx
    m = gm.reshape(-1)
    tot = m.sum()
    assert abs(tot - g["total_mass"]) < 1e-12
    cen = (m[:, None] * idx).sum(0) / tot
    assert np.abs(cen - x.mean(0)).max() < 1e-12  # linear reproduction of the B-spline
    var = (m[:, None] * (idx - cen) ** 2).sum(0) / tot
    assert np.abs(var - x.var(0) - dx * dx / 4).max() < 1e-12  # B-spline variance dx^2/4
    # against the asset: same support box (+-1 node) and moments within sampling noise
    nz = np.argwhere(gm > 0)
    assert np.abs(nz.min(0) - np.array(g["support_min"])).max() <= 1
    assert np.abs(nz.max(0) - np.array(g["support_max"])).max() <= 1
    assert abs(var.mean() - np.mean(g["var"])) < 0.03 * np.mean(g["var"])
    assert abs(gm.max() - g["max"]) < 0.15 * g["max"]


# --------------------------------------------------------------------------
# SVD (ti.svd convention, mpm_simulator.py:127-129) and backward_svd (137-156)
# --------------------------------------------------------------------------
def _svd(A):
    U, s, V = np.zeros(9), np.zeros(3), np.zeros(9)
    O.lib().oracle_svd(O.ptr(np.ascontiguousarray(A.reshape(9))), O.ptr(U), O.ptr(s), O.ptr(V))
    return U.reshape(3, 3), s, V.reshape(3, 3)


@pytest.mark.parametrize("kind", ["random", "near_rotation", "reflection", "degenerate", "identity"])
def test_svd_convention(kind):
    rng = np.random.default_rng(0)
    for _ in range(50):
        if kind == "random":
            A = rng.normal(size=(3, 3))
        elif kind == "near_rotation":
            q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
            A = q * np.sign(np.linalg.det(q)) + 1e-3 * rng.normal(size=(3, 3))
        elif kind == "reflection":
            A = np.diag([1.0, 1.0, -1.0]) @ rng.normal(size=(3, 3))
            if np.linalg.det(A) > 0:
                A[2] *= -1
        elif kind == "degenerate":
            q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
            A = q @ np.diag([1.0, 1.0, 0.5]) @ q.T
        else:
            A = np.eye(3)
        U, s, V = _svd(A)
        assert np.allclose(U @ np.diag(s) @ V.T, A, atol=1e-12)
        assert np.allclose(U.T @ U, np.eye(3), atol=1e-12) and np.allclose(V.T @ V, np.eye(3), atol=1e-12)
        assert abs(np.linalg.det(U) - 1) < 1e-12 and abs(np.linalg.det(V) - 1) < 1e-12
        assert s[0] >= s[1] - 1e-14 and s[1] >= abs(s[2]) - 1e-14
        assert np.sign(s[2]) == np.sign(np.linalg.det(A)) or abs(s[2]) < 1e-12


def test_svd_backward_matches_finite_differences():
    """With well separated singular values the clamped formula is the exact VJP."""
    rng = np.random.default_rng(1)
    for _ in range(20):
        q1, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        q2, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        A = q1 @ np.diag([1.6, 1.1, 0.7]) @ q2.T
        gU, gs, gV = rng.normal(size=9), rng.normal(size=3), rng.normal(size=9)
        U, s, V = _svd(A)
        gA = np.zeros(9)
        O.lib().oracle_svd_bwd(O.ptr(U.reshape(9).copy()), O.ptr(s), O.ptr(V.reshape(9).copy()), O.ptr(gU),
                               O.ptr(gs), O.ptr(gV), O.ptr(gA))

        def f(M):
            u, ss, v = _svd(M)
            return gU @ u.reshape(9) + gs @ ss + gV @ v.reshape(9)

        fd = np.zeros(9)
        for i in range(9):
            e = np.zeros(9)
            e[i] = 1e-6
            fd[i] = (f(A + e.reshape(3, 3)) - f(A - e.reshape(3, 3))) / 2e-6
        assert np.abs(fd - gA).max() < 1e-6 * max(1, np.abs(gA).max())


def test_svd_backward_clamp_at_identity():
    """F = I: s_j^2 - s_i^2 = 0 is clamped to +1e-6 (mpm_simulator.py:184-192), and the
    rotation terms cancel exactly for a gradient that only flows through R = U V^T."""
    U, s, V = _svd(np.eye(3))
    gR = np.random.default_rng(2).normal(size=(3, 3))
    gU, gV = gR @ V, gR.T @ U
    gA = np.zeros(9)
    O.lib().oracle_svd_bwd(O.ptr(U.reshape(9).copy()), O.ptr(s), O.ptr(V.reshape(9).copy()),
                           O.ptr(gU.reshape(9).copy()), O.ptr(np.zeros(3)), O.ptr(gV.reshape(9).copy()), O.ptr(gA))
    assert np.abs(gA).max() < 1e-9


# --------------------------------------------------------------------------
# SDF / normal property (plb/engine/primitive/test_primitives.py:34-67)
# --------------------------------------------------------------------------
@pytest.mark.parametrize("ti", range(5))
def test_tool_normal_matches_sdf_gradient(ti):
    tool = all_tools()[ti]
    ts = O.tool_struct(tool, 666.0)
    pose = np.array(tool.init_state, dtype=np.float64)
    # Primitive.normal rotates by the stored quaternion without normalising it
    # (primive_base.py:85); the property holds exactly for unit quaternions.
    pose[3:7] /= np.linalg.norm(pose[3:7])
    rng = np.random.default_rng(ti)
    pts = pose[:3] + rng.normal(size=(400, 3)) * 0.06
    sdf, nrm = np.zeros(400), np.zeros((400, 3))
    O.lib().oracle_tool_sdf(ctypes_ref(ts), O.ptr(pose), 400, O.ptr(pts), O.ptr(sdf), O.ptr(nrm))
    fd = np.zeros((400, 3))
    for k in range(3):
        e = np.zeros(3)
        e[k] = 1e-7
        sp, sm = np.zeros(400), np.zeros(400)
        O.lib().oracle_tool_sdf(ctypes_ref(ts), O.ptr(pose), 400, O.ptr(pts + e), O.ptr(sp), None)
        O.lib().oracle_tool_sdf(ctypes_ref(ts), O.ptr(pose), 400, O.ptr(pts - e), O.ptr(sm), None)
        fd[:, k] = (sp - sm) / 2e-7
    fdn = fd / np.linalg.norm(fd, axis=1, keepdims=True)
    err = np.linalg.norm(fdn - nrm, axis=1)
    if tool.shape in ("Sphere", "Capsule"):
        assert np.median(err) < 1e-5 and np.mean(err < 1e-5) > 0.95
    else:  # FD normal with d=1e-4: agrees away from edges and corners
        assert np.mean(err < 1e-3) > 0.8


def ctypes_ref(s):
    import ctypes
    return ctypes.byref(s)


# --------------------------------------------------------------------------
# the hand adjoint against FP64 central differences
# --------------------------------------------------------------------------
def _fd_best(f, x0, i, eps_list=(1e-3, 1e-4, 1e-5, 1e-6)):
    vals = []
    for eps in eps_list:
        xp, xm = x0.copy(), x0.copy()
        xp.flat[i] += eps
        xm.flat[i] -= eps
        vals.append((f(xp) - f(xm)) / (2 * eps))
    return vals


@pytest.mark.parametrize("ti", range(5))
def test_substep_adjoint_matches_finite_differences(ti):
    tools = [all_tools()[ti]]
    sc = small_scene(n=250, substeps=3, tools=tools, precision="fp64")
    sc.sim.yield_stress = 5.0  # exercise the plastic branch
    o = O.Oracle(sc.sim, tools)
    st0 = perturbed_state(sc.x0, seed=ti)
    rng = np.random.default_rng(100 + ti)
    W = rng.normal(size=st0.shape)
    a = sc.actions[0]
    K = sc.sim.n_substeps

    def run(st, act, frames=None):
        _, _, pseq = o.tools_action(o.pose0(), act)
        s = st
        for j in range(K):
            if frames is not None:
                frames.append(s)
            s = o.substep(pseq[j], pseq[j + 1], s)
        return float((W * s).sum()), pseq

    frames = []
    _, pseq = run(st0, a, frames)
    g = W.copy()
    gp = np.zeros((K + 1, o.T, 8))
    for f in range(K - 1, -1, -1):
        g = o.substep_bwd(pseq[f], pseq[f + 1], frames[f], g, gp[f], gp[f + 1])
    idx = [int(i) for i in rng.integers(0, st0.size, size=12)]
    for i in idx:
        fds = _fd_best(lambda s: run(s, a)[0], st0, i)
        best = min(abs(v - g.flat[i]) / max(abs(v), 1e-8) for v in fds)
        assert best < 1e-5, (i, g.flat[i], fds)


def test_tools_action_adjoint_matches_finite_differences():
    tools = all_tools()
    sc = small_scene(n=10, substeps=7, tools=tools, precision="fp64")
    o = O.Oracle(sc.sim, tools)
    a = sc.actions[0]
    rng = np.random.default_rng(3)
    W = rng.normal(size=(sc.sim.n_substeps + 1, o.T, 8))

    def f(act):
        return float((W * o.tools_action(o.pose0(), act)[2]).sum())

    acts, vel, pseq = o.tools_action(o.pose0(), a)
    gp = W.copy()
    ga = np.zeros((o.T, 7))
    o.tools_action_bwd(acts, vel, pseq, o.last_coll, gp, ga)
    flat = np.concatenate([ga[i, :o.dims[i + 1] - o.dims[i]] for i in range(o.T)])
    for k in range(len(a)):
        fds = _fd_best(f, a, k, (1e-5, 1e-6))
        best = min(abs(v - flat[k]) / max(abs(v), 1e-8) for v in fds)
        assert best < 1e-6, (k, flat[k], fds)


def test_trajectory_action_gradient_matches_finite_differences():
    sc = small_scene(n=300, n_actions=2, substeps=5, precision="fp64")
    sc.tools[0].action.scale = (0.05, 0.05, 0.05)
    o = O.Oracle(sc.sim, sc.tools)
    loss, grad = o.loss_and_grad(sc.x0, sc.actions, sc.target)
    W = sc.actions.copy()
    for i in range(W.size):
        fds = _fd_best(lambda A: o.loss(o.rollout(sc.x0, A, keep_frames=False)["final"], sc.target), W, i,
                       (1e-6, 1e-7))
        best = min(abs(v - grad.flat[i]) / max(abs(v), 1e-6) for v in fds)
        assert best < 1e-4, (i, grad.flat[i], fds)


def test_grid_mass_conserves_particle_mass():
    sc = small_scene(n=3000, precision="fp64")
    o = O.Oracle(sc.sim, sc.tools)
    gm = o.grid_mass(perturbed_state(sc.x0))
    assert abs(gm.sum() - 3000 * sc.sim.p_mass) < 1e-14


def test_oracle_is_deterministic_across_thread_counts():
    sc = small_scene(n=2000, precision="fp64", tools=all_tools())
    o = O.Oracle(sc.sim, sc.tools)
    st0 = perturbed_state(sc.x0, seed=1)
    _, _, pseq = o.tools_action(o.pose0(), sc.actions[0])
    n0 = O.num_threads()
    try:
        O.set_num_threads(1)
        a = o.substep(pseq[0], pseq[1], st0)
        ga = o.substep_bwd(pseq[0], pseq[1], st0, st0, np.zeros((o.T, 8)), np.zeros((o.T, 8)))
        O.set_num_threads(4)
        b = o.substep(pseq[0], pseq[1], st0)
        gb = o.substep_bwd(pseq[0], pseq[1], st0, st0, np.zeros((o.T, 8)), np.zeros((o.T, 8)))
    finally:
        O.set_num_threads(n0)
    assert np.array_equal(a, b) and np.array_equal(ga, gb)


def test_single_scene_dt_5e4_exceeds_cfl_and_diverges():
    """dt=5e-4 on the single-scene 64^3 workload exceeds the CFL limit dx/c ~ 2.1e-4
    (c = sqrt((lam+2mu)/rho) ~ 74.5): the FP64 oracle produces NaN; the
    reference's own dt=1e-4 (mpm_simulator.py:27) stays finite."""
    sc = scenes.config1(n_actions=4, n_particles=2000, dt=5e-4, substeps=50)
    o = O.Oracle(sc.sim, sc.tools)
    fin = o.rollout(sc.x0, sc.actions, keep_frames=False)["final"]
    assert not np.isfinite(fin[:, 3:]).all()
    sc = scenes.config1(n_actions=4, n_particles=2000, dt=1e-4, substeps=50)
    fin = O.Oracle(sc.sim, sc.tools).rollout(sc.x0, sc.actions, keep_frames=False)["final"]
    assert np.isfinite(fin).all()


# ---------------------------------------------------------------- loss.py terms
def _target_sdf_python(dens, dx, n_iters):
    """update_target (loss.py:105-134) as plain Python loops, for small grids."""
    n = dens.shape[0]
    inf = 1000.0
    sc = np.full((n, n, n), inf)
    nc = np.zeros((n, n, n, 3))
    sdf, near = sc.copy(), nc.copy()
    offs = [(a, b, c) for a in range(-3, 3) for b in range(-3, 3) for c in range(-3, 3)]
    for _ in range(n_iters):
        for i in range(n):
            for j in range(n):
                for k in range(n):
                    gp = np.array([i * dx, j * dx, k * dx])
                    sdf[i, j, k] = inf
                    if dens[i, j, k] > 1e-4:
                        sdf[i, j, k] = 0.0
                        near[i, j, k] = gp
                        continue
                    near[i, j, k] = 0.0
                    for a, b, c in offs:
                        v = (i + a, j + b, k + c)
                        if min(v) < 0 or max(v) >= n or abs(a) + abs(b) + abs(c) == 0:
                            continue
                        if sc[v] < inf:
                            d = gp - nc[v]
                            dist = np.sqrt(((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]) + 1e-8)
                            if dist < sdf[i, j, k]:
                                sdf[i, j, k] = dist
                                near[i, j, k] = nc[v]
        sc, nc = sdf.copy(), near.copy()
    return sdf, near


def _sparse_target(n, seed):
    rng = np.random.default_rng(seed)
    d = np.zeros((n, n, n))
    d[rng.random((n, n, n)) < 0.03] = 1e-3
    d[rng.random((n, n, n)) < 0.05] = 5e-5  # below the threshold
    return d


@pytest.mark.parametrize("n_iters", [1, 2, 6])
def test_target_sdf_matches_python_restatement(n_iters):
    d = _sparse_target(8, 3)
    s_ref, n_ref = _target_sdf_python(d, 1 / 8, n_iters)
    s, near = O.target_sdf(d, 1 / 8, n_iters)
    assert np.array_equal(s, s_ref) and np.array_equal(near, n_ref)


def test_target_sdf_converged_field_properties():
    """After 2 n sweeps every node holds the distance to a dense node (its
    'nearest point'), never less than the true distance to the dense set, and
    dense nodes hold 0."""
    n, dx = 16, 1 / 16
    d = _sparse_target(n, 5)
    d[d < 1e-4] = 0.0
    s, near = O.target_sdf(d, dx, 2 * n)
    dense = np.argwhere(d > 1e-4)
    gp = np.stack(np.meshgrid(*[np.arange(n) * dx] * 3, indexing="ij"), -1)
    assert (s[d > 1e-4] == 0).all()
    assert np.allclose(s, np.sqrt(((gp - near) ** 2).sum(-1) + 1e-8) * (d <= 1e-4), atol=1e-15)
    true = np.sqrt(((gp[:, :, :, None, :] - dense[None, None, None] * dx) ** 2).sum(-1).min(-1))
    assert (s[d <= 1e-4] >= true[d <= 1e-4] - 1e-12).all()
    assert (s < 1000).all()
    # FP32 rounding of the same sweeps stays within FP32 resolution
    s32, _ = O.target_sdf(d, dx, 2 * n, single=True)
    assert np.abs(s32 - s).max() < 1e-6


def test_iou_and_sdf_loss_definitions():
    rng = np.random.default_rng(0)
    a, b = rng.random(512), rng.random(512)
    ma, mb = a.max(), b.max()
    inter = (a * b).sum() / ma / mb
    assert abs(O.iou(a, b) - inter / (a.sum() / ma + b.sum() / mb - inter)) < 1e-15
    # identical normalised grids: I / (2 sum t / mb - I)
    assert O.iou(a, a) == pytest.approx(((a * a).sum() / ma ** 2) / (2 * a.sum() / ma - (a * a).sum() / ma ** 2))
    loss, g = O.sdf_loss(a, b)
    assert loss == pytest.approx(float((a * b).sum())) and np.array_equal(g, b)


def test_contact_min_and_its_adjoint():
    """Hard contact distance: the minimum over particles of max(sdf, 0) and a
    gradient through the argmin particle that matches central differences."""
    tools = all_tools()
    sc = small_scene(n=400, tools=tools)
    o = O.Oracle(sc.sim, tools)
    st = perturbed_state(sc.x0, seed=5)
    pose = o.pose0()
    for t in range(o.T):
        md, am = o.contact_min(t, pose[t], st)
        sd = np.array([o.contact_min(t, pose[t], st[i:i + 1])[0] for i in range(0, st.shape[0], 37)])
        assert md <= sd.min() + 1e-15
        if md <= 0:
            continue
        g = np.zeros_like(st)
        gp = np.zeros(8)
        o.contact_min(t, pose[t], st, 1.0, g, gp)
        for d in range(3):
            e = np.zeros_like(st)
            e[am, d] = 1e-7
            fd = (o.contact_min(t, pose[t], st + e)[0] - o.contact_min(t, pose[t], st - e)[0]) / 2e-7
            assert abs(fd - g[am, d]) < 1e-5


# --------------------------------------------------------------------------
# the remaining tools of primitives.py and the tool-tool collision projection
# --------------------------------------------------------------------------
@pytest.mark.parametrize("ti", range(6))
def test_more_tools_normal_matches_sdf_gradient(ti):
    """test_primitives.py:34-67's property for RollingPin(Ext), Chopsticks,
    Cylinder, Torus and Gripper2: the analytic normal is the normalised SDF
    gradient away from the shapes' kinks."""
    tool = more_tools()[ti]
    ts = O.tool_struct(tool, 666.0)
    pose = np.array(tool.init_state, dtype=np.float64)
    pose[3:7] /= np.linalg.norm(pose[3:7])
    rng = np.random.default_rng(40 + ti)
    pts = pose[:3] + rng.normal(size=(400, 3)) * 0.05
    sdf, nrm = np.zeros(400), np.zeros((400, 3))
    O.lib().oracle_tool_sdf(ctypes_ref(ts), O.ptr(pose), 400, O.ptr(pts), O.ptr(sdf), O.ptr(nrm))
    fd = np.zeros((400, 3))
    for k in range(3):
        e = np.zeros(3)
        e[k] = 1e-7
        sp, sm = np.zeros(400), np.zeros(400)
        O.lib().oracle_tool_sdf(ctypes_ref(ts), O.ptr(pose), 400, O.ptr(pts + e), O.ptr(sp), None)
        O.lib().oracle_tool_sdf(ctypes_ref(ts), O.ptr(pose), 400, O.ptr(pts - e), O.ptr(sm), None)
        fd[:, k] = (sp - sm) / 2e-7
    fdn = fd / np.linalg.norm(fd, axis=1, keepdims=True)
    err = np.linalg.norm(fdn - nrm, axis=1)
    assert np.median(err) < 1e-5 and np.mean(err < 1e-4) > 0.9, (tool.shape, np.median(err))


@pytest.mark.parametrize("ti", range(6))
def test_more_tools_substep_adjoint_matches_finite_differences(ti):
    tools = [more_tools()[ti]]
    sc = small_scene(n=250, substeps=3, tools=tools, precision="fp64")
    sc.sim.yield_stress = 5.0
    o = O.Oracle(sc.sim, tools)
    st0 = perturbed_state(sc.x0, seed=ti)
    rng = np.random.default_rng(200 + ti)
    W = rng.normal(size=st0.shape)
    a = sc.actions[0]
    K = sc.sim.n_substeps

    def run(st, frames=None):
        _, _, pseq = o.tools_action(o.pose0(), a)
        s = st
        for j in range(K):
            if frames is not None:
                frames.append(s)
            s = o.substep(pseq[j], pseq[j + 1], s)
        return float((W * s).sum()), pseq

    frames = []
    _, pseq = run(st0, frames)
    g = W.copy()
    gp = np.zeros((K + 1, o.T, 8))
    for f in range(K - 1, -1, -1):
        g = o.substep_bwd(pseq[f], pseq[f + 1], frames[f], g, gp[f], gp[f + 1])
    for i in [int(i) for i in rng.integers(0, st0.size, size=12)]:
        fds = _fd_best(lambda s: run(s)[0], st0, i)
        best = min(abs(v - g.flat[i]) / max(abs(v), 1e-8) for v in fds)
        assert best < 1e-5, (i, g.flat[i], fds)
    # the tool-pose gradients of the substeps (incl. the Chopsticks gap) through the kinematics
    acts, vel, _ = o.tools_action(o.pose0(), a)
    ga = np.zeros((o.T, 7))
    o.tools_action_bwd(acts, vel, pseq, o.last_coll, gp, ga)
    flat = ga[0, :int(tools[0].action.dim)]

    def loss_of(act):
        _, _, ps = o.tools_action(o.pose0(), act)
        s = st0
        for j in range(K):
            s = o.substep(ps[j], ps[j + 1], s)
        return float((W * s).sum())

    for k in range(len(a)):
        fds = _fd_best(loss_of, a, k, (1e-4, 1e-5, 1e-6))
        best = min(abs(v - flat[k]) / max(abs(v), 1e-7) for v in fds)
        assert best < 1e-4, (tools[0].shape, k, flat[k], fds)


def test_more_tools_kinematics_adjoint_matches_finite_differences():
    tools = more_tools()
    sc = small_scene(n=10, substeps=7, tools=tools, precision="fp64")
    o = O.Oracle(sc.sim, tools)
    a = sc.actions[0]
    rng = np.random.default_rng(5)
    W = rng.normal(size=(sc.sim.n_substeps + 1, o.T, 8))

    def f(act):
        return float((W * o.tools_action(o.pose0(), act)[2]).sum())

    acts, vel, pseq = o.tools_action(o.pose0(), a)
    gp = W.copy()
    ga = np.zeros((o.T, 7))
    o.tools_action_bwd(acts, vel, pseq, o.last_coll, gp, ga)
    flat = np.concatenate([ga[i, :o.dims[i + 1] - o.dims[i]] for i in range(o.T)])
    for k in range(len(a)):
        fds = _fd_best(f, a, k, (1e-5, 1e-6))
        best = min(abs(v - flat[k]) / max(abs(v), 1e-8) for v in fds)
        assert best < 1e-6, (k, flat[k], fds)
    # RollingPin: rot' = w2quat((0,-dth,0)) rot w2quat((0,dw,0)) keeps the pin horizontal
    rp = pseq[-1, 0]
    axis = np.array([0.0, 1.0, 0.0])  # the capsule's local axis
    q = rp[3:7] / np.linalg.norm(rp[3:7])
    w, v = q[0], q[1:]
    world_axis = axis + 2 * (w * np.cross(v, axis) + np.cross(v, np.cross(v, axis)))
    assert abs(world_axis[1]) < 1e-9


def test_collision_projection_picks_first_most_negative_point():
    """set_collision_idx semantics: the first of the 600 surface points with the
    smallest SDF below 0, and after the projection that point lies on the tool
    surface (box against box)."""
    tools = collision_tools()
    sc = small_scene(n=10, substeps=5, tools=tools, precision="fp64")
    o = O.Oracle(sc.sim, tools)
    assert o.n_pairs == 2
    acts, vel, pseq = o.tools_action(o.pose0(), sc.actions[0])
    coll = o.last_coll
    assert (coll[:, :, 0] >= 0).any()
    for j in range(sc.sim.n_substeps):
        # recompute the argmin of step j from the pre-projection poses: FK only
        pre = pseq[j + 1].copy()
        for c, (i, jj) in enumerate([(0, 2), (1, 2)]):
            box = tools[jj]
            rn = o.pts[c]
            local = np.clip(rn * np.array(box.size), -np.array(box.size), np.array(box.size))
            q = pre[jj, 3:7]
            w_, v_ = q[0], q[1:]
            world = local + 2 * (w_ * np.cross(v_, local) + np.cross(v_, np.cross(v_, local))) + pre[jj, :3]
            if coll[j, c, 0] >= 0:
                k = int(coll[j, c, 0])
                assert np.allclose(world[k], coll[j, c, 1:]), (j, c)
                # after the projection the chosen point is on tool i's surface
                sd = np.zeros(1)
                O.lib().oracle_tool_sdf(ctypes_ref(o.tools[i]), O.ptr(pseq[j + 1, i].copy()), 1,
                                        O.ptr(coll[j, c, 1:].copy()), O.ptr(sd), None)
                assert abs(sd[0]) < 1e-6, (j, c, sd)


def test_collision_projection_adjoint_matches_finite_differences():
    """The kinematics adjoint with projections (evaluated, as the reference's
    autodiff does, at the projected poses) against central differences.  For
    translations and the gripper gap of box-shaped tools the normal is constant
    on a face and that evaluation is exact; with rotations the SDF's lever arm
    at the projected position differs from the pre-projection one, so the
    rotation actions are switched off here (the GPU tests compare those with
    the oracle's reference semantics instead)."""
    tools = collision_tools()
    for t in tools:
        sc7 = list(t.action.scale) + [0.0] * (7 - len(t.action.scale))
        sc7[3:6] = [0.0, 0.0, 0.0]
        t.action.scale = tuple(sc7[:max(int(t.action.dim), 0)])
    sc = small_scene(n=10, substeps=5, tools=tools, precision="fp64")
    o = O.Oracle(sc.sim, tools)
    a = sc.actions[0]
    rng = np.random.default_rng(9)
    W = rng.normal(size=(sc.sim.n_substeps + 1, o.T, 8))

    def f(act):
        return float((W * o.tools_action(o.pose0(), act)[2]).sum())

    acts, vel, pseq = o.tools_action(o.pose0(), a)
    assert (o.last_coll[:, :, 0] >= 0).any()
    gp = W.copy()
    ga = np.zeros((o.T, 7))
    o.tools_action_bwd(acts, vel, pseq, o.last_coll, gp, ga)
    flat = np.concatenate([ga[i, :o.dims[i + 1] - o.dims[i]] for i in range(o.T)])
    for k in range(len(a)):
        fds = _fd_best(f, a, k, (1e-6, 1e-7))
        best = min(abs(v - flat[k]) / max(abs(v), 1e-6) for v in fds)
        assert best < 1e-5, (k, flat[k], fds)


# --------------------------------------------------------------------------
# particle-SDF renderer (tina/core/particle_sdf.py)
# --------------------------------------------------------------------------
def test_tina_camera_looks_at_its_center():
    from diffskill_gb300.render import tina_camera
    w2v, v2w = tina_camera((0.5, 0.0, 0.5), 0.0, -0.8, 0.88)
    c = w2v.astype(np.float64) @ np.array([0.5, 0.0, 0.5, 1.0])
    assert abs(c[0] / c[3]) < 1e-6 and abs(c[1] / c[3]) < 1e-6  # the center projects to the image center
    eye = v2w.astype(np.float64) @ np.array([0.0, 0.0, -1.0, 1.0])  # a point on the near plane
    eye = eye[:3] / eye[3]
    assert abs(np.linalg.norm(eye - np.array([0.5, 0.0, 0.5])) - (0.88 - 0.05)) < 1e-3
    assert np.allclose(np.linalg.inv(w2v.astype(np.float64)), v2w, atol=1e-4)


def test_render_bake_volume():
    """The baked SDF is the smoothed, quantised distance to the nearest particle:
    low around particles, 1 far away; the box starts 6 voxels below the particles."""
    rng = np.random.default_rng(1)
    x = np.array([0.5, 0.3, 0.5]) + rng.uniform(-0.05, 0.05, size=(400, 3))
    dx = 1 / 150
    sdf, color, bbox, over = O.render_bake(x, (48, 48, 48), 6, dx)
    assert over == 0
    assert np.allclose(bbox[0], (np.floor((x.astype(np.float32) * np.float32(150)).min(0)) - 6) * np.float32(dx))
    assert np.allclose(bbox[1], bbox[0] + 48 * dx, atol=1e-6)
    idx = ((x.astype(np.float32) - bbox[0]) * np.float32(150)).astype(int)
    v = sdf[tuple(idx.T)]  # 0.2 per voxel of distance (51 / 255), smoothed; particles ~2 voxels apart
    assert v.max() < 0.45 and np.median(v) < 0.3 and sdf[0, 0, 0] == 1.0 and sdf[47, 47, 47] == 1.0
    assert (color == 1.0).all()  # white particles, white empty voxels
    # an undersized volume is reported
    assert O.render_bake(x, (12, 12, 12), 6, dx)[3] == 1
