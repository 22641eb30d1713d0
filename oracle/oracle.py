"""ctypes wrapper of the FP64 CPU oracle (oracle/mpm_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline / reference legs, as the checker.  The product
package ``diffskill_gb300`` never imports this module.

Parity status: partially pinned (see the header of mpm_oracle.cpp): the
reference runtime (taichi 0.7.26) cannot run here, so the oracle is a line-by-
line restatement of plb/engine/mpm_simulator.py and plb/engine/primitive/*,
pinned against the reference's density assets and checked by finite
differences.

The trajectory driver follows ``GradModel.forward_step`` /
``GradModel.backward_step`` (plb/engine/function.py:166-190): actions are
clipped to [-1, 1], ``set_velocity`` spreads each action over the substeps of
that action, and the backward pass returns the gradient w.r.t. the (clipped)
action buffer.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import time
from typing import List, Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "mpm_oracle.cpp")
LIB = os.path.join(HERE, "liboracle_mpm.so")

_dp = ctypes.POINTER(ctypes.c_double)


class OracleSimStruct(ctypes.Structure):
    _fields_ = [("n_grid", ctypes.c_int32), ("pad0", ctypes.c_int32),
                ("dx", ctypes.c_double), ("inv_dx", ctypes.c_double), ("dt", ctypes.c_double),
                ("p_vol", ctypes.c_double), ("p_mass", ctypes.c_double),
                ("mu", ctypes.c_double), ("lam", ctypes.c_double), ("yield_stress", ctypes.c_double),
                ("gravity", ctypes.c_double * 3), ("ground_friction", ctypes.c_double),
                ("lower_bound", ctypes.c_double)]


class OracleToolStruct(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("action_dim", ctypes.c_int32),
                ("friction", ctypes.c_double), ("softness", ctypes.c_double),
                ("radius", ctypes.c_double), ("cap_h", ctypes.c_double), ("cap_r", ctypes.c_double),
                ("size", ctypes.c_double * 3), ("prism_h", ctypes.c_double * 2), ("prot", ctypes.c_double * 4),
                ("min_gap", ctypes.c_double), ("max_gap", ctypes.c_double),
                ("lower", ctypes.c_double * 3), ("upper", ctypes.c_double * 3),
                ("action_scale", ctypes.c_double * 7), ("torus", ctypes.c_double * 2),
                ("collision_mask", ctypes.c_int32), ("pad1", ctypes.c_int32)]


def build(force: bool = False, quiet: bool = True) -> str:
    """Compile the oracle with g++ (OpenMP).  Returns the library path."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    # -ffp-contract=off: every operation rounded on its own, on x86 and Arm alike
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-o", LIB + ".tmp", SRC]
    subprocess.run(cmd, check=True, capture_output=quiet)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.oracle_substep.restype = ctypes.c_int
        L.oracle_substep_bwd.restype = ctypes.c_int
        L.oracle_grid_mass.restype = ctypes.c_int
        L.oracle_grid_mass_bwd.restype = ctypes.c_int
        L.oracle_density_l1.restype = ctypes.c_double
        L.oracle_soft_contact.restype = ctypes.c_double
        L.oracle_num_threads.restype = ctypes.c_int
        L.oracle_soft_contact.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int64, _dp, ctypes.c_double, _dp, _dp]
        L.oracle_contact_min.restype = ctypes.c_double
        L.oracle_contact_min.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int64, _dp, ctypes.c_double, _dp, _dp,
                                         ctypes.POINTER(ctypes.c_int64)]
        L.oracle_collision_pairs.restype = ctypes.c_int
        L.oracle_render_bake.restype = ctypes.c_int
        L.oracle_render_bake.argtypes = [ctypes.c_int64, _dp, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                         ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_target_sdf_f64.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int, _dp, _dp, _dp]
        _fp = ctypes.POINTER(ctypes.c_float)
        L.oracle_target_sdf_f32.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int, _fp, _fp, _fp]
        _lib = L
    return _lib


def ptr(a: Optional[np.ndarray]):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"], (a.dtype, a.flags)
    return a.ctypes.data_as(_dp)


def set_num_threads(n: int) -> None:
    lib().oracle_set_num_threads(int(n))


def num_threads() -> int:
    return int(lib().oracle_num_threads())


def sim_struct(sim) -> OracleSimStruct:
    s = OracleSimStruct()
    s.n_grid = sim.grid
    s.dx, s.inv_dx, s.dt = sim.dx, sim.inv_dx, sim.step_dt
    s.p_vol, s.p_mass = sim.p_vol, sim.p_mass
    s.mu, s.lam, s.yield_stress = sim.mu, sim.lam, sim.yield_stress
    s.gravity[:] = [float(g) for g in sim.gravity]
    s.ground_friction = sim.ground_friction
    s.lower_bound = sim.lower_bound
    return s


def tool_struct(t, softness: float) -> OracleToolStruct:
    s = OracleToolStruct()
    s.type = t.type_code
    s.action_dim = int(t.action.dim)
    s.friction, s.softness = t.friction, softness
    s.radius, s.cap_h, s.cap_r = t.radius, t.h, t.r
    s.size[:] = list(t.size)
    s.prism_h[:] = list(t.prism_h)
    s.prot[:] = list(t.prot)
    s.min_gap, s.max_gap = t.minimal_gap, t.maximal_gap
    s.lower[:] = list(t.lower_bound)
    s.upper[:] = list(t.upper_bound)
    s.action_scale[:] = list(t.scale7())
    s.torus[:] = [t.tx, t.ty]
    s.collision_mask = t.collision_mask
    return s


def collision_points(n_pairs: int) -> np.ndarray:
    """rand_num of the collision projection (mpm_simulator.py:89-96):
    np.random.seed(42); uniform(-1.5, 1.5, (n_pairs, 600, 3))."""
    return np.ascontiguousarray(np.random.RandomState(42).uniform(-1.5, 1.5, (max(n_pairs, 1), 600, 3)))


def init_state(x0: np.ndarray) -> np.ndarray:
    """``reset_kernel`` (mpm_simulator.py:402-409): v=0, F=I, C=0."""
    n = x0.shape[0]
    st = np.zeros((n, 24), dtype=np.float64)
    st[:, 0:3] = x0
    st[:, 15] = st[:, 19] = st[:, 23] = 1.0
    return st


def target_sdf(density: np.ndarray, dx: float, n_iters: int, single: bool = False):
    """``update_target`` (loss.py:129-134, update_target_sdf 105-124) on one
    (n,n,n) target density; ``single`` rounds every operation to FP32 as the
    FP32 simulator does.  Returns (sdf (n,n,n), nearest (n,n,n,3))."""
    n = density.shape[0]
    dt = np.float32 if single else np.float64
    d = np.ascontiguousarray(density, dtype=dt)
    sdf = np.empty((n, n, n), dtype=dt)
    near = np.empty((n, n, n, 3), dtype=dt)
    if single:
        fp = ctypes.POINTER(ctypes.c_float)
        lib().oracle_target_sdf_f32(n, float(dx), int(n_iters), d.ctypes.data_as(fp), sdf.ctypes.data_as(fp),
                                    near.ctypes.data_as(fp))
    else:
        lib().oracle_target_sdf_f64(n, float(dx), int(n_iters), ptr(d), ptr(sdf), ptr(near))
    return sdf, near


def sdf_loss(grid_m: np.ndarray, target_sdf: np.ndarray):
    """``compute_sdf_loss_kernel`` (loss.py:178-180): sum target_sdf * grid_m,
    and its gradient w.r.t. grid_m (= target_sdf)."""
    return float(np.sum(np.asarray(target_sdf, np.float64) * np.asarray(grid_m, np.float64))), np.array(target_sdf)


def iou(grid_m: np.ndarray, target: np.ndarray) -> float:
    """``iou_kernel`` (loss.py:294-308): the maxima start at 0."""
    a = np.asarray(grid_m, np.float64).ravel()
    b = np.asarray(target, np.float64).ravel()
    ma, mb = max(0.0, float(a.max())), max(0.0, float(b.max()))
    inter = float(np.sum(a * b)) / ma / mb
    union = float(a.sum()) / ma + float(b.sum()) / mb
    return inter / (union - inter)


def render_bake(x: np.ndarray, res=(168, 168, 168), bake_size: int = 6, dx: float = 1 / 150, colors=None):
    """``plb_set_particles`` + ``build_sdf_from_particles`` (particle_sdf.py:548-568,
    237-265) in FP32: returns (sdf (res), color (res + (3,)), bbox (2, 3), over)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    r = np.asarray(res, dtype=np.int32)
    sdf = np.empty(tuple(res), dtype=np.float32)
    color = np.empty(tuple(res) + (3,), dtype=np.float32)
    bbox = np.empty(6, dtype=np.float32)
    cols = None if colors is None else np.ascontiguousarray(colors, dtype=np.uint32)
    over = lib().oracle_render_bake(x.shape[0], ptr(x), None if cols is None else cols.ctypes.data_as(ctypes.c_void_p),
                                    r.ctypes.data_as(ctypes.c_void_p), int(bake_size), float(dx),
                                    sdf.ctypes.data_as(ctypes.c_void_p), color.ctypes.data_as(ctypes.c_void_p),
                                    bbox.ctypes.data_as(ctypes.c_void_p))
    return sdf, color, bbox.reshape(2, 3), int(over)


def render_trace(sdf, color, bbox, v2w, w2v, img_res, sdf_threshold=0.37 * 0.56, tools=(), pose=None,
                 tool_color=None, show_particles=True, bias=(0.5, 0.5), softness=666.0):
    """``render_color`` + ``next_hit`` (particle_sdf.py:185-217, 353-440) per pixel, FP32:
    returns depth (rx, ry), normal, color, image (rx, ry, 3)."""
    rx, ry = img_res
    res = np.asarray(sdf.shape, dtype=np.int32)
    cam = np.concatenate([np.asarray(v2w, np.float32).ravel(), np.asarray(w2v, np.float32).ravel()])
    T = len(tools)
    arr = (OracleToolStruct * max(T, 1))()
    for i, t in enumerate(tools):
        arr[i] = tool_struct(t, softness)
    pose = np.zeros((max(T, 1), 8)) if pose is None else np.ascontiguousarray(pose, dtype=np.float64)
    tc = np.zeros((max(T, 1), 3), np.float32) if tool_color is None else np.ascontiguousarray(tool_color, np.float32)
    depth = np.empty((rx, ry), np.float32)
    nrm, col, img = (np.empty((rx, ry, 3), np.float32) for _ in range(3))
    vp = lambda a: np.ascontiguousarray(a).ctypes.data_as(ctypes.c_void_p)
    lib().oracle_render_trace(vp(np.ascontiguousarray(sdf, np.float32)), vp(np.ascontiguousarray(color, np.float32)),
                              vp(np.asarray(bbox, np.float32).ravel()), vp(res), ctypes.c_float(sdf_threshold),
                              vp(cam), int(rx), int(ry), ctypes.c_float(bias[0]), ctypes.c_float(bias[1]), arr, T,
                              ptr(pose), vp(tc), int(bool(show_particles)), vp(depth), vp(nrm), vp(col), vp(img))
    return depth, nrm, col, img


class Oracle:
    """Single-scene FP64 oracle of the substep chain."""

    def __init__(self, sim, tools: Sequence, softness: float = 666.0):
        self.cfg = sim
        self.sim = sim_struct(sim)
        self.tool_cfgs = list(tools)
        self.T = len(self.tool_cfgs)
        arr = (OracleToolStruct * max(self.T, 1))()
        for i, t in enumerate(self.tool_cfgs):
            arr[i] = tool_struct(t, softness)
        self.tools = arr
        self.n_sub = sim.n_substeps
        self.dims = [0]
        for t in self.tool_cfgs:
            self.dims.append(self.dims[-1] + int(t.action.dim))
        self.G = sim.grid ** 3
        self.n_pairs = int(lib().oracle_collision_pairs(self.tools, self.T))
        self.pts = collision_points(self.n_pairs)

    # -- tools ---------------------------------------------------------------
    def pose0(self) -> np.ndarray:
        return np.array([t.init_state for t in self.tool_cfgs], dtype=np.float64).reshape(self.T, 8)

    def expand_action(self, a: np.ndarray) -> np.ndarray:
        a = np.clip(np.asarray(a, dtype=np.float64).reshape(-1), -1, 1)
        out = np.zeros((self.T, 7), dtype=np.float64)
        for i in range(self.T):
            d = self.dims[i + 1] - self.dims[i]
            out[i, :d] = a[self.dims[i]:self.dims[i + 1]]
        return out

    def tools_action(self, pose_start: np.ndarray, a: np.ndarray):
        act = self.expand_action(a)
        vel = np.zeros((self.n_sub, self.T, 8))
        poses = np.zeros((self.n_sub + 1, self.T, 8))
        poses[0] = pose_start
        coll = np.zeros((self.n_sub, max(self.n_pairs, 1), 4))
        lib().oracle_tools_action(self.tools, self.T, self.n_sub, ptr(act), ptr(vel), ptr(poses), ptr(self.pts),
                                  ptr(coll))
        self.last_coll = coll  # collision records of this action, for tools_action_bwd
        return act, vel, poses

    def tools_action_bwd(self, act, vel, pseq, coll, g_pose_seq, g_act) -> None:
        """Adjoint of one action's kinematics: g_pose_seq [(n_sub+1)][T][8] in/out, g_act [T][7] accumulated."""
        lib().oracle_tools_action_bwd(self.tools, self.T, self.n_sub, ptr(act), ptr(vel), ptr(np.ascontiguousarray(pseq)),
                                      ptr(self.pts), ptr(coll), ptr(g_pose_seq), ptr(g_act))

    # -- substep -------------------------------------------------------------
    def substep(self, pose_f, pose_f1, state) -> np.ndarray:
        out = np.empty_like(state)
        rc = lib().oracle_substep(ctypes.byref(self.sim), self.tools, self.T, ptr(np.ascontiguousarray(pose_f)),
                                  ptr(np.ascontiguousarray(pose_f1)), state.shape[0], ptr(state), ptr(out))
        if rc != 0:
            raise RuntimeError("oracle_substep: a particle stencil left the grid")
        return out

    def substep_bwd(self, pose_f, pose_f1, state, g_next, g_pose_f, g_pose_f1) -> np.ndarray:
        g = np.empty_like(state)
        rc = lib().oracle_substep_bwd(ctypes.byref(self.sim), self.tools, self.T, ptr(np.ascontiguousarray(pose_f)),
                                      ptr(np.ascontiguousarray(pose_f1)), state.shape[0], ptr(state), ptr(g_next),
                                      ptr(g), ptr(g_pose_f), ptr(g_pose_f1))
        if rc != 0:
            raise RuntimeError("oracle_substep_bwd: a particle stencil left the grid")
        return g

    def grid_mass(self, state) -> np.ndarray:
        gm = np.zeros(self.G)
        rc = lib().oracle_grid_mass(ctypes.byref(self.sim), state.shape[0], ptr(state), ptr(gm))
        if rc != 0:
            raise RuntimeError("oracle_grid_mass: a particle stencil left the grid")
        return gm

    def grid_mass_bwd(self, state, g_gm, g_state) -> None:
        lib().oracle_grid_mass_bwd(ctypes.byref(self.sim), state.shape[0], ptr(state), ptr(g_gm), ptr(g_state))

    def soft_contact(self, t: int, pose, state, g_min: float = 0.0, g_state=None, g_pose=None) -> float:
        return lib().oracle_soft_contact(ctypes.byref(self.tools[t]), ptr(np.ascontiguousarray(pose)),
                                         state.shape[0], ptr(state), g_min, ptr(g_state), ptr(g_pose))

    def contact_min(self, t: int, pose, state, g_min: float = 0.0, g_state=None, g_pose=None):
        """Hard contact distance of tool t and its argmin particle (loss.py:151-155)."""
        am = ctypes.c_int64(-1)
        md = lib().oracle_contact_min(ctypes.byref(self.tools[t]), ptr(np.ascontiguousarray(pose)), state.shape[0],
                                      ptr(state), g_min, ptr(g_state), ptr(g_pose), ctypes.byref(am))
        return md, int(am.value)

    # -- trajectory ----------------------------------------------------------
    def rollout(self, x0: np.ndarray, actions: np.ndarray, keep_frames: bool = True):
        state = init_state(x0)
        frames: List[np.ndarray] = [state]
        pose = self.pose0()
        poses = [pose[None]]
        vels, acts, colls = [], [], []
        for a in actions:
            act, vel, pseq = self.tools_action(pose, a)
            acts.append(act)
            vels.append(vel)
            colls.append(self.last_coll)
            for j in range(self.n_sub):
                state = self.substep(pseq[j], pseq[j + 1], state)
                if keep_frames:
                    frames.append(state)
            pose = pseq[-1]
            poses.append(pseq[1:])
        if not keep_frames:
            frames = [frames[0], state]
        return dict(frames=frames, poses=np.concatenate(poses), vels=vels, acts=acts, colls=colls, final=state)

    def loss(self, final_state, target, poses_last=None, density_weight=1.0, contact_weight=0.0) -> float:
        gm = self.grid_mass(final_state)
        loss = density_weight * float(np.abs(gm - target).sum())
        if contact_weight:
            for t in range(self.T):
                if self.tool_cfgs[t].action.dim > 0:
                    md = self.soft_contact(t, poses_last[t], final_state)
                    loss += contact_weight * md * md
        return loss

    def loss_and_grad(self, x0, actions, target, density_weight=1.0, contact_weight=0.0, return_rollout=False):
        """Store-all-frames forward, loss, and reverse sweep; returns (loss, d loss / d actions)."""
        ro = self.rollout(x0, actions, keep_frames=True)
        frames, poses = ro["frames"], ro["poses"]
        final = frames[-1]
        F = len(frames) - 1
        gm = self.grid_mass(final)
        diff = gm - target
        loss = density_weight * float(np.abs(diff).sum())
        g_state = np.zeros_like(final)
        self.grid_mass_bwd(final, density_weight * np.sign(diff), g_state)
        g_pose = np.zeros((F + 1, self.T, 8))
        if contact_weight:
            for t in range(self.T):
                if self.tool_cfgs[t].action.dim > 0:
                    md = self.soft_contact(t, poses[F, t], final)
                    loss += contact_weight * md * md
                    gp = np.zeros(8)
                    self.soft_contact(t, poses[F, t], final, 2 * contact_weight * md, g_state, gp)
                    g_pose[F, t] += gp
        for f in range(F - 1, -1, -1):
            g_state = self.substep_bwd(poses[f], poses[f + 1], frames[f], g_state, g_pose[f], g_pose[f + 1])
        A = len(actions)
        g_act = np.zeros((A, self.T, 7))
        for s in range(A - 1, -1, -1):
            sl = g_pose[s * self.n_sub:(s + 1) * self.n_sub + 1]
            assert sl.flags["C_CONTIGUOUS"]
            pseq = np.ascontiguousarray(poses[s * self.n_sub:(s + 1) * self.n_sub + 1])
            self.tools_action_bwd(ro["acts"][s], ro["vels"][s], pseq, ro["colls"][s], sl, g_act[s])
        flat = np.zeros((A, self.dims[-1]))
        for i in range(self.T):
            d = self.dims[i + 1] - self.dims[i]
            flat[:, self.dims[i]:self.dims[i + 1]] = g_act[:, i, :d]
        out = (loss, flat)
        if return_rollout:
            out = out + (ro, g_state)
        return out


def time_fwd_bwd(scene, n_actions: int, threads: Optional[int] = None):
    """Time one store-all forward+backward of ``n_actions`` actions of ``scene``.

    Returns (seconds, particle_substeps) for the bench's CPU baseline.
    """
    if threads:
        set_num_threads(threads)
    o = Oracle(scene.sim, scene.tools)
    acts = scene.actions[:n_actions]
    t0 = time.perf_counter()
    o.loss_and_grad(scene.x0, acts, scene.target, scene.density_weight, scene.contact_weight)
    dt = time.perf_counter() - t0
    return dt, scene.n_particles * n_actions * o.n_sub
