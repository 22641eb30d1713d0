"""Host runtime of the GB300 MPM substep.

``MpmEngine`` owns one C-ABI handle (include/mpm_gb300.h) for a batch of
independent scenes that share the grid resolution, time step and material.
State lives in torch CUDA tensors owned here; the library only receives raw
pointers and the current stream.

``Horizon`` runs a whole action sequence: forward with a checkpoint every
``k`` substeps, then the reverse sweep that recomputes each k-substep segment
from its checkpoint and applies the hand-written adjoint substep by substep.
This replaces the reference's store-every-frame fields (x, v, C, F of shape
``(max_steps, N)``, plb/engine/mpm_simulator.py:38-43) and its per-substep
``substep_grad`` (325-345), so long horizons fit in HBM.
"""
from __future__ import annotations

import ctypes
from typing import List, Optional, Sequence, Union

import numpy as np
import torch

from . import _lib
from .config import (PREC_FP64, TOOL_GRIPPER, PrimitiveConfig, SimulatorConfig, action_dims)

N_ROWS = 24  # x(3) v(3) C(9) F(9)


def _ptr(t: Optional[torch.Tensor]):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class MpmEngine:
    """Batched scenes on one GPU behind one library handle."""

    def __init__(self, sim: SimulatorConfig, tools_per_scene: Sequence[Sequence[PrimitiveConfig]],
                 n_per_scene: Sequence[int], softness: float = 666.0, device: Optional[torch.device] = None):
        if not torch.cuda.is_available():
            raise _lib.MpmError("diffskill_gb300 needs a CUDA device; there is no CPU path")
        self.lib = _lib.load()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.sim = sim
        self.prec = sim.precision_code
        self.dtype = torch.float64 if self.prec == PREC_FP64 else torch.float32
        self.S = len(n_per_scene)
        if len(tools_per_scene) != self.S:
            raise ValueError("tools_per_scene and n_per_scene must have one entry per scene")
        self.n_per_scene = [int(n) for n in n_per_scene]
        self.offsets = np.concatenate([[0], np.cumsum(self.n_per_scene)]).astype(np.int64)
        self.P = int(self.offsets[-1])
        self.ld = max(32, -(-self.P // 32) * 32)
        self.n_grid = sim.grid
        self.G = self.n_grid ** 3
        self.n_sub = sim.n_substeps
        self.softness = float(softness)

        p = _lib.MpmParams()
        p.abi_version = _lib.ABI_VERSION
        p.precision = self.prec
        p.n_grid = self.n_grid
        p.n_scenes = self.S
        p.n_particles = self.P
        p.ld = self.ld
        p.dx, p.inv_dx, p.dt, p.p_vol, p.p_mass = sim.dx, sim.inv_dx, sim.step_dt, sim.p_vol, sim.p_mass
        p.mu, p.lam, p.yield_stress = sim.mu, sim.lam, sim.yield_stress
        p.gravity[:] = [float(g) for g in sim.gravity]
        p.ground_friction = sim.ground_friction
        p.lower_bound = sim.lower_bound
        self.params = p
        offs = (ctypes.c_int64 * (self.S + 1))(*[int(o) for o in self.offsets])
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.mpm_create(ctypes.byref(p), offs, ctypes.byref(h)), None, "mpm_create")
        self.h = h

        # tools, sorted by scene
        self.tool_cfgs: List[PrimitiveConfig] = []
        self.tool_scene: List[int] = []
        self.scene_tools: List[List[int]] = []
        for s, tl in enumerate(tools_per_scene):
            idx = []
            for t in tl:
                idx.append(len(self.tool_cfgs))
                self.tool_cfgs.append(t)
                self.tool_scene.append(s)
            self.scene_tools.append(idx)
        self.T = len(self.tool_cfgs)
        descs = (_lib.MpmToolDesc * max(self.T, 1))()
        for i, (t, s) in enumerate(zip(self.tool_cfgs, self.tool_scene)):
            d = descs[i]
            d.type = t.type_code
            d.action_dim = int(t.action.dim)
            d.scene = s
            d.friction, d.softness = t.friction, self.softness
            d.radius, d.cap_h, d.cap_r = t.radius, t.h, t.r
            d.size[:] = list(t.size)
            d.prism_h[:] = list(t.prism_h)
            d.prot[:] = list(t.prot)
            d.min_gap, d.max_gap = t.minimal_gap, t.maximal_gap
            d.lower[:] = list(t.lower_bound)
            d.upper[:] = list(t.upper_bound)
            d.action_scale[:] = list(t.scale7())
            d.torus[:] = [t.tx, t.ty]
            d.collision_mask = t.collision_mask
        self._descs = descs
        with torch.cuda.device(self.device):
            _lib.check(self.lib.mpm_set_tools(self.h, descs, self.T), self.h, "mpm_set_tools")
            self.n_pairs = int(self.lib.mpm_collision_pairs(self.h))
            if self.n_pairs:
                # rand_num of the collision projection: np.random.seed(42) then
                # uniform(-1.5, 1.5, (n_pairs, 600, 3)) (mpm_simulator.py:89-96);
                # a scene's pair c uses row c of the same stream
                most = max(sum(bin(self.tool_cfgs[i].collision_mask).count("1") for i in idx)
                           for idx in self.scene_tools)
                pts = np.ascontiguousarray(np.random.RandomState(42).uniform(-1.5, 1.5, (most, 600, 3)))
                _lib.check(self.lib.mpm_set_collision_points(self.h, pts.ctypes.data_as(ctypes.c_void_p), most),
                           self.h, "mpm_set_collision_points")
        self.scene_action_dims = [action_dims([self.tool_cfgs[i] for i in idx]) for idx in self.scene_tools]
        self.pose0 = torch.tensor([list(t.init_state) for t in self.tool_cfgs] or np.zeros((0, 8)),
                                  dtype=torch.float64, device=self.device).reshape(self.T, 8)
        self.ds = torch.empty(max(2 * self.T, 2), dtype=torch.float64, device=self.device)  # contact sums

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and self.lib is not None:
            try:
                self.lib.mpm_destroy(h)
            except Exception:
                pass
            self.h = None

    # ------------------------------------------------------------------ state
    def new_state(self) -> torch.Tensor:
        return torch.zeros((N_ROWS, self.ld), dtype=self.dtype, device=self.device)

    def init_state(self, xs: Sequence[np.ndarray]) -> torch.Tensor:
        """``reset_kernel`` (mpm_simulator.py:402-409): x given, v=0, F=I, C=0."""
        st = self.new_state()
        x = np.concatenate([np.asarray(a, dtype=np.float64).reshape(-1, 3) for a in xs])
        if x.shape[0] != self.P:
            raise ValueError(f"expected {self.P} particles, got {x.shape[0]}")
        st[0:3, :self.P] = torch.as_tensor(x.T, dtype=self.dtype, device=self.device)
        st[15, :] = 1
        st[19, :] = 1
        st[23, :] = 1
        return st

    def expand_actions(self, actions_per_scene: Sequence[np.ndarray] | torch.Tensor) -> torch.Tensor:
        """[A, action_dim_s] per scene (reference flat layout) -> [A, T, 8], clipped to [-1, 1]."""
        if isinstance(actions_per_scene, torch.Tensor) and actions_per_scene.dim() == 3 \
                and actions_per_scene.shape[1:] == (self.T, 8):
            return actions_per_scene.to(torch.float64).clamp(-1, 1).contiguous()
        A = int(np.asarray(actions_per_scene[0]).shape[0]) if self.S else 0
        out = torch.zeros((A, self.T, 8), dtype=torch.float64, device=self.device)
        for s, idx in enumerate(self.scene_tools):
            a = torch.as_tensor(np.asarray(actions_per_scene[s], dtype=np.float64), device=self.device).reshape(A, -1)
            a = a.clamp(-1, 1)
            dims = self.scene_action_dims[s]
            for j, t in enumerate(idx):
                d = dims[j + 1] - dims[j]
                out[:, t, :d] = a[:, dims[j]:dims[j + 1]]
        return out

    def collapse_action_grad(self, g: torch.Tensor) -> List[torch.Tensor]:
        """[A, T, 8] -> per scene [A, action_dim_s] (reference flat layout)."""
        out = []
        for s, idx in enumerate(self.scene_tools):
            dims = self.scene_action_dims[s]
            parts = [g[:, t, :dims[j + 1] - dims[j]] for j, t in enumerate(idx)]
            out.append(torch.cat(parts, dim=1) if parts else g.new_zeros((g.shape[0], 0)))
        return out

    # -------------------------------------------------------------- C calls
    def new_coll(self, n_actions: int = 1) -> Optional[torch.Tensor]:
        """[n_actions, n_sub, n_pairs, 4] collision records (None without collision pairs)."""
        if not self.n_pairs:
            return None
        return torch.zeros((n_actions, self.n_sub, self.n_pairs, 4), dtype=torch.float64, device=self.device)

    def tools_action(self, action: torch.Tensor, vel: torch.Tensor, pose: torch.Tensor,
                     coll: Optional[torch.Tensor] = None) -> None:
        if self.n_pairs and coll is None:
            raise ValueError("this scene batch has tool-tool collision pairs: pass a collision record (new_coll)")
        _lib.check(self.lib.mpm_tools_action(self.h, _ptr(action), _ptr(vel), _ptr(pose), _ptr(coll), self.n_sub,
                                             _stream()), self.h, "mpm_tools_action")

    def tools_action_bwd(self, vel, pose, g_pose, g_action, coll: Optional[torch.Tensor] = None) -> None:
        if self.n_pairs and coll is None:
            raise ValueError("this scene batch has tool-tool collision pairs: pass the forward's collision record")
        _lib.check(self.lib.mpm_tools_action_bwd(self.h, _ptr(vel), _ptr(pose), _ptr(coll), _ptr(g_pose),
                                                 _ptr(g_action), self.n_sub, _stream()), self.h,
                   "mpm_tools_action_bwd")

    def set_chained(self, on: bool) -> None:
        """Chained forward substeps (``mpm_set_chained``): each forward substep's
        g2p flags the grid blocks of its output, and the next forward substep on
        that frame skips its marking pass.  Only frames left unmodified between
        substeps (up to the per-scene re-sort) may be chained."""
        _lib.check(self.lib.mpm_set_chained(self.h, 1 if on else 0), self.h, "mpm_set_chained")

    def set_pipelined_adjoint(self, on: bool) -> None:
        """Pipelined adjoint substeps: each adjoint substep's grid preparation runs
        on an internal stream beside the previous substep's p2g.grad.  Only
        between adjoint substeps with no forward substep in between."""
        _lib.check(self.lib.mpm_set_pipelined_adjoint(self.h, 1 if on else 0), self.h, "mpm_set_pipelined_adjoint")

    def substep(self, st0, st1, pose_f, pose_f1, store: "GridStore" = None, slot: int = -1) -> None:
        if store is None:
            _lib.check(self.lib.mpm_substep_fwd(self.h, _ptr(st0), _ptr(st1), _ptr(pose_f), _ptr(pose_f1),
                                                _stream()), self.h, "mpm_substep_fwd")
        else:
            _lib.check(self.lib.mpm_substep_fwd_store(self.h, _ptr(st0), _ptr(st1), _ptr(pose_f), _ptr(pose_f1),
                                                      ctypes.byref(store.struct), slot, _stream()), self.h,
                       "mpm_substep_fwd_store")

    def substep_bwd(self, st0, g1, g0, pose_f, pose_f1, gp_f, gp_f1, store: "GridStore" = None,
                    slot: int = -1, st1: Optional[torch.Tensor] = None) -> None:
        """Adjoint of one substep; ``st1`` (frame f+1 from the forward) is optional."""
        if store is None:
            _lib.check(self.lib.mpm_substep_bwd(self.h, _ptr(st0), _ptr(st1), _ptr(g1), _ptr(g0), _ptr(pose_f),
                                                _ptr(pose_f1), _ptr(gp_f), _ptr(gp_f1), _stream()), self.h,
                       "mpm_substep_bwd")
        else:
            _lib.check(self.lib.mpm_substep_bwd_store(self.h, _ptr(st0), _ptr(st1), _ptr(g1), _ptr(g0), _ptr(pose_f),
                                                      _ptr(pose_f1), _ptr(gp_f), _ptr(gp_f1),
                                                      ctypes.byref(store.struct), slot, _stream()), self.h,
                       "mpm_substep_bwd_store")

    def sort_frame(self, src: torch.Tensor, dst: torch.Tensor, perm: torch.Tensor) -> None:
        """dst = src with its particles sorted by (scene, 4^3 block, cell), stably;
        ``perm`` (int32 [P]) receives the order: dst[:, i] = src[:, perm[i]]."""
        _lib.check(self.lib.mpm_sort_frame(self.h, _ptr(src), _ptr(dst), _ptr(perm), _stream()), self.h,
                   "mpm_sort_frame")

    def unsort_frame(self, g_src: torch.Tensor, g_dst: torch.Tensor, perm: torch.Tensor) -> None:
        """Adjoint of ``sort_frame`` on a frame gradient: g_dst[:, perm[i]] = g_src[:, i]."""
        _lib.check(self.lib.mpm_unsort_frame(self.h, _ptr(g_src), _ptr(g_dst), _ptr(perm), _stream()), self.h,
                   "mpm_unsort_frame")

    def grid_mass(self, st: torch.Tensor, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        if out is None:
            out = torch.empty((self.S, self.G), dtype=self.dtype, device=self.device)
        _lib.check(self.lib.mpm_grid_mass(self.h, _ptr(st), _ptr(out), _stream()), self.h, "mpm_grid_mass")
        return out

    def grid_mass_bwd(self, st, g_gm, g_st) -> None:
        _lib.check(self.lib.mpm_grid_mass_bwd(self.h, _ptr(st), _ptr(g_gm), _ptr(g_st), _stream()), self.h,
                   "mpm_grid_mass_bwd")

    def density_l1(self, gm, target, weight: float = 1.0, g_gm=None) -> torch.Tensor:
        loss = torch.empty(self.S, dtype=torch.float64, device=self.device)
        _lib.check(self.lib.mpm_density_l1(self.h, _ptr(gm), _ptr(target), float(weight), _ptr(loss), _ptr(g_gm),
                                           _stream()), self.h, "mpm_density_l1")
        return loss

    def soft_contact(self, st, pose) -> tuple:
        md = torch.empty(max(self.T, 1), dtype=torch.float64, device=self.device)
        sums = torch.empty((max(self.T, 1), 2), dtype=torch.float64, device=self.device)
        _lib.check(self.lib.mpm_soft_contact(self.h, _ptr(st), _ptr(pose), _ptr(sums), _ptr(md), _stream()),
                   self.h, "mpm_soft_contact")
        return md[:self.T], sums

    def soft_contact_bwd(self, st, pose, sums, g_md, g_st, g_pose) -> None:
        _lib.check(self.lib.mpm_soft_contact_bwd(self.h, _ptr(st), _ptr(pose), _ptr(sums), _ptr(g_md), _ptr(g_st),
                                                 _ptr(g_pose), _stream()), self.h, "mpm_soft_contact_bwd")

    def target_sdf(self, density: torch.Tensor, n_iters: Optional[int] = None) -> tuple:
        """``Loss.update_target`` (loss.py:129-134) on [S, G] target densities:
        returns (target_sdf [S, G], nearest [S, G, 3]); ``n_iters`` defaults to
        the reference's 2 * n_grid."""
        n_iters = 2 * self.n_grid if n_iters is None else int(n_iters)
        density = density.to(self.device, self.dtype).contiguous()
        # (with n_iters = 0 they stay as a fresh taichi field starts: zero)
        sdf = torch.zeros((self.S, self.G), dtype=self.dtype, device=self.device)
        near = torch.zeros((self.S, self.G, 3), dtype=self.dtype, device=self.device)
        work = torch.empty((self.S, self.G, 4), dtype=self.dtype, device=self.device)
        _lib.check(self.lib.mpm_target_sdf(self.h, _ptr(density), _ptr(sdf), _ptr(near), _ptr(work), n_iters,
                                           _stream()), self.h, "mpm_target_sdf")
        return sdf, near

    def sdf_loss(self, gm, target_sdf, weight: float = 1.0, g_gm=None) -> torch.Tensor:
        """[S] weight * sum target_sdf * grid_m; adds weight * target_sdf to ``g_gm``."""
        loss = torch.empty(self.S, dtype=torch.float64, device=self.device)
        _lib.check(self.lib.mpm_sdf_loss(self.h, _ptr(gm), _ptr(target_sdf), float(weight), _ptr(loss), _ptr(g_gm),
                                         _stream()), self.h, "mpm_sdf_loss")
        return loss

    def iou(self, gm, target) -> torch.Tensor:
        """[S] ``iou_kernel`` (loss.py:294-308) of each scene's grid mass and target."""
        out = torch.empty(self.S, dtype=torch.float64, device=self.device)
        _lib.check(self.lib.mpm_iou(self.h, _ptr(gm), _ptr(target), _ptr(out), _stream()), self.h, "mpm_iou")
        return out

    def contact_min_dist(self, st, pose) -> tuple:
        """Hard contact distance of every tool: (min_dist [T] double, argmin [T] int64)."""
        md = torch.empty(max(self.T, 1), dtype=torch.float64, device=self.device)
        am = torch.full((max(self.T, 1),), -1, dtype=torch.int64, device=self.device)
        _lib.check(self.lib.mpm_contact_min_dist(self.h, _ptr(st), _ptr(pose), _ptr(md), _ptr(am), _stream()),
                   self.h, "mpm_contact_min_dist")
        return md[:self.T], am

    def contact_min_dist_bwd(self, st, pose, argmin, g_md, g_st, g_pose) -> None:
        g_md = g_md.to(self.device, torch.float64).contiguous()
        _lib.check(self.lib.mpm_contact_min_dist_bwd(self.h, _ptr(st), _ptr(pose), _ptr(argmin), _ptr(g_md),
                                                     _ptr(g_st), _ptr(g_pose), _stream()), self.h,
                   "mpm_contact_min_dist_bwd")

    @property
    def n_dist_cols(self) -> int:
        return int(self.lib.mpm_tool_distance_cols(self.h))

    def tool_distance(self, st, pose, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """[n_cols, ld] per-particle tool SDFs (Gripper: two finger columns)."""
        if out is None:
            out = torch.empty((max(self.n_dist_cols, 1), self.ld), dtype=self.dtype, device=self.device)
        _lib.check(self.lib.mpm_tool_distance(self.h, _ptr(st), _ptr(pose), _ptr(out), _stream()), self.h,
                   "mpm_tool_distance")
        return out

    def tool_distance_bwd(self, st, pose, g_out, g_st, g_pose) -> None:
        _lib.check(self.lib.mpm_tool_distance_bwd(self.h, _ptr(st), _ptr(pose), _ptr(g_out), _ptr(g_st),
                                                  _ptr(g_pose), _stream()), self.h, "mpm_tool_distance_bwd")

    def status(self, clear: bool = True) -> int:
        v = ctypes.c_uint32(0)
        _lib.check(self.lib.mpm_status(self.h, ctypes.byref(v), int(clear), _stream()), self.h, "mpm_status")
        return int(v.value)

    def check_status(self) -> None:
        st = self.status(clear=True)
        if st & _lib.STATUS_NONFINITE:
            raise FloatingPointError("MPM substep produced a NaN/Inf (device status word)")
        if st & _lib.STATUS_OUT_OF_GRID:
            raise _lib.MpmError("a particle stencil left the grid; its scatter was skipped")

    @property
    def launches(self) -> int:
        return int(self.lib.mpm_launch_count(self.h))

    def profile(self, enable: bool) -> None:
        """Bracket every kernel with CUDA events (not inside graph capture)."""
        _lib.check(self.lib.mpm_profile_enable(self.h, int(enable)), self.h, "mpm_profile_enable")

    def profile_read(self) -> dict:
        """{kind: (total device ms, launches)} since the last read."""
        n = len(_lib.KERNEL_KINDS)
        ms = (ctypes.c_double * n)()
        cnt = (ctypes.c_int64 * n)()
        _lib.check(self.lib.mpm_profile_read(self.h, ms, cnt), self.h, "mpm_profile_read")
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(_lib.KERNEL_KINDS)}

    # ------------------------------------------------------------- helpers
    def targets(self, grids: Sequence[np.ndarray]) -> torch.Tensor:
        return torch.as_tensor(np.stack([np.asarray(g, dtype=np.float64).reshape(-1) for g in grids]),
                               dtype=self.dtype, device=self.device).contiguous()

    def scene_slice(self, s: int) -> slice:
        return slice(int(self.offsets[s]), int(self.offsets[s + 1]))


class GridStore:
    """Caller-owned arena of forward-grid blocks (``MpmGridStore`` of the C ABI).

    Substeps whose forward grids are stored skip the p2g and grid_op
    recomputes in their adjoint; a substep that does not fit is recomputed
    (same result).
    """

    def __init__(self, eng: MpmEngine, n_slots: int, capacity_blocks: int):
        dev = eng.device
        self.capacity = int(max(capacity_blocks, 0))
        # per stored block: the p2g grid block, then the grid_op output block
        self.blocks = torch.empty((max(self.capacity, 1), 2, 64, 4), dtype=eng.dtype, device=dev)
        self.block_ids = torch.empty(max(self.capacity, 1), dtype=torch.int32, device=dev)
        self.slot_start = torch.full((n_slots,), -1, dtype=torch.int64, device=dev)
        self.slot_count = torch.zeros(n_slots, dtype=torch.int32, device=dev)
        self.bump = torch.zeros(1, dtype=torch.int64, device=dev)
        st = _lib.MpmGridStore()
        st.blocks = self.blocks.data_ptr()
        st.block_ids = self.block_ids.data_ptr()
        st.slot_start = self.slot_start.data_ptr()
        st.slot_count = self.slot_count.data_ptr()
        st.bump = self.bump.data_ptr()
        st.capacity = self.capacity
        st.n_slots = int(n_slots)
        self.struct = st

    def reset(self) -> None:
        """Forget every slot (device-side; capturable)."""
        self.bump.zero_()
        self.slot_start.fill_(-1)

    def bytes(self) -> int:
        return sum(t.numel() * t.element_size() for t in (self.blocks, self.block_ids, self.slot_start,
                                                           self.slot_count, self.bump))

    def stored_slots(self) -> int:
        return int((self.slot_start >= 0).sum())


def horizon_frames(n_frames: int, k: int) -> int:
    """State frames a horizon of ``n_frames`` substeps holds at checkpoint interval ``k``:
    the checkpoints (``n_frames / k + 1``) and the recompute segment (``max(k, 2)``)."""
    return n_frames // k + 1 + max(k, 2)


def plan_checkpoint_interval(n_frames: int, frame_bytes: int, budget_bytes: int, fixed_bytes: int = 0) -> int:
    """Checkpoint interval for a horizon of ``n_frames`` substeps under a memory budget.

    The reference stores every frame (``max_steps`` frames of every field,
    mpm_simulator.py:40-43) or, in its long-horizon notebook, checkpoints at a
    hand-picked interval and recomputes (plb/optimizer/long_term_gradient.ipynb,
    cell 4).  Here the interval is chosen: at interval k the adjoint recomputes
    (k - 1) / k of the forward substeps, so the smallest divisor k of the
    horizon whose frames (``horizon_frames``) fit ``budget_bytes - fixed_bytes``
    is the fastest.  Raises ``MemoryError`` when no divisor fits.
    """
    if n_frames <= 0 or frame_bytes < 0:
        raise ValueError("the horizon needs at least one substep and a non-negative frame size")
    room = budget_bytes - fixed_bytes
    for k in range(1, n_frames + 1):
        if n_frames % k == 0 and horizon_frames(n_frames, k) * frame_bytes <= room:
            return k
    best = min((horizon_frames(n_frames, k), k) for k in range(1, n_frames + 1) if n_frames % k == 0)
    raise MemoryError(f"a horizon of {n_frames} substeps needs at least {best[0]} frames of {frame_bytes} B "
                      f"(interval {best[1]}), above the budget of {room} B")


class Horizon:
    """Device buffers and the forward/backward sweep over ``n_actions`` actions.

    ``ckpt_every`` = k: the state is kept every k substeps (k=1 keeps every
    frame, as the reference does); the backward pass recomputes each segment
    of k substeps from its checkpoint before running its adjoint.
    ``ckpt_every="auto"`` takes the smallest k whose frames fit
    ``frame_budget_bytes`` (default: 60 % of the free device memory; the grid
    store then takes a quarter of what is left), see
    ``plan_checkpoint_interval``.

    ``resort_every`` = R (a multiple of k; default one action rounded up to a
    multiple of k, 0 = never): at every R-th frame the particles of each scene
    are re-sorted by grid cell so the scatter and gather kernels keep their
    locality as the material deforms.  The adjoint applies the inverse
    permutation to the frame gradient at the same frames.  Losses and action
    gradients do not depend on the particle order.
    """

    def __init__(self, eng: MpmEngine, n_actions: int, ckpt_every: Union[int, str] = 10, store_grids: bool = True,
                 store_budget_bytes: Optional[int] = None, resort_every: Optional[int] = None,
                 frame_budget_bytes: Optional[int] = None):
        self.eng = eng
        self.A = int(n_actions)
        self.F = self.A * eng.n_sub
        if ckpt_every == "auto":
            if frame_budget_bytes is None:
                free, _ = torch.cuda.mem_get_info(eng.device)
                frame_budget_bytes = int(free * 0.6)
            frame_bytes = N_ROWS * eng.ld * (8 if eng.dtype == torch.float64 else 4)
            ckpt_every = plan_checkpoint_interval(self.F, frame_bytes, frame_budget_bytes)
        k = int(ckpt_every) if ckpt_every else eng.n_sub
        if self.F % k != 0:
            raise ValueError(f"checkpoint interval {k} must divide the horizon of {self.F} substeps")
        self.k = k
        dev, dt = eng.device, eng.dtype
        self.n_ckpt = self.F // k + 1
        self.ckpt = torch.zeros((self.n_ckpt, N_ROWS, eng.ld), dtype=dt, device=dev)
        self.seg = torch.zeros((max(k, 2), N_ROWS, eng.ld), dtype=dt, device=dev)
        T = max(eng.T, 1)
        self.pose = torch.zeros((self.F + 1, T, 8), dtype=torch.float64, device=dev)
        self.vel = torch.zeros((self.F, T, 8), dtype=torch.float64, device=dev)
        self.acts = torch.zeros((self.A, T, 8), dtype=torch.float64, device=dev)
        self.g_pose = torch.zeros_like(self.pose)
        self.g_act = torch.zeros_like(self.acts)
        # the tool kinematics (one warp per scene, serial over substeps) run on
        # a side stream, overlapped with the MPM substeps that do not need them
        self.side = torch.cuda.Stream(device=dev)
        self.coll = eng.new_coll(self.A)
        self.g = torch.zeros((2, N_ROWS, eng.ld), dtype=dt, device=dev)
        self.gm = torch.zeros((eng.S, eng.G), dtype=dt, device=dev)
        self.g_gm = torch.zeros_like(self.gm)
        # contact-term tables (built once: no host->device copy inside a CUDA graph)
        self.movable = torch.tensor([float(t.action.dim > 0) for t in eng.tool_cfgs] or [0.0],
                                    dtype=torch.float64, device=dev)[:eng.T]
        self.tool_scene = torch.tensor(eng.tool_scene or [0], dtype=torch.long, device=dev)[:eng.T]
        # forward-grid store: every substep when every frame is kept (k == 1), else one segment
        self.store = None
        if store_grids:
            n_slots = self.F if k == 1 else k
            block_bytes = 2 * 64 * 4 * (8 if dt == torch.float64 else 4) + 4
            if store_budget_bytes is None:
                free, _ = torch.cuda.mem_get_info(dev)
                store_budget_bytes = free // 4
            worst = n_slots * eng.S * (eng.n_grid // 4) ** 3
            self.store = GridStore(eng, n_slots, min(worst, store_budget_bytes // block_bytes))
        # periodic re-sorting of the particles by cell
        self.perms = None
        self.set_resort_every(k * (-(-eng.n_sub // k)) if resort_every is None else resort_every)
        counts = torch.as_tensor(np.diff(eng.offsets), device=dev)
        self.pscene = torch.repeat_interleave(torch.arange(eng.S, device=dev), counts)
        self.pscene32 = self.pscene.to(torch.int32)
        # the frame a substep writes before it is re-sorted into its checkpoint
        self._tmp = torch.empty((N_ROWS, eng.ld), dtype=dt, device=dev)
        self._perm_tmp = torch.empty(max(eng.P, 1), dtype=torch.int32, device=dev)

    def set_resort_every(self, resort_every: int) -> None:
        """Re-sort the particles by cell every ``resort_every`` substeps (a
        multiple of the checkpoint interval; 0 = never).  Takes effect from
        the next ``forward``; do not change it between a forward and its
        backward, nor after a CUDA graph captured them."""
        R = int(resort_every)
        if R < 0 or (R and R % self.k != 0):
            raise ValueError(f"resort_every ({R}) must be 0 or a multiple of the checkpoint interval ({self.k})")
        self.R = R if 0 < R < self.F else 0
        self.boundaries = list(range(self.R, self.F, self.R)) if self.R else []
        need = (max(len(self.boundaries), 1), max(self.eng.P, 1))
        if self.perms is None or self.perms.shape[0] < need[0]:
            self.perms = torch.zeros(need, dtype=torch.int32, device=self.eng.device)

    def bytes(self) -> int:
        return sum(t.numel() * t.element_size() for t in
                   (self.ckpt, self.seg, self.pose, self.vel, self.g, self.gm, self.g_gm, self.g_pose)) + (
                       self.store.bytes() if self.store is not None else 0)

    @property
    def final(self) -> torch.Tensor:
        return self.ckpt[self.n_ckpt - 1]

    def sort_frame(self, frame: torch.Tensor) -> None:
        """Sort the particles of ``frame`` by (scene, 4^3 block, cell) in place, on
        the device (an initial state: losses and action gradients do not depend
        on the particle order)."""
        if self.eng.P == 0:
            return
        self._tmp.copy_(frame)
        self.eng.sort_frame(self._tmp, frame, self._perm_tmp)

    def forward(self, state0: torch.Tensor, actions: torch.Tensor, pose0: Optional[torch.Tensor] = None,
                keep_grids: bool = True) -> None:
        """Run all actions: ``GradModel.forward_step`` for each action (function.py:166-175).

        ``keep_grids=False`` skips the grid store (a forward that no adjoint follows)."""
        eng, n = self.eng, self.eng.n_sub
        main = torch.cuda.current_stream()
        self.ckpt[0].copy_(state0)
        ready = []  # ready[s]: the poses of action s are computed
        if eng.T:
            self.pose[0].copy_(eng.pose0 if pose0 is None else pose0)
            self.acts.copy_(actions)
            # action s's kinematics run ahead on the side stream; the substeps of
            # action s wait for them only
            self.side.wait_stream(main)
            with torch.cuda.stream(self.side):
                for s in range(self.A):
                    eng.tools_action(self.acts[s], self.vel[s * n], self.pose[s * n],
                                     None if self.coll is None else self.coll[s])
                    ev = torch.cuda.Event()
                    ev.record(self.side)
                    ready.append(ev)
        store = self.store if (keep_grids and self.store is not None and self.k == 1) else None
        if store is not None:
            store.reset()
        cur = self.ckpt[0]
        # each frame goes unmodified (up to the re-sort, a permutation within
        # scenes) from one substep to the next: chain the substeps
        eng.set_chained(True)
        try:
            for f in range(self.F):
                if ready and f % n == 0:
                    main.wait_event(ready[f // n])
                if (f + 1) % self.k == 0:
                    nxt = self.ckpt[(f + 1) // self.k]
                else:
                    nxt = self.seg[(f + 1) % 2]
                if self.R and (f + 1) % self.R == 0 and f + 1 < self.F and eng.P:
                    # a re-sort boundary: the substep writes the scratch frame, which is
                    # sorted into the frame's place (the permutation kept for the adjoint)
                    eng.substep(cur, self._tmp, self.pose[f], self.pose[f + 1], store, f)
                    eng.sort_frame(self._tmp, nxt, self.perms[(f + 1) // self.R - 1])
                else:
                    eng.substep(cur, nxt, self.pose[f], self.pose[f + 1], store, f)
                cur = nxt
        finally:
            eng.set_chained(False)
        if ready:
            main.wait_stream(self.side)

    def loss(self, targets: torch.Tensor, density_weight: float = 1.0, contact_weight: float = 0.0,
             need_grad: bool = True) -> torch.Tensor:
        """Density L1 (loss.py:172-175) per scene + optional soft contact (143-167)."""
        eng = self.eng
        final = self.final
        eng.grid_mass(final, self.gm)
        loss = eng.density_l1(self.gm, targets, density_weight, self.g_gm if need_grad else None)
        g_final = self.g[0]
        if need_grad:
            g_final.zero_()
            eng.grid_mass_bwd(final, self.g_gm, g_final)
            self.g_pose.zero_()
            self._loss_grad_ready = True
        if contact_weight and eng.T:
            md, sums = eng.soft_contact(final, self.pose[self.F])
            movable = self.movable
            loss = loss.index_add(0, self.tool_scene, contact_weight * md * md * movable)
            if need_grad:
                g_md = (2 * contact_weight * md * movable).contiguous()
                eng.soft_contact_bwd(final, self.pose[self.F], sums, g_md, g_final, self.g_pose[self.F])
        return loss

    def backward(self, g_final: Optional[torch.Tensor] = None) -> torch.Tensor:
        """Reverse sweep; returns d loss / d actions as [A, T, 8] (float64).

        ``g_final`` defaults to the gradient left by ``loss`` (which also
        seeds the pose gradients of the contact term); with an explicit
        ``g_final`` and no preceding ``loss`` the pose gradients start at 0.
        """
        eng, n, k = self.eng, self.eng.n_sub, self.k
        cur = self.g[0]
        if g_final is not None:
            cur.copy_(g_final)
            if not getattr(self, "_loss_grad_ready", False):
                self.g_pose.zero_()
        elif not getattr(self, "_loss_grad_ready", False):
            raise RuntimeError("Horizon.backward needs g_final or a preceding loss(need_grad=True)")
        self._loss_grad_ready = False
        nxt = self.g[1]
        self.g_act.zero_()
        store = self.store
        main = torch.cuda.current_stream()
        if eng.T:
            self.side.wait_stream(main)
        pending = self.A - 1  # next action whose kinematics adjoint is due

        def tools_bwd_upto(first_frame: int) -> None:
            # every action whose substeps are all at or after first_frame has its
            # MPM adjoint complete: its kinematics adjoint runs on the side stream,
            # in descending action order, overlapped with the MPM adjoint of the
            # earlier actions (the shared boundary frame takes atomic adds)
            nonlocal pending
            if not eng.T:
                return
            while pending >= 0 and pending * n >= first_frame:
                ev = torch.cuda.Event()
                ev.record(main)
                self.side.wait_event(ev)
                with torch.cuda.stream(self.side):
                    s = pending
                    eng.tools_action_bwd(self.vel[s * n], self.pose[s * n], self.g_pose[s * n], self.g_act[s],
                                         None if self.coll is None else self.coll[s])
                pending -= 1

        # k == 1: no forward recompute between the adjoint substeps, so each one's
        # grid preparation may run beside the previous one's p2g.grad
        eng.set_pipelined_adjoint(k == 1)
        for c in range(self.F // k - 1, -1, -1):
            frames = [self.ckpt[c]]
            if store is not None and k > 1:
                store.reset()  # this segment's substeps are stored while they are recomputed
            for i in range(1, k):
                dst = self.seg[i]
                eng.substep(frames[-1], dst, self.pose[c * k + i - 1], self.pose[c * k + i], store,
                            i - 1 if store is not None else -1)
                frames.append(dst)
            for i in range(k - 1, -1, -1):
                f = c * k + i
                slot = -1 if store is None else (f if k == 1 else i)
                st1 = frames[i + 1] if i + 1 < k else self.ckpt[c + 1]
                if self.R and (f + 1) % self.R == 0 and f + 1 < self.F:
                    st1 = None  # frame f+1 was re-sorted after this substep produced it
                eng.substep_bwd(frames[i], cur, nxt, self.pose[f], self.pose[f + 1], self.g_pose[f],
                                self.g_pose[f + 1], store if slot >= 0 else None, slot, st1=st1)
                cur, nxt = nxt, cur
            f0 = c * k
            if self.R and f0 > 0 and f0 % self.R == 0 and eng.P:
                # the gradient of frame f0 back in the order substep f0 - 1 produced
                eng.unsort_frame(cur, nxt, self.perms[f0 // self.R - 1])
                cur, nxt = nxt, cur
            tools_bwd_upto(f0)
        tools_bwd_upto(0)
        eng.set_pipelined_adjoint(False)
        if eng.T:
            main.wait_stream(self.side)
        self.g_state0 = cur
        return self.g_act
