"""Tool API mirroring plb/engine/primitive (Primitive, Primitives).

Per-frame tool poses, per-substep velocities, the action buffer and all their
gradients live in FP64 device tensors owned by the simulator
(``MPMSimulator``); these classes are the reference-shaped views on them.

Differences from the reference, by design: ``set_action`` runs set_velocity
and the forward kinematics of all substeps of that action in one kernel
launch (``mpm_tools_action``) -- tool kinematics do not depend on the
particles, so this equals the reference's per-substep ``forward_kinematics``;
``set_velocity_grad`` likewise runs the kinematics adjoint of a whole action.
"""
from __future__ import annotations

from typing import List, Optional, Sequence

import numpy as np

from .config import PrimitiveConfig, make_primitive


class Primitive:
    """One tool (primive_base.py:12-329); ``index`` is its row in the tool tables."""

    def __init__(self, cfg: PrimitiveConfig, index: int):
        self.cfg = cfg
        self.index = index
        self.sim = None  # bound by MPMSimulator
        self.softness_value = 666.0

    # -- reference attributes ------------------------------------------------
    @property
    def action_dim(self) -> int:
        return int(self.cfg.action.dim)

    @property
    def state_dim(self) -> int:
        return self.cfg.state_dim

    pos_dim = 3
    rotation_dim = 4

    @property
    def init_state(self):
        return tuple(self.cfg.init_state[:self.state_dim])

    # -- state (primive_base.py:164-191) ---------------------------------------
    def get_state(self, f: int) -> np.ndarray:
        p = self.sim._pose[f, self.index].cpu().numpy()
        return p[:self.state_dim].astype(np.float64)

    def get_state_tensor(self, f: int):
        return self.sim._pose[f, self.index, :self.state_dim].float()

    def set_state(self, f: int, state) -> None:
        state = np.asarray(state, dtype=np.float64).reshape(-1)
        cur = self.sim._pose[f, self.index].cpu().numpy()
        cur[:len(state)] = state
        self.sim._pose[f, self.index] = self.sim._t64(cur)

    # -- actions (primive_base.py:241-282) --------------------------------------
    def set_action(self, s: int, n_substeps: int, action) -> None:
        """Single-tool form of ``Primitives.set_action``."""
        if self.action_dim > 0:
            a = np.zeros(self.sim.primitives.action_dim)
            d = self.sim.primitives.action_dims
            a[d[self.index]:d[self.index + 1]] = np.asarray(action, dtype=np.float64).reshape(-1)[:self.action_dim]
            self.sim.primitives.set_action(s, n_substeps, a, only=self.index)

    def get_action_grad(self, s: int, n: int) -> Optional[np.ndarray]:
        if self.action_dim == 0:
            return None
        g = self.sim._g_act[s:s + n, self.index, :self.action_dim].cpu().numpy()
        return g.astype(np.float64)

    def set_velocity_grad(self, s: int, n_substeps: int) -> None:
        """``set_velocity.grad`` (+ forward_kinematics.grad) for action ``s``."""
        self.sim._tools_action_bwd(s)

    def sdf(self, f: int, points: np.ndarray) -> np.ndarray:
        """World SDF at frame ``f`` (Primitive.sdf / Gripper.sdf) for host points."""
        return self.sim.tool_sdf(self.index, f, points)


class Primitives:
    """Container (primitives.py:820-897)."""

    def __init__(self, cfgs: Sequence, max_timesteps: int = 1024):
        self.primitives: List[Primitive] = []
        self.action_dims = [0]
        for i, c in enumerate(cfgs):
            if isinstance(c, dict):
                c = dict(c)
                c = make_primitive(c.pop("shape"), **c)
            self.primitives.append(Primitive(c, i))
            self.action_dims.append(self.action_dims[-1] + self.primitives[-1].action_dim)
        self.n = len(self.primitives)
        self.sim = None

    @property
    def cfgs(self) -> List[PrimitiveConfig]:
        return [p.cfg for p in self.primitives]

    @property
    def action_dim(self) -> int:
        return self.action_dims[-1]

    @property
    def state_dim(self) -> int:
        return sum(p.state_dim for p in self.primitives)

    @property
    def state_dims(self):
        return [p.state_dim for p in self.primitives]

    def __getitem__(self, item):
        if isinstance(item, tuple):
            item = item[0]
        return self.primitives[item]

    def __len__(self) -> int:
        return self.n

    def __iter__(self):
        return iter(self.primitives)

    def set_action(self, s: int, n_substeps: int, action, only: Optional[int] = None) -> None:
        """Clip to [-1, 1] and run set_velocity + kinematics for action ``s`` (primitives.py:863-867)."""
        if isinstance(action, np.ndarray) or not hasattr(action, "detach"):
            action = np.asarray(action, dtype=np.float64).reshape(-1)
        else:
            action = action.detach().double().reshape(-1).cpu().numpy()
        if len(action) != self.action_dim:
            raise ValueError(f"action has {len(action)} entries, expected {self.action_dim}")
        if n_substeps != self.sim.substeps:
            raise ValueError("n_substeps must equal the simulator's substeps")
        self.sim._set_action(s, np.clip(action, -1, 1), only=only)

    def get_grad(self, n: int) -> np.ndarray:
        grads = [g for g in (p.get_action_grad(0, n) for p in self.primitives) if g is not None]
        return np.concatenate(grads, axis=1) if grads else np.zeros((n, 0))

    def set_softness(self, softness: float = 666.0) -> None:
        for p in self.primitives:
            p.softness_value = float(softness)
        if self.sim is not None:
            self.sim._set_softness(float(softness))

    def get_softness(self) -> float:
        return self.primitives[0].softness_value if self.primitives else 666.0

    def initialize(self) -> None:
        if self.sim is not None:
            for p in self.primitives:
                p.set_state(0, p.init_state)
