"""Shared helpers for the parity tests (oracle <-> GPU layout conversion)."""
from __future__ import annotations

import numpy as np

from diffskill_gb300 import scenes
from diffskill_gb300.config import ActionConfig, PrimitiveConfig

# row groups of the 24-row particle state
GROUPS = {"x": slice(0, 3), "v": slice(3, 6), "C": slice(6, 15), "F": slice(15, 24)}


def perturbed_state(x0: np.ndarray, seed: int = 0, v=0.1, C=0.5, F=0.01) -> np.ndarray:
    """AoS (n, 24) state with velocities, affine fields and deformations."""
    rng = np.random.default_rng(seed)
    n = x0.shape[0]
    st = np.zeros((n, 24))
    st[:, 0:3] = x0
    st[:, 3:6] = rng.normal(size=(n, 3)) * v
    st[:, 6:15] = rng.normal(size=(n, 9)) * C
    st[:, 15:24] = np.eye(3).reshape(9) + rng.normal(size=(n, 9)) * F
    return st


def rel_err(a: np.ndarray, b: np.ndarray) -> float:
    """max |a-b| / max |b| (inf-norm relative error)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / den)


def group_errors(gpu_aos: np.ndarray, ref_aos: np.ndarray) -> dict:
    return {k: rel_err(gpu_aos[:, sl], ref_aos[:, sl]) for k, sl in GROUPS.items()}


def all_tools():
    """One tool of every type, placed to touch the dough of ``small_scene``."""
    rot6 = ActionConfig(dim=6, scale=(0.02, 0.02, 0.02, 0.05, 0.05, 0.05))
    return [
        scenes.sphere((0.42, 0.215, 0.5), radius=0.04, scale=0.02),
        PrimitiveConfig(shape="Capsule", init_pos=(0.5, 0.2, 0.45), init_rot=(0.707, 0.707, 0.0, 0.0), r=0.03,
                        h=0.2, action=rot6),
        PrimitiveConfig(shape="Box", init_pos=(0.58, 0.205, 0.5), init_rot=(0.9, 0.1, 0.3, 0.2),
                        size=(0.04, 0.01, 0.05), action=rot6),
        PrimitiveConfig(shape="Knife", init_pos=(0.5, 0.23, 0.56), size=(0.125, 0.075, 0.004),
                        prism_h=(0.15, 0.15), prot=(1.0, 0.0, 0.0, 0.58), friction=0.3, action=rot6),
        PrimitiveConfig(shape="Gripper", init_pos=(0.5, 0.15, 0.5), size=(0.01, 0.04, 0.04), init_gap=0.12,
                        minimal_gap=0.04, maximal_gap=0.3, friction=2.0, init_rot=(0.9, 0.1, 0.3, 0.2),
                        action=ActionConfig(dim=7, scale=(0.02, 0.02, 0.02, 0.05, 0.05, 0.05, 0.02))),
    ]


def small_scene(n: int = 2000, n_actions: int = 1, substeps: int = 10, tools=None, seed: int = 1001,
                precision: str = "fp64", dt: float = 1e-4):
    sc = scenes.config1(n_actions=n_actions, n_particles=n, dt=dt, substeps=substeps, seed=seed)
    sc.sim.precision = precision
    if tools is not None:
        sc.tools = list(tools)
        rng = np.random.default_rng(seed + 7)
        dims = sum(int(t.action.dim) for t in sc.tools)
        sc.actions = rng.uniform(-1, 1, size=(n_actions, dims))
    return sc


def more_tools():
    """One tool of each remaining shape (RollingPin, RollingPinExt, Chopsticks,
    Cylinder, Torus, Gripper2), placed to touch the dough of ``small_scene``."""
    rot6 = ActionConfig(dim=6, scale=(0.02, 0.02, 0.02, 0.05, 0.05, 0.05))
    return [
        PrimitiveConfig(shape="RollingPin", init_pos=(0.45, 0.22, 0.5), init_rot=(0.707, 0.707, 0.0, 0.0), h=0.2,
                        r=0.03, action=ActionConfig(dim=3, scale=(0.7, 0.02, 0.01))),
        PrimitiveConfig(shape="RollingPinExt", init_pos=(0.55, 0.22, 0.5), init_rot=(0.707, 0.707, 0.0, 0.0),
                        h=0.2, r=0.03, action=ActionConfig(dim=6, scale=(0.7, 0.02, 0.01, 0.01, 0.0, 0.0))),
        PrimitiveConfig(shape="Chopsticks", init_pos=(0.45, 0.25, 0.48), init_rot=(0.9, 0.1, 0.3, 0.2), h=0.12,
                        r=0.015, init_gap=0.07, minimal_gap=0.03,
                        action=ActionConfig(dim=7, scale=(0.02, 0.02, 0.02, 0.05, 0.05, 0.05, 0.02))),
        PrimitiveConfig(shape="Cylinder", init_pos=(0.56, 0.215, 0.45), init_rot=(0.9, 0.1, 0.3, 0.2), h=0.04,
                        r=0.02, action=rot6),
        PrimitiveConfig(shape="Torus", init_pos=(0.5, 0.21, 0.56), init_rot=(0.9, 0.1, 0.3, 0.2), tx=0.04, ty=0.015,
                        action=rot6),
        PrimitiveConfig(shape="Gripper2", init_pos=(0.5, 0.17, 0.5), init_rot=(0.9, 0.1, 0.3, 0.2), h=0.06, r=0.015,
                        init_gap=0.1, minimal_gap=0.04, maximal_gap=0.3, friction=2.0,
                        action=ActionConfig(dim=7, scale=(0.02, 0.02, 0.02, 0.05, 0.05, 0.05, 0.02))),
    ]


def collision_tools():
    """A gripper and a lifter box projected out of a static obstacle box
    (collision_group (0, 0, 1) as in plb/envs/gather_move.yml), overlapping it
    at the start so that the projection acts."""
    return [
        PrimitiveConfig(shape="Gripper", init_pos=(0.5, 0.215, 0.5), size=(0.01, 0.04, 0.04), init_gap=0.12,
                        minimal_gap=0.04, maximal_gap=0.3, friction=2.0, init_rot=(1.0, 0.0, 0.0, 0.0),
                        collision_group=(0, 0, 1),
                        action=ActionConfig(dim=7, scale=(0.02, 0.03, 0.02, 0.0, 0.05, 0.0, 0.02))),
        PrimitiveConfig(shape="Box", init_pos=(0.42, 0.21, 0.42), size=(0.03, 0.01, 0.03), friction=5.0,
                        collision_group=(0, 0, 1),
                        action=ActionConfig(dim=6, scale=(0.02, 0.03, 0.02, 0.0, 0.05, 0.0))),
        PrimitiveConfig(shape="Box", init_pos=(0.5, 0.16, 0.5), size=(0.12, 0.04, 0.12), friction=5.0,
                        action=ActionConfig(dim=0)),
    ]
