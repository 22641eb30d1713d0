"""Seeded synthetic workloads (the reference's datasets are not shipped).

The particle samplers restate plb/engine/shapes/shape_maker.py:
``add_box`` (81-91) draws ``(U[0,1)*2-1) * width/2 + centre`` and ``add_sphere``
(104-116) draws a normal direction scaled by ``U^(1/3) * r``.  Every workload
draws from ``numpy.random.default_rng(seed)`` so the oracle and the GPU path see
identical inputs.

Workloads (sizes from the project's benchmark definitions):

* ``config1``: FP64 single scene, 64^3, dt=5e-4, 10k particles, one capsule.
* ``config2``: single scene, 64^3, 30k particles, box spatula + capsule pin.
* ``config3``: 64 batched scenes, 5k-40k particles each, 1-3 tools each
  (every tool starts resting on a dough blob).
* ``config4``: 128^3 cutting/gripping scene, 100k particles, knife + gripper.
* ``config5``: 16 batched 128^3 scenes, 100k-500k particles, 3 tools each.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional, Union

import numpy as np

from .config import ActionConfig, PrimitiveConfig, SimulatorConfig, action_dims


@dataclass
class Scene:
    sim: SimulatorConfig
    tools: List[PrimitiveConfig]
    x0: np.ndarray                  # (N, 3) float64 initial positions
    target: np.ndarray              # (n_grid^3,) float64 target density grid
    actions: np.ndarray             # (n_actions, action_dim) float64 in [-1, 1]
    softness: float = 666.0
    density_weight: float = 1.0
    contact_weight: float = 0.0     # soft tool-contact term (loss.py:143-167)
    checkpoint_every: Union[int, str] = 10  # "auto": planned from the free device memory
    name: str = ""

    @property
    def n_particles(self) -> int:
        return int(self.x0.shape[0])

    @property
    def n_actions(self) -> int:
        return int(self.actions.shape[0])

    @property
    def action_dim(self) -> int:
        return action_dims(self.tools)[-1]


# ----------------------------------------------------------------------------
# samplers (shape_maker.py)
# ----------------------------------------------------------------------------
def sample_box(rng: np.random.Generator, n: int, centre, width) -> np.ndarray:
    width = np.asarray(width, dtype=np.float64)
    return (rng.random((n, 3)) * 2 - 1) * (0.5 * width) + np.asarray(centre, dtype=np.float64)


def sample_sphere(rng: np.random.Generator, n: int, centre, radius: float) -> np.ndarray:
    p = rng.normal(size=(n, 3))
    p /= np.linalg.norm(p, axis=-1, keepdims=True)
    u = rng.random((n, 1)) ** (1.0 / 3)
    return p * u * radius + np.asarray(centre, dtype=np.float64)


def density_grid(x: np.ndarray, n_grid: int, p_mass: float) -> np.ndarray:
    """Host-side density grid used only to build target inputs.

    Same quadratic B-spline stencil as ``compute_grid_m_kernel``
    (mpm_simulator.py:456-466); returns a flat C-order (n^3,) float64 array.
    """
    x = np.asarray(x, dtype=np.float64)
    inv_dx = float(n_grid)
    base = (x * inv_dx - 0.5).astype(np.int64)  # truncation toward zero
    fx = x * inv_dx - base
    w = [0.5 * (1.5 - fx) ** 2, 0.75 - (fx - 1) ** 2, 0.5 * (fx - 0.5) ** 2]
    out = np.zeros(n_grid ** 3, dtype=np.float64)
    ok = np.all((base >= 0) & (base + 2 < n_grid), axis=1)
    base, fx = base[ok], fx[ok]
    w = [wi[ok] for wi in w]
    for i in range(3):
        for j in range(3):
            for k in range(3):
                idx = ((base[:, 0] + i) * n_grid + base[:, 1] + j) * n_grid + base[:, 2] + k
                np.add.at(out, idx, w[i][:, 0] * w[j][:, 1] * w[k][:, 2] * p_mass)
    return out


def clip_particles(x: np.ndarray, sim: SimulatorConfig) -> np.ndarray:
    """Keep samples inside the simulated domain [lower_bound*dx, 1-3dx]."""
    lo, hi = sim.lower_bound * sim.dx, 1.0 - 3 * sim.dx
    return np.clip(x, lo, hi)


# ----------------------------------------------------------------------------
# tools
# ----------------------------------------------------------------------------
ROT_Y_TO_Z = (0.707, 0.707, 0.0, 0.0)  # rollingpin.yml:16 orientation


def capsule(pos, r=0.03, h=0.2, scale=0.005, rot=ROT_Y_TO_Z) -> PrimitiveConfig:
    return PrimitiveConfig(shape="Capsule", init_pos=tuple(pos), init_rot=tuple(rot), r=r, h=h, friction=0.9,
                           action=ActionConfig(dim=3, scale=(scale,) * 3))


def sphere(pos, radius=0.03, scale=0.005) -> PrimitiveConfig:
    return PrimitiveConfig(shape="Sphere", init_pos=tuple(pos), radius=radius, friction=0.9,
                           action=ActionConfig(dim=3, scale=(scale,) * 3))


def box(pos, size, scale=0.005, rot=(1.0, 0.0, 0.0, 0.0)) -> PrimitiveConfig:
    return PrimitiveConfig(shape="Box", init_pos=tuple(pos), init_rot=tuple(rot), size=tuple(size), friction=0.9,
                           action=ActionConfig(dim=3, scale=(scale,) * 3))


# ----------------------------------------------------------------------------
# workloads
# ----------------------------------------------------------------------------
def config1(n_actions: int = 10, n_particles: int = 10000, dt: float = 5e-4, substeps: int = 50,
            seed: int = 1001) -> Scene:
    """FP64 reference method, single scene, one capsule; density L1 to the dough shifted +0.1 in x."""
    sim = SimulatorConfig(E=5e3, nu=0.2, yield_stress=50.0, gravity=(0.0, -9.8, 0.0), n_grid=64, dt=dt,
                          substeps=substeps, dtype="float64", n_particles=n_particles)
    rng = np.random.default_rng(seed)
    x0 = sample_box(rng, n_particles, (0.5, 0.15, 0.5), (0.2, 0.1, 0.2))
    tools = [capsule((0.5, 0.23, 0.5), r=0.03, h=0.2, scale=0.005)]
    actions = rng.uniform(-1, 1, size=(n_actions, 3))
    target = density_grid(clip_particles(x0 + np.array([0.1, 0.0, 0.0]), sim), sim.grid, sim.p_mass)
    return Scene(sim, tools, clip_particles(x0, sim), target, actions, name="config1")


def config2(n_actions: int = 50, n_particles: int = 30000, substeps: int = 50, dt: Optional[float] = None,
            seed: int = 1002, precision: str = "fp32") -> Scene:
    """Single scene, FP32 adjoint: box spatula + capsule pin flatten a slab."""
    sim = SimulatorConfig(E=5e3, nu=0.2, yield_stress=50.0, gravity=(0.0, -9.8, 0.0), n_grid=64, dt=dt,
                          substeps=substeps, precision=precision, n_particles=n_particles)
    rng = np.random.default_rng(seed)
    x0 = sample_box(rng, n_particles, (0.5, 0.09, 0.5), (0.25, 0.08, 0.25))
    # both tools rest on the slab top (y = 0.13), pressing 3 mm into it
    tools = [box((0.5, 0.1295, 0.5), (0.075, 0.0025, 0.075)),
             capsule((0.3, 0.157, 0.5), r=0.03, h=0.25)]
    actions = rng.uniform(-1, 1, size=(n_actions, 6))
    tx = sample_box(rng, n_particles, (0.5, 0.07, 0.5), (0.35, 0.04, 0.35))
    target = density_grid(clip_particles(tx, sim), sim.grid, sim.p_mass)
    return Scene(sim, tools, clip_particles(x0, sim), target, actions, checkpoint_every=10, name="config2")


def _random_tools(rng: np.random.Generator, k: int, blobs) -> List[PrimitiveConfig]:
    """``k`` tools of random type and size, each resting on top of one dough
    blob (``blobs``: list of (centre, half-height)) and pressing 5 mm into it,
    so every tool is in contact from the first substep."""
    tools = []
    for _ in range(k):
        (cx, cy, cz), hh = blobs[int(rng.integers(0, len(blobs)))]
        top = cy + hh
        dx, dz = rng.uniform(-0.5, 0.5, size=2) * hh
        kind = rng.integers(0, 3)
        if kind == 0:
            r = float(rng.uniform(0.03, 0.06))
            tools.append(sphere((cx + dx, top + r - 0.005, cz + dz), radius=r))
        elif kind == 1:
            tools.append(capsule((cx + dx, top + 0.03 - 0.005, cz + dz), r=0.03, h=float(rng.uniform(0.2, 0.25))))
        else:
            tools.append(box((cx + dx, top + 0.0025 - 0.005, cz + dz),
                             (float(rng.uniform(0.02, 0.075)), 0.0025, float(rng.uniform(0.02, 0.075)))))
    return tools


def config3(n_scenes: int = 64, n_actions: int = 20, substeps: int = 50, dt: Optional[float] = None,
            seed: int = 1003, precision: str = "fp32", n_min: int = 5000, n_max: int = 40000) -> List[Scene]:
    """Batched scenes: 1-4 dough spheres each, 1-3 tools each, target = dough shifted +0.1 in x."""
    rng = np.random.default_rng(seed)
    scenes = []
    for s in range(n_scenes):
        n = int(round(np.exp(rng.uniform(np.log(n_min), np.log(n_max)))))
        sim = SimulatorConfig(E=5e3, nu=0.2, yield_stress=50.0, gravity=(0.0, -9.8, 0.0), n_grid=64, dt=dt,
                              substeps=substeps, precision=precision, n_particles=n)
        k = int(rng.integers(1, 5))
        radii = rng.uniform(0.04, 0.08, size=k)
        vol = radii ** 3
        counts = np.floor(n * vol / vol.sum()).astype(int)
        counts[0] += n - counts.sum()
        parts, blobs = [], []
        for r, c in zip(radii, counts):
            centre = (rng.uniform(0.3, 0.6), 0.05 + r, rng.uniform(0.3, 0.7))
            parts.append(sample_sphere(rng, int(c), centre, float(r)))
            blobs.append((centre, float(r)))
        x0 = clip_particles(np.concatenate(parts), sim)
        tools = _random_tools(rng, int(rng.integers(1, 4)), blobs)
        adim = action_dims(tools)[-1]
        actions = rng.uniform(-1, 1, size=(n_actions, adim))
        target = density_grid(clip_particles(x0 + np.array([0.1, 0.0, 0.0]), sim), sim.grid, sim.p_mass)
        scenes.append(Scene(sim, tools, x0, target, actions, name=f"config3[{s}]"))
    return scenes


def config4(n_actions: int = 30, n_particles: int = 100000, substeps: int = 50, dt: Optional[float] = None,
            seed: int = 1004, precision: str = "fp32_svd64") -> Scene:
    """Cutting and gripping: knife (box ∩ prism) + two-finger gripper on a 128^3 grid."""
    sim = SimulatorConfig(E=5e3, nu=0.2, yield_stress=50.0, gravity=(0.0, -9.8, 0.0), n_grid=128, dt=dt,
                          substeps=substeps, precision=precision, n_particles=n_particles)
    rng = np.random.default_rng(seed)
    x0 = clip_particles(sample_box(rng, n_particles, (0.5, 0.1, 0.5), (0.3, 0.1, 0.3)), sim)
    knife = PrimitiveConfig(shape="Knife", init_pos=(0.5, 0.25, 0.5), size=(0.125, 0.075, 0.002),
                            prism_h=(0.15, 0.15), prot=(1.0, 0.0, 0.0, 0.0), friction=0.0,
                            action=ActionConfig(dim=3, scale=(0.005, 0.005, 0.005)))
    gripper = PrimitiveConfig(shape="Gripper", init_pos=(0.5, 0.12, 0.75), size=(0.01, 0.04, 0.04),
                              init_gap=0.18, minimal_gap=0.04, maximal_gap=0.3, friction=5.0,
                              init_rot=(1.0, 0.0, 0.0, 0.0),
                              action=ActionConfig(dim=7, scale=(0.005, 0.005, 0.005, 0.0, 0.0, 0.0, 0.005)))
    actions = rng.uniform(-1, 1, size=(n_actions, 10))
    left = x0[x0[:, 0] < 0.5] + np.array([-0.15, 0.0, 0.0])
    right = x0[x0[:, 0] >= 0.5] + np.array([0.15, 0.0, 0.0])
    target = density_grid(clip_particles(np.concatenate([left, right]), sim), sim.grid, sim.p_mass)
    return Scene(sim, [knife, gripper], x0, target, actions, density_weight=10.0, contact_weight=1.0,
                 name="config4")


def config5(n_scenes: int = 16, n_actions: int = 100, substeps: int = 50, dt: Optional[float] = None,
            seed: int = 1005, precision: str = "fp32_svd64", n_min: int = 100000, n_max: int = 500000) -> List[Scene]:
    """Large batched long horizon: random boxes/spheres of dough, 3 tools each, 128^3 grids."""
    rng = np.random.default_rng(seed)
    scenes = []
    for s in range(n_scenes):
        n = int(round(np.exp(rng.uniform(np.log(n_min), np.log(n_max)))))
        sim = SimulatorConfig(E=5e3, nu=0.2, yield_stress=50.0, gravity=(0.0, -9.8, 0.0), n_grid=128, dt=dt,
                              substeps=substeps, precision=precision, n_particles=n)
        if rng.random() < 0.5:
            w = rng.uniform(0.15, 0.3, size=3)
            w[1] = rng.uniform(0.06, 0.12)
            centre = (rng.uniform(0.35, 0.65), 0.04 + w[1] / 2, rng.uniform(0.35, 0.65))
            x0 = sample_box(rng, n, centre, w)
            blob = (centre, float(w[1] / 2))
        else:
            r = rng.uniform(0.08, 0.14)
            centre = (rng.uniform(0.35, 0.65), 0.04 + r, rng.uniform(0.35, 0.65))
            x0 = sample_sphere(rng, n, centre, r)
            blob = (centre, float(r))
        x0 = clip_particles(x0, sim)
        tools = _random_tools(rng, 3, [blob])
        adim = action_dims(tools)[-1]
        actions = rng.uniform(-1, 1, size=(n_actions, adim))
        target = density_grid(clip_particles(x0 + np.array([0.1, 0.0, 0.0]), sim), sim.grid, sim.p_mass)
        scenes.append(Scene(sim, tools, x0, target, actions, checkpoint_every="auto", name=f"config5[{s}]"))
    return scenes
