"""Configuration objects for the MPM substep.

Field names mirror the reference's yacs defaults so a YAML written for the
reference maps one to one:

* ``SimulatorConfig``  <- ``cfg.SIMULATOR`` (plb/config/default_config.py:11-22)
  plus the derived constants of ``MPMSimulator.__init__``
  (plb/engine/mpm_simulator.py:19-39).
* ``PrimitiveConfig``  <- one entry of ``cfg.PRIMITIVES``
  (plb/engine/primitive/primive_base.py:313-329 and the per-shape
  ``default_config`` of plb/engine/primitive/primitives.py).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Optional, Sequence, Tuple

# Tool type codes shared with the C ABI (include/mpm_gb300.h, MPM_TOOL_*)
TOOL_SPHERE = 0
TOOL_CAPSULE = 1
TOOL_BOX = 2
TOOL_KNIFE = 3
TOOL_GRIPPER = 4
TOOL_ROLLINGPIN = 5
TOOL_ROLLINGPINEXT = 6
TOOL_CHOPSTICKS = 7
TOOL_CYLINDER = 8
TOOL_TORUS = 9
TOOL_GRIPPER2 = 10
SHAPE_CODES = {"Sphere": TOOL_SPHERE, "Capsule": TOOL_CAPSULE, "Box": TOOL_BOX,
               "Knife": TOOL_KNIFE, "Gripper": TOOL_GRIPPER, "RollingPin": TOOL_ROLLINGPIN,
               "RollingPinExt": TOOL_ROLLINGPINEXT, "Chopsticks": TOOL_CHOPSTICKS, "Cylinder": TOOL_CYLINDER,
               "Torus": TOOL_TORUS, "Gripper2": TOOL_GRIPPER2}
# tools whose state carries a gap (state_dim 8)
GAP_SHAPES = ("Gripper", "Chopsticks", "Gripper2")
# per-shape default_config values that differ from the Capsule defaults
# (Cylinder primitives.py:323-326, Gripper2 688-697)
SHAPE_DEFAULTS = {"Cylinder": {"h": 0.2, "r": 0.1}, "Gripper2": {"r": 0.015}}

# Precision modes shared with the C ABI (MPM_PREC_*)
PREC_FP32 = 0        # state, grid and SVD in FP32; reductions in FP64
PREC_FP32_SVD64 = 1  # FP32 state and grid; SVD, return map and its adjoint in FP64
PREC_FP64 = 2        # everything FP64 (the plain reference method on the GPU)
PRECISIONS = {"fp32": PREC_FP32, "fp32_svd64": PREC_FP32_SVD64, "fp64": PREC_FP64}


@dataclass
class SimulatorConfig:
    """``cfg.SIMULATOR`` (default_config.py:11-22) with the derived constants.

    ``n_grid``/``dt``/``substeps`` default to the reference's derivation
    (mpm_simulator.py:19-39: ``n_grid = int(128*q)``, ``dt = 0.5e-4/q``,
    ``substeps = int(2e-3 // dt)`` with ``q = quality*quality_multiplier*0.5``)
    and may be overridden for the synthetic workloads.
    """

    dim: int = 3
    quality: float = 1.0
    quality_multiplier: float = 1.0
    yield_stress: float = 50.0
    dtype: str = "float32"
    max_steps: int = 1024
    n_particles: int = 30000
    lower_bound: float = 0.0
    E: float = 5e3
    nu: float = 0.15
    ground_friction: float = 1.5
    gravity: Tuple[float, float, float] = (0.0, -1.0, 0.0)
    # explicit overrides (None = reference derivation)
    n_grid: Optional[int] = None
    dt: Optional[float] = None
    substeps: Optional[int] = None
    # GB300 path precision: "fp32", "fp32_svd64" or "fp64"; None follows dtype
    precision: Optional[str] = None

    # -- derived ---------------------------------------------------------
    @property
    def _q(self) -> float:
        return self.quality * self.quality_multiplier * (0.5 if self.dim == 3 else 1.0)

    @property
    def grid(self) -> int:
        return int(self.n_grid) if self.n_grid is not None else int(128 * self._q)

    @property
    def dx(self) -> float:
        return 1.0 / self.grid

    @property
    def inv_dx(self) -> float:
        return float(self.grid)

    @property
    def step_dt(self) -> float:
        return float(self.dt) if self.dt is not None else 0.5e-4 / self._q

    @property
    def n_substeps(self) -> int:
        return int(self.substeps) if self.substeps is not None else int(2e-3 // self.step_dt)

    @property
    def p_vol(self) -> float:
        return (self.dx * 0.5) ** 2  # squared even in 3D (mpm_simulator.py:28)

    @property
    def p_mass(self) -> float:
        return self.p_vol * 1.0

    @property
    def mu(self) -> float:
        return self.E / (2 * (1 + self.nu))

    @property
    def lam(self) -> float:
        return self.E * self.nu / ((1 + self.nu) * (1 - 2 * self.nu))

    @property
    def precision_code(self) -> int:
        name = self.precision or ("fp64" if self.dtype == "float64" else "fp32")
        if name not in PRECISIONS:
            raise ValueError(f"unknown precision {name!r}; expected one of {sorted(PRECISIONS)}")
        return PRECISIONS[name]


@dataclass
class ActionConfig:
    dim: int = 0
    scale: Tuple[float, ...] = ()


@dataclass
class PrimitiveConfig:
    """One rigid tool (``cfg.PRIMITIVES`` entry).

    ``shape`` is one of Sphere, Capsule, Box, Knife, Gripper, RollingPin,
    RollingPinExt, Chopsticks, Cylinder, Torus, Gripper2.  Sizes follow the
    reference's fields: ``radius`` (Sphere), ``h``/``r`` (Capsule segment along
    local y of length h, also RollingPin(Ext), Chopsticks and the Gripper2
    fingers; Cylinder radial extent h and half height r), ``size`` (Box half
    extents; Knife box; Gripper finger), ``prism_h``/``prot`` (Knife prism, the
    reference's ``h``/``prot``), ``tx``/``ty`` (Torus),
    ``minimal_gap``/``maximal_gap``/``init_gap`` (Gripper, Chopsticks,
    Gripper2), ``collision_group`` (entry j > 0: project this tool out of tool
    j after every kinematics step, mpm_simulator.py:69-80).
    """

    shape: str = "Sphere"
    init_pos: Tuple[float, float, float] = (0.3, 0.3, 0.3)
    init_rot: Tuple[float, float, float, float] = (1.0, 0.0, 0.0, 0.0)
    lower_bound: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    upper_bound: Tuple[float, float, float] = (1.0, 1.0, 1.0)
    friction: float = 0.9
    action: ActionConfig = field(default_factory=ActionConfig)
    radius: float = 1.0
    h: float = 0.06
    r: float = 0.03
    size: Tuple[float, float, float] = (0.1, 0.1, 0.1)
    prism_h: Tuple[float, float] = (0.1, 0.1)
    prot: Tuple[float, float, float, float] = (1.0, 0.0, 0.0, 0.0)
    minimal_gap: float = 0.06
    maximal_gap: float = 1.0
    init_gap: float = 0.06
    tx: float = 0.2
    ty: float = 0.1
    collision_group: Tuple[float, ...] = ()

    @property
    def type_code(self) -> int:
        if self.shape not in SHAPE_CODES:
            raise ValueError(f"unsupported primitive shape {self.shape!r}; expected one of {sorted(SHAPE_CODES)}")
        return SHAPE_CODES[self.shape]

    @property
    def state_dim(self) -> int:
        return 8 if self.shape in GAP_SHAPES else 7

    @property
    def init_state(self) -> Tuple[float, ...]:
        st = tuple(self.init_pos) + tuple(self.init_rot)
        return st + ((self.init_gap,) if self.shape in GAP_SHAPES else (0.0,))

    @property
    def collision_mask(self) -> int:
        """Bit j set iff collision_group[j] > 0."""
        return sum(1 << j for j, g in enumerate(self.collision_group) if float(g) > 0)

    def scale7(self) -> Tuple[float, ...]:
        s = list(self.action.scale) + [0.0] * (7 - len(self.action.scale))
        return tuple(float(v) for v in s[:7])


def make_primitive(shape: str, **kw) -> PrimitiveConfig:
    """Build a PrimitiveConfig from reference-style keyword arguments."""
    action = kw.pop("action", None)
    if isinstance(action, dict):
        action = ActionConfig(dim=int(action.get("dim", 0)), scale=tuple(action.get("scale", ())))
    kw = dict(SHAPE_DEFAULTS.get(shape, {}), **kw)
    cfg = PrimitiveConfig(shape=shape, **kw)
    if action is not None:
        cfg.action = action
    return cfg


def action_dims(prims: Sequence[PrimitiveConfig]):
    """``Primitives.action_dims`` (primitives.py:830-837): prefix sums."""
    dims = [0]
    for p in prims:
        dims.append(dims[-1] + int(p.action.dim))
    return dims


def ceil_div(a: int, b: int) -> int:
    return -(-a // b)


def isclose(a: float, b: float) -> bool:
    return math.isclose(a, b, rel_tol=1e-12, abs_tol=0.0)
