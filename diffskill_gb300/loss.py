"""``Loss`` with the reference's API (plb/engine/losses/loss.py), on the GB300
kernels.

One scene, over a ``diffskill_gb300.mpm_simulator.MPMSimulator``.  The loss at
frame f is, as ``compute_loss_kernel`` (loss.py:240-262) builds it,
``contact + density_weight * sum|grid_m - target| + sdf_weight * sum target_sdf * grid_m``
with ``contact = sum_i contact_weight * min_dist_i^2`` over the movable tools,
``min_dist`` soft (loss.py:144-162) or hard (loss.py:151-155).  ``loss``
accumulates over calls until ``clear``, as the reference's ``loss[None] +=``
does; ``compute_loss`` returns the per-step increment and the reward.
``compute_loss_kernel.grad(f)`` is ``compute_loss_kernel_grad`` (loss.py:264-291):
it accumulates the frame-f particle gradient and tool-pose gradient of the
simulator.  The chamfer term is not part of the reference's loss (its call is
commented out, loss.py:254) and is not provided.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field
from typing import Optional

import numpy as np
import torch


@dataclass
class LossWeights:
    """``ENV.loss.weight`` defaults (plb/config/default_config.py:72-75)."""
    sdf: float = 10.0
    density: float = 10.0
    contact: float = 1.0


@dataclass
class LossConfig:
    """``ENV.loss`` defaults (plb/config/default_config.py:70-76)."""
    soft_contact: bool = False
    weight: LossWeights = field(default_factory=LossWeights)
    target_path: str = ""


class _LossKernel:
    """``compute_loss_kernel(f)`` and its ``.grad(f)``."""

    def __init__(self, loss: "Loss"):
        self.L = loss

    def __call__(self, f: int) -> None:
        self.L._forward(f)

    def grad(self, f: int, loss_grad: float = 1.0) -> None:
        self.L._backward(f, loss_grad)


class Loss:
    def __init__(self, cfg: Optional[LossConfig], sim):
        self.cfg = cfg if cfg is not None else LossConfig()
        self.sim = sim
        self.inf = 1000
        self.enable_target_update = True
        self.sdf_weight = float(self.cfg.weight.sdf)
        self.density_weight = float(self.cfg.weight.density)
        self.contact_weight = [float(self.cfg.weight.contact)] * max(sim.n_primitive, 1)
        self.soft_contact_loss = bool(self.cfg.soft_contact)
        self.target_density: Optional[torch.Tensor] = None
        self.target_sdf: Optional[torch.Tensor] = None
        self.nearest_point: Optional[torch.Tensor] = None
        self.loss = 0.0
        self.density_loss = self.sdf_loss = self.contact_loss = 0.0
        self.compute_loss_kernel = _LossKernel(self)
        self._iou = None
        self._target_iou = None
        self._start_loss = self._last_loss = self._init_iou = 0.0
        self._fwd = None  # what the last forward computed, for the adjoint

    @property
    def _eng(self):
        if self.sim._eng is None:
            raise RuntimeError("initialize the simulator first")
        return self.sim._eng

    # ------------------------------------------------------------- targets
    def load_target_density(self, path: Optional[str] = None, grids=None) -> None:
        """``load_target_density`` (loss.py:58-75); ``path`` is a .npy file."""
        if path is None and grids is None:
            return
        if path:
            grids = np.load(os.path.expanduser(path))
        grids = np.asarray(grids, dtype=np.float64)
        eng = self._eng
        self.target_density = torch.as_tensor(grids.reshape(1, -1), dtype=eng.dtype, device=eng.device).contiguous()
        self.update_target()
        # the reference leaves the target in grid_mass and records its IoU with itself
        self.sim.grid_m_t.copy_(self.target_density)
        self.iou()
        self._target_iou = self._iou

    def initialize(self) -> None:
        """``initialize`` (loss.py:77-86)."""
        self.sdf_weight = float(self.cfg.weight.sdf)
        self.density_weight = float(self.cfg.weight.density)
        self.contact_weight = [float(self.cfg.weight.contact)] * len(self.contact_weight)
        self.soft_contact_loss = bool(self.cfg.soft_contact)
        self.load_target_density(self.cfg.target_path or None)

    def set_weights(self, sdf, density, contact, is_soft_contact, chamfer=0.0) -> None:
        """``set_weights`` (loss.py:88-95)."""
        self.sdf_weight, self.density_weight = float(sdf), float(density)
        self.contact_weight = [float(contact)] * len(self.contact_weight)
        self.soft_contact_loss = bool(is_soft_contact)
        self.reset()

    def set_target_update(self, flag: bool) -> None:
        self.enable_target_update = bool(flag)

    def update_target(self) -> None:
        """``update_target`` (loss.py:129-134): 2 * n_grid propagation sweeps."""
        eng = self._eng
        n_iters = 2 * eng.n_grid if self.enable_target_update else 0
        if self.target_sdf is not None and n_iters == 0:
            return  # the reference leaves target_sdf as it was
        self.target_sdf, self.nearest_point = eng.target_sdf(self.target_density, n_iters)

    # --------------------------------------------------------------- losses
    def _movable(self):
        eng = self._eng
        return [t for t in range(eng.T) if eng.tool_cfgs[t].action.dim > 0]

    def _forward(self, f: int) -> None:
        eng, sim = self._eng, self.sim
        st, pose = sim._frames[f], sim._pose[f]
        gm = sim.grid_m_t
        eng.grid_mass(st, gm)
        dens = float(eng.density_l1(gm, self.target_density)[0])
        sdfl = float(eng.sdf_loss(gm, self.target_sdf)[0])
        contact, extra = 0.0, None
        mov = self._movable()
        if mov:
            if self.soft_contact_loss:
                md, sums = eng.soft_contact(st, pose)
                extra = ("soft", sums)
            else:
                md, am = eng.contact_min_dist(st, pose)
                extra = ("hard", am)
            mdh = md.double().cpu().numpy()
            for i, t in enumerate(mov):
                contact += self.contact_weight[i] * float(mdh[t]) ** 2
            extra = extra + (mdh,)
        self.density_loss, self.sdf_loss, self.contact_loss = dens, sdfl, contact
        self.loss += contact + dens * self.density_weight + sdfl * self.sdf_weight
        self._fwd = (f, extra)

    def _backward(self, f: int, loss_grad: float = 1.0) -> None:
        eng, sim = self._eng, self.sim
        st, pose = sim._frames[f], sim._pose[f]
        g_st, g_pose = sim._gframes[f], sim._g_pose[f]
        gm = sim.grid_m_t
        eng.grid_mass(st, gm)
        g_gm = sim.grid_m_grad_t
        eng.density_l1(gm, self.target_density, weight=self.density_weight * loss_grad, g_gm=g_gm)
        eng.sdf_loss(gm, self.target_sdf, weight=self.sdf_weight * loss_grad, g_gm=g_gm)
        eng.grid_mass_bwd(st, g_gm, g_st)
        mov = self._movable()
        if mov:
            if self._fwd is None or self._fwd[0] != f:
                self._forward_contact_only(f)
            kind, aux, mdh = self._fwd[1]
            g_md = torch.zeros(max(eng.T, 1), dtype=torch.float64)
            for i, t in enumerate(mov):
                g_md[t] = loss_grad * self.contact_weight[i] * 2.0 * float(mdh[t])
            g_md = g_md.to(eng.device)
            if kind == "soft":
                eng.soft_contact_bwd(st, pose, aux, g_md, g_st, g_pose)
            else:
                eng.contact_min_dist_bwd(st, pose, aux, g_md, g_st, g_pose)

    def _forward_contact_only(self, f: int) -> None:
        eng, sim = self._eng, self.sim
        st, pose = sim._frames[f], sim._pose[f]
        if self.soft_contact_loss:
            md, sums = eng.soft_contact(st, pose)
            self._fwd = (f, ("soft", sums, md.double().cpu().numpy()))
        else:
            md, am = eng.contact_min_dist(st, pose)
            self._fwd = (f, ("hard", am, md.double().cpu().numpy()))

    def iou(self) -> None:
        """``iou`` (loss.py:314-316) on the simulator's current grid_mass."""
        self._iou = float(self._eng.iou(self.sim.grid_m_t, self.target_density)[0])

    def _extract_loss(self, f: int) -> dict:
        self.compute_loss_kernel(f)
        self.iou()
        return {"loss": self.loss, "contact_loss": self.contact_loss, "density_loss": self.density_loss,
                "sdf_loss": self.sdf_loss, "iou": self._iou, "target_iou": self._target_iou}

    def reset(self) -> None:
        """``reset`` (loss.py:335-340)."""
        self.loss = 0.0
        info = self._extract_loss(0)
        self._start_loss = info["loss"]
        self._init_iou = info["iou"]
        self._last_loss = 0.0

    def compute_loss(self, f: int) -> dict:
        """``compute_loss`` (loss.py:342-351)."""
        info = self._extract_loss(f)
        r = self._start_loss - (info["loss"] - self._last_loss)
        cur = info["loss"] - self._last_loss
        self._last_loss = info["loss"]
        denom = info["target_iou"] - self._init_iou
        inc = (info["iou"] - self._init_iou) / denom if denom != 0 else 0.0
        info["reward"] = r
        info["incremental_iou"] = max(min(inc, 1), 0)
        info["loss"] = cur
        return info

    def clear(self) -> None:
        self.loss = 0.0
        self._last_loss = 0.0

    def get_state(self) -> dict:
        return {"_start_loss": self._start_loss, "_last_loss": self._last_loss, "_init_iou": self._init_iou}

    def set_state(self, _start_loss, _last_loss, _init_iou) -> None:
        self._start_loss, self._last_loss, self._init_iou = _start_loss, _last_loss, _init_iou
