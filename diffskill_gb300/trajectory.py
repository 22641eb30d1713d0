"""Batched trajectory optimisation: forward, density loss, adjoint, Adam.

One ``BatchedTrajectory.step()`` is one iteration of
``Solver.solve_one_plan`` (plb/optimizer/solver.py:97-152) for every scene of
the batch at once: reset to the initial state, run all actions forward,
compute the per-scene loss, run the checkpointed adjoint, take an Adam step on
the actions (torch.optim.Adam semantics, lr 0.01 default) and clip them to
[-1, 1].  The whole step is capturable as one CUDA graph: no host sync, no
allocation after the first call.
"""
from __future__ import annotations

from typing import List, Optional, Sequence, Union

import numpy as np
import torch

from .engine import Horizon, MpmEngine
from .scenes import Scene


def spatial_order(x: np.ndarray, n_grid: int) -> np.ndarray:
    """Permutation sorting particles by base cell, block-major (4^3 cells per
    block, then cell within block), so that neighbouring threads of the p2g
    scatter and the g2p gather touch the same grid nodes."""
    base = np.clip((np.asarray(x) * n_grid - 0.5).astype(np.int64), 0, n_grid - 1)
    nb = n_grid // 4
    blk = ((base[:, 0] >> 2) * nb + (base[:, 1] >> 2)) * nb + (base[:, 2] >> 2)
    loc = ((base[:, 0] & 3) << 4) | ((base[:, 1] & 3) << 2) | (base[:, 2] & 3)
    return np.argsort(blk * 64 + loc, kind="stable")


def adam_update(actions: torch.Tensor, grad: torch.Tensor, mask: torch.Tensor, m: torch.Tensor, v: torch.Tensor,
                t: torch.Tensor, betas=(0.9, 0.999), lr: float = 0.01, eps: float = 1e-8) -> None:
    """One ``torch.optim.Adam`` step on ``actions`` (no weight decay, no
    amsgrad: ``actions -= lr * m_hat / (sqrt(v_hat) + eps)``), then
    ``clamp(-1, 1)`` and the action mask, as ``Solver.solve_one_plan`` applies
    them (plb/optimizer/solver.py:98, 128-133).  The step count ``t`` is a
    device tensor, so the bias corrections change between replays of a CUDA
    graph that captured this update.  ``mask`` zeroes the padding lanes of the
    [A, T, 8] action layout (their gradient is zero too)."""
    b1, b2 = float(betas[0]), float(betas[1])
    g = grad * mask
    t.add_(1)
    m.mul_(b1).add_(g, alpha=1 - b1)
    v.mul_(b2).addcmul_(g, g, value=1 - b2)
    bc1 = 1 - torch.pow(b1, t)
    bc2 = 1 - torch.pow(b2, t)
    denom = (v / bc2).sqrt_().add_(eps)
    actions.sub_(lr * (m / bc1) / denom)
    actions.clamp_(-1, 1).mul_(mask)


def _check_compatible(scenes: Sequence[Scene]) -> None:
    s0 = scenes[0].sim
    for sc in scenes[1:]:
        s = sc.sim
        same = (s.grid == s0.grid and s.step_dt == s0.step_dt and s.n_substeps == s0.n_substeps and s.E == s0.E
                and s.nu == s0.nu and s.yield_stress == s0.yield_stress and tuple(s.gravity) == tuple(s0.gravity)
                and s.ground_friction == s0.ground_friction and s.precision_code == s0.precision_code
                and sc.n_actions == scenes[0].n_actions)
        if not same:
            raise ValueError("batched scenes must share grid, dt, substeps, material, precision and horizon")


class BatchedTrajectory:
    def __init__(self, scenes: Sequence[Scene], ckpt_every: Union[int, str, None] = None, lr: float = 0.01,
                 betas=(0.9, 0.999), eps: float = 1e-8, softness: float = 666.0, sort_particles: bool = True,
                 autotune: bool = False):
        scenes = list(scenes)
        _check_compatible(scenes)
        self.scenes = scenes
        self.eng = MpmEngine(scenes[0].sim, [sc.tools for sc in scenes], [sc.n_particles for sc in scenes],
                             softness=softness)
        k = ckpt_every if ckpt_every else (scenes[0].checkpoint_every or scenes[0].sim.n_substeps)
        self.hz = Horizon(self.eng, scenes[0].n_actions, ckpt_every=k)
        eng = self.eng
        # particle order is internal: losses and action gradients do not depend on it
        self.orders = [spatial_order(sc.x0, eng.n_grid) if sort_particles else np.arange(sc.n_particles)
                       for sc in scenes]
        self.state0 = eng.init_state([sc.x0[o] for sc, o in zip(scenes, self.orders)])
        self.targets = eng.targets([sc.target for sc in scenes])
        self.actions = eng.expand_actions([sc.actions for sc in scenes])
        mask = torch.zeros((1, max(eng.T, 1), 8), dtype=torch.float64, device=eng.device)
        for t, cfg in enumerate(eng.tool_cfgs):
            mask[0, t, :int(cfg.action.dim)] = 1
        self.mask = mask
        self.density_weight = scenes[0].density_weight
        self.contact_weight = scenes[0].contact_weight
        self.lr, self.betas, self.eps = lr, betas, eps
        self.m = torch.zeros_like(self.actions)
        self.v = torch.zeros_like(self.actions)
        self.t = torch.zeros((), dtype=torch.float64, device=eng.device)
        self.loss = torch.zeros(eng.S, dtype=torch.float64, device=eng.device)
        self.grad = torch.zeros_like(self.actions)
        self.graph: Optional[torch.cuda.CUDAGraph] = None
        self.tuning = None
        if autotune:
            self.autotune()

    def autotune(self, **kw):
        """Pick launch shapes and the re-sort cadence for this batch by
        measurement (``diffskill_gb300.autotune.tune``); before ``capture``."""
        from .autotune import tune
        if self.graph is not None:
            raise RuntimeError("autotune before capturing the CUDA graph")
        self.tuning = tune(self, **kw)
        return self.tuning

    @property
    def particle_substeps(self) -> int:
        return self.eng.P * self.hz.F

    def forward_backward(self) -> None:
        hz = self.hz
        hz.forward(self.state0, self.actions)
        self.loss.copy_(hz.loss(self.targets, self.density_weight, self.contact_weight))
        self.grad.copy_(hz.backward())

    def set_initial_positions(self, x: torch.Tensor) -> None:
        """New initial positions ``x`` ([3, P] on the device, scenes concatenated
        in their order, particles of a scene in any order): the initial state
        becomes ``reset_kernel``'s (mpm_simulator.py:402-409: v = 0, C = 0,
        F = I) at ``x``, with each scene's particles sorted by grid cell on the
        device."""
        P = self.eng.P
        st = self.state0
        st[0:3, :P].copy_(x)
        st[3:24, :P].zero_()
        st[15, :P].fill_(1)
        st[19, :P].fill_(1)
        st[23, :P].fill_(1)
        self.hz.sort_frame(st)

    def forward_only(self) -> None:
        """Forward of every action and the per-scene loss, no adjoint."""
        hz = self.hz
        hz.forward(self.state0, self.actions, keep_grids=False)
        self.loss.copy_(hz.loss(self.targets, self.density_weight, self.contact_weight, need_grad=False))

    def adam(self) -> None:
        """torch.optim.Adam update, then clamp to [-1, 1] and mask (solver.py:128-133)."""
        adam_update(self.actions, self.grad, self.mask, self.m, self.v, self.t, self.betas, self.lr, self.eps)

    def step(self) -> None:
        """One optimisation iteration (replays the CUDA graph when captured)."""
        if self.graph is not None:
            self.graph.replay()
        else:
            self.forward_backward()
            self.adam()

    def capture(self) -> None:
        """Capture forward + backward + Adam of one iteration as a CUDA graph."""
        self.graph = self._capture(lambda: (self.forward_backward(), self.adam()), self.forward_backward)

    def capture_forward(self) -> torch.cuda.CUDAGraph:
        """Capture the forward and the loss of one iteration (no adjoint) as a
        CUDA graph, returned for the caller to replay."""
        return self._capture(self.forward_only, self.forward_only)

    @staticmethod
    def _capture(body, warm) -> torch.cuda.CUDAGraph:
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):  # warm allocations outside the capture
            warm()
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            body()
        torch.cuda.synchronize()
        return g

    def reset_optimizer(self, actions: Optional[List] = None) -> None:
        if actions is not None:
            self.actions.copy_(self.eng.expand_actions(actions))
        self.m.zero_()
        self.v.zero_()
        self.t.zero_()

    def action_grads(self) -> List[torch.Tensor]:
        return self.eng.collapse_action_grad(self.grad)
