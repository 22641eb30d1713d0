"""``GradModel``: the differentiable torch boundary of plb/engine/function.py
on the GB300 kernels.

Same methods and return tuple as the reference: ``reset``, ``get_obs``,
``set_obs_grad``, ``forward_step``, ``backward_step`` and ``forward`` (a
``torch.autograd.Function`` over one action returning the observation
``(x||v [, tool distances]) (N x 6[+k]), tool states (T x 8) [, grid_m]`` at
the next action boundary).  ``SimEnv`` is the subset of ``TaichiEnv``
(plb/engine/taichi_env.py) that GradModel needs: a simulator, its
primitives, and get_state / set_state.
"""
from __future__ import annotations

from typing import Optional, Sequence

import numpy as np
import torch
from torch.autograd import Function

from .config import PrimitiveConfig, SimulatorConfig
from .mpm_simulator import MPMSimulator
from .primitives import Primitives


class SimEnv:
    """Minimal ``TaichiEnv`` (taichi_env.py:46-177): simulator + primitives + state io."""

    def __init__(self, sim_cfg: SimulatorConfig, primitive_cfgs: Sequence[PrimitiveConfig], x0: np.ndarray,
                 softness: float = 666.0, device=None):
        self.primitives = Primitives(primitive_cfgs)
        self.simulator = MPMSimulator(sim_cfg, self.primitives, device=device)
        self.primitives.set_softness(softness)
        self.simulator.initialize(len(x0))
        self.primitives.initialize()
        self.simulator.reset(x0)
        self._is_copy = True

    def get_state(self):
        assert self.simulator.cur == 0
        return {"state": self.simulator.get_state(0), "softness": self.primitives.get_softness(),
                "is_copy": self._is_copy}

    def set_state(self, state, softness=None, is_copy=None, **kwargs):
        if softness is None:
            softness, is_copy, state = state["softness"], state["is_copy"], state["state"]
        self.simulator.cur = 0
        self.simulator.set_state(0, state)
        self.primitives.set_softness(softness)
        self._is_copy = is_copy

    def step(self, action=None):
        if action is not None:
            action = np.array(action)
        self.simulator.step(is_copy=self._is_copy, action=action)


class GradModel:
    def __init__(self, env, softness: float = 666.0, init_sampler=None, output_grid=(), return_dist: bool = False):
        self.env = env
        self.sim: MPMSimulator = env.simulator
        self.dim = self.sim.dim
        self.primitives = self.sim.primitives
        self.substeps = self.sim.substeps
        self.softness = softness
        self._forward_func = None
        self.output_grid = output_grid
        self.return_dist = return_dist
        self.init_state = self.env.get_state()["state"]
        self.init_sampler = init_sampler if init_sampler is not None else (lambda: self.init_state)
        self.device = "cuda"

    # ------------------------------------------------------------------ reset
    def reset(self, initial_states=None, device="cuda", clear_grad=True):
        """function.py:39-64."""
        self.device = device
        if initial_states is None:
            initial_states = self.init_sampler()
        if clear_grad:
            self.sim.zero_grad()
        self.env.set_state(initial_states, self.softness, False)
        return self.get_obs(0, self.device)

    # -------------------------------------------------------------- obs / grad
    def _dists(self, f: int) -> torch.Tensor:
        eng = self.sim._eng
        return eng.tool_distance(self.sim._frames[f], self.sim._pose[f])

    def get_obs(self, s: int, device):
        """function.py:104-128: (x||v [, dists]) (N x 6[+k]), tool states (T x 8) [, grid_m]."""
        f = s * self.substeps
        n = self.sim.n_particles[None]
        fr = self.sim._frames[f]
        x = fr[0:6, :n].t().float()
        c = torch.zeros((len(self.primitives), 8), dtype=torch.float32, device=fr.device)
        for i, p in enumerate(self.primitives):
            c[i, :p.state_dim] = self.sim._pose[f, i, :p.state_dim].float()
        if self.return_dist:
            d = self._dists(f)[:, :n].t().float()
            x = torch.cat((x, d), 1)
        outputs = (x.clone().to(device), c.clone().to(device))
        for _ in self.output_grid:
            self.sim.compute_grid_m_kernel(f)
            outputs = outputs + (self.sim.grid_m_t[0].float().reshape((self.sim.n_grid,) * 3).clone().to(device),)
        return outputs

    def set_obs_grad(self, s: int, obs_grad, manipulator_grad, *args):
        """function.py:144-164: accumulate observation gradients into frame s*substeps."""
        f = s * self.substeps
        sim, eng = self.sim, self.sim._eng
        n = sim.n_particles[None]
        if len(self.output_grid) > 0 and len(args) > 0 and args[0] is not None:
            sim.compute_grid_m_kernel(f)
            sim.grid_m_grad_t[0].copy_(args[0].reshape(-1).to(sim.grid_m_grad_t.dtype))
            sim.compute_grid_m_kernel.grad(f)
        if self.return_dist:
            k = eng.n_dist_cols
            g = torch.zeros((max(k, 1), eng.ld), dtype=eng.dtype, device=eng.device)
            g[:k, :n] = obs_grad[:, -k:].t().to(eng.dtype)
            eng.tool_distance_bwd(sim._frames[f], sim._pose[f], g, sim._gframes[f], sim._g_pose[f])
            obs_grad = obs_grad[..., :-k]
        obs_grad = obs_grad.reshape(-1, self.dim * 2)
        sim._gframes[f, 0:6, :n].add_(obs_grad.t().to(sim._gframes.dtype))
        mg = manipulator_grad.reshape(len(self.primitives), 8)
        for i, p in enumerate(self.primitives):
            sim._g_pose[f, i, :p.state_dim] += mg[i, :p.state_dim].to(torch.float64)

    # ------------------------------------------------------------ steps
    def forward_step(self, s: int, a) -> None:
        """function.py:166-175."""
        a = a.reshape(-1).clamp(-1, 1)
        self.primitives.set_action(s, self.substeps, a)
        for i in range(s * self.substeps, (s + 1) * self.substeps):
            self.sim.substep(i)

    def backward_step(self, s: int) -> torch.Tensor:
        """function.py:177-190: adjoint of action s; returns d/d(action s) (flat)."""
        for i in range((s + 1) * self.substeps - 1, s * self.substeps - 1, -1):
            self.sim.substep_grad(i)
        self.sim._tools_action_bwd(s)
        grads = [torch.as_tensor(p.get_action_grad(s, 1)[0]) for p in self.primitives if p.action_dim > 0]
        return torch.cat(grads).to(self.device) if grads else torch.zeros(0, device=self.device)

    @property
    def forward(self):
        if self._forward_func is None:
            model = self

            class forward(Function):
                @staticmethod
                def forward(ctx, s, a, *past_obs):
                    ctx.save_for_backward(torch.tensor([s]), *[torch.zeros_like(i) for i in past_obs])
                    model.forward_step(s, a)
                    return model.get_obs(s + 1, a.device)

                @staticmethod
                def backward(ctx, *obs_grad):
                    tmp = ctx.saved_tensors
                    s = int(tmp[0].item())
                    model.set_obs_grad(s + 1, *obs_grad)
                    actor_grad = model.backward_step(s)
                    return (None, actor_grad.reshape(-1).to(obs_grad[0].dtype)) + tmp[1:]

            self._forward_func = forward
        return self._forward_func.apply
