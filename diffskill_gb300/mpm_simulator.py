"""``MPMSimulator`` with the reference's API (plb/engine/mpm_simulator.py),
running on the GB300 kernels.

Frame semantics are the reference's: ``substep(s)`` reads frame ``s`` and
writes frame ``s+1`` of ``max_steps`` stored frames (fields x, v, C, F of
shape ``(max_steps, N)``, mpm_simulator.py:38-43); ``substep_grad(s)``
accumulates the adjoint of frame ``s`` from that of frame ``s+1``, as the
taichi ``.grad`` fields do.  For horizons longer than ``max_steps`` use
``diffskill_gb300.engine.Horizon`` (checkpointed recompute) instead.
"""
from __future__ import annotations

from typing import List, Optional

import numpy as np
import torch

from .config import PREC_FP64, SimulatorConfig
from .engine import MpmEngine
from .primitives import Primitives


class _Scalar:
    """Stand-in for a taichi 0-d field: ``n_particles[None]``."""

    def __init__(self, v=0):
        self.v = v

    def __getitem__(self, k):
        return self.v

    def __setitem__(self, k, v):
        self.v = int(v)


class _GridMassKernel:
    """``compute_grid_m_kernel(f)`` and its ``.grad(f)`` (mpm_simulator.py:456-466)."""

    def __init__(self, sim: "MPMSimulator"):
        self.sim = sim

    def __call__(self, f: int) -> None:
        sim = self.sim
        sim._eng.grid_mass(sim._frames[f], sim.grid_m_t)

    def grad(self, f: int) -> None:
        sim = self.sim
        sim._eng.grid_mass_bwd(sim._frames[f], sim.grid_m_grad_t, sim._gframes[f])


class MPMSimulator:
    def __init__(self, cfg: SimulatorConfig, primitives: Primitives = None, device=None):
        self.cfg = cfg
        self.dim = 3
        self.primitives = primitives if primitives is not None else Primitives([])
        self.primitives.sim = self
        for p in self.primitives:
            p.sim = self
        self.n_primitive = len(self.primitives)
        self.n_grid = cfg.grid
        self.dx, self.inv_dx = cfg.dx, cfg.inv_dx
        self.dt = cfg.step_dt
        self.p_vol, self.p_rho = cfg.p_vol, 1
        self.p_mass = cfg.p_mass
        self.substeps = cfg.n_substeps
        self.max_steps = int(cfg.max_steps)
        self.lower_bound = cfg.lower_bound
        self.n_particles = _Scalar(0)
        self.dtype = "float64" if cfg.precision_code == PREC_FP64 else "float32"
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self._eng: Optional[MpmEngine] = None
        self.compute_grid_m_kernel = _GridMassKernel(self)
        self.cur = 0
        self._fk_bwd_done = set()

    # ------------------------------------------------------------ lifetime
    def initialize(self, n_particles: int) -> None:
        """``initialize`` (mpm_simulator.py:82-97): allocate for ``n_particles``."""
        n = int(n_particles)
        self.n_particles[None] = n
        self._eng = MpmEngine(self.cfg, [self.primitives.cfgs], [n], softness=self.primitives.get_softness(),
                              device=self.device)
        eng = self._eng
        T = max(eng.T, 1)
        M = self.max_steps
        self._frames = torch.zeros((M, 24, eng.ld), dtype=eng.dtype, device=eng.device)
        self._gframes = torch.zeros_like(self._frames)
        self._tmp = eng.new_state()
        self._pose = torch.zeros((M + 1, T, 8), dtype=torch.float64, device=eng.device)
        self._pose[0, :eng.T] = eng.pose0
        self._vel = torch.zeros((M, T, 8), dtype=torch.float64, device=eng.device)
        self._g_pose = torch.zeros_like(self._pose)
        n_act = M // self.substeps + 1
        self._act = torch.zeros((n_act, T, 8), dtype=torch.float64, device=eng.device)
        self._g_act = torch.zeros_like(self._act)
        self._coll = eng.new_coll(n_act)  # tool-tool collision records per action
        self.grid_m_t = torch.zeros((1, eng.G), dtype=eng.dtype, device=eng.device)
        self.grid_m_grad_t = torch.zeros_like(self.grid_m_t)
        self.cur = 0

    def _t64(self, a) -> torch.Tensor:
        return torch.as_tensor(np.asarray(a, dtype=np.float64), device=self.device)

    def _set_softness(self, softness: float) -> None:
        if self._eng is not None and softness != self._eng.softness:
            # tool tables carry the softness; rebuild them on change
            eng = self._eng
            for i in range(eng.T):
                eng._descs[i].softness = softness
            eng.softness = softness
            from . import _lib
            _lib.check(eng.lib.mpm_set_tools(eng.h, eng._descs, eng.T), eng.h, "mpm_set_tools")

    # ------------------------------------------------------------- tools
    def _set_action(self, s: int, action: np.ndarray, only: Optional[int] = None) -> None:
        eng, n = self._eng, self.substeps
        if (s + 1) * n > self.max_steps - 1:
            raise IndexError(f"action {s} runs past max_steps={self.max_steps}")
        row = self._act[s].clone()
        dims = self.primitives.action_dims
        for i in range(eng.T):
            if only is not None and i != only:
                continue
            d = dims[i + 1] - dims[i]
            row[i, :d] = self._t64(action[dims[i]:dims[i + 1]])
        self._act[s].copy_(row)
        if eng.T:
            eng.tools_action(self._act[s], self._vel[s * n], self._pose[s * n],
                             None if self._coll is None else self._coll[s])

    def _tools_action_bwd(self, s: int) -> None:
        if s in self._fk_bwd_done or not self._eng.T:
            return
        n = self.substeps
        self._eng.tools_action_bwd(self._vel[s * n], self._pose[s * n], self._g_pose[s * n], self._g_act[s],
                                   None if self._coll is None else self._coll[s])
        self._fk_bwd_done.add(s)

    def tool_sdf(self, t: int, f: int, points: np.ndarray) -> np.ndarray:
        raise NotImplementedError("per-point tool SDFs are exposed through GradModel(return_dist=True)")

    # ------------------------------------------------------------ substeps
    def substep(self, s: int) -> None:
        """``substep`` (mpm_simulator.py:307-323)."""
        self._eng.substep(self._frames[s], self._frames[s + 1], self._pose[s], self._pose[s + 1])

    def substep_grad(self, s: int) -> None:
        """``substep_grad`` (mpm_simulator.py:325-345): frame-(s+1) adjoint -> frame s (accumulated)."""
        self._eng.substep_bwd(self._frames[s], self._gframes[s + 1], self._tmp, self._pose[s], self._pose[s + 1],
                              self._g_pose[s], self._g_pose[s + 1], st1=self._frames[s + 1])
        self._gframes[s].add_(self._tmp)

    def step(self, is_copy: bool, action=None) -> None:
        """``step`` (mpm_simulator.py:440-451)."""
        start = 0 if is_copy else self.cur
        self.cur = start + self.substeps
        if action is not None:
            self.primitives.set_action(start // self.substeps, self.substeps, action)
        for s in range(start, self.cur):
            self.substep(s)
        if is_copy:
            self.copyframe(self.cur, 0)
            self.cur = 0

    def copyframe(self, source: int, target: int) -> None:
        self._frames[target].copy_(self._frames[source])
        self._pose[target].copy_(self._pose[source])

    # ----------------------------------------------------------------- io
    def _rows(self, f: int, r0: int, r1: int) -> np.ndarray:
        n = self.n_particles[None]
        return self._frames[f, r0:r1, :n].double().cpu().numpy().T.copy()

    def get_x(self, f: int) -> np.ndarray:
        return self._rows(f, 0, 3)

    def get_v(self, f: int) -> np.ndarray:
        return self._rows(f, 3, 6)

    def get_torch_x(self, f: int, device) -> torch.Tensor:
        n = self.n_particles[None]
        return self._frames[f, 0:3, :n].t().float().to(device).contiguous()

    def get_state(self, f: int) -> List[np.ndarray]:
        """``get_state`` (380-390): [x, v, F(N,3,3), C(N,3,3), tool states...]."""
        n = self.n_particles[None]
        st = self._frames[f, :, :n].double().cpu().numpy()
        out = [st[0:3].T.copy(), st[3:6].T.copy(), st[15:24].T.reshape(n, 3, 3).copy(),
               st[6:15].T.reshape(n, 3, 3).copy()]
        for p in self.primitives:
            out.append(p.get_state(f))
        return out

    def set_state(self, f: int, state) -> None:
        """``set_state`` (392-396)."""
        n = len(state[0])
        if self._eng is None or n != self.n_particles[None]:
            self.initialize(n)
        fr = torch.zeros((24, n), dtype=torch.float64)
        fr[0:3] = torch.as_tensor(np.asarray(state[0], dtype=np.float64).T)
        fr[3:6] = torch.as_tensor(np.asarray(state[1], dtype=np.float64).T)
        fr[15:24] = torch.as_tensor(np.asarray(state[2], dtype=np.float64).reshape(n, 9).T)
        fr[6:15] = torch.as_tensor(np.asarray(state[3], dtype=np.float64).reshape(n, 9).T)
        self._frames[f, :, :n].copy_(fr.to(self.device, self._frames.dtype))
        for s, p in zip(state[4:], self.primitives):
            p.set_state(f, s)

    def set_primitive_state(self, f: int, state) -> None:
        for s, p in zip(state[4:], self.primitives):
            p.set_state(f, s)

    def reset(self, x) -> None:
        """``reset`` (402-413): x given, v = 0, F = I, C = 0 at frame 0."""
        x = np.asarray(x, dtype=np.float64)
        if self._eng is None or x.shape[0] != self.n_particles[None]:
            self.initialize(x.shape[0])
        self._frames[0].copy_(self._eng.init_state([x]))
        self.cur = 0

    def get_m(self) -> np.ndarray:
        return self.grid_m_t[0].double().cpu().numpy().reshape(self.n_grid, self.n_grid, self.n_grid)

    def clear_and_compute_grid_m(self, f: int) -> None:
        self.compute_grid_m_kernel(f)

    # ------------------------------------------------------------- grads
    def zero_grad(self) -> None:
        """The ``.grad.fill(0)`` calls of GradModel.reset (function.py:45-61)."""
        self._gframes.zero_()
        self._g_pose.zero_()
        self._g_act.zero_()
        self._fk_bwd_done.clear()

    def check_status(self) -> None:
        self._eng.check_status()
