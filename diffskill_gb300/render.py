"""Particle-SDF renderer on the GB300 kernels, with the API of
``TinaRenderer`` (plb/env_modeling/tina_renderer.py) for what it draws: the
particle SDF (``tina.core.particle_sdf.ParticleSDFRaster``) and the tools.

``mpm_render_bake`` builds the SDF volume of one scene's particles and
``mpm_render_trace`` casts one ray per pixel.  The camera is tina's orbit
camera (``tina.util.control.Control.get_camera``: rotation
euler(-theta, phi, -pi/2) about static x, y, z, the eye at ``center + R (0, 0,
radius)``, a 60 degree perspective with near 0.05 and far 500).  The image is
the linear Lambert shading of tina's ``Lighting.shade_color`` with its default
lights; tina's tone mapping, temporal anti-aliasing (random sample jitter) and
GUI are not part of the raster and are not reproduced.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass
from typing import Optional, Sequence, Tuple

import numpy as np
import torch

from . import _lib
from .engine import MpmEngine, _ptr, _stream


@dataclass
class RenderConfig:
    """``cfg.RENDERER`` defaults (plb/config/default_config.py:37-63) used here."""
    voxel_res: Tuple[int, int, int] = (168, 168, 168)
    dx: float = 1.0 / 150
    bake_size: int = 6
    sdf_threshold: float = 0.37 * 0.56
    tina_img_res: int = 1024
    cam_center: Tuple[float, float, float] = (0.5, 0.0, 0.5)
    cam_theta: float = 0.0
    cam_phi: float = -0.8
    cam_radius: float = 0.88


def _rx(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[1, 0, 0], [0, c, -s], [0, s, c]])


def _ry(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])


def _rz(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]])


def _frustum(l, r, b, t, n, f):
    m = np.eye(4)
    m[0, 0] = 2 * n / (r - l)
    m[1, 1] = 2 * n / (t - b)
    m[0, 2] = (r + l) / (r - l)
    m[1, 2] = (t + b) / (t - b)
    m[2, 2] = -(f + n) / (f - n)
    m[2, 3] = -2 * f * n / (f - n)
    m[3, 2] = -1
    m[3, 3] = 0
    return m


def tina_camera(center, theta: float, phi: float, radius: float, fov: float = 60.0,
                aspect: float = 1.0) -> Tuple[np.ndarray, np.ndarray]:
    """(W2V, V2W) float32 4x4 of tina's perspective orbit camera."""
    R = _rz(-math.pi / 2) @ _ry(phi) @ _rx(-theta)  # rotations about static x, then y, then z
    eye = np.asarray(center, dtype=np.float64) + R @ np.array([0.0, 0.0, radius])
    cam = np.eye(4)
    cam[:3, :3] = R
    cam[:3, 3] = eye
    view = np.linalg.inv(cam)
    f = math.tan(math.radians(fov) / 2)
    near, far = 0.05, 500.0
    proj = _frustum(-near * f * aspect, near * f * aspect, -near * f, near * f, near, far)
    w2v = proj @ view
    return np.array(w2v, dtype=np.float32), np.array(np.linalg.inv(w2v), dtype=np.float32)


class ParticleSDFRenderer:
    """Renders one scene of an ``MpmEngine``: ``set_particles`` bakes the SDF
    volume of a state frame, ``render`` traces the image."""

    def __init__(self, eng: MpmEngine, scene: int = 0, cfg: Optional[RenderConfig] = None,
                 tool_colors: Optional[Sequence[Sequence[float]]] = None):
        self.eng, self.scene = eng, int(scene)
        self.cfg = cfg if cfg is not None else RenderConfig()
        dev = eng.device
        res = tuple(int(r) for r in self.cfg.voxel_res)
        nv = res[0] * res[1] * res[2]
        self.packed = torch.empty(nv, dtype=torch.int64, device=dev)
        self.sdf = torch.empty(nv, dtype=torch.float32, device=dev)
        self.sdf_copy = torch.empty_like(self.sdf)
        self.color = torch.empty((nv, 3), dtype=torch.float32, device=dev)
        self.bbox = torch.zeros(6, dtype=torch.float32, device=dev)
        self.kbox = torch.zeros(8, dtype=torch.int32, device=dev)
        v = _lib.MpmRenderVolume()
        v.res[:] = res
        v.bake_size, v.dx = int(self.cfg.bake_size), float(self.cfg.dx)
        v.packed, v.sdf, v.sdf_copy = self.packed.data_ptr(), self.sdf.data_ptr(), self.sdf_copy.data_ptr()
        v.color, v.bbox, v.kbox = self.color.data_ptr(), self.bbox.data_ptr(), self.kbox.data_ptr()
        self.vol = v
        tools = [t for t, s in zip(eng.tool_cfgs, eng.tool_scene) if s == self.scene]
        self.tool_idx = [i for i, s in enumerate(eng.tool_scene) if s == self.scene]
        cols = np.full((max(eng.T, 1), 3), 0.3, np.float32)  # Primitive default color (primive_base.py:319)
        if tool_colors is not None:
            for i, c in zip(self.tool_idx, tool_colors):
                cols[i] = c
        self.tool_color = torch.as_tensor(cols, device=dev)
        self.n_tools = len(tools)
        self.update_camera(self.cfg.cam_center, self.cfg.cam_theta, self.cfg.cam_phi, self.cfg.cam_radius)

    def update_camera(self, center, theta, phi, radius) -> None:
        """``TinaRenderer.update_camera`` (tina_renderer.py:35-36)."""
        self.w2v, self.v2w = tina_camera(center, theta, phi, radius)

    def set_particles(self, state: torch.Tensor, colors: Optional[torch.Tensor] = None) -> None:
        """Bake the SDF volume of this scene's particles in a state frame
        (``TinaRenderer.set_particles`` + ``plb_set_particles``)."""
        _lib.check(self.eng.lib.mpm_render_bake(self.eng.h, _ptr(state), self.scene, _ptr(colors),
                                                ctypes.byref(self.vol), _stream()), self.eng.h, "mpm_render_bake")

    def trace(self, pose: Optional[torch.Tensor] = None, img_res: Optional[int] = None,
              show_particles: bool = True) -> dict:
        """depth (view-space z), normal, color and shaded image of every pixel, as device tensors."""
        r = int(img_res or self.cfg.tina_img_res)
        view = _lib.MpmRenderView()
        view.v2w[:] = self.v2w.ravel().tolist()
        view.w2v[:] = self.w2v.ravel().tolist()
        view.res[:] = [r, r]
        view.bias[:] = [0.5, 0.5]
        view.sdf_threshold = float(self.cfg.sdf_threshold)
        view.show_particles = int(bool(show_particles))
        dev = self.eng.device
        out = {"depth": torch.empty((r, r), dtype=torch.float32, device=dev),
               "normal": torch.empty((r, r, 3), dtype=torch.float32, device=dev),
               "color": torch.empty((r, r, 3), dtype=torch.float32, device=dev),
               "image": torch.empty((r, r, 3), dtype=torch.float32, device=dev)}
        if pose is None:
            pose = self.eng.pose0
        pose = pose.to(dev, torch.float64).contiguous()
        _lib.check(self.eng.lib.mpm_render_trace(self.eng.h, ctypes.byref(self.vol), ctypes.byref(view), self.scene,
                                                 _ptr(pose), _ptr(self.tool_color), _ptr(out["depth"]),
                                                 _ptr(out["normal"]), _ptr(out["color"]), _ptr(out["image"]),
                                                 _stream()), self.eng.h, "mpm_render_trace")
        return out

    def render(self, mode: str = "rgb", img_size: int = 64, pose: Optional[torch.Tensor] = None) -> np.ndarray:
        """``TinaRenderer.render(mode='rgb')`` (tina_renderer.py:100-125): (img_size, img_size, 4)
        of rgb and depth, area-averaged from tina_img_res (a multiple of img_size)."""
        if mode != "rgb":
            raise ValueError("only mode='rgb' renders headless")
        out = self.trace(pose)
        img = np.concatenate([out["image"].cpu().numpy(),
                              np.clip(out["depth"].cpu().numpy(), 0.0, 3.0)[..., None]], axis=-1)
        r = img.shape[0]
        if r != img_size:
            if r % img_size:
                raise ValueError(f"tina_img_res {r} is not a multiple of img_size {img_size}")
            f = r // img_size
            img = img.reshape(img_size, f, img_size, f, 4).mean(axis=(1, 3))
        return img
