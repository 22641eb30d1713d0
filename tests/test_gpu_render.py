"""GPU parity of the particle-SDF renderer (taichi_three/tina/core/particle_sdf.py)
against the oracle's FP32 restatement: the baked volume bit-exact, the traced
G-buffer (depth, normal, colour) and shading per pixel."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from _util import all_tools, small_scene
from diffskill_gb300.engine import MpmEngine
from diffskill_gb300.render import ParticleSDFRenderer, RenderConfig
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CFG = RenderConfig(voxel_res=(64, 72, 64), bake_size=6, tina_img_res=64)


def _scene(tools=(), prec="fp32"):
    sc = small_scene(n=3000, precision=prec, tools=list(tools) if tools else None)
    if not tools:
        sc.tools = []
    eng = MpmEngine(sc.sim, [sc.tools], [sc.n_particles])
    return sc, eng


@pytest.mark.parametrize("with_colors", [False, True])
def test_bake_bit_exact(gpu_lib, with_colors):
    sc, eng = _scene()
    st = eng.init_state([sc.x0])
    cols = None
    if with_colors:
        cols = np.random.default_rng(0).integers(0, 1 << 24, size=sc.n_particles, dtype=np.uint32)
    r = ParticleSDFRenderer(eng, cfg=CFG)
    r.set_particles(st, None if cols is None else torch.as_tensor(cols.astype(np.int32), device=eng.device))
    torch.cuda.synchronize()
    assert eng.status() == 0
    x = st[0:3, :sc.n_particles].double().cpu().numpy().T
    sdf, color, bbox, over = O.render_bake(x, CFG.voxel_res, CFG.bake_size, CFG.dx, cols)
    assert over == 0
    assert np.array_equal(r.bbox.cpu().numpy().reshape(2, 3), bbox)
    assert np.array_equal(r.sdf.cpu().numpy().reshape(CFG.voxel_res), sdf)
    assert np.array_equal(r.color.cpu().numpy().reshape(CFG.voxel_res + (3,)), color)
    assert sdf.min() < 0.2 and sdf.max() == 1.0


def test_bake_reports_a_volume_too_small(gpu_lib):
    sc, eng = _scene()
    st = eng.init_state([sc.x0])
    # the reference compares the particles' extent (30 voxels along x here) with the volume
    r = ParticleSDFRenderer(eng, cfg=RenderConfig(voxel_res=(20, 20, 20), tina_img_res=16))
    r.set_particles(st)
    torch.cuda.synchronize()
    assert eng.status() & 4  # MPM_STATUS_RENDER_BOX


def _compare(out, ref, exact):
    depth, nrm, col, img = ref
    d = out["depth"].cpu().numpy()
    hit = d < 0.99
    assert hit.mean() > 0.02  # the dough is in view
    if exact:
        assert np.array_equal(d, depth)
        assert np.array_equal(out["normal"].cpu().numpy(), nrm)
        assert np.array_equal(out["color"].cpu().numpy(), col)
        assert np.array_equal(out["image"].cpu().numpy(), img)
    else:  # tool SDFs differ in rounding between the two implementations
        same = np.isclose(d, depth, atol=1e-4)
        assert same.mean() > 0.99, same.mean()
        assert np.abs(out["image"].cpu().numpy() - img)[same].max() < 1e-3


def test_trace_particles_matches_oracle(gpu_lib):
    sc, eng = _scene()
    st = eng.init_state([sc.x0])
    r = ParticleSDFRenderer(eng, cfg=CFG)
    r.set_particles(st)
    out = r.trace()
    torch.cuda.synchronize()
    ref = O.render_trace(r.sdf.cpu().numpy().reshape(CFG.voxel_res), r.color.cpu().numpy().reshape(CFG.voxel_res + (3,)),
                         r.bbox.cpu().numpy(), r.v2w, r.w2v, (64, 64), CFG.sdf_threshold)
    _compare(out, ref, exact=True)


def test_trace_with_tools_matches_oracle(gpu_lib):
    tools = all_tools()[:3]
    sc, eng = _scene(tools, prec="fp64")
    st = eng.init_state([sc.x0])
    r = ParticleSDFRenderer(eng, cfg=CFG, tool_colors=[(0.8, 0.2, 0.2), (0.2, 0.8, 0.2), (0.2, 0.2, 0.8)])
    r.set_particles(st)
    out = r.trace()
    torch.cuda.synchronize()
    ref = O.render_trace(r.sdf.cpu().numpy().reshape(CFG.voxel_res), r.color.cpu().numpy().reshape(CFG.voxel_res + (3,)),
                         r.bbox.cpu().numpy(), r.v2w, r.w2v, (64, 64), CFG.sdf_threshold, tools=tools,
                         pose=eng.pose0.cpu().numpy(), tool_color=r.tool_color.cpu().numpy())
    _compare(out, ref, exact=False)
    # some pixels see a tool (its colour times 3)
    c = out["color"].cpu().numpy()
    assert (np.abs(c - np.array([0.6, 2.4, 0.6], np.float32)).max(-1) < 1e-6).any()


def test_render_api_shape(gpu_lib):
    sc, eng = _scene()
    r = ParticleSDFRenderer(eng, cfg=RenderConfig(voxel_res=(64, 72, 64), tina_img_res=128))
    r.set_particles(eng.init_state([sc.x0]))
    img = r.render("rgb", img_size=64)
    assert img.shape == (64, 64, 4) and np.isfinite(img).all()
    assert 0 < img[..., 3].min() and img[..., 3].max() <= 0.99 + 1e-6
