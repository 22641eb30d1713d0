"""The allocation-free substep (mpm_substep_fwd_static) against the handle-based
one (mpm_substep_fwd), through the C ABI.

mpm_substep_fwd_static serves callers that cannot call cudaMalloc: code that
steps a scene from inside another framework's GPU memory pool, or a
latency-bound loop that cannot afford cudaMalloc's device-wide
synchronisation.  Its scratch is a static device array shared by all calls,
so the test makes two calls in a row: the second must not see the first one's
grid.  This file sorts last so a stop-at-first-failure run has already run
every other test; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

from _util import all_tools, group_errors, perturbed_state, small_scene
from diffskill_gb300 import _lib
from diffskill_gb300.engine import MpmEngine

pytestmark = pytest.mark.gpu

# same bound as the FP32 / FP64 substep parity tests (tests/test_gpu_parity.py)
TOL = {"fp32": 1e-4, "fp64": 1e-9}


def _static_call(lib, eng, s0, s1, pose):
    return lib.mpm_substep_fwd_static(ctypes.byref(eng.params), eng._descs, eng.T, ctypes.c_void_p(s0.data_ptr()),
                                      ctypes.c_void_p(s1.data_ptr()), ctypes.c_void_p(pose[0].data_ptr()),
                                      ctypes.c_void_p(pose[1].data_ptr()),
                                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_static_substep_matches_handle_substep_twice(gpu_lib, prec):
    tools = [all_tools()[1], all_tools()[4]]  # capsule + gripper
    sc = small_scene(n=3000, tools=tools, precision=prec)
    eng = MpmEngine(sc.sim, [tools], [sc.n_particles])
    st = perturbed_state(sc.x0, seed=21)
    s0 = eng.new_state()
    s0[:, :sc.n_particles] = torch.as_tensor(st.T, dtype=eng.dtype, device=eng.device)
    pose = eng.pose0.unsqueeze(0).repeat(2, 1, 1).contiguous()
    pose[1, :, 0] += 0.001  # moving tools: collider velocity is exercised
    ref = eng.new_state()
    eng.substep(s0, ref, pose[0], pose[1])
    torch.cuda.synchronize()
    assert eng.status() == 0
    r = ref[:, :sc.n_particles].double().cpu().numpy().T
    for call in range(2):
        out = eng.new_state()
        rc = _static_call(gpu_lib, eng, s0, out, pose)
        assert rc == 0, _lib.last_error(None)
        torch.cuda.synchronize()
        o = out[:, :sc.n_particles].double().cpu().numpy().T
        errs = group_errors(o, r)
        assert max(errs.values()) < TOL[prec], (call, errs)


def test_static_substep_rejects_sizes_beyond_its_limit(gpu_lib):
    sc = small_scene(n=100, precision="fp64")
    sc.sim.n_grid = 128  # two FP64 grids of 128^3 nodes: 128 MiB > 16 MiB
    eng = MpmEngine(sc.sim, [sc.tools], [sc.n_particles])
    s0, s1 = eng.init_state([sc.x0]), eng.new_state()
    pose = eng.pose0.unsqueeze(0).repeat(2, 1, 1).contiguous()
    rc = _static_call(gpu_lib, eng, s0, s1, pose)
    assert rc == 1
    assert "static limit" in _lib.last_error(None)
