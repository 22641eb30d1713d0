"""The allocation-free substep (mpm_substep_fwd_static) against the FP64 oracle
and against the handle-based substep (mpm_substep_fwd), through the C ABI.

mpm_substep_fwd_static serves callers that cannot call cudaMalloc: code that
steps a scene from inside another framework's GPU memory pool, or a
latency-bound loop that cannot afford cudaMalloc's device-wide
synchronisation.  Its scratch is a static device array shared by all calls,
so every case makes calls in a row: a later call must not see an earlier
call's grid, tool table or status.  Cases cover no tools, two tools, FP64 at
n_grid = 64 (the two grids then fill the 16 MiB grid area exactly),
consecutive calls with different grid sizes, and the status word a caller
reads back.  This file sorts last so a stop-at-first-failure run has already
run every other test; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

from _util import all_tools, group_errors, perturbed_state, small_scene
from diffskill_gb300 import _lib
from diffskill_gb300.engine import MpmEngine
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

# same bounds as the FP32 / FP64 substep parity tests (tests/test_gpu_parity.py)
TOL = {"fp32": 1e-4, "fp64": 1e-9}


def _static_call(lib, eng, s0, s1, pose, status=None):
    st = ctypes.c_void_p(status.data_ptr()) if status is not None else None
    return lib.mpm_substep_fwd_static(ctypes.byref(eng.params), eng._descs, eng.T, ctypes.c_void_p(s0.data_ptr()),
                                      ctypes.c_void_p(s1.data_ptr()), ctypes.c_void_p(pose[0].data_ptr()),
                                      ctypes.c_void_p(pose[1].data_ptr()), st,
                                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


def _scene(prec, tools, n=3000, n_grid=None, seed=21):
    sc = small_scene(n=n, tools=tools, precision=prec)
    if n_grid is not None:
        sc.sim.n_grid = n_grid
    eng = MpmEngine(sc.sim, [sc.tools], [sc.n_particles])
    st = perturbed_state(sc.x0, seed=seed)
    s0 = eng.new_state()
    s0[:, :sc.n_particles] = torch.as_tensor(st.T, dtype=eng.dtype, device=eng.device)
    return sc, eng, st, s0


def _poses(eng, o, sc):
    """Tool poses of frames f, f+1 of the first action (moving tools: the
    collider velocity is exercised), from the oracle's kinematics."""
    if eng.T == 0:
        return torch.zeros((2, 1, 8), dtype=torch.float64, device=eng.device), np.zeros((2, 0, 8))
    _, _, pseq = o.tools_action(o.pose0(), sc.actions[0])
    return torch.as_tensor(pseq[:2], device=eng.device).contiguous(), pseq


def _aos(st, n):
    return st[:, :n].double().cpu().numpy().T


@pytest.mark.parametrize("prec,which", [("fp32", "two"), ("fp64", "two"), ("fp32", "none"), ("fp64", "none")])
def test_static_substep_matches_oracle_and_handle_twice(gpu_lib, prec, which):
    tools = [all_tools()[1], all_tools()[4]] if which == "two" else []  # capsule + gripper, or none
    sc, eng, st, s0 = _scene(prec, tools)
    o = Oracle(sc.sim, tools)
    pose, pseq = _poses(eng, o, sc)
    ref = o.substep(pseq[0], pseq[1], st)
    handle = eng.new_state()
    eng.substep(s0, handle, pose[0], pose[1])
    torch.cuda.synchronize()
    assert eng.status() == 0
    h = _aos(handle, sc.n_particles)
    status = torch.zeros(1, dtype=torch.int32, device=eng.device)
    for call in range(2):
        out = eng.new_state()
        rc = _static_call(gpu_lib, eng, s0, out, pose, status)
        assert rc == 0, _lib.last_error(None)
        torch.cuda.synchronize()
        o_st = _aos(out, sc.n_particles)
        e_oracle = group_errors(o_st, ref)
        e_handle = group_errors(o_st, h)
        assert max(e_oracle.values()) < TOL[prec], (call, "oracle", e_oracle)
        assert max(e_handle.values()) < TOL[prec], (call, "handle", e_handle)
        assert int(status.item()) == 0


def test_static_substep_consecutive_grid_sizes(gpu_lib):
    """Calls alternating between grids of 32^3 and 48^3 nodes: each matches
    the handle path of its own size (the block flags, list and grids shared by
    the calls are cleared per call)."""
    tools = [all_tools()[0]]
    for n_grid in (32, 48, 32, 48):
        sc, eng, st, s0 = _scene("fp32", tools, n=2000, n_grid=n_grid, seed=n_grid)
        o = Oracle(sc.sim, tools)
        pose, pseq = _poses(eng, o, sc)
        handle = eng.new_state()
        eng.substep(s0, handle, pose[0], pose[1])
        out = eng.new_state()
        rc = _static_call(gpu_lib, eng, s0, out, pose)
        assert rc == 0, _lib.last_error(None)
        torch.cuda.synchronize()
        errs = group_errors(_aos(out, sc.n_particles), _aos(handle, sc.n_particles))
        assert max(errs.values()) < TOL["fp32"], (n_grid, errs)
        ref = o.substep(pseq[0], pseq[1], st)
        errs = group_errors(_aos(out, sc.n_particles), ref)
        assert max(errs.values()) < TOL["fp32"], (n_grid, errs)


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_static_substep_reports_out_of_grid_particle(gpu_lib, prec):
    """A particle whose stencil leaves the grid is skipped (its state copied
    unchanged, as the handle path does) and sets MPM_STATUS_OUT_OF_GRID in the
    caller's status word; the next clean call leaves a cleared word at 0."""
    sc, eng, st, s0 = _scene(prec, [], n=500)
    s0[0:3, 7] = torch.tensor([0.999, 0.5, 0.5], dtype=eng.dtype, device=eng.device)
    pose = torch.zeros((2, 1, 8), dtype=torch.float64, device=eng.device)
    status = torch.zeros(1, dtype=torch.int32, device=eng.device)
    out = eng.new_state()
    rc = _static_call(gpu_lib, eng, s0, out, pose, status)
    assert rc == 0, _lib.last_error(None)
    torch.cuda.synchronize()
    assert int(status.item()) & _lib.STATUS_OUT_OF_GRID
    assert torch.equal(out[:15, 7], s0[:15, 7])
    # without a status word the bits go to the scratch word; the call still succeeds
    rc = _static_call(gpu_lib, eng, s0, out, pose, None)
    assert rc == 0, _lib.last_error(None)
    s0[0:3, 7] = s0[0:3, 8]
    status.zero_()
    rc = _static_call(gpu_lib, eng, s0, out, pose, status)
    assert rc == 0, _lib.last_error(None)
    torch.cuda.synchronize()
    assert int(status.item()) == 0


def test_static_substep_rejects_sizes_beyond_its_limit(gpu_lib):
    sc = small_scene(n=100, precision="fp64")
    sc.sim.n_grid = 128  # two FP64 grids of 128^3 nodes: 128 MiB > 16 MiB
    eng = MpmEngine(sc.sim, [sc.tools], [sc.n_particles])
    s0, s1 = eng.init_state([sc.x0]), eng.new_state()
    pose = eng.pose0.unsqueeze(0).repeat(2, 1, 1).contiguous()
    rc = _static_call(gpu_lib, eng, s0, s1, pose)
    assert rc == 1
    assert "static limit" in _lib.last_error(None)


def test_static_substep_rejects_tool_types_above_gripper(gpu_lib):
    from _util import more_tools
    sc = small_scene(n=100, tools=[more_tools()[0]], precision="fp32")  # RollingPin
    eng = MpmEngine(sc.sim, [sc.tools], [sc.n_particles])
    s0, s1 = eng.init_state([sc.x0]), eng.new_state()
    pose = eng.pose0.unsqueeze(0).repeat(2, 1, 1).contiguous()
    rc = _static_call(gpu_lib, eng, s0, s1, pose)
    assert rc == 1
    assert "unknown type" in _lib.last_error(None)
