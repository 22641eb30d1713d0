"""CPU tests of the host side: configuration, workloads, the C-ABI surface,
and the multi-process scene sharding (gloo, world size 2)."""
import ctypes
import os
import re

import numpy as np
import pytest

from diffskill_gb300 import config as C
from diffskill_gb300 import scenes
from diffskill_gb300.sharding import shard_scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_simulator_constants_follow_reference_derivation():
    """mpm_simulator.py:19-39 with quality=1: n_grid=64, dt=1e-4, substeps=19, p_vol=(dx/2)^2."""
    s = C.SimulatorConfig()
    assert s.grid == 64 and s.dx == 1 / 64 and s.step_dt == 1e-4 and s.n_substeps == 19
    assert s.p_vol == (0.5 / 64) ** 2 and s.p_mass == s.p_vol
    assert abs(s.mu - 5e3 / (2 * 1.15)) < 1e-9 and abs(s.lam - 5e3 * 0.15 / (1.15 * 0.7)) < 1e-9
    cut = C.SimulatorConfig(quality_multiplier=1.25)  # plb/cut/cut_rearrange.yml:4
    assert cut.grid == 80
    assert C.SimulatorConfig(dtype="float64").precision_code == C.PREC_FP64
    with pytest.raises(ValueError):
        C.SimulatorConfig(precision="bf16").precision_code


def test_primitive_config_and_action_dims():
    g = C.make_primitive("Gripper", action={"dim": 7, "scale": (1,) * 7}, init_gap=0.1)
    b = C.make_primitive("Box", action={"dim": 3, "scale": (0.5,) * 3})
    assert g.state_dim == 8 and b.state_dim == 7 and g.init_state[-1] == 0.1
    assert C.action_dims([b, g, b]) == [0, 3, 10, 13]
    assert b.scale7() == (0.5, 0.5, 0.5, 0.0, 0.0, 0.0, 0.0)
    with pytest.raises(ValueError):
        C.make_primitive("Teapot").type_code
    # the remaining primitives of primitives.py
    codes = {n: C.make_primitive(n).type_code for n in ("RollingPin", "RollingPinExt", "Chopsticks", "Cylinder",
                                                        "Torus", "Gripper2")}
    assert sorted(codes.values()) == list(range(5, 11))
    assert C.make_primitive("Chopsticks").state_dim == 8 and C.make_primitive("Gripper2").state_dim == 8
    assert C.make_primitive("Torus").state_dim == 7
    cyl = C.make_primitive("Cylinder")
    assert (cyl.h, cyl.r) == (0.2, 0.1) and C.make_primitive("Gripper2").r == 0.015
    assert C.make_primitive("Box", collision_group=(0, 0, 1)).collision_mask == 4
    assert C.make_primitive("Box", collision_group=(1., 0, 1)).collision_mask == 5


def test_workloads_are_seeded_and_in_bounds():
    a, b = scenes.config2(), scenes.config2()
    assert np.array_equal(a.x0, b.x0) and np.array_equal(a.actions, b.actions) and np.array_equal(a.target, b.target)
    assert a.n_particles == 30000 and a.actions.shape == (50, 6)
    c3 = scenes.config3()
    ns = [s.n_particles for s in c3]
    assert len(c3) == 64 and 5000 <= min(ns) and max(ns) <= 40000
    assert all(1 <= len(s.tools) <= 3 for s in c3)
    for s in c3[:8] + [a]:
        lo, hi = s.sim.lower_bound * s.sim.dx, 1 - 3 * s.sim.dx
        assert s.x0.min() >= lo and s.x0.max() <= hi
        assert abs(s.target.sum() - s.n_particles * s.sim.p_mass) < 1e-9


def test_density_grid_helper_conserves_mass():
    sc = scenes.config1(n_particles=5000)
    g = scenes.density_grid(sc.x0, 64, sc.sim.p_mass)
    assert abs(g.sum() - 5000 * sc.sim.p_mass) < 1e-12


def _header_functions():
    src = open(os.path.join(ROOT, "include", "mpm_gb300.h")).read()
    return sorted(set(re.findall(r"^(?:int|int64_t|const char\*)\s+(mpm_\w+)\(", src, re.M)))


def test_c_abi_library_exports_every_declared_symbol():
    """The built library loads without a GPU and exports every entry point of
    include/mpm_gb300.h; the ctypes table binds exactly those."""
    from diffskill_gb300 import _lib, build
    build.build()
    lib = ctypes.CDLL(build.LIB)
    names = _header_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(_lib.SIGNATURES) == names
    lib.mpm_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.mpm_version()


def test_c_abi_rejects_bad_arguments_without_a_gpu():
    """Argument checks run before any device call."""
    from diffskill_gb300 import _lib
    lib = _lib.load()
    p = _lib.MpmParams()
    p.abi_version = 99
    h = ctypes.c_void_p()
    offs = (ctypes.c_int64 * 2)(0, 0)
    assert lib.mpm_create(ctypes.byref(p), offs, ctypes.byref(h)) == 1
    assert "ABI version" in _lib.last_error(None)
    p.abi_version = _lib.ABI_VERSION
    p.precision = 0
    p.n_grid = 60
    p.n_scenes = 1
    assert lib.mpm_create(ctypes.byref(p), offs, ctypes.byref(h)) == 1
    assert "multiple of 8" in _lib.last_error(None)
    assert lib.mpm_substep_fwd(None, None, None, None, None, None) == 1
    assert lib.mpm_sort_frame(None, None, None, None, None) == 1
    assert "NULL handle" in _lib.last_error(None)
    assert lib.mpm_unsort_frame(None, None, None, None, None) == 1
    assert lib.mpm_set_pipelined_adjoint(None, 1) == 1


def test_shard_scenes_balances_and_covers():
    rng = np.random.default_rng(0)
    ns = [int(v) for v in rng.integers(5000, 40000, size=64)]
    for world in (1, 2, 3, 8):
        parts = [shard_scenes(ns, world, r) for r in range(world)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(64))
        loads = [sum(ns[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(ns)


def _gloo_worker(rank, world, port, ns, q):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = shard_scenes(ns, world, rank)
    t = torch.zeros(len(ns), dtype=torch.int64)
    t[mine] = 1
    dist.all_reduce(t)
    load = torch.tensor([float(sum(ns[i] for i in mine))])
    dist.all_reduce(load, op=dist.ReduceOp.MAX)
    q.put((rank, t.tolist(), float(load)))
    dist.destroy_process_group()


def test_scene_sharding_two_ranks_gloo():
    """World size 2 over gloo: every scene is owned by exactly one rank and
    the max-over-ranks reduction the bench uses agrees on both ranks."""
    import multiprocessing as mp
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ns = [7000, 12000, 30000, 5000, 9000, 22000, 15000]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_gloo_worker, args=(r, 2, port, ns, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, cover, load in out:
        assert cover == [1] * len(ns)
        assert load == max(sum(ns[i] for i in shard_scenes(ns, 2, r)) for r in range(2))


def test_checkpoint_planner_picks_smallest_interval_that_fits():
    """The interval planner of long horizons: store every frame when it fits,
    else the smallest divisor of the horizon whose frames fit the budget."""
    from diffskill_gb300.engine import horizon_frames, plan_checkpoint_interval
    fb = 100
    # everything fits: every frame is kept, as the reference does
    assert plan_checkpoint_interval(1000, fb, 10 ** 9) == 1
    assert horizon_frames(1000, 1) == 1003
    # one byte short of store-all: the next divisor that fits
    k = plan_checkpoint_interval(1000, fb, horizon_frames(1000, 1) * fb - 1)
    assert k == 2 and 1000 % k == 0
    # the chosen interval always fits, and every smaller divisor does not
    for budget in (600 * fb, 200 * fb, 80 * fb, 70 * fb):
        k = plan_checkpoint_interval(1000, fb, budget)
        assert 1000 % k == 0 and horizon_frames(1000, k) * fb <= budget
        for j in range(1, k):
            assert 1000 % j or horizon_frames(1000, j) * fb > budget
    # the fixed share comes off the budget
    assert plan_checkpoint_interval(1000, fb, 10 ** 9, fixed_bytes=10 ** 9 - 600 * fb) > 1
    # config 5 shapes: 100 actions x 50 substeps, 384 MiB frames, 189 GiB for frames
    assert plan_checkpoint_interval(5000, 384 << 20, 189 << 30) == 20
    # below the minimum (near sqrt of the horizon) no interval fits
    with pytest.raises(MemoryError):
        plan_checkpoint_interval(1000, fb, 60 * fb)
    with pytest.raises(ValueError):
        plan_checkpoint_interval(0, fb, 10 ** 9)


def test_config5_asks_for_a_planned_interval():
    sc = scenes.config5(n_scenes=2, n_actions=2, n_min=1000, n_max=2000)
    assert all(s.checkpoint_every == "auto" for s in sc)


def test_build_flags_keep_the_renderer_exact():
    """The substep units take the fast FP32 divide/sqrt and flush-to-zero; the
    renderer keeps IEEE rounding without FMA contraction (its parity with the
    oracle's restatement is bit-level)."""
    from diffskill_gb300 import build
    render = build.EXTRA["mpm_render.cu"]
    assert "-fmad=false" in render
    assert not any(f.startswith(("-prec-", "-ftz", "-use_fast_math")) for f in render)
    for src in ("mpm_fwd.cu", "mpm_bwd.cu", "mpm_static.cu"):
        assert {"-ftz=true", "-prec-div=false", "-prec-sqrt=false"} <= set(build.EXTRA[src])
    for src in build.SOURCES:
        assert "-use_fast_math" not in build.EXTRA.get(src, ())
