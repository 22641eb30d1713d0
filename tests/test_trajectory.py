"""The timed iteration: the batched Adam step and the CUDA-graph replay of one
optimisation iteration (forward + loss + adjoint + Adam).

The reference's iteration is ``Solver.solve_one_plan`` (plb/optimizer/
solver.py:97-152): ``torch.optim.Adam([action], lr)``, ``optim.step()``, then
``action.data = clamp(action.data, -1, 1)`` and ``action.data *= action_mask``.
"""
import numpy as np
import pytest
import torch

from diffskill_gb300.trajectory import adam_update


def _reference_adam(actions0, grads, mask, lr, betas, eps):
    """torch.optim.Adam + clamp + mask, as solve_one_plan runs them."""
    p = torch.nn.Parameter(actions0.clone())
    opt = torch.optim.Adam([p], lr=lr, betas=betas, eps=eps)
    out = []
    for g in grads:
        opt.zero_grad()
        p.grad = g.clone()
        opt.step()
        p.data.copy_(torch.clamp(p.data, -1, 1))
        p.data.copy_(p.data * mask)
        out.append(p.data.clone())
    return out


@pytest.mark.parametrize("lr,betas", [(0.01, (0.9, 0.999)), (0.1, (0.8, 0.99))])
def test_adam_update_matches_torch_adam_with_clamp_and_mask(lr, betas):
    rng = np.random.default_rng(7)
    A, T = 6, 3
    mask = torch.zeros((1, T, 8), dtype=torch.float64)
    for t, d in enumerate((3, 7, 6)):  # per-tool action dims in the [A, T, 8] layout
        mask[0, t, :d] = 1
    a0 = (torch.as_tensor(rng.uniform(-1, 1, (A, T, 8))) * mask).contiguous()
    # gradients over five decades, so that the clamp to [-1, 1] is reached
    grads = [torch.as_tensor(rng.normal(size=(A, T, 8)) * 10.0 ** (i % 5 - 2)) * mask for i in range(40)]
    ref = _reference_adam(a0, grads, mask, lr, betas, 1e-8)
    a = a0.clone()
    m, v = torch.zeros_like(a), torch.zeros_like(a)
    t = torch.zeros((), dtype=torch.float64)
    for i, g in enumerate(grads):
        adam_update(a, g, mask, m, v, t, betas, lr, 1e-8)
        assert torch.allclose(a, ref[i], rtol=0, atol=1e-14), (i, (a - ref[i]).abs().max())
    assert float(a.abs().max()) == 1.0  # the clamp took part
    assert float(t) == len(grads)


@pytest.mark.gpu
def test_graph_replay_equals_eager_iterations(gpu_lib):
    """BatchedTrajectory.capture() + step() against eager forward_backward() +
    adam() on FP64 scenes: after three iterations the losses, the action
    gradients and the actions agree to 1e-12 (FP64 atomics may reorder sums)."""
    from diffskill_gb300 import scenes
    from diffskill_gb300.trajectory import BatchedTrajectory

    def make():
        scs = scenes.config3(n_scenes=3, n_actions=2, substeps=10, precision="fp64", n_min=1500, n_max=3000)
        return BatchedTrajectory(scs, ckpt_every=5, lr=0.05)

    eager, graph = make(), make()
    for _ in range(3):
        eager.forward_backward()
        eager.adam()
    graph.capture()
    for _ in range(3):
        graph.step()
    torch.cuda.synchronize()
    eager.eng.check_status()
    graph.eng.check_status()
    for name in ("loss", "grad", "actions"):
        e, g = getattr(eager, name), getattr(graph, name)
        den = float(e.abs().max())
        assert den > 0, name
        err = float((e - g).abs().max()) / den
        assert err <= 1e-12, (name, err)
    assert float(graph.t) == 3.0


@pytest.mark.gpu
def test_autotune_picks_candidates_and_keeps_results(gpu_lib, tmp_path, monkeypatch):
    """The autotuner's choices are launch shapes and a re-sort cadence only:
    the loss and the action gradients of a tuned batch equal the defaults'
    (FP64, 1e-10: atomics may reorder sums), and every choice is a candidate."""
    from diffskill_gb300 import autotune, scenes
    from diffskill_gb300.trajectory import BatchedTrajectory

    monkeypatch.setenv("DIFFSKILL_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))

    def make():
        return BatchedTrajectory(scenes.config3(n_scenes=3, n_actions=3, substeps=10, precision="fp64",
                                                n_min=1500, n_max=3000), ckpt_every=5)

    ref = make()
    ref.forward_backward()
    tuned = make()
    t = tuned.autotune(reps=2)
    for name, cands in autotune.CANDIDATES.items():
        assert getattr(t, name) in cands
    assert t.resort_every in autotune.resort_candidates(10, 5, 30)
    assert tuned.hz.R == (t.resort_every if 0 < t.resort_every < 30 else 0)
    tuned.forward_backward()
    torch.cuda.synchronize()
    for name in ("loss", "grad"):
        e, g = getattr(ref, name), getattr(tuned, name)
        assert float((e - g).abs().max()) <= 1e-10 * float(e.abs().max()), name
    # a second batch of the same shape reads the cache
    again = make()
    t2 = again.autotune()
    assert t2.shapes() == t.shapes() and t2.resort_every == t.resort_every
    assert (tmp_path / "tune.json").exists()
