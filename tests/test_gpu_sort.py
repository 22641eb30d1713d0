"""The particle re-sort (mpm_sort_frame / mpm_unsort_frame) on the GPU.

The permutation must be the stable sort of the (scene, 4^3 block, cell) key,
bit for bit, for any input order (random, nearly sorted, positions outside
the grid that clamp to its edge cells); the sorted frame is the source frame
gathered through it, and the adjoint puts a frame gradient back in place.
"""
import numpy as np
import pytest
import torch

from diffskill_gb300.config import SimulatorConfig
from diffskill_gb300.engine import N_ROWS, MpmEngine

pytestmark = pytest.mark.gpu


def torch_keys(frame: torch.Tensor, pscene: torch.Tensor, n: int) -> torch.Tensor:
    """The sort key restated with torch ops (the order before this kernel existed)."""
    nb = n // 4
    base = (frame[0:3] * n - 0.5).to(torch.int64).clamp_(0, n - 1)
    blk = ((base[0] >> 2) * nb + (base[1] >> 2)) * nb + (base[2] >> 2)
    loc = ((base[0] & 3) << 4) | ((base[1] & 3) << 2) | (base[2] & 3)
    return (pscene * nb ** 3 + blk) * 64 + loc


def engine(counts, n_grid, precision):
    sim = SimulatorConfig(n_grid=n_grid, precision=precision)
    return MpmEngine(sim, [[] for _ in counts], counts)


def frame_for(eng, order: str, seed: int) -> torch.Tensor:
    g = torch.Generator(device="cpu").manual_seed(seed)
    fr = torch.rand((N_ROWS, eng.ld), generator=g, dtype=torch.float64)
    x = torch.rand((3, eng.P), generator=g, dtype=torch.float64) * 1.1 - 0.05  # some outside [0, 1)
    if order == "nearly_sorted":
        pscene = torch.as_tensor(np.repeat(np.arange(eng.S), eng.n_per_scene))
        key = torch_keys(x, pscene, eng.n_grid)
        x = x[:, torch.argsort(key, stable=True)]
        x = x + (torch.rand(x.shape, generator=g, dtype=torch.float64) - 0.5) * (0.5 / eng.n_grid)
    fr[0:3, :eng.P] = x
    return fr.to(device=eng.device, dtype=eng.dtype).contiguous()


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("counts,n_grid", [
    ([9000, 0, 5123], 64),   # three passes (20-bit keys), an empty scene, ragged tiles
    ([70001], 16),           # two passes (12-bit keys), many keys per digit
    ([1], 8),                # a single particle
])
@pytest.mark.parametrize("order", ["random", "nearly_sorted"])
def test_sort_frame_is_the_stable_key_sort(gpu_lib, precision, counts, n_grid, order):
    eng = engine(counts, n_grid, precision)
    P = eng.P
    src = frame_for(eng, order, seed=P + n_grid)
    dst = torch.full_like(src, float("nan"))
    perm = torch.full((P,), -1, dtype=torch.int32, device=eng.device)
    eng.sort_frame(src, dst, perm)
    torch.cuda.synchronize()
    pscene = torch.as_tensor(np.repeat(np.arange(eng.S), eng.n_per_scene), device=eng.device)
    key = torch_keys(src[:, :P].double(), pscene, eng.n_grid) if precision == "fp64" else \
        torch_keys(src[:, :P], pscene, eng.n_grid)
    want = torch.argsort(key, stable=True)
    assert torch.equal(perm.long(), want)
    assert torch.equal(dst[:, :P], src[:, want])
    # particles stay in their scene
    assert torch.equal(pscene[perm.long()], pscene)
    # the adjoint puts a gradient back where it came from
    g = torch.randn_like(src)
    back = torch.zeros_like(src)
    eng.unsort_frame(g, back, perm)
    torch.cuda.synchronize()
    assert torch.equal(back[:, want], g[:, :P])


def test_sort_frame_rejects_overlapping_frames(gpu_lib):
    from diffskill_gb300._lib import MpmError
    eng = engine([3000], 32, "fp32")
    buf = torch.zeros((N_ROWS + 1, eng.ld), dtype=torch.float32, device=eng.device)
    perm = torch.empty(eng.P, dtype=torch.int32, device=eng.device)
    with pytest.raises(MpmError, match="overlap"):
        eng.sort_frame(buf[0:N_ROWS], buf[1:N_ROWS + 1], perm)
    with pytest.raises(MpmError, match="overlap"):
        eng.unsort_frame(buf[0:N_ROWS], buf[0:N_ROWS], perm)
