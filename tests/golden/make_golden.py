"""Generate tests/golden/density_assets.json from the reference's density assets.

Reads plb/envs/assets/*3D-v*.npy of the reference checkout (64^3 float64 grids
written by MPMSimulator.compute_grid_m_kernel, plb/engine/mpm_simulator.py:
456-466) and records, per grid: total mass, mass-weighted centroid and second
central moments in world units (node I at I*dx), and the support box.  The
quadratic B-spline stencil reproduces linear functions exactly and adds a
variance of dx^2/4 per axis, so these statistics pin p_mass, the grid layout
and the weights of the oracle's compute_grid_m without the (unshipped)
particle sets.  Usage: python tests/golden/make_golden.py REFERENCE_CHECKOUT
(the root of a DiffSkill checkout, the directory holding plb/).
"""
import glob
import json
import os
import sys

import numpy as np

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "density_assets.json")


def stats(a: np.ndarray) -> dict:
    n = a.shape[0]
    dx = 1.0 / n
    idx = np.indices(a.shape).reshape(3, -1).T * dx
    m = a.reshape(-1)
    tot = float(m.sum())
    c = (m[:, None] * idx).sum(0) / tot
    var = (m[:, None] * (idx - c) ** 2).sum(0) / tot
    nz = np.argwhere(a > 0)
    return {"n_grid": int(n), "total_mass": tot, "centroid": c.tolist(), "var": var.tolist(),
            "support_min": nz.min(0).tolist(), "support_max": nz.max(0).tolist(),
            "max": float(a.max()), "nonzero": int((a > 0).sum())}


def main() -> None:
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py REFERENCE_CHECKOUT  (the directory holding plb/envs/assets)")
    ref = sys.argv[1]
    files = sorted(glob.glob(os.path.join(ref, "plb/envs/assets/*3D-v*.npy")))
    if not files:
        sys.exit(f"no plb/envs/assets/*3D-v*.npy under {ref}")
    out = {"source": "plb/envs/assets/*3D-v*.npy", "grids": {}}
    for f in files:
        out["grids"][os.path.basename(f)] = stats(np.load(f))
    # Move3D-v1 target: a sphere of diameter 0.2049069760770578 (plb/envs/move.yml:6)
    out["move3d_v1_sphere_radius"] = 0.2049069760770578 / 2
    with open(OUT, "w") as fh:
        json.dump(out, fh, indent=1)
    print(f"wrote {OUT} ({len(files)} grids)")


if __name__ == "__main__":
    main()
