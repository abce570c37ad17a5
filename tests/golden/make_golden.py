"""Generates the golden fixtures in this folder from the CPU FP64 oracle.

The reference publishes no golden vectors and cannot be built here, so these
fixtures pin the oracle (itself cross-checked against an independent
brute-force restatement in tests/bruteforce.py) on small seeded scenes:
initialize + a few advance steps, every intermediate of the projection, and
the DEM sand step (boundary volumes, states after each advance).  Liquid inputs
are rounded through float32, sand velocities too, so the GPU path sees
identical values.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "sand-water-coupling_gb300"))

from oracle import oracle as orc  # noqa: E402
from swc import scenes  # noqa: E402

CASES = {
    "dam_break_2d_small": (lambda: scenes.dam_break_2d(seed=11, height_cells=16, width_cells=12), 3),
    "projection_block_3d_n8": (lambda: scenes.projection_block_3d(n=8, seed=12), 2),
}


# DEM sand: the oracle's boundary volumes and states after each advance.
SAND_CASES = {
    "sand_contact_block_2d": (lambda: scenes.sand_contact_block(2, scale=30, seed=5), 4),
}


def make_sand(name):
    build, steps = SAND_CASES[name]
    s = build()
    s.velocities = s.velocities.astype(np.float32).astype(np.float64)  # the GPU keeps FP32 velocities
    o = orc.DemOracle(s.dim, s.radius, s.mass)
    o.set_particles(s.positions, s.velocities)
    o.set_boundary(s.boundary_positions, s.boundary_normals)
    o.initialize()
    rho, vol = o.boundary_info()
    out = {"positions": s.positions, "velocities": s.velocities, "steps": steps, "dt": s.dt, "brho": rho, "bvol": vol}
    for k in range(steps):
        o.advance(s.dt)
        out[f"s{k}_x"], out[f"s{k}_v"] = o.particles()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    return out


def make(name):
    build, steps = CASES[name]
    s = build().rounded_to_float32()
    o = orc.Oracle(s)
    o.initialize()
    out = {"positions": s.positions, "velocities": s.velocities, "steps": steps, "dt": s.dt}
    rho, vol = o.real_info()
    rb, vb = o.boundary_info()
    sc = o.scalars()
    out.update(init_rho=rho, init_vol=vol, init_brho=rb, init_bvol=vb, rho0=sc["rho0"], alpha0=sc["alpha0"],
               kappa=sc["kappa"])
    for k in range(steps):
        o.advance(s.dt)
        v = o.virtual()
        x, vel = o.particles()
        st = o.stats()
        for f in ("node", "rho", "vol", "div", "alpha_hat", "p"):
            out[f"s{k}_{f}"] = v[f]
        out[f"s{k}_x"] = x
        out[f"s{k}_v"] = vel
        out[f"s{k}_iters"] = st["iterations"]
        out[f"s{k}_relres"] = st["rel_residual"]
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    return out


if __name__ == "__main__":
    for n in CASES:
        make(n)
        print("wrote", n)
    for n in SAND_CASES:
        make_sand(n)
        print("wrote", n)
