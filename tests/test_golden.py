"""The oracle reproduces the committed golden fixtures (regression pin)."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden  # noqa: E402


@pytest.mark.parametrize("name", sorted(make_golden.CASES))
def test_oracle_reproduces_golden(oracle_mod, name):
    g = np.load(os.path.join(HERE, "golden", name + ".npz"))
    build, steps = make_golden.CASES[name]
    s = build().rounded_to_float32()
    assert np.array_equal(s.positions, g["positions"]) and np.array_equal(s.velocities, g["velocities"])
    o = oracle_mod.Oracle(s)
    o.initialize()
    rho, vol = o.real_info()
    np.testing.assert_allclose(rho, g["init_rho"], rtol=1e-12)
    np.testing.assert_allclose(vol, g["init_vol"], rtol=1e-12)
    assert o.scalars()["alpha0"] == pytest.approx(float(g["alpha0"]), rel=1e-12)
    for k in range(steps):
        o.advance(s.dt)
        v = o.virtual()
        assert np.array_equal(v["node"], g[f"s{k}_node"])
        for f in ("rho", "vol", "div", "alpha_hat"):
            np.testing.assert_allclose(v[f], g[f"s{k}_{f}"], rtol=1e-9, atol=1e-12 * np.abs(g[f"s{k}_{f}"]).max())
        x, vel = o.particles()
        np.testing.assert_allclose(x, g[f"s{k}_x"], rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(vel, g[f"s{k}_v"], rtol=1e-8, atol=1e-10)
