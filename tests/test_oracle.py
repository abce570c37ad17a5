"""CPU checks of the FP64 oracle: analytic known answers of the reference's
kernel and lattice, and agreement with an independent brute-force restatement."""
import itertools

import numpy as np
import pytest

from bruteforce import BruteForce
from swc import scenes


def test_kernel_normalisation(oracle_mod):
    # integral of the cubic spline over its support is 1 (coefficients SmoothedParticles.cpp:19-22)
    for dim in (2, 3):
        r = 0.005
        h = 4 * r
        rs = np.linspace(0, h, 20001)
        w = np.array([oracle_mod.kernel(dim, r, x) for x in rs])
        shell = 2 * np.pi * rs if dim == 2 else 4 * np.pi * rs**2
        integral = np.trapezoid(w * shell, rs)
        assert abs(integral - 1.0) < 1e-6, (dim, integral)


def test_kernel_derivative_and_self_term(oracle_mod):
    for dim in (2, 3):
        r = 0.005
        h = 4 * r
        assert oracle_mod.kernel(dim, r, 0.0, derivative=True) == 0.0  # W'(0) = 0 -> alpha_II = 0
        assert oracle_mod.kernel(dim, r, h) == 0.0
        assert oracle_mod.kernel(dim, r, h, derivative=True) == 0.0
        # W' matches a central difference of W inside both branches
        for x in (0.2 * h, 0.45 * h, 0.7 * h, 0.95 * h):
            e = 1e-9
            fd = (oracle_mod.kernel(dim, r, x + e) - oracle_mod.kernel(dim, r, x - e)) / (2 * e)
            assert abs(fd - oracle_mod.kernel(dim, r, x, derivative=True)) < 1e-4 * abs(fd)


def test_packed_kernel_sum(oracle_mod):
    # getPackedKernelSum: hexagonal (2D) / FCC (3D) first shells (SmoothedParticles.cpp:74-80)
    for dim in (2, 3):
        r = 0.005
        k = lambda x: oracle_mod.kernel(dim, r, x)
        if dim == 2:
            expect = k(0) + 6 * k(2 * r) + 6 * k(2 * r * np.sqrt(3))
        else:
            expect = k(0) + 12 * k(2 * r) + 6 * k(2 * r * np.sqrt(2)) + 24 * k(2 * r * np.sqrt(3))
        assert oracle_mod.packed_kernel_sum(dim, r) == pytest.approx(expect, rel=1e-15)


def _lattice_scene(dim, n):
    # power-of-two spacing: lattice coordinates and distances are exact in FP64
    sp = 1.0 / 128
    s = scenes.projection_block_3d(n=n, seed=0, spacing=sp) if dim == 3 else \
        scenes.projection_block_2d(n=n, seed=0, spacing=sp)
    return s.copy(positions=scenes.lattice_block((n,) * dim, sp), velocities=np.zeros((n**dim, dim)))


@pytest.mark.parametrize("dim,count_h,count_H", [(2, 9, 45), (3, 27, 251)])
def test_lattice_neighbour_counts(oracle_mod, dim, count_h, count_H):
    # perfect lattice: |k|^2 < 4 within h = 2 spacing, |k|^2 < 16 within H = 4 spacing (strict)
    n = 12
    s = _lattice_scene(dim, n)
    o = oracle_mod.Oracle(s)
    o.initialize()
    centre = s.positions[np.argmin(np.linalg.norm(s.positions - s.positions.mean(0), axis=1))]
    counts, _, _ = o.neighbors("real", centre[None, :])
    assert counts[0] == count_h
    expect_H = sum(1 for k in itertools.product(range(-4, 5), repeat=dim) if sum(c * c for c in k) < 16)
    assert expect_H == count_H
    v = o.virtual()
    interior = v["node"][len(v["node"]) // 2]
    nx, ny = s.grid_size[0], s.grid_size[1]
    k = np.array([interior % nx, (interior // nx) % ny, interior // (nx * ny)])[:dim]
    q = np.asarray(s.grid_origin[:dim]) + k * s.grid_spacing
    cv, _, _ = o.neighbors("virtual", q[None, :])
    assert cv[0] == count_H


def test_operator_on_constant_interior(oracle_mod):
    # A c = (alpha_hat_I + sum_{J != I} alpha_IJ) c on rows whose stencil is fully active
    s = scenes.projection_block_3d(n=10, seed=3)
    o = oracle_mod.Oracle(s)
    o.initialize()
    o.project()
    v = o.virtual()
    y = o.apply_operator(np.ones_like(v["p"]))
    # the unclamped row sum is alpha_hat - (-sum alpha_IJ): clamp rows give alpha_hat - rowsum_unclamped
    assert np.all(np.isfinite(y))
    assert np.all(v["alpha_hat"] >= o.scalars()["alpha0"] - 1e-9)
    # y_I = alpha_hat_I + sum_J alpha_IJ >= 0 because alpha_hat_I >= -sum_J alpha_IJ
    assert np.all(y >= -1e-9 * np.abs(v["alpha_hat"]))


def test_cg_converges_to_tolerance(oracle_mod):
    s = scenes.dam_break_2d(seed=1, height_cells=20, width_cells=12)
    o = oracle_mod.Oracle(s)
    o.initialize()
    o.advance(s.dt)
    st = o.stats()
    assert st["status"] == 0 and st["rel_residual"] < 1e-6
    v = o.virtual()
    r = np.linalg.norm(v["div"] - o.apply_operator(v["p"])) / np.linalg.norm(v["div"])
    assert r < 2e-6


@pytest.mark.parametrize("which", ["2d", "3d"])
def test_oracle_matches_bruteforce(oracle_mod, which):
    if which == "2d":
        s = scenes.dam_break_2d(seed=4, height_cells=10, width_cells=8)
    else:
        s = scenes.projection_block_3d(n=6, seed=5)
    o = oracle_mod.Oracle(s, tolerance=1e-12)
    b = BruteForce(s, tolerance=1e-12)
    o.initialize()
    b.initialize()
    rho, vol = o.real_info()
    np.testing.assert_allclose(rho, b.rho, rtol=1e-12)
    np.testing.assert_allclose(vol, b.vol, rtol=1e-12)
    rb, vb = o.boundary_info()
    np.testing.assert_allclose(rb, b.rhob, rtol=1e-12)
    sc = o.scalars()
    assert sc["rho0"] == pytest.approx(b.rho0, rel=1e-13)
    assert sc["alpha0"] == pytest.approx(b.alpha0, rel=1e-12)
    assert sc["kappa"] == pytest.approx(b.kappa, rel=1e-13)
    for step in range(3):
        o.advance(s.dt)
        b.move_and_forces(s.dt)
        b.generate()
        ov = o.virtual()
        x, v_pre = o.particles()
        b.project(p_solve=ov["p"])
        assert np.array_equal(ov["node"], b.node)
        np.testing.assert_allclose(ov["rho"], b.rhov, rtol=1e-11)
        np.testing.assert_allclose(ov["vol"], b.volv, rtol=1e-11)
        np.testing.assert_allclose(ov["div"], b.D, rtol=1e-9, atol=1e-9 * np.abs(b.D).max())
        np.testing.assert_allclose(ov["alpha_hat"], b.ahat, rtol=1e-11)
        y = o.apply_operator(ov["p"])
        np.testing.assert_allclose(y, b.A @ ov["p"], rtol=1e-9, atol=1e-10 * np.abs(y).max())
        # the oracle's CG solution solves the brute-force system to tolerance
        res = np.linalg.norm(b.D - b.A @ ov["p"]) / np.linalg.norm(b.D)
        assert res < 1e-8  # recursive vs true residual drift of CG on the non-symmetric system
        np.testing.assert_allclose(x, b.x, rtol=1e-13, atol=1e-15)
        np.testing.assert_allclose(v_pre, b.v, rtol=1e-9, atol=1e-12)


def test_warm_start_prefix_quirk(oracle_mod):
    # the previous pressure vector (by position in the active list) is the next CG start:
    # re-projecting the same state from its own solution needs (almost) no iterations
    s = scenes.dam_break_2d(seed=2, height_cells=12, width_cells=10)
    o = oracle_mod.Oracle(s)
    o.initialize()
    o.advance(s.dt)
    x, v = o.particles()
    o.set_pressure(np.zeros(0))
    o.project()
    cold = o.stats()["iterations"]
    p_star = o.virtual()["p"].copy()
    o.set_particles(x, v)
    o.set_pressure(p_star)
    o.project()
    assert cold > 5 and o.stats()["iterations"] <= 1


@pytest.mark.parametrize("build", [lambda: scenes.dam_break_2d(seed=4),
                                   lambda: scenes.projection_block_3d(n=12, seed=4),
                                   lambda: scenes.paddle_tank_3d(seed=4, cells=(12, 6, 12), domain=(0.24, 0.12, 0.24),
                                                                 paddle_particles=400, paddle_half=(0.03, 0.01, 0.05))])
def test_cell_grid_searcher_matches_hash(oracle_mod, build):
    """The cell-grid searcher (used at full benchmark size) visits the reference
    hash grid's neighbour sets: identical sorted sets for real, boundary and
    virtual queries, and every field of two advance steps equal up to FP64
    rounding of the changed summation order."""
    s = build().rounded_to_float32()
    out = {}
    for kind in ("hash", "cells"):
        o = oracle_mod.Oracle(s, searcher=kind)
        if "paddle_omega" in s.meta:
            moving = np.zeros(s.n_boundary, np.uint8)
            moving[s.meta["n_walls"]:] = 1
            o.set_boundary_motion(moving, s.meta["paddle_center"], s.meta["paddle_omega"])
        o.initialize()
        for _ in range(2):
            o.advance(s.dt)
        rng = np.random.default_rng(0)
        x, v = o.particles()
        q = np.concatenate([x[rng.choice(len(x), 200)] + rng.uniform(-0.03, 0.03, (200, s.dim)), x[:50]])
        nbr = {w: o.neighbors(w, q) for w in ("real", "boundary", "virtual")}
        out[kind] = (o.virtual(), x, v, nbr, o.stats())
    (vh, xh, velh, nh, sh), (vc, xc, velc, nc, sc) = out["hash"], out["cells"]
    for w in nh:
        for a, b in zip(nh[w], nc[w]):
            assert np.array_equal(a, b), w
    assert np.array_equal(vh["node"], vc["node"])
    for f in ("rho", "vol", "div", "alpha_hat"):
        np.testing.assert_allclose(vc[f], vh[f], rtol=1e-11, atol=1e-13 * np.abs(vh[f]).max())
    np.testing.assert_allclose(xc, xh, rtol=0, atol=1e-14)
    assert np.linalg.norm(velc - velh) / np.linalg.norm(velh) < 1e-9
    assert abs(sc["iterations"] - sh["iterations"]) <= 1


def test_hash_candidates_power_of_two_buckets(oracle_mod):
    """The reference's hash (OR of three prime products mod 2N) fills few buckets
    when 2N is a power of two: a 32^3 block (2N = 2^16) visits far more candidates
    per query than a 31^3 block, while the cell grid visits about 27 cells' worth."""
    per = {}
    for n in (31, 32):
        s = scenes.projection_block_3d(n=n, seed=0)
        o = oracle_mod.Oracle(s)
        per[n] = o.hash_candidates("real", s.positions[::7])
    # 27 cells of side h = 2 spacings hold ~27 * 8 = 216 particles
    assert per[31] < 20 * 216 < per[32], per
