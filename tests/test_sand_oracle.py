"""CPU checks of the DEM sand oracle (oracle/dem_oracle.cpp): known answers of the
contact model, the boundary friction cases, the unreachable capillary branch,
agreement with the independent brute-force restatement, the golden fixture,
and the scene builders (Shapes::generateBox / BoundaryParticles::addSurface)."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden  # noqa: E402
import sand_bruteforce as B  # noqa: E402

R = 1.0 / 120  # DEMParticleSandBuilder case 0 at its default scale 30


def test_model_constants(oracle_mod):
    p = oracle_mod.dem_params(3, R)
    m = oracle_mod.dem_model(p)
    assert m["K_norm"] == pytest.approx(1e9 * R, rel=1e-15)
    assert m["K_tang"] == pytest.approx(0.3e9 * R, rel=1e-15)
    assert m["tan_fric"] == pytest.approx(np.tan(0.5), rel=1e-15)
    # G.calculate(0.1) with px1 = 0.1: t = 1, the curve's value is py1 = cmc = 1
    assert m["coeff_c"] == pytest.approx(1.0, rel=1e-15)
    vb = 4.0 / 3.0 * np.pi * R**3 * 1e-4
    theta = np.pi / 6
    assert m["v_bridge"] == pytest.approx(vb, rel=1e-14)
    assert m["d_rupture"] == pytest.approx((1 + 0.5 * theta) * (vb ** (1 / 3) + 0.1 * vb ** (2 / 3)), rel=1e-14)
    m2 = oracle_mod.dem_model(oracle_mod.dem_params(3, R, young=2e8, poisson=0.25, fric_angle=0.3))
    assert m2["K_norm"] == pytest.approx(2e8 * R) and m2["K_tang"] == pytest.approx(0.25 * 2e8 * R)
    assert m2["tan_fric"] == pytest.approx(np.tan(0.3))


@pytest.mark.parametrize("dim", [2, 3])
def test_contact_normal_only(oracle_mod, dim):
    p = oracle_mod.dem_params(dim, R)
    Kn = 1e9 * R
    n = np.zeros(dim)
    n[0] = 0.6
    n[1] = 0.8
    for gap in (0.999, 0.9, 0.5):
        d = n * 2 * R * gap
        f, cap = oracle_mod.dem_pair_force(p, d, np.zeros(dim))
        np.testing.assert_allclose(f, -Kn * 2 * R * (1 - gap) * n, rtol=1e-13)
        assert not cap.any()
    f, _ = oracle_mod.dem_pair_force(p, n * 2 * R * 1.0001, np.zeros(dim))  # no overlap
    assert not f.any()


def test_contact_shear_below_and_at_the_cap(oracle_mod):
    p = oracle_mod.dem_params(3, R)
    Kn, Kt, tf = 1e9 * R, 0.3e9 * R, np.tan(0.5)
    d = np.array([2 * R * 0.99, 0.0, 0.0])
    pen = 2 * R * 0.01
    cap = Kn * pen * tf
    # tangential relative velocity small enough to stay under the Coulomb cap
    wt = 0.5 * cap / Kt
    f, _ = oracle_mod.dem_pair_force(p, d, [0.3, wt, 0.0])
    np.testing.assert_allclose(f, [-Kn * pen, Kt * wt, 0.0], rtol=1e-12)
    # far above: the shear is scaled to the cap, direction kept
    f, _ = oracle_mod.dem_pair_force(p, d, [0.0, 3.0, -4.0])
    np.testing.assert_allclose(f, [-Kn * pen, cap * 0.6, -cap * 0.8], rtol=1e-12)


def test_contact_distance_clamp(oracle_mod):
    """dist <= 1e-4 r: the penetration uses the true distance, the normal the clamped one."""
    p = oracle_mod.dem_params(2, R)
    Kn = 1e9 * R
    d = np.array([1e-6 * R, 0.0])
    f, _ = oracle_mod.dem_pair_force(p, d, np.zeros(2))
    n = d / (1e-4 * R)
    np.testing.assert_allclose(f, -Kn * (2 * R - 1e-6 * R) * n, rtol=1e-12)
    f0, _ = oracle_mod.dem_pair_force(p, np.zeros(2), np.array([1.0, 2.0]))  # coincident: no direction, no force
    assert not f0.any()


def test_capillary_formula_and_unreachable_branch(oracle_mod):
    p = oracle_mod.dem_params(3, R)
    m = oracle_mod.dem_model(p)
    theta, vb, c = np.pi / 6, m["v_bridge"], m["coeff_c"]
    H = 0.5 * m["d_rupture"]
    d = np.array([0.0, 2 * R + H, 0.0])
    _, cap = oracle_mod.dem_pair_force(p, d, np.zeros(3))
    dd = -H + np.sqrt(H * H + vb / (np.pi * R))
    phi = np.sqrt(2 * H / R * (-1 + np.float32(np.sqrt(np.float32(1 + vb / (np.pi * R * H * H))))))
    s = -2 * np.pi * c * R * np.cos(theta) / (1 + H / (2 * dd)) - 2 * np.pi * c * R * phi * np.sin(theta)
    np.testing.assert_allclose(cap, [0.0, -s, 0.0], rtol=1e-6)
    assert cap[1] > 0  # the bridge pulls i towards j
    # beyond the rupture distance, and for every pair the searcher visits (|d| < 2r), nothing
    _, cap = oracle_mod.dem_pair_force(p, [0.0, 2 * R + 1.01 * m["d_rupture"], 0.0], np.zeros(3))
    assert not cap.any()
    rng = np.random.default_rng(0)
    for _ in range(200):
        d = rng.normal(size=3)
        d *= rng.uniform(0, 2 * R) / np.linalg.norm(d)
        _, cap = oracle_mod.dem_pair_force(p, d, rng.normal(size=3))
        assert not cap.any()


def test_boundary_friction_cases(oracle_mod):
    p = oracle_mod.dem_params(3, R)
    Kt, tf = 0.3e9 * R, np.tan(0.5)
    nb = np.array([0.0, 1.0, 0.0])
    # moving into the wall with a tiny tangential part: |F_t| <= 1e-6 adds it in full
    dv = np.array([1e-13, -2.0, 0.0])
    f = oracle_mod.dem_boundary_term(p, dv, nb, 3.0, 5.0)
    np.testing.assert_allclose(f, [-Kt * 1e-13, 3.0 * 2.0 * 5.0, 0.0], rtol=1e-12)
    # tangential sliding, pressed into the wall: the friction is capped at |F_n| tan
    dv = np.array([1.0, -2.0, 0.0])
    f = oracle_mod.dem_boundary_term(p, dv, nb, 3.0, 5.0)
    Fn = 30.0
    np.testing.assert_allclose(f, [-Fn * tf, Fn, 0.0], rtol=1e-12)
    # moving away from the wall: no normal term, so the friction cap is zero
    f = oracle_mod.dem_boundary_term(p, np.array([1.0, 2.0, 0.0]), nb, 3.0, 5.0)
    np.testing.assert_allclose(f, 0.0, atol=1e-300)


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_matches_bruteforce(oracle_mod, dim):
    from swc import scenes

    s = scenes.sand_contact_block(dim, scale=30 if dim == 2 else 10, seed=2, wall_depth=12 * (1 / 120 if dim == 2 else 1 / 40))
    o = oracle_mod.DemOracle(dim, s.radius, s.mass)
    o.set_particles(s.positions, s.velocities)
    o.set_boundary(s.boundary_positions, s.boundary_normals)
    o.initialize()
    rho, vol = o.boundary_info()
    # brute-force volumes of the boundary particles near the sand corner (their 4r
    # neighbourhoods lie inside the selection)
    corner = -0.5 * np.ones(dim)
    far = np.linalg.norm(s.boundary_positions - corner, axis=1)
    sel = far < 0.3
    inner = far < 0.3 - 4.01 * s.radius
    rb, vb = B.boundary_volumes(s.boundary_positions[sel], s.radius, s.mass, dim)
    np.testing.assert_allclose(rho[sel][inner[sel]], rb[inner[sel]], rtol=1e-12)
    # every boundary particle within 4r (+ the steps' travel) of the sand block's box
    lo, hi = s.positions.min(axis=0), s.positions.max(axis=0)
    gap = np.linalg.norm(np.maximum(np.maximum(lo - s.boundary_positions, s.boundary_positions - hi), 0), axis=1)
    near = gap < 5 * s.radius
    x, v = s.positions.copy(), s.velocities.copy()
    for _ in range(3):
        o.advance(s.dt)
        x, v = B.step(x, v, s.boundary_positions[near], s.boundary_normals[near], vol[near], s.dt, s.radius)
        xo, vo = o.particles()
        np.testing.assert_allclose(xo, x, rtol=0, atol=1e-14)
        np.testing.assert_allclose(vo, v, rtol=0, atol=1e-11 * np.abs(v).max())
    assert np.abs(v - s.velocities).max() > 0.01  # contacts acted


def test_oracle_reproduces_sand_golden(oracle_mod):
    name = "sand_contact_block_2d"
    g = np.load(os.path.join(HERE, "golden", name + ".npz"))
    build, steps = make_golden.SAND_CASES[name]
    s = build()
    np.testing.assert_array_equal(s.positions, g["positions"])
    np.testing.assert_array_equal(s.velocities.astype(np.float32).astype(np.float64), g["velocities"])
    o = oracle_mod.DemOracle(s.dim, s.radius, s.mass)
    o.set_particles(g["positions"], g["velocities"])
    o.set_boundary(s.boundary_positions, s.boundary_normals)
    o.initialize()
    rho, vol = o.boundary_info()
    np.testing.assert_allclose(rho, g["brho"], rtol=1e-12)
    np.testing.assert_allclose(vol, g["bvol"], rtol=1e-12)
    for k in range(steps):
        o.advance(float(g["dt"]))
        x, v = o.particles()
        np.testing.assert_allclose(x, g[f"s{k}_x"], rtol=0, atol=1e-14)
        np.testing.assert_allclose(v, g[f"s{k}_v"], rtol=0, atol=1e-10 * np.abs(g[f"s{k}_v"]).max())


def test_time_step(oracle_mod):
    o = oracle_mod.DemOracle(2, R)
    o.set_particles(np.zeros((3, 2)), np.array([[0.0, 1.0], [3.0, 4.0], [-1.0, 0.0]]))
    assert o.time_step(0.4) == pytest.approx(0.4 * 2 * R / 5.0, rel=1e-15)


def test_packed_box_matches_generate_box():
    from swc import scenes

    # 2D: rows of round(2 hx / 2r) and round(2 hx / 2r) - 1 points, row pitch sqrt(3) r
    pts = scenes.packed_box(2, R, [0.0, 0.0], [0.125, 0.125])
    xs = int(np.floor(0.25 / (2 * R) + 0.5))
    ys = int(np.floor((0.25 / (2 * R) - 1) * 2 / np.sqrt(3) + 1 + 0.5))
    assert pts.shape[0] == sum(xs - (j & 1) for j in range(ys))
    np.testing.assert_allclose(pts.mean(axis=0)[0], 0.0, atol=1e-12)
    # 3D: faces of three axes then nodes of the staggered grid, nearest distance 2r
    pts = scenes.packed_box(3, R, [0.0, 0.0, 0.0], [0.125] * 3)
    res = int(np.floor((0.125 - R) * 2 / (2 * np.sqrt(2) * R) + 0.5))
    assert pts.shape[0] == 3 * res * res * (res + 1) + (res + 1) ** 3
    from scipy.spatial import cKDTree

    dd, _ = cKDTree(pts).query(pts, 2)
    np.testing.assert_allclose(dd[:, 1], 2 * R, rtol=1e-12)
    # std::round semantics: 2.5 -> 3 (numpy would give 2)
    assert scenes._round_half_away(2.5) == 3.0 and scenes._round_half_away(-2.5) == -3.0


def test_complement_box_boundary_normals_point_into_the_box():
    from swc import scenes

    pts, nrm = scenes.complement_box_boundary(2, R, [-0.5, -0.5], [0.5, 0.5], [0.0, 0.0], [0.6, 0.6])
    assert pts.shape[0] > 0
    assert np.all(np.any(np.abs(pts) >= 0.5 - 1e-12, axis=1))  # outside or on the box
    # stepping along the normal moves towards the box
    inward = np.abs(pts + 0.01 * nrm).max(axis=1) < np.abs(pts).max(axis=1)
    assert inward.all()
    np.testing.assert_allclose(np.linalg.norm(nrm, axis=1), 1.0, rtol=1e-12)
    deep, _ = scenes.complement_box_boundary(2, R, [-0.5, -0.5], [0.5, 0.5], [0.0, 0.0], [0.6, 0.6], depth=8 * R)
    assert 0 < deep.shape[0] < pts.shape[0]


def test_rotating_box_builder():
    from swc import scenes

    s = scenes.sand_rotating_box(2, 30)
    assert s.radius == pytest.approx(1 / 120)
    assert s.mass == pytest.approx(1000.0 / s.n_particles)
    np.testing.assert_allclose(s.velocities[:, 0], 2.0 * s.positions[:, 1])
    np.testing.assert_allclose(s.velocities[:, 1], -2.0 * s.positions[:, 0])
    assert s.boundary_positions.min() < -1.1 and s.boundary_positions.max() > 1.1  # the builder's 1.2 shell
