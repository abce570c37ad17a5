"""GPU parity of the DEM sand step (include/swc_sand.h) against the FP64 oracle.

Tolerances: positions are float-float on the device, so they agree with the
oracle to 1e-12 absolute; velocities and forces are FP32, so a step's velocity
agrees to 2e-5 of the largest speed (an FP32 contact force is good to ~1e-6 of
its size, and the stored velocity to 6e-8 of itself).  Boundary volumes are FP32
kernel sums: 2e-6 relative."""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _f32(a):
    return np.asarray(a, dtype=np.float64).astype(np.float32).astype(np.float64)


def _pair(scene, oracle_mod, swc_mod, with_boundary=True, gravity=True):
    from swc.sand import DEMParticleSand

    v0 = _f32(scene.velocities)
    g = DEMParticleSand(scene.radius, dim=scene.dim, mass=scene.mass, enable_gravity=gravity)
    g.setParticles(scene.positions, v0)
    o = oracle_mod.DemOracle(scene.dim, scene.radius, scene.mass, enable_gravity=gravity)
    o.set_particles(scene.positions, v0)
    if with_boundary:
        g.setBoundary(scene.boundary_positions, scene.boundary_normals)
        o.set_boundary(scene.boundary_positions, scene.boundary_normals)
    g.initialize()
    o.initialize()
    return g, o


def _check_step(g, o, dt, vtol=2e-5):
    """One step from the same state on both sides; returns the velocity error / max speed."""
    x, v = g.getParticles()
    o.set_particles(x, v)
    g.advance(dt)
    o.advance(dt)
    xg, vg = g.getParticles()
    xo, vo = o.particles()
    np.testing.assert_allclose(xg, xo, rtol=0, atol=1e-12)
    scale = max(np.abs(vo).max(), 1e-3)
    err = np.abs(vg - vo).max() / scale
    assert err < vtol, f"velocity error {err:.3e} of max speed {scale:.3e}"
    return err, np.abs(vo - v).max()


@pytest.mark.parametrize("dim,scale", [(2, 30), (3, 10)])
def test_boundary_volumes(oracle_mod, swc_mod, dim, scale):
    from swc import scenes

    s = scenes.sand_rotating_box(dim, scale, wall_depth=None if dim == 2 else 12 / (4 * scale))
    g, o = _pair(s, oracle_mod, swc_mod)
    rg, vg = g.boundaryInfo()
    ro, vo = o.boundary_info()
    np.testing.assert_allclose(rg, ro, rtol=2e-6)
    np.testing.assert_allclose(vg, vo, rtol=2e-6)


@pytest.mark.parametrize("dim,scale", [(2, 30), (3, 10), (3, 16)])
def test_contact_steps_match_oracle(oracle_mod, swc_mod, dim, scale):
    """Squeezed, jittered block in the container's corner: contacts, Coulomb caps
    and boundary friction from the first step; each step from the same state."""
    from swc import scenes

    s = scenes.sand_contact_block(dim, scale=scale, seed=7, wall_depth=12 / (4 * scale))
    g, o = _pair(s, oracle_mod, swc_mod)
    moved = 0.0
    for _ in range(4):
        _, dv = _check_step(g, o, s.dt)
        moved = max(moved, dv)
    assert moved > 0.05  # the forces changed the velocities


def test_golden_fixture_on_gpu(swc_mod):
    """The committed oracle fixture, run free (no re-sync) for its four steps."""
    from swc import scenes
    from swc.sand import DEMParticleSand

    here = os.path.dirname(os.path.abspath(__file__))
    gd = np.load(os.path.join(here, "golden", "sand_contact_block_2d.npz"))
    s = scenes.sand_contact_block(2, scale=30, seed=5)
    g = DEMParticleSand(s.radius, dim=2, mass=s.mass)
    g.setParticles(gd["positions"], gd["velocities"])
    g.setBoundary(s.boundary_positions, s.boundary_normals)
    g.initialize()
    _, vol = g.boundaryInfo()
    np.testing.assert_allclose(vol, gd["bvol"], rtol=2e-6)
    for k in range(int(gd["steps"])):
        g.advance(float(gd["dt"]))
        x, v = g.getParticles()
        # free run: the FP32 velocity differences (<= 1e-4 of the speed) move positions by dt times that
        np.testing.assert_allclose(x, gd[f"s{k}_x"], rtol=0, atol=(k + 1) * 1e-4 * float(gd["dt"]) * np.abs(gd[f"s{k}_v"]).max())
        assert np.abs(v - gd[f"s{k}_v"]).max() < 1e-4 * np.abs(gd[f"s{k}_v"]).max()


def test_reference_scene_rotating_box_2d(oracle_mod, swc_mod):
    """DEMParticleSandBuilder case 0 as built (full 1.2 shell), 20 steps free-running."""
    from swc import scenes

    s = scenes.sand_rotating_box(2, 30)
    g, o = _pair(s, oracle_mod, swc_mod)
    for _ in range(20):
        g.advance(s.dt)
        o.advance(s.dt)
    xg, vg = g.getParticles()
    xo, vo = o.particles()
    np.testing.assert_allclose(xg, xo, rtol=0, atol=20 * 2e-5 * s.dt * np.abs(vo).max())
    assert np.abs(vg - vo).max() < 2e-5 * np.abs(vo).max()


def test_reference_scene_rotating_box_3d(oracle_mod, swc_mod):
    """DEMParticleSandBuilder case 0 in 3D at its default scale 30 as built: 4,631 sand
    particles and the full 1.2 shell of boundary particles; volumes, then 5 steps."""
    from swc import scenes

    s = scenes.sand_rotating_box(3, 30)
    assert s.n_particles == 4631
    g, o = _pair(s, oracle_mod, swc_mod)
    rg, vg = g.boundaryInfo()
    ro, vo = o.boundary_info()
    np.testing.assert_allclose(vg, vo, rtol=2e-6)
    for _ in range(5):
        _check_step(g, o, s.dt)


def test_without_boundary_and_gravity_momentum_is_kept(oracle_mod, swc_mod):
    """Pair forces are antisymmetric (F_ij = -F_ji), so with no boundary and no gravity
    a step leaves the total momentum unchanged; checked at 3D scale 120 (307,063 particles)."""
    from swc import scenes
    from swc.sand import DEMParticleSand

    s = scenes.sand_contact_block(3, scale=120, seed=3, wall_depth=0.0)
    assert s.n_particles == 307063
    g = DEMParticleSand(s.radius, dim=3, mass=s.mass, enable_gravity=False)
    g.setParticles(s.positions, s.velocities)
    g.initialize()
    x0, v0 = g.getParticles()
    g.advance(s.dt)
    _, v1 = g.getParticles()
    dv = v1 - v0
    assert np.abs(dv).sum() > 1.0
    drift = np.abs(dv.sum(axis=0)).max() / np.abs(dv).sum(axis=0).max()
    assert drift < 1e-5, drift


def test_edge_cases(oracle_mod, swc_mod):
    from swc import scenes
    from swc.sand import DEMParticleSand

    s = scenes.sand_contact_block(2, scale=30, seed=9, wall_depth=12 / 120)
    # a particle far outside the container (clamped into border cells), and a pair of
    # coincident particles inside the block
    x = np.concatenate([s.positions, [[30.0, -40.0]], s.positions[:1]])
    v = np.concatenate([s.velocities, [[1.0, 2.0]], [[0.3, -0.1]]])
    s2 = scenes.SandScene(name="edge", dim=2, radius=s.radius, mass=s.mass, positions=x, velocities=v,
                          boundary_positions=s.boundary_positions, boundary_normals=s.boundary_normals)
    g, o = _pair(s2, oracle_mod, swc_mod)
    for _ in range(3):
        _check_step(g, o, s.dt)
    # no sand, boundary only
    e = DEMParticleSand(s.radius, dim=2, mass=s.mass)
    e.setParticles(np.zeros((0, 2)), np.zeros((0, 2)))
    e.setBoundary(s.boundary_positions, s.boundary_normals)
    e.initialize()
    e.advance(s.dt)
    assert e.getParticles()[0].shape == (0, 2)
    # no boundary at all
    g2, o2 = _pair(s, oracle_mod, swc_mod, with_boundary=False)
    for _ in range(2):
        _check_step(g2, o2, s.dt)


def test_time_step_matches_oracle(oracle_mod, swc_mod):
    from swc import scenes

    s = scenes.sand_rotating_box(2, 30)
    g, o = _pair(s, oracle_mod, swc_mod)
    g.advance(s.dt)
    o.advance(s.dt)
    assert g.getTimeStep(10000, 0.4) == pytest.approx(o.time_step(0.4), rel=1e-6)


def test_status_codes(swc_mod):
    from swc import _lib

    L = _lib.load()
    p = _lib.SandParams()
    L.swc_sand_default_params(C.byref(p))
    h = C.c_void_p()
    assert L.swc_sand_create(C.byref(p), C.byref(h)) == _lib.SWC_OK
    try:
        assert L.swc_sand_advance(h, 1e-4) == _lib.SWC_NOT_INITIALIZED
        assert L.swc_sand_set_boundary(h, None, None, 5) == _lib.SWC_BAD_ARG
        x = np.zeros((4, 2))
        dp = x.ctypes.data_as(C.POINTER(C.c_double))
        assert L.swc_sand_set_particles(h, dp, None, 4) == _lib.SWC_OK
        assert L.swc_sand_get_particles(h, dp, None, 3) == _lib.SWC_BAD_ARG
        assert L.swc_sand_initialize(h) == _lib.SWC_OK
        assert L.swc_sand_advance(h, float("nan")) == _lib.SWC_BAD_ARG
        assert L.swc_sand_advance(h, 1e-4) == _lib.SWC_OK
    finally:
        L.swc_sand_destroy(h)
    bad = _lib.SandParams()
    L.swc_sand_default_params(C.byref(bad))
    bad.dim = 4
    assert L.swc_sand_create(C.byref(bad), C.byref(h)) == _lib.SWC_BAD_ARG


def test_frames_round_trip(tmp_path, swc_mod):
    from swc import scenes
    from swc.sand import DEMParticleSand

    s = scenes.sand_rotating_box(3, 10, wall_depth=12 / 40)
    g = DEMParticleSand.from_scene(s)
    g.initialize()
    for _ in range(3):
        g.advance(s.dt)
    x, v = g.getParticles()
    g.saveFrame(str(tmp_path / "f3"))
    g.writeFrame(str(tmp_path / "f3"))
    g.writeDescription(str(tmp_path / "description.yaml"))
    n = x.shape[0]
    assert os.path.getsize(tmp_path / "f3" / "particles.mesh") == 4 + n * (12 + 12 + 4)
    assert os.path.getsize(tmp_path / "f3" / "boundary_particles.mesh") == 4 + s.n_boundary * 24
    h = DEMParticleSand.from_scene(s)
    h.loadFrame(str(tmp_path / "f3"))
    x2, v2 = h.getParticles()
    np.testing.assert_array_equal(x2, x)
    np.testing.assert_array_equal(v2, v)
    g.advance(s.dt)
    h.advance(s.dt)
    np.testing.assert_allclose(h.getParticles()[1], g.getParticles()[1], rtol=0, atol=1e-6)
