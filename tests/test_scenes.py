"""Scene builders: particle counts and boundary normals of the benchmarked workloads."""
import numpy as np

from swc import scenes


def test_dam_break_2d_counts():
    s = scenes.dam_break_2d(seed=0)
    assert s.n_particles == 3200
    assert s.n_boundary == 104 * 104 - 100 * 100
    assert s.mass == 1000 * 0.01**2 and s.kappa == s.mass / 1000
    assert s.grid_size[:2] == (107, 107)
    assert np.all(np.abs(s.positions - scenes.lattice_block((40, 80), 0.01)) <= 1e-4)


def test_projection_block_counts():
    n = 32
    s = scenes.projection_block_3d(n=n, seed=1)
    assert s.n_particles == n**3
    assert s.n_boundary == (n + 4) ** 3 - n**3
    # 128^3 benchmark: counts only (no 2M arrays needed)
    assert 132**3 - 128**3 == 202_816 and 128**3 == 2_097_152


def test_boundary_normals_point_inward():
    s = scenes.projection_block_3d(n=8, seed=0)
    c = np.full(3, 8 * 0.01 / 2)
    nrm = s.boundary_normals
    assert np.allclose(np.linalg.norm(nrm, axis=1), 1.0)
    assert np.all(np.einsum("ij,ij->i", nrm, c - s.boundary_positions) > 0)


def test_seeded_determinism():
    a = scenes.projection_block_3d(n=8, seed=7)
    b = scenes.projection_block_3d(n=8, seed=7)
    assert np.array_equal(a.positions, b.positions) and np.array_equal(a.velocities, b.velocities)


def test_dam_break_3d_counts():
    s = scenes.dam_break_3d(seed=0, cells=(32, 16, 16), domain=(0.5, 0.25, 0.25))
    assert s.n_particles == 32 * 16 * 16
    assert s.n_boundary == 54 * 29 * 29 - 50 * 25 * 25
