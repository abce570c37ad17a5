"""Seeded synthetic scenes for the dual-particle SPH projection.

The reference ships no scene builder for ``DualParticleSphLiquid`` (nothing in
it constructs one; the SPH builder in
Demos/SmthPartHydrodLiquidTest/SmthPartHydrodLiquidBuilder.h:28-52 only makes
WCSPH/PCISPH liquids).  These builders follow that builder's conventions:

* particle radius ``r = spacing / 2``; real and boundary kernel radius
  ``h = 4 r`` (Cores/Structures/SmoothedParticles.cpp:17);
* the virtual node grid spacing equals the particle spacing, and the virtual
  kernel radius is ``H = 4 * grid_spacing`` (Cores/Physics/DualParticleSphLiquid.h:28);
* the node grid is a StaggeredGrid node lattice:
  ``origin = center - (res + 2 bw) * spacing / 2``, ``res + 2 bw + 1`` nodes per axis
  (Cores/Structures/StaggeredGrid.cpp:20-34);
* boundary particles carry the inward normal of a complementary box
  (Cores/Geometries/Surface.h:50-69, ImplicitSurface.h:45-73) and zero velocity
  (Cores/Physics/DualParticleSphLiquid.cpp:84);
* the boundary mass equals the fluid mass (DualParticleSphLiquid.cpp:86).

The workloads are the ones the projection is benchmarked on: a 2D dam break
(40 x 80 particles at 0.01), a 3D dam break (128 x 64 x 64), an isolated 3D
projection block (128^3 = 2,097,152 particles) and a paddle tank.  Every
builder is deterministic in its seed (numpy PCG64).
"""
from __future__ import annotations

from dataclasses import dataclass, field, replace

import numpy as np


@dataclass
class Scene:
    name: str
    dim: int
    particle_radius: float
    mass: float
    boundary_mass: float
    grid_origin: tuple
    grid_spacing: float
    grid_size: tuple
    positions: np.ndarray
    velocities: np.ndarray
    boundary_positions: np.ndarray
    boundary_normals: np.ndarray
    boundary_velocities: np.ndarray
    gravity: tuple = (0.0, -9.8, 0.0)
    enable_gravity: bool = True
    viscosity: float = 0.01
    target_density: float = -1.0  # <= 0: max rho_i at initialize (reference)
    kappa: float = -1.0  # < 0: 1 / packed kernel sum (reference)
    dt: float = 1e-3
    steps: int = 1
    tolerance: float = 1e-6
    seed: int = 0
    meta: dict = field(default_factory=dict)

    @property
    def n_particles(self) -> int:
        return int(self.positions.shape[0])

    @property
    def n_boundary(self) -> int:
        return int(self.boundary_positions.shape[0])

    @property
    def n_nodes(self) -> int:
        return int(np.prod(self.grid_size[: self.dim]))

    def copy(self, **kw) -> "Scene":
        s = replace(self, **kw)
        for k in ("positions", "velocities", "boundary_positions", "boundary_normals", "boundary_velocities"):
            if k not in kw:
                setattr(s, k, getattr(self, k).copy())
        return s

    def rounded_to_float32(self) -> "Scene":
        """Same scene with every array rounded through float32 (the GPU state type)."""
        f = lambda a: a.astype(np.float32).astype(np.float64)
        return self.copy(
            positions=f(self.positions),
            velocities=f(self.velocities),
            boundary_positions=f(self.boundary_positions),
            boundary_normals=f(self.boundary_normals),
            boundary_velocities=f(self.boundary_velocities),
        )


def staggered_node_grid(boundary_width: int, spacing: float, resolution, center):
    """Node lattice of StaggeredGrid(bw, spacing, resolution, center)
    (Cores/Structures/StaggeredGrid.cpp:20-34): returns (origin, node counts)."""
    res = np.asarray(resolution, dtype=np.int64) + 2 * boundary_width
    origin = np.asarray(center, dtype=np.float64) - res.astype(np.float64) * spacing / 2
    return tuple(float(v) for v in origin), tuple(int(v) + 1 for v in res)


def box_inward_normals(points: np.ndarray, lo, hi) -> np.ndarray:
    """closestNormal of ComplementarySurface(ImplicitBox(lo, hi - lo)) for points
    outside the box: minus the outward box normal (Surface.h:64-68, ImplicitSurface.h:57-66)."""
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    c = (lo + hi) / 2
    half = (hi - lo) / 2
    d = points - c
    phi = np.abs(d) - half
    inside = np.all(phi <= 0, axis=1)
    n = np.maximum(phi, 0.0)
    if np.any(inside):
        ax = np.argmax(phi[inside], axis=1)
        m = np.zeros_like(phi[inside])
        m[np.arange(m.shape[0]), ax] = 1.0
        n[inside] = m
    n = n * np.sign(d)
    nrm = np.linalg.norm(n, axis=1, keepdims=True)
    nrm[nrm == 0] = 1.0
    return -(n / nrm)


def lattice_block(counts, spacing, offset=None):
    """Cell-centred lattice points ((i + 0.5) * spacing + offset), x fastest."""
    counts = tuple(int(c) for c in counts)
    axes = [(np.arange(c) + 0.5) * spacing for c in counts]
    grids = np.meshgrid(*axes[::-1], indexing="ij")[::-1]
    pts = np.stack([g.ravel() for g in grids], axis=1)
    if offset is not None:
        pts = pts + np.asarray(offset, dtype=np.float64)
    return pts


def box_wall_layers(cells, spacing, layers):
    """`layers` layers of lattice particles around the box [0, cells * spacing],
    same spacing as the fluid, with inward normals."""
    cells = np.asarray(cells, dtype=np.int64)
    dim = cells.shape[0]
    full = lattice_block(cells + 2 * layers, spacing, offset=-layers * spacing * np.ones(dim))
    idx = np.floor(full / spacing + 1e-9).astype(np.int64)
    outside = np.any((idx < 0) | (idx >= cells), axis=1)
    pts = full[outside]
    normals = box_inward_normals(pts, np.zeros(dim), cells * spacing)
    return pts, normals


def _finish(name, dim, spacing, pos, vel, bpos, bnrm, grid_origin, grid_size, **kw):
    r = spacing / 2
    rho0 = 1000.0
    mass = rho0 * spacing**dim
    gsize = tuple(grid_size) + (1,) * (3 - dim)
    gorig = tuple(grid_origin) + (0.0,) * (3 - dim)
    return Scene(
        name=name,
        dim=dim,
        particle_radius=r,
        mass=mass,
        boundary_mass=mass,
        grid_origin=gorig,
        grid_spacing=spacing,
        grid_size=gsize,
        positions=pos,
        velocities=vel,
        boundary_positions=bpos,
        boundary_normals=bnrm,
        boundary_velocities=np.zeros_like(bpos),
        **kw,
    )


def dam_break_2d(seed: int = 0, height_cells: int = 80, width_cells: int = 40, spacing: float = 0.01,
                 jitter: float = 1e-4, steps: int = 200) -> Scene:
    """2D dam break: block 0.4 x 0.8 in the bottom-left corner of [0,1]^2 at
    spacing 0.01 (3200 particles), uniform +-1e-4 jitter, two wall layers,
    m = rho0 spacing^2, kappa = m / rho0, gravity -9.8, dt 1e-3, tol 1e-6."""
    rng = np.random.default_rng(seed)
    pos = lattice_block((width_cells, height_cells), spacing)
    pos = pos + rng.uniform(-jitter, jitter, size=pos.shape)
    vel = np.zeros_like(pos)
    dom = int(round(1.0 / spacing))
    bpos, bnrm = box_wall_layers((dom, dom), spacing, 2)
    origin, size = staggered_node_grid(3, spacing, (dom, dom), (0.5, 0.5))
    s = _finish("dam_break_2d", 2, spacing, pos, vel, bpos, bnrm, origin, size,
                dt=1e-3, steps=steps, tolerance=1e-6, seed=seed)
    s.kappa = s.mass / 1000.0
    s.gravity = (0.0, -9.8, 0.0)
    return s


def dam_break_3d(seed: int = 0, cells=(128, 64, 64), spacing: float = 0.01, jitter: float = 1e-4,
                 domain=(2.0, 1.0, 1.0), steps: int = 100) -> Scene:
    """3D dam break: domain [0,2]x[0,1]x[0,1], fluid block 1.28 (x) x 0.64 x 0.64
    at spacing 0.01 (524,288 particles) in the corner, +-1e-4 jitter, two wall
    layers, dt 5e-4, tol 1e-5.  (The 1.28 extent only fits along x.)"""
    rng = np.random.default_rng(seed)
    pos = lattice_block(cells, spacing)
    pos = pos + rng.uniform(-jitter, jitter, size=pos.shape)
    vel = np.zeros_like(pos)
    dom = tuple(int(round(d / spacing)) for d in domain)
    bpos, bnrm = box_wall_layers(dom, spacing, 2)
    center = tuple(d / 2 for d in domain)
    origin, size = staggered_node_grid(3, spacing, dom, center)
    return _finish("dam_break_3d", 3, spacing, pos, vel, bpos, bnrm, origin, size,
                   dt=5e-4, steps=steps, tolerance=1e-5, seed=seed)


def projection_block_3d(n: int = 128, seed: int = 0, spacing: float = 0.01, sigma: float = 0.1,
                        steps: int = 50) -> Scene:
    """Isolated projection benchmark: n^3 fluid particles (128^3 = 2,097,152) at
    spacing 0.01 with U(+-0.1 spacing) jitter, velocities N(0, sigma^2) per
    component, two boundary layers on all six faces (132^3 - 128^3 = 202,816
    for n = 128), dt 5e-4 with gravity, tol 1e-5."""
    rng = np.random.default_rng(seed)
    pos = lattice_block((n, n, n), spacing)
    pos = pos + rng.uniform(-0.1 * spacing, 0.1 * spacing, size=pos.shape)
    vel = rng.normal(0.0, sigma, size=pos.shape)
    bpos, bnrm = box_wall_layers((n, n, n), spacing, 2)
    origin, size = staggered_node_grid(3, spacing, (n, n, n), (n * spacing / 2,) * 3)
    return _finish(f"projection_block_3d_n{n}", 3, spacing, pos, vel, bpos, bnrm, origin, size,
                   dt=5e-4, steps=steps, tolerance=1e-5, seed=seed)


def projection_block_2d(n: int = 64, seed: int = 0, spacing: float = 0.01, sigma: float = 0.1,
                        steps: int = 10) -> Scene:
    """2D counterpart of the projection block (small parity case)."""
    rng = np.random.default_rng(seed)
    pos = lattice_block((n, n), spacing)
    pos = pos + rng.uniform(-0.1 * spacing, 0.1 * spacing, size=pos.shape)
    vel = rng.normal(0.0, sigma, size=pos.shape)
    bpos, bnrm = box_wall_layers((n, n), spacing, 2)
    origin, size = staggered_node_grid(3, spacing, (n, n), (n * spacing / 2,) * 2)
    return _finish(f"projection_block_2d_n{n}", 2, spacing, pos, vel, bpos, bnrm, origin, size,
                   dt=5e-4, steps=steps, tolerance=1e-5, seed=seed)


def dam_break_3d_variant(seed: int, height: float, target_particles: int = 400_000,
                         spacing: float = 0.01) -> Scene:
    """Dam-break variant used to log learned-warm-start training data: block of
    height `height` along x, square cross-section sized so N ~ target_particles."""
    nx = int(round(height / spacing))
    side = max(8, int(round(np.sqrt(target_particles / nx))))
    dom_x = max(2.0, (nx + 40) * spacing)
    dom_yz = max(1.0, (side + 40) * spacing)
    return dam_break_3d(seed=seed, cells=(nx, side, side), spacing=spacing,
                        domain=(dom_x, dom_yz, dom_yz))


def paddle_tank_3d(seed: int = 0, spacing: float = 0.01, n_fluid: int = 8_388_608, cells=None,
                   domain=(4.0, 2.0, 2.0), paddle_particles: int = 1_000_000,
                   paddle_half=(0.05, 0.5, 0.25), omega: float = 2.0, steps: int = 100) -> Scene:
    """Largest scene: tank [0,4]x[0,2]x[0,2] (y up) filled from the floor with
    n_fluid = 8,388,608 fluid particles on the lattice of spacing 0.01 (400 x 200
    points per layer, about 105 layers, the top one partial) with seeded +-1e-4
    jitter, walls of two layers, and about 1M solid particles sampled uniformly
    inside a paddle blade centred in the tank, 0.1 thick (x) x 1.0 tall (y) x 0.5
    wide (z), rotating at 2 rad/s about the vertical (y) axis through its centre.
    Paddle particles carry the rigid velocity omega x (x - c); their normals point
    away from the blade's mid-plane (along x before rotation).  Lattice points inside
    the blade are left out and further points fill the count.

    `cells` instead places a block of that many lattice points in the tank's
    corner (small test tanks).  The fluid must lie inside the tank: particles
    beyond its walls would sit outside the node lattice."""
    rng = np.random.default_rng(seed)
    dom = tuple(int(round(d / spacing)) for d in domain)
    c = np.array(domain, dtype=np.float64) / 2
    ph = np.asarray(paddle_half, dtype=np.float64)

    def outside_blade(p):
        return ~np.all(np.abs(p - c) < ph + spacing / 2, axis=1)

    if cells is not None:
        if any(int(n) > d for n, d in zip(cells, dom)):
            raise ValueError(f"fluid block {tuple(cells)} does not fit the tank's {dom} lattice cells")
        pos = lattice_block(cells, spacing)
        pos = pos + rng.uniform(-1e-4, 1e-4, size=pos.shape)
        pos = pos[outside_blade(pos)]
    else:
        layer = lattice_block((dom[0], 1, dom[2]), spacing)  # one y layer, x fastest
        parts, count, k = [], 0, 0
        while count < n_fluid:
            if k >= dom[1]:
                raise ValueError(f"{n_fluid} fluid particles do not fit the tank")
            pts = layer + np.array([0.0, k * spacing, 0.0])
            pts = pts[outside_blade(pts)]
            parts.append(pts)
            count += pts.shape[0]
            k += 1
        pos = np.concatenate(parts)[:n_fluid]
        pos = pos + rng.uniform(-1e-4, 1e-4, size=pos.shape)
    vel = np.zeros_like(pos)
    wpos, wnrm = box_wall_layers(dom, spacing, 2)
    ppos = c + rng.uniform(-1.0, 1.0, size=(paddle_particles, 3)) * ph
    # outward normal of the blade along x (its thin axis at the default size)
    pn = np.zeros_like(ppos)
    pn[:, 0] = np.sign(ppos[:, 0] - c[0])
    pn[pn[:, 0] == 0, 0] = 1.0
    pvel = np.zeros_like(ppos)
    rel = ppos - c
    pvel[:, 0] = omega * rel[:, 2]
    pvel[:, 2] = -omega * rel[:, 0]
    bpos = np.concatenate([wpos, ppos])
    bnrm = np.concatenate([wnrm, pn])
    bvel = np.concatenate([np.zeros_like(wpos), pvel])
    origin, size = staggered_node_grid(3, spacing, dom, tuple(c))
    s = _finish("paddle_tank_3d", 3, spacing, pos, vel, bpos, bnrm, origin, size,
                dt=5e-4, steps=steps, tolerance=1e-5, seed=seed)
    s.boundary_velocities = bvel
    s.meta = {"paddle_center": tuple(c), "paddle_omega": omega, "n_walls": int(wpos.shape[0]),
              "paddle_half": tuple(ph)}
    return s


CONFIGS = {
    "dam_break_2d": dam_break_2d,
    "dam_break_3d": dam_break_3d,
    "projection_block_3d": projection_block_3d,
    "paddle_tank_3d": paddle_tank_3d,
}


# ---------------------------------------------------------------------------
# DEM sand scenes
# ---------------------------------------------------------------------------
def _round_half_away(x):
    """std::round / Eigen round: halves away from zero (numpy rounds them to even)."""
    x = np.asarray(x, dtype=np.float64)
    return np.sign(x) * np.floor(np.abs(x) + 0.5)


def packed_box(dim: int, radius: float, center, half_lengths) -> np.ndarray:
    """Shapes::generateBox without Poisson sampling (Cores/Utilities/Shapes.h:32-58), the
    same packing as BoundaryParticles::addSurface (Cores/Structures/SmoothedParticles.cpp:111-155):
    2D rows of a hexagonal lattice at spacing 2r; 3D the faces and nodes of a
    StaggeredGrid of spacing 2 sqrt(2) r (faces of axis 0, 1, 2, then nodes; x fastest)."""
    center = np.asarray(center, dtype=np.float64)[:dim]
    half = np.asarray(half_lengths, dtype=np.float64)[:dim] * np.ones(dim)
    if dim == 2:
        spacing = radius * 2
        xs = int(_round_half_away(half[0] * 2 / spacing))
        ys = int(_round_half_away((half[1] * 2 / spacing - 1) * 2 / np.sqrt(3.0) + 1))
        origin = center - np.array([xs - 1, (ys - 1.0) * np.sqrt(3.0) / 2]) * spacing / 2
        rows = []
        for j in range(ys):
            y0 = origin + np.array([0.5 if j & 1 else 0.0, j * np.sqrt(3.0) / 2]) * spacing
            i = np.arange(xs - (j & 1), dtype=np.float64)
            rows.append(np.stack([y0[0] + i * spacing, np.full(i.shape, y0[1])], axis=1))
        return np.concatenate(rows, axis=0) if rows else np.zeros((0, 2))
    spacing = 2 * np.sqrt(2.0) * radius
    res = _round_half_away((half - radius) * 2 / spacing).astype(np.int64)
    origin = center - res.astype(np.float64) * spacing / 2
    parts = []
    for axis in range(3):
        size = res + np.eye(3, dtype=np.int64)[axis]
        parts.append(_grid_points(size, origin + (1 - np.eye(3)[axis]) * spacing / 2, spacing))
    parts.append(_grid_points(res + 1, origin, spacing))
    return np.concatenate(parts, axis=0)


def _grid_points(size, off, spacing):
    """Grid::dataPosition = origin + index * spacing over the grid, x fastest
    (Cores/Structures/Grid.h:51, Grid.cpp:231-243)."""
    kz, ky, kx = np.meshgrid(np.arange(size[2]), np.arange(size[1]), np.arange(size[0]), indexing="ij")
    idx = np.stack([kx.ravel(), ky.ravel(), kz.ravel()], axis=1)
    return off + idx * spacing


def complement_box_boundary(dim: int, radius: float, box_lo, box_hi, center, half_lengths, depth=None):
    """BoundaryParticles::addSurface(ComplementarySurface(ImplicitBox(box_lo, box_hi - box_lo)),
    center, half_lengths): the packed points outside (or on) the box with its inward
    normals.  `depth` keeps only the points within that distance of the box (the
    reference keeps the whole shell; every boundary particle within 4r of the box
    has the same neighbours whenever depth >= 8r)."""
    lo = np.asarray(box_lo, dtype=np.float64)[:dim]
    hi = np.asarray(box_hi, dtype=np.float64)[:dim]
    if dim == 3 and depth is not None:
        pts = _packed_box_3d_shell(radius, center, half_lengths, lo, hi, depth)
    else:
        pts = packed_box(dim, radius, center, half_lengths)
    c, h = (lo + hi) / 2, (hi - lo) / 2
    phi = np.abs(pts - c) - h
    sd = np.where(np.all(phi <= 0, axis=1), phi.max(axis=1), np.linalg.norm(np.maximum(phi, 0), axis=1))
    keep = sd >= 0  # ComplementarySurface::isInside: -sd <= 0 (Cores/Geometries/Surface.h:68)
    if depth is not None:
        keep &= sd <= depth
    pts = pts[keep]
    return pts, box_inward_normals(pts, lo, hi)


def _packed_box_3d_shell(radius, center, half_lengths, lo, hi, depth):
    """The points of packed_box(3, ...) within `depth` outside the faces of [lo, hi],
    in the same order, without generating the interior (one slab per face and
    side, merged per sub-grid by linear index)."""
    center = np.asarray(center, dtype=np.float64)[:3]
    half = np.asarray(half_lengths, dtype=np.float64)[:3] * np.ones(3)
    spacing = 2 * np.sqrt(2.0) * radius
    res = _round_half_away((half - radius) * 2 / spacing).astype(np.int64)
    origin = center - res.astype(np.float64) * spacing / 2
    grids = [(res + np.eye(3, dtype=np.int64)[a], origin + (1 - np.eye(3)[a]) * spacing / 2) for a in range(3)]
    grids.append((res + 1, origin))
    out = []
    eps = 1e-9 * spacing
    for size, off in grids:
        keys = []
        for b in range(3):
            for side in (0, 1):
                rlo, rhi = lo - depth, hi + depth
                rlo, rhi = rlo.copy(), rhi.copy()
                if side == 0:
                    rhi[b] = lo[b]
                else:
                    rlo[b] = hi[b]
                i0 = np.maximum(np.ceil((rlo - off) / spacing - eps), 0).astype(np.int64)
                i1 = np.minimum(np.floor((rhi - off) / spacing + eps), size - 1).astype(np.int64)
                if np.any(i1 < i0):
                    continue
                ax = [np.arange(i0[a], i1[a] + 1) for a in range(3)]
                kz, ky, kx = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
                keys.append((kx + size[0] * (ky + size[1] * kz)).ravel())
        if not keys:
            continue
        k = np.unique(np.concatenate(keys))
        idx = np.stack([k % size[0], (k // size[0]) % size[1], k // (size[0] * size[1])], axis=1)
        out.append(off + idx * spacing)
    return np.concatenate(out, axis=0) if out else np.zeros((0, 3))


@dataclass
class SandScene:
    name: str
    dim: int
    radius: float
    mass: float
    positions: np.ndarray
    velocities: np.ndarray
    boundary_positions: np.ndarray
    boundary_normals: np.ndarray
    enable_gravity: bool = True
    young: float = 1e9
    poisson: float = 0.3
    fric_angle: float = 0.5
    dt: float = 1e-4
    meta: dict = field(default_factory=dict)

    @property
    def n_particles(self) -> int:
        return int(self.positions.shape[0])

    @property
    def n_boundary(self) -> int:
        return int(self.boundary_positions.shape[0])


def rotate_velocities(pos: np.ndarray, omega: float, center=None) -> np.ndarray:
    """Shapes::generateRotate (Cores/Utilities/Shapes.h:95-101): v = omega (y - c_y) e_x - omega (x - c_x) e_y."""
    c = np.zeros(pos.shape[1]) if center is None else np.asarray(center, dtype=np.float64)[: pos.shape[1]]
    v = np.zeros_like(pos)
    v[:, 0] = omega * (pos[:, 1] - c[1])
    v[:, 1] = -omega * (pos[:, 0] - c[0])
    return v


def sand_rotating_box(dim: int = 2, scale: int = 30, omega: float = 2.0, length: float = 1.0, wall_depth=None,
                      density: float = 1000.0) -> SandScene:
    """DEMParticleSandBuilder case 0 (Demos/DEMParticleSandTest/DEMParticleSandBuilder.h:25-57):
    r = length / 2 / scale / 2, a packed box of half-length length / 8 at the origin
    rotating at omega, mass density / N, the boundary shell of the box
    [-length/2, length/2]^dim sampled over half-length 1.2 length (`wall_depth`
    trims it to the layers within that distance of the box)."""
    r = length / 2 / scale / 2
    pos = packed_box(dim, r, np.zeros(dim), np.ones(dim) * length / 8)
    vel = rotate_velocities(pos, omega)
    bpos, bnrm = complement_box_boundary(dim, r, -length / 2 * np.ones(dim), length / 2 * np.ones(dim), np.zeros(dim),
                                         np.ones(dim) * length * 1.2, depth=wall_depth)
    return SandScene(name=f"sand_rotating_box_{dim}d_s{scale}", dim=dim, radius=r, mass=density / pos.shape[0],
                     positions=pos, velocities=vel, boundary_positions=bpos, boundary_normals=bnrm,
                     meta={"scale": scale, "omega": omega, "wall_depth": wall_depth})


def sand_contact_block(dim: int = 2, scale: int = 30, seed: int = 0, squeeze: float = 0.99, jitter: float = 0.05,
                       sigma: float = 0.05, length: float = 1.0, wall_depth=None) -> SandScene:
    """The builder's packed block squeezed by `squeeze` (every touching pair then
    overlaps by (1 - squeeze) 2r), jittered by U(+-jitter r), with N(0, sigma) velocities,
    set down in the corner of the container 1.5 r from the floor and the x = -length/2
    wall: contacts, Coulomb caps and boundary friction act from the first step."""
    base = sand_rotating_box(dim, scale, omega=0.0, length=length, wall_depth=wall_depth)
    r = base.radius
    rng = np.random.default_rng(seed)
    pos = base.positions * squeeze + rng.uniform(-jitter * r, jitter * r, base.positions.shape)
    lo = pos.min(axis=0)
    shift = np.zeros(dim)
    shift[0] = -length / 2 + 1.5 * r - lo[0]
    shift[1] = -length / 2 + 1.5 * r - lo[1]
    pos = pos + shift
    vel = rng.normal(0.0, sigma, pos.shape)
    return SandScene(name=f"sand_contact_block_{dim}d_s{scale}", dim=dim, radius=r, mass=base.mass, positions=pos,
                     velocities=vel, boundary_positions=base.boundary_positions, boundary_normals=base.boundary_normals,
                     meta={"scale": scale, "seed": seed, "squeeze": squeeze, "wall_depth": wall_depth})
