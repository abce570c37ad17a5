"""Independent O(N^2) numpy restatement of the dual-particle projection, for
tiny scenes only.  It shares no code with the C++ oracle (no hash grid, dense
pair matrices, dense linear algebra) so the two check each other.

Reference behaviour restated (skytang0205/sand-water-coupling):
  kernel             Cores/Structures/SmoothedParticles.h:60-72, .cpp:17-22
  densities/volumes  SmoothedParticles.cpp:25-41
  virtual particles  Cores/Structures/VirtualParticle.cpp:18-62
  vbar / D / coef    VirtualParticle.cpp:137-201
  pressure gradient  VirtualParticle.cpp:111-134
  move / viscosity   Cores/Physics/SmthParticleHydrodLiquid.cpp:72-98
"""
from __future__ import annotations

import numpy as np


def kernel_coeffs(h, dim):
    c0 = (1.0 / np.pi) * (1.0 / (h * h)) * (40.0 / 7.0 if dim == 2 else 8.0 / h)
    return c0, 6.0 / h * c0


def W(r, h, dim):
    c0, _ = kernel_coeffs(h, dim)
    q = r / h
    return np.where(q < 0.5, c0 * (6 * q * q * (q - 1) + 1), np.where(q < 1, 2 * c0 * (1 - q) ** 3, 0.0))


def dW(r, h, dim):
    _, c1 = kernel_coeffs(h, dim)
    q = r / h
    return np.where(q < 0.5, c1 * q * (3 * q - 2), np.where(q < 1, c1 * (1 - q) * (q - 1), 0.0))


def pairs(a, b, h):
    d = a[:, None, :] - b[None, :, :]
    r2 = np.einsum("ijk,ijk->ij", d, d)
    return d, np.sqrt(r2), r2 < h * h


def grad(d, r, h, dim):
    """-W'(r) d / r with zero at r = 0 (gradientKernel)."""
    with np.errstate(invalid="ignore", divide="ignore"):
        s = np.where(r > 0, -dW(r, h, dim) / np.where(r > 0, r, 1.0), 0.0)
    return s[..., None] * d


class BruteForce:
    def __init__(self, scene, tolerance=None):
        self.s = scene
        self.dim = scene.dim
        self.h = 4 * scene.particle_radius
        self.H = 4 * scene.grid_spacing
        self.m = scene.mass
        self.mb = scene.boundary_mass
        self.x = scene.positions.copy()
        self.v = scene.velocities.copy()
        self.xb = scene.boundary_positions.copy()
        self.nb_ = scene.boundary_normals.copy()
        self.vb = scene.boundary_velocities.copy()
        self.tol = scene.tolerance if tolerance is None else tolerance
        self.p = np.zeros(0)
        dim = self.dim
        nx, ny = scene.grid_size[0], scene.grid_size[1]
        nz = scene.grid_size[2] if dim == 3 else 1
        ids = np.arange(nx * ny * nz)
        k = np.stack([ids % nx, (ids // nx) % ny, ids // (nx * ny)], axis=1)[:, :dim]
        self.all_nodes = np.asarray(scene.grid_origin[:dim]) + k * scene.grid_spacing

    def densities(self):
        _, r, m = pairs(self.x, self.x, self.h)
        return self.m * np.where(m, W(r, self.h, self.dim), 0).sum(1)

    def generate(self):
        _, r, m = pairs(self.all_nodes, self.x, self.h)
        w = np.where(m, W(r, self.h, self.dim), 0).sum(1)
        act = np.nonzero(w > 1e-6)[0]
        self.node = act
        self.xv = self.all_nodes[act]
        _, r, m = pairs(self.xv, self.x, self.h)
        self.rhov = self.m * np.where(m, W(r, self.H, self.dim), 0).sum(1)
        self.volv = np.where(m, W(r, self.h, self.dim) * self.vol[None, :] ** 2, 0).sum(1)

    def matrix(self, alpha0):
        d, r, m = pairs(self.xv, self.xv, self.H)
        a = np.where(m, 2 * self.volv[None, :] * dW(r, self.H, self.dim) / (r + 1e-6), 0.0)
        diag = np.maximum(-a.sum(1), alpha0)
        A = a.copy()
        np.fill_diagonal(A, np.diag(a) + diag)
        return A, diag

    def initialize(self):
        self.rho = self.densities()
        self.vol = self.m / self.rho
        self.rho0 = self.rho.max() if self.s.target_density <= 0 else self.s.target_density
        _, r, m = pairs(self.xb, self.xb, self.h)
        self.rhob = self.mb * np.where(m, W(r, self.h, self.dim), 0).sum(1)
        self.volb = self.mb / self.rhob
        self.generate()
        _, diag = self.matrix(-1e6)
        self.alpha0 = diag.max()
        if self.s.kappa >= 0:
            self.kappa = self.s.kappa
        else:
            r0 = self.s.particle_radius
            h, dim = self.h, self.dim
            if dim == 2:
                pk = W(0.0, h, 2) + 6 * W(2 * r0, h, 2) + 6 * W(2 * r0 * np.sqrt(3), h, 2)
            else:
                pk = W(0.0, h, 3) + 12 * W(2 * r0, h, 3) + 6 * W(2 * r0 * np.sqrt(2), h, 3) + \
                    24 * W(2 * r0 * np.sqrt(3), h, 3)
            self.kappa = 1.0 / float(pk)
        self.p = np.zeros(0)

    def rhs(self):
        dim, h = self.dim, self.h
        d, r, m = pairs(self.xv, self.x, h)
        w = np.where(m, W(r, h, dim), 0)
        g = np.where(m[..., None], grad(d, r, h, dim), 0)
        db, rb, mb = pairs(self.xv, self.xb, h)
        wb = np.where(mb, W(rb, h, dim), 0)
        gb = np.where(mb[..., None], grad(db, rb, h, dim), 0)
        num = self.m * (w / self.rho[None, :]) @ self.v + self.mb * (wb / self.rhob[None, :]) @ self.vb
        den = w @ self.vol + wb @ self.volb + 1e-6
        vbar = num / den[:, None]
        div_r = np.einsum("ijk,jk,j->i", g, self.v, self.vol)
        div_b = np.einsum("ijk,jk,j->i", gb, self.vb, self.volb)
        bg_r = np.einsum("ijk,j->ik", g, self.vol)
        bg_b = np.einsum("ijk,j->ik", gb, self.volb)
        D = div_r - (vbar * bg_r).sum(1) + div_b - (vbar * bg_b).sum(1) - \
            self.kappa * np.maximum(self.rhov - self.rho0, 0) / self.rho0
        return vbar, D

    def gradient_update(self, p):
        dim = self.dim
        d, r, m = pairs(self.x, self.xv, self.H)
        g = np.where(m[..., None], grad(d, r, self.H, dim), 0)
        f = np.einsum("ijk,j->ik", g, self.volv * p)
        db, rb, mb = pairs(self.x, self.xb, self.h)
        wb = np.where(mb, W(rb, self.h, dim), 0)
        vn = np.minimum(np.einsum("jk,ijk->ij", self.nb_, self.v[:, None, :] - self.vb[None, :, :]), 0)
        f -= np.einsum("ij,j,ij,jk->ik", wb, self.volb, vn, self.nb_)
        return self.v + f

    def project(self, p_solve=None):
        """Returns the linear system and the updated velocities; solves exactly
        unless a pressure vector is given."""
        self.vbar, self.D = self.rhs()
        self.A, self.ahat = self.matrix(self.alpha0)
        n = self.xv.shape[0]
        p0 = np.zeros(n)
        k = min(n, self.p.shape[0])
        p0[:k] = self.p[:k]
        self.p0 = p0
        p = np.linalg.solve(self.A, self.D) if p_solve is None else p_solve
        self.p = p
        self.v = self.gradient_update(p)
        return p

    def move_and_forces(self, dt):
        self.x = self.x + self.v * dt
        self.rho = self.densities()
        if self.s.enable_gravity:
            self.v = self.v + np.asarray(self.s.gravity[: self.dim]) * dt
        if self.s.viscosity != 0:
            d, r, m = pairs(self.x, self.x, self.h)  # x_i - x_j
            dp = -d  # x_j - x_i
            r2 = np.einsum("ijk,ijk->ij", dp, dp)
            ok = m & (r2 > 0)
            dv = self.v[None, :, :] - self.v[:, None, :]
            with np.errstate(invalid="ignore", divide="ignore"):
                s = np.where(ok, np.einsum("ijk,ijk->ij", dv, dp) / np.where(ok, r2, 1), 0)
            g = np.where(ok[..., None], grad(dp, r, self.h, self.dim), 0)
            lapl = np.einsum("ij,ijk,j->ik", s, g, 1 / self.rho)
            self.v = self.v + self.s.viscosity * lapl * 2 * (self.dim + 2) * self.m * dt
