"""Independent O(N^2) numpy restatement of the DEM sand step, for tiny scenes
only.  It shares no code with the C++ oracle (dense pair matrices instead of the
hash searcher) so the two check each other.

Reference behaviour restated (skytang0205/sand-water-coupling):
  contact model      Cores/Structures/DEMParticle.cpp:15-96, 126-134
  capillary bridge   DEMParticle.cpp:98-124 (never active between pairs within 2r)
  boundary friction  Cores/Physics/DEMParticleSand.cpp:130-151
  move / gravity     DEMParticleSand.cpp:90-115
  boundary volumes   Cores/Structures/SmoothedParticles.cpp:25-41 (kernel radius 4r)
Velocities of one pass are read at its start (see dem_oracle.cpp).
"""
from __future__ import annotations

import numpy as np


def kernel_W(r, h, dim):
    c0 = (1.0 / np.pi) / (h * h) * (40.0 / 7.0 if dim == 2 else 8.0 / h)
    q = r / h
    return np.where(q < 0.5, c0 * (6 * q * q * (q - 1) + 1), np.where(q < 1, 2 * c0 * (1 - q) ** 3, 0.0))


def boundary_volumes(xb, radius, mass, dim):
    d = xb[:, None, :] - xb[None, :, :]
    r2 = np.einsum("ijk,ijk->ij", d, d)
    h = 4 * radius
    w = np.where(r2 < h * h, kernel_W(np.sqrt(r2), h, dim), 0.0)
    rho = mass * w.sum(axis=1)
    return rho, mass / rho


def step(x, v, xb, nb, volb, dt, radius, young=1e9, poisson=0.3, fric_angle=0.5, gravity=True):
    n, dim = x.shape
    Kn = young * radius
    Kt = Kn * poisson
    tf = np.tan(fric_angle)
    x = x + v * dt
    d = x[None, :, :] - x[:, None, :]  # d[i, j] = x_j - x_i
    w = v[None, :, :] - v[:, None, :]
    dist = np.sqrt(np.einsum("ijk,ijk->ij", d, d))
    near = dist * dist < (2 * radius) ** 2
    pen = 2 * radius - dist
    act = near & (pen > 0)
    dc = np.where(dist <= 1e-4 * radius, 1e-4 * radius, dist)
    nvec = d / dc[:, :, None]
    dn = np.einsum("ijk,ijk->ij", w, nvec)
    normal = (Kn * pen)[:, :, None] * nvec
    shear = -Kt * (w - dn[:, :, None] * nvec)
    max_fs = np.linalg.norm(normal, axis=2) * tf
    sn = np.linalg.norm(shear, axis=2)
    scale = np.where(sn > max_fs, max_fs / np.where(sn > 0, sn, 1.0), 1.0)
    f = -normal - shear * scale[:, :, None]
    f = np.where(act[:, :, None], f, 0.0).sum(axis=1)
    force = f * dt
    if xb.shape[0]:
        db = x[:, None, :] - xb[None, :, :]
        rb = np.sqrt(np.einsum("ijk,ijk->ij", db, db))
        nearb = rb * rb < (4 * radius) ** 2
        wb = kernel_W(rb, 4 * radius, dim)
        dv = np.broadcast_to(v[:, None, :], db.shape)
        dvn = np.einsum("ijk,jk->ij", dv, nb)
        Fn = (-volb[None, :] * np.minimum(dvn, 0.0))[:, :, None] * nb[None, :, :] * wb[:, :, None]
        Ft = -Kt * (dv - dvn[:, :, None] * nb[None, :, :])
        nt = np.linalg.norm(Ft, axis=2)
        nn = np.linalg.norm(Fn, axis=2)
        k = np.where(nt <= 1e-6, 1.0, np.where(nn * tf > nt, 1.0, nn * tf / np.where(nt > 0, nt, 1.0)))
        fb = Fn + k[:, :, None] * Ft
        force = force + np.where(nearb[:, :, None], fb, 0.0).sum(axis=1)
    v = v + force
    if gravity:
        v = v.copy()
        v[:, 1] -= 9.8 * dt
    return x, v
