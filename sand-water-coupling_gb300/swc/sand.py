"""DEMParticleSand over the C ABI of include/swc_sand.h.

Mirrors the reference's Simulation interface for the DEM sand solver
(Cores/Physics/DEMParticleSand.h:13-58): ``initialize``, ``advance``,
``getTimeStep``, ``writeDescription``, ``writeFrame``, ``saveFrame``,
``loadFrame``, ``addShape`` and the DEMParticle setters ``setYoung``,
``setPoisson``, ``setfricangle`` (Cores/Structures/DEMParticle.h:96-103).
Every call runs on the GPU; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import struct

import numpy as np

from . import _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def _f64(a, dim):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1, dim))


class DEMParticleSand:
    def __init__(self, particle_radius, dim=2, mass=1.0, enable_gravity=True, young=1e9, poisson=0.3,
                 fric_angle=0.5):
        self.L = _lib.load()
        p = _lib.SandParams()
        self.L.swc_sand_default_params(C.byref(p))
        p.dim, p.enable_gravity, p.radius, p.mass = int(dim), 1 if enable_gravity else 0, float(particle_radius), float(mass)
        p.young, p.poisson, p.fric_angle = float(young), float(poisson), float(fric_angle)
        self._params = p
        self.dim = int(dim)
        self.h = C.c_void_p()
        self._check(self.L.swc_sand_create(C.byref(p), C.byref(self.h)), "swc_sand_create")
        self.n = 0
        self.boundary_positions = np.zeros((0, self.dim))
        self.boundary_normals = np.zeros((0, self.dim))
        self._initialized = False

    @classmethod
    def from_scene(cls, scene):
        s = cls(scene.radius, dim=scene.dim, mass=scene.mass, enable_gravity=scene.enable_gravity, young=scene.young,
                poisson=scene.poisson, fric_angle=scene.fric_angle)
        s.setParticles(scene.positions, scene.velocities)
        s.setBoundary(scene.boundary_positions, scene.boundary_normals)
        return s

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.swc_sand_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, where):
        if rc != _lib.SWC_OK:
            detail = self.L.swc_sand_last_error(self.h).decode() if getattr(self, "h", None) and self.h.value else ""
            raise _lib.SwcError(rc, where, detail)

    # -- state ------------------------------------------------------------
    def dimension(self):
        return self.dim

    def setParticles(self, x, v=None):
        x = _f64(x, self.dim)
        v = None if v is None else _f64(v, self.dim)
        self._check(self.L.swc_sand_set_particles(self.h, _dp(x), _dp(v), x.shape[0]), "swc_sand_set_particles")
        self.n = x.shape[0]

    def getParticles(self):
        x = np.zeros((self.n, self.dim))
        v = np.zeros((self.n, self.dim))
        self._check(self.L.swc_sand_get_particles(self.h, _dp(x), _dp(v), self.n), "swc_sand_get_particles")
        return x, v

    def addShape(self, positions, velocities):
        """DEMParticleSand::addShape (DEMParticleSand.cpp:167-175): appends particles."""
        x, v = self.getParticles() if self.n else (np.zeros((0, self.dim)), np.zeros((0, self.dim)))
        self.setParticles(np.concatenate([x, _f64(positions, self.dim)]), np.concatenate([v, _f64(velocities, self.dim)]))

    def setBoundary(self, x, normals):
        x = _f64(x, self.dim)
        nrm = _f64(normals, self.dim)
        self._check(self.L.swc_sand_set_boundary(self.h, _dp(x), _dp(nrm), x.shape[0]), "swc_sand_set_boundary")
        self.boundary_positions, self.boundary_normals = x.copy(), nrm.copy()
        self._initialized = False

    def setYoung(self, k):
        self._reparam(young=k)

    def setPoisson(self, k):
        self._reparam(poisson=k)

    def setfricangle(self, k):
        self._reparam(fric_angle=k)

    def _reparam(self, **kw):
        """The contact constants are fixed at creation: a new context takes the state over."""
        was_initialized = self._initialized
        x, v = self.getParticles() if self.n else (None, None)
        p = self._params
        for k, val in kw.items():
            setattr(p, k, float(val))
        self.close()
        self._check(self.L.swc_sand_create(C.byref(p), C.byref(self.h)), "swc_sand_create")
        if x is not None:
            self.setParticles(x, v)
        if self.boundary_positions.shape[0]:
            self.setBoundary(self.boundary_positions, self.boundary_normals)
        if was_initialized:
            self.initialize()

    def boundaryInfo(self):
        nb = self.boundary_positions.shape[0]
        rho, vol = np.zeros(nb), np.zeros(nb)
        self._check(self.L.swc_sand_get_boundary_info(self.h, _dp(rho), _dp(vol), nb), "swc_sand_get_boundary_info")
        return rho, vol

    # -- Simulation interface ---------------------------------------------
    def initialize(self):
        self._check(self.L.swc_sand_initialize(self.h), "swc_sand_initialize")
        self._initialized = True

    def advance(self, dt):
        self._check(self.L.swc_sand_advance(self.h, float(dt)), "swc_sand_advance")

    def getTimeStep(self, frameRate, stepRate):
        """stepRate * 2r / max|v| (DEMParticleSand.h:38-40); frameRate is unused there too."""
        dt = C.c_double()
        self._check(self.L.swc_sand_get_time_step(self.h, float(stepRate), C.byref(dt)), "swc_sand_get_time_step")
        return dt.value

    def timeKernel(self, which, reps=20):
        ms = C.c_double()
        self._check(self.L.swc_sand_time_kernel(self.h, int(which), int(reps), C.byref(ms)), "swc_sand_time_kernel")
        return ms.value

    def setStream(self, stream_handle):
        self._check(self.L.swc_sand_set_stream(self.h, C.c_void_p(stream_handle)), "swc_sand_set_stream")

    def writeDescription(self, root_path):
        """description.yaml objects of DEMParticleSand::writeDescription (DEMParticleSand.cpp:7-28)."""
        albedo = [52 / 255, 108 / 255, 156 / 255, 1.0]
        lines = [f"dimension: {self.dim}", "objects:"]
        for name, cmap in (("particles", True), ("boundary_particles", False)):
            lines += [f"  - name: {name}", "    data_mode: dynamic", "    primitive_type: point_list",
                      "    material:", f"      diffuse_albedo: [{', '.join(f'{a:.9g}' for a in albedo)}]",
                      "    indexed: false", "    color_map:", f"      enabled: {'true' if cmap else 'false'}"]
        with open(root_path, "w") as f:
            f.write("\n".join(lines) + "\n")

    def _write_mesh(self, path, pos, scalar):
        n = pos.shape[0]
        with open(path, "wb") as f:
            f.write(struct.pack("<I", n))
            f.write(np.ascontiguousarray(pos, dtype=np.float32).tobytes())
            if self.dim == 3:
                nrm = np.zeros((n, 3), dtype=np.float32)
                nrm[:, 2] = 1
                f.write(nrm.tobytes())
            if scalar is not None:
                f.write(np.ascontiguousarray(scalar, dtype=np.float32).tobytes())

    def writeFrame(self, frameDir, staticDraw=False):
        """particles.mesh (positions, unit-z normals in 3D, |v|) and boundary_particles.mesh
        (DEMParticleSand.cpp:30-53)."""
        os.makedirs(frameDir, exist_ok=True)
        x, v = self.getParticles()
        self._write_mesh(os.path.join(frameDir, "particles.mesh"), x, np.linalg.norm(v, axis=1))
        self._write_mesh(os.path.join(frameDir, "boundary_particles.mesh"), self.boundary_positions, None)

    def saveFrame(self, frameDir):
        """particles.sav / velocities.sav as raw FP64 (DEMParticleSand.cpp:55-64)."""
        os.makedirs(frameDir, exist_ok=True)
        x, v = self.getParticles()
        x.astype(np.float64).tofile(os.path.join(frameDir, "particles.sav"))
        v.astype(np.float64).tofile(os.path.join(frameDir, "velocities.sav"))

    def loadFrame(self, frameDir):
        """DEMParticleSand::loadFrame (DEMParticleSand.cpp:66-76).  A resumed reference run
        skips initialize (Simulator.cpp:43-45) and so never computes the boundary
        volumes; here a context that was not initialized is initialized after the load."""
        x = np.fromfile(os.path.join(frameDir, "particles.sav"), dtype=np.float64).reshape(-1, self.dim)
        v = np.fromfile(os.path.join(frameDir, "velocities.sav"), dtype=np.float64).reshape(-1, self.dim)
        self.setParticles(x, v)
        if not self._initialized:
            self.initialize()
