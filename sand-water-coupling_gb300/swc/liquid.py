"""DualParticleSphLiquid on GB300: the reference's Simulation-shaped API over the C ABI.

Mirrors Cores/Physics/DualParticleSphLiquid.{h,cpp} and the Simulation
interface (Cores/Physics/Simulation.h:25-34) of skytang0205/sand-water-coupling:

    initialize()                 DualParticleSphLiquid.cpp:78-110
    advance(dt)                  DualParticleSphLiquid.cpp:112-126
    getTimeStep(frameRate, stepRate)   SmthParticleHydrodLiquid.h:39-41
    dimension()
    writeDescription(root)       DualParticleSphLiquid.cpp:8-40 (YAML text)
    writeFrame(frameDir, staticDraw)   DualParticleSphLiquid.cpp:42-76 (.mesh)
    saveFrame(frameDir) / loadFrame(frameDir)   SmthParticleHydrodLiquid.cpp:34-55 (.sav)

Errors are raised as SwcError carrying the C status code; the reference's
std::exit(-1) on solver failure becomes an exception only when
``raise_on_nonconvergence`` is set (otherwise the status is kept in
``last_stats``).  All compute runs in libswc_gb300.so on the GPU.
"""
from __future__ import annotations

import ctypes as C
import os
import struct

import numpy as np

from . import _lib
from ._lib import SwcError


def _dp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None and a.shape != shape:
        raise ValueError(f"expected shape {shape}, got {a.shape}")
    return a


class DualParticleSphLiquid:
    def __init__(self, scene, tolerance=None, max_iterations=-1, warm_start="prefix", keep_virtual_velocity=False,
                 compute_true_residual=False, keep_features=False, check_interval=0, raise_on_nonconvergence=False,
                 learned_no_fallback=False, learned_gate=0):
        self.L = _lib.load()
        self.scene = scene
        self.dim = scene.dim
        s = _lib.Scene()
        s.dim = scene.dim
        s.enable_gravity = 1 if scene.enable_gravity else 0
        s.particle_radius = scene.particle_radius
        s.mass = scene.mass
        s.boundary_mass = scene.boundary_mass
        for a in range(3):
            s.grid_origin[a] = scene.grid_origin[a]
            s.grid_size[a] = scene.grid_size[a]
            s.gravity[a] = scene.gravity[a]
        s.grid_spacing = scene.grid_spacing
        s.viscosity = scene.viscosity
        s.target_density = scene.target_density
        s.kappa = scene.kappa
        o = _lib.SolverOpts()
        self.L.swc_default_solver_opts(C.byref(o))
        o.tolerance = scene.tolerance if tolerance is None else tolerance
        o.max_iterations = max_iterations
        o.warm_start = _lib.WARM_NAMES[warm_start] if isinstance(warm_start, str) else int(warm_start)
        o.check_interval = check_interval
        o.keep_virtual_velocity = 1 if keep_virtual_velocity else 0
        o.compute_true_residual = 1 if compute_true_residual else 0
        o.keep_features = 1 if keep_features else 0
        o.learned_no_fallback = 1 if learned_no_fallback else 0
        o.learned_gate = int(learned_gate)
        self._opts = o
        self._scene_c = s
        h = C.c_void_p()
        rc = self.L.swc_create(C.byref(s), C.byref(o), C.byref(h))
        if rc != _lib.SWC_OK:
            raise SwcError(rc, "swc_create")
        self.h = h
        self.raise_on_nonconvergence = raise_on_nonconvergence
        self.last_stats = None
        self.n = 0
        self.nb = 0
        self.setParticles(scene.positions, scene.velocities)
        self.setBoundary(scene.boundary_positions, scene.boundary_normals, scene.boundary_velocities)
        meta = getattr(scene, "meta", None) or {}
        if "paddle_omega" in meta:
            moving = np.zeros(self.nb, dtype=np.uint8)
            moving[meta.get("n_walls", 0):] = 1
            self.setBoundaryMotion(moving, meta["paddle_center"], meta["paddle_omega"])

    # -- lifetime ---------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.L.swc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, where, allow_nonconv=True):
        if rc == _lib.SWC_OK:
            return rc
        if allow_nonconv and rc in (_lib.SWC_CG_NOT_CONVERGED,) and not self.raise_on_nonconvergence:
            return rc
        raise SwcError(rc, where, self.L.swc_last_error(self.h).decode(errors="replace"))

    # -- state ------------------------------------------------------------
    def setParticles(self, x, v=None):
        x = _f64(x)
        n = x.shape[0]
        v = None if v is None else _f64(v, x.shape)
        self._check(self.L.swc_set_particles(self.h, _dp(x), _dp(v), n), "swc_set_particles")
        self.n = n

    def getParticles(self):
        x = np.empty((self.n, self.dim))
        v = np.empty((self.n, self.dim))
        self._check(self.L.swc_get_particles(self.h, _dp(x), _dp(v), self.n), "swc_get_particles")
        return x, v

    def setBoundary(self, x, normals, v=None):
        x = _f64(x)
        nb = x.shape[0]
        nrm = _f64(normals, x.shape)
        v = None if v is None else _f64(v, x.shape)
        self._check(self.L.swc_set_boundary(self.h, _dp(x), _dp(nrm), _dp(v), nb), "swc_set_boundary")
        self.nb = nb

    def setBoundaryMotion(self, moving, center, omega):
        m = np.ascontiguousarray(moving, dtype=np.uint8)
        c = _f64(np.asarray(center, dtype=np.float64).reshape(-1)[:3])
        self._check(self.L.swc_set_boundary_motion(self.h, m.ctypes.data_as(C.POINTER(C.c_uint8)), _dp(c),
                                                   float(omega)), "swc_set_boundary_motion")

    def setSolverOptions(self, **kw):
        o = self._opts
        for k, v in kw.items():
            if k == "warm_start" and isinstance(v, str):
                v = _lib.WARM_NAMES[v]
            setattr(o, k, v)
        self._check(self.L.swc_set_solver_opts(self.h, C.byref(o)), "swc_set_solver_opts")

    # -- Simulation API ---------------------------------------------------
    def dimension(self):
        return self.dim

    def initialize(self):
        self._check(self.L.swc_initialize(self.h), "swc_initialize")

    def advance(self, dt):
        st = _lib.Stats()
        rc = self.L.swc_advance(self.h, float(dt), C.byref(st))
        self.last_stats = st.as_dict()
        self._check(rc, "swc_advance")
        return self.last_stats

    def project(self):
        """Projection of the current state (rho_i, virtual generation, VirtualParticle::project)."""
        st = _lib.Stats()
        rc = self.L.swc_project(self.h, C.byref(st))
        self.last_stats = st.as_dict()
        self._check(rc, "swc_project")
        return self.last_stats

    def getTimeStep(self, frameRate, stepRate):
        dt = C.c_double()
        self._check(self.L.swc_get_time_step(self.h, float(stepRate), C.byref(dt)), "swc_get_time_step")
        return dt.value

    # -- inspection -------------------------------------------------------
    def scalars(self):
        r, a, k = C.c_double(), C.c_double(), C.c_double()
        self._check(self.L.swc_get_scalars(self.h, C.byref(r), C.byref(a), C.byref(k)), "swc_get_scalars")
        return {"rho0": r.value, "alpha0": a.value, "kappa": k.value}

    def setScalars(self, rho0, alpha0, kappa):
        self._check(self.L.swc_set_scalars(self.h, rho0, alpha0, kappa), "swc_set_scalars")

    def realInfo(self):
        rho = np.empty(self.n)
        vol = np.empty(self.n)
        self._check(self.L.swc_get_real_info(self.h, _dp(rho), _dp(vol), self.n), "swc_get_real_info")
        return rho, vol

    def setVolumes(self, vol):
        vol = _f64(vol, (self.n,))
        self._check(self.L.swc_set_volumes(self.h, _dp(vol), self.n), "swc_set_volumes")

    def boundaryInfo(self):
        rho = np.empty(self.nb)
        vol = np.empty(self.nb)
        self._check(self.L.swc_get_boundary_info(self.h, _dp(rho), _dp(vol), self.nb), "swc_get_boundary_info")
        return rho, vol

    def getBoundary(self):
        """Boundary positions, inward normals and velocities as they stand (a moving
        paddle turns every advance), in the order of setBoundary."""
        x, n, v = (np.empty((self.nb, self.dim)) for _ in range(3))
        self._check(self.L.swc_get_boundary(self.h, _dp(x), _dp(n), _dp(v), self.nb), "swc_get_boundary")
        return x, n, v

    def setBoundaryInfo(self, rho, vol):
        rho = _f64(rho, (self.nb,))
        vol = _f64(vol, (self.nb,))
        self._check(self.L.swc_set_boundary_info(self.h, _dp(rho), _dp(vol), self.nb), "swc_set_boundary_info")

    def numVirtual(self):
        return int(self.L.swc_num_virtual(self.h))

    def virtual(self, with_vbar=False):
        n = self.numVirtual()
        out = {
            "node": np.empty(n, dtype=np.int64),
            "rho": np.empty(n),
            "vol": np.empty(n),
            "div": np.empty(n),
            "alpha_hat": np.empty(n),
            "p": np.empty(n),
        }
        vb = np.empty((n, self.dim)) if with_vbar else None
        rc = self.L.swc_get_virtual(self.h, out["node"].ctypes.data_as(C.POINTER(C.c_int64)), _dp(out["rho"]),
                                    _dp(out["vol"]), _dp(vb), _dp(out["div"]), _dp(out["alpha_hat"]),
                                    _dp(out["p"]), max(n, 1))
        self._check(rc, "swc_get_virtual")
        if with_vbar:
            out["vbar"] = vb
        return out

    def setPressure(self, p):
        p = _f64(p)
        self._check(self.L.swc_set_pressure(self.h, _dp(p), p.shape[0]), "swc_set_pressure")

    def applyOperator(self, x):
        x = _f64(x)
        y = np.empty_like(x)
        self._check(self.L.swc_apply_operator(self.h, _dp(x), _dp(y), x.shape[0]), "swc_apply_operator")
        return y

    def neighbors(self, which, queries):
        """Sorted neighbour ids per query point (product cell search; see swc_debug_neighbors)."""
        w = {"real": 0, "boundary": 1, "virtual": 2}[which]
        q = _f64(queries)
        nq = q.shape[0]
        counts = np.zeros(nq, dtype=np.int64)
        ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int64))
        self._check(self.L.swc_debug_neighbors(self.h, w, nq, _dp(q), ip(counts), None, None), "swc_debug_neighbors")
        offsets = np.zeros(nq + 1, dtype=np.int64)
        offsets[1:] = np.cumsum(counts)
        ids = np.zeros(max(1, int(offsets[-1])), dtype=np.int64)
        self._check(self.L.swc_debug_neighbors(self.h, w, nq, _dp(q), ip(counts), ip(offsets), ip(ids)),
                    "swc_debug_neighbors")
        ids = ids[: offsets[-1]]
        for t in range(nq):
            ids[offsets[t]:offsets[t + 1]].sort()
        return counts, offsets, ids

    def setMlp(self, params, norm):
        """Network of the learned warm start (see swc.learn)."""
        p = np.ascontiguousarray(params, dtype=np.float32).ravel()
        q = np.ascontiguousarray(norm, dtype=np.float32).ravel()
        if p.size != _lib.MLP_PARAMS or q.size != _lib.MLP_NORM:
            raise ValueError(f"network of {p.size} parameters / {q.size} normalisation values; "
                             f"expected {_lib.MLP_PARAMS} / {_lib.MLP_NORM}")
        fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        self._check(self.L.swc_set_mlp(self.h, fp(p), fp(q)), "swc_set_mlp")

    def features(self):
        """(features[n, MLP_IN], targets[n]) logged by the last projection (keep_features=True)."""
        n = self.numVirtual()
        f = np.empty((max(n, 1), _lib.MLP_IN), dtype=np.float32)
        t = np.empty(max(n, 1), dtype=np.float32)
        got = C.c_int64()
        fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        self._check(self.L.swc_get_features(self.h, fp(f), fp(t), max(n, 1), C.byref(got)), "swc_get_features")
        return f[: got.value], t[: got.value]

    def setProfiling(self, on=True):
        self._check(self.L.swc_set_profiling(self.h, 1 if on else 0), "swc_set_profiling")

    def phaseTimes(self):
        ms = np.zeros(8)
        self._check(self.L.swc_get_phase_times(self.h, _dp(ms), 8), "swc_get_phase_times")
        names = ["binning", "densities", "forces", "virtual_generation", "warm_start", "cg", "pressure_gradient",
                 "export"]
        return dict(zip(names, ms.tolist()))

    def timeKernel(self, which, reps=20):
        ms = C.c_double()
        self._check(self.L.swc_time_kernel(self.h, int(which), int(reps), C.byref(ms)), "swc_time_kernel")
        return ms.value

    def setStream(self, stream_handle):
        self._check(self.L.swc_set_stream(self.h, C.c_void_p(stream_handle)), "swc_set_stream")

    # -- frame / checkpoint formats ----------------------------------------
    def nodePositions(self, node_ids):
        sc = self.scene
        nx, ny = sc.grid_size[0], sc.grid_size[1]
        k = np.stack([node_ids % nx, (node_ids // nx) % ny, node_ids // (nx * ny)], axis=1)[:, : self.dim]
        return np.asarray(sc.grid_origin[: self.dim]) + k * sc.grid_spacing

    def writeDescription(self, root_path):
        """description.yaml objects of DualParticleSphLiquid::writeDescription (DualParticleSphLiquid.cpp:8-40)."""
        albedo = [52 / 255, 108 / 255, 156 / 255, 1.0]
        lines = [f"dimension: {self.dim}", "objects:"]
        for name, cmap in (("particles", True), ("virtual_particles", True), ("boundary_particles", False)):
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
        """particles / virtual_particles / boundary_particles .mesh (DualParticleSphLiquid.cpp:42-76)."""
        os.makedirs(frameDir, exist_ok=True)
        x, v = self.getParticles()
        self._write_mesh(os.path.join(frameDir, "particles.mesh"), x, np.linalg.norm(v, axis=1))
        vi = self.virtual()
        self._write_mesh(os.path.join(frameDir, "virtual_particles.mesh"), self.nodePositions(vi["node"]), vi["vol"])
        self._write_mesh(os.path.join(frameDir, "boundary_particles.mesh"), self.scene.boundary_positions, None)

    def saveFrame(self, frameDir):
        """particles.sav / velocities.sav as raw FP64 (SmthParticleHydrodLiquid.cpp:34-43), plus
        dual_state.sav (V_i, rho0, alpha0, kappa, last pressure) so a resumed run needs no
        re-initialisation (the reference skips initialize on resume, Simulator.cpp:43-45)."""
        os.makedirs(frameDir, exist_ok=True)
        x, v = self.getParticles()
        x.astype(np.float64).tofile(os.path.join(frameDir, "particles.sav"))
        v.astype(np.float64).tofile(os.path.join(frameDir, "velocities.sav"))
        _, vol = self.realInfo()
        sc = self.scalars()
        p = self.virtual()["p"]
        with open(os.path.join(frameDir, "dual_state.sav"), "wb") as f:
            f.write(struct.pack("<qqddd", self.n, p.shape[0], sc["rho0"], sc["alpha0"], sc["kappa"]))
            f.write(vol.astype(np.float64).tobytes())
            f.write(p.astype(np.float64).tobytes())

    def loadFrame(self, frameDir):
        x = np.fromfile(os.path.join(frameDir, "particles.sav"), dtype=np.float64).reshape(-1, self.dim)
        v = np.fromfile(os.path.join(frameDir, "velocities.sav"), dtype=np.float64).reshape(-1, self.dim)
        self.setParticles(x, v)
        ds = os.path.join(frameDir, "dual_state.sav")
        if os.path.exists(ds):
            with open(ds, "rb") as f:
                n, nv, rho0, alpha0, kappa = struct.unpack("<qqddd", f.read(40))
                vol = np.frombuffer(f.read(8 * n), dtype=np.float64)
                p = np.frombuffer(f.read(8 * nv), dtype=np.float64)
            self.initialize()  # boundary information; particle volumes and scalars restored below
            self.setVolumes(vol)
            self.setScalars(rho0, alpha0, kappa)
            self.setPressure(p)
        else:
            self.initialize()
