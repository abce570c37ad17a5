"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of the CPU FP64 oracle (swc_oracle.cpp).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py may
import this module; it is the checker, never the measured or shipped path.
See swc_oracle.cpp for which reference files each routine restates and for the
parity status ("parity unpinned" against an executable of the reference).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libswc_oracle.so")


class Params(C.Structure):
    _fields_ = [
        ("dim", C.c_int32),
        ("enable_gravity", C.c_int32),
        ("particle_radius", C.c_double),
        ("mass", C.c_double),
        ("boundary_mass", C.c_double),
        ("grid_origin", C.c_double * 3),
        ("grid_spacing", C.c_double),
        ("grid_size", C.c_int32 * 3),
        ("max_iterations", C.c_int32),
        ("gravity", C.c_double * 3),
        ("viscosity", C.c_double),
        ("target_density", C.c_double),
        ("kappa", C.c_double),
        ("tolerance", C.c_double),
    ]


class DemParams(C.Structure):
    _fields_ = [
        ("dim", C.c_int32),
        ("enable_gravity", C.c_int32),
        ("radius", C.c_double),
        ("mass", C.c_double),
        ("young", C.c_double),
        ("poisson", C.c_double),
        ("fric_angle", C.c_double),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle with make (g++ -fopenmp)."""
    srcs = [os.path.join(HERE, f) for f in ("swc_oracle.cpp", "dem_oracle.cpp", "orc_core.h", "Makefile")]
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(map(os.path.getmtime, srcs)):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P, D, I64, I32 = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int64), C.POINTER(C.c_int32)
        L.orc_create.restype = P
        L.orc_create.argtypes = [C.POINTER(Params)]
        L.orc_destroy.argtypes = [P]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_num_threads.restype = C.c_int
        L.orc_set_particles.argtypes = [P, C.c_int64, D, D]
        L.orc_get_particles.argtypes = [P, D, D]
        L.orc_set_boundary.argtypes = [P, C.c_int64, D, D, D]
        L.orc_set_boundary_motion.argtypes = [P, C.POINTER(C.c_uint8), D, C.c_double]
        L.orc_set_searcher.argtypes = [P, C.c_int]
        L.orc_hash_candidates.restype = C.c_int64
        L.orc_hash_candidates.argtypes = [P, C.c_int, C.c_int64, D]
        for n in ("orc_initialize", "orc_project", "orc_compute_densities"):
            getattr(L, n).argtypes = [P]
        L.orc_advance.argtypes = [P, C.c_double]
        L.orc_move_and_forces.argtypes = [P, C.c_double]
        L.orc_get_scalars.argtypes = [P, D]
        L.orc_set_scalars.argtypes = [P, D]
        L.orc_get_real_info.argtypes = [P, D, D]
        L.orc_set_volumes.argtypes = [P, D]
        L.orc_get_boundary_info.argtypes = [P, D, D]
        L.orc_set_boundary_info.argtypes = [P, D, D]
        L.orc_num_virtual.restype = C.c_int64
        L.orc_num_virtual.argtypes = [P]
        L.orc_get_virtual.argtypes = [P, I64, D, D, D, D, D, D]
        L.orc_set_pressure.argtypes = [P, C.c_int64, D]
        L.orc_apply_operator.argtypes = [P, D, D]
        L.orc_get_stats.argtypes = [P, I32, I32, D, D, I32]
        L.orc_neighbors.argtypes = [P, C.c_int, C.c_int64, D, I64, I64, I64]
        L.orc_kernel.restype = C.c_double
        L.orc_kernel.argtypes = [C.c_int, C.c_double, C.c_int, C.c_double]
        L.orc_packed_kernel_sum.restype = C.c_double
        L.orc_packed_kernel_sum.argtypes = [C.c_int, C.c_double]
        # DEM sand step (dem_oracle.cpp)
        DP = C.POINTER(DemParams)
        L.dem_create.restype = P
        L.dem_create.argtypes = [DP]
        L.dem_destroy.argtypes = [P]
        L.dem_set_particles.argtypes = [P, C.c_longlong, D, D]
        L.dem_get_particles.argtypes = [P, D, D]
        L.dem_set_boundary.argtypes = [P, C.c_longlong, D, D, D]
        L.dem_initialize.argtypes = [P]
        L.dem_advance.argtypes = [P, C.c_double]
        L.dem_get_boundary_info.argtypes = [P, D, D]
        L.dem_time_step.restype = C.c_double
        L.dem_time_step.argtypes = [P, C.c_double]
        L.dem_model.argtypes = [DP, D]
        L.dem_pair_force.argtypes = [DP, D, D, D, D]
        L.dem_boundary_term.argtypes = [DP, D, D, C.c_double, C.c_double, D]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int64)) if a is not None else None


def kernel(dim, radius, dist, derivative=False):
    return lib().orc_kernel(dim, radius, 1 if derivative else 0, dist)


def packed_kernel_sum(dim, radius):
    return lib().orc_packed_kernel_sum(dim, radius)


def set_threads(n: int):
    lib().orc_set_threads(int(n))


def num_threads() -> int:
    return lib().orc_num_threads()


class Oracle:
    """FP64 CPU restatement of DualParticleSphLiquid (initialize / advance / project)."""

    def __init__(self, scene, tolerance=None, max_iterations=-1, searcher="hash"):
        self.scene = scene
        self.dim = scene.dim
        p = Params()
        p.dim = scene.dim
        p.enable_gravity = 1 if scene.enable_gravity else 0
        p.particle_radius = scene.particle_radius
        p.mass = scene.mass
        p.boundary_mass = scene.boundary_mass
        for a in range(3):
            p.grid_origin[a] = scene.grid_origin[a]
            p.grid_size[a] = scene.grid_size[a]
            p.gravity[a] = scene.gravity[a]
        p.grid_spacing = scene.grid_spacing
        p.max_iterations = max_iterations
        p.viscosity = scene.viscosity
        p.target_density = scene.target_density
        p.kappa = scene.kappa
        p.tolerance = scene.tolerance if tolerance is None else tolerance
        self._p = p
        self.h = lib().orc_create(C.byref(p))
        if not self.h:
            raise ValueError("oracle: bad parameters")
        self.set_particles(scene.positions, scene.velocities)
        self.set_boundary(scene.boundary_positions, scene.boundary_normals, scene.boundary_velocities)
        self.set_searcher(searcher)

    def set_searcher(self, kind: str):
        """Neighbour searcher of every query: "hash", the reference's hash grid (its
        enumeration order), or "cells", a cell grid over the same cells (the same
        neighbour sets in cell order; FP64 sums differ in rounding only).  The
        reference's hash degenerates when its 2N bucket count is a power of two
        (128^3 particles), so scenes of that size use "cells"."""
        if kind not in ("hash", "cells"):
            raise ValueError(f"searcher {kind!r}")
        self.searcher = kind
        lib().orc_set_searcher(self.h, 1 if kind == "cells" else 0)

    def hash_candidates(self, which: str, queries) -> float:
        """Mean number of candidates the reference's hash grid visits per query
        (bucket entries before the distance test) on the current real / boundary /
        virtual set: the reference searcher's per-query cost."""
        w = {"real": 0, "boundary": 1, "virtual": 2}[which]
        q = np.ascontiguousarray(queries, dtype=np.float64)
        return lib().orc_hash_candidates(self.h, w, q.shape[0], _dp(q)) / max(q.shape[0], 1)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def set_particles(self, x, v):
        x = np.ascontiguousarray(x, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        self.n = x.shape[0]
        lib().orc_set_particles(self.h, self.n, _dp(x), _dp(v))

    def set_boundary(self, x, nrm, v):
        x = np.ascontiguousarray(x, dtype=np.float64)
        nrm = np.ascontiguousarray(nrm, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        self.nb = x.shape[0]
        lib().orc_set_boundary(self.h, self.nb, _dp(x), _dp(nrm), _dp(v))

    def set_boundary_motion(self, moving, center, omega):
        """Rigid rotation of the flagged boundary particles about the vertical axis
        through `center` at `omega` rad/s, applied at the start of every advance."""
        m = np.ascontiguousarray(moving, dtype=np.uint8)
        assert m.shape[0] == self.nb
        c = np.ascontiguousarray(np.asarray(center, dtype=np.float64).reshape(-1)[:3])
        lib().orc_set_boundary_motion(self.h, m.ctypes.data_as(C.POINTER(C.c_uint8)), _dp(c), float(omega))

    def particles(self):
        x = np.zeros((self.n, self.dim))
        v = np.zeros((self.n, self.dim))
        lib().orc_get_particles(self.h, _dp(x), _dp(v))
        return x, v

    def initialize(self):
        lib().orc_initialize(self.h)

    def advance(self, dt):
        lib().orc_advance(self.h, dt)

    def move_and_forces(self, dt):
        lib().orc_move_and_forces(self.h, dt)

    def project(self):
        lib().orc_project(self.h)

    def compute_densities(self):
        lib().orc_compute_densities(self.h)

    def scalars(self):
        o = np.zeros(3)
        lib().orc_get_scalars(self.h, _dp(o))
        return {"rho0": o[0], "alpha0": o[1], "kappa": o[2]}

    def set_scalars(self, rho0, alpha0, kappa):
        o = np.array([rho0, alpha0, kappa], dtype=np.float64)
        lib().orc_set_scalars(self.h, _dp(o))

    def real_info(self):
        rho = np.zeros(self.n)
        vol = np.zeros(self.n)
        lib().orc_get_real_info(self.h, _dp(rho), _dp(vol))
        return rho, vol

    def set_volumes(self, vol):
        vol = np.ascontiguousarray(vol, dtype=np.float64)
        lib().orc_set_volumes(self.h, _dp(vol))

    def boundary_info(self):
        rho = np.zeros(self.nb)
        vol = np.zeros(self.nb)
        lib().orc_get_boundary_info(self.h, _dp(rho), _dp(vol))
        return rho, vol

    def set_boundary_info(self, rho, vol):
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        vol = np.ascontiguousarray(vol, dtype=np.float64)
        lib().orc_set_boundary_info(self.h, _dp(rho), _dp(vol))

    def num_virtual(self):
        return int(lib().orc_num_virtual(self.h))

    def virtual(self):
        n = self.num_virtual()
        out = {
            "node": np.zeros(n, dtype=np.int64),
            "rho": np.zeros(n),
            "vol": np.zeros(n),
            "vbar": np.zeros((n, self.dim)),
            "div": np.zeros(n),
            "alpha_hat": np.zeros(n),
            "p": np.zeros(n),
        }
        lib().orc_get_virtual(self.h, _ip(out["node"]), _dp(out["rho"]), _dp(out["vol"]), _dp(out["vbar"]),
                              _dp(out["div"]), _dp(out["alpha_hat"]), _dp(out["p"]))
        return out

    def set_pressure(self, p):
        p = np.ascontiguousarray(p, dtype=np.float64)
        lib().orc_set_pressure(self.h, p.shape[0], _dp(p))

    def apply_operator(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        lib().orc_apply_operator(self.h, _dp(x), _dp(y))
        return y

    def stats(self):
        it, eit, st = C.c_int32(), C.c_int32(), C.c_int32()
        rr, bn = C.c_double(), C.c_double()
        lib().orc_get_stats(self.h, C.byref(it), C.byref(eit), C.byref(rr), C.byref(bn), C.byref(st))
        return {"iterations": it.value, "eigen_iterations": eit.value, "rel_residual": rr.value,
                "rhs_norm": bn.value, "status": st.value}

    def neighbors(self, which: str, queries):
        """Sorted neighbour ids per query (reference searcher semantics)."""
        w = {"real": 0, "boundary": 1, "virtual": 2}[which]
        q = np.ascontiguousarray(queries, dtype=np.float64)
        nq = q.shape[0]
        counts = np.zeros(nq, dtype=np.int64)
        lib().orc_neighbors(self.h, w, nq, _dp(q), _ip(counts), None, None)
        offsets = np.zeros(nq + 1, dtype=np.int64)
        offsets[1:] = np.cumsum(counts)
        ids = np.zeros(max(1, offsets[-1]), dtype=np.int64)
        lib().orc_neighbors(self.h, w, nq, _dp(q), _ip(counts), _ip(offsets), _ip(ids))
        return counts, offsets, ids[: offsets[-1]]


def dem_params(dim, radius, mass=1.0, young=1e9, poisson=0.3, fric_angle=0.5, enable_gravity=True):
    p = DemParams()
    p.dim, p.enable_gravity, p.radius, p.mass = int(dim), 1 if enable_gravity else 0, float(radius), float(mass)
    p.young, p.poisson, p.fric_angle = float(young), float(poisson), float(fric_angle)
    return p


def dem_model(p):
    """K_norm, K_tang, tan(friction angle), d_rupture, capillary coefficient, liquid-bridge volume."""
    o = np.zeros(6)
    lib().dem_model(C.byref(p), _dp(o))
    return dict(zip(("K_norm", "K_tang", "tan_fric", "d_rupture", "coeff_c", "v_bridge"), o))


def dem_pair_force(p, d, w):
    """(contact, capillary) force of one pair, d = x_j - x_i, w = v_j - v_i (3 components)."""
    d = np.ascontiguousarray(np.resize(np.asarray(d, dtype=np.float64), 3))
    w = np.ascontiguousarray(np.resize(np.asarray(w, dtype=np.float64), 3))
    if p.dim == 2:
        d[2] = w[2] = 0.0
    f0, f1 = np.zeros(3), np.zeros(3)
    lib().dem_pair_force(C.byref(p), _dp(d), _dp(w), _dp(f0), _dp(f1))
    return f0[: p.dim], f1[: p.dim]


def dem_boundary_term(p, dv, nb, vol, w):
    dv = np.zeros(3) + np.pad(np.asarray(dv, dtype=np.float64), (0, 3 - len(dv)))
    nb = np.zeros(3) + np.pad(np.asarray(nb, dtype=np.float64), (0, 3 - len(nb)))
    out = np.zeros(3)
    lib().dem_boundary_term(C.byref(p), _dp(dv), _dp(nb), float(vol), float(w), _dp(out))
    return out[: p.dim]


class DemOracle:
    """FP64 CPU restatement of DEMParticleSand (initialize / advance / getTimeStep)."""

    def __init__(self, dim, radius, mass=1.0, young=1e9, poisson=0.3, fric_angle=0.5, enable_gravity=True):
        self.dim = int(dim)
        self._p = dem_params(dim, radius, mass, young, poisson, fric_angle, enable_gravity)
        self.h = lib().dem_create(C.byref(self._p))
        if not self.h:
            raise ValueError("dem oracle: bad parameters")
        self.n = self.nb = 0

    def __del__(self):
        if getattr(self, "h", None):
            lib().dem_destroy(self.h)
            self.h = None

    def set_particles(self, x, v):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, self.dim)
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(-1, self.dim)
        self.n = x.shape[0]
        lib().dem_set_particles(self.h, self.n, _dp(x), _dp(v))

    def set_boundary(self, x, nrm, v=None):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, self.dim)
        nrm = np.ascontiguousarray(nrm, dtype=np.float64).reshape(-1, self.dim)
        v = None if v is None else np.ascontiguousarray(v, dtype=np.float64).reshape(-1, self.dim)
        self.nb = x.shape[0]
        lib().dem_set_boundary(self.h, self.nb, _dp(x), _dp(nrm), _dp(v))

    def initialize(self):
        lib().dem_initialize(self.h)

    def advance(self, dt):
        lib().dem_advance(self.h, float(dt))

    def particles(self):
        x = np.zeros((self.n, self.dim))
        v = np.zeros((self.n, self.dim))
        lib().dem_get_particles(self.h, _dp(x), _dp(v))
        return x, v

    def boundary_info(self):
        rho, vol = np.zeros(self.nb), np.zeros(self.nb)
        lib().dem_get_boundary_info(self.h, _dp(rho), _dp(vol))
        return rho, vol

    def time_step(self, step_rate):
        return lib().dem_time_step(self.h, float(step_rate))
