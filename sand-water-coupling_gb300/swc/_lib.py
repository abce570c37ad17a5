"""ctypes binding of the C ABI in include/swc.h and include/swc_sand.h (libswc_gb300.so).

Loading fails loudly when the library is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

LIB_PATH = _build.LIB_PATH

SWC_OK = 0
SWC_CG_NOT_CONVERGED = 1
SWC_NAN_DETECTED = 2
SWC_BAD_ARG = 3
SWC_CUDA_ERROR = 4
SWC_NOT_INITIALIZED = 5
SWC_OUT_OF_MEMORY = 6

WARM_PREFIX, WARM_NODE, WARM_ZERO, WARM_LEARNED, WARM_EXTRAPOLATE = 0, 1, 2, 3, 4

# learned warm-start network sizes (SWC_MLP_IN / SWC_MLP_PARAMS / SWC_MLP_NORM)
MLP_IN = 8
MLP_SCALE_EPS = 1e-4
MLP_PARAMS = 64 * MLP_IN + 64 + 64 * 64 + 64 + 64 + 1
MLP_NORM = 2 * MLP_IN + 2
WARM_NAMES = {"prefix": WARM_PREFIX, "node": WARM_NODE, "zero": WARM_ZERO, "learned": WARM_LEARNED,
              "extrapolate": WARM_EXTRAPOLATE}


class Scene(C.Structure):
    _fields_ = [
        ("dim", C.c_int32),
        ("enable_gravity", C.c_int32),
        ("particle_radius", C.c_double),
        ("mass", C.c_double),
        ("boundary_mass", C.c_double),
        ("grid_origin", C.c_double * 3),
        ("grid_spacing", C.c_double),
        ("grid_size", C.c_int32 * 3),
        ("reserved0", C.c_int32),
        ("gravity", C.c_double * 3),
        ("viscosity", C.c_double),
        ("target_density", C.c_double),
        ("kappa", C.c_double),
    ]


class SolverOpts(C.Structure):
    _fields_ = [
        ("tolerance", C.c_double),
        ("max_iterations", C.c_int32),
        ("warm_start", C.c_int32),
        ("check_interval", C.c_int32),
        ("keep_virtual_velocity", C.c_int32),
        ("compute_true_residual", C.c_int32),
        ("keep_features", C.c_int32),
        ("learned_no_fallback", C.c_int32),
        ("learned_gate", C.c_int32),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("n_particles", C.c_int64),
        ("n_boundary", C.c_int64),
        ("n_virtual", C.c_int64),
        ("active_bricks", C.c_int32),
        ("cg_iterations", C.c_int32),
        ("rel_residual", C.c_double),
        ("true_rel_residual", C.c_double),
        ("rhs_norm", C.c_double),
        ("initial_rel_residual", C.c_double),
        ("warm_start_used", C.c_int32),
        ("status", C.c_int32),
        ("device_ms", C.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class SandParams(C.Structure):
    _fields_ = [
        ("dim", C.c_int32),
        ("enable_gravity", C.c_int32),
        ("radius", C.c_double),
        ("mass", C.c_double),
        ("young", C.c_double),
        ("poisson", C.c_double),
        ("fric_angle", C.c_double),
    ]


# Every symbol declared in include/swc.h and include/swc_sand.h, with its ctypes signature.
_P, _D, _I64, _U8 = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int64), C.POINTER(C.c_uint8)
SIGNATURES = {
    "swc_default_solver_opts": (None, [C.POINTER(SolverOpts)]),
    "swc_status_str": (C.c_char_p, [C.c_int]),
    "swc_last_error": (C.c_char_p, [_P]),
    "swc_create": (C.c_int, [C.POINTER(Scene), C.POINTER(SolverOpts), C.POINTER(_P)]),
    "swc_destroy": (None, [_P]),
    "swc_set_stream": (C.c_int, [_P, _P]),
    "swc_set_solver_opts": (C.c_int, [_P, C.POINTER(SolverOpts)]),
    "swc_set_particles": (C.c_int, [_P, _D, _D, C.c_int64]),
    "swc_get_particles": (C.c_int, [_P, _D, _D, C.c_int64]),
    "swc_set_boundary": (C.c_int, [_P, _D, _D, _D, C.c_int64]),
    "swc_set_boundary_motion": (C.c_int, [_P, _U8, _D, C.c_double]),
    "swc_initialize": (C.c_int, [_P]),
    "swc_advance": (C.c_int, [_P, C.c_double, C.POINTER(Stats)]),
    "swc_project": (C.c_int, [_P, C.POINTER(Stats)]),
    "swc_get_time_step": (C.c_int, [_P, C.c_double, _D]),
    "swc_get_real_info": (C.c_int, [_P, _D, _D, C.c_int64]),
    "swc_set_volumes": (C.c_int, [_P, _D, C.c_int64]),
    "swc_get_boundary_info": (C.c_int, [_P, _D, _D, C.c_int64]),
    "swc_set_boundary_info": (C.c_int, [_P, _D, _D, C.c_int64]),
    "swc_get_boundary": (C.c_int, [_P, _D, _D, _D, C.c_int64]),
    "swc_get_scalars": (C.c_int, [_P, _D, _D, _D]),
    "swc_set_scalars": (C.c_int, [_P, C.c_double, C.c_double, C.c_double]),
    "swc_num_virtual": (C.c_int64, [_P]),
    "swc_get_virtual": (C.c_int, [_P, _I64, _D, _D, _D, _D, _D, _D, C.c_int64]),
    "swc_set_pressure": (C.c_int, [_P, _D, C.c_int64]),
    "swc_apply_operator": (C.c_int, [_P, _D, _D, C.c_int64]),
    "swc_debug_neighbors": (C.c_int, [_P, C.c_int, C.c_int64, _D, _I64, _I64, _I64]),
    "swc_set_profiling": (C.c_int, [_P, C.c_int]),
    "swc_get_phase_times": (C.c_int, [_P, _D, C.c_int]),
    "swc_time_kernel": (C.c_int, [_P, C.c_int, C.c_int, _D]),
    "swc_set_mlp": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "swc_get_features": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int64, _I64]),
    "swc_trainer_create": (C.c_int, [C.c_int64, C.c_int32, C.POINTER(_P)]),
    "swc_trainer_destroy": (None, [_P]),
    "swc_trainer_add": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int64]),
    "swc_trainer_set_params": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "swc_trainer_get_params": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "swc_trainer_fit": (C.c_int, [_P, C.c_int32, C.c_float, C.c_uint64, C.POINTER(C.c_float)]),
    "swc_mlp_forward": (C.c_int, [C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int64,
                                  C.POINTER(C.c_float)]),
    "swc_mlp_gradient": (C.c_int, [C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                   C.POINTER(C.c_float), C.c_int64, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "swc_mlp_gradient_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                           C.c_void_p, C.c_void_p]),
    "swc_debug_fail_alloc": (C.c_int, [C.c_int64]),
    "swc_host_alloc": (C.c_void_p, [C.c_size_t]),
    "swc_host_free": (None, [C.c_void_p]),
    # DEM sand step (include/swc_sand.h)
    "swc_sand_default_params": (None, [C.POINTER(SandParams)]),
    "swc_sand_last_error": (C.c_char_p, [_P]),
    "swc_sand_create": (C.c_int, [C.POINTER(SandParams), C.POINTER(_P)]),
    "swc_sand_destroy": (None, [_P]),
    "swc_sand_set_stream": (C.c_int, [_P, _P]),
    "swc_sand_set_particles": (C.c_int, [_P, _D, _D, C.c_int64]),
    "swc_sand_get_particles": (C.c_int, [_P, _D, _D, C.c_int64]),
    "swc_sand_set_boundary": (C.c_int, [_P, _D, _D, C.c_int64]),
    "swc_sand_initialize": (C.c_int, [_P]),
    "swc_sand_advance": (C.c_int, [_P, C.c_double]),
    "swc_sand_get_time_step": (C.c_int, [_P, C.c_double, _D]),
    "swc_sand_get_boundary_info": (C.c_int, [_P, _D, _D, C.c_int64]),
    "swc_sand_time_kernel": (C.c_int, [_P, C.c_int, C.c_int, _D]),
}

_lib = None


def load(build_if_missing: bool = True):
    """Load libswc_gb300.so (building it with nvcc first when absent or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        _build.build()
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"GB300 library not built: {LIB_PATH} is missing (run __graft_entry__.build())")
    L = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


class SwcError(RuntimeError):
    def __init__(self, status, where, detail=""):
        self.status = status
        msg = f"{where}: {load().swc_status_str(status).decode()}"
        if detail:
            msg += f" ({detail})"
        super().__init__(msg)
