"""CPU checks of the C-ABI library: it loads, exports every symbol declared in
include/*.h, and refuses to run without a GPU (no CPU fallback)."""
import ctypes as C
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b(swc_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_header_declares_the_api():
    names = declared_symbols()
    for must in ("swc_create", "swc_destroy", "swc_initialize", "swc_advance", "swc_project", "swc_set_particles",
                 "swc_get_particles", "swc_get_virtual", "swc_status_str"):
        assert must in names


def test_library_exports_every_declared_symbol(swc_mod):
    from swc import _lib

    lib = C.CDLL(_lib.LIB_PATH)
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding covers the whole header too
    assert declared_symbols() <= set(_lib.SIGNATURES)


def test_status_strings_and_defaults(swc_mod):
    from swc import _lib

    L = _lib.load()
    assert L.swc_status_str(0) == b"ok"
    assert L.swc_status_str(1) == b"CG did not converge"
    o = _lib.SolverOpts()
    L.swc_default_solver_opts(C.byref(o))
    assert o.tolerance == 1e-6 and o.max_iterations == -1 and o.warm_start == 0


def test_bad_arguments_are_rejected_without_gpu(swc_mod):
    from swc import _lib

    L = _lib.load()
    h = C.c_void_p()
    assert L.swc_create(None, None, C.byref(h)) == _lib.SWC_BAD_ARG
    s = _lib.Scene()
    s.dim = 4
    assert L.swc_create(C.byref(s), None, C.byref(h)) == _lib.SWC_BAD_ARG


def test_no_cpu_fallback(swc_mod):
    import numpy as np
    import swc
    from swc import scenes

    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("GPU present")
    with pytest.raises(swc.SwcError):
        swc.DualParticleSphLiquid(scenes.dam_break_2d(height_cells=4, width_cells=4))


def test_sand_params_layout_and_defaults(swc_mod):
    """swc_sand_params as laid out in include/swc_sand.h; defaults are the reference's
    (DEMParticle.cpp:18-22, DEMParticleSandBuilder case 0 radius at scale 30)."""
    from swc import _lib

    assert C.sizeof(_lib.SandParams) == 2 * 4 + 5 * 8
    assert _lib.SandParams.radius.offset == 8
    L = _lib.load()
    p = _lib.SandParams()
    L.swc_sand_default_params(C.byref(p))
    assert (p.dim, p.enable_gravity, p.mass) == (2, 1, 1.0)
    assert p.young == 1e9 and p.poisson == 0.3 and p.fric_angle == 0.5
    assert p.radius == pytest.approx(1.0 / 120)
    h = C.c_void_p()
    assert L.swc_sand_create(None, C.byref(h)) == _lib.SWC_BAD_ARG
    p.radius = -1.0
    assert L.swc_sand_create(C.byref(p), C.byref(h)) == _lib.SWC_BAD_ARG


def test_sand_no_cpu_fallback(swc_mod):
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("GPU present")
    from swc.sand import DEMParticleSand

    with pytest.raises(swc_mod.SwcError):
        DEMParticleSand(1.0 / 120, dim=2)
