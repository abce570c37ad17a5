"""Failure paths of the C ABI with host-made failures: a device allocation made to
fail by the library's test hook (swc_debug_fail_alloc), never a GPU fault.

A set call whose allocation fails returns SWC_OUT_OF_MEMORY and leaves the
context without particles (or boundary) and uninitialized, so the next advance
returns SWC_NOT_INITIALIZED instead of launching on freed buffers; setting the
state again and initializing recovers the context.
"""
import ctypes as C

import numpy as np
import pytest

from swc import _lib, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture
def lib(swc_mod):
    L = swc_mod.load()
    yield L
    L.swc_debug_fail_alloc(-1)


@pytest.mark.parametrize("which", ["particles", "boundary"])
def test_sand_failed_allocation(swc_mod, lib, which):
    sd = scenes.sand_contact_block(2, scale=30, seed=1, wall_depth=12 / 120)
    gs = swc_mod.DEMParticleSand(sd.radius, dim=2, mass=sd.mass)
    gs.setParticles(sd.positions, sd.velocities)
    gs.setBoundary(sd.boundary_positions, sd.boundary_normals)
    gs.initialize()
    gs.advance(sd.dt)
    lib.swc_debug_fail_alloc(2)  # the third allocation from now
    with pytest.raises(swc_mod.SwcError) as e:
        if which == "particles":
            gs.setParticles(sd.positions[:-7], sd.velocities[:-7])  # a new count reallocates
        else:
            gs.setBoundary(sd.boundary_positions[:-5], sd.boundary_normals[:-5])
    assert e.value.status == _lib.SWC_OUT_OF_MEMORY
    lib.swc_debug_fail_alloc(-1)
    assert lib.swc_sand_advance(gs.h, sd.dt) == _lib.SWC_NOT_INITIALIZED
    # recovery: state again, initialize, advance
    gs.setParticles(sd.positions[:-7], sd.velocities[:-7])
    gs.setBoundary(sd.boundary_positions, sd.boundary_normals)
    gs.initialize()
    gs.advance(sd.dt)
    assert np.isfinite(gs.getParticles()[1]).all()
    gs.close()


def test_liquid_failed_boundary_allocation(swc_mod, lib):
    s = scenes.dam_break_2d(seed=2).rounded_to_float32()
    liq = swc_mod.DualParticleSphLiquid(s)
    liq.initialize()
    assert liq.advance(s.dt)["status"] == 0
    lib.swc_debug_fail_alloc(3)
    with pytest.raises(swc_mod.SwcError) as e:
        liq.setBoundary(s.boundary_positions[:-4], s.boundary_normals[:-4])
    assert e.value.status == _lib.SWC_OUT_OF_MEMORY
    lib.swc_debug_fail_alloc(-1)
    st = _lib.Stats()
    assert lib.swc_advance(liq.h, s.dt, C.byref(st)) == _lib.SWC_NOT_INITIALIZED
    liq.setBoundary(s.boundary_positions, s.boundary_normals, s.boundary_velocities)
    liq.initialize()
    assert liq.advance(s.dt)["status"] == 0
    liq.close()


def test_liquid_failed_particle_allocation(swc_mod, lib):
    """A particle count changes only before initialize (afterwards it is refused with
    SWC_BAD_ARG before any allocation): the failed set leaves no particles, and a
    failed swc_create releases what it had allocated and returns no context."""
    s = scenes.dam_break_2d(seed=2).rounded_to_float32()
    ref = swc_mod.DualParticleSphLiquid(s)  # for its scene and option structs
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    h = C.c_void_p()
    lib.swc_debug_fail_alloc(5)
    assert lib.swc_create(C.byref(ref._scene_c), C.byref(ref._opts), C.byref(h)) == _lib.SWC_OUT_OF_MEMORY
    assert not h.value
    lib.swc_debug_fail_alloc(-1)
    assert lib.swc_create(C.byref(ref._scene_c), C.byref(ref._opts), C.byref(h)) == _lib.SWC_OK
    x, v = np.ascontiguousarray(s.positions), np.ascontiguousarray(s.velocities)
    lib.swc_debug_fail_alloc(1)
    assert lib.swc_set_particles(h, dp(x), dp(v), s.n_particles) == _lib.SWC_OUT_OF_MEMORY
    lib.swc_debug_fail_alloc(-1)
    st = _lib.Stats()
    assert lib.swc_advance(h, s.dt, C.byref(st)) == _lib.SWC_NOT_INITIALIZED
    assert lib.swc_set_particles(h, dp(x), dp(v), s.n_particles) == _lib.SWC_OK
    bx, bn = np.ascontiguousarray(s.boundary_positions), np.ascontiguousarray(s.boundary_normals)
    assert lib.swc_set_boundary(h, dp(bx), dp(bn), None, s.n_boundary) == _lib.SWC_OK
    assert lib.swc_initialize(h) == _lib.SWC_OK
    assert lib.swc_advance(h, s.dt, C.byref(st)) == _lib.SWC_OK
    lib.swc_destroy(h)
    ref.close()
