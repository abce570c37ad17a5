"""CFL time step and frame driver on the GPU against the FP64 oracle.

getTimeStep = stepRate * 2 r / max_i |v_i| (SmthParticleHydrodLiquid.h:39-41,
ParticlesAttribute::normMax ParticlesAttribute.h:61-67) with the maximum reduced
on the device, and frames substepped by swc.Simulator / swc::Simulator as
Simulator::advanceTimeBySteps does (Simulator.cpp:103-128), compared with the
same rule restated here over the oracle's own FP64 run.
"""
import os
import subprocess

import numpy as np
import pytest

from swc import scenes

pytestmark = pytest.mark.gpu


def oracle_time_step(ref, step_rate, radius):
    _, v = ref.particles()
    vmax = np.sqrt(np.max(np.sum(v * v, axis=1))) if len(v) else 0.0
    return step_rate * radius * 2 / vmax if vmax > 0 else np.inf


def oracle_frame(ref, target, step_rate, radius):
    """Simulator::advanceTimeBySteps restated over the oracle (Simulator.cpp:103-128)."""
    t, taken = 0.0, []
    while True:
        dt = oracle_time_step(ref, step_rate, radius)
        last = t + dt >= target
        if last:
            dt = target - t
        elif t + 2 * dt >= target:
            dt = (target - t) / 2
        ref.advance(dt)
        t += dt
        taken.append(dt)
        if last:
            return taken


def test_time_step_matches_oracle(swc_mod, oracle_mod):
    s = scenes.projection_block_3d(n=20, seed=8).rounded_to_float32()
    liq = swc_mod.DualParticleSphLiquid(s)
    liq.initialize()
    ref = oracle_mod.Oracle(s)
    ref.initialize()
    for step_rate in (0.4, 1.0):
        assert liq.getTimeStep(100, step_rate) == pytest.approx(oracle_time_step(ref, step_rate, s.particle_radius),
                                                                rel=1e-12)
    for _ in range(3):
        liq.advance(s.dt)
        ref.advance(s.dt)
    # after steps the two FP32 / FP64 trajectories differ by ~1e-7
    assert liq.getTimeStep(100, 0.5) == pytest.approx(oracle_time_step(ref, 0.5, s.particle_radius), rel=1e-5)
    # a particle far faster than the rest sets the step; at rest the step is unbounded
    x, v = liq.getParticles()
    v[123] = [3.0, -4.0, 12.0]
    liq.setParticles(x, v)
    assert liq.getTimeStep(100, 0.5) == pytest.approx(0.5 * 2 * s.particle_radius / 13.0, rel=1e-7)
    liq.setParticles(x, np.zeros_like(v))
    assert liq.getTimeStep(100, 0.5) == np.inf


def test_simulator_frames_match_oracle(swc_mod, oracle_mod, tmp_path):
    """Three frames at 100 frames/s, CFL 0.05 on a 2D block with N(0, 0.1^2)
    velocities (several substeps per frame, the last two of each frame sharing
    the rest): same substep sequence and frame-end velocities as the oracle
    driven by the same rule; frame files and resume."""
    s = scenes.projection_block_2d(n=32, seed=9).rounded_to_float32()
    liq = swc_mod.DualParticleSphLiquid(s)
    sim = swc_mod.Simulator(str(tmp_path / "run"), 0, 4, 100, 0.05, liq)
    sim.Simulate()
    ref = oracle_mod.Oracle(s)
    ref.initialize()
    counts = []
    for frame in (1, 2, 3):
        gpu = [dt for f, dt in sim.substeps if f == frame]
        orc = oracle_frame(ref, 0.01, 0.05, s.particle_radius)
        assert len(gpu) == len(orc), (frame, gpu, orc)
        # the two free-running FP32 / FP64 trajectories (max |v| sets the step) part by ~1e-5 in 7 steps
        np.testing.assert_allclose(gpu, orc, rtol=1e-4)
        assert sum(gpu) == pytest.approx(0.01, abs=1e-15)
        counts.append(len(gpu))
    assert max(counts) >= 3, counts  # the even split of the last two substeps is exercised
    x, v = liq.getParticles()
    xr, vr = ref.particles()
    assert np.linalg.norm(v - vr) / np.linalg.norm(vr) < 1e-4
    for f in range(4):
        assert (tmp_path / "run" / str(f) / "particles.sav").stat().st_size == s.n_particles * 2 * 8
    assert (tmp_path / "run" / "end_frame.txt").read_text().strip() == "4"
    # resume from frame 3 in a fresh object: the next frame matches the continuing run
    liq2 = swc_mod.DualParticleSphLiquid(s)
    swc_mod.Simulator(str(tmp_path / "run"), 4, 5, 100, 0.05, liq2).Simulate()
    cont = swc_mod.Simulator(str(tmp_path / "cont"), 1, 1, 100, 0.05, liq)
    cont.advanceTimeBySteps(0.01)
    assert np.linalg.norm(liq2.getParticles()[1] - liq.getParticles()[1]) / np.linalg.norm(liq.getParticles()[1]) < 1e-5


def test_cpp_simulator_frames(tmp_path):
    """include/swc/Simulator.hpp drives the C++ liquid: frame files, description,
    and substeps that land every frame on 1/100 s."""
    from swc import build

    exe = [e for e in build.build_examples() if e.endswith("dam_break_2d")][0]
    r = subprocess.run([exe, "0", "frames", "3"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    frames, cur = [], []
    for line in r.stdout.splitlines():
        if line.startswith("substep"):
            cur.append(float(line.split("dt")[1].split()[0]))
        elif line.startswith("frame"):
            frames.append(cur)
            cur = []
    assert len(frames) == 3
    for f in frames:
        assert sum(f) == pytest.approx(0.01, abs=1e-15)
    out = tmp_path / "dam_break_2d_frames"
    for f in range(4):
        assert os.path.getsize(out / str(f) / "particles.sav") == 3200 * 2 * 8
        assert (out / str(f) / "dual_state.sav").exists()
    assert (out / "end_frame.txt").read_text().strip() == "4"
    assert (out / "description.yaml").read_text().startswith("dimension: 2")
