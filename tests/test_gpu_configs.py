"""GPU parity at the benchmark workloads' own sizes: the CUDA path through the C ABI
against the FP64 oracle (VirtualParticle.cpp:18-201, DualParticleSphLiquid.cpp:112-126).

Per-step replay: before the compared step the oracle is handed the GPU's state
(particles, V_i, boundary particles as they stand, rho_b / V_b, rho0, alpha0,
kappa), so a comparison measures one step of the path and not the divergence of
two chaotic FP32 / FP64 trajectories; after its own move (checked against the
GPU's to 1e-6) it projects the GPU's moved positions (see replay).

  2D dam break, 3,200 particles: all 200 steps replayed, both solvers starting CG
      from the same vector (the reference's stale prefix of the GPU's last
      solution), iteration counts compared.
  3D dam break, 524,288 particles: one step after 10 advances, same start.
  isolated projection block, 128^3 = 2,097,152 particles: one step after 5
      advances with the learned warm start the benchmark runs.
  paddle tank, 8,388,608 particles filling the tank from the floor with a
      1M-particle rotating paddle blade: one step after 3 advances with the learned
      warm start (a smaller tank when the host has no room for the oracle's
      ~8.9M-row operator; the size is printed).

For the learned steps the oracle's CG starts from the GPU's solution: its FP64
residual must already be near the tolerance (the oracle then adds a few
iterations at most), and the velocity update compared is the one of that pressure.
The plain steps start both solvers from the same stale-prefix vector and compare
their iteration counts.

Bars (FP32 state and sums against FP64): identical active virtual sets; rho_I,
V_I, alpha_hat 2e-5 relative; D_I 1e-4 of max |D|; vbar_I and post-projection
velocity 1e-4 relative (norm); the GPU pressure solves the oracle's FP64 system:
|D - A p| / |D| below 20 x tolerance + 1e-5.
"""
import os

import numpy as np
import pytest

from swc import learn, scenes

pytestmark = pytest.mark.gpu

MODEL = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "sand-water-coupling_gb300", "swc",
                     "models", "warm_start.npz")


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def mem_available_gb():
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) / 2**20
    except OSError:
        pass
    return 0.0


def sync(liq, ref, boundary=False):
    """The GPU's pre-step state into the oracle."""
    if boundary:
        xb, nb, vb = liq.getBoundary()
        ref.set_boundary(xb, nb, vb)
    x, v = liq.getParticles()
    ref.set_particles(x, v)
    ref.set_volumes(liq.realInfo()[1])
    ref.set_boundary_info(*liq.boundaryInfo())
    sc = liq.scalars()
    ref.set_scalars(sc["rho0"], sc["alpha0"], sc["kappa"])


def compare(liq, ref, st, tol, label):
    gv = liq.virtual(with_vbar=True)
    ov = ref.virtual()
    assert np.array_equal(gv["node"], ov["node"]), f"{label}: active virtual sets differ"
    np.testing.assert_allclose(gv["rho"], ov["rho"], rtol=2e-5, atol=1e-6 * np.abs(ov["rho"]).max())
    np.testing.assert_allclose(gv["vol"], ov["vol"], rtol=2e-5, atol=1e-6 * np.abs(ov["vol"]).max())
    np.testing.assert_allclose(gv["alpha_hat"], ov["alpha_hat"], rtol=2e-5)
    np.testing.assert_allclose(gv["div"], ov["div"], rtol=0, atol=1e-4 * np.abs(ov["div"]).max())
    e_vbar = rel(gv["vbar"], ov["vbar"])
    assert e_vbar < 1e-4, (label, e_vbar)
    x, v = liq.getParticles()
    xr, vr = ref.particles()
    np.testing.assert_allclose(x, xr, rtol=0, atol=1e-6)
    e_v = rel(v, vr)
    assert e_v < 1e-4, (label, e_v)
    res = np.linalg.norm(ov["div"] - ref.apply_operator(gv["p"])) / np.linalg.norm(ov["div"])
    assert res < 20 * tol + 1e-5, (label, res)
    return {"velocity": e_v, "vbar": e_vbar, "fp64_residual_of_gpu_p": float(res), "n_virtual": len(gv["node"]),
            "gpu_iterations": st["cg_iterations"], "oracle_iterations": ref.stats()["iterations"]}


def replay(liq, ref, s, label, start, boundary=False):
    """One advance on both sides from the GPU's pre-step state.  The oracle moves
    the particles and applies gravity and viscosity itself (FP64), then takes the
    GPU's moved positions (and boundary) before its projection, so that both
    project the same positions: the FP32 rounding of the move is checked on its
    own (1e-6) and cannot flip a neighbour at r = h, where rho_I's W_H cut at h
    jumps.  start: "prefix" hands the oracle the GPU's previous solution as the
    stale-prefix warm start (the same CG iteration from the same vector), "gpu"
    the GPU's solution of this step."""
    sync(liq, ref, boundary)
    p_prev = liq.virtual()["p"]
    st = liq.advance(s.dt)
    assert st["status"] == 0, (label, st)
    ref.move_and_forces(s.dt)
    xg, _ = liq.getParticles()
    xo, vo = ref.particles()
    np.testing.assert_allclose(xg, xo, rtol=0, atol=1e-6)
    ref.set_particles(xg, vo)
    if boundary:
        xb, nb, vb = liq.getBoundary()
        ref.set_boundary(xb, nb, vb)
    ref.set_pressure(p_prev if start == "prefix" else liq.virtual()["p"])
    ref.project()
    out = compare(liq, ref, st, s.tolerance, label)
    if start == "gpu":
        # the GPU's pressure is converged in FP64 too: the oracle has little left to do
        assert out["oracle_iterations"] <= max(5, out["gpu_iterations"]), (label, out)
    return out


def test_dam_break_2d_all_200_steps(swc_mod, oracle_mod):
    s = scenes.dam_break_2d(seed=0).rounded_to_float32()
    assert s.n_particles == 3200 and s.steps == 200
    liq = swc_mod.DualParticleSphLiquid(s, keep_virtual_velocity=True)
    liq.initialize()
    ref = oracle_mod.Oracle(s)
    ref.initialize()
    worst = {"velocity": 0.0, "vbar": 0.0, "fp64_residual_of_gpu_p": 0.0}
    it_diff = []
    for step in range(s.steps):
        out = replay(liq, ref, s, f"step {step}", "prefix")
        for k in worst:
            worst[k] = max(worst[k], out[k])
        it_diff.append(out["gpu_iterations"] - out["oracle_iterations"])
    # the same Hestenes-Stiefel iteration from the same start: FP32 SpMVs move the
    # crossing of the tolerance by at most one iteration
    assert max(abs(d) for d in it_diff) <= 1, it_diff
    print(f"\n2D dam break, 200 steps: worst {worst}, iteration differences {np.bincount(np.abs(it_diff))}")


def test_dam_break_3d_524k(swc_mod, oracle_mod):
    s = scenes.dam_break_3d(seed=0).rounded_to_float32()
    assert s.n_particles == 524288
    liq = swc_mod.DualParticleSphLiquid(s, keep_virtual_velocity=True)
    liq.initialize()
    for _ in range(10):
        assert liq.advance(s.dt)["status"] == 0
    ref = oracle_mod.Oracle(s, searcher="cells")
    out = replay(liq, ref, s, "3D dam break 524,288, step 11", "prefix")
    assert abs(out["gpu_iterations"] - out["oracle_iterations"]) <= 1, out
    print(f"\n3D dam break, step 11: {out}")


def test_projection_block_2m(swc_mod, oracle_mod):
    s = scenes.projection_block_3d(n=128, seed=0).rounded_to_float32()
    assert s.n_particles == 2097152 and s.n_boundary == 202816
    liq = swc_mod.DualParticleSphLiquid(s, warm_start="learned", learned_gate=2, keep_virtual_velocity=True)
    liq.setMlp(*learn.load_model(MODEL))
    liq.initialize()
    for _ in range(5):
        assert liq.advance(s.dt)["status"] == 0
    ref = oracle_mod.Oracle(s, searcher="cells")
    print(f"\n{replay(liq, ref, s, 'projection block 2,097,152, step 6', 'gpu')}")


def test_paddle_tank(swc_mod, oracle_mod):
    # the oracle's operator holds ~3.1 kB per active node (about 8.9M nodes at full size)
    full = mem_available_gb() >= 64
    kw = {} if full else dict(n_fluid=1_048_576, domain=(2.0, 1.0, 1.0), paddle_particles=125_000,
                              paddle_half=(0.025, 0.25, 0.125))
    s = scenes.paddle_tank_3d(seed=0, **kw).rounded_to_float32()
    label = f"paddle tank {s.n_particles} particles, {s.n_boundary} boundary ({'full size' if full else 'reduced'})"
    liq = swc_mod.DualParticleSphLiquid(s, warm_start="learned", learned_gate=2, keep_virtual_velocity=True)
    liq.setMlp(*learn.load_model(MODEL))
    liq.initialize()
    for _ in range(3):
        assert liq.advance(s.dt)["status"] == 0
    ref = oracle_mod.Oracle(s, searcher="cells")
    moving = np.zeros(s.n_boundary, np.uint8)
    moving[s.meta["n_walls"]:] = 1
    ref.set_boundary_motion(moving, s.meta["paddle_center"], s.meta["paddle_omega"])
    print(f"\n{label}: {replay(liq, ref, s, label, 'gpu', boundary=True)}")
