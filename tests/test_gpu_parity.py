"""GPU parity: the CUDA path (through the C ABI) against the FP64 oracle.

Inputs are rounded through float32 first so both sides see identical values.
Per-projection replay: before each compared step the oracle is handed the GPU's
state (positions, velocities, per-particle volumes, boundary volumes, rho0,
alpha0, kappa), so each comparison measures one step of the path and not the
divergence of two chaotic trajectories.

Tolerances (FP32 state and kernel sums vs FP64):
  neighbour sets and the active virtual set: identical
  rho_i, V_i, rho_I, V_I, alpha_hat: 2e-5 relative (element-wise)
  D_I: 1e-4 of max |D|
  post-projection velocity: 1e-4 relative (norm), the path's stated bar
"""
import numpy as np
import pytest

from swc import scenes

pytestmark = pytest.mark.gpu

TOL_V = 1e-4


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def make_pair(swc_mod, oracle_mod, scene, **kw):
    s = scene.rounded_to_float32()
    liq = swc_mod.DualParticleSphLiquid(s, keep_virtual_velocity=True, keep_features=True, **kw)
    liq.initialize()
    ref = oracle_mod.Oracle(s, tolerance=kw.get("tolerance"))
    ref.initialize()
    return s, liq, ref


def sync_oracle(liq, ref):
    """Hand the GPU's state to the oracle (replay)."""
    x, v = liq.getParticles()
    ref.set_particles(x, v)
    _, vol = liq.realInfo()
    ref.set_volumes(vol)
    rb, vb = liq.boundaryInfo()
    ref.set_boundary_info(rb, vb)
    sc = liq.scalars()
    ref.set_scalars(sc["rho0"], sc["alpha0"], sc["kappa"])


SCENES = {
    "dam_break_2d": lambda: scenes.dam_break_2d(seed=0),
    "block_3d_n16": lambda: scenes.projection_block_3d(n=16, seed=1),
    "block_3d_n24": lambda: scenes.projection_block_3d(n=24, seed=2),
    "dam_break_3d_small": lambda: scenes.dam_break_3d(seed=3, cells=(24, 12, 12), domain=(0.4, 0.2, 0.2)),
}


@pytest.mark.parametrize("name", sorted(SCENES))
def test_initialize_parity(swc_mod, oracle_mod, name):
    s, liq, ref = make_pair(swc_mod, oracle_mod, SCENES[name]())
    rg, vg = liq.realInfo()
    rr, vr = ref.real_info()
    np.testing.assert_allclose(rg, rr, rtol=2e-5)
    np.testing.assert_allclose(vg, vr, rtol=2e-5)
    brg, bvg = liq.boundaryInfo()
    brr, bvr = ref.boundary_info()
    np.testing.assert_allclose(brg, brr, rtol=2e-5)
    np.testing.assert_allclose(bvg, bvr, rtol=2e-5)
    g, o = liq.scalars(), ref.scalars()
    assert g["rho0"] == pytest.approx(o["rho0"], rel=2e-5)
    assert g["alpha0"] == pytest.approx(o["alpha0"], rel=2e-5)
    assert g["kappa"] == pytest.approx(o["kappa"], rel=1e-12)


@pytest.mark.parametrize("name", sorted(SCENES))
def test_projection_step_parity(swc_mod, oracle_mod, name):
    s, liq, ref = make_pair(swc_mod, oracle_mod, SCENES[name]())
    for step in range(3):
        sync_oracle(liq, ref)
        gp = liq.virtual()["p"] if step else np.zeros(0)
        ref.set_pressure(gp)  # same warm start (reference prefix semantics)
        st = liq.advance(s.dt)
        ref.advance(s.dt)
        assert st["status"] == 0
        gv = liq.virtual(with_vbar=True)
        ov = ref.virtual()
        assert np.array_equal(gv["node"], ov["node"]), "active virtual sets differ"
        np.testing.assert_allclose(gv["rho"], ov["rho"], rtol=2e-5, atol=1e-6 * np.abs(ov["rho"]).max())
        np.testing.assert_allclose(gv["vol"], ov["vol"], rtol=2e-5, atol=1e-6 * np.abs(ov["vol"]).max())
        np.testing.assert_allclose(gv["alpha_hat"], ov["alpha_hat"], rtol=2e-5)
        np.testing.assert_allclose(gv["div"], ov["div"], rtol=0, atol=1e-4 * np.abs(ov["div"]).max())
        assert rel(gv["vbar"], ov["vbar"]) < 1e-4
        x, v = liq.getParticles()
        xr, vr = ref.particles()
        np.testing.assert_allclose(x, xr, rtol=0, atol=1e-6)
        assert rel(v, vr) < TOL_V, (step, rel(v, vr))
        # the GPU pressure solves the oracle's FP64 system to the CG tolerance
        res = np.linalg.norm(ov["div"] - ref.apply_operator(gv["p"])) / np.linalg.norm(ov["div"])
        assert res < 20 * s.tolerance + 1e-5, res
        # same Hestenes-Stiefel iteration on both sides: iteration counts agree
        # (FP32 SpMV vs FP64 can move the crossing of the tolerance by one)
        assert abs(st["cg_iterations"] - ref.stats()["iterations"]) <= 1, (st["cg_iterations"], ref.stats())


def test_moving_paddle_parity(swc_mod, oracle_mod):
    """Rotating solid (paddle-tank extension): both sides turn the paddle particles
    rigidly each step, rebuild the boundary grid and use v_b = omega x (x - c)."""
    sc = scenes.paddle_tank_3d(seed=5, cells=(20, 10, 20), domain=(0.4, 0.2, 0.4), paddle_particles=3000,
                               paddle_half=(0.05, 0.01, 0.08), omega=2.0)
    moving = np.zeros(sc.n_boundary, np.uint8)
    moving[sc.meta["n_walls"]:] = 1
    s, liq, ref = make_pair(swc_mod, oracle_mod, sc)
    liq.setBoundaryMotion(moving, sc.meta["paddle_center"], sc.meta["paddle_omega"])
    ref.set_boundary_motion(moving, sc.meta["paddle_center"], sc.meta["paddle_omega"])
    for step in range(3):
        sync_oracle(liq, ref)
        ref.set_pressure(liq.virtual()["p"] if step else np.zeros(0))
        st = liq.advance(s.dt)
        ref.advance(s.dt)
        assert st["status"] == 0
        gv, ov = liq.virtual(), ref.virtual()
        assert np.array_equal(gv["node"], ov["node"]), "active virtual sets differ"
        x, v = liq.getParticles()
        xr, vr = ref.particles()
        assert rel(v, vr) < TOL_V, (step, rel(v, vr))


def scene_with_outliers():
    """block_3d_n16 with 30 particles moved outside the node lattice: 24 far beyond
    each face (no neighbours) and 6 within 0.3 spacings of a face, in reach of the
    border nodes (both sides clamp them into the border cells of their grids)."""
    sc = scenes.projection_block_3d(n=16, seed=6)
    o = np.asarray(sc.grid_origin[:3])
    hi = o + (np.asarray(sc.grid_size[:3]) - 1) * sc.grid_spacing
    mid = (o + hi) / 2
    x = sc.positions.copy()
    rng = np.random.default_rng(6)
    k = 0
    for axis in range(3):
        for side, edge in ((-1, o[axis]), (1, hi[axis])):
            for _ in range(4):
                p = mid + rng.uniform(-0.05, 0.05, 3)
                p[axis] = edge + side * rng.uniform(0.05, 0.2)
                x[k] = p
                k += 1
            p = mid + rng.uniform(-0.05, 0.05, 3)
            p[axis] = edge + side * 0.3 * sc.grid_spacing
            x[k] = p
            k += 1
    sc.positions = x
    return sc


def test_particles_outside_the_lattice(swc_mod, oracle_mod):
    """Particles beyond the node lattice (escaped past the walls) sit in the border
    cells on the GPU: the same neighbour sets, virtual sets and velocities as the
    oracle over three steps."""
    s, liq, ref = make_pair(swc_mod, oracle_mod, scene_with_outliers())
    for step in range(3):
        sync_oracle(liq, ref)
        ref.set_pressure(liq.virtual()["p"] if step else np.zeros(0))
        st = liq.advance(s.dt)
        ref.advance(s.dt)
        assert st["status"] == 0
        gv, ov = liq.virtual(), ref.virtual()
        assert np.array_equal(gv["node"], ov["node"]), "active virtual sets differ"
        np.testing.assert_allclose(gv["rho"], ov["rho"], rtol=2e-5, atol=1e-6 * np.abs(ov["rho"]).max())
        x, v = liq.getParticles()
        xr, vr = ref.particles()
        np.testing.assert_allclose(x, xr, rtol=0, atol=1e-6)
        assert rel(v, vr) < TOL_V, (step, rel(v, vr))
        outer = np.arange(30)  # the outliers keep their rows (ids) in getParticles
        assert rel(v[outer], vr[outer]) < TOL_V, (step, rel(v[outer], vr[outer]))
    for which in ("real", "boundary", "virtual"):
        cg, og, ig = liq.neighbors(which, x[:30])
        co, oo, io = ref.neighbors(which, x[:30])
        assert np.array_equal(cg, co), which
        if which == "virtual":
            io = ref.virtual()["node"][io]
            for t in range(30):
                io[oo[t]:oo[t + 1]].sort()
        assert np.array_equal(ig, io), which


@pytest.mark.parametrize("name", ["dam_break_2d", "block_3d_n16"])
def test_neighbour_sets_exact(swc_mod, oracle_mod, name):
    s, liq, ref = make_pair(swc_mod, oracle_mod, SCENES[name]())
    sync_oracle(liq, ref)
    liq.advance(s.dt)
    ref.advance(s.dt)
    x, _ = liq.getParticles()
    rng = np.random.default_rng(0)
    # queries: real particles, virtual node positions, and random points near the fluid
    v = liq.virtual()
    q_nodes = liq.nodePositions(v["node"][rng.choice(len(v["node"]), size=min(400, len(v["node"])), replace=False)])
    q_rand = x[rng.choice(len(x), 300)] + rng.uniform(-0.02, 0.02, size=(300, s.dim))
    q_real = x[rng.choice(len(x), 300)]
    for which in ("real", "boundary", "virtual"):
        for q in (q_real, q_nodes, q_rand):
            cg, og, ig = liq.neighbors(which, q)
            co, oo, io = ref.neighbors(which, q)
            assert np.array_equal(cg, co), which
            if which == "virtual":
                node_ids = ref.virtual()["node"]
                io = node_ids[io]
                for t in range(len(q)):
                    io[oo[t]:oo[t + 1]].sort()
            assert np.array_equal(ig, io), which


def test_apply_operator_parity(swc_mod, oracle_mod):
    s, liq, ref = make_pair(swc_mod, oracle_mod, SCENES["block_3d_n24"]())
    sync_oracle(liq, ref)
    ref.set_pressure(np.zeros(0))
    liq.advance(s.dt)
    ref.advance(s.dt)
    n = liq.numVirtual()
    x = np.random.default_rng(1).normal(size=n).astype(np.float32).astype(np.float64)
    yg = liq.applyOperator(x)
    yo = ref.apply_operator(x)
    assert rel(yg, yo) < 2e-6


@pytest.mark.parametrize("name", ["dam_break_2d_small", "projection_block_3d_n8"])
def test_against_golden_fixture(swc_mod, name):
    import os
    import sys

    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(here, "golden"))
    import make_golden

    g = np.load(os.path.join(here, "golden", name + ".npz"))
    build, steps = make_golden.CASES[name]
    s = build().rounded_to_float32()
    liq = swc_mod.DualParticleSphLiquid(s)
    liq.initialize()
    rho, vol = liq.realInfo()
    np.testing.assert_allclose(rho, g["init_rho"], rtol=2e-5)
    np.testing.assert_allclose(vol, g["init_vol"], rtol=2e-5)
    assert liq.scalars()["alpha0"] == pytest.approx(float(g["alpha0"]), rel=2e-5)
    for k in range(steps):
        liq.advance(s.dt)
        v = liq.virtual()
        assert np.array_equal(v["node"], g[f"s{k}_node"])
        np.testing.assert_allclose(v["alpha_hat"], g[f"s{k}_alpha_hat"], rtol=5e-5)
        x, vel = liq.getParticles()
        np.testing.assert_allclose(x, g[f"s{k}_x"], rtol=0, atol=1e-6)
        assert rel(vel, g[f"s{k}_v"]) < 5 * TOL_V


def test_warm_start_modes_agree(swc_mod, oracle_mod):
    base = SCENES["block_3d_n24"]().rounded_to_float32()
    results = {}
    for mode in ("prefix", "node", "zero"):
        liq = swc_mod.DualParticleSphLiquid(base, warm_start=mode, compute_true_residual=True)
        liq.initialize()
        for _ in range(3):
            st = liq.advance(base.dt)
            assert st["status"] == 0 and st["true_rel_residual"] < 5 * base.tolerance
        results[mode] = (liq.getParticles()[1], st["cg_iterations"])
    for mode in ("node", "zero"):
        assert rel(results[mode][0], results["prefix"][0]) < 1e-4
    assert results["node"][1] <= results["zero"][1]


def test_switch_to_prefix_warm_start(swc_mod):
    """Modes other than the stale prefix skip the per-step export of the solution in
    reference order; switching to the prefix mode exports the last solution, so
    the next solve starts from it as if the prefix mode had run all along."""
    base = SCENES["block_3d_n24"]().rounded_to_float32()
    out = {}
    for first in ("prefix", "node"):
        liq = swc_mod.DualParticleSphLiquid(base, warm_start=first)
        liq.initialize()
        for _ in range(3):
            assert liq.advance(base.dt)["status"] == 0
        liq.setSolverOptions(warm_start="prefix")
        st = liq.advance(base.dt)
        assert st["status"] == 0
        out[first] = (liq.getParticles()[1], st["cg_iterations"], st["initial_rel_residual"])
        liq.close()
    assert rel(out["node"][0], out["prefix"][0]) < 1e-4
    assert abs(out["node"][1] - out["prefix"][1]) <= 2, (out["node"][1], out["prefix"][1])
    # an empty prefix (no export) would start from zero: initial residual 1
    assert out["node"][2] < 0.9 and abs(out["node"][2] - out["prefix"][2]) < 0.1 * out["prefix"][2] + 1e-3


def test_extrapolated_warm_start(swc_mod):
    """Warm start extrapolated in time per lattice node (quadratic, 3 p1 - 3 p2 + p3): the
    same solution as the node-mapped start to the CG tolerance; the node-mapped
    start on the first advance (no history) and after a standalone project() or a
    switch into the mode, the extrapolation from the next advance on."""
    base = SCENES["block_3d_n24"]().rounded_to_float32()
    out = {}
    for mode in ("node", "extrapolate"):
        liq = swc_mod.DualParticleSphLiquid(base, warm_start=mode, compute_true_residual=True)
        liq.initialize()
        its, used = [], []
        for _ in range(8):
            st = liq.advance(base.dt)
            assert st["status"] == 0 and st["true_rel_residual"] < 5 * base.tolerance
            its.append(st["cg_iterations"])
            used.append(st["warm_start_used"])
        out[mode] = (liq.getParticles()[1], np.array(its), used)
        if mode == "extrapolate":
            liq.project()
            assert [liq.advance(base.dt)["warm_start_used"] for _ in range(2)] == [1, 4]
        else:
            liq.setSolverOptions(warm_start="extrapolate")
            assert [liq.advance(base.dt)["warm_start_used"] for _ in range(2)] == [1, 4]
        liq.close()
    v_node, it_node, _ = out["node"]
    v_ex, it_ex, used = out["extrapolate"]
    assert used == [1] + [4] * 7  # SWC_WARM_NODE, then SWC_WARM_EXTRAPOLATE
    assert rel(v_ex, v_node) < 1e-4
    assert it_ex[2:].mean() <= it_node[2:].mean() + 1.0
    print(f"\nCG iterations  node-mapped: {it_node.tolist()}  extrapolated: {it_ex.tolist()}")


def test_deterministic_repeat(swc_mod):
    s = SCENES["block_3d_n16"]().rounded_to_float32()
    outs = []
    for _ in range(2):
        liq = swc_mod.DualParticleSphLiquid(s)
        liq.initialize()
        for _ in range(3):
            liq.advance(s.dt)
        outs.append(liq.getParticles())
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_status_codes(swc_mod):
    s = SCENES["block_3d_n16"]().rounded_to_float32()
    liq = swc_mod.DualParticleSphLiquid(s, max_iterations=1, tolerance=1e-12)
    liq.initialize()
    st = liq.advance(s.dt)
    assert st["status"] == 1 and st["cg_iterations"] == 1  # SWC_CG_NOT_CONVERGED, no exit
    liq2 = swc_mod.DualParticleSphLiquid(s, raise_on_nonconvergence=True, max_iterations=1, tolerance=1e-12)
    liq2.initialize()
    with pytest.raises(swc_mod.SwcError):
        liq2.advance(s.dt)
    # NaN velocities: detected and reported, the context stays usable
    liq3 = swc_mod.DualParticleSphLiquid(s)
    liq3.initialize()
    x, v = liq3.getParticles()
    v[5, 0] = np.nan
    liq3.setParticles(x, v)
    with pytest.raises(swc_mod.SwcError) as e:
        liq3.project()
    assert e.value.status == 2
    v[5, 0] = 0.0
    liq3.setParticles(x, v)
    assert liq3.project()["status"] == 0
    with pytest.raises(swc_mod.SwcError):
        liq3.setParticles(x[:10], v[:10])  # count change after initialize
    with pytest.raises(swc_mod.SwcError) as e:
        liq3.setSolverOptions(warm_start=5)  # no such warm-start mode
    assert e.value.status == 3


def test_frame_roundtrip(swc_mod, tmp_path):
    s = SCENES["dam_break_2d"]().rounded_to_float32()
    a = swc_mod.DualParticleSphLiquid(s)
    a.initialize()
    for _ in range(3):
        a.advance(s.dt)
    a.saveFrame(str(tmp_path / "3"))
    a.writeFrame(str(tmp_path / "3"))
    a.writeDescription(str(tmp_path / "description.yaml"))
    b = swc_mod.DualParticleSphLiquid(s)
    b.loadFrame(str(tmp_path / "3"))
    a.advance(s.dt)
    b.advance(s.dt)
    xa, va = a.getParticles()
    xb, vb = b.getParticles()
    np.testing.assert_array_equal(xa, xb)
    assert rel(vb, va) < 1e-5
    n = np.frombuffer((tmp_path / "3" / "particles.mesh").read_bytes()[:4], dtype=np.uint32)[0]
    assert n == s.n_particles
