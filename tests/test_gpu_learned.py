"""GPU checks of the learned CG warm start: the tensor-core forward pass and the
tensor-core training gradient against the FP64 MLP oracle, and what the trained network
gains (or not) over the plain node-mapped warm start, with the same solution."""
import numpy as np
import pytest

from oracle import mlp_oracle as M
from swc import scenes

pytestmark = pytest.mark.gpu


def _synthetic(n=5000, seed=0):
    rng = np.random.default_rng(seed)
    f = rng.normal(size=(n, M.N_IN)).astype(np.float32)
    t = (np.tanh(f[:, 0]) + 0.5 * f[:, 4] - 0.2 * f[:, 1] * f[:, 5]).astype(np.float32)
    norm = np.concatenate([f.mean(0), f.std(0), [t.mean(), t.std()]]).astype(np.float32)
    return f, t, norm


def test_tensor_core_forward_matches_oracle(swc_mod):
    from swc import learn

    f, t, norm = _synthetic(1000)
    p = learn.init_params(4)
    p[-1] = 0.3
    gpu = learn.forward(p, norm, f)
    ref16 = M.forward(p.astype(np.float64), norm, f, bf16=True)
    ref64 = M.forward(p.astype(np.float64), norm, f, bf16=False)
    scale = np.abs(ref64).max()
    # BF16 operands, FP32 accumulation: against the BF16-emulating oracle ~1e-3, against FP64 ~1e-2
    assert np.abs(gpu - ref16).max() <= 2e-3 * scale, np.abs(gpu - ref16).max() / scale
    assert np.abs(gpu - ref64).max() <= 3e-2 * scale


@pytest.mark.parametrize("n", [777, 4096])
def test_gradient_matches_oracle(swc_mod, n):
    """The tensor-core gradient pass (forward, backward and weight gradients as
    tcgen05 BF16 products, FP32 accumulation) against the FP64 oracle that rounds
    to bfloat16 where the pass does: within 2e-3 (relative norm) for every
    parameter group; against the exact FP64 gradient within the BF16 error."""
    from swc import learn

    f, t, norm = _synthetic(n, seed=1)
    p = learn.init_params(5)
    p[-1] = 0.1
    g, loss = learn.gradient(p, norm, f, t)
    lb, gb = M.loss_and_grad(p.astype(np.float64), norm, f, t, bf16=True)
    lo, go = M.loss_and_grad(p.astype(np.float64), norm, f, t)
    assert loss == pytest.approx(lb, rel=2e-3)
    for name, sl in M.param_groups().items():
        rel = np.linalg.norm(g[sl] - gb[sl]) / np.linalg.norm(gb[sl])
        assert rel < 2e-3, (name, rel)
    rel = np.linalg.norm(g - go) / np.linalg.norm(go)
    assert rel < 3e-2, rel


def test_training_reduces_loss(swc_mod):
    from swc import learn

    f, t, _ = _synthetic(20000, seed=2)
    p, q, loss = learn.train(f, t, epochs=8, lr=3e-3, batch=2048, seed=3)
    assert loss[-1] < 0.3 * loss[0], loss
    pred = learn.forward(p, q, f)
    assert np.mean((pred - t) ** 2) / np.var(t) < 0.3


def test_learned_warm_start_end_to_end(swc_mod):
    """Train on logged data of one seed, evaluate on a held-out seed: same
    solution as the plain solver, and the iteration counts of both."""
    from swc import learn

    train_scene = scenes.projection_block_3d(n=24, seed=11, steps=12)
    f, t = learn.collect(train_scene, steps=12)
    assert f.shape[1] == learn.N_IN and f.shape[0] == t.shape[0] > 1000
    assert np.all(np.isfinite(f)) and np.all(np.isfinite(t))
    p, q, loss = learn.train(f, t, epochs=20, lr=1e-3, batch=4096, seed=0)
    assert loss[-1] <= loss[0]

    test_scene = scenes.projection_block_3d(n=24, seed=99).rounded_to_float32()
    out = {}
    for mode in ("node", "extrapolate", "learned"):
        liq = swc_mod.DualParticleSphLiquid(test_scene, warm_start=mode, compute_true_residual=True)
        if mode == "learned":
            liq.setMlp(p, q)
        liq.initialize()
        its, used = [], []
        for _ in range(8):
            st = liq.advance(test_scene.dt)
            assert st["status"] == 0 and st["true_rel_residual"] < 5 * test_scene.tolerance
            its.append(st["cg_iterations"])
            used.append(st["warm_start_used"])
        out[mode] = (liq.getParticles()[1], np.array(its), used)
        liq.close()
    v_node, it_node, _ = out["node"]
    v_ex, it_ex, _ = out["extrapolate"]
    v_learn, it_learn, used = out["learned"]
    assert np.linalg.norm(v_learn - v_node) / np.linalg.norm(v_node) < 1e-4
    # the residual-based fallback never starts from a worse residual than its base start
    assert it_learn[1:].mean() <= it_ex[1:].mean() + 1.0
    assert used[0] == 1 and all(u in (3, 4) for u in used[1:])  # NODE (no history), then LEARNED / EXTRAPOLATE
    print(f"\nCG iterations  node-mapped: {it_node.tolist()}  extrapolated: {it_ex.tolist()}  "
          f"learned: {it_learn.tolist()}  used: {used}")


def test_history_features_match_pressure_history(swc_mod):
    """The logged features and targets follow their definitions (include/swc.h)
    when recomputed on the host from the pressures of the previous projections,
    matched by lattice node id: the two-level history shift, its activity masks,
    the extrapolated base and the history scale."""
    from swc import _lib

    sc = scenes.projection_block_3d(n=16, seed=5).rounded_to_float32()
    liq = swc_mod.DualParticleSphLiquid(sc, warm_start="extrapolate", keep_features=True)
    liq.initialize()
    hist = []
    for k in range(6):
        liq.advance(sc.dt)
        v = liq.virtual()
        f, t = liq.features()
        ids, p, ah, D = v["node"], v["p"], v["alpha_hat"], v["div"]
        assert f.shape == (ids.shape[0], _lib.MLP_IN)
        sD = np.sqrt(np.mean(D.astype(np.float64) ** 2))
        w = ah / sD
        prev = [dict(zip(h["node"].tolist(), h["p"].tolist())) for h in hist[::-1]]  # one, two, three steps back

        def back(j):
            return np.array([prev[j].get(i, 0.0) if j < len(prev) else 0.0 for i in ids.tolist()])

        def alive(j):
            return np.array([j < len(prev) and i in prev[j] for i in ids.tolist()])

        a1 = alive(0)
        a2 = a1 & alive(1)
        a3 = a2 & alive(2)
        p1, p2, p3 = back(0) * a1, back(1) * a2, back(2) * a3
        dp1, dp2 = np.where(a2, p1 - p2, 0.0), np.where(a3, p1 - 2 * p2 + p3, 0.0)
        base = p1 + dp1 + dp2  # quadratic extrapolation where the history allows
        d1, d2, q = dp1 * w, dp2 * w, p1 * w
        s = np.sqrt(d1 * d1 + d2 * d2) + _lib.MLP_SCALE_EPS
        # FP32 pressures on the device: compare in the units of each quantity
        tol = 2e-5 * np.abs(p).max() * np.abs(w).max()
        np.testing.assert_allclose(f[:, 3] * s, d1, atol=tol)
        np.testing.assert_allclose(f[:, 4] * s, d2, atol=tol)
        np.testing.assert_allclose(np.exp(f[:, 5]), s, rtol=1e-3, atol=tol)
        np.testing.assert_allclose(f[:, 6] * (np.abs(q) + s), q, atol=tol)
        np.testing.assert_allclose(t * s, (p - base) * w, atol=tol)
        np.testing.assert_allclose(f[:, 0], D / sD, rtol=1e-4, atol=1e-6)
        if k >= 3:
            assert a3.sum() > 0.5 * ids.shape[0]
        hist.append(v)
    liq.close()


def test_committed_model_without_fallback(swc_mod):
    """The shipped model (swc/models/warm_start.npz) drives CG on a held-out block
    with the prediction always kept: same solution as the node-mapped start, and
    the learned start is the one used on every step."""
    import os

    from swc import learn

    path = os.path.join(os.path.dirname(learn.__file__), "models", "warm_start.npz")
    p, q = learn.load_model(path)
    sc = scenes.projection_block_3d(n=32, seed=77).rounded_to_float32()
    out = {}
    for mode in ("node", "learned"):
        liq = swc_mod.DualParticleSphLiquid(sc, warm_start=mode, compute_true_residual=True,
                                            learned_no_fallback=True)
        if mode == "learned":
            liq.setMlp(p, q)
        liq.initialize()
        its, used = [], []
        for _ in range(6):
            st = liq.advance(sc.dt)
            assert st["status"] == 0 and st["true_rel_residual"] < 5 * sc.tolerance
            its.append(st["cg_iterations"])
            used.append(st["warm_start_used"])
        out[mode] = (liq.getParticles()[1], its, used)
        liq.close()
    assert all(u == 3 for u in out["learned"][2])  # SWC_WARM_LEARNED
    v_node, v_learn = out["node"][0], out["learned"][0]
    assert np.linalg.norm(v_learn - v_node) / np.linalg.norm(v_node) < 1e-4
    print(f"\nCG iterations  node-mapped: {out['node'][1]}  learned (kept): {out['learned'][1]}")


def test_learned_start_with_feature_logging(swc_mod):
    """Learned start and training-data logging together (the residual test's base
    pass and the logging reduction both run): same solution as the node-mapped
    start, features logged every step."""
    import os

    from swc import learn

    path = os.path.join(os.path.dirname(learn.__file__), "models", "warm_start.npz")
    sc = scenes.projection_block_3d(n=20, seed=21).rounded_to_float32()
    vel = {}
    for mode in ("node", "learned"):
        liq = swc_mod.DualParticleSphLiquid(sc, warm_start=mode, keep_features=(mode == "learned"))
        if mode == "learned":
            liq.setMlp(*learn.load_model(path))
        liq.initialize()
        for _ in range(5):
            st = liq.advance(sc.dt)
            assert st["status"] == 0
            if mode == "learned":
                f, t = liq.features()
                assert f.shape == (liq.numVirtual(), learn.N_IN) and np.all(np.isfinite(f)) and np.all(np.isfinite(t))
        vel[mode] = liq.getParticles()[1]
        liq.close()
    assert np.linalg.norm(vel["learned"] - vel["node"]) / np.linalg.norm(vel["node"]) < 1e-4


@pytest.mark.parametrize("gate", [1, 2])
def test_learned_gate(swc_mod, gate):
    """learned_gate: after that many consecutive rejections by the residual test the
    network is skipped (base start) for 4 x gate steps; after a window one rejection
    of the re-test starts the next, twice as long, until a prediction is kept; the
    solution stays the extrapolated start's to the CG tolerance and skipped steps
    report the base."""
    import os

    from swc import learn

    path = os.path.join(os.path.dirname(learn.__file__), "models", "warm_start.npz")
    sc = scenes.projection_block_3d(n=20, seed=8).rounded_to_float32()
    out = {}
    for mode, g in (("extrapolate", 0), ("learned", gate)):
        liq = swc_mod.DualParticleSphLiquid(sc, warm_start=mode, learned_gate=g)
        if mode == "learned":
            liq.setMlp(*learn.load_model(path))
        liq.initialize()
        used = []
        for _ in range(24):
            st = liq.advance(sc.dt)
            assert st["status"] == 0
            used.append(st["warm_start_used"])
        out[mode] = (liq.getParticles()[1], used)
        liq.close()
    used = out["learned"][1]
    assert np.linalg.norm(out["learned"][0] - out["extrapolate"][0]) / np.linalg.norm(out["extrapolate"][0]) < 1e-4
    # replay the gate on the reported starts: no learned start inside a skip window,
    # every window since the prediction was last kept twice the one before, and a
    # single rejection after a window starting the next
    skip = rejects = windows = failed = 0
    for u in used:
        if skip > 0:
            assert u != 3, used
            skip -= 1
            continue
        rejects = 0 if u == 3 else rejects + 1
        if u == 3:
            failed = 0
        if rejects >= gate or (failed > 0 and rejects > 0):
            skip, rejects, windows = (4 * gate) << min(failed, 4), 0, windows + 1
            failed += 1
    assert windows >= 1 and 3 in used, used
    print(f"\nwarm start used with learned_gate={gate}: {used}")


@pytest.mark.parametrize("case", ["block_64", "dam_break"])
def test_shipped_model_gain_over_extrapolation(swc_mod, case):
    """What the trained network gains over the same method without it, on held-out
    scenes (seeds and sizes outside the training recipe's), over the first 15
    steps with the residual test (the shipped swc/models/warm_start.npz) against
    the quadratic extrapolation it corrects, to the same tolerance and solution:
      random-velocity 64^3 block: fewer CG iterations in total (measured: 202
        against 221);
      3D dam-break column: the residual test rejects the prediction after the
        second step, so the network gains nothing there and costs no iteration
        (measured: 229 and 229)."""
    import os

    from swc import learn

    path = os.path.join(os.path.dirname(learn.__file__), "models", "warm_start.npz")
    if case == "block_64":
        sc = scenes.projection_block_3d(n=64, seed=4321).rounded_to_float32()
    else:
        sc = scenes.dam_break_3d_variant(seed=57, height=0.9, target_particles=120_000).rounded_to_float32()
    out = {}
    for mode in ("extrapolate", "learned"):
        liq = swc_mod.DualParticleSphLiquid(sc, warm_start=mode, compute_true_residual=True)
        if mode == "learned":
            liq.setMlp(*learn.load_model(path))
        liq.initialize()
        its, used = [], []
        for _ in range(15):
            st = liq.advance(sc.dt)
            assert st["status"] == 0 and st["true_rel_residual"] < 5 * sc.tolerance
            its.append(st["cg_iterations"])
            used.append(st["warm_start_used"])
        out[mode] = (liq.getParticles()[1], np.array(its), used)
        liq.close()
    v_ex, it_ex, _ = out["extrapolate"]
    v_l, it_l, used = out["learned"]
    print(f"\n{case}: CG iterations  extrapolated {it_ex.tolist()} (sum {it_ex.sum()})  "
          f"learned {it_l.tolist()} (sum {it_l.sum()})  starts used {used}")
    assert np.linalg.norm(v_l - v_ex) / np.linalg.norm(v_ex) < 1e-4
    assert 3 in used  # the prediction was kept on some steps
    if case == "block_64":
        assert it_l.sum() <= 0.95 * it_ex.sum(), (it_l.tolist(), it_ex.tolist())
    else:
        assert it_l.sum() <= it_ex.sum(), (it_l.tolist(), it_ex.tolist())


def test_training_recipe_end_to_end(swc_mod, tmp_path):
    """The shipped model's recipe (python -m swc.train_warm_start) run end to end at
    a small size: dam-break variants and random-velocity blocks logged by the
    plain solver started from the extrapolated pressure, GPU training on the
    tensor cores, evaluation, and a model file that drives the learned start to
    the plain solver's solution."""
    from swc import learn, train_warm_start

    out = str(tmp_path / "model.npz")
    train_warm_start.main(["--out", out, "--seeds", "2", "--steps", "12", "--particles", "20000",
                           "--keep", "0.5", "--block-seeds", "1", "--block-n", "24", "--block-steps", "10",
                           "--epochs", "4", "--eval-n", "24", "--eval-steps", "6"])
    p, q = learn.load_model(out)
    assert p.shape == (learn.N_PARAMS,) and np.all(np.isfinite(p)) and np.all(np.isfinite(q))
    sc = scenes.projection_block_3d(n=20, seed=31).rounded_to_float32()
    vel = {}
    for mode in ("node", "learned"):
        liq = swc_mod.DualParticleSphLiquid(sc, warm_start=mode)
        if mode == "learned":
            liq.setMlp(p, q)
        liq.initialize()
        for _ in range(5):
            assert liq.advance(sc.dt)["status"] == 0
        vel[mode] = liq.getParticles()[1]
        liq.close()
    assert np.linalg.norm(vel["learned"] - vel["node"]) / np.linalg.norm(vel["node"]) < 1e-4
