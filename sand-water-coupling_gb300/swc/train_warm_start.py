"""Train the learned CG warm start and evaluate it on the 2M projection block.

Training data: 3D dam-break variants (block height along x drawn from
U(0.64, 1.28), square cross-section sized to ~`--particles` particles) and,
with `--block-seeds`, random-velocity projection blocks of `--block-n`^3
particles, each run by the plain solver (CG from the pressure extrapolated in
time to the scene tolerance) with feature logging; a random `--keep` fraction
of the active nodes of every step is kept.  Training: Adam, learning rate 1e-3,
`--epochs` epochs, on the GPU (swc_trainer_*).  Evaluation: the 128^3
projection block with a held-out seed (1234), CG iterations per step from the
node-mapped, extrapolated, learned (with and without the residual fallback)
and zero starts.

    python -m swc.train_warm_start --out swc/models/warm_start.npz
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

if __package__ in (None, ""):
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from swc import learn, scenes  # noqa: E402
from swc.liquid import DualParticleSphLiquid  # noqa: E402


def collect_dataset(seeds, steps, particles, keep, every, block_seeds=0, block_n=80, block_steps=100, rng_seed=0):
    """Dam-break variants (seeds 0..seeds-1) and, optionally, random-velocity
    projection blocks of block_n^3 particles (seeds 100..100+block_seeds-1; the
    held-out evaluation block uses seed 1234)."""
    rng = np.random.default_rng(rng_seed)
    fs, ts, info = [], [], []

    def add(sc, n_steps, s, **meta):
        t0 = time.perf_counter()
        f, t = learn.collect(sc, steps=n_steps, every=every, keep_fraction=keep, seed=s)
        info.append(dict(meta, seed=s, particles=sc.n_particles, rows=int(f.shape[0]),
                         seconds=time.perf_counter() - t0))
        fs.append(f)
        ts.append(t)
        print(json.dumps(info[-1]), flush=True)

    for s in range(seeds):
        height = float(rng.uniform(0.64, 1.28))
        add(scenes.dam_break_3d_variant(seed=s, height=height, target_particles=particles), steps, s,
            scene="dam_break_3d_variant", height=height)
    for s in range(100, 100 + block_seeds):
        add(scenes.projection_block_3d(n=block_n, seed=s), block_steps, s, scene="projection_block_3d")
    return np.concatenate(fs), np.concatenate(ts), info


def evaluate(params, norm, n=128, seed=1234, steps=20):
    """Mean CG iterations per step on the n^3 block (first step excluded: no previous p)."""
    sc = scenes.projection_block_3d(n=n, seed=seed)
    out = {}
    for key, mode, no_fallback in (("node", "node", False), ("extrapolate", "extrapolate", False),
                                   ("learned", "learned", False), ("learned_no_fallback", "learned", True),
                                   ("zero", "zero", False)):
        liq = DualParticleSphLiquid(sc, warm_start=mode, tolerance=sc.tolerance, learned_no_fallback=no_fallback)
        if mode == "learned":
            liq.setMlp(params, norm)
        liq.initialize()
        its, used = [], []
        for _ in range(steps):
            st = liq.advance(sc.dt)
            its.append(int(st["cg_iterations"]))
            used.append(int(st["warm_start_used"]))
        liq.close()
        out[key] = {"iterations": its, "mean": float(np.mean(its[1:])), "warm_start_used": used}
        print(key, json.dumps(out[key]), flush=True)
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--out", required=True)
    ap.add_argument("--seeds", type=int, default=8)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--particles", type=int, default=400_000)
    ap.add_argument("--keep", type=float, default=0.02)
    ap.add_argument("--every", type=int, default=1)
    ap.add_argument("--block-seeds", type=int, default=12)
    ap.add_argument("--block-n", type=int, default=80)
    ap.add_argument("--block-steps", type=int, default=100)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--eval-n", type=int, default=128)
    ap.add_argument("--eval-steps", type=int, default=50)
    args = ap.parse_args(argv)

    f, t, info = collect_dataset(args.seeds, args.steps, args.particles, args.keep, args.every, args.block_seeds,
                                 args.block_n, args.block_steps)
    print(f"dataset: {f.shape[0]} rows", flush=True)
    t0 = time.perf_counter()
    p, q, loss = learn.train(f, t, epochs=args.epochs, lr=args.lr, batch=4096, seed=0)
    print(f"trained in {time.perf_counter() - t0:.1f} s, loss {loss.tolist()}", flush=True)
    ev = evaluate(p, q, n=args.eval_n, steps=args.eval_steps) if args.eval_n > 0 else {}
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    learn.save(args.out, p, q, loss=loss, info=json.dumps({"data": info, "args": vars(args), "eval": ev}))
    print("saved", args.out)


if __name__ == "__main__":
    main()
