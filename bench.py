"""Benchmark of the GB300 dual-particle SPH projection.

Workload (default): the isolated projection benchmark, 128^3 = 2,097,152 fluid
particles at spacing 0.01 with U(+-0.1 spacing) jitter, N(0, 0.1^2) velocities,
two boundary layers on all faces (202,816 particles), dt = 5e-4 with gravity,
CG relative tolerance 1e-5.  One step = DualParticleSphLiquid::advance(dt):
advection, rho_i, gravity + viscosity, virtual generation, projection (CG), G_i.

Metric: projection steps/s at 2M particles.  ``value`` is device time (CUDA
events on the library's stream) with the state resident in HBM; ``e2e`` runs the
same steps through the public API with host FP64 buffers (pinned), the
host->device copy of each step's particle state and the device->host read of
its result inside the timed region.  The headline form is the learned warm
start (the trained model in swc/models/: a per-node correction of the
pressure extrapolated in time, kept when it starts CG from a smaller residual
than the extrapolation itself, the network skipped for 8 steps after 2
consecutive rejections, each further window without a kept prediction twice
as long); ``forms`` reports plain CG from the node-mapped previous pressure,
from the reference's stale prefix and from zero, the extrapolated start alone,
the learned start evaluated every step and the learned start without the
residual test, all on the same scene and steps.
``sand`` measures the DEM sand step (DEMParticleSand::advance) on a 2,009,840
particle block the same way (device steps/s, e2e, roofline, CPU port).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl swc|reference]

--impl reference times the reference algorithm's CPU implementation (the FP64
OpenMP restatement in oracle/, all host threads) on the same full-size block:
one untimed step, then up to --steps timed steps within about a minute (the
line's ``steps`` is the number timed).
Under torchrun each rank runs an independent replica (the path does not
shard); value = all ranks' steps / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "sand-water-coupling_gb300"))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "projection steps/s at 2M particles (CG to 1e-5 relative residual)"
UNIT = "steps/s"
# learned warm start trained by swc/train_warm_start.py (dam-break variants + blocks, seeds
# disjoint from the benchmark block's)
MODEL = os.path.join(ROOT, "sand-water-coupling_gb300", "swc", "models", "warm_start.npz")
# the headline learned form skips the network for 8 steps after 2 consecutive
# rejections by the residual test, doubling while it keeps being rejected
# (learned_always evaluates it every step)
LEARNED_GATE = 2


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


SM_MAX_MHZ = 2070.0
# ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch on the 128^3 block,
# per active node of the captured launch: k_cg_spmv 32,769,792 B at 2,246,535 nodes,
# k_node_gather 90,965,504 + 13,017,856 B and k_pressure_gradient 113,461,248 + 12,455,680 B
# at 2,246,538 nodes (profiles/)
DRAM_BYTES_PER_NODE = {"cg_spmv": 32769792 / 2246535, "virtual_gather": (90965504 + 13017856) / 2246538,
                       "pressure_gradient": (113461248 + 12455680) / 2246538}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        # one nvidia-smi in loop mode (50 ms period), read line by line until stopped
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self._proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                           "--format=csv,noheader,nounits", "-lms", "50"],
                                          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            return
        for line in self._proc.stdout:
            if self._stop.is_set():
                break
            line = line.strip()
            if line:
                self.samples.append([x.strip() for x in line.split(",")])

    def __enter__(self):
        self._proc = None
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._proc is not None:
            self._proc.terminate()  # our own child process, by handle
            try:
                self._proc.wait(timeout=5)
            except Exception:
                self._proc.kill()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if len(s) > 3 + k and
                          s[3 + k].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist

        backend = os.environ.get("SWC_DIST_BACKEND") or ("nccl" if torch.cuda.is_available() else "gloo")
        if backend == "nccl":
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group(backend=backend)
        return dist, rank, ws
    return None, rank, ws


def reduce_max(dist, value):
    if dist is None:
        return value
    import torch

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def replica_value(ws, steps, ms_max):
    """Whole-job steps/s of `ws` independent replicas that each ran `steps` steps, the
    slowest taking `ms_max` milliseconds (replicas only: the path does not shard)."""
    return ws * steps / (ms_max / 1e3)


def cpu_reference(args, steps=2, warmup=1, policy=False, time_cap=None):
    """The reference algorithm's CPU implementation (the FP64 oracle port, all host
    threads) on the full benchmark block: `warmup` untimed advance steps, then up to
    `steps` timed ones (fewer when `time_cap` seconds run out, at least one).

    The oracle searches neighbours with a cell grid over the reference's own hash
    cells (the same neighbour sets).  The reference's hash (OR of three prime
    products mod 2N buckets) fills few buckets when 2N is a power of two, as at
    128^3 = 2^21 particles; its per-query candidate count is measured here on the
    same state and reported beside the time, so the reference's own searcher would
    be far slower than this baseline."""
    from oracle import oracle as orc
    from swc import scenes

    orc.build()
    threads = os.cpu_count() or 1
    orc.set_threads(threads)
    s = scenes.projection_block_3d(n=args.n, seed=args.seed)
    o = orc.Oracle(s, searcher="cells")
    t0 = time.perf_counter()
    o.initialize()
    t_init = time.perf_counter() - t0
    for _ in range(warmup):
        o.advance(s.dt)
    times, iters = [], []
    while len(times) < max(steps, 1):
        t0 = time.perf_counter()
        o.advance(s.dt)
        times.append(time.perf_counter() - t0)
        iters.append(o.stats()["iterations"])
        if time_cap is not None and sum(times) > time_cap:
            break
    sec = float(np.mean(times))
    # per-query candidates of the reference's hash grid against the cell grid's
    # 27 cells, on a sample of particle positions of the current state
    x, _ = o.particles()
    q = x[:: max(1, len(x) // 20000)]
    hash_cand = o.hash_candidates("real", q)
    out = {"value": 1.0 / sec, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"the full {args.n}^3 = {s.n_particles} particle block ({s.n_boundary} boundary): "
                     f"{warmup} untimed + {len(times)} timed advance steps (not extrapolated), "
                     f"{np.mean(iters):.1f} CG iterations per step",
           "steps": len(times), "seconds_per_step": sec, "initialize_seconds": t_init,
           "reference_searcher": {
               "real_candidates_per_query": hash_cand,
               "note": "the reference's HashGridSearcher (2N buckets, OR-combined key) visits this many "
                       "candidates per query at this size; the timed port visits the 27 cells of h "
                       f"(about 216 candidates) and finds the same neighbours, so the reference's own code "
                       f"would run slower than this baseline"}}
    if policy:
        # the reference demos' own thread count, max(procs / 3, 1)
        # (Demos/SmthPartHydrodLiquidTest/SmthPartHydrodLiquidTest.cpp:28), one step
        t3 = max(threads // 3, 1)
        orc.set_threads(t3)
        t0 = time.perf_counter()
        o.advance(s.dt)
        d3 = time.perf_counter() - t0
        orc.set_threads(threads)
        out["reference_thread_policy"] = {"threads": t3, "value": 1.0 / d3, "unit": UNIT, "steps": 1}
    return out


def run_reference_arm(args):
    dist, rank, ws = dist_setup()
    if rank != 0:
        return
    # each oracle step at 2M particles is seconds of CPU work: one untimed step and
    # at most args.steps timed ones within about a minute; `steps` reports the
    # number actually timed
    cb = cpu_reference(args, steps=args.steps, warmup=min(args.warmup, 1), time_cap=60.0)
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": cb["steps"], "warmup": min(args.warmup, 1), "ms_per_step": 1e3 / cb["value"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "config": workload_config(args),
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "reference_searcher": cb["reference_searcher"],
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# DEM sand leg: DEMParticleSandBuilder's layout (packed block of half-length 1/8 in the
# container [-1/2, 1/2]^3) at scale 225, r = 1/900: 2,009,840 particles, the block
# squeezed by 1e-4 (every touching pair overlaps by 2e-4 r) and set down in the
# container's corner on the floor, N(0, 0.01^2) velocities, walls 8r deep,
# dt = 1e-4 (the demo's frame rate 10000).
SAND_SCALE = 225
SAND_METRIC = "DEM sand advance steps/s at 2,009,840 particles"


def sand_scene(scale=SAND_SCALE, seed=0):
    from swc import scenes

    r = 1.0 / (4 * scale)
    return scenes.sand_contact_block(3, scale=scale, seed=seed, squeeze=0.9999, jitter=0.0, sigma=0.01,
                                     wall_depth=8 * r)


def sand_cpu_reference(scale=120, steps=5):
    """The DEM step's CPU restatement (oracle, all host threads) on the same layout at a
    smaller scale; steps/s scaled by the particle count to the benchmark's."""
    from oracle import oracle as orc

    orc.build()
    threads = os.cpu_count() or 1
    orc.set_threads(threads)
    s = sand_scene(scale)
    o = orc.DemOracle(3, s.radius, s.mass)
    o.set_particles(s.positions, s.velocities)
    o.set_boundary(s.boundary_positions, s.boundary_normals)
    o.initialize()
    o.advance(s.dt)
    t0 = time.perf_counter()
    for _ in range(steps):
        o.advance(s.dt)
    dt = time.perf_counter() - t0
    n_full = 2009840
    sps = steps / dt
    return {"value": sps * s.n_particles / n_full, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} advance steps at scale {scale} ({s.n_particles} particles, {sps:.3f} steps/s), "
                      f"scaled by {s.n_particles}/{n_full} particles"}


def run_sand_leg(args, torch, stream, hbm, peak_kind, with_cpu):
    """Device-resident steps/s, e2e through the public C ABI with pinned host FP64
    buffers, the contact pass against the HBM roof, and the CPU port beside it."""
    from swc import _lib
    from swc.sand import DEMParticleSand

    s = sand_scene(args.sand_scale)
    n = s.n_particles
    g = DEMParticleSand.from_scene(s)
    g.setStream(stream.cuda_stream)
    g.initialize()
    for _ in range(args.warmup):
        g.advance(s.dt)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        g.advance(s.dt)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    kern = {"contacts": g.timeKernel(0, 20), "binning": g.timeKernel(1, 20)}
    # algorithmic bytes: the contact pass reads pos, pos_lo, vel and writes vel (16 B each);
    # the binning moves them (48 B in, 32 B out), writes key / rank, scatters, permutes
    # pos, pos_lo, vel, id (52 B in and out)
    alg = {"contacts": 64 * n, "binning": (48 + 32 + 8) * n + (8 + 4) * n + (4 + 52 + 52) * n}
    dom = max(kern, key=kern.get)
    ach = alg[dom] / (kern[dom] / 1e3) / 1e9
    roof = {"kernel": dom, "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
            "peak_source": peak_kind, "traffic": None, "per_kernel_ms": kern,
            "per_kernel_GBps": {k: alg[k] / (kern[k] / 1e3) / 1e9 for k in kern}}
    # e2e: host FP64 state in, one advance, host FP64 state out, every step
    L = _lib.load()
    nbytes = n * 3 * 8
    hx_p, hv_p = L.swc_host_alloc(nbytes), L.swc_host_alloc(nbytes)
    hx = np.frombuffer((C.c_double * (n * 3)).from_address(hx_p), dtype=np.float64).reshape(n, 3)
    hv = np.frombuffer((C.c_double * (n * 3)).from_address(hv_p), dtype=np.float64).reshape(n, 3)
    x0, v0 = g.getParticles()
    hx[:], hv[:] = x0, v0
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))

    def e2e_step():
        rc = L.swc_sand_set_particles(g.h, dp(hx), dp(hv), n)
        rc |= L.swc_sand_advance(g.h, s.dt)
        rc |= L.swc_sand_get_particles(g.h, dp(hx), dp(hv), n)
        if rc:
            raise RuntimeError("sand e2e step failed")

    for _ in range(args.warmup):
        e2e_step()
    torch.cuda.synchronize()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    f1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = f0.elapsed_time(f1)
    L.swc_host_free(hx_p)
    L.swc_host_free(hv_p)
    g.close()
    out = {"metric": SAND_METRIC if n == 2009840 else f"DEM sand advance steps/s at {n} particles", "value": args.steps / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / args.steps,
           "steps": args.steps, "warmup": args.warmup, "dtype": "f32 (float-float positions)",
           "config": {"workload": f"DEM sand block (DEMParticleSandBuilder layout, scale {args.sand_scale}, "
                                  f"r = 1/{4 * args.sand_scale}): "
                                  f"{n} particles squeezed by 1e-4 on the container floor, {s.n_boundary} wall "
                                  f"particles 8r deep, dt 1e-4", "particles": n, "boundary": s.n_boundary,
                      "l2": "inputs larger than L2 (particle state 128 MB + sort scratch per step)"},
           "e2e": {"value": args.steps / (e2e_ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": 2 * nbytes,
                   "d2h_bytes_per_step": 2 * nbytes},
           "roofline": roof, "gpu_launches_per_step": 10}
    if with_cpu:
        out["cpu_baseline"] = sand_cpu_reference()
    return out


def host_link(torch, stream, nbytes, reps=10):
    """The host link's own copy rate (pinned host <-> device, one direction at a
    time, CUDA events) for the e2e step's byte count, and the time its copies
    take at that rate."""
    h = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    out = {}
    for name, (dst, src) in (("h2d", (d, h)), ("d2h", (h, d))):
        with torch.cuda.stream(stream):
            dst.copy_(src, non_blocking=True)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                dst.copy_(src, non_blocking=True)
            e1.record(stream)
        torch.cuda.synchronize()
        out[f"{name}_GBps"] = nbytes * reps / (e0.elapsed_time(e1) / 1e3) / 1e9
    out["copy_ms_at_link_rate"] = 1e3 * nbytes * (1 / out["h2d_GBps"] + 1 / out["d2h_GBps"]) / 1e9
    del h, d
    return out


def run_training_leg(args, torch, epochs=5):
    """The learned warm start's training path on the tensor cores: the loss-gradient
    pass alone (rows of seeded synthetic features, CUDA events) and Adam epochs
    through the trainer (wall clock, the dataset resident on the device)."""
    from swc import learn

    rng = np.random.default_rng(0)

    def data(n):
        f = rng.normal(size=(n, learn.N_IN)).astype(np.float32)
        return f, (np.tanh(f[:, 0]) + 0.5 * f[:, 4]).astype(np.float32)

    f, t = data(args.train_rows)
    norm = learn.normalisation(f, t)
    p = learn.init_params(1)
    for _ in range(3):
        g, loss = learn.gradient(p, norm, f, t)  # host arrays in and out (allocating helper)
    out = {"gradient_rows": args.train_rows, "loss": float(loss)}
    if epochs:
        # the trainer's epochs over a device-resident dataset (the dataset upload and
        # the trainer's set-up are timed apart)
        F, T = data(1 << 21)
        t0 = time.perf_counter()
        tr = learn.Trainer(F.shape[0], 16384)
        tr.add(F, T)
        tr.set_params(learn.init_params(0), learn.normalisation(F, T))
        tr.fit(1, 1e-3, 0)  # first use of the kernels
        t1 = time.perf_counter()
        ep_loss = tr.fit(epochs, 1e-3, 1)
        t2 = time.perf_counter()
        tr.close()
        out.update({"train_rows": F.shape[0], "epochs": epochs, "batch": 16384, "seconds": t2 - t1,
                    "setup_seconds": t1 - t0, "rows_per_s": epochs * F.shape[0] / (t2 - t1),
                    "epoch_loss": [float(x) for x in ep_loss],
                    "note": "per batch: device shuffle gather, fused tcgen05 gradient pass (BF16 operands, FP32 "
                            "accumulation), Adam; the epoch loss over the whole dataset on the device"})
    return out


def workload_config(args):
    return {"workload": f"isolated projection block {args.n}^3 = {args.n**3} fluid particles, "
                        f"{(args.n + 4)**3 - args.n**3} boundary, spacing 0.01, dt 5e-4, tol 1e-5",
            "particles": args.n**3, "steps_per_replica": args.steps, "warm_start": args.warm_start,
            "l2": "inputs larger than L2 (particle + node state > 129 MB per step)",
            "parallelism": f"replicas x{args.gpus}"}


def run_gpu_arm(args):
    import torch

    import swc
    from swc import _lib, learn, scenes

    dist, rank, ws = dist_setup()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    scene = scenes.projection_block_3d(n=args.n, seed=args.seed + rank)
    stream = torch.cuda.Stream()

    def make(warm):
        no_fallback = warm == "learned_no_fallback"
        mode = "learned" if warm.startswith("learned") else warm
        gate = LEARNED_GATE if warm == "learned" else 0
        liq = swc.DualParticleSphLiquid(scene, warm_start=mode, tolerance=1e-5, learned_no_fallback=no_fallback,
                                        learned_gate=gate)
        if mode == "learned":
            liq.setMlp(*learn.load_model(MODEL))
        liq.setStream(stream.cuda_stream)
        liq.initialize()
        return liq

    liq = make(args.warm_start)
    for _ in range(args.warmup):
        liq.advance(scene.dt)
    torch.cuda.synchronize()
    barrier(dist)
    iters = []
    with ClockSampler(dev) as clk:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0.record(stream)
        for _ in range(args.steps):
            st = liq.advance(scene.dt)
            iters.append(st["cg_iterations"])
            if st["status"] != 0:
                raise RuntimeError(f"step failed: {st}")
        e1.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    barrier(dist)
    ms = e0.elapsed_time(e1)
    ms_max = reduce_max(dist, ms)
    value = replica_value(ws, args.steps, ms_max)
    nv = st["n_virtual"]
    if args.profile_run:
        # minimal run for profiler captures: the timed steps only
        if rank == 0:
            print(json.dumps({"profile_run": True, "steps": args.steps, "ms_per_step": ms_max / args.steps,
                              "cg_iterations_mean": float(np.mean(iters)), "n_virtual": nv}), flush=True)
        liq.close()
        return

    # per-phase device time of one step (profiling events)
    liq.setProfiling(True)
    liq.advance(scene.dt)
    phases = liq.phaseTimes()
    liq.setProfiling(False)

    # dominant kernels timed live (CUDA events on the library stream)
    hbm, peak_kind = peaks()
    kern = {}
    for which, name in ((6, "cg_direction"), (0, "cg_spmv"), (1, "cg_update"), (2, "virtual_gather"),
                        (3, "pressure_gradient"), (4, "density"), (5, "forces")):
        kern[name] = liq.timeKernel(which, 20)
    if args.warm_start.startswith("learned"):
        kern["mlp_forward"] = liq.timeKernel(7, 20)
    n, nb = scene.n_particles, scene.n_boundary
    # algorithmic bytes per launch (each array touched once per pass)
    alg = {
        "cg_direction": 20 * nv,  # reads d, r, V; writes d, u = V d
        "cg_spmv": 16 * nv,  # reads u (halo tiles from L2), d, alpha_hat; writes q (FP32)
        "cg_update": 24 * nv,  # reads x, r, d, q; writes x, r
        "virtual_gather": 32 * (n + nb) + 16 * nv,  # particle pos/vel once; V, D, rho, flag out
        "pressure_gradient": 32 * n + 8 * nv + 48 * nb,  # pos, vel r/w; V, p; boundary pos/vel/nrm
        "density": 16 * n + 4 * n + 4 * n,
        "forces": 32 * n + 16 * n,
        "mlp_forward": 32 * nv,  # per slot: flag, D, alpha_hat, n_real, p_base, p1, d2, rho read; p0 written
    }
    cg_ms = kern["cg_direction"] + kern["cg_spmv"] + kern["cg_update"]
    dominant = max(("cg_spmv", "virtual_gather", "pressure_gradient"),
                   key=lambda k: kern[k] * (np.mean(iters) if k == "cg_spmv" else 1))
    ach = alg[dominant] / (kern[dominant] / 1e3) / 1e9
    # DRAM bytes (read + write) per active node of one launch, from the ncu captures of
    # the same workload summarised in profiles/
    traffic = DRAM_BYTES_PER_NODE[dominant] * nv if dominant in DRAM_BYTES_PER_NODE else None
    roofline = {"kernel": dominant, "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                "frac": ach / hbm, "peak_source": peak_kind, "traffic": traffic,
                "per_kernel_ms": kern, "per_kernel_GBps": {k: alg[k] / (kern[k] / 1e3) / 1e9 for k in kern},
                "cg_iteration_ms": cg_ms}
    if dominant == "pressure_gradient":
        # the gradient is bound by instruction issue, not HBM: its arithmetic against the
        # FP32 roof (nominal: SMs x 128 lanes x 2 x max clock).  Per particle, the
        # 268 lattice nodes within H = 4 spacings (4/3 pi 4^3) at 22 FLOP each: r^2 (5),
        # 1/r (1), r (1), a = 1 - r/4 (2), b = max(a - 1/2, 0) (2), a^2 - 4 b^2 (3),
        # w = (a^2 - 4 b^2) u / r (2), the three components w d (6)
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        fp32_peak = sms * 128 * 2 * SM_MAX_MHZ * 1e6 / 1e12
        flops = 268 * 22 * n
        roofline["fp32"] = {"achieved": flops / (kern["pressure_gradient"] / 1e3) / 1e12, "peak": fp32_peak,
                            "unit": "TFLOP/s", "peak_source": "nominal",
                            "frac": flops / (kern["pressure_gradient"] / 1e3) / 1e12 / fp32_peak}
    if dominant == "cg_spmv":
        # the stencil's arithmetic against the FP32 FMA roof (nominal: SMs x 128 lanes x 2 x max clock)
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        fp32_peak = sms * 128 * 2 * SM_MAX_MHZ * 1e6 / 1e12
        flops = 2 * 250 * nv  # 250 off-diagonal taps per active row (the reference's per-row work)
        roofline["fp32"] = {"achieved": flops / (kern["cg_spmv"] / 1e3) / 1e12, "peak": fp32_peak,
                            "unit": "TFLOP/s", "peak_source": "nominal"}

    # end-to-end through the public API with pinned host buffers, on a fresh
    # context over the same steps as the device-resident measurement (the state
    # evolves, so later steps are a different workload)
    L = _lib.load()
    dim = 3
    nbytes = n * dim * 8
    hx_p = L.swc_host_alloc(nbytes)
    hv_p = L.swc_host_alloc(nbytes)
    hx = np.frombuffer((C.c_double * (n * dim)).from_address(hx_p), dtype=np.float64).reshape(n, dim)
    hv = np.frombuffer((C.c_double * (n * dim)).from_address(hv_p), dtype=np.float64).reshape(n, dim)
    le = make(args.warm_start)
    x0, v0 = le.getParticles()
    hx[:] = x0
    hv[:] = v0
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    stt = _lib.Stats()

    def e2e_step():
        rc = L.swc_set_particles(le.h, dp(hx), dp(hv), n)
        rc |= L.swc_advance(le.h, scene.dt, C.byref(stt))
        rc |= L.swc_get_particles(le.h, dp(hx), dp(hv), n)
        if rc:
            raise RuntimeError("e2e step failed")

    for _ in range(args.warmup):
        e2e_step()
    torch.cuda.synchronize()
    barrier(dist)
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    f1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = reduce_max(dist, f0.elapsed_time(f1))
    e2e = {"value": ws * args.steps / (e2e_ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": 2 * nbytes,
           "d2h_bytes_per_step": 2 * nbytes, "host_link": host_link(torch, stream, 2 * nbytes)}
    e2e["host_link"]["copy_share_of_e2e_step"] = e2e["host_link"]["copy_ms_at_link_rate"] / (e2e_ms / args.steps)
    le.close()
    L.swc_host_free(hx_p)
    L.swc_host_free(hv_p)

    # plain-CG comparison forms (same scene, same steps)
    forms = {}
    if args.compare_forms:
        cands = ["prefix", "node", "zero", "extrapolate"] + (["learned", "learned_always", "learned_no_fallback"]
                                                             if os.path.exists(MODEL) else [])
        for warm in cands:
            if warm == args.warm_start:
                continue
            l2 = make(warm)
            for _ in range(args.warmup):
                l2.advance(scene.dt)
            torch.cuda.synchronize()
            g0 = torch.cuda.Event(enable_timing=True)
            g1 = torch.cuda.Event(enable_timing=True)
            its = []
            g0.record(stream)
            for _ in range(args.steps):
                its.append(l2.advance(scene.dt)["cg_iterations"])
            g1.record(stream)
            torch.cuda.synchronize()
            forms[warm] = {"steps_per_s": args.steps / (g0.elapsed_time(g1) / 1e3),
                           "cg_iterations_mean": float(np.mean(its))}
            l2.close()

    # Whole-step HBM roofline per warm-start form, on the algorithmic bytes of one
    # step (each array once per pass; FP32 state): binning 92 N, rho_i 20 N,
    # viscosity + gravity 48 N, node activation 12 per lattice node, the fused
    # gather 36 (N + N_b) + 16 N_v, alpha_hat 8 N_v, CG 52 N_v per iteration
    # (SpMV + dot 16, x/r update 24, direction 12), the pressure gradient
    # 48 N + 8 N_v + 36 N_b.  The network's 28 N_v on the steps it runs is left out.
    def step_bytes(cg_its):
        return (92 + 20 + 48 + 48) * n + 12 * scene.n_nodes + 36 * (n + nb) + (16 + 8 + 8) * nv + 36 * nb + \
            52 * nv * cg_its
    step_roof = {"bytes_model": "92N + 20N + 48N + 12 N_nodes + 36(N+N_b) + 16N_v + 8N_v + 52 N_v x iterations "
                                "+ 48N + 8N_v + 36N_b (FP32 state, each array once per pass)",
                 "n_nodes": scene.n_nodes}
    for form, sps, its in [(args.warm_start, value / ws, float(np.mean(iters)))] + \
            [(k, v["steps_per_s"], v["cg_iterations_mean"]) for k, v in forms.items()]:
        b = step_bytes(its)
        step_roof[form] = {"bytes_per_step": b, "GBps": b * sps / 1e9, "frac": b * sps / 1e9 / hbm,
                           "cg_iterations_mean": its}
    roofline["step"] = step_roof

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu = cpu_reference(args, steps=args.cpu_steps, warmup=1, policy=True)
    training = run_training_leg(args, torch) if args.training else None
    sand = None
    if args.sand:
        sand = run_sand_leg(args, torch, stream, hbm, peak_kind, with_cpu=rank == 0 and ws == 1 and not args.no_cpu)

    # kernels launched per step (counted in the ncu launch list of this workload):
    # binning 7 (count, three scan passes, scatter, segment sort, permute), density 2,
    # viscosity 2, virtual generation 8 (brick marking, two brick lists, gather, segment
    # count and its three scan passes), alpha_hat 1, warm start 1, CG start 3, 3 per CG
    # iteration, gradient 1; a step that evaluates the network adds 4 more (not counted
    # here, so this is a lower bound)
    launches_per_step = 25 + 3 * float(np.mean(iters))
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FP64 CG reductions)",
                "data": "synthetic (seeded)", "config": workload_config(args),
                "wall_s_timed": wall, "cg_iterations_mean": float(np.mean(iters)), "n_virtual": nv,
                "phases_ms": phases, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
                "clocks": clk.summary(), "gpu_launches": int(round(launches_per_step * args.steps)),
                "forms": forms, "sand": sand, "training": training}
        print(json.dumps(line), flush=True)
    liq.close()
    if dist is not None:
        dist.destroy_process_group()


def run_scene_leg(args):
    """Throughput of the other configurations (wall time of the device steps on the
    library's stream, CUDA events) for the node-mapped, extrapolated and learned
    warm starts, after one untimed step, with one profiled step's phase split."""
    import torch

    import swc
    from swc import learn, scenes

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    build = {"dam_break_2d": scenes.dam_break_2d, "dam_break_3d": scenes.dam_break_3d,
             "paddle_tank": scenes.paddle_tank_3d}[args.scene]
    scene = build(seed=args.seed)
    stream = torch.cuda.Stream()
    forms = {}
    for warm in ("node", "extrapolate", "learned"):
        liq = swc.DualParticleSphLiquid(scene, warm_start=warm, tolerance=scene.tolerance,
                                        learned_gate=LEARNED_GATE if warm == "learned" else 0)
        if warm == "learned":
            liq.setMlp(*learn.load_model(MODEL))
        liq.setStream(stream.cuda_stream)
        liq.initialize()
        liq.advance(scene.dt)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        its = []
        e0.record(stream)
        for _ in range(args.steps):
            st = liq.advance(scene.dt)
            if st["status"] not in (0, 1):
                raise RuntimeError(f"step failed: {st}")
            its.append(st["cg_iterations"])
        e1.record(stream)
        torch.cuda.synchronize()
        liq.setProfiling(True)
        liq.advance(scene.dt)
        phases = liq.phaseTimes()
        liq.setProfiling(False)
        forms[warm] = {"steps_per_s": args.steps / (e0.elapsed_time(e1) / 1e3),
                       "cg_iterations_mean": float(np.mean(its)), "n_virtual": st["n_virtual"],
                       "phases_ms": phases}
        liq.close()
    return {"scene": scene.name, "particles": scene.n_particles, "boundary": scene.n_boundary,
            "steps": args.steps, "dt": scene.dt, "tolerance": scene.tolerance, "forms": forms}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # the benchmark configuration: 50 repetitions of advect + projection (the
    # state evolves, so the step count is part of the workload)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="swc", choices=["swc", "reference"])
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--warm-start", dest="warm_start", default="auto",
                    choices=["auto", "prefix", "node", "zero", "extrapolate", "learned", "learned_always",
                             "learned_no_fallback"],
                    help="auto: the learned start (residual test, gated) when the trained model is present, "
                         "else the node-mapped previous pressure")
    ap.add_argument("--cpu-steps", dest="cpu_steps", type=int, default=2,
                    help="timed oracle steps of the CPU baseline (full-size block, after one untimed step)")
    ap.add_argument("--no-cpu", dest="no_cpu", action="store_true")
    ap.add_argument("--compare-forms", dest="compare_forms", type=int, default=1)
    ap.add_argument("--sand", type=int, default=1, help="also measure the DEM sand step (the 'sand' object)")
    ap.add_argument("--sand-scale", dest="sand_scale", type=int, default=SAND_SCALE,
                    help="builder scale of the sand block (225: 2,009,840 particles)")
    ap.add_argument("--sand-only", dest="sand_only", action="store_true",
                    help="only the DEM sand leg (for profiler captures); prints the sand object")
    ap.add_argument("--profile-run", dest="profile_run", action="store_true",
                    help="only the timed steps (for profiler captures); prints a reduced line")
    ap.add_argument("--training", type=int, default=1, help="also time the learned warm start's training path")
    ap.add_argument("--train-rows", dest="train_rows", type=int, default=65536,
                    help="rows of the timed loss-gradient pass")
    ap.add_argument("--scene", default="block", choices=["block", "dam_break_2d", "dam_break_3d", "paddle_tank"],
                    help="block: the benchmark; the others print the throughput of that configuration "
                         "(2D dam break, 3,200 particles; 3D dam break, 524,288 particles; paddle tank, "
                         "8,388,608 particles with a rotating paddle)")
    ap.add_argument("--train-only", dest="train_only", action="store_true",
                    help="only the loss-gradient pass on --train-rows rows (for profiler captures)")
    args = ap.parse_args()
    if args.warm_start == "auto":
        args.warm_start = "learned" if os.path.exists(MODEL) else "node"
    if args.impl == "reference":
        run_reference_arm(args)
    elif args.scene != "block":
        print(json.dumps(run_scene_leg(args)), flush=True)
    elif args.train_only:
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        print(json.dumps(run_training_leg(args, torch, epochs=0)), flush=True)
    elif args.sand_only:
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        hbm, peak_kind = peaks()
        print(json.dumps(run_sand_leg(args, torch, torch.cuda.Stream(), hbm, peak_kind, with_cpu=not args.no_cpu)),
              flush=True)
    else:
        run_gpu_arm(args)


if __name__ == "__main__":
    main()
