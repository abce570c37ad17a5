"""The bench's multi-process path on the CPU (gloo, world size 2, 127.0.0.1):
`python -m torch.distributed.run --nproc-per-node N bench.py` runs one independent
replica per rank (the projection does not shard), times each, takes the maximum
over the ranks and reports the steps of all replicas over that time; the reference
arm runs on rank 0 alone and the other ranks exit without work."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank),
                      LOCAL_RANK=str(rank), SWC_DIST_BACKEND="gloo")
    sys.path.insert(0, ROOT)
    import io
    import json
    from contextlib import redirect_stdout
    from types import SimpleNamespace

    import bench

    try:
        dist, r, ws = bench.dist_setup()
        assert dist is not None and r == rank and ws == 2 and dist.get_backend() == "gloo"
        ms = [120.0, 150.0][rank]  # the slower replica sets the time
        m = bench.reduce_max(dist, ms)
        bench.barrier(dist)
        dist.destroy_process_group()
        # the reference arm under the same launcher: rank 0 alone times the CPU
        # implementation (stubbed here: the full oracle step takes seconds) and prints
        bench.cpu_reference = lambda *a, **k: {"value": 0.3, "unit": "steps/s", "cores": 1, "kind": "port",
                                               "sample": "stub", "steps": 2, "reference_searcher": {}}
        args = SimpleNamespace(gpus=2, steps=2, warmup=1, n=8, warm_start="node", seed=0)
        buf = io.StringIO()
        with redirect_stdout(buf):
            bench.run_reference_arm(args)
        printed = buf.getvalue().strip()
        line = json.loads(printed) if printed else None
        q.put((rank, m, bench.replica_value(ws, 10, m), line, None))
    except Exception as e:  # reported to the parent
        q.put((rank, None, None, None, repr(e)))


def test_two_replicas_gloo():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=worker, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    for _ in range(2):
        rank, m, value, printed, err = q.get(timeout=120)
        out[rank] = (m, value, printed, err)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank in (0, 1):
        m, value, line, err = out[rank]
        assert err is None, err
        assert m == 150.0
        assert value == pytest.approx(2 * 10 / 0.150)
    assert out[0][2]["impl"] == "reference" and out[0][2]["value"] == 0.3
    assert out[1][2] is None
