"""CPU: bench.py's multi-rank plumbing with two gloo ranks on 127.0.0.1.

Under torchrun every rank steps its own realization (replicas: no collective
on the data path); the ranks meet only in a barrier around the timed region
and in two scalar reductions: the maximum of the per-rank times and the sum
of the per-rank m*t, whose quotient is the whole-job value."""
import importlib.util
import multiprocessing as mp
import os
import socket
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2",
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    spec = importlib.util.spec_from_file_location("bench_module", ROOT / "bench.py")
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    d = bench.Dist()
    d.barrier()
    ms = d.reduce(10.0 + rank, "max")      # per-rank timed region (ms)
    mt = d.reduce(0.5 * (rank + 1), "sum")  # per-rank m*t advanced
    d.barrier()
    d.close()
    q.put((rank, d.ws, ms, mt))


def test_two_gloo_ranks_reduce_time_and_work():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ws, ms, mt in out:
        assert ws == 2
        assert ms == 11.0 and mt == 1.5
    # the whole-job value bench.py prints: summed work over the slowest rank
    assert out[0][3] / (out[0][2] / 1e3) == pytest.approx(136.36, rel=1e-4)
