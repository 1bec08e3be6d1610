"""The multi-GPU path is replicas only: every rank solves its own seeded
systems, with no collective on the data path; ranks meet only for the timing
barrier and the max/sum of the per-rank numbers.  Tested with two gloo
processes on the CPU, each solving its own system (the oracle standing in
for the rank's GPU solver)."""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, out_dir: str) -> None:
    sys.path[:0] = [str(REPO), str(REPO / "t-flows_gb300")]
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import json
    import time

    import numpy as np

    import bench
    from oracle import tfs_oracle as O
    from tflows.synth import POISSON, SynthSystem
    d = bench.Dist()
    try:
        d.barrier()
        mx = d.max(float(rank + 1) * 10.0)
        sm = d.sum(float(rank + 1))
        specs = bench.batch_specs(8, bench.BASE_SEED + rank)
        # One replica step: this rank's own seeded system solved with no
        # exchange (the oracle stands in for the rank's solver on the CPU),
        # then the bench's aggregation: solves of all ranks over the slowest
        # rank's time.
        s = SynthSystem(POISSON, 10, 9, 8, jitter=0.2, seed=bench.BASE_SEED + rank)
        tol = 1e-8 * float(np.linalg.norm(s.b))
        x, r = np.zeros(s.n), s.b.copy()
        d.barrier()
        t = time.perf_counter()
        it, _, fin = O.solve(0, s.n, s.row, s.col, s.dia, s.val, x, r, 1, 2000, tol)
        dt = time.perf_counter() - t
        d.barrier()
        rt = s.b.copy()
        O.residual(s.n, s.row, s.col, s.val, x, rt)
        t_max = d.max(dt)
        solves = d.sum(1.0)
        with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
            json.dump({"max": mx, "sum": sm, "specs": specs, "it": it, "true_res": float(np.linalg.norm(rt)),
                       "tol": tol, "dt": dt, "t_max": t_max, "solves": solves, "x0": float(x[0])}, f)
    finally:
        d.close()


def test_two_replicas_gloo(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    mp.spawn(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    import json
    r0 = json.loads((tmp_path / "r0.json").read_text())
    r1 = json.loads((tmp_path / "r1.json").read_text())
    assert r0["max"] == r1["max"] == 20.0          # max over ranks of the step time
    assert r0["sum"] == r1["sum"] == 3.0           # whole-job count
    assert r0["specs"] != r1["specs"]              # each rank has its own systems
    seeds0 = {s[4] for s in r0["specs"]}
    seeds1 = {s[4] for s in r1["specs"]}
    assert not seeds0 & seeds1
    # each rank solved its own system to the tolerance ...
    for r in (r0, r1):
        assert r["it"] <= 2000 and r["true_res"] < r["tol"]
    assert r0["x0"] != r1["x0"]                     # different systems
    # ... and both agree on the whole-job throughput: every rank's solve over
    # the slowest rank's time
    assert r0["solves"] == r1["solves"] == 2.0
    assert r0["t_max"] == r1["t_max"] == max(r0["dt"], r1["dt"])
