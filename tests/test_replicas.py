"""The multi-GPU path is replicas only: every rank solves its own seeded
systems, with no collective on the data path; ranks meet only for the timing
barrier and the max/sum of the per-rank numbers.  Tested with two gloo
processes on the CPU."""
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

    import bench
    d = bench.Dist()
    try:
        d.barrier()
        mx = d.max(float(rank + 1) * 10.0)
        sm = d.sum(float(rank + 1))
        specs = bench.batch_specs(8, bench.BASE_SEED + rank)
        with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
            json.dump({"max": mx, "sum": sm, "specs": specs}, f)
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
