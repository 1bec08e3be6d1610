"""GPU tests of the request loop: every result equals the same solve run
alone (bit for bit), eviction under a tight device-memory budget, refusal of
a system larger than the budget."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from helpers import SOL_REL, iter_ok, oracle_solve, rel_l2, system
from tflows import TFS_BICG, TFS_CG, TFS_CGS, TFS_FP64, TFS_MIXED, Server
from tflows.lib import TFS_ERR_BUDGET, check, load_library
from tflows.synth import CONVDIFF, POISSON

pytestmark = pytest.mark.gpu


class DevArrays:
    """Device copies of a system's val and b plus x, r1 work arrays."""

    def __init__(self, s):
        self.lib = load_library()
        self.s = s
        self.p = {}
        for name, nbytes in (("val", 8 * s.nnz), ("b", 8 * s.n), ("x", 8 * s.n), ("r", 8 * s.n)):
            q = C.c_void_p()
            check(self.lib.tfs_device_alloc(nbytes, C.byref(q)), "alloc")
            self.p[name] = q.value
        self._h2d("val", s.val)
        self._h2d("b", s.b)
        self.reset()

    def _rt(self):
        for name in ("libcudart.so.13", "libcudart.so"):
            try:
                rt = C.CDLL(name)
                rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
                return rt
            except OSError:
                pass
        raise RuntimeError("no libcudart")

    def _h2d(self, name, a):
        assert self._rt().cudaMemcpy(self.p[name], a.ctypes.data, a.nbytes, 1) == 0

    def reset(self, x0=None):
        self._h2d("x", np.zeros(self.s.n) if x0 is None else x0)
        self._h2d("r", self.s.b)

    def get(self, name):
        a = np.empty(self.s.n)
        assert self._rt().cudaMemcpy(a.ctypes.data, self.p[name], a.nbytes, 2) == 0
        return a

    def free(self):
        for q in self.p.values():
            self.lib.tfs_device_free(C.c_void_p(q))


@pytest.fixture(scope="module")
def pool(gpu):
    specs = [(POISSON, 16, 15, 14, 1), (CONVDIFF, 12, 12, 11, 2), (POISSON, 11, 10, 9, 3),
             (POISSON, 20, 18, 18, 4)]
    out = [(system(k, nx, ny, nz, seed=sd)) for k, nx, ny, nz, sd in specs]
    yield out


REQUESTS = [(0, TFS_CG, 1, TFS_FP64), (1, TFS_CGS, 1, TFS_MIXED), (2, TFS_CG, 2, TFS_MIXED),
            (3, TFS_BICG, 1, TFS_FP64), (0, TFS_CG, 2, TFS_MIXED), (2, TFS_CGS, 0, TFS_FP64),
            (3, TFS_CG, 1, TFS_MIXED), (1, TFS_CGS, 2, TFS_FP64)]


def _run(pool, requests, max_inflight, budget=1 << 34):
    arrs = [[DevArrays(pool[k]) for _ in range(2)] for k in range(len(pool))]
    used = {}
    out = []
    with Server(budget, max_inflight=max_inflight) as srv:
        ids = [srv.add_system(s.n, s.row, s.col, s.dia) for s in pool]
        tickets = []
        for j, (k, method, prec, mode) in enumerate(requests):
            # two concurrent requests of one system use different arrays
            slot = used.get(k, 0)
            used[k] = slot + 1
            a = arrs[k][slot % 2]
            s = pool[k]
            tol = 1e-8 * np.linalg.norm(s.b)
            tickets.append((srv.submit(ids[k], method, prec, a.p["val"], a.p["x"], a.p["r"], 2000,
                                       tol, mode), a))
        for t, a in tickets:
            res = srv.wait(t)
            out.append((res, a.get("x"), a.get("r")))
        stats = srv.stats()
    for row in arrs:
        for a in row:
            a.free()
    return out, stats


def test_results_alone_equal_results_in_the_mix(pool):
    """Each request gives bitwise the same result run alone (one at a time)
    and submitted together with the others (overlapping on the GPU)."""
    reqs = REQUESTS[:4]   # one request per system, so arrays are not reused
    alone = []
    for r in reqs:
        out, _ = _run(pool, [r], max_inflight=1)
        alone.append(out[0])
    mix, stats = _run(pool, reqs, max_inflight=8)
    for (ra, xa, rra), (rm, xm, rrm) in zip(alone, mix):
        assert ra["status"] == rm["status"] == 0
        assert ra["niter"] == rm["niter"] and ra["fin_res"] == rm["fin_res"]
        assert np.array_equal(xa, xm) and np.array_equal(rra, rrm)
    assert stats["completed"] == len(reqs)


def test_mixed_stream_of_requests_matches_oracle(pool):
    out, stats = _run(pool, REQUESTS, max_inflight=4)
    for (res, x, _), (k, method, prec, mode) in zip(out, REQUESTS):
        ref = oracle_solve(pool[k], method, prec)
        assert res["status"] == 0
        if mode == TFS_FP64:
            assert iter_ok(res["niter"], ref["niter"]) and rel_l2(x, ref["x"]) <= SOL_REL
        else:
            assert res["fin_res"] < ref["tol"] and rel_l2(x, ref["x"]) < 1e-6
        assert res["latency_ms"] >= res["run_ms"] >= 0.0
    assert stats["completed"] == len(REQUESTS)


def test_budget_eviction_and_refusal(pool):
    """A budget that holds one system at a time: requests alternate between
    systems and evict each other, results stay correct; a system larger than
    the whole budget is refused."""
    from tflows.lib import load_library
    lib = load_library()
    small = [pool[0], pool[3]]

    def est(s):   # tfs_estimate_bytes
        n_pad = (s.n + 1023) // 1024 * 1024 + 32 * 64
        return n_pad * 200 + s.n * 20 + s.nnz * 29 + (64 << 10)

    budget = int(1.15 * max(est(s) for s in small))
    assert est(small[0]) + est(small[1]) > budget
    reqs = [(0, TFS_CG, 1, TFS_FP64), (1, TFS_CG, 1, TFS_FP64), (0, TFS_CG, 2, TFS_FP64)]
    out, stats = _run(small, reqs, max_inflight=1, budget=budget)
    for (res, x, _), (k, method, prec, mode) in zip(out, reqs):
        ref = oracle_solve(small[k], method, prec)
        assert res["status"] == 0 and rel_l2(x, ref["x"]) <= SOL_REL
    assert stats["evictions"] >= 1
    out, stats = _run([pool[3]], [(0, TFS_CG, 1, TFS_FP64)], max_inflight=1, budget=1 << 20)
    assert out[0][0]["status"] == TFS_ERR_BUDGET and stats["refused"] == 1


def test_separate_b_and_zero_start(pool):
    """b read from its own array (kept intact), x started from zero whatever
    d_x holds, r1 written to d_r1."""
    s = pool[2]
    a = DevArrays(s)
    try:
        a.reset(x0=np.full(s.n, 7.0))
        with Server(1 << 34) as srv:
            sid = srv.add_system(s.n, s.row, s.col, s.dia)
            ref = oracle_solve(s, TFS_CG, 1)
            t = srv.submit(sid, TFS_CG, 1, a.p["val"], a.p["x"], a.p["r"], 2000, ref["tol"],
                           d_b=a.p["b"], x0_zero=True)
            res = srv.wait(t)
        assert res["status"] == 0 and iter_ok(res["niter"], ref["niter"])
        assert rel_l2(a.get("x"), ref["x"]) <= SOL_REL
        assert np.array_equal(a.get("b"), s.b)
    finally:
        a.free()


def test_continuous_batching_requests_overlap_on_the_device(gpu):
    """Requests that arrive while others are on the GPU are admitted at once
    and their solves overlap on the device: request k + 1 is submitted only
    after request k has been launched (the server reports it running), the
    server reports at least two solves running at once, and the device
    intervals of consecutive requests (the GPU's global timer at each
    solve's first kernel and at its epilogue) intersect.  Every result is
    bitwise the result of the same request run alone."""
    import time
    specs = [(POISSON, 40, 40, 40, 11), (POISSON, 36, 36, 36, 12), (POISSON, 44, 40, 38, 13),
             (POISSON, 38, 38, 38, 14)]
    pool = [system(k, nx, ny, nz, seed=sd) for k, nx, ny, nz, sd in specs]
    reqs = [(k, TFS_CG, 2, TFS_FP64 if k % 2 == 0 else TFS_MIXED) for k in range(len(pool))]
    alone = []
    for r in reqs:
        out, _ = _run(pool, [r], max_inflight=1)
        alone.append(out[0])
    arrs = [DevArrays(s) for s in pool]
    try:
        with Server(1 << 34, max_inflight=8) as srv:
            ids = [srv.add_system(s.n, s.row, s.col, s.dia) for s in pool]
            # resident systems and captured graphs first, so that admission is
            # a launch and not a layout build
            for k, (_, method, prec, mode) in enumerate(reqs):
                srv.wait(srv.submit(ids[k], method, prec, arrs[k].p["val"], arrs[k].p["x"], arrs[k].p["r"],
                                    2000, 1e-8 * np.linalg.norm(pool[k].b), mode))
                arrs[k].reset()
            tickets = []
            for k, (_, method, prec, mode) in enumerate(reqs):
                tickets.append(srv.submit(ids[k], method, prec, arrs[k].p["val"], arrs[k].p["x"],
                                          arrs[k].p["r"], 2000, 1e-8 * np.linalg.norm(pool[k].b), mode))
                if k + 1 < len(reqs):
                    t0 = time.perf_counter()
                    # the next request arrives once this one is on the GPU
                    while srv.stats()["running"] < 1 and time.perf_counter() - t0 < 5.0:
                        time.sleep(1e-5)
            results = [srv.wait(t) for t in tickets]
            stats = srv.stats()
        assert stats["peak_running"] >= 2, stats
        spans = [(r["device_begin_ns"], r["device_end_ns"]) for r in results]
        assert all(0 < b < e for b, e in spans), spans
        overlaps = sum(1 for (b0, e0), (b1, e1) in zip(spans, spans[1:]) if b1 < e0 and b0 < e1)
        assert overlaps >= 1, spans
        for k, res in enumerate(results):
            ra, xa, rra = alone[k]
            assert res["status"] == ra["status"] == 0
            assert res["niter"] == ra["niter"] and res["fin_res"] == ra["fin_res"]
            assert np.array_equal(arrs[k].get("x"), xa) and np.array_equal(arrs[k].get("r"), rra)
    finally:
        for a in arrs:
            a.free()


def test_wait_timeout_is_reported_and_the_ticket_survives(gpu):
    """A wait that runs out reports TFS_ERR_TIMEOUT (TimeoutError here) with
    the request still running; the same ticket can be waited for again and
    gives the solve's result.  The limit is the host's: no device wait is
    involved."""
    s = system(POISSON, 48, 48, 48, seed=21)
    a = DevArrays(s)
    try:
        with Server(1 << 34) as srv:
            sid = srv.add_system(s.n, s.row, s.col, s.dia)
            tol = 1e-8 * np.linalg.norm(s.b)
            t = srv.submit(sid, TFS_CG, 2, a.p["val"], a.p["x"], a.p["r"], 2000, tol)
            with pytest.raises(TimeoutError):
                srv.wait(t, timeout_s=0.0)
            res = srv.wait(t)
        assert res["status"] == 0 and res["fin_res"] < tol
    finally:
        a.free()
