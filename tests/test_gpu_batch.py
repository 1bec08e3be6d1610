"""GPU tests of the batched cluster solver: every system of a batch against
the single-system path and the oracle, and bitwise equality of a system's
result alone and in a mix of other systems."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import SOL_REL, iter_ok, oracle_solve, rel_l2, system
from tflows import TFS_BICG, TFS_CG, TFS_FP64, TFS_MIXED, Batch, Solver
from tflows.synth import CONVDIFF, POISSON

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def systems(gpu):
    specs = [(POISSON, 9, 8, 7, 1), (POISSON, 14, 12, 11, 2), (CONVDIFF, 10, 9, 9, 3),
             (POISSON, 5, 4, 3, 4), (POISSON, 20, 18, 17, 5), (CONVDIFF, 7, 7, 6, 6)]
    out = []
    for kind, nx, ny, nz, seed in specs:
        s = system(kind, nx, ny, nz, seed=seed)
        out.append((s, Solver(s.matrix())))
    return out


def _run(batch, sys_list, method, prec, mode):
    xs = [np.zeros(s.n) for s, _ in sys_list]
    rs = [s.b.copy() for s, _ in sys_list]
    tols = [1e-8 * np.linalg.norm(s.b) for s, _ in sys_list]
    res = batch.solve(method, prec, [s.val for s, _ in sys_list], xs, rs, 2000, tols, mode=mode)
    return xs, rs, res


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("method", [TFS_CG, TFS_BICG])
def test_batch_fp64_matches_oracle(method, prec, systems):
    sel = [t for t in systems if method == TFS_BICG or t[0].kind == POISSON]
    with Batch([sv for _, sv in sel], cluster=4, threads=256) as b:
        xs, rs, res = _run(b, sel, method, prec, TFS_FP64)
    for k, (s, _) in enumerate(sel):
        ref = oracle_solve(s, method, prec)
        assert res.status[k] == 0
        assert iter_ok(int(res.niter[k]), ref["niter"]), (k, res.niter[k], ref["niter"])
        assert rel_l2(xs[k], ref["x"]) <= SOL_REL
        assert res.ini_res[k] == pytest.approx(ref["ini"], rel=1e-13)


@pytest.mark.parametrize("method", [TFS_CG, TFS_BICG])
def test_batch_mixed_converges(method, systems):
    # The convection-diffusion systems are excluded: the reference's BiCG
    # (= CG, see the BiCG test of test_gpu_parity) does not converge on them
    # even in binary64, so there is no tolerance to reach.
    sel = [t for t in systems if t[0].kind == POISSON]
    with Batch([sv for _, sv in sel], cluster=8, threads=256) as b:
        xs, rs, res = _run(b, sel, method, 1, TFS_MIXED)
    from oracle import tfs_oracle as O
    for k, (s, _) in enumerate(sel):
        tol = 1e-8 * np.linalg.norm(s.b)
        assert res.status[k] == 0 and res.fin_res[k] < tol
        rt = s.b.copy()
        O.residual(s.n, s.row, s.col, s.val, xs[k], rt)
        assert np.linalg.norm(rt) < tol
        ref = oracle_solve(s, method, 1)
        assert rel_l2(xs[k], ref["x"]) < 1e-6


@pytest.mark.parametrize("mode", [TFS_FP64, TFS_MIXED])
def test_batch_alone_equals_in_mix(mode, systems):
    """A system's result does not depend on the rest of the batch (bitwise)."""
    sel = [t for t in systems if t[0].kind == POISSON]
    target = sel[1]
    with Batch([target[1]], cluster=4, threads=256) as b:
        xa, ra, resa = _run(b, [target], TFS_CG, 1, mode)
    with Batch([sv for _, sv in sel], cluster=4, threads=256) as b:
        xm, rm, resm = _run(b, sel, TFS_CG, 1, mode)
    k = 1
    assert np.array_equal(xa[0], xm[k]) and np.array_equal(ra[0], rm[k])
    assert resa.niter[0] == resm.niter[k] and resa.fin_res[0] == resm.fin_res[k]


@pytest.mark.parametrize("cluster,threads", [(1, 128), (2, 512), (16, 256)])
def test_batch_cluster_shapes(cluster, threads, systems):
    sel = [t for t in systems if t[0].kind == POISSON]
    with Batch([sv for _, sv in sel], cluster=cluster, threads=threads) as b:
        xs, rs, res = _run(b, sel, TFS_CG, 1, TFS_FP64)
    for k, (s, _) in enumerate(sel):
        ref = oracle_solve(s, TFS_CG, 1)
        assert iter_ok(int(res.niter[k]), ref["niter"]) and rel_l2(xs[k], ref["x"]) <= SOL_REL


def test_batch_semantics_small_b_and_limit(systems):
    sel = [t for t in systems if t[0].kind == POISSON][:2]
    with Batch([sv for _, sv in sel], cluster=2, threads=128) as b:
        xs = [np.ones(s.n) for s, _ in sel]
        rs = [s.b * 1e-12 for s, _ in sel]
        res = b.solve(TFS_CG, 1, [s.val for s, _ in sel], xs, rs, 100, [1.0, 1.0], ini_res=-5.0)
        assert list(res.niter) == [0, 0] and list(res.ini_res) == [-5.0, -5.0]
        assert all(np.array_equal(x, np.ones(x.size)) for x in xs)
        xs = [np.zeros(s.n) for s, _ in sel]
        rs = [s.b.copy() for s, _ in sel]
        res = b.solve(TFS_CG, 1, [s.val for s, _ in sel], xs, rs, 5, [1e-30, 1e-30])
        assert list(res.niter) == [6, 6]


@pytest.mark.parametrize("method", [TFS_CG, TFS_BICG])
def test_batch_dic_matches_oracle(method, systems):
    """DIC in the batch (the factor and both triangular sweeps level by level
    inside each system's cluster): binary64 within the parity gates of the
    oracle's DIC solve (BiCG is the CG sequence), mixed precision converged
    on the binary64 true residual within 1e-6 of the oracle."""
    from helpers import iter_ok_mixed
    sel = [t for t in systems if t[0].kind == POISSON]
    for mode in (TFS_FP64, TFS_MIXED):
        with Batch([sv for _, sv in sel], cluster=4, threads=256) as b:
            xs, rs, res = _run(b, sel, method, 2, mode)
        for k, (s, _) in enumerate(sel):
            ref = oracle_solve(s, method, 2)
            assert res.status[k] == 0
            if mode == TFS_FP64:
                assert iter_ok(int(res.niter[k]), ref["niter"]), (k, res.niter[k], ref["niter"])
                assert rel_l2(xs[k], ref["x"]) <= SOL_REL
                assert res.ini_res[k] == pytest.approx(ref["ini"], rel=1e-13)
            else:
                assert iter_ok_mixed(int(res.niter[k]), ref["niter"]), (k, res.niter[k], ref["niter"])
                assert res.fin_res[k] < 1e-8 * np.linalg.norm(s.b)
                assert rel_l2(xs[k], ref["x"]) < 1e-6


def test_batch_dic_alone_equals_in_mix(systems):
    """With DIC too a system's result does not depend on the rest of the
    batch (bitwise)."""
    sel = [t for t in systems if t[0].kind == POISSON]
    target = sel[2]
    with Batch([target[1]], cluster=8, threads=512) as b:
        xa, ra, resa = _run(b, [target], TFS_CG, 2, TFS_FP64)
    with Batch([sv for _, sv in sel], cluster=8, threads=512) as b:
        xm, rm, resm = _run(b, sel, TFS_CG, 2, TFS_FP64)
    assert np.array_equal(xa[0], xm[2]) and np.array_equal(ra[0], rm[2])
    assert resa.niter[0] == resm.niter[2]


def test_batch_literal_bicg_refuses_dic(systems):
    from tflows.lib import TFS_OPT_BICG, TfsError
    s, _ = systems[0]
    with Solver(s.matrix(), options={TFS_OPT_BICG: 1}) as sv:
        with Batch([sv], cluster=2, threads=128) as b:
            with pytest.raises(TfsError):
                b.solve(TFS_BICG, 2, [s.val], [np.zeros(s.n)], [s.b.copy()], 100, [1e-8])
