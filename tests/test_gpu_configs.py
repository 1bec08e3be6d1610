"""GPU parity at the benchmark's own configurations, against the oracle.

The per-routine and small-system tests elsewhere pin the arithmetic; these
run the systems the benchmark measures, at full size, through the C ABI:

  config 0  32^3 jittered-hex pressure Poisson, diagonal CG, limit 2000
  config 1  128^3 of the same construction, DIC-CG (the default workload)
  config 2  160^3 upwind convection-diffusion, diagonal CGS (and a bounded
            run of the reference's BiCG, which does not converge on it)
  config 3  a seeded sample of 32 systems of the 256-system batch, every one
            against its own oracle solve

Gates (the hot-path contract): binary64 iteration count within +-2% of the
oracle's (never tighter than +-1) and solution relative L2 difference
<= 1e-9, at ||r|| < 1e-8 ||b|| from x0 = 0; mixed precision: binary64 true
residual below the tolerance, iterations from -2% to +25% of the binary64
oracle's (binary32 inner iterations lose orthogonality earlier: one system
of the batch sample takes 286 against 277), solution within 1e-6 of the
binary64 oracle.  The oracle solve of config 1 takes about 40 s on
one host core.
"""
from __future__ import annotations

import multiprocessing as mp

import numpy as np
import pytest

from helpers import SOL_REL, iter_ok, iter_ok_mixed, oracle_solve, rel_l2, system
from oracle import tfs_oracle as O
from tflows import TFS_BICG, TFS_CG, TFS_CGS, TFS_FP64, TFS_MIXED, Batch, Solver
from tflows.synth import BASE_SEED, CONVDIFF, POISSON, batched_poisson_specs

pytestmark = pytest.mark.gpu

MIXED_REL = 1e-6


def _gpu_solve(s, method, prec, mode, niter, tol):
    with Solver(s.matrix(), precision=mode) as sol:
        x, r = np.zeros(s.n), s.b.copy()
        res = sol.solve(method, s.val, x, r, prec, niter, tol)
    return res, x, r


def _check(s, ref, method, prec, niter):
    for mode in (TFS_FP64, TFS_MIXED):
        res, x, r = _gpu_solve(s, method, prec, mode, niter, ref["tol"])
        assert res.status == 0, (mode, res)
        ok = iter_ok if mode == TFS_FP64 else iter_ok_mixed
        assert ok(res.niter, ref["niter"]), (mode, res.niter, ref["niter"])
        err = rel_l2(x, ref["x"])
        if mode == TFS_FP64:
            assert err <= SOL_REL, err
            assert res.ini_res == pytest.approx(ref["ini"], rel=1e-12)
        else:
            assert err <= MIXED_REL, err
            # the mixed solve stops on its binary64 true residual: check it
            rt = s.b.copy()
            O.residual(s.n, s.row, s.col, s.val, x, rt)
            assert np.linalg.norm(rt) < ref["tol"]
            assert res.fin_res < ref["tol"]


def test_config0_poisson32_diag_cg(gpu):
    s = system(POISSON, 32, jitter=0.2, seed=BASE_SEED)
    assert (s.n, s.nnz) == (32768, 223232)
    ref = oracle_solve(s, TFS_CG, 1, niter=2000)
    assert ref["niter"] <= 2000
    _check(s, ref, TFS_CG, 1, 2000)


@pytest.fixture(scope="module")
def poisson128(gpu):
    s = system(POISSON, 128, jitter=0.2, seed=BASE_SEED)
    assert (s.n, s.nnz) == (2097152, 14581760)
    return s, oracle_solve(s, TFS_CG, 2, niter=5000)


def test_config1_poisson128_dic_cg(poisson128):
    s, ref = poisson128
    _check(s, ref, TFS_CG, 2, 5000)


def test_config1_bicg_is_the_cg_sequence(poisson128):
    """The reference's BiCG call on the same system returns CG's iterate."""
    s, ref = poisson128
    res, x, _ = _gpu_solve(s, TFS_BICG, 2, TFS_FP64, 5000, ref["tol"])
    assert res.status == 0 and iter_ok(res.niter, ref["niter"]) and rel_l2(x, ref["x"]) <= SOL_REL


@pytest.fixture(scope="module")
def convdiff160(gpu):
    s = system(CONVDIFF, 160, jitter=0.2, seed=BASE_SEED)
    assert (s.n, s.nnz) == (4096000, 28518400)
    return s


def test_config2_convdiff160_diag_cgs(convdiff160):
    s = convdiff160
    ref = oracle_solve(s, TFS_CGS, 1, niter=5000)
    _check(s, ref, TFS_CGS, 1, 5000)


def test_config2_convdiff160_diag_bicg_bounded(convdiff160):
    """The reference's BiCG is CG on this non-symmetric system and does not
    converge (the benchmark reaches its 5000-iteration limit); the first 25
    iterations are compared with the oracle's: same residual history
    length (limit + 1) and the iterate within the binary64 gate."""
    s = convdiff160
    tol = 1e-8 * float(np.linalg.norm(s.b))
    xo, ro = np.zeros(s.n), s.b.copy()
    it, ini, fin = O.solve(TFS_BICG, s.n, s.row, s.col, s.dia, s.val, xo, ro, 1, 25, tol)
    res, x, r = _gpu_solve(s, TFS_BICG, 1, TFS_FP64, 25, tol)
    assert it == 26 and res.niter == 26
    assert res.ini_res == pytest.approx(ini, rel=1e-12)
    assert res.fin_res == pytest.approx(fin, rel=1e-9)
    assert rel_l2(x, xo) <= SOL_REL
    assert rel_l2(r, ro) <= 1e-8


def _oracle_batch_one(spec):
    import sys
    from pathlib import Path
    repo = Path(__file__).resolve().parents[1]
    sys.path[:0] = [str(repo), str(repo / "t-flows_gb300"), str(repo / "tests")]
    from helpers import oracle_solve as osolve
    from helpers import system as msys
    nx, ny, nz, jit, sd = spec
    s = msys(POISSON, nx, ny, nz, jitter=jit, seed=sd)
    ref = osolve(s, TFS_CG, 1, niter=5000)
    return ref["x"], ref["niter"], ref["ini"]


@pytest.fixture(scope="module")
def batch_sample(gpu):
    """32 systems of the 256-system batch (every eighth of the seeded
    specification, so the sizes span the log-uniform range), with their
    oracle solutions computed on the host cores (spawned processes: a
    forked pool would inherit the CUDA context)."""
    specs = batched_poisson_specs(256, BASE_SEED)[::8]
    with mp.get_context("spawn").Pool(min(16, mp.cpu_count())) as pool:
        refs = pool.map(_oracle_batch_one, specs)
    systems = [system(POISSON, nx, ny, nz, jitter=jit, seed=sd) for nx, ny, nz, jit, sd in specs]
    return systems, refs


@pytest.mark.parametrize("mode", [TFS_FP64, TFS_MIXED])
def test_config3_batch_sample_against_the_oracle(mode, batch_sample):
    systems, refs = batch_sample
    solvers = [Solver(s.matrix()) for s in systems]
    try:
        with Batch(solvers, cluster=8, threads=512) as b:
            xs = [np.zeros(s.n) for s in systems]
            rs = [s.b.copy() for s in systems]
            tols = [1e-8 * np.linalg.norm(s.b) for s in systems]
            res = b.solve(TFS_CG, 1, [s.val for s in systems], xs, rs, 5000, tols, mode=mode)
        for k, s in enumerate(systems):
            xo, it, ini = refs[k]
            assert res.status[k] == 0, k
            ok = iter_ok if mode == TFS_FP64 else iter_ok_mixed
            assert ok(int(res.niter[k]), it), (k, int(res.niter[k]), it)
            err = rel_l2(xs[k], xo)
            assert err <= (SOL_REL if mode == TFS_FP64 else MIXED_REL), (k, err)
            if mode == TFS_FP64:
                assert res.ini_res[k] == pytest.approx(ini, rel=1e-12)
            else:
                assert res.fin_res[k] < tols[k]
    finally:
        for sv in solvers:
            sv.close()
