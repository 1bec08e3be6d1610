"""Solves on the reference's own test meshes (tests/golden/gambit_*.npz,
built from Gambit neutral files of its Tests/ directory): real unstructured
orderings instead of the synthetic random numbering.  Parity gates as for
the synthetic systems; topology and assembly on the device bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

from gambit_fixture import NAMES, load
from helpers import SOL_REL, iter_ok, rel_l2
from oracle import tfs_oracle as O
from tflows import TFS_BICG, TFS_CG, TFS_CGS, TFS_FP64, TFS_MIXED, Solver
from tflows.matrix_mod import Matrix_Mod_Topology_Device

pytestmark = pytest.mark.gpu


def oracle(s, method, prec):
    tol = 1e-8 * float(np.linalg.norm(s.b))
    x, r = np.zeros(s.n), s.b.copy()
    it, ini, fin = O.solve(method, s.n, s.row, s.col, s.dia, s.val, x, r, prec, 5000, tol)
    return dict(x=x, niter=it, fin=fin, tol=tol)


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("prec", [0, 1, 2])
def test_cg_on_reference_mesh(name, prec, gpu):
    """CG in binary64 within the parity gates of the oracle (iterations
    within 2%, solution within 1e-9 relative L2), BiCG (the reference's
    A-driven BiCG is CG) the same, CGS converging, and mixed precision
    converged on the binary64 true residual.

    These meshes are far worse conditioned than the synthetic cubes (wall
    refinement, stretched cells: 3469 unpreconditioned iterations on
    plain_50).  Without a preconditioner the two binary64 solutions, each
    stopped at ||r|| < 1e-8 ||b||, differ by the reduction order amplified by
    the conditioning (1.5e-9 and 2.3e-9 measured, iterations equal), so that
    case is held to 1e-8; the mixed-precision solve may take up to a quarter
    more iterations than the binary64 oracle (517 against 460 measured on
    plain_50 with the diagonal preconditioner)."""
    s = load(name)
    ref = oracle(s, 0, prec)
    assert ref["niter"] <= 5000
    sol_rel = SOL_REL if prec else 1e-8
    with Solver(s.matrix()) as sol:
        x, r = np.zeros(s.n), s.b.copy()
        res = sol.solve(TFS_CG, s.val, x, r, prec, 5000, ref["tol"])
        assert res.status == 0 and iter_ok(res.niter, ref["niter"]) and rel_l2(x, ref["x"]) <= sol_rel
        x, r = np.zeros(s.n), s.b.copy()
        res = sol.solve(TFS_BICG, s.val, x, r, prec, 5000, ref["tol"])
        assert res.status == 0 and iter_ok(res.niter, ref["niter"]) and rel_l2(x, ref["x"]) <= sol_rel
        ref_s = oracle(s, 2, prec)
        x, r = np.zeros(s.n), s.b.copy()
        res = sol.solve(TFS_CGS, s.val, x, r, prec, 5000, ref_s["tol"])
        if ref_s["niter"] <= 5000:
            assert res.status == 0 and res.fin_res < ref_s["tol"]
    with Solver(s.matrix(), precision=TFS_MIXED) as sol:
        x, r = np.zeros(s.n), s.b.copy()
        res = sol.solve(TFS_CG, s.val, x, r, prec, 5000, ref["tol"])
        assert res.status == 0 and res.fin_res < ref["tol"]
        assert res.niter <= 1.25 * ref["niter"] and rel_l2(x, ref["x"]) < 1e-6


@pytest.mark.parametrize("name", NAMES)
def test_preconditioner_and_spmv_bitwise(name, gpu):
    """Prec_Form, Prec_Solve (diagonal and DIC on the mesh's own numbering,
    which gives a deep level schedule) and the SpMV bitwise equal to the
    oracle."""
    s = load(name)
    rng = np.random.default_rng(3)
    b = rng.uniform(-1, 1, s.n)
    with Solver(s.matrix()) as sol:
        assert np.array_equal(sol.spmv(s.val, b), O.spmv(s.n, s.row, s.col, s.val, b))
        for prec in (1, 2):
            assert np.array_equal(sol.prec_form(s.val, prec), O.prec_form(s.n, s.row, s.col, s.dia, s.val, prec))
            assert np.array_equal(sol.prec_solve(s.val, prec, b),
                                  O.prec_solve(s.n, s.row, s.col, s.dia, s.val, prec, b))


@pytest.mark.parametrize("name", NAMES)
def test_device_topology_and_assembly(name, gpu):
    """Matrix_Mod_Topology on the device and the face-loop assembly on the
    device reproduce the host arrays and values bit for bit."""
    s = load(name)
    D = Matrix_Mod_Topology_Device(s.n, s.faces_c)
    assert np.array_equal(D.row, s.row) and np.array_equal(D.col, s.col)
    assert np.array_equal(D.dia, s.dia) and np.array_equal(D.pos, s.pos)
    interior = s.faces_c[:, 1] > 0
    off = np.where(interior, s.coef, 0.0)
    with Solver(s.matrix()) as sol:
        sol.faces_register(s.faces_c, s.pos)
        val = sol.assemble(off, off, s.coef, off)
    assert np.array_equal(val, s.val)


def test_solve_from_reference_format_files(gpu):
    """A mesh stored in the reference's own .cns/.geo format solves on the
    GPU within the parity gates (binary64) and converges in mixed precision."""
    from pathlib import Path
    from tflows import cns_geo
    golden = Path(__file__).resolve().parent / "golden"
    s = cns_geo.pressure_system(golden / "chan.cns", golden / "chan.geo", dirichlet_bcs=(1,))
    for prec in (1, 2):
        ref = oracle(s, 0, prec)
        with Solver(s.matrix()) as sol:
            x, r = np.zeros(s.n), s.b.copy()
            res = sol.solve(TFS_CG, s.val, x, r, prec, 5000, ref["tol"])
            assert res.status == 0 and iter_ok(res.niter, ref["niter"]) and rel_l2(x, ref["x"]) <= SOL_REL
        with Solver(s.matrix(), precision=TFS_MIXED) as sol:
            x, r = np.zeros(s.n), s.b.copy()
            res = sol.solve(TFS_CG, s.val, x, r, prec, 5000, ref["tol"])
            assert res.status == 0 and res.fin_res < ref["tol"] and rel_l2(x, ref["x"]) < 1e-6


@pytest.mark.parametrize("name", NAMES)
def test_one_block_dic_on_reference_mesh(name, gpu):
    """The reference's meshes in their own numbering have deep level
    schedules (plain_50: 148 levels of at most 149 rows), which is what the
    one-block DIC (the swept vector in shared memory) is for: Prec_Form and
    Prec_Solve bitwise equal to the oracle, and DIC-CG solves in both
    arithmetics bitwise equal to the level kernels' (TFS_OPT_DIC_BLOCK = 0,
    with level 0 not fused, so that rho is reduced by the same kernel)."""
    from tflows.lib import TFS_OPT_DIC_BLOCK, TFS_OPT_FUSE_L0
    s = load(name)
    b = np.random.default_rng(3).uniform(-1, 1, s.n)
    ref = oracle(s, TFS_CG, 2)
    out = {}
    for blk in (1, 0):
        res = []
        for mode in (TFS_FP64, TFS_MIXED):
            with Solver(s.matrix(), precision=mode, options={TFS_OPT_DIC_BLOCK: blk, TFS_OPT_FUSE_L0: 0}) as sol:
                if mode == TFS_FP64:
                    d = sol.prec_form(s.val, 2)
                    z = sol.prec_solve(s.val, 2, b)
                    assert sol.stats()["dic_kernel"] == blk
                    assert np.array_equal(d, O.prec_form(s.n, s.row, s.col, s.dia, s.val, 2))
                    assert np.array_equal(z, O.prec_solve(s.n, s.row, s.col, s.dia, s.val, 2, b))
                    res += [d, z]
                x, r = np.zeros(s.n), s.b.copy()
                st = sol.solve(TFS_CG, s.val, x, r, 2, 5000, ref["tol"])
                assert st.status == 0 and st.fin_res < ref["tol"]
                assert sol.stats()["dic_kernel"] == blk
                if mode == TFS_FP64:
                    assert iter_ok(st.niter, ref["niter"]) and rel_l2(x, ref["x"]) <= SOL_REL
                res += [x, r, st.niter, st.fin_res]
        out[blk] = res
    for a, c in zip(out[1], out[0]):
        assert np.array_equal(a, c)


def test_one_block_dic_wait_runs_out(gpu):
    """The one-block DIC's bounded waits: with its copy lane staging nothing
    and a 2 ms limit (tfs_diag_dic_timeout), its first wait runs out and the
    solve returns TFS_ERR_TIMEOUT promptly; with the normal limit restored
    the same handle solves as before, bit for bit (the GPU still answers and
    nothing of the aborted launch lingers)."""
    import time
    from tflows.lib import TFS_ERR_TIMEOUT, TfsError, load_library
    lib = load_library()
    s = load("plain50")
    ref = oracle(s, TFS_CG, 2)
    with Solver(s.matrix()) as sol:
        x, r = np.zeros(s.n), s.b.copy()
        good = sol.solve(TFS_CG, s.val, x, r, 2, 5000, ref["tol"])
        assert good.status == 0 and sol.stats()["dic_kernel"] == 1
        assert lib.tfs_diag_dic_timeout(sol.h, 2_000_000) == 0
        t = time.perf_counter()
        with pytest.raises(TfsError) as e:
            sol.solve(TFS_CG, s.val, np.zeros(s.n), s.b.copy(), 2, 5000, ref["tol"])
        assert e.value.status == TFS_ERR_TIMEOUT
        assert time.perf_counter() - t < 5.0
        assert lib.tfs_diag_dic_timeout(sol.h, 0) == 0
        x2, r2 = np.zeros(s.n), s.b.copy()
        again = sol.solve(TFS_CG, s.val, x2, r2, 2, 5000, ref["tol"])
        assert again.status == 0 and again.niter == good.niter
        assert np.array_equal(x2, x) and np.array_equal(r2, r)
        assert lib.tfs_diag_dic_timeout(sol.h, -1) != 0
