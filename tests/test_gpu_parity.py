"""GPU parity: the CUDA path through the C ABI against the oracle.

Per-row routines (SpMV, Residual, Prec_Form, Prec_Solve) must be bitwise
equal to the oracle: the kernels keep the reference's per-row arithmetic.
Whole solves differ from the oracle only through the order of the dot
product sums, so they are gated by the tolerances of the hot-path contract:
iteration count within +-2% (never tighter than +-1) and solution relative L2
difference <= 1e-9 at a 1e-8 relative stopping tolerance.
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import SOL_REL, iter_ok, oracle_solve, rel_l2, system
from oracle import tfs_oracle as O
from tflows import (TFS_BICG, TFS_CG, TFS_CGS, TFS_FP64, TFS_MIXED, Matrix_Type, Solver)
from tflows.lib import (TFS_ERR_NONFINITE, TFS_OPT_BICG, TFS_OPT_BWD_PRE, TFS_OPT_FUSE_L0, TFS_OPT_FWD_PRE,
                        TFS_OPT_LEVEL_TPB, TFS_OPT_SELL_UNIFORM, TFS_OPT_SPMV, TFS_OPT_SPMV_GRID,
                        TFS_OPT_TAIL_PF)
from tflows.synth import CONVDIFF, POISSON

pytestmark = pytest.mark.gpu

METHODS = [TFS_CG, TFS_BICG, TFS_CGS]
PRECS = [0, 1, 2]


@pytest.fixture(scope="module")
def poisson16(gpu):
    s = system(POISSON, 16)
    return s, Solver(s.matrix())


@pytest.fixture(scope="module")
def convdiff12(gpu):
    s = system(CONVDIFF, 12, 11, 10)
    return s, Solver(s.matrix())


# ------------------------------------------------------ per-row routines

@pytest.mark.parametrize("which", ["poisson", "convdiff"])
def test_spmv_bitwise(which, poisson16, convdiff12):
    s, sol = poisson16 if which == "poisson" else convdiff12
    p = np.random.default_rng(1).uniform(-1, 1, s.n)
    q = sol.spmv(s.val, p)
    assert np.array_equal(q, O.spmv(s.n, s.row, s.col, s.val, p))


def test_residual_bitwise(poisson16):
    s, sol = poisson16
    x = np.random.default_rng(2).uniform(-1, 1, s.n)
    r_gpu = s.b.copy()
    sol.residual(s.val, x, r_gpu)
    r_ref = s.b.copy()
    O.residual(s.n, s.row, s.col, s.val, x, r_ref)
    assert np.array_equal(r_gpu, r_ref)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("which", ["poisson", "convdiff"])
def test_prec_form_bitwise(prec, which, poisson16, convdiff12):
    s, sol = poisson16 if which == "poisson" else convdiff12
    d = sol.prec_form(s.val, prec)
    assert np.array_equal(d, O.prec_form(s.n, s.row, s.col, s.dia, s.val, prec))


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("which", ["poisson", "convdiff"])
def test_prec_solve_bitwise(prec, which, poisson16, convdiff12):
    s, sol = poisson16 if which == "poisson" else convdiff12
    b = np.random.default_rng(3).uniform(-1, 1, s.n)
    x = sol.prec_solve(s.val, prec, b)
    assert np.array_equal(x, O.prec_solve(s.n, s.row, s.col, s.dia, s.val, prec, b))


def test_level_schedule_valid(poisson16):
    """Every lower neighbour of a row sits on a strictly smaller level and the
    levels are the longest-path depths (host recomputation)."""
    s, sol = poisson16
    lv = sol.levels()
    want = np.zeros(s.n, np.int64)
    for i in range(s.n):
        lo = s.row[i] - 1
        cols = s.col[lo:s.dia[i] - 1] - 1
        want[i] = 0 if cols.size == 0 else 1 + want[cols].max()
    assert np.array_equal(lv, want)


def test_level_schedule_natural_order(gpu):
    """Unpermuted cell numbering: the levels are the i+j+k hyperplanes."""
    s = system(POISSON, 6, 5, 4, permute=False)
    lv = Solver(s.matrix()).levels()
    ijk = np.array([i + j + k for k in range(4) for j in range(5) for i in range(6)])
    assert np.array_equal(lv, ijk)


# ------------------------------------------------------ whole solves

@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("method", METHODS)
def test_solve_matches_oracle_poisson(method, prec, poisson16):
    s, sol = poisson16
    ref = oracle_solve(s, method, prec)
    x = np.zeros(s.n)
    r = s.b.copy()
    res = sol.solve(method, s.val, x, r, prec, 2000, ref["tol"])
    assert res.status == 0
    assert iter_ok(res.niter, ref["niter"]), (res.niter, ref["niter"])
    assert rel_l2(x, ref["x"]) <= SOL_REL
    assert res.ini_res == pytest.approx(ref["ini"], rel=1e-13)
    assert res.fin_res < ref["tol"]
    # r1 returns the final recursive residual (Cg.f90:159-162); it is ~tol in
    # size, so its difference is gated relative to ||b|| like the solution.
    assert np.linalg.norm(r - ref["r"]) <= SOL_REL * np.linalg.norm(s.b)


@pytest.mark.parametrize("prec", [1, 2])
@pytest.mark.parametrize("method", [TFS_BICG, TFS_CGS])
def test_solve_matches_oracle_convdiff(method, prec, convdiff12):
    s, sol = convdiff12
    ref = oracle_solve(s, method, prec)
    x = np.zeros(s.n)
    r = s.b.copy()
    res = sol.solve(method, s.val, x, r, prec, 2000, ref["tol"])
    assert res.status == 0
    assert iter_ok(res.niter, ref["niter"]), (res.niter, ref["niter"])
    assert rel_l2(x, ref["x"]) <= SOL_REL


def test_solve_32_cube_dic_cg(gpu):
    s = system(POISSON, 32)
    ref = oracle_solve(s, TFS_CG, 2)
    x = np.zeros(s.n)
    r = s.b.copy()
    res = Solver(s.matrix()).solve(TFS_CG, s.val, x, r, 2, 2000, ref["tol"])
    assert iter_ok(res.niter, ref["niter"]) and rel_l2(x, ref["x"]) <= SOL_REL


def test_nonzero_initial_guess(poisson16):
    s, sol = poisson16
    x0 = np.random.default_rng(4).uniform(-1, 1, s.n)
    ref = oracle_solve(s, TFS_CG, 1, x0=x0)
    x, r = x0.copy(), s.b.copy()
    res = sol.solve(TFS_CG, s.val, x, r, 1, 2000, ref["tol"])
    assert iter_ok(res.niter, ref["niter"]) and rel_l2(x, ref["x"]) <= SOL_REL


def test_reproducible_bitwise(poisson16):
    s, sol = poisson16
    outs = []
    for _ in range(2):
        x, r = np.zeros(s.n), s.b.copy()
        res = sol.solve(TFS_BICG, s.val, x, r, 2, 500, 1e-10)
        outs.append((x, r, res))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
    assert outs[0][2] == outs[1][2]


# ------------------------------------------------------ reference semantics

@pytest.mark.parametrize("method", METHODS)
def test_early_exit_small_b(method, poisson16):
    """||b|| < tol: iter = 0, x and r1 untouched, ini_res untouched,
    fin_res = ||b|| (Cg.f90:55-58)."""
    s, sol = poisson16
    b = s.b * 1e-12
    x, r = np.ones(s.n), b.copy()
    res = sol.solve(method, s.val, x, r, 1, 100, 1.0, ini_res=-7.0)
    assert res.niter == 0 and res.ini_res == -7.0
    assert res.fin_res == pytest.approx(np.linalg.norm(b), rel=1e-13)
    assert np.array_equal(x, np.ones(s.n)) and np.array_equal(r, b)


@pytest.mark.parametrize("method", METHODS)
def test_early_exit_exact_guess(method, poisson16):
    """||b - A x0|| < tol: iter = 0, ini_res = fin_res (Cg.f90:85-90)."""
    s, sol = poisson16
    xs = np.random.default_rng(5).uniform(-1, 1, s.n)
    b = O.spmv(s.n, s.row, s.col, s.val, xs)
    ref_x, ref_r = xs.copy(), b.copy()
    it, ini, fin = O.solve(method, s.n, s.row, s.col, s.dia, s.val, ref_x, ref_r, 1, 100, 1e-6)
    x, r = xs.copy(), b.copy()
    res = sol.solve(method, s.val, x, r, 1, 100, 1e-6)
    assert res.niter == it == 0
    assert res.ini_res == res.fin_res and res.ini_res == pytest.approx(ini, rel=1e-12, abs=1e-15)
    assert np.array_equal(r, ref_r)


@pytest.mark.parametrize("method", METHODS)
def test_not_converged_returns_limit_plus_one(method, poisson16):
    s, sol = poisson16
    ref = oracle_solve(s, method, 1, niter=7, rel=1e-14)
    x, r = np.zeros(s.n), s.b.copy()
    res = sol.solve(method, s.val, x, r, 1, 7, ref["tol"])
    assert res.niter == ref["niter"] == 8
    assert rel_l2(x, ref["x"]) <= 1e-12
    assert res.fin_res == pytest.approx(ref["fin"], rel=1e-10)


def test_zero_iteration_limit(poisson16):
    s, sol = poisson16
    ref = oracle_solve(s, TFS_CG, 1, niter=0)
    x, r = np.zeros(s.n), s.b.copy()
    res = sol.solve(TFS_CG, s.val, x, r, 1, 0, ref["tol"])
    assert res.niter == ref["niter"] == 1
    assert res.fin_res == pytest.approx(ref["fin"], rel=1e-13)


def test_nan_rhs_reports_nonfinite(poisson16):
    s, sol = poisson16
    b = s.b.copy()
    b[3] = np.nan
    x, r = np.zeros(s.n), b.copy()
    res = sol.solve(TFS_CG, s.val, x, r, 1, 50, 1e-8)
    assert res.status == TFS_ERR_NONFINITE
    assert np.isnan(res.fin_res) and res.niter == 51


def test_tiny_systems(gpu):
    """n = 1 (a single diagonal entry) and ragged n < 32."""
    A = Matrix_Type(1, [1, 2], [1], [1], [4.0])
    with Solver(A) as sol:
        x, r = np.zeros(1), np.array([2.0])
        res = sol.solve(TFS_CG, A.val, x, r, 1, 10, 1e-12)
        assert res.niter == 1 and x[0] == 0.5
    s = system(POISSON, 3, 2, 1)
    ref = oracle_solve(s, TFS_CG, 2)
    x, r = np.zeros(s.n), s.b.copy()
    res = Solver(s.matrix()).solve(TFS_CG, s.val, x, r, 2, 100, ref["tol"])
    assert iter_ok(res.niter, ref["niter"]) and rel_l2(x, ref["x"]) <= SOL_REL


def test_fortran_shaped_entry_points(poisson16):
    """tfs_cg/tfs_bicg/tfs_cgs with no handle (cached by array identity)."""
    import ctypes as C
    from tflows.matrix_mod import ptr
    s, _ = poisson16
    from tflows.lib import load_library
    lib = load_library()
    for fn, method in ((lib.tfs_cg, TFS_CG), (lib.tfs_bicg, TFS_BICG), (lib.tfs_cgs, TFS_CGS)):
        ref = oracle_solve(s, method, 1)
        x, r = np.zeros(s.n), s.b.copy()
        it, ini, fin = C.c_int32(2000), C.c_double(0), C.c_double(0)
        st = fn(s.n, s.nnz, ptr(s.row, C.c_int32), ptr(s.col, C.c_int32), ptr(s.dia, C.c_int32),
                ptr(s.val, C.c_double), ptr(x, C.c_double), ptr(r, C.c_double), 1,
                C.byref(it), ref["tol"], C.byref(ini), C.byref(fin))
        assert st == 0 and iter_ok(it.value, ref["niter"]) and rel_l2(x, ref["x"]) <= SOL_REL


# ------------------------------------------------------ mixed precision

@pytest.mark.parametrize("prec", [1, 2])
@pytest.mark.parametrize("method", METHODS)
def test_mixed_precision_converges(method, prec, poisson16):
    """Binary32 inner iterations with binary64 reliable updates reach the same
    absolute tolerance on the binary64 true residual; error vs the FP64 oracle
    is bounded by the conditioning at that tolerance."""
    s, _ = poisson16
    ref = oracle_solve(s, method, prec)
    with Solver(s.matrix(), precision=TFS_MIXED) as sol:
        x, r = np.zeros(s.n), s.b.copy()
        res = sol.solve(method, s.val, x, r, prec, 2000, ref["tol"])
        st = sol.stats()
    assert res.status == 0
    assert res.fin_res < ref["tol"]
    rt = s.b.copy()
    O.residual(s.n, s.row, s.col, s.val, x, rt)
    assert np.linalg.norm(rt) < ref["tol"]          # true residual, binary64
    assert np.array_equal(r, rt) or rel_l2(r, rt) < 1e-12
    assert rel_l2(x, ref["x"]) < 1e-6
    assert res.niter <= 1.3 * ref["niter"] + 5
    assert st["true_residuals"] >= 2


# ------------------------------------------------------ non-symmetric pattern

def test_matrix_mod_example_nonsymmetric_pattern(gpu):
    """The documented CSR example of Matrix_Mod.f90:15-34 is not structurally
    symmetric; the level analysis must then also order the backward sweep's
    dependencies.  Per-row routines stay bitwise equal to the oracle."""
    from pathlib import Path
    g = np.load(Path(__file__).resolve().parent / "golden" / "matrix_mod_example.npz")
    A = Matrix_Type(4, g["row"], g["col"], g["dia"], g["val"])
    b = np.array([1.0, 2.0, 3.0, 4.0])
    with Solver(A) as sol:
        p = np.array([1.0, -2.0, 0.5, 3.0])
        assert np.array_equal(sol.spmv(A.val, p), O.spmv(4, A.row, A.col, A.val, p))
        for prec in PRECS:
            assert np.array_equal(sol.prec_form(A.val, prec),
                                  O.prec_form(4, A.row, A.col, A.dia, A.val, prec))
            assert np.array_equal(sol.prec_solve(A.val, prec, b),
                                  O.prec_solve(4, A.row, A.col, A.dia, A.val, prec, b))
        for method in METHODS:
            xo, ro = np.zeros(4), b.copy()
            it, ini, fin = O.solve(method, 4, A.row, A.col, A.dia, A.val, xo, ro, 2, 50, 1e-12)
            x, r = np.zeros(4), b.copy()
            res = sol.solve(method, A.val, x, r, 2, 50, 1e-12)
            assert iter_ok(res.niter, it) and rel_l2(x, xo) <= 1e-12


@pytest.mark.parametrize("tpb", [128, 256, 512, 1024])
def test_level_kernel_block_sizes_agree(tpb, gpu):
    """The level kernels at every block size the autotuner may pick do the
    same per-row arithmetic: Prec_Form and Prec_Solve bitwise equal to the
    oracle, and solves within the parity gates.  The 40^3 system has levels
    of more than a block, so several blocks run per level, not only the
    tail."""
    for s, method in ((system(CONVDIFF, 10, 9, 8), TFS_BICG), (system(POISSON, 40, 40, 40), TFS_CG)):
        b = np.random.default_rng(9).uniform(-1, 1, s.n)
        with Solver(s.matrix(), options={TFS_OPT_LEVEL_TPB: tpb}) as sol:
            assert np.array_equal(sol.prec_form(s.val, 2), O.prec_form(s.n, s.row, s.col, s.dia, s.val, 2))
            assert np.array_equal(sol.prec_solve(s.val, 2, b),
                                  O.prec_solve(s.n, s.row, s.col, s.dia, s.val, 2, b))
            ref = oracle_solve(s, method, 2)
            x, r = np.zeros(s.n), s.b.copy()
            res = sol.solve(method, s.val, x, r, 2, 2000, ref["tol"])
            assert res.status == 0
            assert iter_ok(res.niter, ref["niter"]) and rel_l2(x, ref["x"]) <= SOL_REL
        if s.n > 60000:
            with Solver(s.matrix(), precision=TFS_MIXED, options={TFS_OPT_LEVEL_TPB: tpb}) as sol:
                x, r = np.zeros(s.n), s.b.copy()
                res = sol.solve(method, s.val, x, r, 2, 2000, ref["tol"])
                assert res.status == 0 and res.fin_res < ref["tol"]
                assert iter_ok(res.niter, ref["niter"]) and rel_l2(x, ref["x"]) < 1e-6


@pytest.mark.parametrize("grid", [0, 1])
def test_spmv_kernels_bitwise(grid, gpu):
    """The software-pipelined CG SpMV for uniform-width matrices (the next
    row's column indices loaded while the current row's gathers are in
    flight) takes the direct kernel's rows, dot-product order and reductions
    over the same grid (8 blocks per SM, or one block per chunk): q = A p and
    whole CG solves (binary64 and mixed, diagonal and DIC) are bitwise those
    of the direct kernel (TFS_OPT_SPMV = 0)."""
    s = system(POISSON, 40, 40, 40)
    ref = oracle_solve(s, TFS_CG, 2)
    pv = np.random.default_rng(5).uniform(-1, 1, s.n)
    out = {}
    for k in (1, 0):
        res = []
        for mode in (TFS_FP64, TFS_MIXED):
            opts = {TFS_OPT_SPMV: k, TFS_OPT_SPMV_GRID: grid}
            with Solver(s.matrix(), precision=mode, options=opts) as sol:
                if mode == TFS_FP64:
                    res.append(sol.spmv(s.val, pv))
                for prec in (1, 2):
                    x, r = np.zeros(s.n), s.b.copy()
                    st = sol.solve(TFS_CG, s.val, x, r, prec, 2000, ref["tol"])
                    assert st.status == 0 and st.fin_res < ref["tol"]
                    res += [x, r, st.niter, st.fin_res]
                assert sol.stats()["spmv_kernel"] == k
        out[k] = res
    assert np.array_equal(out[0][0], O.spmv(s.n, s.row, s.col, s.val, pv))
    for a, b in zip(out[1], out[0]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("shape", [(40, 40, 40), (23, 19, 17), (9, 8, 8)])
def test_tail_prefetch_bitwise(shape, gpu):
    """The one-row-per-thread tail (every row's entries, right-hand side and
    diagonal loaded before the dependency wait) gives the DIC application
    and whole DIC-CG solves bitwise equal to the level-by-level tail loop
    (TFS_OPT_TAIL_PF = 0), and Prec_Solve equal to the oracle."""
    s = system(POISSON, *shape)
    ref = oracle_solve(s, TFS_CG, 2)
    b = np.random.default_rng(4).uniform(-1, 1, s.n)
    out = {}
    for pf in (1, 0):
        res = []
        for mode in (TFS_FP64, TFS_MIXED):
            with Solver(s.matrix(), precision=mode, options={TFS_OPT_TAIL_PF: pf}) as sol:
                if mode == TFS_FP64:
                    res.append(sol.prec_solve(s.val, 2, b))
                x, r = np.zeros(s.n), s.b.copy()
                st = sol.solve(TFS_CG, s.val, x, r, 2, 2000, ref["tol"])
                assert st.status == 0 and st.fin_res < ref["tol"]
                res += [x, r, st.niter]
        out[pf] = res
    assert np.array_equal(out[1][0], O.prec_solve(s.n, s.row, s.col, s.dia, s.val, 2, b))
    for a, c in zip(out[1], out[0]):
        assert np.array_equal(a, c)


@pytest.mark.parametrize("kind", [POISSON, CONVDIFF])
def test_per_slice_width_layout(kind, gpu):
    """Per-slice SELL widths (TFS_OPT_SELL_UNIFORM = 0: slice offsets loaded
    instead of computed, so the direct SpMV kernels and the level-loop tail
    run instead of the uniform-width ones): SpMV, Prec_Solve bitwise equal
    to the oracle and CG / BiCG / CGS within the parity gates."""
    opts = {TFS_OPT_SELL_UNIFORM: 0}
    s = system(kind, 23, 19, 17)
    b = np.random.default_rng(8).uniform(-1, 1, s.n)
    methods = (TFS_CG,) if kind == POISSON else (TFS_BICG, TFS_CGS)
    with Solver(s.matrix(), options=opts) as sol:
        assert np.array_equal(sol.spmv(s.val, b), O.spmv(s.n, s.row, s.col, s.val, b))
        assert sol.stats()["sell_width"] == 0
        for prec in (1, 2):
            assert np.array_equal(sol.prec_solve(s.val, prec, b),
                                  O.prec_solve(s.n, s.row, s.col, s.dia, s.val, prec, b))
        for method in methods:
            for prec in (1, 2):
                ref = oracle_solve(s, method, prec)
                x, r = np.zeros(s.n), s.b.copy()
                res = sol.solve(method, s.val, x, r, prec, 2000, ref["tol"])
                assert iter_ok(res.niter, ref["niter"])
                if ref["niter"] <= 2000:
                    assert res.status == 0 and rel_l2(x, ref["x"]) <= SOL_REL
    with Solver(s.matrix(), precision=TFS_MIXED, options=opts) as sol:
        ref = oracle_solve(s, methods[0], 2)
        x, r = np.zeros(s.n), s.b.copy()
        res = sol.solve(methods[0], s.val, x, r, 2, 2000, ref["tol"])
        if ref["niter"] <= 2000:
            assert res.status == 0 and res.fin_res < ref["tol"]


@pytest.mark.parametrize("knob", ["bwd", "fwd"])
@pytest.mark.parametrize("shape", [(40, 40, 40), (23, 19, 17)])
def test_backward_precompute_bitwise(shape, knob, gpu):
    """Level kernels that load or compute their rows' start values before
    the dependency wait -- backward: y_i / (D_i + TINY) (the tail releases
    them only past its own wait); forward: b_i and D_i (written before the
    level chain starts) -- give the DIC application, DIC-CG solves in both
    precisions and the literal two-sequence BiCG bitwise equal to loading
    them after the wait (TFS_OPT_BWD_PRE = 0, TFS_OPT_FWD_PRE = 0)."""
    opt = TFS_OPT_BWD_PRE if knob == "bwd" else TFS_OPT_FWD_PRE
    s = system(POISSON, *shape)
    ref = oracle_solve(s, TFS_CG, 2)
    b = np.random.default_rng(6).uniform(-1, 1, s.n)
    out = {}
    for pre in (1, 0):
        res = []
        for mode in (TFS_FP64, TFS_MIXED):
            with Solver(s.matrix(), precision=mode, options={opt: pre}) as sol:
                if mode == TFS_FP64:
                    res.append(sol.prec_solve(s.val, 2, b))
                x, r = np.zeros(s.n), s.b.copy()
                st = sol.solve(TFS_CG, s.val, x, r, 2, 2000, ref["tol"])
                assert st.status == 0 and st.fin_res < ref["tol"]
                res += [x, r, st.niter]
        with Solver(s.matrix(), options={opt: pre, TFS_OPT_BICG: 1}) as sol:
            x, r = np.zeros(s.n), s.b.copy()
            st = sol.solve(TFS_BICG, s.val, x, r, 2, 2000, ref["tol"])
            res += [x, r, st.niter]
        out[pre] = res
    assert np.array_equal(out[1][0], O.prec_solve(s.n, s.row, s.col, s.dia, s.val, 2, b))
    for a, c in zip(out[1], out[0]):
        assert np.array_equal(a, c)


@pytest.mark.parametrize("fuse", [0, 1, 2])
def test_level0_fusion_parity(fuse, gpu):
    """DIC-CG with level 0 swept inside the residual, update and rho kernels
    (TFS_OPT_FUSE_L0: 0 off, 1 binary32 iteration, 2 binary64 too) stays
    within the parity gates of the oracle in both precisions on the 40^3
    system."""
    s = system(POISSON, 40, 40, 40)
    ref = oracle_solve(s, TFS_CG, 2)
    for mode, sol_tol in ((TFS_FP64, SOL_REL), (TFS_MIXED, 1e-6)):
        with Solver(s.matrix(), precision=mode, options={TFS_OPT_FUSE_L0: fuse}) as sol:
            x, r = np.zeros(s.n), s.b.copy()
            res = sol.solve(TFS_CG, s.val, x, r, 2, 2000, ref["tol"])
            assert res.status == 0 and res.fin_res < ref["tol"]
            assert iter_ok(res.niter, ref["niter"]) and rel_l2(x, ref["x"]) <= sol_tol


@pytest.mark.parametrize("mode", [TFS_FP64, TFS_MIXED])
@pytest.mark.parametrize("prec", [1, 2])
def test_bicg_equals_cg_bitwise(mode, prec, gpu):
    """The reference's BiCG (shadow residual r2 = r1, driven by A) produces the
    CG iterates bit for bit; the library runs it through the CG kernels.  In
    binary64 the literal two-sequence BiCG (TFS_BICG=literal) and CG agree
    bitwise.  In mixed precision the CG vector kernels split the rows over the
    threads differently from the BiCG kernels (16-byte loads), so the binary32
    partial sums round differently: there both converge on the binary64 true
    residual with iteration counts within 2% and solutions within the
    tolerance-implied distance, or both reach the iteration limit where the
    binary64 oracle does (this BiCG is CG and need not converge on a
    non-symmetric system)."""
    s = system(CONVDIFF, 9, 8, 8)
    tol = 1e-8 * np.linalg.norm(s.b)
    # Both runs reduce rho with the same kernel: the CG body's fusion of rho
    # into the level-0 backward sweep sums the partials in another order.
    out = {}
    for tag in ("cg", "literal"):
        opts = {TFS_OPT_FUSE_L0: 0, TFS_OPT_BICG: 1 if tag == "literal" else 0}
        with Solver(s.matrix(), precision=mode, options=opts) as sol:
            x, r = np.zeros(s.n), s.b.copy()
            method = TFS_CG if tag == "cg" else TFS_BICG
            out[tag] = (x, r, sol.solve(method, s.val, x, r, prec, 2000, tol))
    (xa, ra, resa), (xb, rb, resb) = out["cg"], out["literal"]
    if mode == TFS_FP64:
        assert np.array_equal(xa, xb) and np.array_equal(ra, rb)
        assert resa == resb
    # the oracle's Bicg equals its Cg
    ref_b, ref_c = oracle_solve(s, TFS_BICG, prec), oracle_solve(s, TFS_CG, prec)
    if mode == TFS_MIXED:
        if ref_b["niter"] <= 2000:
            assert resa.fin_res < tol and resb.fin_res < tol
            assert iter_ok(resa.niter, resb.niter)
            assert rel_l2(xa, xb) < 1e-5
        else:
            assert resa.niter == resb.niter == 2001
    assert np.array_equal(ref_b["x"], ref_c["x"]) and ref_b["niter"] == ref_c["niter"]


@pytest.mark.parametrize("prec", [1, 2])
def test_mixed_cgs_nonsymmetric(prec, convdiff12):
    """Mixed-precision CGS on the non-symmetric convection-diffusion system
    reaches the binary64 tolerance on the true residual."""
    s, _ = convdiff12
    ref = oracle_solve(s, TFS_CGS, prec)
    assert ref["niter"] < 2000
    with Solver(s.matrix(), precision=TFS_MIXED) as sol:
        x, r = np.zeros(s.n), s.b.copy()
        res = sol.solve(TFS_CGS, s.val, x, r, prec, 2000, ref["tol"])
    assert res.status == 0 and res.fin_res < ref["tol"]
    rt = s.b.copy()
    O.residual(s.n, s.row, s.col, s.val, x, rt)
    assert np.linalg.norm(rt) < ref["tol"]
    assert rel_l2(x, ref["x"]) < 1e-6


def test_bicg_nonconvergence_matches_reference(convdiff12):
    """On the non-symmetric system the reference's BiCG (= CG) does not reach
    1e-8 within the limit; the library reproduces the limit+1 return and the
    iterate."""
    s, sol = convdiff12
    ref = oracle_solve(s, TFS_BICG, 1, niter=300)
    x, r = np.zeros(s.n), s.b.copy()
    res = sol.solve(TFS_BICG, s.val, x, r, 1, 300, ref["tol"])
    assert ref["niter"] == 301 and res.niter == 301
    assert res.fin_res == pytest.approx(ref["fin"], rel=1e-6)


@pytest.mark.parametrize("mode", [TFS_FP64, TFS_MIXED])
def test_autotune_keeps_parity(mode, gpu):
    """tfs_autotune times the launch-shape candidates on the handle's own
    system, keeps the fastest and drops the cached graphs; solves after it
    still meet the parity gates."""
    s = system(POISSON, 40, 40, 40)
    ref = oracle_solve(s, TFS_CG, 2)
    with Solver(s.matrix(), precision=mode) as sol:
        x, r = np.zeros(s.n), s.b.copy()
        sol.solve(TFS_CG, s.val, x, r, 2, 2000, ref["tol"])      # a graph exists before tuning
        t = sol.autotune(s.val, mode, 2, 3)
        assert t["level_tpb"] in (128, 256, 512, 1024) and t["spmv_chunks"] in (0, 1)
        assert all(v > 0 for v in t["prec_ms"].values()) and all(v > 0 for v in t["spmv_ms"].values())
        assert t["prec_ms"][t["level_tpb"]] == min(t["prec_ms"].values())
        x, r = np.zeros(s.n), s.b.copy()
        res = sol.solve(TFS_CG, s.val, x, r, 2, 2000, ref["tol"])
        assert res.status == 0 and res.fin_res < ref["tol"] and iter_ok(res.niter, ref["niter"])
        assert rel_l2(x, ref["x"]) <= (SOL_REL if mode == TFS_FP64 else 1e-6)


@pytest.mark.parametrize("kind,shape", [(POISSON, (16, 16, 16)), (POISSON, (23, 19, 17)),
                                        (CONVDIFF, (12, 11, 10))])
def test_one_block_dic_bitwise(kind, shape, gpu):
    """The one-block DIC (forward sweep, scaling and backward sweep, and the
    Prec_Form recurrence, in one thread block with the vector in shared
    memory and each level's rows staged ahead) gives the level kernels'
    results bit for bit: Prec_Form and Prec_Solve equal to the oracle, whole
    DIC solves (CG in both arithmetics, CGS in binary64) equal to
    TFS_OPT_DIC_BLOCK = 0 with level 0 not fused.  The systems keep the
    mesh's own (lexicographic) cell numbering, whose level schedules are deep
    and narrow (46, 57 and 31 levels of at most 281 rows) -- what the kernel
    is for; under the random numbering of the benchmark the levels are too
    wide for its ring of level slots and the level kernels run."""
    from tflows.lib import TFS_OPT_DIC_BLOCK
    s = system(kind, *shape, permute=False)
    b = np.random.default_rng(12).uniform(-1, 1, s.n)
    methods = [TFS_CG] if kind == POISSON else [TFS_CGS]
    out = {}
    for blk in (1, 0):
        res = []
        for mode in (TFS_FP64, TFS_MIXED):
            with Solver(s.matrix(), precision=mode, options={TFS_OPT_DIC_BLOCK: blk, TFS_OPT_FUSE_L0: 0}) as sol:
                if mode == TFS_FP64:
                    res += [sol.prec_form(s.val, 2), sol.prec_solve(s.val, 2, b)]
                    assert sol.stats()["dic_kernel"] == blk
                for method in methods:
                    if mode == TFS_MIXED and method == TFS_CGS:
                        continue
                    ref = oracle_solve(s, method, 2)
                    x, r = np.zeros(s.n), s.b.copy()
                    st = sol.solve(method, s.val, x, r, 2, 2000, ref["tol"])
                    if ref["niter"] <= 2000:
                        assert st.status == 0 and st.fin_res < ref["tol"]
                    res += [x, r, st.niter]
        out[blk] = res
    assert np.array_equal(out[1][0], O.prec_form(s.n, s.row, s.col, s.dia, s.val, 2))
    assert np.array_equal(out[1][1], O.prec_solve(s.n, s.row, s.col, s.dia, s.val, 2, b))
    for a, c in zip(out[1], out[0]):
        assert np.array_equal(a, c)


def test_profile_prec_stamps_every_level_launch(gpu):
    """tfs_profile_prec stamps one DIC application's launches in order:
    forward levels ascending, the one-block tail, backward levels
    descending, each with a start before its end; the stamps do not change
    the application's result (Prec_Solve still equals the oracle)."""
    from tflows.lib import TFS_OPT_DIC_BLOCK
    s = system(POISSON, 40, 40, 40)
    b = np.random.default_rng(2).uniform(-1, 1, s.n)
    with Solver(s.matrix(), options={TFS_OPT_DIC_BLOCK: 0}) as sol:
        prof = sol.profile_prec(s.val, TFS_FP64)
        assert np.array_equal(sol.prec_solve(s.val, 2, b), O.prec_solve(s.n, s.row, s.col, s.dia, s.val, 2, b))
        nl = sol.stats()["n_levels"]
    kinds = [p["launch"] for p in prof]
    fwd = [int(k.split()[1]) for k in kinds if k.startswith("fwd")]
    bwd = [int(k.split()[1]) for k in kinds if k.startswith("bwd")]
    assert fwd == sorted(fwd) and fwd[0] == 0 and bwd == sorted(bwd, reverse=True) and bwd[-1] == 0
    assert kinds.count("tail") == 1 and kinds.index("tail") == len(fwd)
    assert len(fwd) < nl
    for p in prof:
        assert 0.0 <= p["start_us"] <= p["end_us"], p


def test_one_block_dic_not_used_on_wide_levels(gpu):
    """With the benchmark's random numbering a 24^3 system has 15 levels of
    up to 2074 rows: the ring of level slots does not fit beside the vector,
    so the level kernels run whatever TFS_OPT_DIC_BLOCK says."""
    s = system(POISSON, 24, 24, 24)
    b = np.random.default_rng(1).uniform(-1, 1, s.n)
    with Solver(s.matrix()) as sol:
        z = sol.prec_solve(s.val, 2, b)
        assert sol.stats()["dic_kernel"] == 0
    assert np.array_equal(z, O.prec_solve(s.n, s.row, s.col, s.dia, s.val, 2, b))


@pytest.mark.parametrize("launch", [0, 1])
def test_l2_window_changes_no_result(launch, gpu):
    """The column indices marked persisting in L2 (TFS_OPT_L2_WINDOW = 1,
    the default) change where the cache keeps them, not what any kernel
    computes: DIC-CG and diagonal CGS solves in both arithmetics, in the
    CUDA graph and launched eagerly, bitwise equal to TFS_OPT_L2_WINDOW = 0."""
    from tflows.lib import TFS_OPT_L2_WINDOW, TFS_OPT_LAUNCH
    s = system(POISSON, 24, 24, 24)
    tol = 1e-8 * float(np.linalg.norm(s.b))
    out = {}
    for win in (1, 0):
        res = []
        for mode in (TFS_FP64, TFS_MIXED):
            with Solver(s.matrix(), precision=mode, options={TFS_OPT_L2_WINDOW: win, TFS_OPT_LAUNCH: launch}) as sol:
                for method, prec in ((TFS_CG, 2), (TFS_CGS, 1)):
                    x, r = np.zeros(s.n), s.b.copy()
                    st = sol.solve(method, s.val, x, r, prec, 2000, tol)
                    assert st.status == 0
                    res += [x, r, st.niter]
        out[win] = res
    for a, c in zip(out[1], out[0]):
        assert np.array_equal(a, c)
