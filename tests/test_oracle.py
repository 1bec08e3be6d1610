"""CPU tests of the oracle: known answers, the reference's documented CSR
example, the reference's output semantics, and the golden fixtures."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

from oracle import tfs_oracle as O

GOLD = Path(__file__).resolve().parent / "golden"
TINY = 1.e-30


@pytest.fixture(scope="module")
def kat():
    return dict(np.load(GOLD / "matrix_mod_example.npz"))


# -------------------------------------------- Matrix_Mod.f90:15-34 example

def test_layout_example_dense(kat):
    """val/col/row/dia of Matrix_Mod.f90:30-34 describe the matrix drawn at
    Matrix_Mod.f90:23-26 (row gains its n+1 terminator 13)."""
    n = 4
    a = np.zeros((n, n))
    for i in range(n):
        for j in range(kat["row"][i] - 1, kat["row"][i + 1] - 1):
            a[i, kat["col"][j] - 1] = kat["val"][j]
    assert np.array_equal(a, kat["dense"])
    for i in range(n):
        assert kat["col"][kat["dia"][i] - 1] == i + 1
    # the documented dia (Matrix_Mod.f90:34) points row 3 at column 4
    doc = kat["dia_documented"]
    assert [int(kat["col"][doc[i] - 1]) for i in range(n)] == [1, 2, 4, 4]


def test_layout_example_spmv_residual(kat):
    p = np.array([1.0, -2.0, 0.5, 3.0])
    q = O.spmv(4, kat["row"], kat["col"], kat["val"], p)
    assert np.array_equal(q, kat["dense"] @ p)        # small integers: exact
    r = np.array([1.0, 2.0, 3.0, 4.0])
    O.residual(4, kat["row"], kat["col"], kat["val"], p, r)
    assert np.array_equal(r, np.array([1.0, 2.0, 3.0, 4.0]) - kat["dense"] @ p)


def test_layout_example_prec_form(kat):
    d1 = O.prec_form(4, kat["row"], kat["col"], kat["dia"], kat["val"], 1)
    assert np.array_equal(d1, [10.0, 12.0, 99.0, 53.0])
    d0 = O.prec_form(4, kat["row"], kat["col"], kat["dia"], kat["val"], 0)
    assert np.array_equal(d0, np.ones(4))
    # DIC recurrence D_i = 1/(a_ii - sum_{lower} D_k a_ik a_ik), Prec_Form.f90:32-40
    D = [0.0] * 4
    D[0] = 1.0 / 10.0
    D[1] = 1.0 / (12.0 - D[0] * 2.0 * 2.0)
    D[2] = 1.0 / (99.0 - D[1] * 1.0 * 1.0)
    D[3] = 1.0 / ((53.0 - D[0] * -3.0 * -3.0) - D[1] * 11.0 * 11.0)
    d2 = O.prec_form(4, kat["row"], kat["col"], kat["dia"], kat["val"], 2)
    assert np.array_equal(d2, D)


def test_layout_example_prec_solve(kat):
    b = np.array([1.0, 2.0, 3.0, 4.0])
    D = O.prec_form(4, kat["row"], kat["col"], kat["dia"], kat["val"], 2)
    # forward (Prec_Solve.f90:46-53), scaling (:55-57), backward (:60-67)
    y = [0.0] * 4
    y[0] = b[0] * D[0]
    y[1] = (b[1] - 2.0 * y[0]) * D[1]
    y[2] = (b[2] - 1.0 * y[1]) * D[2]
    y[3] = ((b[3] - -3.0 * y[0]) - 11.0 * y[1]) * D[3]
    y = [y[i] / (D[i] + TINY) for i in range(4)]
    x = [0.0] * 4
    x[3] = y[3] * D[3]
    x[2] = (y[2] - 7.0 * x[3]) * D[2]
    x[1] = (y[1] - -1.0 * x[2]) * D[1]
    x[0] = ((y[0] - 4.0 * x[2]) - 5.0 * x[3]) * D[0]
    got = O.prec_solve(4, kat["row"], kat["col"], kat["dia"], kat["val"], 2, b)
    assert np.array_equal(got, x)
    got1 = O.prec_solve(4, kat["row"], kat["col"], kat["dia"], kat["val"], 1, b)
    assert np.array_equal(got1, b / np.array([10.0, 12.0, 99.0, 53.0]))


# ------------------------------------------------------ known answers

def csr_from_dense(a):
    n = a.shape[0]
    row, col, val, dia = [1], [], [], []
    for i in range(n):
        for j in range(n):
            if a[i, j] != 0 or i == j:
                if i == j:
                    dia.append(len(col) + 1)
                col.append(j + 1)
                val.append(a[i, j])
        row.append(len(col) + 1)
    return (np.array(row, np.int32), np.array(col, np.int32), np.array(dia, np.int32),
            np.array(val, np.float64))


def test_cg_2x2_two_iterations():
    """CG on an SPD 2x2 system terminates in n = 2 iterations."""
    row, col, dia, val = csr_from_dense(np.array([[4.0, 1.0], [1.0, 3.0]]))
    x, r = np.zeros(2), np.array([1.0, 2.0])
    it, ini, fin = O.solve(0, 2, row, col, dia, val, x, r, 0, 10, 1e-12)
    assert it == 2
    assert np.allclose(x, [1 / 11, 7 / 11], rtol=0, atol=1e-15)
    assert ini == pytest.approx(np.sqrt(5.0), rel=1e-15)


@pytest.mark.parametrize("method", [0, 1, 2])
def test_diagonal_system_one_iteration(method):
    d = np.array([2.0, 5.0, 0.25, 8.0, 3.0])
    row, col, dia, val = csr_from_dense(np.diag(d))
    b = np.array([1.0, -2.0, 3.0, 0.5, -1.5])
    x, r = np.zeros(5), b.copy()
    it, _, fin = O.solve(method, 5, row, col, dia, val, x, r, 1, 10, 1e-10)
    assert it == 1 and fin < 1e-10
    assert np.allclose(x, b / d, rtol=1e-15, atol=0)


@pytest.mark.parametrize("method,prec", [(0, 0), (0, 1), (0, 2), (1, 1), (2, 1), (2, 2)])
def test_1d_poisson_manufactured(method, prec):
    """Tridiagonal (-1, 2, -1) system with a manufactured x* (b = A x*): the
    solvers reach x* to the accuracy the conditioning allows."""
    n = 60
    a = 2 * np.eye(n) - np.eye(n, k=1) - np.eye(n, k=-1)
    t = np.arange(1, n + 1) / (n + 1)
    xs = t * (1 - t) * np.exp(t) + 0.1 * np.cos(7 * t)
    b = a @ xs
    row, col, dia, val = csr_from_dense(a)
    x, r = np.zeros(n), b.copy()
    it, ini, fin = O.solve(method, n, row, col, dia, val, x, r, prec, 500, 1e-12 * np.linalg.norm(b))
    assert fin < 1e-12 * np.linalg.norm(b)
    assert np.linalg.norm(x - xs) / np.linalg.norm(xs) < 1e-9
    if method == 0 and prec == 0:
        assert it <= n + 5          # CG terminates in <= n steps, up to rounding


def test_scipy_jacobi_cg_cross_check():
    """Independent sanity check: scipy's Jacobi-preconditioned CG (relative
    tolerance, different update order) lands near the oracle's solution."""
    sp = pytest.importorskip("scipy.sparse")
    spla = pytest.importorskip("scipy.sparse.linalg")
    from tflows import SynthSystem
    s = SynthSystem(0, 12, 11, 10)
    A = sp.csr_matrix((s.val, s.col - 1, s.row - 1), shape=(s.n, s.n))
    x, r = np.zeros(s.n), s.b.copy()
    tol = 1e-10 * np.linalg.norm(s.b)
    O.solve(0, s.n, s.row, s.col, s.dia, s.val, x, r, 1, 5000, tol)
    M = sp.diags(1.0 / A.diagonal())
    xs, info = spla.cg(A, s.b, rtol=1e-12, M=M, maxiter=5000)
    assert info == 0
    assert np.linalg.norm(x - xs) / np.linalg.norm(xs) < 1e-7


def test_scipy_jacobi_cgs_cross_check():
    """Independent sanity check of the CGS restatement on a non-symmetric
    (upwind convection-diffusion) system: scipy's Jacobi-preconditioned CGS
    lands near the oracle's solution, and so does a dense solve."""
    sp = pytest.importorskip("scipy.sparse")
    spla = pytest.importorskip("scipy.sparse.linalg")
    from tflows import SynthSystem
    s = SynthSystem(1, 10, 9, 8)
    A = sp.csr_matrix((s.val, s.col - 1, s.row - 1), shape=(s.n, s.n))
    assert abs(A - A.T).max() > 0          # really non-symmetric
    x, r = np.zeros(s.n), s.b.copy()
    tol = 1e-11 * np.linalg.norm(s.b)
    it, _, fin = O.solve(2, s.n, s.row, s.col, s.dia, s.val, x, r, 1, 5000, tol)
    assert fin < tol and it <= 5000
    M = sp.diags(1.0 / A.diagonal())
    xs, info = spla.cgs(A, s.b, rtol=1e-13, M=M, maxiter=5000)
    assert info == 0
    xd = np.linalg.solve(A.toarray(), s.b)
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-8
    assert np.linalg.norm(x - xs) / np.linalg.norm(xs) < 1e-8


def _textbook(method, A, b, minv, k):
    """k iterations from x0 = 0 of the published preconditioned CG
    (Hestenes-Stiefel) or CGS (Sonneveld) recurrences, as Barrett et al.,
    Templates for the Solution of Linear Systems (SIAM 1994), state them,
    with the preconditioner applied by minv(v) = M^-1 v; numpy, independent
    of the oracle's code."""
    x = np.zeros_like(b)
    r = b.copy()
    rt = r.copy()
    rho_old = None
    p = q = None
    for _ in range(k):
        if method == 0:
            z = minv(r)
            rho = r @ z
            p = z if rho_old is None else z + (rho / rho_old) * p
            qv = A @ p
            alpha = rho / (p @ qv)
            x = x + alpha * p
            r = r - alpha * qv
        else:
            rho = rt @ r
            if rho_old is None:
                u = r.copy()
                p = u.copy()
            else:
                beta = rho / rho_old
                u = r + beta * q
                p = u + beta * (q + beta * p)
            vh = A @ minv(p)
            alpha = rho / (rt @ vh)
            q = u - alpha * vh
            uh = minv(u + q)
            x = x + alpha * uh
            r = r - alpha * (A @ uh)
        rho_old = rho
    return x


def _dic_inverse(A):
    """M^-1 of the diagonal incomplete Cholesky preconditioner written from
    its definition, independent of the oracle: A = L + diag(A) + U,
    D_i = 1 / (a_ii - sum_{k<i} D_k a_ik^2) over the stored lower entries of
    row i, M = (D^-1 + L) D (D^-1 + U); applied as two triangular solves
    (scipy) and a scaling."""
    from scipy.sparse import diags, tril, triu
    from scipy.sparse.linalg import spsolve_triangular
    A = A.tocsr()
    n = A.shape[0]
    d = np.zeros(n)
    for i in range(n):
        s = A[i, i]
        for jj in range(A.indptr[i], A.indptr[i + 1]):
            k = A.indices[jj]
            if k < i:
                s = s - d[k] * A.data[jj] * A.data[jj]
        d[i] = 1.0 / s
    lower = (diags(1.0 / d) + tril(A, k=-1)).tocsr()
    upper = (diags(1.0 / d) + triu(A, k=1)).tocsr()
    return lambda v: spsolve_triangular(upper, spsolve_triangular(lower, v, lower=True) / d, lower=False)


@pytest.mark.parametrize("method,kind,book", [(0, 0, 0), (1, 0, 0), (2, 1, 2)],
                         ids=["cg-poisson", "bicg-poisson", "cgs-convdiff"])
@pytest.mark.parametrize("prec", [0, 1, 2])
def test_iterates_follow_the_published_recurrence(method, kind, book, prec):
    """After each of the first iterations the oracle's x equals the iterate
    of the published recurrence (to rounding: the sums run in another
    order), so the restatement follows the algorithm step by step, not only
    to the same limit.  BiCG on a symmetric system with the shadow residual
    equal to the residual is CG (Bicg.f90 runs its second sequence with A
    itself), so it is held to the CG recurrence; a CG iterate on the
    non-symmetric system differs from the CGS one by 0.3-19%, which the
    tolerance separates by ten orders of magnitude."""
    sp = pytest.importorskip("scipy.sparse")
    from tflows import SynthSystem
    s = SynthSystem(kind, 7, 6, 5)
    A = sp.csr_matrix((s.val, s.col - 1, s.row - 1), shape=(s.n, s.n))
    minv = _dic_inverse(A) if prec == 2 else (lambda v, d=A.diagonal() if prec == 1 else 1.0: v / d)
    for k in range(1, 7):
        x, r = np.zeros(s.n), s.b.copy()
        O.solve(method, s.n, s.row, s.col, s.dia, s.val, x, r, prec, k, 1e-300)
        xt = _textbook(book, A, s.b, minv, k)
        assert np.linalg.norm(x - xt) <= 1e-11 * np.linalg.norm(xt), (k, np.linalg.norm(x - xt))


# ------------------------------------------------------ semantics

def _poisson(n=8):
    from tflows import SynthSystem
    return SynthSystem(0, n)


@pytest.mark.parametrize("method", [0, 1, 2])
def test_semantics_small_b(method):
    s = _poisson()
    b = s.b * 1e-9
    x, r = np.ones(s.n), b.copy()
    it, ini, fin = O.solve(method, s.n, s.row, s.col, s.dia, s.val, x, r, 1, 10, 1.0, ini_res=-3.0)
    assert it == 0 and ini == -3.0 and fin == pytest.approx(np.linalg.norm(b))
    assert np.array_equal(x, np.ones(s.n)) and np.array_equal(r, b)


@pytest.mark.parametrize("method", [0, 1, 2])
def test_semantics_limit_plus_one(method):
    s = _poisson()
    x, r = np.zeros(s.n), s.b.copy()
    it, ini, fin = O.solve(method, s.n, s.row, s.col, s.dia, s.val, x, r, 1, 5, 1e-30)
    assert it == 6 and fin > 1e-30
    x, r = np.zeros(s.n), s.b.copy()
    it, ini, fin = O.solve(method, s.n, s.row, s.col, s.dia, s.val, x, r, 1, 0, 1e-30)
    assert it == 1 and fin == ini


def test_semantics_r1_is_recursive_residual():
    """r1 leaves as the recursive residual, close to (not equal to) b - A x."""
    s = _poisson()
    x, r = np.zeros(s.n), s.b.copy()
    O.solve(0, s.n, s.row, s.col, s.dia, s.val, x, r, 1, 1000, 1e-8 * np.linalg.norm(s.b))
    rt = s.b.copy()
    O.residual(s.n, s.row, s.col, s.val, x, rt)
    assert np.linalg.norm(r - rt) < 1e-12 * np.linalg.norm(s.b)


# ------------------------------------------------------ golden fixtures

@pytest.mark.parametrize("path", sorted(GOLD.glob("solve_*.npz")), ids=lambda p: p.stem)
def test_golden_solves(path):
    g = np.load(path)
    n = g["dia"].size
    for method in (0, 1, 2):
        for prec in (0, 1, 2):
            key = f"m{method}p{prec}"
            x, r = np.zeros(n), g["b"].copy()
            it, ini, fin = O.solve(method, n, g["row"], g["col"], g["dia"], g["val"], x, r, prec,
                                   1000, float(g["tol"]))
            assert np.array_equal(x, g[key + "_x"]) and np.array_equal(r, g[key + "_r"]), key
            assert [it, ini, fin] == list(g[key + "_scal"]), key


def test_golden_topology():
    """The oracle's Topology.f90 restatement reproduces the fixtures' CSR."""
    for path in sorted(GOLD.glob("solve_*.npz")):
        g = np.load(path)
        row, col, dia, mir, pos = O.topology(g["dia"].size, g["faces_c"])
        assert np.array_equal(row, g["row"]) and np.array_equal(col, g["col"])
        assert np.array_equal(dia, g["dia"])
        # mirror of a mirror is the entry itself; pos points at (c1,c2),(c2,c1)
        assert np.array_equal(mir[mir - 1] , np.arange(1, col.size + 1))
        f = g["faces_c"]
        assert np.array_equal(col[pos[:, 0] - 1], f[:, 1]) and np.array_equal(col[pos[:, 1] - 1], f[:, 0])


@pytest.mark.parametrize("kind,dims", [(0, (6, 5, 4)), (1, (5, 5, 7))])
def test_topology_pattern_from_an_independent_construction(kind, dims):
    """The oracle's Topology.f90 restatement gives the sorted compressed-row
    pattern that scipy builds from the same faces (every cell's diagonal,
    both directions of every interior face), mir pairs (i, j) with (j, i)
    and dia points at the diagonal."""
    sp = pytest.importorskip("scipy.sparse")
    from tflows import SynthSystem
    s = SynthSystem(kind, *dims, seed=9, permute=True)
    f = s.faces_c
    inner = f[:, 1] > 0
    c1, c2 = f[inner, 0] - 1, f[inner, 1] - 1
    i = np.concatenate([np.arange(s.n), c1, c2])
    j = np.concatenate([np.arange(s.n), c2, c1])
    P = sp.csr_matrix((np.ones(i.size), (i, j)), shape=(s.n, s.n))
    P.sort_indices()
    row, col, dia, mir, pos = O.topology(s.n, f)
    assert np.array_equal(row - 1, P.indptr) and np.array_equal(col - 1, P.indices)
    rows_of = np.repeat(np.arange(1, s.n + 1), np.diff(row))
    assert np.array_equal(col[dia - 1], np.arange(1, s.n + 1))
    assert np.array_equal(rows_of[mir - 1], col) and np.array_equal(col[mir - 1], rows_of)


def test_assemble_faces_known_answer():
    """Face-loop assembly (NewUVW.f90:366-384, :500-505) on a three-cell
    chain with two boundary faces, against the matrix written out by hand."""
    faces = np.array([[1, 2], [2, 3], [1, -1], [3, -2]], np.int32)
    row, col, dia, mir, pos = O.topology(3, faces)
    off12 = np.array([1.5, 2.0, 0.0, 0.0])
    off21 = np.array([1.25, 2.5, 0.0, 0.0])
    dia12 = np.array([1.5, 2.0, 0.75, 0.0])     # face 4: a boundary type that adds nothing
    dia21 = np.array([1.25, 2.5, 0.0, 0.0])
    cell = np.array([0.125, 0.25, 0.5])
    val = O.assemble_faces(3, faces.reshape(-1), pos.reshape(-1), dia, off12, off21, dia12, dia21,
                           cell, np.zeros(len(col)))
    dense = np.zeros((3, 3))
    for i in range(3):
        for j in range(row[i] - 1, row[i + 1] - 1):
            dense[i, col[j] - 1] = val[j]
    want = np.array([[1.5 + 0.75 + 0.125, -1.5, 0.0],
                     [-1.25, 1.25 + 2.0 + 0.25, -2.0],
                     [0.0, -2.5, 2.5 + 0.5]])
    assert np.array_equal(dense, want)
