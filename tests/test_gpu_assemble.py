"""Device-side assembly through the face -> entry map (Matrix_Type%pos)
against the oracle's face loops, bitwise, and a solve on the assembled
matrix against the oracle."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import SOL_REL, iter_ok, rel_l2, system
from oracle import tfs_oracle as O
from tflows import TFS_CG, TFS_BICG, Matrix_Type, Solver
from tflows.lib import TfsError
from tflows.synth import CONVDIFF, POISSON

pytestmark = pytest.mark.gpu


def mesh_with_boundary(kind, nx, ny, nz, seed=5):
    """Interior faces of a synthetic mesh plus one boundary face for a
    random third of the cells, interleaved with the interior faces."""
    s = system(kind, nx, ny, nz)
    rng = np.random.default_rng(seed)
    cells = rng.choice(s.n, size=s.n // 3, replace=False) + 1
    bnd = np.stack([cells, -np.arange(1, cells.size + 1)], axis=1).astype(np.int32)
    faces = np.concatenate([s.faces_c, bnd])
    faces = faces[rng.permutation(len(faces))]
    return s, np.ascontiguousarray(faces, np.int32)


@pytest.mark.parametrize("kind", [POISSON, CONVDIFF])
def test_assemble_faces_bitwise(kind, gpu):
    s, faces = mesh_with_boundary(kind, 14, 12, 11)
    row, col, dia, mir, pos = O.topology(s.n, faces)
    nf = len(faces)
    rng = np.random.default_rng(7)
    a12 = rng.uniform(0.1, 2.0, nf)
    a21 = rng.uniform(0.1, 2.0, nf)
    bnd = faces[:, 1] <= 0
    d12 = a12.copy()
    d12[bnd & (rng.uniform(size=nf) < 0.4)] = 0.0      # boundary types that add nothing
    cell = rng.uniform(0.0, 1.0, s.n)
    val0 = np.zeros(len(col))
    want = O.assemble_faces(s.n, faces.reshape(-1), pos.reshape(-1), dia, a12, a21, d12, a21, cell, val0)
    A = Matrix_Type(s.n, row, col, dia, want.copy())
    with Solver(A) as sol:
        sol.faces_register(faces, pos)
        got = sol.assemble(a12, a21, d12, a21, cell)
        assert np.array_equal(got, want)
        # starting from non-zero values (NewUVW.f90 accumulates into A%val)
        start = rng.uniform(-1, 1, len(col))
        want2 = O.assemble_faces(s.n, faces.reshape(-1), pos.reshape(-1), dia, a12, a21, d12, a21, None,
                                 start)
        assert np.array_equal(sol.assemble(a12, a21, d12, a21, None, start), want2)


def test_assembled_matrix_solves(gpu):
    """A diagonally dominant matrix assembled on the device (pressure-like:
    off12 = off21 = dia12 = dia21) solves to the oracle's answer."""
    s, faces = mesh_with_boundary(POISSON, 16, 15, 14)
    row, col, dia, mir, pos = O.topology(s.n, faces)
    nf = len(faces)
    rng = np.random.default_rng(11)
    a = rng.uniform(0.5, 1.5, nf)
    cell = np.full(s.n, 1e-3)
    A = Matrix_Type(s.n, row, col, dia, np.zeros(len(col)))
    with Solver(A) as sol:
        sol.faces_register(faces, pos)
        val = sol.assemble(a, a, a, a, cell)
        b = rng.uniform(-1, 1, s.n)
        tol = 1e-8 * np.linalg.norm(b)
        xo, ro = np.zeros(s.n), b.copy()
        it, ini, fin = O.solve(TFS_CG, s.n, row, col, dia, val, xo, ro, 2, 2000, tol)
        x, r = np.zeros(s.n), b.copy()
        res = sol.solve(TFS_CG, val, x, r, 2, 2000, tol)
        assert res.status == 0 and iter_ok(res.niter, it) and rel_l2(x, xo) <= SOL_REL


def test_faces_register_rejects_mismatch(gpu):
    s, faces = mesh_with_boundary(POISSON, 6, 6, 6)
    row, col, dia, mir, pos = O.topology(s.n, faces)
    A = Matrix_Type(s.n, row, col, dia, np.zeros(len(col)))
    with Solver(A) as sol:
        bad = pos.copy()
        k = int(np.nonzero(faces[:, 1] > 0)[0][0])
        bad[k, 0] = dia[faces[k, 0] - 1]          # points at the diagonal
        with pytest.raises(TfsError):
            sol.faces_register(faces, bad)
        bad2 = faces.copy()
        bad2[0, 0] = s.n + 5
        with pytest.raises(TfsError):
            sol.faces_register(bad2, pos)
        with pytest.raises(TfsError):
            sol.assemble(np.zeros(len(faces)), np.zeros(len(faces)), np.zeros(len(faces)),
                         np.zeros(len(faces)))
