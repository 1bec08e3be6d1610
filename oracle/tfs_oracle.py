"""ctypes wrapper of the oracle library (oracle/tfs_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by the CPU-baseline leg of bench.py, always as the checker.  It restates the
reference's sequential solver (Sources/Process/Solvers_Mod/*.f90) on the CPU;
the GPU library never uses it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "tfs_oracle.c"
LIB = HERE / "_build" / "libtfs_oracle.so"

_i, _d = C.POINTER(C.c_int32), C.POINTER(C.c_double)
_lib = None


def build(force: bool = False) -> Path:
    if force or not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        LIB.parent.mkdir(exist_ok=True)
        subprocess.run(["gcc", "-O3", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
                        "-shared", "-o", str(LIB), str(SRC), "-lm"], check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        L = C.CDLL(str(build()))
        L.tfo_topology_count.restype = C.c_int
        L.tfo_topology_count.argtypes = [C.c_int, C.c_int, _i]
        L.tfo_topology_fill.restype = None
        L.tfo_topology_fill.argtypes = [C.c_int, C.c_int, _i, _i, _i, _i, _i, _i]
        L.tfo_prec_form.argtypes = [C.c_int, _i, _i, _i, _d, C.c_int, _d]
        L.tfo_prec_solve.argtypes = [C.c_int, _i, _i, _i, _d, _d, _d, _d, C.c_int]
        L.tfo_residual.argtypes = [C.c_int, _i, _i, _d, _d, _d]
        L.tfo_spmv.argtypes = [C.c_int, _i, _i, _d, _d, _d]
        for name in ("tfo_cg", "tfo_bicg", "tfo_cgs"):
            getattr(L, name).argtypes = [C.c_int, _i, _i, _i, _d, _d, _d, C.c_int, _i, C.c_double, _d, _d]
        L.tfo_solve.argtypes = [C.c_int, C.c_int, _i, _i, _i, _d, _d, _d, C.c_int, _i, C.c_double, _d, _d]
        L.tfo_assemble_faces.restype = None
        L.tfo_assemble_faces.argtypes = [C.c_int, C.c_int, _i, _i, _i, _d, _d, _d, _d, _d, _d]
        _lib = L
    return _lib


def _pi(a):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_i)


def _pd(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_d)


def topology(n_cells: int, faces_c: np.ndarray):
    """Matrix_Mod_Topology (Topology.f90:2-127): row, col, dia, mir, pos."""
    f = np.ascontiguousarray(faces_c, np.int32).reshape(-1)
    nf = f.size // 2
    nnz = lib().tfo_topology_count(n_cells, nf, _pi(f))
    row = np.zeros(n_cells + 1, np.int32)
    col = np.zeros(nnz + 1, np.int32)     # the reference's padding slot
    dia = np.zeros(n_cells, np.int32)
    mir = np.zeros(nnz + 1, np.int32)
    pos = np.zeros(2 * nf, np.int32)
    lib().tfo_topology_fill(n_cells, nf, _pi(f), _pi(row), _pi(col), _pi(dia), _pi(mir), _pi(pos))
    return row, col[:nnz].copy(), dia, mir[:nnz].copy(), pos.reshape(-1, 2)


def prec_form(n, row, col, dia, val, prec):
    d = np.zeros(n)
    lib().tfo_prec_form(n, _pi(row), _pi(col), _pi(dia), _pd(val), prec, _pd(d))
    return d


def prec_solve(n, row, col, dia, val, prec, b):
    d = prec_form(n, row, col, dia, val, prec)
    x = np.zeros(n)
    lib().tfo_prec_solve(n, _pi(row), _pi(col), _pi(dia), _pd(val), _pd(d), _pd(x),
                         _pd(np.ascontiguousarray(b, np.float64)), prec)
    return x


def residual(n, row, col, val, x, r1):
    lib().tfo_residual(n, _pi(row), _pi(col), _pd(val), _pd(x), _pd(r1))


def spmv(n, row, col, val, p):
    q = np.zeros(n)
    lib().tfo_spmv(n, _pi(row), _pi(col), _pd(val), _pd(np.ascontiguousarray(p, np.float64)), _pd(q))
    return q


def solve(method, n, row, col, dia, val, x, r1, prec, niter, tol, ini_res=0.0):
    """Cg / Bicg / Cgs (method 0 / 1 / 2); x and r1 updated in place.
    Returns (niter, ini_res, fin_res) as the Fortran writes them back."""
    it, ini, fin = C.c_int32(niter), C.c_double(ini_res), C.c_double(0.0)
    lib().tfo_solve(method, n, _pi(row), _pi(col), _pi(dia), _pd(val), _pd(x), _pd(r1), prec,
                    C.byref(it), tol, C.byref(ini), C.byref(fin))
    return it.value, ini.value, fin.value


def assemble_faces(n_cells, faces_c, pos, dia, off12, off21, dia12, dia21, cell, val0):
    """Values from per-face coefficients (the reference's face loops);
    returns a new array starting from val0."""
    val = np.array(val0, dtype=np.float64)
    n_faces = len(faces_c) // 2
    cellp = _pd(np.ascontiguousarray(cell, dtype=np.float64)) if cell is not None else None
    lib().tfo_assemble_faces(n_cells, n_faces, _pi(np.ascontiguousarray(faces_c, dtype=np.int32)),
                             _pi(np.ascontiguousarray(pos, dtype=np.int32)),
                             _pi(np.ascontiguousarray(dia, dtype=np.int32)),
                             _pd(np.ascontiguousarray(off12, dtype=np.float64)),
                             _pd(np.ascontiguousarray(off21, dtype=np.float64)),
                             _pd(np.ascontiguousarray(dia12, dtype=np.float64)),
                             _pd(np.ascontiguousarray(dia21, dtype=np.float64)), cellp, _pd(val))
    return val
