"""Solvers_Mod of T-FlowS (Sources/Process/Solvers_Mod.f90) on the GB300.

``Cg``, ``Bicg`` and ``Cgs`` keep the argument meaning of the Fortran
subroutines (Cg.f90:2-4): ``x`` and ``r1`` are updated in place (r1 enters as
b and leaves as the final residual), ``tol`` is absolute, and the call returns
what the Fortran writes back into ``niter``, ``ini_res`` and ``fin_res``.
``ini_res`` is returned unchanged when ||b|| < tol, as in the reference.
All work runs in libtfs_gb300.so on the GPU.
"""
from __future__ import annotations

import ctypes as C
from typing import NamedTuple

import numpy as np

from .lib import (TFS_BICG, TFS_CG, TFS_CGS, TFS_ERR_NONFINITE, TFS_FP64, TFS_OK, TfsError,
                  check, last_error, load_library, tfs_stats)
from .matrix_mod import Matrix_Type, ptr

# SpMV kernels of the CG iterations (tfs_stats.spmv_kernel, tfs_tuning.spmv_kernel).
SPMV_KERNELS = {0: "direct", 1: "pipe", 2: "bulk", 3: "async"}

_dbl, _i32 = C.c_double, C.c_int32


class SolveResult(NamedTuple):
    niter: int
    ini_res: float
    fin_res: float
    status: int


def _vec(a: np.ndarray, n: int, name: str) -> np.ndarray:
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags.c_contiguous \
            or a.shape != (n,):
        raise ValueError(f"{name} must be a contiguous float64 array of length {n}")
    return a


class Solver:
    """A registered topology (one tfs_handle): device layout, DIC level
    schedule and work vectors stay resident between solves."""

    def __init__(self, A: Matrix_Type, precision: int = TFS_FP64, options: dict | None = None):
        """options: {TFS_OPT_*: value} (include/tfs_solver.h), set before the
        first solve."""
        self.lib = load_library()
        self.n, self.nnz = A.n_cells, A.nnz
        self._row, self._col, self._dia = A.row, A.col, A.dia
        h = C.c_void_p()
        check(self.lib.tfs_topology_register(self.n, self.nnz, ptr(A.row, _i32), ptr(A.col, _i32),
                                             ptr(A.dia, _i32), C.byref(h)), "tfs_topology_register")
        self.h = h
        self.set_precision(precision)
        for opt, value in (options or {}).items():
            self.set_option(opt, value)

    def set_precision(self, mode: int) -> None:
        check(self.lib.tfs_set_precision(self.h, mode), "tfs_set_precision")
        self.precision = mode

    def set_option(self, option: int, value: int) -> None:
        check(self.lib.tfs_set_option(self.h, option, value), "tfs_set_option")

    def get_option(self, option: int) -> int:
        v = C.c_int(0)
        check(self.lib.tfs_get_option(self.h, option, C.byref(v)), "tfs_get_option")
        return v.value

    def close(self) -> None:
        if self.h:
            self.lib.tfs_release(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve(self, method: int, val: np.ndarray, x: np.ndarray, r1: np.ndarray, prec: int,
              niter: int, tol: float, ini_res: float = 0.0) -> SolveResult:
        val = _vec(val, self.nnz, "val")
        x, r1 = _vec(x, self.n, "x"), _vec(r1, self.n, "r1")
        it, ini, fin = _i32(niter), _dbl(ini_res), _dbl(0.0)
        st = self.lib.tfs_solve(method, self.h, self.n, self.nnz, ptr(self._row, _i32),
                                ptr(self._col, _i32), ptr(self._dia, _i32), ptr(val, _dbl),
                                ptr(x, _dbl), ptr(r1, _dbl), prec, C.byref(it), tol,
                                C.byref(ini), C.byref(fin))
        if st not in (TFS_OK, TFS_ERR_NONFINITE):
            raise TfsError(st, "tfs_solve", last_error())
        return SolveResult(it.value, ini.value, fin.value, st)

    def solve_device(self, method: int, d_val: int, d_x: int, d_r1: int, prec: int, niter: int,
                     tol: float, ini_res: float = 0.0) -> SolveResult:
        """Solve on device arrays given as raw CUDA pointers (natural order)."""
        it, ini, fin = _i32(niter), _dbl(ini_res), _dbl(0.0)
        st = self.lib.tfs_solve_device(method, self.h, C.c_void_p(d_val), C.c_void_p(d_x),
                                       C.c_void_p(d_r1), prec, C.byref(it), tol, C.byref(ini),
                                       C.byref(fin))
        if st not in (TFS_OK, TFS_ERR_NONFINITE):
            raise TfsError(st, "tfs_solve_device", last_error())
        return SolveResult(it.value, ini.value, fin.value, st)

    def spmv(self, val: np.ndarray, p: np.ndarray) -> np.ndarray:
        q = np.empty(self.n)
        check(self.lib.tfs_spmv(self.h, ptr(_vec(val, self.nnz, "val"), _dbl),
                                ptr(_vec(p, self.n, "p"), _dbl), ptr(q, _dbl)), "tfs_spmv")
        return q

    def residual(self, val: np.ndarray, x: np.ndarray, r1: np.ndarray) -> None:
        check(self.lib.tfs_residual(self.h, ptr(_vec(val, self.nnz, "val"), _dbl),
                                    ptr(_vec(x, self.n, "x"), _dbl),
                                    ptr(_vec(r1, self.n, "r1"), _dbl)), "tfs_residual")

    def prec_form(self, val: np.ndarray, prec: int) -> np.ndarray:
        d = np.empty(self.n)
        check(self.lib.tfs_prec_form(self.h, ptr(_vec(val, self.nnz, "val"), _dbl), prec,
                                     ptr(d, _dbl)), "tfs_prec_form")
        return d

    def prec_solve(self, val: np.ndarray, prec: int, b: np.ndarray) -> np.ndarray:
        x = np.empty(self.n)
        check(self.lib.tfs_prec_solve(self.h, ptr(_vec(val, self.nnz, "val"), _dbl), prec,
                                      ptr(_vec(b, self.n, "b"), _dbl), ptr(x, _dbl)),
              "tfs_prec_solve")
        return x

    def levels(self) -> np.ndarray:
        lv = np.empty(self.n, np.int32)
        check(self.lib.tfs_get_levels(self.h, ptr(lv, _i32)), "tfs_get_levels")
        return lv

    def stats(self) -> dict:
        s = tfs_stats()
        check(self.lib.tfs_get_stats(self.h, C.byref(s)), "tfs_get_stats")
        return {k: getattr(s, k) for k, _ in tfs_stats._fields_}

    def time_spmv(self, val: np.ndarray, mode: int = TFS_FP64, reps: int = 20) -> float:
        ms = _dbl(0.0)
        check(self.lib.tfs_time_spmv(self.h, ptr(_vec(val, self.nnz, "val"), _dbl), mode, reps,
                                     C.byref(ms)), "tfs_time_spmv")
        return ms.value

    def faces_register(self, faces_c: np.ndarray, pos: np.ndarray) -> None:
        """Attach the mesh faces (n_faces x 2 cells, 1-based, c2 <= 0 on the
        boundary) and Matrix_Type%pos (n_faces x 2) for device assembly."""
        fc = np.ascontiguousarray(faces_c, dtype=np.int32).reshape(-1)
        ps = np.ascontiguousarray(pos, dtype=np.int32).reshape(-1)
        if fc.size != ps.size or fc.size % 2:
            raise ValueError("faces_c and pos must both be n_faces x 2")
        check(self.lib.tfs_faces_register(self.h, fc.size // 2, ptr(fc, _i32), ptr(ps, _i32)),
              "tfs_faces_register")
        self.n_faces = fc.size // 2

    def assemble(self, off12: np.ndarray, off21: np.ndarray, dia12: np.ndarray, dia21: np.ndarray,
                 cell: np.ndarray | None = None, val0: np.ndarray | None = None) -> np.ndarray:
        """Matrix values from per-face coefficients, assembled on the device
        (tfs_assemble_faces_device); host arrays in, CSR values out."""
        nf = getattr(self, "n_faces", None)
        if nf is None:   # no faces registered: the library reports it
            check(self.lib.tfs_assemble_faces_device(self.h, None, None, None, None, None, None),
                  "tfs_assemble_faces_device")
        arrays = [np.ascontiguousarray(a, dtype=np.float64) for a in (off12, off21, dia12, dia21)]
        if any(a.shape != (nf,) for a in arrays):
            raise ValueError(f"face coefficients must have length {nf}")
        val = np.zeros(self.nnz) if val0 is None else np.array(val0, dtype=np.float64)
        host = arrays + ([np.ascontiguousarray(cell, dtype=np.float64)] if cell is not None else []) + [val]
        dev = []
        try:
            for a in host:
                q = C.c_void_p()
                check(self.lib.tfs_device_alloc(max(a.nbytes, 8), C.byref(q)), "tfs_device_alloc")
                dev.append(q.value)
                check(self.lib.tfs_copy(self.h, C.c_void_p(q.value), a.ctypes.data_as(C.c_void_p), a.nbytes),
                      "tfs_copy")
            d_cell = C.c_void_p(dev[4]) if cell is not None else None
            check(self.lib.tfs_assemble_faces_device(self.h, *(C.c_void_p(d) for d in dev[:4]), d_cell,
                                                     C.c_void_p(dev[-1])), "tfs_assemble_faces_device")
            check(self.lib.tfs_copy(self.h, val.ctypes.data_as(C.c_void_p), C.c_void_p(dev[-1]), val.nbytes),
                  "tfs_copy")
            check(self.lib.tfs_sync(self.h), "tfs_sync")
        finally:
            for d in dev:
                self.lib.tfs_device_free(C.c_void_p(d))
        return val

    def autotune(self, val: np.ndarray, mode: int = TFS_FP64, prec: int = 2, reps: int = 10) -> dict:
        """Time the candidate launch shapes on this system and keep the
        fastest (tfs_autotune); returns the choice and the timings."""
        from .lib import tfs_tuning
        t = tfs_tuning()
        check(self.lib.tfs_autotune(self.h, ptr(_vec(val, self.nnz, "val"), _dbl), mode, prec, reps,
                                    C.byref(t)), "tfs_autotune")
        return {"level_tpb": t.level_tpb, "spmv_chunks": t.spmv_chunks,
                "spmv_kernel": SPMV_KERNELS.get(t.spmv_kernel, str(t.spmv_kernel)),
                "prec_ms": {c: t.prec_ms[k] for k, c in enumerate((128, 256, 512, 1024))},
                "spmv_ms": {"direct_sm8": t.spmv_ms[0], "direct_chunks": t.spmv_ms[1],
                            "pipe_sm8": t.spmv_pipe_ms[0], "pipe_chunks": t.spmv_pipe_ms[1]}}

    def profile_prec(self, val: np.ndarray, mode: int = TFS_FP64) -> list[dict]:
        """Device stamps of one DIC application's level launches
        (tfs_profile_prec): per launch, when its blocks passed their
        dependency wait and when they had finished (us)."""
        self.levels()                       # builds the level layout first
        m = 4 * max(1, self.stats()["n_levels"]) + 8
        st, en = np.zeros(m), np.zeros(m)
        kd, n = np.zeros(m, np.int32), _i32(0)
        check(self.lib.tfs_profile_prec(self.h, ptr(_vec(val, self.nnz, "val"), _dbl), mode, m, ptr(st, _dbl),
                                        ptr(en, _dbl), ptr(kd, _i32), C.byref(n)), "tfs_profile_prec")
        out = []
        for k in range(n.value):
            kind = int(kd[k])
            what = "tail" if kind == 1 << 20 else (f"fwd {kind}" if kind >= 0 else f"bwd {-1 - kind}")
            out.append({"launch": what, "start_us": float(st[k]), "end_us": float(en[k])})
        return out

    def time_prec(self, val: np.ndarray, mode: int = TFS_FP64, reps: int = 20) -> float:
        """Milliseconds per DIC preconditioner application (both sweeps)."""
        ms = _dbl(0.0)
        check(self.lib.tfs_time_prec(self.h, ptr(_vec(val, self.nnz, "val"), _dbl), mode, reps,
                                     C.byref(ms)), "tfs_time_prec")
        return ms.value


def _solver_of(A: Matrix_Type) -> Solver:
    if A._solver is None:
        A._solver = Solver(A)
    return A._solver


def _call(method: int, A: Matrix_Type, x, r1, prec, niter, tol, ini_res):
    res = _solver_of(A).solve(method, A.val, x, r1, prec, niter, tol, ini_res)
    return res.niter, res.ini_res, res.fin_res


def Cg(A: Matrix_Type, x: np.ndarray, r1: np.ndarray, prec: int, niter: int, tol: float,
       ini_res: float = 0.0):
    """Preconditioned CG (Cg.f90:2-183). Returns (niter, ini_res, fin_res)."""
    return _call(TFS_CG, A, x, r1, prec, niter, tol, ini_res)


def Bicg(A: Matrix_Type, x: np.ndarray, r1: np.ndarray, prec: int, niter: int, tol: float,
         ini_res: float = 0.0):
    """Preconditioned BiCG, A (not A^T) on the shadow system (Bicg.f90:2-196)."""
    return _call(TFS_BICG, A, x, r1, prec, niter, tol, ini_res)


def Cgs(A: Matrix_Type, x: np.ndarray, r1: np.ndarray, prec: int, niter: int, tol: float,
        ini_res: float = 0.0):
    """Preconditioned CGS (Cgs.f90:2-232)."""
    return _call(TFS_CGS, A, x, r1, prec, niter, tol, ini_res)


def Prec_Form(A: Matrix_Type, prec: int) -> np.ndarray:
    """D % val(D % dia(i)) for i = 1..n (Prec_Form.f90:2-51)."""
    return _solver_of(A).prec_form(A.val, prec)


def Prec_Solve(A: Matrix_Type, b: np.ndarray, prec: int) -> np.ndarray:
    """x = M^-1 b with M formed from A (Prec_Form.f90 then Prec_Solve.f90)."""
    return _solver_of(A).prec_solve(A.val, prec, b)


def Residual(A: Matrix_Type, x: np.ndarray, r1: np.ndarray) -> None:
    """r1 <- r1 - A x in place (Residual.f90:2-40)."""
    _solver_of(A).residual(A.val, x, r1)


def spmv(A: Matrix_Type, p: np.ndarray) -> np.ndarray:
    """q = A p (the product loop of Cg.f90:128-134)."""
    return _solver_of(A).spmv(A.val, p)
