"""Batches of independent systems solved by one persistent cluster kernel
(tfs_batch_* in include/tfs_solver.h)."""
from __future__ import annotations

import ctypes as C
from typing import NamedTuple, Sequence

import numpy as np

from .lib import TFS_ERR_NONFINITE, TFS_FP64, TFS_OK, TfsError, check, last_error, load_library
from .solvers_mod import Solver

_dbl, _i32 = C.c_double, C.c_int32


class BatchResult(NamedTuple):
    niter: np.ndarray
    ini_res: np.ndarray
    fin_res: np.ndarray
    status: np.ndarray
    ms: float


def _ptr_array(ptrs):
    arr = (C.c_void_p * len(ptrs))()
    for k, p in enumerate(ptrs):
        arr[k] = p
    return arr


class Batch:
    """A fixed set of registered systems (Solver objects) solved together."""

    def __init__(self, solvers: Sequence[Solver], cluster: int = 8, threads: int = 256):
        self.lib = load_library()
        self.solvers = list(solvers)
        hs = _ptr_array([s.h.value for s in self.solvers])
        b = C.c_void_p()
        check(self.lib.tfs_batch_create(len(self.solvers), hs, C.byref(b)), "tfs_batch_create")
        self.b = b
        self.configure(cluster, threads)

    def configure(self, cluster: int, threads: int) -> None:
        check(self.lib.tfs_batch_configure(self.b, cluster, threads), "tfs_batch_configure")
        self.cluster, self.threads = cluster, threads

    def close(self) -> None:
        if self.b:
            self.lib.tfs_batch_release(self.b)
            self.b = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _outputs(self, niter, tol, ini_res):
        n = len(self.solvers)
        it = np.ascontiguousarray(np.broadcast_to(np.asarray(niter, np.int32), (n,)))
        tl = np.ascontiguousarray(np.broadcast_to(np.asarray(tol, np.float64), (n,)))
        ini = np.ascontiguousarray(np.broadcast_to(np.asarray(ini_res, np.float64), (n,))).copy()
        return it, tl, np.zeros(n, np.int32), ini, np.zeros(n), np.zeros(n, np.int32)

    def _finish(self, st, it_out, ini, fin, status, where):
        if st not in (TFS_OK, TFS_ERR_NONFINITE):
            raise TfsError(st, where, last_error())
        ms = _dbl()
        self.lib.tfs_batch_last_ms(self.b, C.byref(ms))
        return BatchResult(it_out, ini, fin, status, ms.value)

    def solve(self, method: int, prec: int, vals, xs, r1s, niter, tol, mode: int = TFS_FP64,
              ini_res=0.0) -> BatchResult:
        """Host arrays per system (x and r1 updated in place)."""
        it, tl, it_out, ini, fin, status = self._outputs(niter, tol, ini_res)
        for a, s in zip(vals, self.solvers):
            assert a.dtype == np.float64 and a.flags.c_contiguous and a.shape == (s.nnz,)
        for a, s in zip(list(xs) + list(r1s), self.solvers + self.solvers):
            assert a.dtype == np.float64 and a.flags.c_contiguous and a.shape == (s.n,)
        st = self.lib.tfs_batch_solve(
            self.b, method, prec, mode, _ptr_array([a.ctypes.data for a in vals]),
            _ptr_array([a.ctypes.data for a in xs]), _ptr_array([a.ctypes.data for a in r1s]),
            it.ctypes.data_as(C.POINTER(_i32)), tl.ctypes.data_as(C.POINTER(_dbl)),
            it_out.ctypes.data_as(C.POINTER(_i32)), ini.ctypes.data_as(C.POINTER(_dbl)),
            fin.ctypes.data_as(C.POINTER(_dbl)), status.ctypes.data_as(C.POINTER(_i32)))
        return self._finish(st, it_out, ini, fin, status, "tfs_batch_solve")

    def solve_device(self, method: int, prec: int, d_vals, d_xs, d_r1s, niter, tol,
                     mode: int = TFS_FP64, ini_res=0.0) -> BatchResult:
        """Device pointers per system (natural order)."""
        it, tl, it_out, ini, fin, status = self._outputs(niter, tol, ini_res)
        st = self.lib.tfs_batch_solve_device(
            self.b, method, prec, mode, _ptr_array(d_vals), _ptr_array(d_xs), _ptr_array(d_r1s),
            it.ctypes.data_as(C.POINTER(_i32)), tl.ctypes.data_as(C.POINTER(_dbl)),
            it_out.ctypes.data_as(C.POINTER(_i32)), ini.ctypes.data_as(C.POINTER(_dbl)),
            fin.ctypes.data_as(C.POINTER(_dbl)), status.ctypes.data_as(C.POINTER(_i32)))
        return self._finish(st, it_out, ini, fin, status, "tfs_batch_solve_device")
