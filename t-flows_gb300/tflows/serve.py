"""Request loop for solves that arrive over time (tfs_server_* in
include/tfs_solver.h): continuous admission onto the GPU, device-resident
systems, a device-memory budget."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .lib import (TFS_ERR_TIMEOUT, TFS_FP64, TFS_OK, TfsError, check, last_error, load_library,
                  tfs_result, tfs_server_stats)
from .matrix_mod import ptr


class Server:
    def __init__(self, budget_bytes: int, max_inflight: int = 8, device: int = 0):
        self.lib = load_library()
        s = C.c_void_p()
        check(self.lib.tfs_server_create(device, int(budget_bytes), max_inflight, C.byref(s)),
              "tfs_server_create")
        self.s = s

    def close(self) -> None:
        if self.s:
            self.lib.tfs_server_destroy(self.s)
            self.s = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def add_system(self, n: int, row1: np.ndarray, col1: np.ndarray, dia1: np.ndarray) -> int:
        sid = C.c_int64()
        nnz = int(row1[-1]) - 1
        check(self.lib.tfs_server_add_system(self.s, n, nnz, ptr(row1, C.c_int32), ptr(col1, C.c_int32),
                                             ptr(dia1, C.c_int32), C.byref(sid)), "tfs_server_add_system")
        return sid.value

    def submit(self, sys_id: int, method: int, prec: int, d_val: int, d_x: int, d_r1: int,
               niter: int, tol: float, mode: int = TFS_FP64, d_b: int | None = None,
               x0_zero: bool = False) -> int:
        """Queue a solve; b from d_b (default: d_r1, in/out), x0 = 0 if x0_zero."""
        t = C.c_int64()
        check(self.lib.tfs_server_submit(self.s, sys_id, method, prec, mode, C.c_void_p(d_val),
                                         C.c_void_p(d_b) if d_b else None, C.c_void_p(d_x),
                                         C.c_void_p(d_r1), 1 if x0_zero else 0, niter, tol,
                                         C.byref(t)),
              "tfs_server_submit")
        return t.value

    def submit_host(self, sys_id: int, method: int, prec: int, val: np.ndarray, x: np.ndarray,
                    r1: np.ndarray, niter: int, tol: float, mode: int = TFS_FP64,
                    x0_zero: bool = False) -> int:
        """Queue a solve on host arrays (the drop-in call's arguments): val and
        r1 = b copied in, x and r1 copied out by the request itself.  The
        arrays must stay alive until the ticket is waited for."""
        t = C.c_int64()
        check(self.lib.tfs_server_submit_host(self.s, sys_id, method, prec, mode,
                                              val.ctypes.data_as(C.c_void_p), x.ctypes.data_as(C.c_void_p),
                                              r1.ctypes.data_as(C.c_void_p), 1 if x0_zero else 0, niter,
                                              tol, C.byref(t)),
              "tfs_server_submit_host")
        return t.value

    def wait(self, ticket: int, timeout_s: float = 600.0) -> dict:
        r = tfs_result()
        st = self.lib.tfs_server_wait(self.s, ticket, timeout_s, C.byref(r))
        if st == TFS_ERR_TIMEOUT:
            raise TimeoutError(f"ticket {ticket} still running after {timeout_s} s")
        if st != TFS_OK:
            raise TfsError(st, "tfs_server_wait", last_error())
        return {k: getattr(r, k) for k, _ in tfs_result._fields_}

    def stats(self) -> dict:
        st = tfs_server_stats()
        check(self.lib.tfs_server_get_stats(self.s, C.byref(st)), "tfs_server_get_stats")
        return {k: getattr(st, k) for k, _ in tfs_server_stats._fields_}
