"""The entry point that allocates nothing (tfs_residual_norm_noalloc).

It serves callers that cannot allocate device memory when they call the
library -- code working inside a fixed device arena handed over by its host
framework, or issuing work while another thread captures a CUDA graph.  Its
results must match the allocating entry point tfs_residual: the same residual
(the same per-row arithmetic, so bit for bit) and its norm, on two calls in a
row that reuse the static scratch array.  This file is collected last.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from helpers import system
from tflows import Solver
from tflows.lib import TFS_ERR_ARG, TFS_OK, last_error, load_library

MAX_ROWS = 4194304          # TFS_NOALLOC_MAX_ROWS
H2D, D2H = 1, 2             # cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost


def _cudart():
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            rt = C.CDLL(name)
            rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
            rt.cudaMemcpy.restype = C.c_int
            rt.cudaDeviceSynchronize.restype = C.c_int
            rt.cudaStreamCreate.argtypes = [C.POINTER(C.c_void_p)]
            rt.cudaStreamSynchronize.argtypes = [C.c_void_p]
            rt.cudaStreamDestroy.argtypes = [C.c_void_p]
            return rt
        except OSError:
            continue
    pytest.fail("libcudart not found")


def test_noalloc_rejects_more_rows_than_its_scratch_holds():
    lib = load_library()
    dummy = C.c_void_p(1)   # never dereferenced: the size check comes first
    st = lib.tfs_residual_norm_noalloc(MAX_ROWS + 1, dummy, dummy, dummy, dummy, dummy, dummy, None)
    assert st == TFS_ERR_ARG
    assert "TFS_NOALLOC_MAX_ROWS" in last_error()


@pytest.mark.gpu
@pytest.mark.parametrize("stream", ["default", "created"])
def test_noalloc_residual_norm_matches_tfs_residual(stream, gpu):
    """Two calls in a row on the default stream, or on a stream the caller
    created (the calls serialised by synchronising that stream), each equal
    to the allocating entry point."""
    s = system(0, 24, 20, 18, seed=7)
    x = np.random.default_rng(11).uniform(-1, 1, s.n)
    with Solver(s.matrix()) as sol:            # the existing, allocating entry point
        r_ref = s.b.copy()
        sol.residual(s.val, x, r_ref)
    norm_ref = float(np.linalg.norm(r_ref))

    lib, rt = load_library(), _cudart()
    bufs = {}
    strm = C.c_void_p()
    if stream == "created":
        assert rt.cudaStreamCreate(C.byref(strm)) == 0
    host = {"row": s.row, "col": s.col, "val": s.val, "x": x}
    try:
        # The test allocates the caller's device arrays; the entry point does not.
        for name, a in list(host.items()) + [("r1", s.b), ("norm", np.zeros(1))]:
            p = C.c_void_p()
            assert lib.tfs_device_alloc(a.nbytes, C.byref(p)) == TFS_OK
            bufs[name] = p
            if name in host:
                assert rt.cudaMemcpy(p, a.ctypes.data, a.nbytes, H2D) == 0
        for call in range(2):
            assert rt.cudaMemcpy(bufs["r1"], s.b.ctypes.data, s.b.nbytes, H2D) == 0
            st = lib.tfs_residual_norm_noalloc(s.n, bufs["row"], bufs["col"], bufs["val"],
                                               bufs["x"], bufs["r1"], bufs["norm"], strm if strm.value else None)
            assert st == TFS_OK, last_error()
            if strm.value:
                assert rt.cudaStreamSynchronize(strm) == 0
            assert rt.cudaDeviceSynchronize() == 0
            r = np.empty(s.n)
            nrm = np.zeros(1)
            assert rt.cudaMemcpy(r.ctypes.data, bufs["r1"], r.nbytes, D2H) == 0
            assert rt.cudaMemcpy(nrm.ctypes.data, bufs["norm"], 8, D2H) == 0
            assert np.array_equal(r, r_ref), f"call {call}"
            assert nrm[0] == pytest.approx(norm_ref, rel=1e-12), f"call {call}"
    finally:
        for p in bufs.values():
            lib.tfs_device_free(p)
        if strm.value:
            rt.cudaStreamDestroy(strm)
