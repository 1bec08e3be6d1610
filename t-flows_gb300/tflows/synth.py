"""Seeded synthetic systems (include/tfs_synth.h) for tests and benchmarks.

The generator lives in libtfs_synth.so, a host-only library: building a
system never loads the GPU solver library."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .lib import TFS_SYNTH_CONVDIFF, TFS_SYNTH_POISSON, load_synth_library
from .matrix_mod import Matrix_Type, ptr

POISSON, CONVDIFF = TFS_SYNTH_POISSON, TFS_SYNTH_CONVDIFF
BASE_SEED = 20261203


def _check(status: int, where: str) -> None:
    # The generator reports argument errors only (no error text); the
    # message is built here so that no other library is loaded.
    if status != 0:
        raise ValueError(f"{where}: invalid arguments (status {status})")


class SynthSystem:
    """A jittered-hex finite-volume system: faces_c (1-based), CSR row/col/dia
    (1-based), val and the right-hand side b."""

    def __init__(self, kind: int, nx: int, ny: int | None = None, nz: int | None = None,
                 jitter: float = 0.2, seed: int = BASE_SEED, permute: bool = True):
        lib = load_synth_library()
        ny = nx if ny is None else ny
        nz = nx if nz is None else nz
        h = C.c_void_p()
        _check(lib.tfs_synth_create(kind, nx, ny, nz, float(jitter), seed & (2**64 - 1),
                                    1 if permute else 0, C.byref(h)), "tfs_synth_create")
        try:
            n, nnz, nf = C.c_int32(), C.c_int32(), C.c_int32()
            lib.tfs_synth_dims(h, C.byref(n), C.byref(nnz), C.byref(nf))
            self.kind, self.dims, self.jitter, self.seed = kind, (nx, ny, nz), jitter, seed
            self.n, self.nnz, self.n_faces = n.value, nnz.value, nf.value
            self.faces_c = np.zeros((self.n_faces, 2), np.int32)
            self.row = np.zeros(self.n + 1, np.int32)
            self.col = np.zeros(self.nnz, np.int32)
            self.dia = np.zeros(self.n, np.int32)
            self.val = np.zeros(self.nnz)
            self.b = np.zeros(self.n)
            i32 = C.c_int32
            _check(lib.tfs_synth_export(h, ptr(self.faces_c, i32), ptr(self.row, i32),
                                        ptr(self.col, i32), ptr(self.dia, i32),
                                        ptr(self.val, C.c_double), ptr(self.b, C.c_double)),
                   "tfs_synth_export")
        finally:
            lib.tfs_synth_free(h)

    def matrix(self) -> Matrix_Type:
        return Matrix_Type(self.n, self.row, self.col, self.dia, self.val)


def loguniform(lo: int, hi: int, seed: int, index: int) -> int:
    return int(load_synth_library().tfs_synth_loguniform(lo, hi, seed & (2**64 - 1), index))


def uniform(seed: int, stream: int, index: int) -> float:
    return float(load_synth_library().tfs_synth_uniform(seed & (2**64 - 1), stream, index))


def batched_poisson_specs(n_sys: int, seed: int) -> list[tuple[int, int, int, float, int]]:
    """(nx, ny, nz, jitter, seed) of every system of the batched workload:
    cells log-uniform in [5k, 500k] realised as k x k x m meshes (k =
    round(cbrt(n)), m = round(n / k^2)), jitter U(0, 25%), own seed each."""
    out = []
    for k in range(n_sys):
        n = loguniform(5000, 500000, seed, k)
        kk = max(2, int(round(n ** (1.0 / 3.0))))
        m = max(1, int(round(n / (kk * kk))))
        jit = 0.25 * uniform(seed, 21, k)
        out.append((kk, kk, m, jit, seed * 1000 + k))
    return out


def serving_pool_specs(n_pool: int, seed: int) -> list[tuple[int, int, int, int, int]]:
    """(kind, nx, ny, nz, seed) of the resident systems of the serving trace:
    70% pressure-Poisson, 30% convection-diffusion, cells log-uniform in
    [10k, 2M]."""
    out = []
    for k in range(n_pool):
        kind = POISSON if uniform(seed, 31, k) < 0.7 else CONVDIFF
        n = loguniform(10000, 2000000, seed, 1000 + k)
        kk = max(2, int(round(n ** (1.0 / 3.0))))
        m = max(1, int(round(n / (kk * kk))))
        out.append((kind, kk, kk, m, seed * 100 + k))
    return out
