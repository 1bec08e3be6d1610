"""Matrix_Type of T-FlowS (Sources/Process/Matrix_Mod.f90:36-49) as numpy
arrays with the reference's 1-based contents, and its topology builder
(Sources/Process/Matrix_Mod/Topology.f90:2-127) through the C ABI."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from .lib import check, load_library


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


def ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


@dataclass
class Matrix_Type:
    """Compressed-row matrix: row(1:n+1), col(1:nnz), dia(1:n), val(1:nnz),
    1-based like the Fortran arrays (stored in 0-based numpy arrays).
    ``nonzeros`` follows the reference: nnz + 1 (one padding slot)."""
    n_cells: int
    row: np.ndarray
    col: np.ndarray
    dia: np.ndarray
    val: np.ndarray
    mir: np.ndarray | None = None
    pos: np.ndarray | None = None
    _solver: object = field(default=None, repr=False, compare=False)

    def __post_init__(self):
        self.row = _i32(self.row)
        self.col = _i32(self.col)
        self.dia = _i32(self.dia)
        self.val = np.ascontiguousarray(self.val, dtype=np.float64)
        if self.row.shape != (self.n_cells + 1,) or self.dia.shape != (self.n_cells,):
            raise ValueError("row must have n+1 entries and dia n entries")
        if self.col.shape != (self.nnz,) or self.val.shape != (self.nnz,):
            raise ValueError("col and val must have row(n+1)-1 entries")

    @property
    def nnz(self) -> int:
        return int(self.row[-1]) - 1

    @property
    def nonzeros(self) -> int:
        return self.nnz + 1

    def to_dense(self) -> np.ndarray:
        n = self.n_cells
        a = np.zeros((n, n))
        for i in range(n):
            for j in range(self.row[i] - 1, self.row[i + 1] - 1):
                a[i, self.col[j] - 1] = self.val[j]
        return a


def Matrix_Mod_Topology(n_cells: int, faces_c: np.ndarray) -> Matrix_Type:
    """Build row/col/dia/mir/pos from face connectivity faces_c (n_faces x 2,
    1-based cell numbers, c2 <= 0 for boundary faces); val is zero."""
    lib = load_library()
    f = _i32(faces_c).reshape(-1)
    n_faces = f.size // 2
    nnz = lib.tfs_topology_count(n_cells, n_faces, ptr(f, C.c_int32))
    if nnz < 0:
        raise ValueError("invalid face list")
    row = np.zeros(n_cells + 1, np.int32)
    col = np.zeros(nnz, np.int32)
    dia = np.zeros(n_cells, np.int32)
    mir = np.zeros(nnz, np.int32)
    pos = np.zeros(2 * n_faces, np.int32)
    check(lib.tfs_topology_build(n_cells, n_faces, ptr(f, C.c_int32), ptr(row, C.c_int32),
                                 ptr(col, C.c_int32), ptr(dia, C.c_int32), ptr(mir, C.c_int32),
                                 ptr(pos, C.c_int32)), "tfs_topology_build")
    return Matrix_Type(n_cells, row, col, dia, np.zeros(nnz), mir=mir, pos=pos.reshape(-1, 2))


def Matrix_Mod_Topology_Device(n_cells: int, faces_c: np.ndarray) -> Matrix_Type:
    """Matrix_Mod_Topology built on the GPU (tfs_topology_build_device): the
    same row/col/dia/mir/pos as Matrix_Mod_Topology, bit for bit."""
    lib = load_library()
    fc = np.ascontiguousarray(faces_c, dtype=np.int32).reshape(-1)
    n_faces = fc.size // 2
    cap = n_cells + 2 * n_faces
    sizes = {"fc": max(fc.nbytes, 4), "row": 4 * (n_cells + 1), "col": 4 * cap, "dia": 4 * n_cells,
             "mir": 4 * cap, "pos": 4 * max(2 * n_faces, 1)}
    dev = {}
    try:
        for k, nb in sizes.items():
            q = C.c_void_p()
            check(lib.tfs_device_alloc(nb, C.byref(q)), "tfs_device_alloc")
            dev[k] = q.value
        check(lib.tfs_memcpy(C.c_void_p(dev["fc"]), fc.ctypes.data_as(C.c_void_p), fc.nbytes), "tfs_memcpy")
        nnz = C.c_int32()
        check(lib.tfs_topology_build_device(n_cells, n_faces, *(C.c_void_p(dev[k]) for k in
                                                               ("fc", "row", "col", "dia", "mir", "pos")),
                                            C.byref(nnz)), "tfs_topology_build_device")
        nnz = nnz.value
        out = {"row": np.zeros(n_cells + 1, np.int32), "col": np.zeros(nnz, np.int32),
               "dia": np.zeros(n_cells, np.int32), "mir": np.zeros(nnz, np.int32),
               "pos": np.zeros(2 * n_faces, np.int32)}
        for k, a in out.items():
            check(lib.tfs_memcpy(a.ctypes.data_as(C.c_void_p), C.c_void_p(dev[k]), a.nbytes), "tfs_memcpy")
    finally:
        for d in dev.values():
            lib.tfs_device_free(C.c_void_p(d))
    return Matrix_Type(n_cells, out["row"], out["col"], out["dia"], np.zeros(nnz), mir=out["mir"],
                       pos=out["pos"].reshape(-1, 2))
