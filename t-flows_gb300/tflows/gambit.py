"""Gambit neutral meshes (.neu, optionally gzipped) as solver inputs.

The reference reads its meshes as `.cns`/`.geo` files written by its own
Fortran converters (Generate, Neu2TFlowS); those records cannot be produced
without a Fortran compiler.  The meshes of the reference's test cases come
as Gambit neutral files, the input of Neu2TFlowS
(Sources/Neu2TFlowS/Load_Neu.f90), so this module reads them directly and
derives what the solver path needs:

  read_neu        nodes, cells (brick, wedge, tetrahedron, pyramid) and the
                  named boundary-condition sets (element, Gambit face number);
  mesh_faces      the face list faces_c (n_faces x 2, 1-based, c2 = 0 on the
                  boundary) -- faces matched by their node sets, as
                  Find_Faces.f90 does -- and the face of every (cell, local
                  face) pair;
  geometry        cell centres and face centres (node averages) and face area
                  vectors out of c1 (half the sum of the cross products of
                  consecutive face nodes);
  poisson_system  the pressure-Poisson system of the scope's configs on the
                  mesh: a_f = |S_f| / |d_f| between cell centres,
                  off-diagonals -a_f, diagonal sum a_f, Dirichlet faces
                  (chosen boundary sets) adding |S_b| / |d_b| (cell centre to
                  face centre), zero flux elsewhere, a seeded U[-1, 1]
                  right-hand side; CSR through Matrix_Mod_Topology and values
                  through the face loop.

Periodic boundary sets are treated as walls (zero flux): the reference joins
periodic faces in its converters, which this reader does not restate.
"""
from __future__ import annotations

import gzip
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

# Local faces of each Gambit element type, by the number of element nodes,
# in Gambit's face numbering (face k of the list is Gambit face k + 1;
# 0-based local node numbers).  Gambit's numbering is a property of the file
# format; the reference's converter holds the same sets (neu_mod.f90).
GAMBIT_FACES = {
    8: ((0, 4, 5, 1), (1, 5, 7, 3), (3, 7, 6, 2), (2, 6, 4, 0), (0, 1, 3, 2), (4, 6, 7, 5)),  # brick
    6: ((0, 3, 4, 1), (1, 4, 5, 2), (2, 5, 3, 0), (0, 1, 2), (3, 5, 4)),                      # wedge
    4: ((0, 1, 2), (0, 3, 1), (1, 3, 2), (2, 3, 0)),                                           # tetrahedron
    5: ((0, 1, 3, 2), (0, 4, 1), (1, 4, 3), (3, 4, 2), (2, 4, 0)),                             # pyramid
}
GAMBIT_TYPES = {4: 8, 5: 6, 6: 4, 7: 5}   # Gambit element type -> nodes


@dataclass
class BoundarySet:
    name: str
    cells: np.ndarray      # 0-based cell numbers
    faces: np.ndarray      # 0-based Gambit face numbers


@dataclass
class GambitMesh:
    nodes: np.ndarray                  # (n_nodes, 3)
    cell_ptr: np.ndarray               # (n_cells + 1,) offsets into cell_nodes
    cell_nodes: np.ndarray             # 0-based node numbers of every cell
    bc: list[BoundarySet] = field(default_factory=list)

    @property
    def n_cells(self) -> int:
        return len(self.cell_ptr) - 1

    def cell_size(self) -> np.ndarray:
        return np.diff(self.cell_ptr)


def _lines(path: Path):
    opener = gzip.open if str(path).endswith(".gz") else open
    with opener(path, "rt") as f:
        for line in f:
            yield line.rstrip("\n")


def read_neu(path) -> GambitMesh:
    """Parse a Gambit neutral file (Load_Neu.f90 reads the same sections)."""
    it = _lines(Path(path))
    nodes = cells = None
    n_np = n_el = 0
    bc: list[BoundarySet] = []
    for line in it:
        head = line.strip()
        if head.startswith("NUMNP"):
            n_np, n_el = (int(v) for v in next(it).split()[:2])
        elif head.startswith("NODAL COORDINATES"):
            nodes = np.zeros((n_np, 3))
            for k in range(n_np):
                v = next(it).split()
                nodes[int(v[0]) - 1] = [float(x) for x in v[1:4]]
        elif head.startswith("ELEMENTS/CELLS"):
            sizes = np.zeros(n_el, np.int64)
            flat: list[list[int]] = [None] * n_el  # type: ignore[list-item]
            for _ in range(n_el):
                v = next(it).split()
                e, etype, nn = int(v[0]), int(v[1]), int(v[2])
                if GAMBIT_TYPES.get(etype) != nn:
                    raise ValueError(f"element {e}: unsupported type {etype} with {nn} nodes")
                ids = [int(x) for x in v[3:]]
                while len(ids) < nn:
                    ids += [int(x) for x in next(it).split()]
                sizes[e - 1] = nn
                flat[e - 1] = [i - 1 for i in ids]
            ptr = np.zeros(n_el + 1, np.int64)
            np.cumsum(sizes, out=ptr[1:])
            cells = (ptr, np.array([i for c in flat for i in c], np.int64))
        elif head.startswith("BOUNDARY CONDITIONS"):
            v = next(it).split()
            name, itype, nentry = v[0], int(v[1]), int(v[2])
            if itype != 1:
                raise ValueError(f"boundary set {name}: only element/face sets are read")
            cl = np.zeros(nentry, np.int64)
            fl = np.zeros(nentry, np.int64)
            for k in range(nentry):
                w = next(it).split()
                cl[k], fl[k] = int(w[0]) - 1, int(w[2]) - 1
            bc.append(BoundarySet(name, cl, fl))
    if nodes is None or cells is None:
        raise ValueError(f"{path}: no nodes or cells")
    return GambitMesh(nodes, cells[0], cells[1], bc)


@dataclass
class MeshFaces:
    faces_c: np.ndarray        # (n_faces, 2) 1-based, c2 = 0 on the boundary
    face_nodes: np.ndarray     # (n_faces, 4) 0-based node numbers, -1 padded
    face_of: np.ndarray        # (n_cells, 6) face number of (cell, local face), -1 unused


def mesh_faces(m: GambitMesh) -> MeshFaces:
    """Faces shared by two cells are matched by their sorted node numbers
    (Find_Faces.f90 matches by node numbers as well); faces in cell order,
    interior faces at the first cell that owns them."""
    nc = m.n_cells
    size = m.cell_size()
    rows = []   # (cell, local face, 4 node numbers)
    for nn, faces in GAMBIT_FACES.items():
        cs = np.nonzero(size == nn)[0]
        if cs.size == 0:
            continue
        base = m.cell_ptr[cs]
        for lf, loc in enumerate(faces):
            nodes = np.full((cs.size, 4), -1, np.int64)
            for k, ln in enumerate(loc):
                nodes[:, k] = m.cell_nodes[base + ln]
            rows.append((cs, np.full(cs.size, lf), nodes))
    cell = np.concatenate([r[0] for r in rows])
    lface = np.concatenate([r[1] for r in rows])
    fn = np.concatenate([r[2] for r in rows])
    order = np.lexsort((lface, cell))
    cell, lface, fn = cell[order], lface[order], fn[order]
    key = np.sort(np.where(fn < 0, np.iinfo(np.int64).max, fn), axis=1)
    _, first, inv, cnt = np.unique(key, axis=0, return_index=True, return_inverse=True, return_counts=True)
    inv = inv.reshape(-1)
    if cnt.max() > 2:
        raise ValueError("a face is shared by more than two cells")
    # Faces numbered by their first occurrence in (cell, local face) order.
    rank = np.empty(len(first), np.int64)
    rank[np.argsort(first, kind="stable")] = np.arange(len(first))
    fid = rank[inv]
    nf = len(first)
    c1 = np.full(nf, -1, np.int64)
    c2 = np.zeros(nf, np.int64)
    nodes = np.full((nf, 4), -1, np.int64)
    first_occ = np.zeros(len(cell), bool)
    first_occ[first] = True
    f_first = fid[first_occ]
    c1[f_first] = cell[first_occ] + 1
    nodes[f_first] = fn[first_occ]
    second = ~first_occ
    c2[fid[second]] = cell[second] + 1
    face_of = np.full((nc, 6), -1, np.int64)
    face_of[cell, lface] = fid
    return MeshFaces(np.stack([c1, c2], axis=1).astype(np.int32), nodes, face_of)


@dataclass
class Geometry:
    cell_centre: np.ndarray    # (n_cells, 3)
    face_centre: np.ndarray    # (n_faces, 3)
    face_area: np.ndarray      # (n_faces, 3) area vectors pointing out of c1 (towards c2)


def geometry(m: GambitMesh, f: MeshFaces) -> Geometry:
    size = m.cell_size()
    sums = np.zeros((m.n_cells, 3))
    cidx = np.repeat(np.arange(m.n_cells), size)
    np.add.at(sums, cidx, m.nodes[m.cell_nodes])
    cc = sums / size[:, None]
    valid = f.face_nodes >= 0
    nv = valid.sum(axis=1)
    xyz = m.nodes[np.where(valid, f.face_nodes, 0)] * valid[:, :, None]
    fc = xyz.sum(axis=1) / nv[:, None]
    s = np.zeros_like(fc)
    for k in range(4):
        nxt = np.where(k + 1 < nv, k + 1, 0)
        a = xyz[:, k]
        b = xyz[np.arange(len(nv)), nxt]
        s += np.where((k < nv)[:, None], np.cross(a, b), 0.0)
    # Gambit's local face loops run clockwise seen from outside the cell, so
    # the cross products point into c1: negate for vectors out of c1.
    return Geometry(cc, fc, -0.5 * s)


@dataclass
class MeshSystem:
    name: str
    n: int
    faces_c: np.ndarray
    row: np.ndarray            # 1-based CSR (Matrix_Type)
    col: np.ndarray
    dia: np.ndarray
    pos: np.ndarray            # (n_faces, 2) 1-based entry of (c1,c2) and (c2,c1)
    val: np.ndarray
    b: np.ndarray
    coef: np.ndarray           # a_f per face (interior) or Dirichlet |S|/|d| (0 for walls)
    dirichlet_sets: tuple

    @property
    def nnz(self) -> int:
        return len(self.val)

    def matrix(self):
        from .matrix_mod import Matrix_Type
        return Matrix_Type(self.n, self.row, self.col, self.dia, self.val)


def poisson_coefficients(m: GambitMesh, f: MeshFaces, g: Geometry, dirichlet_sets=(0,)) -> np.ndarray:
    """a_f = |S_f| / |d_f| on interior faces; |S_b| / |d_b| on the faces of
    the Dirichlet sets, 0 on the other boundary faces."""
    c1 = f.faces_c[:, 0].astype(np.int64) - 1
    c2 = f.faces_c[:, 1].astype(np.int64) - 1
    interior = c2 >= 0
    d = np.where(interior[:, None], g.cell_centre[np.where(interior, c2, 0)], g.face_centre) - g.cell_centre[c1]
    coef = np.linalg.norm(g.face_area, axis=1) / np.linalg.norm(d, axis=1)
    dir_faces = np.zeros(len(c1), bool)
    for k in dirichlet_sets:
        bs = m.bc[k]
        fid = f.face_of[bs.cells, bs.faces]
        dir_faces[fid] = True
    return np.where(interior | dir_faces, coef, 0.0)


def assemble_values(nnz: int, faces_c: np.ndarray, pos: np.ndarray, dia: np.ndarray,
                    off12: np.ndarray, off21: np.ndarray, dia12: np.ndarray, dia21: np.ndarray) -> np.ndarray:
    """Matrix values by the reference's face loop (Compute_Pressure_Simple.f90
    style: for every face in order, val(pos(1,s)) -= off12, val(dia(c1)) +=
    dia12, val(pos(2,s)) -= off21, val(dia(c2)) += dia21; a boundary face
    adds dia12 to its cell when that is non-zero).  The updates are applied
    one at a time in exactly that order, so every entry is summed in the
    loop's order."""
    c1 = faces_c[:, 0].astype(np.int64)
    c2 = faces_c[:, 1].astype(np.int64)
    nf = len(c1)
    interior = c2 > 0
    d1 = dia[c1 - 1].astype(np.int64) - 1
    d2 = dia[np.where(interior, c2, 1) - 1].astype(np.int64) - 1
    idx = np.stack([pos[:, 0].astype(np.int64) - 1, d1, pos[:, 1].astype(np.int64) - 1, d2], axis=1)
    add = np.stack([-off12, dia12, -off21, dia21], axis=1)
    keep = np.zeros((nf, 4), bool)
    keep[interior] = True
    keep[~interior, 1] = dia12[~interior] != 0.0
    val = np.zeros(nnz)
    # x - y and x + (-y) round identically, so the subtractions become adds.
    np.add.at(val, idx[keep], add[keep])
    return val


def poisson_system(m: GambitMesh, name: str = "mesh", dirichlet_sets=(0,), seed: int = 20261203) -> MeshSystem:
    """The pressure-Poisson system on the mesh (module docstring), CSR by the
    library's Matrix_Mod_Topology and values by the face loop."""
    from .matrix_mod import Matrix_Mod_Topology
    f = mesh_faces(m)
    g = geometry(m, f)
    coef = poisson_coefficients(m, f, g, dirichlet_sets)
    A = Matrix_Mod_Topology(m.n_cells, f.faces_c)
    interior = f.faces_c[:, 1] > 0
    zero = np.zeros_like(coef)
    val = assemble_values(len(A.col), f.faces_c, A.pos, A.dia, np.where(interior, coef, 0.0),
                          np.where(interior, coef, 0.0), coef, np.where(interior, coef, zero))
    b = np.random.default_rng(seed).uniform(-1.0, 1.0, m.n_cells)
    return MeshSystem(name, m.n_cells, f.faces_c, A.row, A.col, A.dia, A.pos, val, b, coef,
                      tuple(dirichlet_sets))


def system_from_fixture(path) -> MeshSystem:
    """Rebuild a MeshSystem from a fixture written by make_gambit.py (face
    list, face coefficients, Dirichlet sets and right-hand-side seed): CSR by
    the library's Matrix_Mod_Topology, values by the face loop."""
    from .matrix_mod import Matrix_Mod_Topology
    d = np.load(path)
    faces_c, coef = d["faces_c"], d["coef"]
    n = int(d["n_cells"])
    A = Matrix_Mod_Topology(n, faces_c)
    off = np.where(faces_c[:, 1] > 0, coef, 0.0)
    val = assemble_values(len(A.col), faces_c, A.pos, A.dia, off, off, coef, off)
    b = np.random.default_rng(int(d["seed"])).uniform(-1.0, 1.0, n)
    name = Path(str(path)).stem.replace("gambit_", "")
    return MeshSystem(name, n, faces_c, A.row, A.col, A.dia, A.pos, val, b, coef,
                      tuple(int(k) for k in d["dirichlet"]))
