"""The reference's own mesh files: `name.cns` (connectivity) and `name.geo`
(geometry), as Process reads them (Sources/Process/Load_Cns.f90:29-69,
Sources/Shared/Load_Geo.f90:21-50) and Divide/Generate write them
(Sources/Shared/Save_Cns_Geo.f90).

Both are Fortran sequential unformatted files: every `read(9)`/`write(9)` is
one record framed by its byte length (4-byte little-endian markers before
and after).  Integers are 4 bytes, `real` is 8 bytes (every build passes
-fdefault-real-8 / -r8), names are character(len=80).

  .cns   n_cells; n_bnd_cells; n_faces; n_sh; n_materials;
         n_boundary_conditions; one record per material name; one per
         boundary-condition name; material(1..n_cells);
         material(-1..-n_bnd_cells); faces_c(1, 1..n_faces);
         faces_c(2, 1..n_faces); bcmark(-1..-n_bnd_cells);
         CopyC(-1..-n_bnd_cells)
  .geo   xc, yc, zc of the cells; xc, yc, zc of the boundary cells
         (-1..-n_bnd_cells); vol; delta; WallDs; sx, sy, sz; dx, dy, dz; f;
         xf, yf, zf of the faces (one record each)

Boundary faces join a cell c1 > 0 to a boundary cell c2 < 0, which the
topology builder takes as "c2 <= 0: boundary".  `write_cns` / `write_geo`
produce the same record sequence (used to turn a Gambit mesh into the
reference's format and for round-trip tests); `pressure_system` builds the
pressure-correction matrix of Compute_Pressure_Simple.f90 from them.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

NAME_LEN = 80


class RecordFile:
    """Sequential unformatted Fortran records (4-byte length markers)."""

    def __init__(self, data: bytes):
        self.data = data
        self.pos = 0

    def record(self) -> bytes:
        if self.pos + 4 > len(self.data):
            raise ValueError("unexpected end of file")
        (n,) = struct.unpack_from("<i", self.data, self.pos)
        body = self.data[self.pos + 4:self.pos + 4 + n]
        if n < 0 or len(body) != n or self.pos + 8 + n > len(self.data):
            raise ValueError("truncated record")
        (tail,) = struct.unpack_from("<i", self.data, self.pos + 4 + n)
        if tail != n:
            raise ValueError("record markers do not match")
        self.pos += 8 + n
        return body

    def ints(self, count: int | None = None) -> np.ndarray:
        a = np.frombuffer(self.record(), dtype="<i4").astype(np.int32)
        if count is not None and a.size != count:
            raise ValueError(f"record holds {a.size} integers, {count} expected")
        return a

    def int(self) -> int:
        return int(self.ints(1)[0])

    def reals(self, count: int) -> np.ndarray:
        a = np.frombuffer(self.record(), dtype="<f8").astype(np.float64)
        if a.size != count:
            raise ValueError(f"record holds {a.size} reals, {count} expected")
        return a

    def name(self) -> str:
        b = self.record()
        if len(b) != NAME_LEN:
            raise ValueError(f"name record of {len(b)} bytes, {NAME_LEN} expected")
        return b.decode("latin-1").rstrip()


def _rec(payload: bytes) -> bytes:
    n = struct.pack("<i", len(payload))
    return n + payload + n


@dataclass
class Cns:
    n_cells: int
    n_bnd_cells: int
    n_faces: int
    n_sh: int
    materials: list[str]
    boundary_conditions: list[str]
    material: np.ndarray          # (n_cells,)
    material_bnd: np.ndarray      # boundary cells -1, -2, ...
    faces_c: np.ndarray           # (n_faces, 2): c1 > 0, c2 > 0 inside, c2 < 0 boundary cell
    bcmark: np.ndarray            # boundary condition of boundary cells -1, -2, ...
    copy_c: np.ndarray            # copy cell of boundary cells -1, -2, ... (0: none)


@dataclass
class Geo:
    xc: np.ndarray                # (n_cells, 3) cell centres
    xc_bnd: np.ndarray            # (n_bnd_cells, 3) boundary cell centres
    vol: np.ndarray
    delta: np.ndarray
    wall_dist: np.ndarray
    s: np.ndarray                 # (n_faces, 3) face area vectors
    d: np.ndarray                 # (n_faces, 3) c1 -> c2 centre distance vectors
    f: np.ndarray                 # (n_faces,) interpolation factors
    xf: np.ndarray                # (n_faces, 3) face centres
    extra: dict = field(default_factory=dict)


def read_cns(path) -> Cns:
    r = RecordFile(Path(path).read_bytes())
    nc, nb, nf, nsh, nm, nbc = (r.int() for _ in range(6))
    if min(nc, nb, nf, nm, nbc) < 0:
        raise ValueError("negative count in .cns header")
    mats = [r.name() for _ in range(nm)]
    bcs = [r.name() for _ in range(nbc)]
    material = r.ints(nc)
    material_bnd = r.ints(nb)
    c1 = r.ints(nf)
    c2 = r.ints(nf)
    bcmark = r.ints(nb)
    copy_c = r.ints(nb)
    return Cns(nc, nb, nf, nsh, mats, bcs, material, material_bnd, np.stack([c1, c2], axis=1),
               bcmark, copy_c)


def read_geo(path, cns: Cns) -> Geo:
    r = RecordFile(Path(path).read_bytes())
    nc, nb, nf = cns.n_cells, cns.n_bnd_cells, cns.n_faces
    xc = np.stack([r.reals(nc) for _ in range(3)], axis=1)
    xb = np.stack([r.reals(nb) for _ in range(3)], axis=1)
    vol, delta, wall = r.reals(nc), r.reals(nc), r.reals(nc)
    s = np.stack([r.reals(nf) for _ in range(3)], axis=1)
    d = np.stack([r.reals(nf) for _ in range(3)], axis=1)
    f = r.reals(nf)
    xf = np.stack([r.reals(nf) for _ in range(3)], axis=1)
    return Geo(xc, xb, vol, delta, wall, s, d, f, xf)


def write_cns(path, c: Cns) -> None:
    out = [_rec(struct.pack("<i", v)) for v in (c.n_cells, c.n_bnd_cells, c.n_faces, c.n_sh,
                                                  len(c.materials), len(c.boundary_conditions))]
    for name in list(c.materials) + list(c.boundary_conditions):
        out.append(_rec(name.encode("latin-1")[:NAME_LEN].ljust(NAME_LEN)))
    for a in (c.material, c.material_bnd, c.faces_c[:, 0], c.faces_c[:, 1], c.bcmark, c.copy_c):
        out.append(_rec(np.ascontiguousarray(a, dtype="<i4").tobytes()))
    Path(path).write_bytes(b"".join(out))


def write_geo(path, g: Geo) -> None:
    arrays = [g.xc[:, 0], g.xc[:, 1], g.xc[:, 2], g.xc_bnd[:, 0], g.xc_bnd[:, 1], g.xc_bnd[:, 2],
              g.vol, g.delta, g.wall_dist, g.s[:, 0], g.s[:, 1], g.s[:, 2], g.d[:, 0], g.d[:, 1], g.d[:, 2],
              g.f, g.xf[:, 0], g.xf[:, 1], g.xf[:, 2]]
    Path(path).write_bytes(b"".join(_rec(np.ascontiguousarray(a, dtype="<f8").tobytes()) for a in arrays))


def from_gambit(m, mf, geom) -> tuple[Cns, Geo]:
    """The reference's files for a Gambit mesh read by tflows.gambit: one
    boundary cell per boundary face (numbered -1, -2, ... in face order, its
    centre the face centre, its condition the face's boundary set), one
    material, no copy cells.  Volumes, delta, wall distances and
    interpolation factors are not derived (zeros); the solver path does not
    read them."""
    nf = len(mf.faces_c)
    bnd = np.nonzero(mf.faces_c[:, 1] == 0)[0]
    nb = len(bnd)
    faces = mf.faces_c.astype(np.int32).copy()
    faces[bnd, 1] = -(np.arange(nb, dtype=np.int32) + 1)
    bcmark = np.zeros(nb, np.int32)
    setno = np.zeros(nf, np.int32)
    for k, bs in enumerate(m.bc):
        setno[mf.face_of[bs.cells, bs.faces]] = k + 1
    bcmark[:] = setno[bnd]
    c1 = faces[:, 0] - 1
    d = np.empty((nf, 3))
    inner = faces[:, 1] > 0
    d[inner] = geom.cell_centre[faces[inner, 1] - 1] - geom.cell_centre[c1[inner]]
    d[~inner] = geom.face_centre[~inner] - geom.cell_centre[c1[~inner]]
    cns = Cns(m.n_cells, nb, nf, 0, ["air"], [b.name for b in m.bc], np.ones(m.n_cells, np.int32),
              np.ones(nb, np.int32), faces, bcmark, np.zeros(nb, np.int32))
    geo = Geo(geom.cell_centre.copy(), geom.face_centre[bnd].copy(), np.zeros(m.n_cells),
              np.zeros(m.n_cells), np.zeros(m.n_cells), geom.face_area.copy(), d, np.zeros(nf),
              geom.face_centre.copy())
    return cns, geo


def faces_for_topology(c: Cns) -> np.ndarray:
    """faces_c for Matrix_Mod_Topology: boundary faces with c2 = 0."""
    f = c.faces_c.astype(np.int32).copy()
    f[f[:, 1] < 0, 1] = 0
    return f


def pressure_coefficients(c: Cns, g: Geo, dirichlet_bcs=(1,), form: str = "area_over_distance") -> np.ndarray:
    """Face coefficients of the pressure matrix: inside a_f = |S|/|d|
    (form "area_over_distance", the scope's synthetic systems) or
    |S|^2 / (S . d) (form "reference", Compute_Pressure_Simple.f90 with
    density 1); on boundary faces whose boundary cell carries one of the
    conditions dirichlet_bcs (1-based), the same with d to the face centre;
    0 on the other boundary faces."""
    if form == "reference":
        coef = np.einsum("ij,ij->i", g.s, g.s) / np.einsum("ij,ij->i", g.s, g.d)
    else:
        coef = np.linalg.norm(g.s, axis=1) / np.linalg.norm(g.d, axis=1)
    bnd = c.faces_c[:, 1] < 0
    dirichlet = np.zeros(len(coef), bool)
    if bnd.any():
        mark = c.bcmark[-c.faces_c[bnd, 1] - 1]
        dirichlet[np.nonzero(bnd)[0]] = np.isin(mark, np.asarray(dirichlet_bcs))
    return np.where(~bnd | dirichlet, coef, 0.0)


def pressure_system(cns_path, geo_path, dirichlet_bcs=(1,), form: str = "area_over_distance",
                    seed: int = 20261203):
    """A pressure system on a mesh stored in the reference's format: CSR by
    the library's Matrix_Mod_Topology, values by the face loop, a seeded
    U[-1, 1] right-hand side."""
    from . import gambit as G
    from .matrix_mod import Matrix_Mod_Topology
    c = read_cns(cns_path)
    g = read_geo(geo_path, c)
    coef = pressure_coefficients(c, g, dirichlet_bcs, form)
    faces = faces_for_topology(c)
    A = Matrix_Mod_Topology(c.n_cells, faces)
    off = np.where(faces[:, 1] > 0, coef, 0.0)
    val = G.assemble_values(len(A.col), faces, A.pos, A.dia, off, off, coef, off)
    b = np.random.default_rng(seed).uniform(-1.0, 1.0, c.n_cells)
    return G.MeshSystem(Path(str(cns_path)).stem, c.n_cells, faces, A.row, A.col, A.dia, A.pos, val, b,
                        coef, tuple(dirichlet_bcs))
