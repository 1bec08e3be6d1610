"""The reference's own test meshes (Gambit neutral files) as solver inputs:
the reader against the meshes themselves where the reference tree is
present, and the committed mesh fixtures against the oracle's topology,
face loop and solver."""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np
import pytest

from gambit_fixture import NAMES, load
from oracle import tfs_oracle as O
from tflows import gambit as G

# Root of a T-FlowS source tree (its Tests/ directory holds the meshes); the
# reader tests run only where one is named.
REF = Path(os.environ.get("TFS_REFERENCE_ROOT", "") or "/nonexistent")
MESHES = ["Tests/Rans/Channel_Re_Tau_590/chan.neu.gz",
          "Tests/Rans/Channel_Re_Tau_590_Rsm/chan_full.neu.gz",
          "Tests/Rans/Flow_over_plain/plain_50.neu.gz",
          "Tests/Rans/Impinging_Jet_2d_Distant_Re_23000/jet.neu.gz",
          "Tests/Les/Pipe_Re_Tau_180/pipe.neu.gz"]
needs_ref = pytest.mark.skipif(not (REF / "Tests").is_dir(),
                               reason="no T-FlowS tree named by TFS_REFERENCE_ROOT")


@needs_ref
@pytest.mark.parametrize("path", MESHES)
def test_reader_on_reference_meshes(path):
    """Every boundary-condition face (element, Gambit face number) is a face
    of exactly one cell -- which pins the face numbering of bricks and
    wedges -- every boundary face belongs to a set, and every cell is closed
    (its outward area vectors sum to zero)."""
    m = G.read_neu(REF / path)
    f = G.mesh_faces(m)
    g = G.geometry(m, f)
    bnd = f.faces_c[:, 1] == 0
    in_set = np.zeros(len(bnd), bool)
    for bs in m.bc:
        fid = f.face_of[bs.cells, bs.faces]
        assert (fid >= 0).all() and bnd[fid].all()
        in_set[fid] = True
    assert np.array_equal(in_set, bnd)
    c1 = f.faces_c[:, 0] - 1
    c2 = f.faces_c[:, 1] - 1
    S = np.zeros((m.n_cells, 3))
    np.add.at(S, c1, g.face_area)
    np.add.at(S, c2[~bnd], -g.face_area[~bnd])
    assert np.abs(S).max() <= 1e-12 * np.abs(g.face_area).max()
    # interior faces point from c1 to c2
    d = g.cell_centre[c2[~bnd]] - g.cell_centre[c1[~bnd]]
    assert (np.einsum("ij,ij->i", d, g.face_area[~bnd]) > 0).all()


@needs_ref
@pytest.mark.parametrize("name", NAMES)
def test_fixture_is_reproduced(name):
    """The committed fixture is what the reader makes of the mesh today."""
    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    import make_gambit
    d = make_gambit.build(REF, name)
    g = np.load(Path(__file__).resolve().parent / "golden" / f"gambit_{name}.npz")
    assert np.array_equal(d["faces_c"], g["faces_c"]) and np.array_equal(d["coef"], g["coef"])
    assert str(d["sha256"]) == str(g["sha256"])


@pytest.mark.parametrize("name", NAMES)
def test_fixture_system_against_oracle(name):
    """Matrix_Mod_Topology of the library and the face loop give the
    oracle's row/col/dia/pos and values bit for bit; the Poisson matrix is
    symmetric; the oracle's diagonal CG converges on it."""
    s = load(name)
    row, col, dia, mir, pos = O.topology(s.n, s.faces_c)
    assert np.array_equal(s.row, row) and np.array_equal(s.col, col)
    assert np.array_equal(s.dia, dia) and np.array_equal(s.pos, pos)
    interior = s.faces_c[:, 1] > 0
    off = np.where(interior, s.coef, 0.0)
    val = O.assemble_faces(s.n, s.faces_c.reshape(-1), pos.reshape(-1), dia, off, off, s.coef, off,
                           None, np.zeros(len(col)))
    assert np.array_equal(s.val, val)
    p = s.pos[interior] - 1
    assert np.array_equal(s.val[p[:, 0]], s.val[p[:, 1]])
    tol = 1e-8 * np.linalg.norm(s.b)
    x, r = np.zeros(s.n), s.b.copy()
    it, ini, fin = O.solve(0, s.n, s.row, s.col, s.dia, s.val, x, r, 1, 5000, tol)
    assert it <= 5000 and fin < tol


GOLDEN = Path(__file__).resolve().parent / "golden"


def test_cns_geo_fixture_matches_gambit_system():
    """The chan mesh in the reference's .cns/.geo format (read as Process's
    Load_Cns / Load_Geo read it) gives the same faces, coefficients, matrix
    and values bit for bit as the Gambit-derived fixture."""
    from tflows import cns_geo
    a = cns_geo.pressure_system(GOLDEN / "chan.cns", GOLDEN / "chan.geo", dirichlet_bcs=(1,))
    b = load("chan")
    assert np.array_equal(a.faces_c, b.faces_c) and np.array_equal(a.coef, b.coef)
    for k in ("row", "col", "dia", "pos", "val", "b"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k


def test_cns_geo_roundtrip_and_errors(tmp_path):
    """Reading and writing back reproduces the files byte for byte; a cut
    file or a damaged record marker is refused."""
    from tflows import cns_geo
    c = cns_geo.read_cns(GOLDEN / "chan.cns")
    g = cns_geo.read_geo(GOLDEN / "chan.geo", c)
    assert c.n_cells == 480 and c.n_faces == 1711 and c.n_bnd_cells == 542
    assert c.boundary_conditions[:2] == ["one", "two"]
    assert (c.faces_c[:, 0] > 0).all() and (c.faces_c[c.faces_c[:, 1] < 0, 1] >= -c.n_bnd_cells).all()
    cns_geo.write_cns(tmp_path / "x.cns", c)
    cns_geo.write_geo(tmp_path / "x.geo", g)
    assert (tmp_path / "x.cns").read_bytes() == (GOLDEN / "chan.cns").read_bytes()
    assert (tmp_path / "x.geo").read_bytes() == (GOLDEN / "chan.geo").read_bytes()
    raw = (GOLDEN / "chan.cns").read_bytes()
    (tmp_path / "cut.cns").write_bytes(raw[:-6])
    with pytest.raises(ValueError):
        cns_geo.read_cns(tmp_path / "cut.cns")
    bad = bytearray(raw)
    bad[4 + 4] ^= 1          # tail marker of the first record
    (tmp_path / "bad.cns").write_bytes(bytes(bad))
    with pytest.raises(ValueError):
        cns_geo.read_cns(tmp_path / "bad.cns")


@needs_ref
def test_cns_geo_fixture_is_reproduced(tmp_path):
    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    import make_gambit
    make_gambit.write_reference_format(REF, "chan", tmp_path)
    for ext in ("cns", "geo"):
        assert (tmp_path / f"chan.{ext}").read_bytes() == (GOLDEN / f"chan.{ext}").read_bytes()


def test_neu_reader_small_synthetic(tmp_path):
    """A two-brick Gambit file written here: the shared face is found once,
    boundary-set faces map to boundary faces, area vectors point out of c1,
    and an unsupported element type is refused."""
    nodes = [(x, y, z) for z in (0.0, 1.0) for y in (0.0, 1.0) for x in (0.0, 1.0, 2.0)]
    # brick node order of Gambit: (0,0,0),(1,0,0),(0,1,0),(1,1,0),(0,0,1),(1,0,1),(0,1,1),(1,1,1)
    def nid(ix, iy, iz):
        return 1 + ix + 3 * iy + 6 * iz
    cells = []
    for c in range(2):
        cells.append([nid(c + dx, dy, dz) for dz in (0, 1) for dy in (0, 1) for dx in (0, 1)])
    lines = ["        CONTROL INFO 2.3.16", "** GAMBIT NEUTRAL FILE", "t", "PROGRAM:  test", "date",
             "     NUMNP     NELEM     NGRPS    NBSETS     NDFCD     NDFVL",
             f"{len(nodes):10d}{len(cells):10d}         1         1         3         3", "ENDOFSECTION",
             "   NODAL COORDINATES 2.3.16"]
    for k, (x, y, z) in enumerate(nodes):
        lines.append(f"{k + 1:10d}{x:20.11e}{y:20.11e}{z:20.11e}")
    lines += ["ENDOFSECTION", "      ELEMENTS/CELLS 2.3.16"]
    for k, c in enumerate(cells):
        lines.append(f"{k + 1:8d} 4  8 " + " ".join(str(v) for v in c[:7]))
        lines.append("               " + str(c[7]))
    # face 4 of Gambit's brick is the x = 0 side: cell 1's left face
    lines += ["ENDOFSECTION", " BOUNDARY CONDITIONS 2.3.16", "                            left       1       1       0       6",
              "         1    4    4", "ENDOFSECTION"]
    p = tmp_path / "two.neu"
    p.write_text("\n".join(lines) + "\n")
    m = G.read_neu(p)
    f = G.mesh_faces(m)
    g = G.geometry(m, f)
    assert m.n_cells == 2 and len(f.faces_c) == 11
    inner = f.faces_c[:, 1] > 0
    assert inner.sum() == 1 and tuple(f.faces_c[inner][0]) == (1, 2)
    assert np.allclose(g.face_area[inner][0], [1.0, 0.0, 0.0])
    fid = f.face_of[m.bc[0].cells, m.bc[0].faces][0]
    assert f.faces_c[fid, 1] == 0 and np.allclose(g.face_centre[fid], [0.0, 0.5, 0.5])
    assert np.allclose(g.face_area[fid], [-1.0, 0.0, 0.0])
    bad = p.read_text().replace("       1 4  8 ", "       1 9  8 ", 1)
    (tmp_path / "bad.neu").write_text(bad)
    with pytest.raises(ValueError):
        G.read_neu(tmp_path / "bad.neu")
