"""The reference's own test meshes (Gambit neutral files) as solver inputs:
the reader against the meshes themselves where the reference tree is
present, and the committed mesh fixtures against the oracle's topology,
face loop and solver."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

from gambit_fixture import NAMES, load
from oracle import tfs_oracle as O
from tflows import gambit as G

REF = Path("/root/reference")
MESHES = ["Tests/Rans/Channel_Re_Tau_590/chan.neu.gz",
          "Tests/Rans/Channel_Re_Tau_590_Rsm/chan_full.neu.gz",
          "Tests/Rans/Flow_over_plain/plain_50.neu.gz",
          "Tests/Rans/Impinging_Jet_2d_Distant_Re_23000/jet.neu.gz",
          "Tests/Les/Pipe_Re_Tau_180/pipe.neu.gz"]
needs_ref = pytest.mark.skipif(not (REF / "Tests").is_dir(), reason="reference tree not present")


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
