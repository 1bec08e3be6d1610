"""Regenerate the mesh fixtures of tests/golden/ from the reference's own test
meshes (run from the repo root where the reference tree is present):

    python tests/golden/make_gambit.py <root of the T-FlowS source tree>

(or with the root in TFS_REFERENCE_ROOT)

The reference's test cases ship their meshes as Gambit neutral files (the
input of its Neu2TFlowS converter).  The two smallest are turned into
solver inputs by t-flows_gb300/tflows/gambit.py and stored here, so that
the GPU tests and the bench can solve systems on real meshes where the
reference tree is absent:

  gambit_chan.npz     Tests/Rans/Channel_Re_Tau_590/chan.neu.gz (480 bricks)
  gambit_plain50.npz  Tests/Rans/Flow_over_plain/plain_50.neu.gz (14,490 bricks)

and the first also in the reference's own mesh format, as written by
tflows.cns_geo (chan.cns, chan.geo: the record layout Process reads in
Load_Cns.f90 / Load_Geo.f90).

Each .npz holds the face list faces_c (1-based, c2 = 0 on the boundary), the
pressure-Poisson face coefficients coef (a_f = |S_f|/|d_f| inside,
|S_b|/|d_b| on the Dirichlet set's faces, 0 on the other boundary faces),
the Dirichlet set, the right-hand-side seed and the SHA-256 of the source
file.  Matrix, values and right-hand side are rebuilt from these by
tests/gambit_fixture.py.
"""
from __future__ import annotations

import hashlib
import os
import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(REPO / "t-flows_gb300"))

from tflows import gambit as G  # noqa: E402

MESHES = {
    "chan": "Tests/Rans/Channel_Re_Tau_590/chan.neu.gz",
    "plain50": "Tests/Rans/Flow_over_plain/plain_50.neu.gz",
}
DIRICHLET = (0,)
SEED = 20261203


def build(root: Path, name: str) -> dict:
    src = root / MESHES[name]
    m = G.read_neu(src)
    f = G.mesh_faces(m)
    g = G.geometry(m, f)
    coef = G.poisson_coefficients(m, f, g, DIRICHLET)
    return {"faces_c": f.faces_c.astype(np.int32), "coef": coef, "n_cells": np.int64(m.n_cells),
            "dirichlet": np.array(DIRICHLET, np.int64), "seed": np.int64(SEED),
            "bc_names": np.array([b.name for b in m.bc]),
            "source": np.array(MESHES[name]),
            "sha256": np.array(hashlib.sha256(src.read_bytes()).hexdigest())}


def write_reference_format(root: Path, name: str, out_dir: Path) -> None:
    """The mesh in the reference's own .cns/.geo format (tflows.cns_geo)."""
    from tflows import cns_geo
    m = G.read_neu(root / MESHES[name])
    f = G.mesh_faces(m)
    g = G.geometry(m, f)
    cns, geo = cns_geo.from_gambit(m, f, g)
    cns_geo.write_cns(out_dir / f"{name}.cns", cns)
    cns_geo.write_geo(out_dir / f"{name}.geo", geo)


def main() -> None:
    arg = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("TFS_REFERENCE_ROOT")
    if not arg:
        sys.exit("usage: make_gambit.py <root of the T-FlowS source tree>")
    root = Path(arg)
    golden = REPO / "tests" / "golden"
    for name in MESHES:
        d = build(root, name)
        out = golden / f"gambit_{name}.npz"
        np.savez_compressed(out, **d)
        print(f"{out.name}: {int(d['n_cells'])} cells, {len(d['faces_c'])} faces, {out.stat().st_size} bytes")
    write_reference_format(root, "chan", golden)
    print("chan.cns, chan.geo:", (golden / "chan.cns").stat().st_size, (golden / "chan.geo").stat().st_size, "bytes")


if __name__ == "__main__":
    main()
