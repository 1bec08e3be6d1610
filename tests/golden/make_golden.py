"""Regenerate the golden fixtures of tests/golden/ (run from the repo root):

    python tests/golden/make_golden.py

Fixtures:
  matrix_mod_example.npz  the compressed-row layout example documented in
                          Sources/Process/Matrix_Mod.f90:15-34 (val, col, row
                          with its n+1 terminator, dia) -- the only artefact of
                          the reference that pins this path's data layout.
                          Its documented dia has a typo (row 3); the fixture
                          keeps it as dia_documented next to the derived dia.
  solve_<name>.npz        small seeded systems (CSR, b) with the oracle's
                          Cg/Bicg/Cgs outputs (x, r1, niter, ini_res, fin_res)
                          for every preconditioner.  The reference cannot be
                          built here (Fortran 90, no Fortran compiler on either
                          machine), so these vectors pin the oracle against
                          drift and across x86-64/AArch64, and feed the GPU
                          parity tests with fixed inputs.
  synth_hashes.json       SHA-256 of the synthetic systems of each workload
                          family at small size (cross-host determinism).
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path[:0] = [str(REPO), str(REPO / "t-flows_gb300")]

from oracle import tfs_oracle as O  # noqa: E402
from tflows.synth import CONVDIFF, POISSON, SynthSystem  # noqa: E402

CASES = {
    # name: (kind, nx, ny, nz, jitter, seed, permute)
    "poisson_6x5x4": (POISSON, 6, 5, 4, 0.2, 11, True),
    "poisson_7x7x7_natural": (POISSON, 7, 7, 7, 0.1, 12, False),
    "convdiff_6x6x5": (CONVDIFF, 6, 6, 5, 0.2, 13, True),
}
SYNTH_HASH_CASES = {
    "poisson_10": (POISSON, 10, 10, 10, 0.2, 20261203, True),
    "poisson_9x8x7_j25": (POISSON, 9, 8, 7, 0.25, 5, True),
    "convdiff_10": (CONVDIFF, 10, 10, 10, 0.2, 20261203, True),
}


def matrix_mod_example() -> dict:
    return dict(
        val=np.array([10, 4, 5, 2, 12, -1, 1, 99, 7, -3, 11, 53], np.float64),
        col=np.array([1, 3, 4, 1, 2, 3, 2, 3, 4, 1, 2, 4], np.int32),
        row=np.array([1, 4, 7, 10, 13], np.int32),
        # Matrix_Mod.f90:34 documents dia = [1 5 9 12], but position 9 holds
        # column 4: row 3's diagonal (column 3) is at position 8.  The
        # Topology.f90:80-81 rule (dia(c) = position with col == c) gives:
        dia=np.array([1, 5, 8, 12], np.int32),
        dia_documented=np.array([1, 5, 9, 12], np.int32),
        dense=np.array([[10, 0, 4, 5], [2, 12, -1, 0], [0, 1, 99, 7], [-3, 11, 0, 53]], np.float64),
    )


def synth_hash(s: SynthSystem) -> str:
    h = hashlib.sha256()
    for a in (s.faces_c, s.row, s.col, s.dia, s.val, s.b):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def solve_case(s: SynthSystem) -> dict:
    out = dict(row=s.row, col=s.col, dia=s.dia, val=s.val, b=s.b,
               faces_c=s.faces_c, tol=np.array(1e-8 * np.linalg.norm(s.b)))
    for method in (0, 1, 2):
        for prec in (0, 1, 2):
            x, r = np.zeros(s.n), s.b.copy()
            it, ini, fin = O.solve(method, s.n, s.row, s.col, s.dia, s.val, x, r, prec, 1000,
                                   float(out["tol"]))
            key = f"m{method}p{prec}"
            out[key + "_x"], out[key + "_r"] = x, r
            out[key + "_scal"] = np.array([it, ini, fin])
    return out


def main() -> None:
    np.savez(HERE / "matrix_mod_example.npz", **matrix_mod_example())
    for name, (kind, nx, ny, nz, jit, seed, perm) in CASES.items():
        s = SynthSystem(kind, nx, ny, nz, jitter=jit, seed=seed, permute=perm)
        np.savez_compressed(HERE / f"solve_{name}.npz", **solve_case(s))
    hashes = {}
    for name, (kind, nx, ny, nz, jit, seed, perm) in SYNTH_HASH_CASES.items():
        hashes[name] = synth_hash(SynthSystem(kind, nx, ny, nz, jitter=jit, seed=seed, permute=perm))
    (HERE / "synth_hashes.json").write_text(json.dumps(hashes, indent=1) + "\n")
    print("wrote", sorted(p.name for p in HERE.glob("*.npz")), "and synth_hashes.json")


if __name__ == "__main__":
    main()
