"""Systems on the reference's test meshes, rebuilt from tests/golden/gambit_*.npz
(made by tests/golden/make_gambit.py)."""
from __future__ import annotations

from pathlib import Path

from tflows import gambit as G

GOLDEN = Path(__file__).resolve().parent / "golden"
NAMES = ("chan", "plain50")


def load(name: str) -> G.MeshSystem:
    return G.system_from_fixture(GOLDEN / f"gambit_{name}.npz")
