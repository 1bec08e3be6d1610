"""Matrix_Mod_Topology on the device (tfs_topology_build_device) against the
oracle's restatement of Topology.f90 and the host builder, bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import system
from oracle import tfs_oracle as O
from tflows.lib import TfsError
from tflows.matrix_mod import Matrix_Mod_Topology, Matrix_Mod_Topology_Device
from tflows.synth import CONVDIFF, POISSON

pytestmark = pytest.mark.gpu


def faces_with_boundary(kind, nx, ny, nz, seed):
    s = system(kind, nx, ny, nz)
    rng = np.random.default_rng(seed)
    cells = rng.choice(s.n, size=s.n // 4, replace=False) + 1
    bnd = np.stack([cells, -np.arange(1, cells.size + 1)], axis=1).astype(np.int32)
    faces = np.concatenate([s.faces_c, bnd])
    return s.n, np.ascontiguousarray(faces[rng.permutation(len(faces))], np.int32)


@pytest.mark.parametrize("kind,dims", [(POISSON, (9, 8, 7)), (CONVDIFF, (17, 13, 11)), (POISSON, (40, 36, 33))])
def test_topology_device_bitwise(kind, dims, gpu):
    n, faces = faces_with_boundary(kind, *dims, seed=sum(dims))
    row, col, dia, mir, pos = O.topology(n, faces)
    dev = Matrix_Mod_Topology_Device(n, faces)
    assert np.array_equal(dev.row, row) and np.array_equal(dev.col, col)
    assert np.array_equal(dev.dia, dia) and np.array_equal(dev.mir, mir)
    assert np.array_equal(dev.pos, pos)
    host = Matrix_Mod_Topology(n, faces)
    assert np.array_equal(host.col, dev.col) and np.array_equal(host.pos, dev.pos)


def test_topology_device_edge_cases(gpu):
    # a single cell and no faces; then boundary faces around one interior face
    one = Matrix_Mod_Topology_Device(1, np.zeros((0, 2), np.int32))
    assert list(one.row) == [1, 2] and list(one.col) == [1] and list(one.dia) == [1]
    faces = np.array([[1, -1], [2, -2], [1, 2]], np.int32)
    row, col, dia, mir, pos = O.topology(2, faces)
    dev = Matrix_Mod_Topology_Device(2, faces)
    assert np.array_equal(dev.col, col) and np.array_equal(dev.mir, mir) and np.array_equal(dev.pos, pos)
    with pytest.raises(TfsError):
        Matrix_Mod_Topology_Device(2, np.array([[1, 3]], np.int32))     # cell out of range
    with pytest.raises(TfsError):
        Matrix_Mod_Topology_Device(2, np.array([[2, 2]], np.int32))     # c1 == c2
