"""CPU tests of the host side: the C ABI exports, the topology builder, the
synthetic systems, input validation and the replica partition."""
from __future__ import annotations

import ctypes as C
import json
import re
from pathlib import Path

import numpy as np
import pytest

from oracle import tfs_oracle as O
from tflows import Matrix_Mod_Topology, SynthSystem
from tflows.lib import (SIGNATURES, SYNTH_SIGNATURES, TFS_ERR_ARG, TFS_ERR_MATRIX, lib_path,
                        load_library, load_synth_library)
from tflows.matrix_mod import ptr
from tflows.synth import CONVDIFF, POISSON, loguniform

REPO = Path(__file__).resolve().parents[1]
GOLD = REPO / "tests" / "golden"


def header_functions(pattern: str = "*.h") -> set[str]:
    names = set()
    for h in (REPO / "include").glob(pattern):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(tfs_[a-z0-9_]+)\s*\(", text))
    return names


def test_library_exports_every_declared_symbol():
    lib = load_library()
    declared = header_functions("tfs_solver.h")
    assert len(declared) >= 25
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing
    # the ctypes table covers the same set
    assert declared <= set(SIGNATURES), sorted(declared - set(SIGNATURES))


def test_header_constants_match_the_python_mirror():
    """Every numeric constant of include/tfs_solver.h that the Python side
    mirrors has the header's value, and every option, status, method,
    preconditioner and arithmetic code is mirrored."""
    import tflows.lib as L
    text = (REPO / "include" / "tfs_solver.h").read_text()
    defs = {m.group(1): int(m.group(2))
            for m in re.finditer(r"^#define\s+(TFS_[A-Z0-9_]+)\s+(-?\d+)\b", text, flags=re.M)}
    assert len(defs) >= 30
    for name, value in defs.items():
        if hasattr(L, name):
            assert getattr(L, name) == value, name
    required = [n for n in defs if n.startswith(("TFS_OPT_", "TFS_ERR_", "TFS_PREC_"))]
    required += ["TFS_OK", "TFS_CG", "TFS_BICG", "TFS_CGS", "TFS_FP64", "TFS_MIXED"]
    missing = [n for n in required if not hasattr(L, n)]
    assert not missing, missing


def test_synth_library_exports_its_header_and_nothing_of_the_solver():
    """The seeded systems come from a host-only library, so a process that
    only builds inputs (the CPU reference arm of the benchmark) never loads
    the GPU solver library."""
    syn = load_synth_library()
    declared = header_functions("tfs_synth.h")
    assert declared and declared <= set(SYNTH_SIGNATURES)
    assert all(hasattr(syn, n) for n in declared)
    for n in ("tfs_solve", "tfs_cg", "tfs_topology_register", "tfs_batch_create"):
        assert not hasattr(syn, n), n
    lib = load_library()
    assert not hasattr(lib, "tfs_synth_create")


def test_product_never_reaches_the_oracle():
    """The oracle is the checker only: no module or source of the product
    package mentions it (the build script compiles it for the tests, which is
    not a use), the solver library does not link it and exports none of its
    functions."""
    import subprocess
    pkg = REPO / "t-flows_gb300"
    for p in sorted(pkg.rglob("*")):
        if p.suffix not in (".py", ".cu", ".cuh", ".cpp", ".h", ".f90") or p.name == "build.py":
            continue
        text = p.read_text(errors="replace")
        assert "oracle" not in text.lower() and "tfo_" not in text, p
    lib = load_library()
    dyn = subprocess.run(["readelf", "-d", str(lib._name)], capture_output=True, text=True, check=True).stdout
    assert "oracle" not in dyn, dyn
    syms = subprocess.run(["nm", "-D", "--defined-only", str(lib._name)], capture_output=True, text=True,
                          check=True).stdout
    assert not re.search(r"\btfo_", syms)


def test_library_is_in_tree_and_built_for_sm103a():
    from tflows import build
    assert lib_path.is_relative_to(REPO)
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


@pytest.mark.parametrize("kind,dims,perm", [(POISSON, (6, 5, 4), True), (POISSON, (7, 7, 7), False),
                                            (CONVDIFF, (5, 6, 7), True), (POISSON, (1, 1, 9), True)])
def test_topology_matches_oracle(kind, dims, perm):
    s = SynthSystem(kind, *dims, seed=3, permute=perm)
    A = Matrix_Mod_Topology(s.n, s.faces_c)
    row, col, dia, mir, pos = O.topology(s.n, s.faces_c)
    for a, b in ((A.row, row), (A.col, col), (A.dia, dia), (A.mir, mir), (A.pos, pos)):
        assert np.array_equal(a, b)
    assert np.array_equal(A.row, s.row) and np.array_equal(A.col, s.col)


def test_topology_boundary_faces_and_counts():
    """Faces with c2 <= 0 are boundary faces: no entry, pos = 0."""
    faces = np.array([[1, 2], [2, 3], [1, -1], [3, 0]], np.int32)
    A = Matrix_Mod_Topology(3, faces)
    assert A.row.tolist() == [1, 3, 6, 8]
    assert A.col.tolist() == [1, 2, 1, 2, 3, 2, 3]
    assert A.dia.tolist() == [1, 4, 7]
    assert A.pos.tolist() == [[2, 3], [5, 6], [0, 0], [0, 0]]
    assert A.mir.tolist() == [1, 3, 2, 4, 6, 5, 7]
    assert A.nonzeros == A.nnz + 1


def test_synth_sizes_match_hex_stencil():
    for n in (8, 13):
        s = SynthSystem(POISSON, n)
        interior = 3 * n * n * (n - 1)
        assert s.n == n ** 3 and s.n_faces == interior and s.nnz == n ** 3 + 2 * interior
    s = SynthSystem(POISSON, 32)
    assert s.nnz == 223232          # the 32^3 workload


def test_synth_poisson_properties():
    s = SynthSystem(POISSON, 9, 8, 7, jitter=0.25)
    A = Matrix_Mod_Topology(s.n, s.faces_c)
    assert np.array_equal(s.val, s.val[A.mir - 1])              # symmetric
    off = np.ones(s.nnz, bool)
    off[s.dia - 1] = False
    assert (s.val[off] < 0).all() and (s.val[s.dia - 1] > 0).all()
    rowsum = np.add.reduceat(s.val, s.row[:-1] - 1)
    assert (rowsum > -1e-12).all() and (rowsum > 1e-6).sum() == 8 * 7  # x = 0 Dirichlet cells
    assert (np.abs(s.b) <= 1).all()


def test_synth_convdiff_properties():
    s = SynthSystem(CONVDIFF, 10, jitter=0.2)
    off = np.ones(s.nnz, bool)
    off[s.dia - 1] = False
    assert (s.val[off] <= 0).all()
    rowsum = np.add.reduceat(s.val, s.row[:-1] - 1)
    assert (rowsum > 0).all()                                  # V/dt: strictly dominant
    A = Matrix_Mod_Topology(s.n, s.faces_c)
    assert not np.array_equal(s.val, s.val[A.mir - 1])         # upwind: non-symmetric


def test_synth_deterministic_and_golden():
    import hashlib
    expected = json.loads((GOLD / "synth_hashes.json").read_text())
    from golden.make_golden import SYNTH_HASH_CASES, synth_hash
    for name, (kind, nx, ny, nz, jit, seed, perm) in SYNTH_HASH_CASES.items():
        s = SynthSystem(kind, nx, ny, nz, jitter=jit, seed=seed, permute=perm)
        assert synth_hash(s) == expected[name], name
    assert hashlib is not None


def test_loguniform_range_and_determinism():
    v = [loguniform(5000, 500000, 7, i) for i in range(2000)]
    assert min(v) >= 5000 and max(v) <= 500000
    assert v == [loguniform(5000, 500000, 7, i) for i in range(2000)]
    logs = np.log(v)
    assert abs(np.median(logs) - 0.5 * (np.log(5000) + np.log(500000))) < 0.2


def _register(n, nnz, row, col, dia):
    lib = load_library()
    h = C.c_void_p()
    st = lib.tfs_topology_register(n, nnz, ptr(np.asarray(row, np.int32), C.c_int32),
                                   ptr(np.asarray(col, np.int32), C.c_int32),
                                   ptr(np.asarray(dia, np.int32), C.c_int32), C.byref(h))
    if st == 0:
        lib.tfs_release(h)
    return st


@pytest.mark.parametrize("case,want", [
    ("unsorted", TFS_ERR_MATRIX), ("col_range", TFS_ERR_MATRIX), ("bad_dia", TFS_ERR_MATRIX),
    ("row_end", TFS_ERR_MATRIX), ("empty_row", TFS_ERR_MATRIX), ("n_zero", TFS_ERR_ARG)])
def test_malformed_csr_rejected_before_device_work(case, want):
    row = np.array([1, 3, 5, 7], np.int32)
    col = np.array([1, 2, 1, 2, 2, 3], np.int32)
    dia = np.array([1, 4, 6], np.int32)
    n, nnz = 3, 6
    if case == "unsorted":
        col = np.array([2, 1, 1, 2, 2, 3], np.int32)
    elif case == "col_range":
        col = np.array([1, 4, 1, 2, 2, 3], np.int32)
    elif case == "bad_dia":
        dia = np.array([1, 3, 6], np.int32)
    elif case == "row_end":
        nnz = 7
    elif case == "empty_row":
        row = np.array([1, 3, 3, 7], np.int32)
    elif case == "n_zero":
        n = 0
    assert _register(n, nnz, row, col, dia) == want


def test_fortran_shim_binds_the_abi():
    shim = (REPO / "t-flows_gb300" / "fortran" / "Solvers_Mod_Gpu.f90").read_text()
    for name in ("tfs_cg", "tfs_bicg", "tfs_cgs"):
        assert f'bind(C, name="{name}")' in shim
    for sub in ("subroutine Cg(", "subroutine Bicg(", "subroutine Cgs("):
        assert sub in shim


def test_abi_struct_layouts_match_ctypes(tmp_path):
    """The structs of include/tfs_solver.h and their ctypes mirrors have the
    same size and field offsets (compiled with the host C compiler)."""
    import shutil
    import subprocess
    from tflows import lib as L
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    structs = {"tfs_stats": L.tfs_stats, "tfs_tuning": L.tfs_tuning, "tfs_result": L.tfs_result,
               "tfs_server_stats": L.tfs_server_stats}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "tfs_solver.h"', "int main(void) {"]
    for name, py in structs.items():
        lines.append(f'  printf("{name} size %zu\\n", sizeof({name}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("{name} {fname} %zu\\n", offsetof({name}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    include = Path(__file__).resolve().parents[1] / "include"
    subprocess.run([cc, "-std=c11", "-I", str(include), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for ln in out:
        if ln:
            name, field, val = ln.split()
            got[(name, field)] = int(val)
    for name, py in structs.items():
        assert got[(name, "size")] == C.sizeof(py), name
        for fname, _ in py._fields_:
            assert got[(name, fname)] == getattr(py, fname).offset, (name, fname)


def test_noalloc_scratch_address_is_cached_per_context(tmp_path):
    """The no-allocation entry point caches its scratch array's device
    address per CUDA context, not per device ordinal: a call under another
    context (after a device reset, a re-retained primary context or a
    caller's own context) looks the address up again.  The cache logic is
    compiled on the host and driven with simulated context ids."""
    import subprocess
    exe = tmp_path / "ctx_cache_check"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-I", str(REPO / "t-flows_gb300" / "csrc"),
                    str(REPO / "tests" / "native" / "ctx_cache_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout


def test_one_block_dic_plan_invariants(tmp_path):
    """The one-block DIC plan groups the level schedule into ring-slot
    stages: every group fits a slot (rows and entries), the groups cover all
    levels in order and each is greedy, the slot capacity is a multiple of 32,
    the layout adds up to a byte count within the opt-in shared memory, and a
    schedule whose vector or widest level does not fit gets no plan (the
    level kernels run instead).  The planner is compiled on the host."""
    import subprocess
    exe = tmp_path / "dicb_plan_check"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-I", str(REPO / "t-flows_gb300" / "csrc"),
                    str(REPO / "tests" / "native" / "dicb_plan_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout


def test_reference_arm_line_without_the_solver_library():
    """`bench.py --impl reference` on the 32^3 workload prints one JSON line
    with the keys of the bench contract, the `config` our arm reports for the
    same workload and no host-device bytes; it never loads the GPU solver
    library: the path to it points nowhere in the child's environment (any
    load would fail the run, workers included) and the main process's
    mappings hold no copy of it."""
    import os
    import subprocess
    import sys
    code = ("import runpy, sys\n"
            "sys.argv = ['bench.py', '--impl', 'reference', '--workload', 'poisson32_diag_cg',"
            " '--steps', '1', '--warmup', '3']\n"
            "try:\n"
            "    runpy.run_path('bench.py', run_name='__main__')\n"
            "except SystemExit as e:\n"
            "    assert not e.code, e.code\n"
            "maps = open('/proc/self/maps').read()\n"
            "print('MAPPED' if 'libtfs_gb300' in maps else 'CLEAN', file=sys.stderr)\n")
    env = dict(os.environ, TFS_LIBRARY=str(REPO / "nonexistent" / "libtfs_gb300.so"))
    out = subprocess.run([sys.executable, "-c", code], cwd=REPO, env=env, capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stderr.strip().splitlines()[-1] == "CLEAN", out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 3
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"] == d["e2e"]["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    import argparse
    sys.path.insert(0, str(REPO))
    import bench
    args = argparse.Namespace(workload="poisson32_diag_cg", niter=5000)
    s = SynthSystem(*bench.WORKLOADS["poisson32_diag_cg"][:2], jitter=0.2, seed=bench.BASE_SEED)
    assert d["config"] == bench.workload_config(args, s.n, s.nnz)


@pytest.mark.parametrize("case", ["n0", "null"])
def test_noalloc_rejections_set_error_text(case):
    """Every refusal of the no-allocation entry point says why (no GPU call
    happens before the checks)."""
    lib = load_library()
    dummy = C.c_void_p(1)     # never dereferenced: the checks come first
    if case == "n0":
        st = lib.tfs_residual_norm_noalloc(0, dummy, dummy, dummy, dummy, dummy, dummy, None)
        want = "n must be positive"
    else:
        st = lib.tfs_residual_norm_noalloc(10, dummy, None, dummy, dummy, dummy, dummy, None)
        want = "NULL"
    assert st == TFS_ERR_ARG
    from tflows.lib import last_error
    assert want in last_error()


def test_diag_dic_timeout_rejects_without_a_device():
    """The one-block DIC's timeout diagnostic refuses a null handle and a
    limit outside [0, 1e9] ns, with its error text, before any CUDA call."""
    from tflows.lib import last_error
    lib = load_library()
    assert lib.tfs_diag_dic_timeout(None, 1000) == TFS_ERR_ARG
    assert "tfs_diag_dic_timeout" in last_error()
