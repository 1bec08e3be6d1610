"""Build recipe of libtfs_gb300.so (sm_103a only), of the host-only
generator of seeded synthetic systems libtfs_synth.so, and of the oracle
library.

    python -m tflows.build          (from the t-flows_gb300 directory)

libtfs_synth.so holds only the benchmark's input generator (tfs_synth.cpp and
the host topology builder it calls): processes that need the seeded systems
but must not touch the GPU solver (the CPU reference arm of the benchmark)
load it alone.

The CUDA translation unit is compiled with ``--fmad=false`` so that every
binary64 product and sum is rounded separately, as in the reference Fortran
build (gfortran -O3 without FMA contraction); host C/C++ uses
``-ffp-contract=off`` for the same reason (GCC on AArch64 contracts by
default).  Objects are compiled in parallel and linked by nvcc.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent            # t-flows_gb300/tflows
PROJ_DIR = PKG_DIR.parent                             # t-flows_gb300
REPO = PROJ_DIR.parent
CSRC = PROJ_DIR / "csrc"
INCLUDE = REPO / "include"
LIB_DIR = PKG_DIR / "lib"
BUILD_DIR = PROJ_DIR / "_build"
LIB_PATH = LIB_DIR / "libtfs_gb300.so"
SYNTH_PATH = LIB_DIR / "libtfs_synth.so"
SYNTH_SOURCES = ["tfs_synth.cpp", "tfs_topology.cpp"]
ORACLE_SRC = REPO / "oracle" / "tfs_oracle.c"
ORACLE_LIB = REPO / "oracle" / "_build" / "libtfs_oracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run_parallel(cmds: list[list[str]]) -> None:
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for c in cmds]
    failed = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((c, out.decode(errors="replace")))
    if failed:
        msg = "\n\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("build failed:\n" + msg)


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def build_library(force: bool = False, verbose: bool = False) -> Path:
    sources = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cuh")) \
        + [c for c in sorted(CSRC.glob("*.cpp")) if c.name != "tfs_synth.cpp"] \
        + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))
    if not force and not _stale(LIB_PATH, sources):
        return LIB_PATH
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    objs, cmds = [], []
    for cu in sorted(CSRC.glob("*.cu")):
        o = BUILD_DIR / (cu.stem + ".o")
        objs.append(o)
        cmds.append([nvcc, *ARCH, "-O3", "-lineinfo", "--fmad=false", "-std=c++17",
                     "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                     "-I", str(INCLUDE), "-c", str(cu), "-o", str(o)])
    for cpp in sorted(CSRC.glob("*.cpp")):
        if cpp.name == "tfs_synth.cpp":
            continue
        o = BUILD_DIR / (cpp.stem + ".o")
        objs.append(o)
        cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
                     "-I", str(INCLUDE), "-c", str(cpp), "-o", str(o)])
    if verbose:
        for c in cmds:
            print(" ".join(c))
    _run_parallel(cmds)
    tmp = LIB_PATH.with_suffix(".so.tmp")
    _run_parallel([[nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def build_synth(force: bool = False) -> Path:
    """Host-only library of the seeded synthetic systems (no CUDA)."""
    sources = [CSRC / f for f in SYNTH_SOURCES] + sorted(INCLUDE.glob("*.h"))
    if not force and not _stale(SYNTH_PATH, sources):
        return SYNTH_PATH
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    tmp = SYNTH_PATH.with_suffix(".so.tmp")
    _run_parallel([["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-Wall",
                    "-I", str(INCLUDE), "-o", str(tmp), *[str(CSRC / f) for f in SYNTH_SOURCES]]])
    os.replace(tmp, SYNTH_PATH)
    return SYNTH_PATH


def build_oracle(force: bool = False) -> Path:
    """Compile the oracle (test infrastructure) with the reference's FP rules."""
    if not force and not _stale(ORACLE_LIB, [ORACLE_SRC]):
        return ORACLE_LIB
    ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
    tmp = ORACLE_LIB.with_suffix(".so.tmp")
    _run_parallel([["gcc", "-O3", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
                    "-shared", "-o", str(tmp), str(ORACLE_SRC), "-lm"]])
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def main(argv: list[str]) -> int:
    force = "--force" in argv
    print(build_library(force=force, verbose="-v" in argv))
    print(build_synth(force=force))
    print(build_oracle(force=force))
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
