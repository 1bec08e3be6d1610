"""tflows -- host-side Python interface to libtfs_gb300.so.

The GB300 (sm_103a) Krylov solver path of T-FlowS: preconditioned CG, BiCG
and CGS on the compressed-row Matrix_Type, with the reference's Fortran call
shape (Sources/Process/Solvers_Mod/Cg.f90:2-4).  Every compute call goes
through the C ABI of the in-tree shared library; there is no CPU fallback.
"""
from .lib import (TFS_OK, TFS_CG, TFS_BICG, TFS_CGS, TFS_PREC_NONE, TFS_PREC_DIAG,
                  TFS_PREC_DIC, TFS_FP64, TFS_MIXED, TfsError, load_library, lib_path)
from .matrix_mod import Matrix_Type, Matrix_Mod_Topology
from .solvers_mod import Cg, Bicg, Cgs, Prec_Form, Prec_Solve, Residual, Solver, spmv
from .synth import SynthSystem
from .batch import Batch
from .serve import Server

__all__ = [
    "TFS_OK", "TFS_CG", "TFS_BICG", "TFS_CGS", "TFS_PREC_NONE", "TFS_PREC_DIAG", "TFS_PREC_DIC",
    "TFS_FP64", "TFS_MIXED", "TfsError", "load_library", "lib_path", "Matrix_Type",
    "Matrix_Mod_Topology", "Cg", "Bicg", "Cgs", "Prec_Form", "Prec_Solve", "Residual",
    "Solver", "spmv", "SynthSystem", "Batch", "Server",
]
