"""GB300-native batched tridiagonal solvers.

The compute path is libtridiag.so (hand-written sm_103a CUDA behind the C ABI
in include/tridiagonal.h, the reference's Tridiagonal_CUDA/tridiagonal.h
entry points plus extensions).  This package loads it with ctypes and offers
PyTorch-tensor wrappers; it has no CPU fallback.
"""
from ._lib import ALGOS, LAYOUTS, LIB_PATH, TridiagError, check, last_status, lib
from .ops import (Factorization, block2, partition_adjoint, partition_path_counts, ppt_counts, partition_supported, solve_host, convert_check, gtsv, periodic, pge, pge_adjoint, relayout, gtsv_adjoint, gtsv_workspace, pivot_record, reference_call, refine,
                  refine_workspace, solve, solve_out, solve_out_workspace)
from .autograd import TridiagonalSolve, solve_ad
from .ragged import RaggedPlan

__all__ = [
    "ALGOS", "LAYOUTS", "LIB_PATH", "TridiagError", "check", "last_status", "lib",
    "gtsv", "gtsv_adjoint", "gtsv_workspace", "pivot_record", "reference_call", "solve", "solve_out",
    "solve_out_workspace", "TridiagonalSolve", "solve_ad", "refine", "refine_workspace", "convert_check", "pge",
    "pge_adjoint", "RaggedPlan", "relayout", "periodic", "Factorization", "block2", "partition_adjoint", "partition_path_counts", "ppt_counts", "partition_supported", "solve_host",
]
