"""ctypes binding of libtridiag.so (the C ABI in include/tridiagonal.h).

The library is built in-tree (``python -m tridiagonalsolver_gb300.build``)
into ``tridiagonalsolver_gb300/lib/libtridiag.so``.  There is no fallback:
if the library is missing or fails to load, every entry point raises.
"""
from __future__ import annotations

import ctypes
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libtridiag.so"

# status codes (include/tridiagonal.h)
SUCCESS = 0
ERR_INVALID_VALUE = 1
ERR_NOT_SUPPORTED = 2
ERR_CUDA = 3
ERR_WORKSPACE = 4
ERR_SINGULAR = 5
ERR_TIMEOUT = 6

LAYOUTS = {"contiguous": 0, "packed": 1, "interleaved": 2}
ALGOS = {"auto": 0, "thomas": 1, "cr": 2, "pcr": 3, "wm": 4, "gtsv": 5, "pge": 6, "partition": 7}

_lock = threading.Lock()
_lib = None

_P = ctypes.c_void_p
_I = ctypes.c_int
_SZ = ctypes.c_size_t

# name -> (restype, argtypes); only symbols declared in include/tridiagonal.h
_REF_SIG = [_P, _P, _P, _P, _I, _I]
SIGNATURES: dict[str, tuple] = {
    "tridiag_last_status": (_I, []),
    "tridiag_status_string": (ctypes.c_char_p, [_I]),
    "tridiag_version": (_I, []),
    "tridiag_device_error": (_I, [_I]),
    "tridiag_solve_single": (_I, [_I, _I, _P, _P, _P, _P, _I, _I, _P]),
    "tridiag_solve_double": (_I, [_I, _I, _P, _P, _P, _P, _I, _I, _P]),
    "tridiag_gtsv_workspace_size": (_SZ, [_I, _I, _I, _I]),
    "tridiag_solve_out_workspace_size": (_SZ, [_I, _I, _I, _I, _I]),
    "tridiag_solve_out_single": (_I, [_I, _I, _P, _P, _P, _P, _P, _P, _SZ, _I, _I, _P]),
    "tridiag_solve_out_double": (_I, [_I, _I, _P, _P, _P, _P, _P, _P, _SZ, _I, _I, _P]),
    "tridiag_pivot_record_size": (_SZ, [_I, _I]),
    "tridiag_gtsv_single": (_I, [_I, _P, _P, _P, _P, _P, _P, _P, _SZ, _I, _I, _P]),
    "tridiag_gtsv_double": (_I, [_I, _P, _P, _P, _P, _P, _P, _P, _SZ, _I, _I, _P]),
    "tridiag_gtsv_adjoint_single": (_I, [_I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _SZ, _I, _I, _P]),
    "tridiag_gtsv_adjoint_double": (_I, [_I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _SZ, _I, _I, _P]),
    "tridiag_gtsv_noalloc_single": (_I, [_I, _P, _P, _P, _P, _P, _I, _I, _P]),
    "tridiag_gtsv_noalloc_double": (_I, [_I, _P, _P, _P, _P, _P, _I, _I, _P]),
    "tridiag_refine_workspace_size": (_SZ, [_I, _I, _I]),
    "tridiag_refine_double": (_I, [_I, _P, _P, _P, _P, _P, _I, _P, _P, _SZ, _I, _I, _P]),
    "tridiag_refine_ex_double": (_I, [_I] + [_I, _P, _P, _P, _P, _P, _I, _P, _P, _SZ, _I, _I, _P]),
    "tridiag_convert_check": (_I, [_P, _P, _P, _SZ, _P]),
    "tridiag_partition_fallbacks": (ctypes.c_longlong, [_I]),
    "tridiag_partition_path_counts": (_I, [_P, _I]),
    "tridiag_partition_ppt_counts": (_I, [_P, _I]),
    "tridiag_solve_host_single": (_I, [_I, _I, _P, _P, _P, _P, _P, _I, _I, _I, _P]),
    "tridiag_solve_host_double": (_I, [_I, _I, _P, _P, _P, _P, _P, _I, _I, _I, _P]),
    "tridiag_pge_single": (_I, [_I, _P, _P, _P, _P, _P, _P, _I, _I, _P]),
    "tridiag_pge_double": (_I, [_I, _P, _P, _P, _P, _P, _P, _I, _I, _P]),
    "tridiag_relayout_single": (_I, [_I, _I] + [_P] * 8 + [_I, _I, _P]),
    "tridiag_relayout_double": (_I, [_I, _I] + [_P] * 8 + [_I, _I, _P]),
    "tridiag_gtsv2StridedBatch_bufferSize": (_SZ, [_I, _I, _I, _I]),
    "tridiag_Sgtsv2StridedBatch": (_I, [_I, _P, _P, _P, _P, _I, _I, _P, _P]),
    "tridiag_Dgtsv2StridedBatch": (_I, [_I, _P, _P, _P, _P, _I, _I, _P, _P]),
    "tridiag_gtsvInterleavedBatch_bufferSize": (_SZ, [_I, _I, _I, _I]),
    "tridiag_SgtsvInterleavedBatch": (_I, [_I, _I, _P, _P, _P, _P, _I, _P, _P]),
    "tridiag_DgtsvInterleavedBatch": (_I, [_I, _I, _P, _P, _P, _P, _I, _P, _P]),
    "tridiag_periodic_workspace_size": (_SZ, [_I, _I, _I, _I]),
    "tridiag_periodic_single": (_I, [_I, _P, _P, _P, _P, _P, _P, _SZ, _I, _I, _P]),
    "tridiag_periodic_double": (_I, [_I, _P, _P, _P, _P, _P, _P, _SZ, _I, _I, _P]),
    "tridiag_factor_size": (_SZ, [_I, _I, _I]),
    "tridiag_factor_single": (_I, [_I, _P, _P, _P, _P, _SZ, _P, _I, _I, _P]),
    "tridiag_factor_double": (_I, [_I, _P, _P, _P, _P, _SZ, _P, _I, _I, _P]),
    "tridiag_factored_solve_single": (_I, [_I, _I, _P, _SZ, _P, _I, _I, _I, _P]),
    "tridiag_factored_solve_double": (_I, [_I, _I, _P, _SZ, _P, _I, _I, _I, _P]),
    "tridiag_block2_single": (_I, [_I, _I, _P, _P, _P, _P, _P, _I, _I, _P]),
    "tridiag_block2_double": (_I, [_I, _I, _P, _P, _P, _P, _P, _I, _I, _P]),
    "tridiag_ragged_plan_create": (_I, [_P, _I, _P, _I, _P, _I]),
    "tridiag_ragged_plan_create_ex": (_I, [_P, _I, _P, _I, _P, _I, _P]),
    "tridiag_ragged_plan_create_classify": (_I, [_P, _I, _P, _I, _P, _P, _I, _I]),
    "tridiag_ragged_plan_kinds": (_I, [_P, _P]),
    "tridiag_ragged_refine_workspace_size": (_SZ, [ctypes.c_longlong]),
    "tridiag_ragged_refine_double": (_I, [_P] * 6 + [_I, _P, _SZ, _P, _P]),
    "tridiag_ragged_refine_adjoint_double": (_I, [_P] * 10 + [_I, _P, _SZ, _P, _P]),
    "tridiag_ragged_refine_ex_double": (_I, [_P] * 6 + [_I, _I, _P, _SZ, _P, _P]),
    "tridiag_ragged_refine_adjoint_ex_double": (_I, [_P] * 10 + [_I, _I, _P, _SZ, _P, _P]),
    "tridiag_ragged_plan_destroy": (None, [_P]),
    "tridiag_ragged_plan_buckets": (_I, [_P, _P, _I]),
    "tridiag_ragged_variant_max_n": (_I, [_I, _I]),
    "tridiag_ragged_solve_single": (_I, [_P] * 9),
    "tridiag_ragged_solve_double": (_I, [_P] * 9),
    "tridiag_ragged_adjoint_single": (_I, [_P] * 13),
    "tridiag_ragged_adjoint_double": (_I, [_P] * 13),
    "tridiag_pge_adjoint_single": (_I, [_I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _I, _I, _P]),
    "tridiag_pge_adjoint_double": (_I, [_I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _I, _I, _P]),
    "tridiag_partition_supported": (_I, [_I, _I, _I]),
    "tridiag_partition_adjoint_single": (_I, [_I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _I, _I, _P]),
    "tridiag_partition_adjoint_double": (_I, [_I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _I, _I, _P]),
}
# the reference's entry points: void f(T*, T*, T*, T*, int n_eqt, int n_batch)
REFERENCE_SOLVERS = [
    "cuSparse_single", "cuSparse_double", "BPLG_WM", "BPLG_LF", "BPLG_CR", "BPLG_PCR",
    "Thomas_single", "Thomas_double",
    "WM5_shmem_single", "WM4_shmem_single", "WM5_reg_single", "WM4_reg_single",
    "WM5_shmem_double", "WM4_shmem_double", "WM5_reg_double", "WM4_reg_double",
    "PCR5_shmem_single", "PCR4_shmem_single", "PCR5_reg_single", "PCR4_reg_single",
    "PCR5_shmem_double", "PCR4_shmem_double", "PCR5_reg_double", "PCR4_reg_double",
    "CR_single", "CR_double", "CR_reg4_single", "CR_reg8_single", "CR_reg16_single",
    "CR_reg4_double", "CR_reg8_double", "CR_reg16_double",
]
for _name in REFERENCE_SOLVERS:
    SIGNATURES[_name] = (None, _REF_SIG)
# init / final hooks of the reference registry (Tridiagonal_CUDA/helpers.h:12-19)
SIGNATURES["CR_init_single"] = (_I, _REF_SIG)
SIGNATURES["CR_init_double"] = (_I, _REF_SIG)
SIGNATURES["CR_final"] = (None, [])
SIGNATURES["cuSparse_init_single"] = (_I, _REF_SIG)
SIGNATURES["cuSparse_init_double"] = (_I, _REF_SIG)
SIGNATURES["cuSparse_final"] = (None, [])
SIGNATURES["tridiag_vendor_last_status"] = (_I, [])


class TridiagError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = lib().tridiag_status_string(status).decode() if _lib is not None else str(status)
        super().__init__(f"{what}: {msg} (status {status})" if what else f"{msg} (status {status})")


def lib() -> ctypes.CDLL:
    """Load libtridiag.so once; raise if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m tridiagonalsolver_gb300.build`")
            L = ctypes.CDLL(str(LIB_PATH))
            for name, (res, args) in SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def check(status: int, what: str = "") -> None:
    if status != SUCCESS:
        raise TridiagError(status, what)


def last_status() -> int:
    return int(lib().tridiag_last_status())
