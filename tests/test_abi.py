"""The C ABI of libtridiag.so without a GPU: the library builds, loads, and
exports every function include/tridiagonal.h declares; argument checks and
status strings work before any device call."""
import ctypes
import re
import subprocess

import pytest

from tests.conftest import ROOT

HEADER = ROOT / "include" / "tridiagonal.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\([^;]*\)\s*;", text, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from tridiagonalsolver_gb300 import build

    build.build()
    from tridiagonalsolver_gb300 import _lib

    return _lib.lib()


def test_header_declares_reference_names():
    names = declared_functions()
    for n in ("Thomas_single", "Thomas_double", "tridiag_last_status"):
        assert n in names
    assert len(names) >= 10


def test_every_declared_symbol_is_exported(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(ROOT / "tridiagonalsolver_gb300" / "lib" / "libtridiag.so")],
                         capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, f"declared but not exported: {missing}"
    for n in declared_functions():
        assert hasattr(lib, n)


def test_python_signatures_cover_header(lib):
    from tridiagonalsolver_gb300 import _lib

    missing = [n for n in declared_functions() if n not in _lib.SIGNATURES]
    assert not missing, f"no ctypes signature for: {missing}"


def test_status_strings(lib):
    from tridiagonalsolver_gb300 import _lib

    assert lib.tridiag_status_string(_lib.SUCCESS) == b"success"
    assert lib.tridiag_status_string(_lib.ERR_SINGULAR) == b"zero pivot"
    assert lib.tridiag_status_string(12345) == b"unknown status"
    assert lib.tridiag_version() >= 100


def test_argument_checks_need_no_device(lib):
    from tridiagonalsolver_gb300 import _lib

    # invalid sizes and null pointers are rejected before any CUDA call
    assert lib.tridiag_solve_double(1, 0, None, None, None, None, 16, 4, None) == _lib.ERR_INVALID_VALUE
    assert lib.tridiag_solve_single(1, 0, ctypes.c_void_p(16), None, None, None, 0, 4, None) == _lib.ERR_INVALID_VALUE
    assert lib.tridiag_solve_single(1, 7, ctypes.c_void_p(16), None, None, None, 8, 4, None) == _lib.ERR_INVALID_VALUE
    assert lib.tridiag_last_status() == _lib.ERR_INVALID_VALUE
    # gtsv without workspace
    p = ctypes.c_void_p(256)
    st = lib.tridiag_gtsv_double(0, p, p, p, p, None, None, None, 0, 8, 2, None)
    assert st == _lib.ERR_WORKSPACE
    assert lib.tridiag_gtsv_workspace_size(1, 0, 0, 4) == 0
    assert lib.tridiag_gtsv_workspace_size(1, 0, 100, 7) >= 2 * 100 * 7 * 8
    assert lib.tridiag_pivot_record_size(64, 3) == 2 * 3 * 4


def test_host_solve_and_path_count_checks_need_no_device(lib):
    """The host-buffer solve and the path counters reject bad arguments
    before any CUDA call; the gtsv workspace covers the chunked solve's one
    int per system."""
    from tridiagonalsolver_gb300 import _lib

    p = ctypes.c_void_p(256)
    assert lib.tridiag_solve_host_double(0, 0, None, p, p, p, p, 64, 4, 0, None) == _lib.ERR_INVALID_VALUE
    assert lib.tridiag_solve_host_single(0, 0, p, p, p, p, p, 0, 4, 0, None) == _lib.ERR_INVALID_VALUE
    assert lib.tridiag_solve_host_single(0, 0, p, p, p, p, p, 64, 4, -1, None) == _lib.ERR_INVALID_VALUE
    assert lib.tridiag_solve_host_single(0, 9, p, p, p, p, p, 64, 4, 0, None) == _lib.ERR_INVALID_VALUE
    assert lib.tridiag_solve_host_single(0, 1, p, p, p, p, p, 64, 4, 0, None) == _lib.ERR_NOT_SUPPORTED
    assert lib.tridiag_partition_path_counts(None, 0) == _lib.ERR_INVALID_VALUE
    n, batch = 100000, 5
    need = 2 * n * batch * 8 + 4 * ((n + 31) // 32) * batch + 4 * batch
    assert lib.tridiag_gtsv_workspace_size(1, 0, n, batch) >= need


def test_ragged_refine_ex_checks_need_no_device(lib):
    """The refined ragged entry points with pivoted_iters reject a missing
    plan or arrays before any CUDA call."""
    from tridiagonalsolver_gb300 import _lib

    p = ctypes.c_void_p(256)
    assert lib.tridiag_ragged_refine_ex_double(None, p, p, p, p, p, 1, 1, p, 1 << 20, p, None) == _lib.ERR_INVALID_VALUE
    assert lib.tridiag_ragged_refine_adjoint_ex_double(None, p, p, p, p, p, p, p, p, p, 1, 1, p, 1 << 20, p,
                                                       None) == _lib.ERR_INVALID_VALUE
    # the adjoint's gradient outputs are checked first
    assert lib.tridiag_ragged_refine_adjoint_ex_double(p, p, p, p, p, p, None, p, p, p, 1, 1, p, 1 << 20, p,
                                                       None) == _lib.ERR_INVALID_VALUE


def test_gtsv_workspace_covers_the_thread_per_partition_solve(lib):
    """tridiag_gtsv_workspace_size asks for the thread-per-partition solve's
    factor arrays (five n x batch arrays and the rest) exactly where that
    solve serves the shape -- FP64 batches of >= 1024 systems, contiguous ones
    beyond one CTA (up to 27648 rows), interleaved ones from 1024 rows -- and
    for the other paths' two arrays elsewhere; its counters reject a NULL
    array before any CUDA call."""
    from tridiagonalsolver_gb300 import _lib

    al = lambda v: (v + 255) // 256 * 256
    small = lambda n, b: 2 * al(n * b * 8) + al((n + 31) // 32 * b * 4) + al(b * 4)
    for layout, n, batch, big in ((0, 4096, 4096, False), (0, 8192, 2048, True), (0, 27648, 1024, True),
                                  (0, 65536, 1024, False), (0, 8192, 512, False), (2, 4096, 4096, True),
                                  (2, 1024, 16384, True), (2, 512, 16384, False), (1, 8192, 2048, False)):
        got = lib.tridiag_gtsv_workspace_size(1, layout, n, batch)
        assert got >= small(n, batch)
        assert (got >= 5 * n * batch * 8) == big, (layout, n, batch, got)
        # FP32 keeps the other paths' workspace
        assert lib.tridiag_gtsv_workspace_size(0, layout, n, batch) < 5 * n * batch * 4
    assert lib.tridiag_partition_ppt_counts(None, 0) == _lib.ERR_INVALID_VALUE
