"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Imported by tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` to check or time against the CUDA library.  The library itself
never imports this module.

Arrays are numpy, layout 0 (system j occupies rows [j*n, (j+1)*n) of each of
a, b, c, d).  Every solver copies its inputs and returns x, so callers keep
their data; ``*_inplace`` variants follow the reference's in-place contract.

Also loads ``oracle/_ref/libref_avx512.so`` (the reference's own AVX-512 CPU
kernels, built by ``make -C oracle ref`` on x86-64 hosts that have the
reference sources) when present; see :func:`ref_lib`.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
REF_PATH = HERE / "_ref" / "libref_avx512.so"

_lib = None
_ref = None

_F32P = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_F64P = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_I32P = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def build(force: bool = False) -> Path:
    """Compile liboracle.so with make if it is missing (or ``force``)."""
    if force or not LIB_PATH.exists():
        subprocess.run(["make", "-C", str(HERE), "-s", "all"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        for t, P in (("f32", _F32P), ("f64", _F64P)):
            getattr(L, f"orc_thomas_{t}").argtypes = [P, P, P, P, ctypes.c_int, ctypes.c_int]
            getattr(L, f"orc_thomas_{t}").restype = None
            for nm, extra in (("cr", 1), ("pcr", 1), ("wm", 2)):
                f = getattr(L, f"orc_{nm}_{t}")
                f.argtypes = [P, P, P, P, ctypes.c_int, ctypes.c_int] + [ctypes.c_int] * extra
                f.restype = ctypes.c_int
            f = getattr(L, f"orc_gtsv_{t}")
            f.argtypes = [P, P, P, P, ctypes.c_int, ctypes.c_int]
            f.restype = ctypes.c_int
            for nm in ("gbsv", "thomas"):
                f = getattr(L, f"orc_block2_{nm}_{t}")
                f.argtypes = [P, P, P, P, _I32P, ctypes.c_int, ctypes.c_int]
                f.restype = ctypes.c_int
        L.orc_adjoint_f64.argtypes = [_F64P] * 9 + [ctypes.c_int, ctypes.c_int]
        L.orc_adjoint_f64.restype = ctypes.c_int
        L.orc_residual_f64.argtypes = [_F64P] * 6 + [ctypes.c_int, ctypes.c_int]
        L.orc_residual_f64.restype = None
        L.orc_backward_error_f64.argtypes = [_F64P] * 6 + [ctypes.c_int, ctypes.c_int]
        L.orc_backward_error_f64.restype = ctypes.c_double
        L.orc_check_f64.argtypes = [_F64P, _F64P, ctypes.c_int, _F64P]
        L.orc_check_f64.restype = ctypes.c_int
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_get_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def threads() -> int:
    return int(lib().orc_get_threads())


def _sfx(dtype) -> str:
    dt = np.dtype(dtype)
    if dt == np.float32:
        return "f32"
    if dt == np.float64:
        return "f64"
    raise TypeError(f"oracle supports float32/float64, got {dt}")


def _prep(a, b, c, d, n):
    dt = np.result_type(a, b, c, d)
    arrs = [np.ascontiguousarray(np.array(v, dtype=dt, copy=True)).reshape(-1) for v in (a, b, c, d)]
    size = arrs[0].size
    if any(v.size != size for v in arrs) or n <= 0 or size % n:
        raise ValueError("a, b, c, d must have the same size, a multiple of n")
    return arrs, size // n


def _call(name, a, b, c, d, n, *extra):
    (a_, b_, c_, d_), batch = _prep(a, b, c, d, n)
    f = getattr(lib(), f"orc_{name}_{_sfx(a_.dtype)}")
    rc = f(a_, b_, c_, d_, int(n), int(batch), *[int(e) for e in extra])
    if rc not in (None, 0):
        raise RuntimeError(f"oracle {name} failed with code {rc}")
    return d_


def thomas(a, b, c, d, n):
    """Reference Thomas; returns x (layout 0, flat)."""
    return _call("thomas", a, b, c, d, n)


def cr(a, b, c, d, n, levels=7):
    return _call("cr", a, b, c, d, n, levels)


def pcr(a, b, c, d, n, steps):
    return _call("pcr", a, b, c, d, n, steps)


def wm(a, b, c, d, n, rounds, half=0):
    return _call("wm", a, b, c, d, n, rounds, half)


def gtsv(a, b, c, d, n):
    """Partial-pivoting elimination (LAPACK ?gtsv algorithm); returns x."""
    return _call("gtsv", a, b, c, d, n)


def block2(a, b, c, d, n, algo="gbsv"):
    """Block tridiagonal solve with 2 x 2 blocks (a, b, c of shape
    (batch, n, 2, 2) or flat, d of shape (batch, n, 2) or flat).  ``algo`` is
    "gbsv" (partial pivoting, the LAPACK ?gbsv algorithm) or "thomas" (block
    Thomas).  Returns (x flat, per-system info)."""
    dt = np.result_type(a, b, c, d)
    a_, b_, c_, d_ = (np.ascontiguousarray(np.array(v, dtype=dt, copy=True)).reshape(-1) for v in (a, b, c, d))
    if n <= 0 or a_.size % (4 * n) or any(v.size != a_.size for v in (b_, c_)) or d_.size * 2 != a_.size:
        raise ValueError("a, b, c need 4*n*batch values and d 2*n*batch")
    batch = a_.size // (4 * n)
    info = np.zeros(batch, dtype=np.int32)
    getattr(lib(), f"orc_block2_{algo}_{_sfx(dt)}")(a_, b_, c_, d_, info, int(n), int(batch))
    return d_, info


def block2_dense(a, b, c, n):
    """Dense matrices (batch, 2n, 2n) of block tridiagonal systems (FP64)."""
    a, b, c = (np.asarray(v, dtype=np.float64).reshape(-1, n, 2, 2) for v in (a, b, c))
    batch = a.shape[0]
    M = np.zeros((batch, 2 * n, 2 * n))
    for i in range(n):
        M[:, 2 * i:2 * i + 2, 2 * i:2 * i + 2] = b[:, i]
        if i > 0:
            M[:, 2 * i:2 * i + 2, 2 * i - 2:2 * i] = a[:, i]
        if i + 1 < n:
            M[:, 2 * i:2 * i + 2, 2 * i + 2:2 * i + 4] = c[:, i]
    return M


def block2_backward_error(a, b, c, d, x, n):
    """Per-system normwise backward error of block tridiagonal solves in FP64:
    ||d - A x||_inf / (||A||_inf ||x||_inf + ||d||_inf); A_0 and C_{n-1} are
    not part of the matrix."""
    a, b, c = (np.array(v, dtype=np.float64).reshape(-1, n, 2, 2) for v in (a, b, c))
    d, x = (np.asarray(v, dtype=np.float64).reshape(-1, n, 2) for v in (d, x))
    a[:, 0] = 0
    c[:, n - 1] = 0
    xm = np.concatenate([np.zeros_like(x[:, :1]), x[:, :-1]], axis=1)
    xp = np.concatenate([x[:, 1:], np.zeros_like(x[:, :1])], axis=1)
    r = d - (np.einsum("bnij,bnj->bni", a, xm) + np.einsum("bnij,bnj->bni", b, x)
             + np.einsum("bnij,bnj->bni", c, xp))
    rown = np.abs(a).sum(axis=3) + np.abs(b).sum(axis=3) + np.abs(c).sum(axis=3)
    nb = len(x)
    den = rown.reshape(nb, -1).max(axis=1) * np.abs(x).reshape(nb, -1).max(axis=1) \
        + np.abs(d).reshape(nb, -1).max(axis=1)
    eta = np.abs(r).reshape(nb, -1).max(axis=1) / np.where(den > 0, den, 1.0)
    eta = np.where(np.isfinite(x).reshape(nb, -1).all(axis=1), eta, np.inf)
    return eta, float(eta.max()) if eta.size else 0.0


def adjoint_f64(a, b, c, x, xbar, n):
    """FP64 adjoint of x = A^-1 d for L = sum(xbar*x): (ga, gb, gc, gd)."""
    a, b, c, x, xbar = (np.ascontiguousarray(v, dtype=np.float64).reshape(-1) for v in (a, b, c, x, xbar))
    batch = a.size // n
    ga, gb, gc, gd = (np.empty_like(a) for _ in range(4))
    rc = lib().orc_adjoint_f64(a, b, c, x, xbar, ga, gb, gc, gd, int(n), int(batch))
    if rc:
        raise RuntimeError(f"oracle adjoint: zero pivot in row {rc}")
    return ga, gb, gc, gd


def residual_f64(a, b, c, d, x, n):
    a, b, c, d, x = (np.ascontiguousarray(v, dtype=np.float64).reshape(-1) for v in (a, b, c, d, x))
    r = np.empty_like(a)
    lib().orc_residual_f64(a, b, c, d, x, r, int(n), int(a.size // n))
    return r


def backward_error(a, b, c, d, x, n):
    """Per-system normwise backward error in FP64 and its maximum."""
    a, b, c, d, x = (np.ascontiguousarray(v, dtype=np.float64).reshape(-1) for v in (a, b, c, d, x))
    batch = a.size // n
    eta = np.empty(batch, dtype=np.float64)
    worst = lib().orc_backward_error_f64(a, b, c, d, x, eta, int(n), int(batch))
    return eta, float(worst)


def check(x, xref):
    """Reference driver statistics: (mean, rms, max, argmax)."""
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
    xref = np.ascontiguousarray(xref, dtype=np.float64).reshape(-1)
    st = np.zeros(3, dtype=np.float64)
    arg = lib().orc_check_f64(x, xref, int(x.size), st)
    return float(st[0]), float(st[1]), float(st[2]), int(arg)


# --------------------------------------------------------------------------
# The reference's own CPU kernels (x86-64 build of Tridiagonal_AVX512).

REF_FUNCS = {
    # name: (dtype, uses buffer of 4*n*batch)
    "Thomas_single": (np.float32, False), "Thomas_double": (np.float64, False),
    "CR_single": (np.float32, True), "CR_double": (np.float64, True),
    "PCR4_single": (np.float32, False), "PCR3_single": (np.float32, False),
    "WM4_single": (np.float32, False), "WM3_single": (np.float32, False),
    "PCR3_double": (np.float64, False), "PCR2_double": (np.float64, False),
    "WM3_double": (np.float64, False), "WM2_double": (np.float64, False),
}


def ref_available() -> bool:
    return REF_PATH.exists()


def ref_lib():
    """Load oracle/_ref/libref_avx512.so, or return None when it was not built."""
    global _ref
    if _ref is None and REF_PATH.exists():
        _ref = ctypes.CDLL(str(REF_PATH))
        for nm, (dt, _) in REF_FUNCS.items():
            P = ctypes.c_void_p
            f = getattr(_ref, nm)
            f.argtypes = [P, P, P, P, P, ctypes.c_int, ctypes.c_int]
            f.restype = None
    return _ref


def _aligned(arr: np.ndarray, align: int = 64) -> np.ndarray:
    """Copy into a buffer whose data pointer is `align`-byte aligned (the
    reference's AVX-512 kernels use aligned loads)."""
    nbytes = arr.nbytes
    raw = np.empty(nbytes + align, dtype=np.uint8)
    off = (-raw.ctypes.data) % align
    out = raw[off:off + nbytes].view(arr.dtype)
    out[:] = arr.reshape(-1)
    return out


def ref_solve(name: str, a, b, c, d, n):
    """Run the reference's own CPU kernel `name` (e.g. "WM3_double"); returns x."""
    L = ref_lib()
    if L is None:
        raise RuntimeError("reference CPU library not built (make -C oracle ref)")
    dt, needs_buf = REF_FUNCS[name]
    arrs = [_aligned(np.asarray(v, dtype=dt)) for v in (a, b, c, d)]
    batch = arrs[0].size // n
    buf = _aligned(np.zeros(4 * n * batch, dtype=dt)) if needs_buf else None
    ptrs = [ctypes.c_void_p(v.ctypes.data) for v in arrs]
    getattr(L, name)(*ptrs, ctypes.c_void_p(buf.ctypes.data) if buf is not None else None, int(n), int(batch))
    return np.array(arrs[3], copy=True)


def ref_threads_env() -> dict:
    return {"OMP_NUM_THREADS": os.environ.get("OMP_NUM_THREADS", "")}
