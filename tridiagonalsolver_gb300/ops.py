"""PyTorch front end of libtridiag.so: device memory and streams come from
torch, all arithmetic from the CUDA kernels of the library.

Arrays are CUDA tensors holding ``batch`` systems of ``n`` rows in one of the
layouts of include/tridiagonal.h:

* ``"contiguous"`` (reference layout 0): shape ``(batch, n)`` or flat;
* ``"interleaved"``: shape ``(n, batch)`` or flat (row i of system j at
  ``i*batch + j``);
* ``"packed"`` (reference layout 1): one tensor of ``batch*4*n`` elements.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from ._lib import ALGOS, LAYOUTS, check, lib

_DT = {torch.float32: "single", torch.float64: "double"}


def _stream_ptr(stream=None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


def _ptr(t: torch.Tensor | None, dtype=None) -> int | None:
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("tensor must be on a CUDA device")
    if not t.is_contiguous():
        raise ValueError("tensor must be contiguous")
    if dtype is not None and t.dtype != dtype:
        raise TypeError(f"expected {dtype}, got {t.dtype}")
    return int(t.data_ptr())


def _al(t: torch.Tensor | None) -> torch.Tensor | None:
    """A read-only input with a 16-byte aligned start (the TMA kernels need
    one): views at odd offsets are copied, everything else passes through."""
    if t is None or (t.is_contiguous() and t.data_ptr() % 16 == 0):
        return t
    return t.contiguous().clone()


def _prec(t: torch.Tensor) -> str:
    if t.dtype not in _DT:
        raise TypeError(f"unsupported dtype {t.dtype} (float32 or float64)")
    return _DT[t.dtype]


def _dims(t: torch.Tensor, n: int, layout: str) -> int:
    per = 4 * n if layout == "packed" else n
    if n <= 0 or t.numel() % per:
        raise ValueError(f"tensor of {t.numel()} elements does not hold whole systems of n={n}")
    return t.numel() // per


def solve(a, b, c, d, n: int, algo: str = "auto", layout: str = "contiguous", stream=None):
    """In-place solve with the reference's contract: c may be overwritten,
    d receives x.  Returns d.  For layout "packed" pass the packed tensor as
    ``a`` and None for b, c, d (the solution is in rows 3n..4n of each
    system)."""
    p = _prec(a)
    batch = _dims(a, n, layout)
    fn = getattr(lib(), f"tridiag_solve_{p}")
    st = fn(ALGOS[algo], LAYOUTS[layout], _ptr(a, a.dtype), _ptr(b, a.dtype), _ptr(c, a.dtype),
            _ptr(d, a.dtype), n, batch, _stream_ptr(stream))
    check(st, f"tridiag_solve_{p}({algo}, {layout})")
    return d if d is not None else a


def solve_out_workspace(a: torch.Tensor, n: int, algo: str = "auto", layout: str = "contiguous") -> torch.Tensor:
    batch = _dims(a, n, layout)
    nbytes = lib().tridiag_solve_out_workspace_size(1 if a.dtype == torch.float64 else 0, ALGOS[algo],
                                                     LAYOUTS[layout], n, batch)
    return torch.empty(max(nbytes, 1), dtype=torch.uint8, device=a.device)


def solve_out(a, b, c, d, n: int, algo: str = "auto", layout: str = "contiguous", out=None, work=None,
              stream=None):
    """Out-of-place solve: a, b, c, d untouched; returns x (new or ``out``)."""
    p = _prec(a)
    batch = _dims(a, n, layout)
    a, b, c, d = _al(a), _al(b), _al(c), _al(d)
    x = out if out is not None else torch.empty_like(d)
    work = work if work is not None else solve_out_workspace(a, n, algo, layout)
    st = getattr(lib(), f"tridiag_solve_out_{p}")(
        ALGOS[algo], LAYOUTS[layout], _ptr(a, a.dtype), _ptr(b, a.dtype), _ptr(c, a.dtype), _ptr(d, a.dtype),
        _ptr(x, a.dtype), _ptr(work), work.numel(), n, batch, _stream_ptr(stream))
    check(st, f"tridiag_solve_out_{p}({algo}, {layout})")
    return x


def solve_host(a, b, c, d, n: int, algo: str = "auto", layout: str = "contiguous", out=None, chunk: int = 0,
               stream=None):
    """Out-of-place solve of host (CPU) tensors through the chunked
    host -> device -> host pipeline of tridiag_solve_host_*; returns x (a new
    page-locked tensor or ``out``), valid once ``stream`` (default: the
    current CUDA stream) has been synchronised."""
    for t in (a, b, c, d):
        if t.device.type != "cpu":
            raise ValueError("solve_host takes host tensors")
    p = _prec(a)
    batch = _dims(a, n, layout)
    a, b, c, d = (t.contiguous() for t in (a, b, c, d))
    x = out if out is not None else torch.empty(d.shape, dtype=d.dtype).pin_memory()
    st = getattr(lib(), f"tridiag_solve_host_{p}")(
        ALGOS[algo], LAYOUTS[layout], a.data_ptr(), b.data_ptr(), c.data_ptr(), d.data_ptr(), x.data_ptr(), n,
        batch, int(chunk), _stream_ptr(stream))
    check(st, f"tridiag_solve_host_{p}({algo}, {layout})")
    return x


def gtsv_workspace(a: torch.Tensor, n: int, layout: str = "contiguous") -> torch.Tensor:
    batch = _dims(a, n, layout)
    nbytes = lib().tridiag_gtsv_workspace_size(1 if a.dtype == torch.float64 else 0, LAYOUTS[layout], n, batch)
    return torch.empty(nbytes, dtype=torch.uint8, device=a.device)


def pivot_record(a: torch.Tensor, n: int, layout: str = "contiguous") -> torch.Tensor:
    batch = _dims(a, n, layout)
    nbytes = lib().tridiag_pivot_record_size(n, batch)
    return torch.empty(nbytes // 4, dtype=torch.int32, device=a.device)


def gtsv(a, b, c, d, n: int, layout: str = "contiguous", pivots=None, info=None, work=None, out=None,
         stream=None):
    """Partial-pivoting solve; a, b, c, d are not modified.  Returns x (a new
    tensor, or ``out``).  ``pivots`` (from :func:`pivot_record`) receives the
    pivot record for :func:`gtsv_adjoint`; ``info`` (int32, batch) receives
    0 or k+1 for the first zero pivot of each system.  Layout "packed": pass
    the packed tensor as ``a`` (None for b, c, d); the result is a packed
    tensor with x in rows 3n..4n of each system."""
    p = _prec(a)
    batch = _dims(a, n, layout)
    a, b, c = _al(a), _al(b), _al(c)
    if layout == "packed":
        # one packed tensor in (pass it as a, None for b, c, d); x is a copy of
        # it whose right-hand-side rows (3n..4n of each system) receive the solution
        x = out if out is not None else torch.empty_like(a, memory_format=torch.contiguous_format)
        if x.data_ptr() != a.data_ptr():
            x.copy_(a)
        xp = _ptr(x, a.dtype) + 3 * n * x.element_size()
    else:
        x = out if out is not None else torch.empty_like(d, memory_format=torch.contiguous_format)
        if x.data_ptr() != d.data_ptr():
            x.copy_(d)
        xp = _ptr(x, a.dtype)
    work = work if work is not None else gtsv_workspace(a, n, layout)
    st = getattr(lib(), f"tridiag_gtsv_{p}")(
        LAYOUTS[layout], _ptr(a, a.dtype), _ptr(b, a.dtype), _ptr(c, a.dtype), xp,
        _ptr(pivots), _ptr(info), _ptr(work), work.numel(), n, batch, _stream_ptr(stream))
    check(st, f"tridiag_gtsv_{p}")
    return x


def gtsv_adjoint(a, b, c, x, pivots, xbar, n: int, layout: str = "contiguous", work=None, stream=None):
    """Gradients (ga, gb, gc, gd) of L with dL/dx = xbar through x = A^-1 d,
    reusing the forward call's pivot record."""
    p = _prec(a)
    batch = _dims(a, n, layout)
    a, b, c, x, xbar = _al(a), _al(b), _al(c), _al(x), _al(xbar)
    ga, gb, gc, gd = (torch.empty_like(a) for _ in range(4))
    work = work if work is not None else gtsv_workspace(a, n, layout)
    st = getattr(lib(), f"tridiag_gtsv_adjoint_{p}")(
        LAYOUTS[layout], _ptr(a, a.dtype), _ptr(b, a.dtype), _ptr(c, a.dtype), _ptr(x, a.dtype), _ptr(pivots),
        _ptr(xbar, a.dtype), _ptr(ga), _ptr(gb), _ptr(gc), _ptr(gd), _ptr(work), work.numel(), n, batch,
        _stream_ptr(stream))
    check(st, f"tridiag_gtsv_adjoint_{p}")
    return ga, gb, gc, gd


def pge(a, b, c, d, n: int, layout: str = "contiguous", info=None, out=None, stream=None):
    """WM-pGE with partial pivoting inside partitions (one CTA per system);
    a, b, c, d are not modified; returns x.  Raises for sizes it does not
    cover (TRIDIAG_ERR_NOT_SUPPORTED)."""
    p = _prec(a)
    batch = _dims(a, n, layout)
    a, b, c, d = _al(a), _al(b), _al(c), _al(d)
    x = out if out is not None else torch.empty_like(d if d is not None else a)
    st = getattr(lib(), f"tridiag_pge_{p}")(LAYOUTS[layout], _ptr(a, a.dtype), _ptr(b, a.dtype), _ptr(c, a.dtype),
                                          _ptr(d, a.dtype), _ptr(x, a.dtype), _ptr(info), n, batch,
                                          _stream_ptr(stream))
    check(st, f"tridiag_pge_{p}")
    return x


def pge_adjoint(a, b, c, x, xbar, n: int, layout: str = "contiguous", info=None, stream=None):
    """Gradients (ga, gb, gc, gd) of L with dL/dx = xbar through x = A^-1 d,
    by the partitioned solve of A^T lambda = xbar (no pivot record)."""
    p = _prec(a)
    batch = _dims(a, n, layout)
    a, b, c, x, xbar = _al(a), _al(b), _al(c), _al(x), _al(xbar)
    ga, gb, gc, gd = (torch.empty_like(a) for _ in range(4))
    st = getattr(lib(), f"tridiag_pge_adjoint_{p}")(
        LAYOUTS[layout], _ptr(a, a.dtype), _ptr(b, a.dtype), _ptr(c, a.dtype), _ptr(x, a.dtype),
        _ptr(xbar, a.dtype), _ptr(ga), _ptr(gb), _ptr(gc), _ptr(gd), _ptr(info), n, batch, _stream_ptr(stream))
    check(st, f"tridiag_pge_adjoint_{p}")
    return ga, gb, gc, gd


def partition_path_counts(reset: bool = False) -> dict:
    """Paths taken by the partitioned partial-pivoting solve on the current
    device since the last reset: separator systems re-solved with pivoting,
    exact backward-error checks, refinement passes, sequential fallbacks."""
    buf = (ctypes.c_longlong * 4)()
    check(lib().tridiag_partition_path_counts(ctypes.addressof(buf), int(reset)))
    return dict(zip(("pivoted_separators", "exact_checks", "refinement_passes", "fallbacks"), list(buf)))


def ppt_counts(reset: bool = False) -> dict:
    """Systems the thread-per-partition pivoted solve (many contiguous FP64
    systems, gtsv without a pivot record) accepted, and those it handed to
    the one-CTA partitioned solve, on the current device since the last reset."""
    buf = (ctypes.c_longlong * 2)()
    check(lib().tridiag_partition_ppt_counts(ctypes.addressof(buf), int(reset)))
    return dict(zip(("accepted", "listed"), list(buf)))


def partition_supported(a, n: int, layout: str = "contiguous") -> bool:
    """Whether TRIDIAG_ALGO_PARTITION's CTA kernel covers (dtype of a, n, layout)."""
    return bool(lib().tridiag_partition_supported(1 if a.dtype == torch.float64 else 0, LAYOUTS[layout], n))


def partition_adjoint(a, b, c, x, xbar, n: int, stream=None):
    """Gradients (ga, gb, gc, gd) of L with dL/dx = xbar through x = A^-1 d by
    the unpivoted partition method on A^T (contiguous layout; systems that
    need no pivoting)."""
    p = _prec(a)
    batch = _dims(a, n, "contiguous")
    a, b, c, x, xbar = _al(a), _al(b), _al(c), _al(x), _al(xbar)
    ga, gb, gc, gd = (torch.empty_like(a) for _ in range(4))
    st = getattr(lib(), f"tridiag_partition_adjoint_{p}")(
        LAYOUTS["contiguous"], _ptr(a, a.dtype), _ptr(b, a.dtype), _ptr(c, a.dtype), _ptr(x, a.dtype),
        _ptr(xbar, a.dtype), _ptr(ga), _ptr(gb), _ptr(gc), _ptr(gd), n, batch, _stream_ptr(stream))
    check(st, f"tridiag_partition_adjoint_{p}")
    return ga, gb, gc, gd


class Factorization:
    """Partial-pivoting factors of a batch (LAPACK ?gttrf algorithm); solve
    any number of right-hand sides, transposed or not, with :meth:`solve`."""

    def __init__(self, a, b, c, n: int, layout: str = "contiguous", info=None, stream=None):
        p = _prec(a)
        self.n, self.layout, self.dtype = n, layout, a.dtype
        self.batch = _dims(a, n, layout)
        a, b, c = _al(a), _al(b), _al(c)
        nbytes = lib().tridiag_factor_size(1 if a.dtype == torch.float64 else 0, n, self.batch)
        self.factors = torch.empty(nbytes, dtype=torch.uint8, device=a.device)
        st = getattr(lib(), f"tridiag_factor_{p}")(LAYOUTS[layout], _ptr(a, a.dtype), _ptr(b, a.dtype),
                                                   _ptr(c, a.dtype), _ptr(self.factors), nbytes, _ptr(info), n,
                                                   self.batch, _stream_ptr(stream))
        check(st, f"tridiag_factor_{p}")
        self._p = p

    def solve(self, r, transpose: bool = False, stream=None):
        """Solve for r (nrhs blocks of n*batch elements, the factor's layout)
        in place; returns r."""
        nrhs = r.numel() // (self.n * self.batch)
        if nrhs * self.n * self.batch != r.numel():
            raise ValueError("r must hold whole right-hand sides")
        st = getattr(lib(), f"tridiag_factored_solve_{self._p}")(
            LAYOUTS[self.layout], int(transpose), _ptr(self.factors), self.factors.numel(), _ptr(r, self.dtype), nrhs,
            self.n, self.batch, _stream_ptr(stream))
        check(st, f"tridiag_factored_solve_{self._p}")
        return r


BLOCK2_ALGOS = {"pivoted": 0, "thomas": 1}


def block2(a, b, c, d, n: int, algo: str = "pivoted", layout: str = "contiguous", info=None, stream=None):
    """Block tridiagonal systems with 2 x 2 blocks, in place: d receives x.
    Contiguous layout: a, b, c hold (batch, n, 2, 2) blocks row-major and d
    (batch, n, 2); interleaved: a[(i*4 + k)*batch + j], d[(i*2 + r)*batch + j].
    "pivoted" (partial pivoting, the LAPACK ?gbsv algorithm) overwrites a, b,
    c with the factors; "thomas" (block Thomas, no pivoting) overwrites c.
    Returns d."""
    p = _prec(a)
    if n <= 0 or a.numel() % (4 * n) or d.numel() * 2 != a.numel() or b.numel() != a.numel() \
            or c.numel() != a.numel():
        raise ValueError("a, b, c need 4*n*batch elements and d 2*n*batch")
    batch = a.numel() // (4 * n)
    st = getattr(lib(), f"tridiag_block2_{p}")(BLOCK2_ALGOS[algo], LAYOUTS[layout], _ptr(a, a.dtype), _ptr(b, a.dtype),
                                               _ptr(c, a.dtype), _ptr(d, a.dtype), _ptr(info, torch.int32), n, batch,
                                               _stream_ptr(stream))
    check(st, f"tridiag_block2_{p}")
    return d


def periodic(a, b, c, d, n: int, algo: str = "gtsv", out=None, work=None, stream=None):
    """Periodic (cyclic) systems: a_0 couples x_{n-1}, c_{n-1} couples x_0.
    Contiguous layout; returns x."""
    p = _prec(a)
    batch = _dims(a, n, "contiguous")
    a, b, c, d = _al(a), _al(b), _al(c), _al(d)
    x = out if out is not None else torch.empty_like(d)
    if work is None:
        nbytes = lib().tridiag_periodic_workspace_size(1 if a.dtype == torch.float64 else 0, ALGOS[algo], n, batch)
        work = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=a.device)
    st = getattr(lib(), f"tridiag_periodic_{p}")(ALGOS[algo], _ptr(a, a.dtype), _ptr(b, a.dtype), _ptr(c, a.dtype),
                                                 _ptr(d, a.dtype), _ptr(x, a.dtype), _ptr(work), work.numel(), n,
                                                 batch, _stream_ptr(stream))
    check(st, f"tridiag_periodic_{p}")
    return x


def relayout(arrays, n: int, from_layout: str, to_layout: str, out=None, stream=None):
    """a, b, c, d (or one packed tensor) from one layout to another; returns
    the four destination tensors (or one packed tensor)."""
    src = list(arrays) if isinstance(arrays, (list, tuple)) else [arrays]
    t0 = src[0]
    p = _prec(t0)
    batch = _dims(t0, n, from_layout)
    if out is None:
        if to_layout == "packed":
            out = [torch.empty(batch * 4 * n, dtype=t0.dtype, device=t0.device)]
        else:
            out = [torch.empty(batch * n, dtype=t0.dtype, device=t0.device) for _ in range(4)]
    dst = list(out) if isinstance(out, (list, tuple)) else [out]
    sp = [_ptr(src[k]) if k < len(src) else None for k in range(4)]
    dp = [_ptr(dst[k]) if k < len(dst) else None for k in range(4)]
    st = getattr(lib(), f"tridiag_relayout_{p}")(LAYOUTS[from_layout], LAYOUTS[to_layout], *sp, *dp, n, batch,
                                                 _stream_ptr(stream))
    check(st, f"tridiag_relayout_{p}")
    return dst if len(dst) > 1 else dst[0]


def refine_workspace(a: torch.Tensor, n: int, layout: str = "contiguous") -> torch.Tensor:
    batch = _dims(a, n, layout)
    return torch.empty(lib().tridiag_refine_workspace_size(LAYOUTS[layout], n, batch), dtype=torch.uint8,
                       device=a.device)


def refine(a, b, c, d, n: int, iters: int = 2, layout: str = "contiguous", info=None, work=None, out=None,
           stream=None, algo: str = "gtsv"):
    """Mixed-precision solve of FP64 systems: FP32 solves (``algo`` "gtsv":
    partial pivoting; "partition": the unpivoted partition method, for
    systems that need no pivoting), ``iters`` refinement steps with the
    residual d - A x formed in FP64.  a, b, c, d (float64) are not modified;
    returns x (float64)."""
    if a.dtype != torch.float64:
        raise TypeError("refine takes float64 arrays")
    batch = _dims(a, n, layout)
    a, b, c, d = _al(a), _al(b), _al(c), _al(d)
    x = out if out is not None else torch.empty_like(d)
    work = work if work is not None else refine_workspace(a, n, layout)
    st = lib().tridiag_refine_ex_double(ALGOS[algo], LAYOUTS[layout], _ptr(a, a.dtype), _ptr(b, a.dtype),
                                        _ptr(c, a.dtype), _ptr(d, a.dtype), _ptr(x, a.dtype), iters, _ptr(info),
                                        _ptr(work), work.numel(), n, batch, _stream_ptr(stream))
    check(st, "tridiag_refine_ex_double")
    return x


def convert_check(v: torch.Tensor):
    """(float32 narrowing, float64 widening of it) as the refined solve computes them."""
    out = torch.empty(v.numel(), dtype=torch.float32, device=v.device)
    back = torch.empty(v.numel(), dtype=torch.float64, device=v.device)
    check(lib().tridiag_convert_check(_ptr(v, torch.float64), _ptr(out), _ptr(back), v.numel(), _stream_ptr()),
          "tridiag_convert_check")
    return out, back


def reference_call(name: str, a, b, c, d, n: int):
    """Call one of the reference's entry points (e.g. "WM5_reg_double") on
    layout-0 tensors; synchronous like the reference.  Returns d."""
    batch = _dims(a, n, "contiguous")
    f = getattr(lib(), name)
    f(_ptr(a), _ptr(b), _ptr(c), _ptr(d), n, batch)
    check(_lib.last_status(), name)
    return d
