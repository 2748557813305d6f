"""Ragged batches and the per-size-class autotuner.

A ragged batch packs systems of different sizes back to back: system s is
rows ``offsets[s] .. offsets[s+1]-1`` of the 1-D tensors a, b, c, d.  A
:class:`RaggedPlan` (built once on the host from the offsets) groups the
systems into size classes and picks a kernel variant per class; its
:meth:`~RaggedPlan.solve` and :meth:`~RaggedPlan.adjoint` issue one launch
per bucket on the current stream, so the whole call can be captured in one
CUDA graph.  With ``classify=True`` the library itself finds, in each solve,
the systems that need no pivoting (strictly diagonally dominant) and runs
them by the unpivoted partition method, the others by the pivoted variants.
:func:`autotune` measures the pivoted variants on synthetic batches of each
class and returns the fastest per class (the table a plan takes);
:func:`autotune_unpivoted` does the same for the unpivoted systems' variant
and the chunk width of long ones.
"""
from __future__ import annotations

import ctypes
import json
import math
from pathlib import Path

import numpy as np
import torch

from ._lib import TridiagError, check, lib
from .ops import _ptr, _stream_ptr

CLASSES = 18            # TRIDIAG_RAGGED_CLASSES: class k holds 2^(k-1) < n <= 2^k
VARIANTS = {0: "sequential (thread per system)", 1: "partitioned, 1 CTA x 64", 2: "partitioned, 1 CTA x 128",
            3: "partitioned, 1 CTA x 256", 4: "partitioned, cluster of 2", 5: "partitioned, cluster of 4",
            6: "partitioned, cluster of 8", 7: "unpivoted partition method (systems marked no_pivoting)",
            8: "unpivoted partition method, chunked (long systems marked no_pivoting)",
            9: "sequential (thread per system), rows in a workspace: any n",
            10: "partitioned, chunks of 4224 rows per CTA, separators' system in between"}
_P = ctypes.c_void_p


def _sig():
    return lib()


def size_class(n: int) -> int:
    return max(0, math.ceil(math.log2(n))) if n > 1 else 0


def variant_max_n(precision: int, variant: int) -> int:
    return _sig().tridiag_ragged_variant_max_n(precision, variant)


class RaggedPlan:
    """Plan for a ragged batch; ``offsets`` (int64, batch+1 entries) on the
    host or device; ``table`` maps size class -> variant (None: defaults);
    ``no_pivoting`` (bool per system, optional) marks systems that need no
    pivoting (diagonally dominant, say), which then run the unpivoted
    partition method where their size allows; ``classify=True`` lets each
    solve find those systems itself (``unpivoted_table``: class -> variant of
    the unpivoted systems, ``chunk_rows``: 128-byte rows per CTA of long
    ones; the adjoint reuses the marks of the last solve)."""

    def __init__(self, offsets, dtype=torch.float32, table: dict | None = None, device=None, no_pivoting=None,
                 classify: bool = False, unpivoted_table: dict | None = None, chunk_rows: int = 0):
        L = _sig()
        off = offsets.detach().cpu().numpy() if isinstance(offsets, torch.Tensor) else np.asarray(offsets)
        off = np.ascontiguousarray(off, dtype=np.int64)
        self.batch = off.size - 1
        self.precision = 1 if dtype == torch.float64 else 0
        self.dtype = dtype
        tab = np.full(CLASSES, -1, dtype=np.int32)
        for k, v in (table or {}).items():
            tab[int(k)] = int(v)
        self._tab = tab
        h = _P()
        if classify:
            if no_pivoting is not None:
                raise ValueError("classify and no_pivoting exclude each other")
            utab = np.full(CLASSES, -1, dtype=np.int32)
            for k, v in (unpivoted_table or {}).items():
                utab[int(k)] = int(v)
            st = L.tridiag_ragged_plan_create_classify(ctypes.addressof(h), self.precision, off.ctypes.data,
                                                       self.batch, tab.ctypes.data, utab.ctypes.data, CLASSES,
                                                       int(chunk_rows))
        elif no_pivoting is None:
            st = L.tridiag_ragged_plan_create(ctypes.addressof(h), self.precision, off.ctypes.data, self.batch,
                                              tab.ctypes.data, CLASSES)
        else:
            mask = np.ascontiguousarray(np.asarray(no_pivoting, dtype=np.uint8).reshape(-1))
            if mask.size != self.batch:
                raise ValueError("no_pivoting needs one entry per system")
            st = L.tridiag_ragged_plan_create_ex(ctypes.addressof(h), self.precision, off.ctypes.data, self.batch,
                                                 tab.ctypes.data, CLASSES, mask.ctypes.data)
        check(st, "tridiag_ragged_plan_create")
        self._h = h
        dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.offsets = torch.from_numpy(off).to(dev)
        self.rows = int(off[-1] - off[0])

    def kinds(self):
        """Per system: True where the last solve ran it without pivoting
        (synchronous)."""
        out = np.zeros(self.batch, dtype=np.uint8)
        check(_sig().tridiag_ragged_plan_kinds(self._h, out.ctypes.data), "tridiag_ragged_plan_kinds")
        return out.astype(bool)

    def buckets(self):
        """[(class, variant, systems, largest n)], longest class first (for a
        bucket of one kind, systems = the room of its list)."""
        L = _sig()
        out = np.zeros(4 * 3 * CLASSES, dtype=np.int32)  # pivoted and unpivoted buckets per class
        nb = min(L.tridiag_ragged_plan_buckets(self._h, out.ctypes.data, 3 * CLASSES), 3 * CLASSES)
        return [tuple(int(v) for v in out[4 * i:4 * i + 4]) for i in range(nb)]

    def solve(self, a, b, c, d, out=None, info=None, stream=None):
        p = "double" if self.precision else "single"
        x = out if out is not None else torch.empty_like(d)
        st = getattr(_sig(), f"tridiag_ragged_solve_{p}")(self._h, _ptr(a, self.dtype), _ptr(b, self.dtype),
                                                          _ptr(c, self.dtype), _ptr(d, self.dtype),
                                                          _ptr(x, self.dtype), _ptr(info), _ptr(self.offsets),
                                                          _stream_ptr(stream))
        check(st, f"tridiag_ragged_solve_{p}")
        return x

    def adjoint(self, a, b, c, x, xbar, grads=None, info=None, stream=None):
        """(ga, gb, gc, gd) of L with dL/dx = xbar through x = A^-1 d."""
        p = "double" if self.precision else "single"
        ga, gb, gc, gd = grads if grads is not None else (torch.empty_like(x) for _ in range(4))
        st = getattr(_sig(), f"tridiag_ragged_adjoint_{p}")(
            self._h, _ptr(a, self.dtype), _ptr(b, self.dtype), _ptr(c, self.dtype), _ptr(x, self.dtype),
            _ptr(xbar, self.dtype), _ptr(ga), _ptr(gb), _ptr(gc), _ptr(gd), _ptr(info), _ptr(self.offsets),
            _stream_ptr(stream))
        check(st, f"tridiag_ragged_adjoint_{p}")
        return ga, gb, gc, gd

    def refine_workspace(self):
        """Workspace of :meth:`refine` / :meth:`refine_adjoint` (uint8 tensor)."""
        nbytes = _sig().tridiag_ragged_refine_workspace_size(self.rows)
        return torch.empty(nbytes, dtype=torch.uint8, device=self.offsets.device)

    def refine(self, a, b, c, d, iters=1, out=None, work=None, stream=None, pivoted_iters=0):
        """FP64 systems (a, b, c, d float64) solved through this FP32 plan
        with `iters` FP64-residual refinement steps, then `pivoted_iters`
        more on the systems the plan solves with pivoting only; returns x
        (float64)."""
        if self.precision != 0:
            raise ValueError("refine runs through an FP32 plan")
        x = out if out is not None else torch.empty_like(d)
        work = work if work is not None else self.refine_workspace()
        D = torch.float64
        st = _sig().tridiag_ragged_refine_ex_double(self._h, _ptr(a, D), _ptr(b, D), _ptr(c, D), _ptr(d, D),
                                                    _ptr(x, D), int(iters), int(pivoted_iters), _ptr(work),
                                                    work.numel(), _ptr(self.offsets), _stream_ptr(stream))
        check(st, "tridiag_ragged_refine_ex_double")
        return x

    def refine_adjoint(self, a, b, c, x, xbar, iters=1, grads=None, work=None, stream=None, pivoted_iters=0):
        """(ga, gb, gc, gd) in FP64 of L with dL/dx = xbar through x = A^-1 d,
        lambda = A^-T xbar by the refined solve of A^T through this FP32 plan
        (`iters` steps, then `pivoted_iters` on the pivoted systems only)."""
        if self.precision != 0:
            raise ValueError("refine_adjoint runs through an FP32 plan")
        ga, gb, gc, gd = grads if grads is not None else (torch.empty_like(x) for _ in range(4))
        work = work if work is not None else self.refine_workspace()
        D = torch.float64
        st = _sig().tridiag_ragged_refine_adjoint_ex_double(
            self._h, _ptr(a, D), _ptr(b, D), _ptr(c, D), _ptr(x, D), _ptr(xbar, D), _ptr(ga, D), _ptr(gb, D),
            _ptr(gc, D), _ptr(gd, D), int(iters), int(pivoted_iters), _ptr(work), work.numel(), _ptr(self.offsets),
            _stream_ptr(stream))
        check(st, "tridiag_ragged_refine_adjoint_ex_double")
        return ga, gb, gc, gd

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                _sig().tridiag_ragged_plan_destroy(h)
            except Exception:
                pass
            self._h = None


def synthetic_batch(sizes, dtype=torch.float32, nondominant_fraction=0.2, seed=0, device="cuda"):
    """Packed arrays for systems of the given sizes: a, c, d ~ U[-1, 1]
    (a_0 = c_{n-1} = 0); b = |a| + |c| + U[1, 2] for dominant systems, b ~
    U[-1, 1] for the non-dominant fraction (chosen per system)."""
    sizes = np.asarray(sizes, dtype=np.int64)
    off = np.zeros(sizes.size + 1, dtype=np.int64)
    np.cumsum(sizes, out=off[1:])
    N = int(off[-1])
    g = torch.Generator(device=device)
    g.manual_seed(seed)

    def u(lo, hi):
        return torch.rand(N, dtype=dtype, device=device, generator=g) * (hi - lo) + lo

    a, c, d = u(-1, 1), u(-1, 1), u(-1, 1)
    offs = torch.from_numpy(off).to(device)
    a[offs[:-1]] = 0
    c[offs[1:] - 1] = 0
    rng = np.random.default_rng(seed + 1)
    nondom = rng.random(sizes.size) < nondominant_fraction
    row_sys = torch.repeat_interleave(torch.arange(sizes.size, device=device), torch.from_numpy(sizes).to(device))
    nd_rows = torch.from_numpy(nondom).to(device)[row_sys]
    b = torch.where(nd_rows, u(-1, 1), a.abs() + c.abs() + u(1, 2))
    return a, b, c, d, off, nondom


def log_uniform_sizes(count: int, lo: int = 32, hi: int = 65536, seed: int = 0):
    rng = np.random.default_rng(seed)
    return np.rint(np.exp(rng.uniform(math.log(lo), math.log(hi), count))).astype(np.int64)


def _time(fn, reps=3):
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())  # the inputs were made on the caller's stream
    with torch.cuda.stream(s):
        fn()
        s.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(reps):
            fn()
        e1.record(s)
        s.synchronize()
    return e0.elapsed_time(e1) / reps


def candidates(precision: int, cls: int):
    """Variants that serve every n of size class cls (2^(cls-1) < n <= 2^cls)."""
    lo, hi = 2 ** (cls - 1) + 1 if cls > 0 else 1, 2 ** cls
    out = [0] if hi <= 64 else []
    if lo >= 65:
        out += [v for v in range(1, 7) if variant_max_n(precision, v) >= hi]
    if not out and lo >= 65:
        out = ([10] if variant_max_n(precision, 10) >= hi else []) + [9]
    return out or [9]


def autotune(classes, dtype=torch.float32, systems_per_class=None, rows_per_class=2 ** 24, seed=0, reps=3,
             verbose=False):
    """Time every candidate variant on a synthetic batch of each size class
    (sizes log-uniform inside the class, 20% non-dominant systems) and
    return {class: fastest variant} plus the timings."""
    precision = 1 if dtype == torch.float64 else 0
    table, timings = {}, {}
    for k in classes:
        cands = candidates(precision, k)
        if len(cands) <= 1:
            if cands:
                table[k] = cands[0]
            continue
        lo, hi = max(2 ** (k - 1) + 1, 2), 2 ** k
        count = systems_per_class or max(64, min(20000, rows_per_class // hi))
        sizes = log_uniform_sizes(count, lo, hi, seed=seed + k)
        a, b, c, d, off, _ = synthetic_batch(sizes, dtype=dtype, seed=seed + k)
        x = torch.empty_like(d)
        res = {}
        for v in cands:
            plan = RaggedPlan(off, dtype=dtype, table={k: v})
            if plan.buckets()[0][1] != v:
                continue
            res[v] = _time(lambda: plan.solve(a, b, c, d, out=x), reps)
            del plan
        if res:
            table[k] = min(res, key=res.get)
            timings[k] = res
            if verbose:
                print(f"class {k:2d} (n <= {hi:6d}, {count} systems): " +
                      ", ".join(f"v{v} {t:.3f} ms" for v, t in sorted(res.items())) + f" -> v{table[k]}")
        del a, b, c, d, x
    return table, timings


def autotune_unpivoted(classes, dtype=torch.float32, rows_per_class=2 ** 24, seed=0, reps=3, verbose=False):
    """For the systems that need no pivoting: per size class up to the
    one-CTA limit, time variant 7 against the partitioned pivoted variants
    that serve the class; for the longer classes, time the chunk widths 64 /
    128 / 256 (128-byte rows per CTA) of variant 8.  Synthetic batches of
    dominant systems, sizes log-uniform inside each class, through classified
    plans.  Returns ({class: variant}, chunk_rows, timings)."""
    precision = 1 if dtype == torch.float64 else 0
    unp_max = variant_max_n(precision, 7)
    table, timings = {}, {}
    long_classes = []
    for k in classes:
        lo, hi = max(2 ** (k - 1) + 1, 2), 2 ** k
        if hi <= 64:
            continue
        if hi > unp_max:
            long_classes.append(k)
            continue
        count = max(64, min(20000, rows_per_class // hi))
        sizes = log_uniform_sizes(count, lo, hi, seed=seed + k)
        a, b, c, d, off, _ = synthetic_batch(sizes, dtype=dtype, nondominant_fraction=0.0, seed=seed + k)
        x = torch.empty_like(d)
        res = {}
        for v in [7] + [v for v in range(1, 7) if variant_max_n(precision, v) >= hi]:
            plan = RaggedPlan(off, dtype=dtype, classify=True, unpivoted_table={k: v})
            res[v] = _time(lambda: plan.solve(a, b, c, d, out=x), reps)
            del plan
        table[k] = min(res, key=res.get)
        timings[k] = res
        if verbose:
            print(f"class {k:2d} (n <= {hi:6d}, unpivoted): " +
                  ", ".join(f"v{v} {t:.3f} ms" for v, t in sorted(res.items())) + f" -> v{table[k]}")
        del a, b, c, d, x
    chunk = 0
    if long_classes:
        sizes = np.concatenate([log_uniform_sizes(max(16, min(4000, rows_per_class // 2 ** k)), 2 ** (k - 1) + 1,
                                                  2 ** k, seed=seed + k) for k in long_classes])
        a, b, c, d, off, _ = synthetic_batch(sizes, dtype=dtype, nondominant_fraction=0.0, seed=seed + 99)
        x = torch.empty_like(d)
        res = {}
        for r in (64, 128, 256):
            plan = RaggedPlan(off, dtype=dtype, classify=True, chunk_rows=r)
            res[r] = _time(lambda: plan.solve(a, b, c, d, out=x), reps)
            del plan
        chunk = min(res, key=res.get)
        timings["chunk_rows"] = res
        if verbose:
            print("long unpivoted classes " + str(long_classes) + ": " +
                  ", ".join(f"{r} rows {t:.3f} ms" for r, t in sorted(res.items())) + f" -> {chunk}")
        del a, b, c, d, x
    return table, chunk, timings


def save_table(path, table, dtype=torch.float32, timings=None, unpivoted=None, chunk_rows=0):
    """Persist the autotuner's choices (and timings) as JSON."""
    doc = {"device": torch.cuda.get_device_name(), "dtype": str(dtype).replace("torch.", ""),
           "table": {str(k): int(v) for k, v in table.items()},
           "unpivoted": {str(k): int(v) for k, v in (unpivoted or {}).items()}, "chunk_rows": int(chunk_rows),
           "timings_ms": {str(k): ({str(v): t for v, t in r.items()} if isinstance(r, dict) else r)
                          for k, r in (timings or {}).items()}}
    Path(path).write_text(json.dumps(doc, indent=1))


def load_table(path, full: bool = False):
    """The table saved by :func:`save_table` ({class: variant}); with
    full=True also the unpivoted table and chunk width."""
    doc = json.loads(Path(path).read_text())
    table = {int(k): int(v) for k, v in doc["table"].items()}
    if not full:
        return table
    return table, {int(k): int(v) for k, v in doc.get("unpivoted", {}).items()}, int(doc.get("chunk_rows", 0))


__all__ = ["RaggedPlan", "autotune", "autotune_unpivoted", "candidates", "load_table", "log_uniform_sizes", "save_table",
           "synthetic_batch", "size_class", "variant_max_n", "TridiagError", "CLASSES", "VARIANTS"]


def _main() -> None:
    """python -m tridiagonalsolver_gb300.ragged --tune PATH: autotune the
    pivoted variants, the unpivoted variants and the chunk width over the
    size classes of the log-uniform [32, 65536] workload on this GPU and save
    the table (load it with load_table(PATH, full=True))."""
    import argparse

    ap = argparse.ArgumentParser(description=_main.__doc__)
    ap.add_argument("--tune", required=True, help="output JSON path")
    ap.add_argument("--dtype", default="float32", choices=["float32", "float64"])
    ap.add_argument("--reps", type=int, default=3)
    args = ap.parse_args()
    dt = getattr(torch, args.dtype)
    classes = sorted({size_class(int(v)) for v in log_uniform_sizes(100000, 32, 65536, seed=2024)})
    table, timings = autotune(classes, dtype=dt, reps=args.reps, verbose=True)
    utab, chunk, ut = autotune_unpivoted(classes, dtype=dt, reps=args.reps, verbose=True)
    timings.update({f"unpivoted_{k}": v for k, v in ut.items()})
    save_table(args.tune, table, dtype=dt, timings=timings, unpivoted=utab, chunk_rows=chunk)
    print("saved", args.tune)


if __name__ == "__main__":
    _main()
