"""Ragged batches (systems of different sizes packed back to back): the
size-class plan, forward and adjoint against the oracle per system, CUDA
graph capture, the autotuner, and the full ragged workload (100000 systems,
sizes log-uniform in [32, 65536], FP32, 20% non-dominant).

Tolerances: normwise backward error <= 1e-6 (FP32) / 1e-12 (FP64) per
system, for the forward solve and for the adjoint's transposed solve
A^T lambda = xbar; on diagonally dominant systems (well conditioned) the
gradients are within 2e-3 (FP32) / 1e-9 (FP64) of the FP64 oracle adjoint,
relative to the system's largest gradient entry.  (On the non-dominant
systems the conditioning reaches 1e7, where FP32 gradients carry that
relative error; the backward-error bound is the meaningful check there.)
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

ETA = {"float32": 1e-6, "float64": 1e-12}
GTOL = {"float32": 2e-3, "float64": 1e-9}


def _sizes(max_n):
    """Every size class from 1 up to max_n, a few systems each, plus edges."""
    rng = np.random.default_rng(3)
    out = [1, 2, 3, 31, 32, 33, 63, 64, 65, 66, 127, 128, 129]
    k = 8
    while 2 ** (k - 1) < max_n:
        lo, hi = 2 ** (k - 1) + 1, min(2 ** k, max_n)
        out += list(rng.integers(lo, hi + 1, 2)) + [hi]
        k += 1
    return np.array(out, dtype=np.int64)


def _host(t, off, s):
    return t[int(off[s]):int(off[s + 1])].double().cpu().numpy()[None, :]


def _transposed(a, c):
    """Coefficients of A^T: sub-diagonal c_{i-1}, super-diagonal a_{i+1}."""
    at = np.zeros_like(a)
    ct = np.zeros_like(c)
    at[:, 1:] = c[:, :-1]
    ct[:, :-1] = a[:, 1:]
    return at, ct


def _check_system(hs, grads, n, dominant, eta_tol, g_tol):
    a, b, c, d, x, w = hs
    _, eta = O.backward_error(a, b, c, d, x, n)
    assert eta <= eta_tol, ("forward", n, eta)
    lam = grads[3]
    at, ct = _transposed(a, c)
    _, eta_t = O.backward_error(at, b, ct, w, lam, n)
    assert eta_t <= eta_tol, ("adjoint", n, eta_t)
    if dominant and n >= 2:
        ref = O.adjoint_f64(a, b, c, x, w, n)
        for g, r in zip(grads, ref):
            scale = np.max(np.abs(r)) + 1e-300
            assert np.max(np.abs(g[0] - r)) / scale <= g_tol, ("gradient", n)


@pytest.mark.parametrize("dtype_name,max_n", [("float32", 65536), ("float64", 27648)])
def test_ragged_forward_and_adjoint(cuda, dtype_name, max_n):
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300 import ragged

    torch = cuda
    dt = getattr(torch, dtype_name)
    sizes = _sizes(max_n)
    a, b, c, d, off, nondom = ragged.synthetic_batch(sizes, dtype=dt, nondominant_fraction=0.3, seed=1)
    plan = T.RaggedPlan(off, dtype=dt)
    variants = {v for _, v, _, _ in plan.buckets()}
    assert 0 in variants and len(variants) >= 4
    info = torch.full((len(sizes),), -7, dtype=torch.int32, device="cuda")
    x = plan.solve(a, b, c, d, info=info)
    w = torch.rand_like(d) * 2 - 1
    ga, gb, gc, gd = plan.adjoint(a, b, c, x, w)
    torch.cuda.synchronize()
    assert int((info != 0).sum()) == 0
    for s in range(len(sizes)):
        n = int(sizes[s])
        hs = [_host(t, off, s) for t in (a, b, c, d, x, w)]
        grads = [_host(g, off, s) for g in (ga, gb, gc, gd)]
        _check_system(hs, grads, n, not nondom[s], ETA[dtype_name], GTOL[dtype_name])


def test_ragged_graph_capture(cuda):
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300 import ragged

    torch = cuda
    sizes = ragged.log_uniform_sizes(500, 32, 20000, seed=4)
    a, b, c, d, off, _ = ragged.synthetic_batch(sizes, seed=4)
    plan = T.RaggedPlan(off)
    x = torch.empty_like(d)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())  # inputs were made on the current stream
    with torch.cuda.stream(s):
        plan.solve(a, b, c, d, out=x)
    s.synchronize()
    ref = x.clone()
    x.zero_()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        plan.solve(a, b, c, d, out=x)
    with torch.cuda.stream(s):
        g.replay()
    s.synchronize()
    assert torch.equal(x, ref)


def test_ragged_plan_table_and_autotune(cuda):
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300 import ragged

    torch = cuda
    for k in range(0, 17):
        for v in ragged.candidates(0, k):
            hi = 2 ** k
            assert ragged.variant_max_n(0, v) >= hi
    table, timings = ragged.autotune([6, 10, 14], dtype=torch.float32, systems_per_class=256, reps=2)
    assert set(table) == {6, 10, 14}
    for k, v in table.items():
        assert v in ragged.candidates(0, k)
    assert len(timings[10]) >= 2
    sizes = np.array([50, 700, 9000, 12000], dtype=np.int64)
    plan = T.RaggedPlan(np.concatenate([[0], np.cumsum(sizes)]), table=table)
    got = {cls: var for cls, var, _, _ in plan.buckets()}
    assert got[14] == table[14] and got[10] == table[10]
    # a variant that cannot serve a class is refused
    with pytest.raises(T.TridiagError):
        T.RaggedPlan(np.array([0, 30000]), table={15: 1})


@pytest.mark.parametrize("routing", ["pivoted", "caller_mask", "classify"])
def test_ragged_full_workload(cuda, routing):
    """100000 systems, n log-uniform in [32, 65536] (~8.6e8 rows), FP32, 20%
    non-dominant: forward and adjoint; 40 sampled systems checked.  Routing:
    every system pivoted; the dominant systems marked by the caller; or
    found by the library itself (its marks must equal the generator's)."""
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300 import ragged

    torch = cuda
    sizes = ragged.log_uniform_sizes(100000, 32, 65536, seed=2024)
    a, b, c, d, off, nondom = ragged.synthetic_batch(sizes, seed=2024)
    plan = T.RaggedPlan(off, no_pivoting=~nondom if routing == "caller_mask" else None,
                        classify=routing == "classify")
    info = torch.full((len(sizes),), -7, dtype=torch.int32, device="cuda")
    x = plan.solve(a, b, c, d, info=info)
    w = torch.rand_like(d) * 2 - 1
    ga, gb, gc, gd = plan.adjoint(a, b, c, x, w)
    torch.cuda.synchronize()
    assert int((info != 0).sum()) == 0
    if routing == "classify":
        np.testing.assert_array_equal(plan.kinds(), ~nondom & (sizes > 64))
    rng = np.random.default_rng(7)
    pick = list(rng.choice(len(sizes), 36, replace=False)) + list(np.argsort(sizes)[-4:])
    for s in pick:
        n = int(sizes[s])
        hs = [_host(t, off, s) for t in (a, b, c, d, x, w)]
        grads = [_host(g, off, s) for g in (ga, gb, gc, gd)]
        _check_system(hs, grads, n, not nondom[s], 1e-6, 2e-3)


@pytest.mark.parametrize("dtype_name,max_n", [("float32", 65536), ("float64", 27648)])
def test_ragged_unpivoted_buckets(cuda, dtype_name, max_n):
    """Systems marked as needing no pivoting (the dominant ones here) run the
    unpivoted partition method (variant 7) up to its size limit, the rest
    the pivoted variants; forward and adjoint checked per system."""
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300 import ragged

    torch = cuda
    dt = getattr(torch, dtype_name)
    sizes = _sizes(max_n)
    a, b, c, d, off, nondom = ragged.synthetic_batch(sizes, dtype=dt, nondominant_fraction=0.3, seed=5)
    plan = T.RaggedPlan(off, dtype=dt, no_pivoting=~nondom)
    limit = T.lib().tridiag_ragged_variant_max_n(1 if dtype_name == "float64" else 0, 7)
    buckets = plan.buckets()
    assert any(v == 7 for _, v, _, _ in buckets)
    if max_n > limit:
        assert any(v == 8 for _, v, _, _ in buckets)
    assert all(mx <= limit for _, v, _, mx in buckets if v == 7)
    info = torch.full((len(sizes),), -7, dtype=torch.int32, device="cuda")
    x = plan.solve(a, b, c, d, info=info)
    w = torch.rand_like(d) * 2 - 1
    ga, gb, gc, gd = plan.adjoint(a, b, c, x, w)
    torch.cuda.synchronize()
    assert int((info != 0).sum()) == 0
    for s in range(len(sizes)):
        n = int(sizes[s])
        hs = [_host(t, off, s) for t in (a, b, c, d, x, w)]
        grads = [_host(g, off, s) for g in (ga, gb, gc, gd)]
        _check_system(hs, grads, n, not nondom[s], ETA[dtype_name], GTOL[dtype_name])


def _capable(sizes, dtype_name):
    """Sizes the unpivoted method serves (64 < n <= 262144 FP32 / 65536 FP64)."""
    top = 262144 if dtype_name == "float32" else 65536
    return (sizes > 64) & (sizes <= top)


@pytest.mark.parametrize("chunk_rows", [0, 64, 256])
@pytest.mark.parametrize("dtype_name,max_n", [("float32", 65536), ("float64", 27648)])
def test_ragged_classified(cuda, dtype_name, max_n, chunk_rows):
    """The library finds the systems that need no pivoting itself (the
    unpivoted kernels check the rows they stage and hand the others to the
    pivoted buckets): its marks equal the generator's truth (strictly
    dominant rows vs b ~ U[-1, 1]) on every size the unpivoted method serves;
    forward and adjoint checked per system; the adjoint reuses the marks."""
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300 import ragged

    torch = cuda
    dt = getattr(torch, dtype_name)
    sizes = _sizes(max_n)
    a, b, c, d, off, nondom = ragged.synthetic_batch(sizes, dtype=dt, nondominant_fraction=0.3, seed=11)
    plan = T.RaggedPlan(off, dtype=dt, classify=True, chunk_rows=chunk_rows)
    info = torch.full((len(sizes),), -7, dtype=torch.int32, device="cuda")
    x = plan.solve(a, b, c, d, info=info)
    w = torch.rand_like(d) * 2 - 1
    ga, gb, gc, gd = plan.adjoint(a, b, c, x, w)
    torch.cuda.synchronize()
    assert int((info != 0).sum()) == 0
    np.testing.assert_array_equal(plan.kinds(), ~nondom & _capable(sizes, dtype_name))
    for s in range(len(sizes)):
        n = int(sizes[s])
        hs = [_host(t, off, s) for t in (a, b, c, d, x, w)]
        grads = [_host(g, off, s) for g in (ga, gb, gc, gd)]
        _check_system(hs, grads, n, not nondom[s], ETA[dtype_name], GTOL[dtype_name])


def test_ragged_classified_adjoint_first(cuda):
    """An adjoint before any solve of a classifying plan marks the systems in
    a pass of its own; gradients checked against a plan given the truth."""
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300 import ragged

    torch = cuda
    sizes = _sizes(20000)
    a, b, c, d, off, nondom = ragged.synthetic_batch(sizes, nondominant_fraction=0.3, seed=15)
    x = T.RaggedPlan(off, no_pivoting=~nondom).solve(a, b, c, d)
    w = torch.rand_like(d) * 2 - 1
    plan = T.RaggedPlan(off, classify=True)
    ga, gb, gc, gd = plan.adjoint(a, b, c, x, w)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(plan.kinds(), ~nondom & _capable(sizes, "float32"))
    for s in range(len(sizes)):
        n = int(sizes[s])
        hs = [_host(t, off, s) for t in (a, b, c, d, x, w)]
        grads = [_host(g, off, s) for g in (ga, gb, gc, gd)]
        _check_system(hs, grads, n, not nondom[s], ETA["float32"], GTOL["float32"])


def test_ragged_classified_marks_follow_coefficients(cuda):
    """A second solve with other coefficients marks the systems again: rows
    made non-dominant move their systems to the pivoted buckets."""
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300 import ragged

    torch = cuda
    sizes = np.array([100, 700, 3000, 5000, 9000, 200, 40], dtype=np.int64)
    a, b, c, d, off, _ = ragged.synthetic_batch(sizes, nondominant_fraction=0.0, seed=12)
    plan = T.RaggedPlan(off, classify=True)
    plan.solve(a, b, c, d)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(plan.kinds(), sizes > 64)
    b2 = b.clone()
    for s in (1, 4):  # one row of systems 1 and 4 no longer dominant
        r = int(off[s]) + int(sizes[s]) // 2
        b2[r] = 0.5 * (a[r].abs() + c[r].abs())
    x2 = plan.solve(a, b2, c, d)
    torch.cuda.synchronize()
    expect = sizes > 64
    expect[[1, 4]] = False
    np.testing.assert_array_equal(plan.kinds(), expect)
    for s in range(len(sizes)):
        hs = [_host(t, off, s) for t in (a, b2, c, d, x2)]
        _, eta = O.backward_error(*hs, int(sizes[s]))
        assert eta <= 1e-6


def test_ragged_classified_graph_capture(cuda):
    """The resets, every bucket and the hand-overs in one CUDA graph: two
    replays give the eager call's bits, forward and adjoint."""
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300 import ragged

    torch = cuda
    sizes = ragged.log_uniform_sizes(2000, 32, 40000, seed=13)
    a, b, c, d, off, _ = ragged.synthetic_batch(sizes, seed=13)
    plan = T.RaggedPlan(off, classify=True)
    x = torch.empty_like(d)
    w = torch.rand_like(d) * 2 - 1
    grads = [torch.empty_like(d) for _ in range(4)]
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        plan.solve(a, b, c, d, out=x, stream=s)
        plan.adjoint(a, b, c, x, w, grads=grads, stream=s)
    s.synchronize()
    ref = [x.clone()] + [g.clone() for g in grads]
    for t in [x] + grads:
        t.zero_()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        plan.solve(a, b, c, d, out=x, stream=s)
        plan.adjoint(a, b, c, x, w, grads=grads, stream=s)
    with torch.cuda.stream(s):
        g.replay()
        g.replay()
    s.synchronize()
    for got, want in zip([x] + grads, ref):
        assert torch.equal(got, want)


def test_ragged_autotune_unpivoted(cuda):
    """The unpivoted autotuner: a variant per one-CTA class (7 or a pivoted
    one that serves the class), a chunk width for the long classes; the plan
    built from its output solves correctly."""
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300 import ragged

    torch = cuda
    table, chunk, timings = ragged.autotune_unpivoted([8, 12, 14], rows_per_class=2 ** 20, reps=1)
    assert set(table) == {8, 12}
    # (timing decides: any variant that serves the class)
    assert table[8] in (7, 1, 2, 3, 4, 5, 6) and table[12] in (7, 1, 2, 3, 4, 5, 6)
    assert chunk in (64, 128, 256) and set(timings["chunk_rows"]) == {64, 128, 256}
    sizes = np.array([150, 3000, 12000, 70], dtype=np.int64)
    a, b, c, d, off, _ = ragged.synthetic_batch(sizes, nondominant_fraction=0.0, seed=14)
    plan = T.RaggedPlan(off, classify=True, unpivoted_table=table, chunk_rows=chunk)
    x = plan.solve(a, b, c, d)
    torch.cuda.synchronize()
    for s in range(len(sizes)):
        hs = [_host(t, off, s) for t in (a, b, c, d, x)]
        _, eta = O.backward_error(*hs, int(sizes[s]))
        assert eta <= 1e-6


@pytest.mark.parametrize("iters,shape", [(1, "classes"), (2, "classes"), (1, "short"), (3, "classes")])
def test_ragged_refined_forward_and_adjoint(cuda, iters, shape):
    """FP64 ragged systems solved through an FP32 classified plan with FP64
    residual refinement, forward and adjoint: on diagonally dominant systems
    of every size class up to 20000 rows, normwise backward error <= 1e-12 per
    system for x and for lambda (A^T lambda = xbar), gradients within 1e-10
    of the FP64 oracle adjoint (relative to the system's largest entry)."""
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300 import ragged

    torch = cuda
    if shape == "classes":
        sizes = _sizes(20000)
    else:  # many boundaries in one 32-row step, and systems across the 2048-row chunks of the row passes
        sizes = np.array([1] * 40 + [2] * 20 + [3, 5000, 1, 1, 31, 33, 2047, 2049, 4096] + [1] * 33, dtype=np.int64)
    a, b, c, d, off, _ = ragged.synthetic_batch(sizes, dtype=torch.float64, nondominant_fraction=0.0, seed=21)
    plan32 = T.RaggedPlan(off, dtype=torch.float32, classify=True)
    x = plan32.refine(a, b, c, d, iters=iters)
    w = torch.rand_like(d) * 2 - 1
    ga, gb, gc, gd = plan32.refine_adjoint(a, b, c, x, w, iters=iters)
    torch.cuda.synchronize()
    for s in range(len(sizes)):
        n = int(sizes[s])
        hs = [_host(t, off, s) for t in (a, b, c, d, x, w)]
        grads = [_host(g, off, s) for g in (ga, gb, gc, gd)]
        _check_system(hs, grads, n, True, 1e-12, 1e-10)


@pytest.mark.parametrize("shape", ["classes", "long"])
def test_ragged_refined_pivoted_steps(cuda, shape):
    """The refinement steps restricted to the systems the plan solves with
    pivoting (iters = 1, pivoted_iters = 1) on a batch with 30% non-dominant
    systems: normwise backward error <= 1e-12 for x and lambda on every
    system; the systems marked for the unpivoted kernels keep the one-step
    result exactly and the pivoted ones get the two-step result exactly (the
    same arithmetic per system), forward and adjoint."""
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300 import ragged

    torch = cuda
    if shape == "classes":
        sizes = _sizes(20000)
    else:  # long systems: the chunked kernels of both kinds, and systems sharing the row passes' chunks
        sizes = np.array([40000, 3, 70000, 2049, 1, 65536, 33000, 100, 47000, 5], dtype=np.int64)
    a, b, c, d, off, nondom = ragged.synthetic_batch(sizes, dtype=torch.float64, nondominant_fraction=0.3, seed=31)
    plan32 = T.RaggedPlan(off, dtype=torch.float32, classify=True)
    w = torch.rand_like(d) * 2 - 1
    x1 = plan32.refine(a, b, c, d, iters=1).clone()
    x2 = plan32.refine(a, b, c, d, iters=2).clone()
    x = plan32.refine(a, b, c, d, iters=1, pivoted_iters=1)
    kinds = plan32.kinds()
    ga, gb, gc, gd = plan32.refine_adjoint(a, b, c, x, w, iters=1, pivoted_iters=1)
    l1 = plan32.refine_adjoint(a, b, c, x, w, iters=1)[3]
    l2 = plan32.refine_adjoint(a, b, c, x, w, iters=2)[3]
    torch.cuda.synchronize()
    assert nondom.any() and kinds[nondom].max() == 0  # the non-dominant systems are pivoted
    assert kinds.max() == 1  # and some systems are not
    for s in range(len(sizes)):
        n = int(sizes[s])
        lo, hi = int(off[s]), int(off[s + 1])
        ref_x, ref_l = (x1, l1) if kinds[s] == 1 else (x2, l2)
        assert torch.equal(x[lo:hi], ref_x[lo:hi]), ("x", s, n, int(kinds[s]))
        assert torch.equal(gd[lo:hi], ref_l[lo:hi]), ("lambda", s, n, int(kinds[s]))
        hs = [_host(t, off, s) for t in (a, b, c, d, x, w)]
        grads = [_host(g, off, s) for g in (ga, gb, gc, gd)]
        _check_system(hs, grads, n, not nondom[s], 1e-12, 1e-10)


def test_ragged_refined_rejects_fp64_plan(cuda):
    import tridiagonalsolver_gb300 as T

    torch = cuda
    off = np.array([0, 100, 300], dtype=np.int64)
    t = torch.zeros(300, dtype=torch.float64, device="cuda")
    plan64 = T.RaggedPlan(off, dtype=torch.float64)
    with pytest.raises(ValueError):
        plan64.refine(t, t, t, t)


@pytest.mark.parametrize("dtype_name", ["float32", "float64"])
def test_ragged_sequential_variant(cuda, dtype_name):
    """Variant 9 (thread-per-system partial pivoting, rows in the plan's
    workspace) forced for every class above 64 rows: forward and adjoint of
    dominant and non-dominant systems against the oracle."""
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300 import ragged

    torch = cuda
    dt = getattr(torch, dtype_name)
    sizes = _sizes(5000)
    a, b, c, d, off, nondom = ragged.synthetic_batch(sizes, dtype=dt, nondominant_fraction=0.3, seed=31)
    table = {k: 9 for k in range(7, ragged.CLASSES)}
    plan = T.RaggedPlan(off, dtype=dt, table=table)
    assert {v for cls, v, _, _ in plan.buckets() if cls >= 7} == {9}
    info = torch.full((len(sizes),), -7, dtype=torch.int32, device="cuda")
    x = plan.solve(a, b, c, d, info=info)
    w = torch.rand_like(d) * 2 - 1
    ga, gb, gc, gd = plan.adjoint(a, b, c, x, w)
    torch.cuda.synchronize()
    assert int((info != 0).sum()) == 0
    for s in range(len(sizes)):
        n = int(sizes[s])
        hs = [_host(t, off, s) for t in (a, b, c, d, x, w)]
        grads = [_host(g, off, s) for g in (ga, gb, gc, gd)]
        _check_system(hs, grads, n, not nondom[s], ETA[dtype_name], GTOL[dtype_name])


@pytest.mark.parametrize("variant", [10, 9])
@pytest.mark.parametrize("routing", ["pivoted", "classify"])
def test_ragged_fp64_beyond_clusters(cuda, routing, variant):
    """FP64 systems longer than the clusters serve (27648 rows) go to variant
    10 (chunks of 4224 rows) by default, or to variant 9 by the table; with
    the library classifying, the dominant ones run the chunked unpivoted
    method and the others reach the pivoted bucket through the class's
    device-grown list.  Every system checked, forward and adjoint."""
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300 import ragged

    torch = cuda
    sizes = np.array([40000, 65536, 27649, 33000, 50000, 30001, 100, 3000, 20000, 64], dtype=np.int64)
    a, b, c, d, off, nondom = ragged.synthetic_batch(sizes, dtype=torch.float64, nondominant_fraction=0.5, seed=32)
    assert nondom[sizes > 27648].any() and (~nondom[sizes > 27648]).any()
    table = None if variant == 10 else {15: 9, 16: 9}
    plan = T.RaggedPlan(off, dtype=torch.float64, table=table, classify=routing == "classify")
    assert variant in {v for _, v, _, _ in plan.buckets()}
    info = torch.full((len(sizes),), -7, dtype=torch.int32, device="cuda")
    x = plan.solve(a, b, c, d, info=info)
    w = torch.rand_like(d) * 2 - 1
    ga, gb, gc, gd = plan.adjoint(a, b, c, x, w)
    torch.cuda.synchronize()
    assert int((info != 0).sum()) == 0
    if routing == "classify":
        big = sizes > 64
        assert np.array_equal(plan.kinds().astype(bool)[big], ~nondom[big])
    for s in range(len(sizes)):
        n = int(sizes[s])
        hs = [_host(t, off, s) for t in (a, b, c, d, x, w)]
        grads = [_host(g, off, s) for g in (ga, gb, gc, gd)]
        _check_system(hs, grads, n, not nondom[s], ETA["float64"], GTOL["float64"])


@pytest.mark.parametrize("dtype_name", ["float32", "float64"])
def test_ragged_chunked_variant(cuda, dtype_name):
    """Variant 10 (the partitioned solve in chunks of 4224 rows, the
    separators' systems in between) forced on every class above 2048 rows,
    sizes around the chunk boundaries: forward and adjoint of dominant and
    non-dominant systems against the oracle (FP32 systems whose chunk misses
    its bound are re-solved by variant 9)."""
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300 import ragged

    torch = cuda
    dt = getattr(torch, dtype_name)
    top = 65536 if dtype_name == "float32" else 27648
    sizes = np.array([s for s in _sizes(top) if s > 2048] + [4224, 4225, 8448, 8449, 12000, 300], dtype=np.int64)
    a, b, c, d, off, nondom = ragged.synthetic_batch(sizes, dtype=dt, nondominant_fraction=0.4, seed=33)
    table = {k: 10 for k in range(12, ragged.CLASSES)}
    plan = T.RaggedPlan(off, dtype=dt, table=table)
    assert {v for cls, v, _, _ in plan.buckets() if cls >= 12} == {10}
    info = torch.full((len(sizes),), -7, dtype=torch.int32, device="cuda")
    x = plan.solve(a, b, c, d, info=info)
    w = torch.rand_like(d) * 2 - 1
    ga, gb, gc, gd = plan.adjoint(a, b, c, x, w)
    torch.cuda.synchronize()
    assert int((info != 0).sum()) == 0
    for s in range(len(sizes)):
        n = int(sizes[s])
        hs = [_host(t, off, s) for t in (a, b, c, d, x, w)]
        grads = [_host(g, off, s) for g in (ga, gb, gc, gd)]
        _check_system(hs, grads, n, not nondom[s], ETA[dtype_name], GTOL[dtype_name])


def test_ragged_chunked_flagged_system_resolved(cuda):
    """A singular interior block in chunk 2 of one system (a partition's first
    row with zero diagonal and superdiagonal; the matrix is regular): that
    chunk misses its bound, the system is re-solved by variant 9, the others
    keep the chunks' result; forward and adjoint against the oracle."""
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300 import ragged

    torch = cuda
    sizes = np.array([40000, 30000, 50000, 100], dtype=np.int64)
    a, b, c, d, off, _ = ragged.synthetic_batch(sizes, dtype=torch.float64, nondominant_fraction=1.0, seed=34)
    r = int(off[1]) + 2 * 128 * 33 + 5 * 33
    b[r], c[r], a[r] = 0.0, 0.0, 1.0
    plan = T.RaggedPlan(off, dtype=torch.float64)
    assert 10 in {v for _, v, _, _ in plan.buckets()}
    T.lib().tridiag_partition_fallbacks(1)
    info = torch.full((len(sizes),), -7, dtype=torch.int32, device="cuda")
    x = plan.solve(a, b, c, d, info=info)
    torch.cuda.synchronize()
    assert T.lib().tridiag_partition_fallbacks(1) >= 1
    assert int((info != 0).sum()) == 0
    w = torch.rand_like(d) * 2 - 1
    ga, gb, gc, gd = plan.adjoint(a, b, c, x, w)
    torch.cuda.synchronize()
    for s in range(len(sizes)):
        n = int(sizes[s])
        hs = [_host(t, off, s) for t in (a, b, c, d, x, w)]
        grads = [_host(g, off, s) for g in (ga, gb, gc, gd)]
        _check_system(hs, grads, n, False, ETA["float64"], GTOL["float64"])


@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_ragged_results_are_reproducible(cuda, dtype):
    """Forward and adjoint of a classifying plan on a mixed batch (long
    chunked systems, pivoted clusters and tickets, device-grown lists): the
    same inputs give bit-identical x and gradients run after run, whatever
    order the resident CTAs take the systems in."""
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300 import ragged

    torch = cuda
    dt = getattr(torch, dtype)
    sizes = ragged.log_uniform_sizes(600, 32, 65536, seed=17)
    a, b, c, d, off, _ = ragged.synthetic_batch(sizes, dtype=dt, nondominant_fraction=0.3, seed=17)
    w = torch.rand_like(d) * 2 - 1
    plan = T.RaggedPlan(off, dtype=dt, classify=True)
    runs = []
    for _ in range(3):
        x = plan.solve(a, b, c, d)
        g = plan.adjoint(a, b, c, x, w)
        torch.cuda.synchronize()
        runs.append([x.clone()] + [t.clone() for t in g])
    for r in runs[1:]:
        for p, q in zip(runs[0], r):
            assert torch.equal(p, q)


def test_ragged_refined_pivoted_steps_without_marks(cuda):
    """A plan without marks (no classification, no mask) pivots every
    system, so the restricted steps cover all of them: iters = 1,
    pivoted_iters = 1 gives exactly the two-step result, forward and adjoint."""
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300 import ragged

    torch = cuda
    sizes = np.array([3, 700, 5000, 1, 20000, 64, 65], dtype=np.int64)
    a, b, c, d, off, _ = ragged.synthetic_batch(sizes, dtype=torch.float64, nondominant_fraction=0.3, seed=41)
    plan32 = T.RaggedPlan(off, dtype=torch.float32)
    w = torch.rand_like(d) * 2 - 1
    x2 = plan32.refine(a, b, c, d, iters=2).clone()
    x = plan32.refine(a, b, c, d, iters=1, pivoted_iters=1)
    l2 = plan32.refine_adjoint(a, b, c, x, w, iters=2)[3].clone()
    l = plan32.refine_adjoint(a, b, c, x, w, iters=1, pivoted_iters=1)[3]
    torch.cuda.synchronize()
    assert torch.equal(x, x2)
    assert torch.equal(l, l2)
