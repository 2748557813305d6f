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


@pytest.mark.parametrize("mark_dominant", [False, True])
def test_ragged_full_workload(cuda, mark_dominant):
    """100000 systems, n log-uniform in [32, 65536] (~8.6e8 rows), FP32, 20%
    non-dominant: forward and adjoint; 40 sampled systems checked.  With
    mark_dominant the dominant systems run the unpivoted partition method."""
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300 import ragged

    torch = cuda
    sizes = ragged.log_uniform_sizes(100000, 32, 65536, seed=2024)
    a, b, c, d, off, nondom = ragged.synthetic_batch(sizes, seed=2024)
    plan = T.RaggedPlan(off, no_pivoting=~nondom if mark_dominant else None)
    info = torch.full((len(sizes),), -7, dtype=torch.int32, device="cuda")
    x = plan.solve(a, b, c, d, info=info)
    w = torch.rand_like(d) * 2 - 1
    ga, gb, gc, gd = plan.adjoint(a, b, c, x, w)
    torch.cuda.synchronize()
    assert int((info != 0).sum()) == 0
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
