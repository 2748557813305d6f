"""GPU parity of the thread-per-system kernels (Thomas, pivoted gtsv and its
adjoint) against the oracle and the golden fixtures, through the C ABI.

Tolerances (stated per test): FP64 results must have normwise backward error
<= 1e-12 and FP32 results <= 1e-6 (computed in FP64 by the oracle); forward
differences to the oracle are bounded relative to max|x| per system.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tridiagonalsolver_gb300 import inputs

pytestmark = pytest.mark.gpu

ETA = {np.float64: 1e-12, np.float32: 1e-6}


def _dev(torch, arrs, dt, layout):
    """numpy (batch, n) float64 arrays -> CUDA tensors in `layout`."""
    if layout == "interleaved":
        arrs = inputs.to_interleaved(*arrs)
    if layout == "packed":
        return [torch.from_numpy(inputs.to_packed(*arrs).astype(dt)).cuda()]
    return [torch.from_numpy(np.ascontiguousarray(v.astype(dt))).cuda() for v in arrs]


def _host(t, layout, batch, n):
    v = t.double().cpu().numpy()
    if layout == "interleaved":
        return v.reshape(n, batch).T.copy()
    if layout == "packed":
        return v.reshape(batch, 4, n)[:, 3, :].copy()
    return v.reshape(batch, n)


def _rel(x, xr):
    return np.max(np.abs(x - xr), axis=1) / np.maximum(np.max(np.abs(xr), axis=1), 1e-300)


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("layout", ["contiguous", "interleaved", "packed"])
@pytest.mark.parametrize("n,batch", [(1, 3), (2, 5), (7, 33), (48, 36), (64, 64), (257, 100), (1000, 40),
                                     (4096, 64)])
def test_thomas_matches_oracle(cuda, dt, layout, n, batch):
    import tridiagonalsolver_gb300 as T

    a, b, c, d = inputs.dominant(n, batch, seed=n * 7 + batch)
    ts = _dev(cuda, (a, b, c, d), dt, layout)
    if layout == "packed":
        T.solve(ts[0], None, None, None, n, algo="thomas", layout="packed")
        x = _host(ts[0], layout, batch, n)
    else:
        T.solve(*ts, n, algo="thomas", layout=layout)
        x = _host(ts[3], layout, batch, n)
    cuda.cuda.synchronize()
    xo = O.thomas(*(v.astype(dt) for v in (a, b, c, d)), n).reshape(batch, n).astype(np.float64)
    _, eta = O.backward_error(*(v.astype(dt).astype(np.float64) for v in (a, b, c, d)), x, n)
    assert eta <= ETA[dt]
    assert np.max(_rel(x, xo)) <= (1e-13 if dt == np.float64 else 2e-5)


@pytest.mark.parametrize("dt,name", [(np.float64, "Thomas_double"), (np.float32, "Thomas_single")])
@pytest.mark.parametrize("case", ["n128", "n512", "ref256"])
def test_reference_entry_point_vs_golden(cuda, golden, dt, name, case):
    import tridiagonalsolver_gb300 as T

    z = golden["f64" if dt == np.float64 else "f32"]
    n = int(z[f"{case}/n"])
    a, b, c, d = (cuda.from_numpy(z[f"{case}/{k}"].copy()).cuda() for k in "abcd")
    T.reference_call(name, a, b, c, d, n)
    x = d.double().cpu().numpy().reshape(-1, n)
    xr = z[f"{case}/{name}"].astype(np.float64)
    assert np.max(_rel(x, xr)) <= (1e-13 if dt == np.float64 else 2e-5)
    # the reference contract: a and b untouched
    np.testing.assert_array_equal(a.cpu().numpy(), z[f"{case}/a"])
    np.testing.assert_array_equal(b.cpu().numpy(), z[f"{case}/b"])


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("layout", ["contiguous", "interleaved"])
@pytest.mark.parametrize("n,batch", [(1, 2), (2, 3), (3, 31), (33, 65), (48, 36), (64, 64), (65, 7), (96, 40),
                                     (512, 96), (1000, 64), (2049, 17), (4096, 32)])
def test_gtsv_matches_oracle_nondominant(cuda, dt, layout, n, batch):
    import tridiagonalsolver_gb300 as T

    a, b, c, d = inputs.nondominant(n, batch, seed=1000 + n + batch)
    ts = _dev(cuda, (a, b, c, d), dt, layout)
    info = cuda.zeros(batch, dtype=cuda.int32, device="cuda")
    x_t = T.gtsv(*ts, n, layout=layout, info=info)
    cuda.cuda.synchronize()
    x = _host(x_t, layout, batch, n)
    assert int(info.abs().sum()) == 0
    # inputs untouched
    for t, v in zip(ts, (a, b, c, d)):
        np.testing.assert_array_equal(_host(t, layout, batch, n), v.astype(dt).astype(np.float64))
    a_, b_, c_, d_ = (v.astype(dt).astype(np.float64) for v in (a, b, c, d))
    eta, worst = O.backward_error(a_, b_, c_, d_, x, n)
    assert worst <= ETA[dt]
    xo = O.gtsv(a_, b_, c_, d_, n).reshape(batch, n)
    # forward error is bounded by cond(A) * backward error; random U[-1,1]
    # systems reach cond ~1e6, so the bound is loose for FP32
    assert np.median(_rel(x, xo)) <= (1e-11 if dt == np.float64 else 1e-3)


def test_gtsv_lapack_golden(cuda, golden):
    import tridiagonalsolver_gb300 as T

    z = golden["gtsv"]
    for tag, dt in (("f64", np.float64), ("f32", np.float32)):
        n = int(z[f"{tag}/n"])
        a, b, c, d = (cuda.from_numpy(z[f"{tag}/{k}"].copy()).cuda() for k in "abcd")
        x = T.gtsv(a, b, c, d, n).double().cpu().numpy().reshape(-1, n)
        xr = z[f"{tag}/x"].astype(np.float64)
        _, worst = O.backward_error(*(z[f"{tag}/{k}"].astype(np.float64) for k in "abcd"), x, n)
        assert worst <= ETA[dt]
        assert np.max(_rel(x, xr)) <= (1e-10 if dt == np.float64 else 5e-3)


def test_gtsv_zero_pivot_info(cuda):
    import tridiagonalsolver_gb300 as T

    n, batch = 6, 3
    a, b, c, d = inputs.nondominant(n, batch, seed=9)
    # system 1: rows 2.. decoupled and b[2] = 0 -> U(2,2) = 0
    a[1, 2:] = 0.0
    c[1, 1:] = 0.0
    b[1, 2] = 0.0
    ts = [cuda.from_numpy(v.copy()).cuda() for v in (a, b, c, d)]
    info = cuda.full((batch,), -1, dtype=cuda.int32, device="cuda")
    T.gtsv(*ts, n, info=info)
    got = info.cpu().numpy()
    assert got[0] == 0 and got[2] == 0
    assert got[1] == 3


def test_gtsv_kat_laplacian(cuda, golden):
    import tridiagonalsolver_gb300 as T

    z = golden["kat"]
    n = z["a"].shape[1]
    ts = [cuda.from_numpy(z[k].copy()).cuda() for k in "abcd"]
    x = T.gtsv(*ts, n).cpu().numpy()
    assert np.max(np.abs(x - 1.0)) < 1e-12
    T.solve(*ts, n, algo="thomas")
    assert np.max(np.abs(ts[3].cpu().numpy() - 1.0)) < 1e-12


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("layout", ["contiguous", "interleaved"])
@pytest.mark.parametrize("n,batch", [(1, 2), (2, 4), (5, 3), (40, 33), (48, 36), (97, 64), (256, 16), (1000, 32),
                                     (2048, 8)])
def test_gtsv_adjoint_matches_oracle(cuda, dt, layout, n, batch):
    import tridiagonalsolver_gb300 as T

    a, b, c, d = inputs.nondominant(n, batch, seed=77 + n)
    w = np.random.default_rng(5).uniform(-1, 1, (batch, n))
    ts = _dev(cuda, (a, b, c, d), dt, layout)
    (wt,) = _dev(cuda, (w,), dt, layout)
    piv = T.pivot_record(ts[0], n, layout)
    x = T.gtsv(*ts, n, layout=layout, pivots=piv)
    ga, gb, gc, gd = T.gtsv_adjoint(ts[0], ts[1], ts[2], x, piv, wt, n, layout=layout)
    cuda.cuda.synchronize()
    a_, b_, c_ = (v.astype(dt).astype(np.float64) for v in (a, b, c))
    xo = _host(x, layout, batch, n)
    ref = O.adjoint_f64(a_, b_, c_, xo, w.astype(dt).astype(np.float64), n)
    for g, r in zip((ga, gb, gc, gd), ref):
        gh = _host(g, layout, batch, n)
        r = r.reshape(batch, n)
        scale = np.max(np.abs(r), axis=1, keepdims=True) + 1e-300
        err = np.max(np.abs(gh - r) / scale, axis=1)
        assert np.median(err) <= (1e-10 if dt == np.float64 else 2e-3)


def test_gtsv_adjoint_central_differences_fp64(cuda):
    """FP64 gradients against central differences (h = 1e-6) of the oracle."""
    import tridiagonalsolver_gb300 as T

    n, batch = 64, 4
    a, b, c, d = inputs.dominant(n, batch, seed=21)
    w = np.random.default_rng(22).uniform(-1, 1, (batch, n))
    ts = [cuda.from_numpy(v.copy()).cuda() for v in (a, b, c, d)]
    wt = cuda.from_numpy(w.copy()).cuda()
    piv = T.pivot_record(ts[0], n)
    x = T.gtsv(*ts, n, pivots=piv)
    grads = [g.cpu().numpy().reshape(batch, n) for g in T.gtsv_adjoint(ts[0], ts[1], ts[2], x, piv, wt, n)]
    h = 1e-6
    rng = np.random.default_rng(23)

    def loss(v):
        return np.sum(w * O.gtsv(*v, n).reshape(batch, n), axis=1)

    for k in range(4):
        for _ in range(5):
            i = int(rng.integers(1, n - 1))
            vp = [v.copy() for v in (a, b, c, d)]
            vp[k][:, i] += h
            vm = [v.copy() for v in (a, b, c, d)]
            vm[k][:, i] -= h
            fd = (loss(vp) - loss(vm)) / (2 * h)
            np.testing.assert_allclose(grads[k][:, i], fd, rtol=1e-6, atol=1e-8)


GUARD = 4 << 20  # bytes of guard region on each side of the workspace
PATTERN = 0xA5


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("with_pivots", [True, False])
@pytest.mark.parametrize("n,batch", [(3, 8), (33, 37), (300, 8), (511, 64), (1000, 9)])
def test_gtsv_packed_guarded_workspace(cuda, dt, with_pivots, n, batch):
    """Pivoted solve of packed systems ([batch][a|b|c|d][n], the reference's
    layout 1, Tridiagonal_CUDA/utils.cu:254-260) through the C ABI with the
    workspace between two guard regions of a byte pattern: the guard bytes
    must be unchanged afterwards (no scratch write outside the workspace),
    the packed a, b, c rows of the output untouched, and x within backward
    error 1e-12 (FP64) / 1e-6 (FP32) of its system."""
    import ctypes

    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300._lib import SUCCESS

    lib = T.lib()
    a, b, c, d = inputs.nondominant(n, batch, seed=300 + n + batch)
    packed = inputs.to_packed(a, b, c, d).astype(dt)
    p = cuda.from_numpy(packed.copy()).cuda()
    x = p.clone()
    ws = lib.tridiag_gtsv_workspace_size(1 if dt == np.float64 else 0, 1, n, batch)
    buf = cuda.full((GUARD + ws + GUARD,), PATTERN, dtype=cuda.uint8, device="cuda")
    piv = T.pivot_record(p, n, "packed") if with_pivots else None
    info = cuda.full((batch,), -1, dtype=cuda.int32, device="cuda")
    fn = lib.tridiag_gtsv_double if dt == np.float64 else lib.tridiag_gtsv_single
    es = np.dtype(dt).itemsize
    st = fn(1, ctypes.c_void_p(p.data_ptr()), None, None, ctypes.c_void_p(x.data_ptr() + 3 * n * es),
            ctypes.c_void_p(piv.data_ptr()) if piv is not None else None, ctypes.c_void_p(info.data_ptr()),
            ctypes.c_void_p(buf.data_ptr() + GUARD), ctypes.c_size_t(ws), n, batch, None)
    assert st == SUCCESS
    cuda.cuda.synchronize()
    g = buf.cpu().numpy()
    assert np.all(g[:GUARD] == PATTERN), "workspace underrun"
    assert np.all(g[GUARD + ws:] == PATTERN), "workspace overrun"
    assert int(info.abs().sum()) == 0
    xh = x.cpu().numpy().reshape(batch, 4, n)
    np.testing.assert_array_equal(xh[:, :3, :], packed.reshape(batch, 4, n)[:, :3, :])
    np.testing.assert_array_equal(p.cpu().numpy(), packed)
    a_, b_, c_, d_ = (v.astype(dt).astype(np.float64) for v in (a, b, c, d))
    xs = xh[:, 3, :].astype(np.float64)
    _, worst = O.backward_error(a_, b_, c_, d_, xs, n)
    assert worst <= ETA[dt]
    xo = O.gtsv(a_, b_, c_, d_, n).reshape(batch, n)
    assert np.median(_rel(xs, xo)) <= (1e-11 if dt == np.float64 else 1e-3)
    # the Python front end gives the same bits
    xt = T.gtsv(p, None, None, None, n, layout="packed", pivots=piv)
    np.testing.assert_array_equal(xt.cpu().numpy(), x.cpu().numpy())


@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_gtsv_packed_adjoint_refused(cuda, dt):
    """The pivoted adjoint takes contiguous and interleaved systems only."""
    import ctypes

    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300._lib import ERR_NOT_SUPPORTED

    lib = T.lib()
    t = cuda.zeros(4 * 8 * 4, dtype=cuda.float64 if dt == np.float64 else cuda.float32, device="cuda")
    ptr = ctypes.c_void_p(t.data_ptr())
    fn = lib.tridiag_gtsv_adjoint_double if dt == np.float64 else lib.tridiag_gtsv_adjoint_single
    st = fn(1, ptr, ptr, ptr, ptr, ptr, ptr, ptr, ptr, ptr, ptr, ptr, ctypes.c_size_t(1 << 20), 8, 4, None)
    assert st == ERR_NOT_SUPPORTED


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("n,batch", [(96, 100), (100, 37), (257, 129), (1000, 500), (4096, 256), (2049, 4096),
                                     (64, 8000), (513, 20000)])
def test_thomas_interleaved_partitioned(cuda, dt, n, batch):
    """Out-of-place Thomas on interleaved systems: the partitioned sweep
    (several partitions per system, separators by one thread per system).
    Against the oracle's sequential Thomas (the reference's algorithm,
    Tridiagonal_AVX512/tridiagonal_basic.cpp:6-27): per system
    max|x - x_oracle| / max|x_oracle| <= 1e-12 (FP64) / 2e-5 (FP32), backward
    error <= 1e-12 / 1e-6, inputs untouched."""
    import tridiagonalsolver_gb300 as T

    a, b, c, d = inputs.dominant(n, batch, seed=7 * n + batch)
    ts = _dev(cuda, (a, b, c, d), dt, "interleaved")
    x_t = T.solve_out(*ts, n, algo="thomas", layout="interleaved")
    cuda.cuda.synchronize()
    x = _host(x_t, "interleaved", batch, n)
    for t, v in zip(ts, (a, b, c, d)):
        np.testing.assert_array_equal(_host(t, "interleaved", batch, n), v.astype(dt).astype(np.float64))
    a_, b_, c_, d_ = (v.astype(dt).astype(np.float64) for v in (a, b, c, d))
    _, worst = O.backward_error(a_, b_, c_, d_, x, n)
    assert worst <= ETA[dt]
    xo = O.thomas(a_, b_, c_, d_, n).reshape(batch, n)
    assert np.max(_rel(x, xo)) <= (1e-12 if dt == np.float64 else 2e-5)
