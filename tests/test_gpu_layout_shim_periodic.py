"""Layout conversion, the cuSPARSE-shaped entry points and periodic systems.

Tolerances: layout conversion is a copy (bit-exact); the cuSPARSE-shaped
solves meet the backward-error bars of the other solve tests (<= 1e-12 FP64,
<= 1e-6 FP32) and agree with cuSPARSE's own gtsv2StridedBatch to 1e-5
(FP32) / 1e-12 (FP64) relative to max|x| on diagonally dominant systems;
periodic solves are checked against numpy's dense solve of the periodic
matrix (relative residual <= 1e-12 FP64 / 1e-5 FP32).
"""
import numpy as np
import pytest

from oracle import oracle as O
from tridiagonalsolver_gb300 import inputs

pytestmark = pytest.mark.gpu

ETA = {np.float64: 1e-12, np.float32: 1e-6}


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("n,batch", [(1, 1), (5, 3), (33, 70), (100, 31), (1024, 64)])
def test_relayout_all_pairs(cuda, dt, n, batch):
    import tridiagonalsolver_gb300 as T

    torch = cuda
    rng = np.random.default_rng(n + batch)
    arrs = [rng.standard_normal((batch, n)).astype(dt) for _ in range(4)]
    ref = {"contiguous": [v.reshape(-1) for v in arrs],
           "interleaved": [np.ascontiguousarray(v.T).reshape(-1) for v in arrs],
           "packed": [np.stack(arrs, axis=1).reshape(-1)]}
    for src in ref:
        ts = [torch.from_numpy(v.copy()).cuda() for v in ref[src]]
        for dst in ref:
            out = T.relayout(ts if len(ts) > 1 else ts[0], n, src, dst)
            outs = out if isinstance(out, list) else [out]
            for o, r in zip(outs, ref[dst]):
                assert np.array_equal(o.cpu().numpy(), r), (src, dst)


def _solve_check(x, a, b, c, d, dt, n):
    _, worst = O.backward_error(*(v.astype(dt).astype(np.float64) for v in (a, b, c, d)), x, n)
    assert worst <= ETA[dt]


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("n,batch,stride", [(64, 100, 64), (512, 64, 512), (3000, 8, 3000), (3000, 8, 3100),
                                            (700, 20, 1024)])
def test_gtsv2_strided_batch(cuda, dt, n, batch, stride):
    import tridiagonalsolver_gb300 as T

    torch = cuda
    L = T.lib()
    a, b, c, d = inputs.dominant(n, batch, seed=n + stride)
    pad = lambda v: np.pad(v.astype(dt), ((0, 0), (0, stride - n))).reshape(-1)
    ts = [torch.from_numpy(pad(v)).cuda() for v in (a, b, c, d)]
    prec = 1 if dt == np.float64 else 0
    nbytes = L.tridiag_gtsv2StridedBatch_bufferSize(prec, n, batch, stride)
    buf = torch.empty(max(nbytes, 1), dtype=torch.uint8, device="cuda")
    fn = L.tridiag_Dgtsv2StridedBatch if dt == np.float64 else L.tridiag_Sgtsv2StridedBatch
    st = fn(n, ts[0].data_ptr(), ts[1].data_ptr(), ts[2].data_ptr(), ts[3].data_ptr(), batch, stride,
            buf.data_ptr() if nbytes else None, None)
    assert st == 0
    torch.cuda.synchronize()
    x = ts[3].cpu().numpy().reshape(batch, stride)[:, :n].astype(np.float64)
    _solve_check(x, a, b, c, d, dt, n)
    if stride == n:
        # cuSPARSE's own gtsv2StridedBatch (the reference's vendor row) on the same systems
        tv = [torch.from_numpy(v.astype(dt).reshape(-1).copy()).cuda() for v in (a, b, c, d)]
        init = L.cuSparse_init_double if dt == np.float64 else L.cuSparse_init_single
        call = L.cuSparse_double if dt == np.float64 else L.cuSparse_single
        assert init(*[t.data_ptr() for t in tv], n, batch) == 0
        call(*[t.data_ptr() for t in tv], n, batch)
        L.cuSparse_final()
        xv = tv[3].double().cpu().numpy().reshape(batch, n)
        rel = np.max(np.abs(x - xv)) / np.max(np.abs(xv))
        assert rel <= (1e-12 if dt == np.float64 else 1e-5)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("algo", [0, 1, 2])
@pytest.mark.parametrize("n,batch", [(7, 33), (256, 64), (2000, 32)])
def test_gtsv_interleaved_batch(cuda, dt, algo, n, batch):
    import tridiagonalsolver_gb300 as T

    torch = cuda
    L = T.lib()
    gen = inputs.dominant if algo == 2 else inputs.nondominant
    a, b, c, d = gen(n, batch, seed=3 * n + algo)
    ts = [torch.from_numpy(np.ascontiguousarray(v.astype(dt).T).reshape(-1)).cuda() for v in (a, b, c, d)]
    prec = 1 if dt == np.float64 else 0
    nbytes = L.tridiag_gtsvInterleavedBatch_bufferSize(prec, algo, n, batch)
    buf = torch.empty(max(nbytes, 1), dtype=torch.uint8, device="cuda")
    fn = L.tridiag_DgtsvInterleavedBatch if dt == np.float64 else L.tridiag_SgtsvInterleavedBatch
    st = fn(algo, n, ts[0].data_ptr(), ts[1].data_ptr(), ts[2].data_ptr(), ts[3].data_ptr(), batch,
            buf.data_ptr() if nbytes else None, None)
    assert st == 0
    torch.cuda.synchronize()
    x = ts[3].double().cpu().numpy().reshape(n, batch).T
    _solve_check(x, a, b, c, d, dt, n)


def _periodic_dense(a, b, c, n):
    A = np.diag(b) + np.diag(a[1:], -1) + np.diag(c[:-1], 1)
    A[0, n - 1] += a[0]
    A[n - 1, 0] += c[n - 1]
    return A


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("algo", ["gtsv", "wm", "thomas"])
@pytest.mark.parametrize("n,batch", [(3, 5), (50, 9), (600, 6), (5000, 3)])
def test_periodic(cuda, dt, algo, n, batch):
    import tridiagonalsolver_gb300 as T

    torch = cuda
    rng = np.random.default_rng(n)
    a, c, d = (rng.uniform(-1, 1, (batch, n)) for _ in range(3))
    if algo == "gtsv":
        b = rng.uniform(-1, 1, (batch, n)) + np.sign(rng.uniform(-1, 1, (batch, n))) * 0.5
    else:
        b = np.abs(a) + np.abs(c) + rng.uniform(1, 2, (batch, n))
    ts = [torch.from_numpy(v.astype(dt)).cuda() for v in (a, b, c, d)]
    x = T.periodic(*ts, n, algo=algo).double().cpu().numpy().reshape(batch, n)
    a_, b_, c_, d_ = (v.astype(dt).astype(np.float64) for v in (a, b, c, d))
    for j in range(batch):
        A = _periodic_dense(a_[j], b_[j], c_[j], n) if n < 2000 else None
        if A is None:
            # banded residual for large n
            r = b_[j] * x[j] - d_[j]
            r[1:] += a_[j, 1:] * x[j, :-1]
            r[:-1] += c_[j, :-1] * x[j, 1:]
            r[0] += a_[j, 0] * x[j, -1]
            r[-1] += c_[j, -1] * x[j, 0]
            scale = np.max(np.abs(a_[j]) + np.abs(b_[j]) + np.abs(c_[j])) * np.max(np.abs(x[j])) + np.max(np.abs(d_[j]))
        else:
            r = A @ x[j] - d_[j]
            scale = np.max(np.sum(np.abs(A), axis=1)) * np.max(np.abs(x[j])) + np.max(np.abs(d_[j]))
        assert np.max(np.abs(r)) / scale <= (1e-12 if dt == np.float64 else 1e-5), (j, algo)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("layout", ["contiguous", "interleaved"])
@pytest.mark.parametrize("n,batch", [(1, 3), (2, 5), (9, 33), (300, 70), (4096, 16)])
def test_factor_and_solve_many(cuda, dt, layout, n, batch):
    """Factor once, then three right-hand sides and the transposed system."""
    import tridiagonalsolver_gb300 as T

    torch = cuda
    a, b, c, _ = inputs.nondominant(n, batch, seed=7 * n + batch)
    rng = np.random.default_rng(n)
    rhs = [rng.uniform(-1, 1, (batch, n)) for _ in range(3)]

    def dev(v):
        v = v.astype(dt)
        return torch.from_numpy(np.ascontiguousarray(v.T if layout == "interleaved" else v).reshape(-1)).cuda()

    def host(t):
        v = t.double().cpu().numpy()
        return v.reshape(n, batch).T if layout == "interleaved" else v.reshape(batch, n)

    info = torch.full((batch,), -1, dtype=torch.int32, device="cuda")
    F = T.Factorization(dev(a), dev(b), dev(c), n, layout=layout, info=info)
    r = torch.cat([dev(v) for v in rhs])
    F.solve(r)
    rt = dev(rhs[0])
    F.solve(rt, transpose=True)
    torch.cuda.synchronize()
    assert int(info.abs().sum()) == 0
    a_, b_, c_ = (v.astype(dt).astype(np.float64) for v in (a, b, c))
    blk = n * batch
    for k in range(3):
        x = host(r[k * blk:(k + 1) * blk])
        _, worst = O.backward_error(a_, b_, c_, rhs[k].astype(dt).astype(np.float64), x, n)
        assert worst <= ETA[dt]
    # A^T z = r0: the oracle's adjoint gives lambda = A^{-T} xbar (any x)
    lam = O.adjoint_f64(a_, b_, c_, np.zeros((batch, n)), rhs[0].astype(dt).astype(np.float64), n)[3].reshape(batch, n)
    z = host(rt)
    rel = np.max(np.abs(z - lam), axis=1) / np.maximum(np.max(np.abs(lam), axis=1), 1e-300)
    assert np.median(rel) <= (1e-10 if dt == np.float64 else 1e-3)
