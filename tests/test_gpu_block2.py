"""Block tridiagonal systems with 2 x 2 blocks on the GPU vs the oracle.

Tolerances: normwise backward error (FP64 residual) <= 1e-12 for FP64 and
<= 1e-6 for FP32 solves, the bars of the scalar solves; FP64 solutions agree
with the FP64 oracle of the same algorithm to a median relative difference
of 1e-11 (non-dominant systems, pivoted) or a maximum of 1e-12 (dominant
systems, Thomas); FP32 solutions of dominant systems agree with the FP64
oracle to 1e-4 relative to max|x|.  info codes match the oracle exactly.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

ETA = {np.float64: 1e-12, np.float32: 1e-6}
ALGO = {"pivoted": "gbsv", "thomas": "thomas"}


def blocks(n, batch, seed, dominant):
    rng = np.random.default_rng(seed)
    a, b, c = (rng.uniform(-1, 1, (batch, n, 2, 2)) for _ in range(3))
    d = rng.uniform(-1, 1, (batch, n, 2))
    if dominant:
        rows = np.abs(a).sum(-1) + np.abs(c).sum(-1) + np.abs(b).sum(-1)
        for k in range(2):
            b[:, :, k, k] = np.sign(rng.uniform(-1, 1, (batch, n))) * (rows[:, :, k] + rng.uniform(1, 2, (batch, n)))
    return a, b, c, d


def to_layout(v, layout):
    """(batch, n, ...) host array -> flat array in the given layout."""
    if layout == "contiguous":
        return np.ascontiguousarray(v).reshape(-1)
    batch = v.shape[0]
    return np.ascontiguousarray(v.reshape(batch, -1).T).reshape(-1)


def from_layout(flat, layout, batch, n, k):
    if layout == "contiguous":
        return flat.reshape(batch, n, k)
    return flat.reshape(n * k, batch).T.reshape(batch, n, k)


def run(torch, a, b, c, d, n, dt, algo, layout, offset=0):
    import tridiagonalsolver_gb300 as T

    batch = a.shape[0]

    def dev(v):
        flat = to_layout(v.astype(dt), layout)
        buf = torch.zeros(flat.size + offset, dtype=torch.float64 if dt == np.float64 else torch.float32,
                          device="cuda")
        t = buf[offset:]
        t.copy_(torch.from_numpy(flat))
        return t

    ta, tb, tc, td = (dev(v) for v in (a, b, c, d))
    info = torch.full((batch,), -1, dtype=torch.int32, device="cuda")
    T.block2(ta, tb, tc, td, n, algo=algo, layout=layout, info=info)
    torch.cuda.synchronize()
    x = from_layout(td.double().cpu().numpy(), layout, batch, n, 2)
    return x, info.cpu().numpy(), (ta, tb, tc)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("algo", ["pivoted", "thomas"])
@pytest.mark.parametrize("layout", ["contiguous", "interleaved"])
@pytest.mark.parametrize("n,batch", [(1, 1), (2, 3), (5, 33), (64, 100), (1000, 40), (4096, 7)])
def test_block2_vs_oracle(cuda, dt, algo, layout, n, batch):
    dominant = algo == "thomas"
    a, b, c, d = blocks(n, batch, seed=n + 7 * batch, dominant=dominant)
    x, info, _ = run(cuda, a, b, c, d, n, dt, algo, layout)
    assert not info.any()
    a_, b_, c_, d_ = (v.astype(dt).astype(np.float64) for v in (a, b, c, d))
    eta, worst = O.block2_backward_error(a_, b_, c_, d_, x, n)
    assert worst <= ETA[dt], worst
    xo, info_o = O.block2(a_, b_, c_, d_, n, ALGO[algo])
    assert not info_o.any()
    xo = xo.reshape(batch, -1)
    xg = x.reshape(batch, -1)
    rel = np.max(np.abs(xg - xo), axis=1) / np.max(np.abs(xo), axis=1)
    if dt == np.float64:
        assert (np.median(rel) if algo == "pivoted" else rel.max()) <= (1e-11 if algo == "pivoted" else 1e-12)
    elif dominant:
        assert rel.max() <= 1e-4


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_block2_pivoting_where_thomas_fails(cuda, dt):
    """Zero diagonal blocks: the pivoted solve succeeds, Thomas flags M_0."""
    n, batch = 40, 64
    rng = np.random.default_rng(11)
    a, c = (rng.uniform(0.5, 1, (batch, n, 2, 2)) for _ in range(2))
    b = np.zeros((batch, n, 2, 2))
    d = rng.uniform(-1, 1, (batch, n, 2))
    x, info, _ = run(cuda, a, b, c, d, n, dt, "pivoted", "contiguous")
    assert not info.any()
    _, worst = O.block2_backward_error(*(v.astype(dt).astype(np.float64) for v in (a, b, c, d)), x, n)
    assert worst <= ETA[dt]
    _, info_t, _ = run(cuda, a, b, c, d, n, dt, "thomas", "contiguous")
    assert (info_t == 1).all()


@pytest.mark.parametrize("layout", ["contiguous", "interleaved"])
def test_block2_info_codes(cuda, layout):
    n, batch = 6, 5
    a, b, c, d = blocks(n, batch, seed=5, dominant=False)
    b[1, 0, :, 0] = 0          # scalar column 0 zero -> info 1
    a[1, 1, :, 0] = 0
    b[3, 2, :, 0] = 0          # scalar column 4 zero -> info 5
    a[3, 3, :, 0] = 0
    c[3, 1, :, 0] = 0
    _, info, _ = run(cuda, a, b, c, d, n, np.float64, "pivoted", layout)
    _, info_o = O.block2(a, b, c, d, n, "gbsv")
    assert list(info) == list(info_o) == [0, 1, 0, 5, 0]
    bt = b.copy()
    bt[4, 0] = [[1.0, 2.0], [2.0, 4.0]]  # singular B_0 -> Thomas info 1
    _, info_t, _ = run(cuda, a, bt, c, d, n, np.float64, "thomas", layout)
    assert info_t[4] == 1


@pytest.mark.parametrize("algo", ["pivoted", "thomas"])
def test_block2_ignores_a0_and_clast(cuda, algo):
    """A_0 and C_{n-1} are never read: NaN there changes nothing."""
    n, batch = 50, 40
    a, b, c, d = blocks(n, batch, seed=3, dominant=True)
    x0, _, _ = run(cuda, a, b, c, d, n, np.float64, algo, "contiguous")
    a2, c2 = a.copy(), c.copy()
    a2[:, 0] = np.nan
    c2[:, n - 1] = np.nan
    x1, info, _ = run(cuda, a2, b, c2, d, n, np.float64, algo, "contiguous")
    assert not info.any()
    assert np.array_equal(x0, x1)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("algo", ["pivoted", "thomas"])
def test_block2_unaligned_pointers(cuda, dt, algo):
    """Views one element off a 16-byte boundary take the scalar-load path and
    give the same solutions as aligned buffers."""
    n, batch = 77, 50
    a, b, c, d = blocks(n, batch, seed=9, dominant=True)
    x0, _, _ = run(cuda, a, b, c, d, n, dt, algo, "contiguous")
    x1, info, _ = run(cuda, a, b, c, d, n, dt, algo, "contiguous", offset=1)
    assert not info.any()
    assert np.array_equal(x0, x1)


def test_block2_thomas_keeps_a_and_b(cuda):
    import torch

    n, batch = 30, 20
    a, b, c, d = blocks(n, batch, seed=4, dominant=True)
    _, _, (ta, tb, _) = run(cuda, a, b, c, d, n, np.float64, "thomas", "contiguous")
    assert np.array_equal(ta.cpu().numpy(), a.reshape(-1))
    assert np.array_equal(tb.cpu().numpy(), b.reshape(-1))
    del torch


def test_block2_rejects_bad_arguments(cuda):
    import tridiagonalsolver_gb300 as T

    L = T.lib()
    t = cuda.zeros(64, dtype=cuda.float64, device="cuda")
    p = t.data_ptr()
    assert L.tridiag_block2_double(0, 1, p, p, p, p, None, 4, 4, None) != 0   # packed layout
    assert L.tridiag_block2_double(7, 0, p, p, p, p, None, 4, 4, None) != 0   # unknown algo
    assert L.tridiag_block2_double(0, 0, p, p, p, p, None, 0, 4, None) != 0   # n = 0
    assert L.tridiag_block2_double(0, 0, None, p, p, p, None, 4, 4, None) != 0
