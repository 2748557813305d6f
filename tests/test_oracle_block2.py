"""Oracle for block tridiagonal systems with 2 x 2 blocks (CPU only).

The reference has no block solver, so the oracle is pinned to LAPACK: the
pivoted form restates ?gbsv (band LU with partial pivoting, kl = ku = 3 on
the scalar matrix of order 2n) and must agree with scipy's dgbsv/sgbsv to a
few ulps of the solution; block Thomas must agree with a dense solve on
block diagonally dominant systems.  Tolerances: FP64 relative difference
<= 1e-12 (pivoted vs dgbsv, same pivot sequence), <= 1e-13 (Thomas vs dense
solve on dominant systems); FP32 <= 1e-4 against FP64 LAPACK on dominant
systems.
"""
import numpy as np
import pytest

from oracle import oracle as O


def random_blocks(n, batch, seed, dominant=False, dtype=np.float64):
    rng = np.random.default_rng(seed)
    a, b, c = (rng.uniform(-1, 1, (batch, n, 2, 2)) for _ in range(3))
    d = rng.uniform(-1, 1, (batch, n, 2))
    if dominant:
        rows = np.abs(a).sum(-1) + np.abs(c).sum(-1) + np.abs(b).sum(-1)
        for k in range(2):
            b[:, :, k, k] = np.sign(rng.uniform(-1, 1, (batch, n))) * (rows[:, :, k] + rng.uniform(1, 2, (batch, n)))
    return tuple(v.astype(dtype) for v in (a, b, c, d))


def lapack_gbsv(a, b, c, d, n):
    """scipy's ?gbsv on the scalar band form (kl = ku = 3)."""
    from scipy.linalg import lapack

    M = O.block2_dense(a, b, c, n)
    batch, N = M.shape[0], 2 * n
    kl = ku = 3
    out = np.empty((batch, N))
    dt = np.asarray(a).dtype
    fn = lapack.dgbsv if dt == np.float64 else lapack.sgbsv
    for j in range(batch):
        ab = np.zeros((2 * kl + ku + 1, N), dtype=dt)
        for col in range(N):
            for row in range(max(0, col - ku), min(N, col + kl + 1)):
                ab[kl + ku + row - col, col] = M[j, row, col]
        _, _, x, info = fn(kl, ku, ab, np.asarray(d[j], dtype=dt).reshape(N))
        assert info == 0
        out[j] = x
    return out


@pytest.mark.parametrize("n", [1, 2, 3, 8, 37, 200])
def test_block2_gbsv_matches_lapack(n):
    a, b, c, d = random_blocks(n, 6, seed=n)
    x, info = O.block2(a, b, c, d, n, "gbsv")
    assert not info.any()
    xl = lapack_gbsv(a, b, c, d, n)
    x = x.reshape(6, -1)
    rel = np.max(np.abs(x - xl), axis=1) / np.max(np.abs(xl), axis=1)
    assert rel.max() <= 1e-12


def test_block2_gbsv_f32_matches_lapack():
    n = 50
    a, b, c, d = random_blocks(n, 4, seed=1, dominant=True, dtype=np.float32)
    x, info = O.block2(a, b, c, d, n, "gbsv")
    assert not info.any()
    xl = lapack_gbsv(*(v.astype(np.float64) for v in (a, b, c, d)), n)
    assert np.max(np.abs(x.reshape(4, -1) - xl)) / np.max(np.abs(xl)) <= 1e-4


@pytest.mark.parametrize("n", [1, 2, 5, 64])
def test_block2_thomas_matches_dense(n):
    a, b, c, d = random_blocks(n, 5, seed=10 + n, dominant=True)
    x, info = O.block2(a, b, c, d, n, "thomas")
    assert not info.any()
    M = O.block2_dense(a, b, c, n)
    xr = np.linalg.solve(M, d.reshape(5, 2 * n, 1))[..., 0]
    assert np.max(np.abs(x.reshape(5, -1) - xr)) / np.max(np.abs(xr)) <= 1e-13


def test_block2_kat_ones():
    """Block Laplacian-like system whose solution is x = 1."""
    n, batch = 100, 3
    b = np.tile(np.array([[4.0, -1.0], [-1.0, 4.0]]), (batch, n, 1, 1))
    a = np.tile(-np.eye(2), (batch, n, 1, 1))
    c = a.copy()
    ones = np.ones((batch, n, 2))
    d = np.einsum("bnij,bnj->bni", b, ones)
    d[:, 1:] += np.einsum("bnij,bnj->bni", a[:, 1:], ones[:, :-1])
    d[:, :-1] += np.einsum("bnij,bnj->bni", c[:, :-1], ones[:, 1:])
    for algo in ("gbsv", "thomas"):
        x, info = O.block2(a, b, c, d, n, algo)
        assert not info.any()
        assert np.max(np.abs(x - 1)) <= 1e-14


def test_block2_pivoting_needed():
    """Zero diagonal blocks: Thomas fails (singular M_0), gbsv pivots."""
    n = 6
    rng = np.random.default_rng(3)
    a, c = (rng.uniform(0.5, 1, (1, n, 2, 2)) for _ in range(2))
    b = np.zeros((1, n, 2, 2))
    d = rng.uniform(-1, 1, (1, n, 2))
    x, info = O.block2(a, b, c, d, n, "gbsv")
    assert info[0] == 0
    eta, _ = O.block2_backward_error(a, b, c, d, x, n)
    assert eta[0] <= 1e-14
    _, info_t = O.block2(a, b, c, d, n, "thomas")
    assert info_t[0] == 1


def test_block2_info_codes():
    n, batch = 4, 3
    a, b, c, d = random_blocks(n, batch, seed=5)
    # system 1: scalar column 0 is zero (B_0[:, 0] = 0, A_1[:, 0] = 0)
    b[1, 0, :, 0] = 0
    a[1, 1, :, 0] = 0
    # system 2: scalar column 4 is zero (C_1[:, 0] = B_2[:, 0] = A_3[:, 0] = 0)
    b[2, 2, :, 0] = 0
    a[2, 3, :, 0] = 0
    c[2, 1, :, 0] = 0
    _, info = O.block2(a, b, c, d, n, "gbsv")
    assert list(info) == [0, 1, 5]
    bt = b.copy()
    bt[0, 0] = [[1.0, 2.0], [2.0, 4.0]]
    _, info_t = O.block2(a, bt, c, d, n, "thomas")
    assert info_t[0] == 1
