"""Pivoted solve of long systems in chunks (uniform contiguous batches: FP64
from 12288 rows, FP32 beyond the cluster sizes, n > 65536), through
tridiag_gtsv_* without a pivot record, against the oracle.

Tolerances: normwise backward error <= 1e-12 (FP64) / 1e-6 (FP32) computed in
FP64 by the oracle; on diagonally dominant systems also the forward error vs
the oracle's LAPACK-style solve, <= 1e-10 (FP64) / 1e-4 (FP32) relative to
max |x| (random U[-1,1] systems of this length reach condition numbers at
which no FP32 solve has a small forward error: backward error only there).
"""
import numpy as np
import pytest

from oracle import oracle as O
from tridiagonalsolver_gb300 import inputs

pytestmark = pytest.mark.gpu

ETA = {np.float64: 1e-12, np.float32: 1e-6}
FWD = {np.float64: 1e-10, np.float32: 1e-4}


def _run(torch, T, arrs, dt, n):
    batch = arrs[0].shape[0]
    ts = [torch.from_numpy(np.ascontiguousarray(v.astype(dt))).cuda() for v in arrs]
    info = torch.full((batch,), -7, dtype=torch.int32, device="cuda")
    x = T.gtsv(*ts, n, info=info)
    torch.cuda.synchronize()
    return x.double().cpu().numpy().reshape(batch, n), info.cpu().numpy()


def _check(arrs, x, dt, n, forward):
    a_, b_, c_, d_ = (v.astype(dt).astype(np.float64) for v in arrs)
    a_[:, 0] = 0.0
    c_[:, -1] = 0.0
    _, worst = O.backward_error(a_, b_, c_, d_, x, n)
    assert worst <= ETA[dt], worst
    if forward:
        xo = O.gtsv(a_, b_, c_, d_, n).reshape(x.shape)
        rel = np.max(np.abs(x - xo), axis=1) / np.max(np.abs(xo), axis=1)
        assert rel.max() <= FWD[dt], rel


@pytest.mark.parametrize("dt,n,batch", [(np.float64, 65536, 3), (np.float64, 30001, 4), (np.float64, 8448 * 4 + 7, 2),
                                        (np.float64, 12288, 5), (np.float64, 16384, 3), (np.float64, 27648, 2),
                                        (np.float32, 70000, 3), (np.float32, 200000, 2)])
@pytest.mark.parametrize("dominant", [False, True])
def test_long_pivoted_matches_oracle(cuda, dt, n, batch, dominant):
    import tridiagonalsolver_gb300 as T

    gen = inputs.dominant if dominant else inputs.nondominant
    arrs = gen(n, batch, seed=n + batch)
    T.lib().tridiag_partition_fallbacks(1)
    x, info = _run(cuda, T, arrs, dt, n)
    assert (info == 0).all()
    fb = T.lib().tridiag_partition_fallbacks(1)
    assert fb <= batch  # counted per system
    _check(arrs, x, dt, n, forward=dominant)


def test_long_pivoted_flagged_system_takes_sequential_solve(cuda):
    """A singular interior block in chunk 2 of system 1 (the first row of a
    partition with zero diagonal and superdiagonal: its only entry couples to
    the previous separator; the matrix itself is regular): the chunk's
    separator check fails, system 1 is solved sequentially, the others by the
    chunks."""
    import tridiagonalsolver_gb300 as T

    n, batch = 40000, 3
    a, b, c, d = inputs.nondominant(n, batch, seed=17)
    r = 2 * 128 * 33 + 5 * 33
    b[1, r] = 0.0
    c[1, r] = 0.0
    a[1, r] = 1.0
    T.lib().tridiag_partition_fallbacks(1)
    x, info = _run(cuda, T, (a, b, c, d), np.float64, n)
    assert (info == 0).all()
    assert T.lib().tridiag_partition_fallbacks(1) >= 1
    _check((a, b, c, d), x, np.float64, n, forward=False)


def test_long_pivoted_singular_matrix_info(cuda):
    """A zero row: LAPACK's info (k+1) from the sequential solve the chunk
    check hands the system to; the other systems solve normally."""
    from scipy.linalg import lapack

    import tridiagonalsolver_gb300 as T

    n, batch = 30000, 3
    a, b, c, d = inputs.nondominant(n, batch, seed=19)
    a[2, 12345] = b[2, 12345] = c[2, 12345] = 0.0
    _, info = _run(cuda, T, (a, b, c, d), np.float64, n)
    want = lapack.dgtsv(a[2, 1:].copy(), b[2].copy(), c[2, :-1].copy(), d[2].copy())[4]
    assert info[0] == 0 and info[1] == 0
    assert info[2] == want and want > 0
