"""Partition method without pivoting, one CTA per system (TRIDIAG_ALGO_PARTITION),
against the oracle on diagonally dominant systems, through the C ABI.

Tolerances: normwise backward error <= 1e-12 (FP64) / 1e-6 (FP32); max |x -
x_oracle| / max |x_oracle| <= 1e-12 (FP64) / 1e-5 (FP32) against the FP64
pivoted oracle.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tridiagonalsolver_gb300 import inputs

pytestmark = pytest.mark.gpu

ETA = {np.float64: 1e-12, np.float32: 1e-6}
FWD = {np.float64: 1e-12, np.float32: 1e-5}
# eligible sizes: n = R * 128 / sizeof(T) rows, 8 <= R <= 256
SIZES = {np.float32: [256, 1056, 2048, 4096, 8192], np.float64: [128, 528, 2048, 4096]}


def _check(x, a, b, c, d, dt, n):
    batch = x.size // n
    a64, b64, c64, d64 = (v.astype(dt).astype(np.float64) for v in (a, b, c, d))
    _, eta = O.backward_error(a64, b64, c64, d64, x, n)
    assert eta <= ETA[dt], eta
    xo = O.gtsv(a64, b64, c64, d64, n).reshape(batch, n)
    rel = np.max(np.abs(x.reshape(batch, n) - xo), axis=1) / np.max(np.abs(xo), axis=1)
    assert rel.max() <= FWD[dt], rel.max()


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("idx", range(5))
@pytest.mark.parametrize("batch", [1, 7, 100])
def test_partition_in_and_out_of_place(cuda, dt, idx, batch):
    import tridiagonalsolver_gb300 as T

    if idx >= len(SIZES[dt]):
        pytest.skip("size list shorter for this precision")
    n = SIZES[dt][idx]
    a, b, c, d = inputs.dominant(n, batch, seed=n + batch)
    ts = [cuda.from_numpy(v.astype(dt)).cuda() for v in (a, b, c, d)]
    x = T.solve_out(*ts, n, algo="partition").double().cpu().numpy()
    _check(x, a, b, c, d, dt, n)
    # inputs untouched by the out-of-place solve
    for t, v in zip(ts, (a, b, c, d)):
        np.testing.assert_array_equal(t.cpu().numpy(), v.astype(dt))
    T.solve(*ts, n, algo="partition")
    x2 = ts[3].double().cpu().numpy()
    assert np.array_equal(x, x2)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_partition_packed(cuda, dt):
    import tridiagonalsolver_gb300 as T

    n, batch = (2048 if dt == np.float32 else 1024), 9
    a, b, c, d = inputs.dominant(n, batch, seed=5)
    p = cuda.from_numpy(inputs.to_packed(a, b, c, d).astype(dt)).cuda()
    T.solve(p, None, None, None, n, algo="partition", layout="packed")
    x = p.double().cpu().numpy().reshape(batch, 4, n)[:, 3, :]
    _check(x, a, b, c, d, dt, n)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_partition_ignores_a0_and_clast(cuda, dt):
    import tridiagonalsolver_gb300 as T

    n, batch = 4096, 5
    a, b, c, d = inputs.dominant(n, batch, seed=9)
    ts = [cuda.from_numpy(v.astype(dt)).cuda() for v in (a, b, c, d)]
    x0 = T.solve_out(*ts, n, algo="partition").cpu().numpy()
    a2, c2 = a.copy(), c.copy()
    a2[:, 0] = np.nan
    c2[:, -1] = np.nan
    ts2 = [cuda.from_numpy(v.astype(dt)).cuda() for v in (a2, b, c2, d)]
    x1 = T.solve_out(*ts2, n, algo="partition").cpu().numpy()
    assert np.array_equal(x0, x1)


@pytest.mark.parametrize("dt,n", [(np.float32, 1000), (np.float32, 8200), (np.float64, 100), (np.float64, 4100),
                                  (np.float32, 3000), (np.float32, 1), (np.float32, 33), (np.float64, 4095)])
def test_partition_any_n(cuda, dt, n):
    """n not a multiple of the 128-byte row: the element-wise staging up to
    8192 (FP32) / 4096 (FP64) rows, the Thomas sweep beyond (8200, 4100)."""
    import tridiagonalsolver_gb300 as T

    batch = 6
    a, b, c, d = inputs.dominant(n, batch, seed=n)
    ts = [cuda.from_numpy(v.astype(dt)).cuda() for v in (a, b, c, d)]
    x = T.solve_out(*ts, n, algo="partition").double().cpu().numpy()
    _check(x, a, b, c, d, dt, n)
    T.solve(*ts, n, algo="partition")
    _check(ts[3].double().cpu().numpy(), a, b, c, d, dt, n)


@pytest.mark.parametrize("name,dt", [("PCR5_reg_single", np.float32), ("CR_reg8_single", np.float32),
                                     ("PCR5_reg_double", np.float64), ("CR_reg8_double", np.float64)])
def test_reference_cr_pcr_names_long_systems(cuda, name, dt):
    """The reference's CR and PCR entry points beyond one warp's reach run
    the partition kernel (in place, d <- x)."""
    import tridiagonalsolver_gb300 as T

    n, batch = 4096, 6
    a, b, c, d = inputs.dominant(n, batch, seed=2)
    ts = [cuda.from_numpy(v.astype(dt)).cuda() for v in (a, b, c, d)]
    T.reference_call(name, *ts, n)
    _check(ts[3].double().cpu().numpy(), a, b, c, d, dt, n)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_auto_uses_partition_and_is_exact_same(cuda, dt):
    import tridiagonalsolver_gb300 as T

    n, batch = 4096, 4
    a, b, c, d = inputs.dominant(n, batch, seed=12)
    ts = [cuda.from_numpy(v.astype(dt)).cuda() for v in (a, b, c, d)]
    xa = T.solve_out(*ts, n, algo="auto").cpu().numpy()
    xp = T.solve_out(*ts, n, algo="partition").cpu().numpy()
    assert np.array_equal(xa, xp)
    _check(xa.astype(np.float64), a, b, c, d, dt, n)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("n,batch", [(256, 50), (1024, 33), (4096, 5)])
def test_partition_adjoint_vs_oracle(cuda, dt, n, batch):
    """Adjoint of the partition solve (A^T lambda = xbar and the gradients)
    against the FP64 oracle adjoint: max |g - g_oracle| / max |g_oracle| <=
    1e-12 (FP64) / 1e-5 (FP32), per gradient."""
    import tridiagonalsolver_gb300 as T

    if not T.partition_supported(cuda.zeros(1, dtype=cuda.float64 if dt == np.float64 else cuda.float32), n):
        pytest.skip("shape outside the partition kernel")
    a, b, c, d = inputs.dominant(n, batch, seed=n + 3)
    w = np.random.default_rng(n).uniform(-1, 1, (batch, n))
    ts = [cuda.from_numpy(v.astype(dt)).cuda() for v in (a, b, c, d, w)]
    x = T.solve_out(*ts[:4], n, algo="partition")
    grads = T.partition_adjoint(ts[0], ts[1], ts[2], x, ts[4], n)
    h = [v.astype(dt).astype(np.float64) for v in (a, b, c)]
    ref = O.adjoint_f64(*h, x.double().cpu().numpy(), w.astype(dt).astype(np.float64), n)
    tol = 1e-12 if dt == np.float64 else 1e-5
    for gg, r, name in zip(grads, ref, ("ga", "gb", "gc", "gd")):
        g = gg.double().cpu().numpy().reshape(-1)
        assert np.max(np.abs(g - r)) <= tol * np.max(np.abs(r)), name
    # the boundary gradients vanish
    assert float(grads[0].view(batch, n)[:, 0].abs().max()) == 0.0
    assert float(grads[2].view(batch, n)[:, -1].abs().max()) == 0.0


def test_partition_adjoint_unsupported_shape(cuda):
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300 import TridiagError

    t = cuda.ones(9000 * 2, dtype=cuda.float32, device="cuda")
    with pytest.raises(TridiagError):
        T.partition_adjoint(t, t, t, t, t, 9000)


def test_solve_ad_unpivoted_gradcheck(cuda):
    """torch.autograd.gradcheck through the unpivoted partition method (FP64,
    n = 128: the smallest shape the kernel covers)."""
    import torch

    from tridiagonalsolver_gb300 import solve_ad

    n, batch = 128, 3
    a, b, c, d = inputs.dominant(n, batch, seed=1)
    ts = [torch.from_numpy(v).cuda().requires_grad_(True) for v in (a, b, c, d)]
    assert torch.autograd.gradcheck(lambda *v: solve_ad(*v, pivoting=False), ts, eps=1e-6, atol=1e-5, rtol=1e-4)


@pytest.mark.parametrize("dt,n", [(np.float32, 8224), (np.float32, 20000), (np.float32, 65536),
                                  (np.float64, 4112), (np.float64, 12288), (np.float64, 65536)])
def test_partition_long_systems(cuda, dt, n):
    """Systems beyond one CTA: chunks per CTA, the separators' system, chunks
    again (last chunk shorter for 8224, 20000, 4112)."""
    import tridiagonalsolver_gb300 as T

    assert T.lib().tridiag_partition_supported(1 if dt == np.float64 else 0, 0, n) == 0
    batch = 3
    a, b, c, d = inputs.dominant(n, batch, seed=n % 1000)
    ts = [cuda.from_numpy(v.astype(dt)).cuda() for v in (a, b, c, d)]
    x = T.solve_out(*ts, n, algo="partition").double().cpu().numpy()
    _check(x, a, b, c, d, dt, n)
    xa = T.solve_out(*ts, n, algo="auto").double().cpu().numpy()
    assert np.array_equal(x, xa)
    T.solve(*ts, n, algo="partition")
    assert np.array_equal(ts[3].double().cpu().numpy(), x)


@pytest.mark.parametrize("delta", [1.0, 1e-6])
def test_refine_with_partition_solves(cuda, delta):
    """Refined solve with unpivoted FP32 partition solves on the refined
    workload's distribution (diagonally dominant by construction): backward
    error <= 1e-12 after two steps, as the pivoted version."""
    import tridiagonalsolver_gb300 as T

    n, batch = 65536, 4
    rng = np.random.default_rng(7)
    a, c, d = (rng.uniform(-1, 1, (batch, n)) for _ in range(3))
    a[:, 0] = 0
    c[:, -1] = 0
    s_ = np.where(rng.uniform(-1, 1, (batch, n)) >= 0, 1.0, -1.0)
    b = s_ * (1 + delta) * (np.abs(a) + np.abs(c))
    b[b == 0] = 1.0
    ts = [cuda.from_numpy(v).cuda() for v in (a, b, c, d)]
    x = T.refine(*ts, n, iters=2, algo="partition").cpu().numpy()
    _, eta = O.backward_error(a, b, c, d, x, n)
    assert eta <= 1e-12


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("n", [1, 77, 1000, 3001])
def test_partition_adjoint_any_n(cuda, dt, n):
    import tridiagonalsolver_gb300 as T

    if dt == np.float64 and n > 4096:
        pytest.skip("beyond the FP64 single-CTA reach")
    batch = 9
    a, b, c, d = inputs.dominant(n, batch, seed=n + 11)
    w = np.random.default_rng(n).uniform(-1, 1, (batch, n))
    ts = [cuda.from_numpy(v.astype(dt)).cuda() for v in (a, b, c, d, w)]
    x = T.solve_out(*ts[:4], n, algo="partition")
    grads = T.partition_adjoint(ts[0], ts[1], ts[2], x, ts[4], n)
    h = [v.astype(dt).astype(np.float64) for v in (a, b, c)]
    ref = O.adjoint_f64(*h, x.double().cpu().numpy(), w.astype(dt).astype(np.float64), n)
    tol = 1e-12 if dt == np.float64 else 1e-5
    for gg, r, name in zip(grads, ref, ("ga", "gb", "gc", "gd")):
        g = gg.double().cpu().numpy().reshape(-1)
        assert np.max(np.abs(g - r)) <= tol * max(np.max(np.abs(r)), 1e-300), name
