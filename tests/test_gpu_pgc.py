"""Cluster version of the partitioned partial-pivoting solve (one cluster of
2, 4 or 8 CTAs per system, the system kept in distributed shared memory)
for systems longer than one CTA's shared memory, against the oracle.

Tolerances: normwise backward error <= 1e-12 (FP64) / 1e-6 (FP32), computed
in FP64 by the oracle; info is 0 for every system (n + 1 would flag a result
that missed the kernel's own accuracy check).
"""
import numpy as np
import pytest

from oracle import oracle as O
from tridiagonalsolver_gb300 import inputs

pytestmark = pytest.mark.gpu

ETA = {np.float64: 1e-12, np.float32: 1e-6}


def _run(cuda, arrs, dt, n):
    import tridiagonalsolver_gb300 as T

    batch = arrs[0].shape[0]
    ts = [cuda.from_numpy(np.ascontiguousarray(v.astype(dt))).cuda() for v in arrs]
    info = cuda.full((batch,), -7, dtype=cuda.int32, device="cuda")
    x = T.pge(*ts, n, info=info)
    cuda.cuda.synchronize()
    return x.double().cpu().numpy().reshape(batch, n), info.cpu().numpy()


@pytest.mark.parametrize("dist", ["dominant", "nondominant"])
@pytest.mark.parametrize("dt,n,batch", [(np.float32, 9000, 4), (np.float32, 16384, 3), (np.float32, 20000, 3),
                                        (np.float32, 40001, 2), (np.float32, 65536, 2), (np.float64, 4481, 3),
                                        (np.float64, 12000, 2), (np.float64, 27648, 2)])
def test_pgc_matches_oracle(cuda, dist, dt, n, batch):
    gen = inputs.dominant if dist == "dominant" else inputs.nondominant
    a, b, c, d = gen(n, batch, seed=n + batch)
    x, info = _run(cuda, (a, b, c, d), dt, n)
    assert (info == 0).all(), info
    a_, b_, c_, d_ = (v.astype(dt).astype(np.float64) for v in (a, b, c, d))
    _, worst = O.backward_error(a_, b_, c_, d_, x, n)
    assert worst <= ETA[dt]
    if dist == "dominant":
        xo = O.gtsv(a_, b_, c_, d_, n).reshape(batch, n)
        rel = np.max(np.abs(x - xo)) / np.max(np.abs(xo))
        assert rel <= (1e-13 if dt == np.float64 else 1e-5)


@pytest.mark.parametrize("delta", [1.0, 1e-2, 1e-4, 1e-6])
def test_pgc_scaled_fp32(cuda, delta):
    """The refined-solve family b = s (1 + delta)(|a| + |c|), FP32, n = 65536."""
    n, batch = 65536, 2
    a, b, c, d = inputs.scaled(n, batch, delta, seed=5)
    x, info = _run(cuda, (a, b, c, d), np.float32, n)
    assert (info == 0).all()
    _, worst = O.backward_error(*(v.astype(np.float32).astype(np.float64) for v in (a, b, c, d)), x, n)
    assert worst <= 1e-6


def test_pgc_in_place_and_long_gtsv(cuda):
    """tridiag_gtsv_* without a pivot record routes long systems here; in
    place (x aliasing d) works."""
    import tridiagonalsolver_gb300 as T

    n, batch = 30000, 3
    a, b, c, d = inputs.nondominant(n, batch, seed=17)
    ts = [cuda.from_numpy(v.astype(np.float32)).cuda() for v in (a, b, c, d)]
    x = T.gtsv(*ts, n, out=ts[3])
    assert x.data_ptr() == ts[3].data_ptr()
    _, worst = O.backward_error(*(v.astype(np.float32).astype(np.float64) for v in (a, b, c, d)),
                                x.double().cpu().numpy().reshape(batch, n), n)
    assert worst <= 1e-6


@pytest.mark.parametrize("variant,n", [(4, 10399), (5, 10399), (6, 40000)])
def test_cluster_variants_are_deterministic(cuda, variant, n):
    """Repeated solves of the same non-dominant systems through a cluster
    variant give bit-identical results (the cluster-wide maxima of the
    acceptance test are exact, whatever the timing of the CTAs)."""
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300 import ragged

    torch = cuda
    batch = 120 if n < 20000 else 24
    sizes = np.full(batch, n, dtype=np.int64)
    a, b, c, d, off, _ = ragged.synthetic_batch(sizes, seed=9, nondominant_fraction=0.5)
    plan = T.RaggedPlan(off, table={ragged.size_class(n): variant})
    x = torch.empty_like(d)
    plan.solve(a, b, c, d, out=x)
    torch.cuda.synchronize()
    ref = x.clone()
    for _ in range(8):
        x.fill_(float("nan"))
        plan.solve(a, b, c, d, out=x)
        torch.cuda.synchronize()
        assert torch.equal(x, ref)
