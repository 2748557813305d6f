"""Solves with the arrays in host memory (tridiag_solve_host_*): the chunked
host -> device -> host pipeline returns, system by system, the same bits as
the device entry point tridiag_solve_out_* with the same algorithm wherever
both run the same kernels, and meets the oracle's backward-error bar.

Tolerances: normwise backward error <= 1e-12 (FP64) / 1e-6 (FP32) against the
FP64 oracle; equality with the device path is exact where both see the same
kernels (the kernels solve each system independently of the batch around it).
"""
import numpy as np
import pytest

from oracle import oracle as O
from tridiagonalsolver_gb300 import inputs

pytestmark = pytest.mark.gpu

ETA = {np.float64: 1e-12, np.float32: 1e-6}


def _host(torch, arrs, dt, layout):
    td = torch.float32 if dt == np.float32 else torch.float64
    out = []
    for v in arrs:
        v = v.astype(dt)
        if layout == "interleaved":
            v = np.ascontiguousarray(v.T)
        out.append(torch.from_numpy(v).to(td).pin_memory())
    return out


def _case(torch, T, dt, n, batch, algo, layout, chunk, dominant=True, exact=True):
    gen = inputs.dominant if dominant else inputs.nondominant
    a, b, c, d = gen(n, batch, seed=n + batch)
    ha, hb, hc, hd = _host(torch, (a, b, c, d), dt, layout)
    x = T.solve_host(ha, hb, hc, hd, n, algo=algo, layout=layout, chunk=chunk)
    torch.cuda.synchronize()
    # the device path on the same inputs
    da, db, dc, dd = (t.cuda() for t in (ha, hb, hc, hd))
    xd = T.solve_out(da, db, dc, dd, n, algo=algo, layout=layout)
    torch.cuda.synchronize()
    if exact:
        assert torch.equal(x, xd.cpu())
    xs = x.numpy()
    if layout == "interleaved":
        xs = np.ascontiguousarray(xs.T)
    a64, b64, c64, d64 = (v.astype(dt).astype(np.float64) for v in (a, b, c, d))
    a64[:, 0] = 0.0
    c64[:, -1] = 0.0
    _, eta = O.backward_error(a64, b64, c64, d64, xs.astype(np.float64).reshape(-1), n)
    assert eta <= ETA[dt], eta


@pytest.mark.parametrize("dt,n,batch,algo,chunk", [
    (np.float32, 512, 3000, "pcr", 700),      # five chunks, the last one short
    (np.float32, 512, 2048, "cr", 0),         # automatic chunk
    (np.float64, 4096, 300, "wm", 128),       # the pivoted partitioned solve per chunk
    (np.float64, 1000, 77, "gtsv", 10),
    (np.float32, 4096, 96, "partition", 40),
])
def test_host_solve_contiguous(cuda, dt, n, batch, algo, chunk):
    import tridiagonalsolver_gb300 as T

    _case(cuda, T, dt, n, batch, algo, "contiguous", chunk, dominant=algo not in ("wm", "gtsv"))


@pytest.mark.parametrize("dt,algo", [(np.float32, "thomas"), (np.float64, "thomas"), (np.float64, "gtsv")])
@pytest.mark.parametrize("batch,chunk", [(512, 128), (517, 100)])
def test_host_solve_interleaved(cuda, dt, algo, batch, chunk):
    """Interleaved rows move by 2-D copies.  Bit equality with the device path
    holds where both see the same kernels: the interleaved sweeps take TMA
    boxes only when a row of the batch is a multiple of 16 bytes, so a batch
    of 517 (device path: plain loads) and its chunks of 100 (TMA) may differ
    in the last bits; both meet the bar."""
    import tridiagonalsolver_gb300 as T

    _case(cuda, T, dt, 1000, batch, algo, "interleaved", chunk, exact=batch % 4 == 0)


def test_host_solves_from_two_streams(cuda):
    """Two calls queued from independent streams share the pipeline; both
    results are complete after both streams are synchronised."""
    import tridiagonalsolver_gb300 as T

    torch = cuda
    n, batch = 512, 1024
    sets = []
    for seed in (1, 2):
        a, b, c, d = inputs.dominant(n, batch, seed=seed)
        sets.append((a, b, c, d, _host(torch, (a, b, c, d), np.float32, "contiguous")))
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    xs = [T.solve_host(*h, n, algo="pcr", chunk=200, stream=s) for (_, _, _, _, h), s in zip(sets, (s1, s2))]
    s1.synchronize()
    s2.synchronize()
    for (a, b, c, d, _), x in zip(sets, xs):
        a64, b64, c64, d64 = (v.astype(np.float32).astype(np.float64) for v in (a, b, c, d))
        a64[:, 0] = 0.0
        c64[:, -1] = 0.0
        _, eta = O.backward_error(a64, b64, c64, d64, x.numpy().astype(np.float64).reshape(-1), n)
        assert eta <= ETA[np.float32], eta


def test_host_solve_arguments(cuda):
    import tridiagonalsolver_gb300 as T

    torch = cuda
    h = torch.ones(4 * 64, dtype=torch.float32).pin_memory()
    with pytest.raises(T.TridiagError):
        T.solve_host(h, h, h, h, 64, layout="packed")
    with pytest.raises(ValueError):
        T.solve_host(h.cuda(), h, h, h, 64)
    assert T.lib().tridiag_solve_host_single(0, 0, None, None, None, None, None, 64, 4, 0, None) != 0
