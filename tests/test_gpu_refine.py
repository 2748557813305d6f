"""Mixed-precision refined solve (FP32 pivoted solves + FP64 residuals)
against the FP64 pivoted oracle, and the integer-pipe FP64 <-> FP32
conversions it uses against numpy's IEEE conversions (bit-exact).

Tolerances: after two refinement steps the normwise backward error is
<= 1e-12 (the FP64 bar) for every delta of the b_i = s_i (1 + delta)
(|a_i| + |c_i|) family, and the forward error to the FP64 oracle is
<= 1e-10 relative to max|x|; with no refinement step the backward error is
the FP32 bar, <= 1e-6.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tridiagonalsolver_gb300 import inputs

pytestmark = pytest.mark.gpu


def test_conversions_bit_exact(cuda):
    import tridiagonalsolver_gb300 as T

    torch = cuda
    rng = np.random.default_rng(0)
    v = np.concatenate([
        rng.uniform(-1, 1, 100000),
        rng.standard_normal(100000) * 10.0 ** rng.uniform(-50, 50, 100000),
        # round-to-even ties and their neighbours in the dropped 29 bits
        (np.float32(rng.uniform(1, 2, 1000)).astype(np.float64).view(np.uint64) + np.uint64(1 << 28)).view(
            np.float64),
        (np.float32(rng.uniform(1, 2, 1000)).astype(np.float64).view(np.uint64) + np.uint64((1 << 28) - 1)).view(
            np.float64),
        (np.float32(rng.uniform(1, 2, 1000)).astype(np.float64).view(np.uint64) + np.uint64((1 << 28) + 1)).view(
            np.float64),
        np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324, 1e-310, 3.4028234663852886e38,
                  3.4028235677973366e38, 3.5e38, -3.5e38, 1.1754943508222875e-38, 1.4e-45, 7e-46, 1e-40,
                  np.finfo(np.float32).max, np.finfo(np.float32).tiny, 1.0 + 2.0 ** -24, 1.0 + 3 * 2.0 ** -24]),
    ])
    out, back = T.convert_check(torch.from_numpy(v).cuda())
    out = out.cpu().numpy()
    back = back.cpu().numpy()
    with np.errstate(over="ignore"):
        ref = v.astype(np.float32)
    nan = np.isnan(v)
    assert np.isnan(out[nan]).all() and np.isnan(back[nan]).all()  # NaN payloads are not compared
    assert np.array_equal(out[~nan].view(np.uint32), ref[~nan].view(np.uint32))
    assert np.array_equal(back[~nan].view(np.uint64), ref[~nan].astype(np.float64).view(np.uint64))


@pytest.mark.parametrize("layout", ["contiguous", "interleaved"])
@pytest.mark.parametrize("delta", [1.0, 1e-2, 1e-4, 1e-6])
@pytest.mark.parametrize("n,batch", [(4096, 16), (1000, 33), (37, 8)])
def test_refine_matches_fp64_oracle(cuda, layout, delta, n, batch):
    import tridiagonalsolver_gb300 as T

    torch = cuda
    a, b, c, d = inputs.scaled(n, batch, delta, seed=int(n + 1e6 * delta) % 1000)
    arrs = (a, b, c, d)
    if layout == "interleaved":
        arrs = inputs.to_interleaved(*arrs)
    ts = [torch.from_numpy(np.ascontiguousarray(v)).cuda() for v in arrs]
    info = torch.zeros(batch, dtype=torch.int32, device="cuda")
    x = T.refine(*ts, n, iters=2, layout=layout, info=info)
    x0 = T.refine(*ts, n, iters=0, layout=layout)
    torch.cuda.synchronize()
    assert int(info.abs().sum()) == 0

    def host(t):
        h = t.cpu().numpy()
        return h.reshape(n, batch).T.copy() if layout == "interleaved" else h.reshape(batch, n)

    xo = O.gtsv(a, b, c, d, n).reshape(batch, n)
    _, eta = O.backward_error(a, b, c, d, host(x), n)
    _, eta0 = O.backward_error(a, b, c, d, host(x0), n)
    assert eta <= 1e-12
    assert eta0 <= 1e-6
    fe = np.max(np.abs(host(x) - xo)) / np.max(np.abs(xo))
    assert fe <= 1e-10


def test_refine_full_size_delta_sweep(cuda):
    """n = 65536, batch = 1024, every delta; backward error of 16 sampled
    systems per delta against the FP64 oracle."""
    import tridiagonalsolver_gb300 as T

    torch = cuda
    n, batch = 65536, 1024
    g = torch.Generator(device="cuda")
    g.manual_seed(65536)
    work = None
    for delta in (1.0, 1e-2, 1e-4, 1e-6):
        def u(lo, hi):
            return torch.rand((batch, n), dtype=torch.float64, device="cuda", generator=g) * (hi - lo) + lo

        a, c, d = u(-1, 1), u(-1, 1), u(-1, 1)
        a[:, 0] = 0
        c[:, -1] = 0
        s = torch.where(u(0, 1) < 0.5, -1.0, 1.0)
        b = s * (1 + delta) * (a.abs() + c.abs())
        work = work if work is not None else T.refine_workspace(a, n)
        x = T.refine(a, b, c, d, n, iters=2, work=work)
        idx = torch.arange(0, batch, batch // 16, device="cuda")
        host = [t.index_select(0, idx).cpu().numpy() for t in (a, b, c, d, x)]
        _, eta = O.backward_error(*host, n)
        assert eta <= 1e-12, (delta, eta)
        del a, b, c, d, x


def test_refine_argument_errors(cuda):
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300 import TridiagError

    torch = cuda
    n, batch = 64, 4
    ts = [torch.ones(batch * n, dtype=torch.float64, device="cuda") for _ in range(4)]
    with pytest.raises(TridiagError):
        T.refine(*ts, n, iters=9)
    with pytest.raises(TridiagError):
        T.refine(*ts, n, layout="packed")
    with pytest.raises(TridiagError):
        T.refine(*ts, n, work=torch.empty(16, dtype=torch.uint8, device="cuda"))
