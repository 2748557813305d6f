"""Forward + adjoint through the torch.autograd wrapper (FP32 pivoted solve,
loss = sum(w * x)), checked against FP64 central differences and the
oracle's FP64 adjoint.

Tolerances: FP64 gradients agree with torch.autograd.gradcheck's central
differences (eps 1e-6, atol 1e-5, rtol 1e-4); FP32 gradients of the
n = 1024 workload agree with the FP64 oracle adjoint and with FP64 central
differences (h = 1e-6) of the oracle to 2e-3 relative to the largest
gradient entry of the system.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tridiagonalsolver_gb300 import inputs

pytestmark = pytest.mark.gpu


def test_gradcheck_fp64(cuda):
    from tridiagonalsolver_gb300.autograd import solve_ad

    torch = cuda
    n, batch = 12, 3
    a, b, c, d = inputs.nondominant(n, batch, seed=3)
    ts = [torch.from_numpy(v.copy()).cuda().requires_grad_() for v in (a, b, c, d)]
    assert torch.autograd.gradcheck(lambda *v: solve_ad(*v), ts, eps=1e-6, atol=1e-5, rtol=1e-4)


def test_gradcheck_fp64_partitioned(cuda):
    """n = 100: the partitioned solve forward and its transposed solve backward."""
    from tridiagonalsolver_gb300.autograd import TridiagonalSolve, solve_ad

    torch = cuda
    n, batch = 100, 2
    a, b, c, d = inputs.nondominant(n, batch, seed=13)
    ts = [torch.from_numpy(v.copy()).cuda().requires_grad_() for v in (a, b, c, d)]
    x = solve_ad(*ts)
    assert x.grad_fn is not None and type(x.grad_fn).__name__.startswith(TridiagonalSolve.__name__)
    assert torch.autograd.gradcheck(lambda *v: solve_ad(*v), ts, eps=1e-6, atol=1e-5, rtol=1e-4)


def test_pge_adjoint_matches_gtsv_adjoint(cuda):
    """The two adjoint paths agree (FP64, n = 4096 and a cluster-sized n)."""
    import tridiagonalsolver_gb300 as T

    torch = cuda
    for n, batch in ((4096, 8), (20000, 2)):
        a, b, c, d = inputs.nondominant(n, batch, seed=n)
        w = np.random.default_rng(n).uniform(-1, 1, (batch, n))
        ts = [torch.from_numpy(v.copy()).cuda() for v in (a, b, c, d)]
        wt = torch.from_numpy(w).cuda()
        x = T.pge(*ts, n)
        g1 = T.pge_adjoint(ts[0], ts[1], ts[2], x, wt, n)
        xo = O.gtsv(a, b, c, d, n).reshape(batch, n)
        ref = O.adjoint_f64(a, b, c, xo, w, n)
        for g, r in zip(g1, ref):
            r = r.reshape(batch, n)
            err = np.max(np.abs(g.cpu().numpy() - r), axis=1) / np.max(np.abs(r), axis=1)
            assert np.max(err) <= 1e-9


@pytest.mark.parametrize("layout", ["contiguous", "interleaved"])
def test_gradcheck_fp64_layouts(cuda, layout):
    from tridiagonalsolver_gb300.autograd import solve_ad

    torch = cuda
    n, batch = 33, 5
    a, b, c, d = inputs.dominant(n, batch, seed=4)
    if layout == "interleaved":
        a, b, c, d = inputs.to_interleaved(a, b, c, d)
    ts = [torch.from_numpy(np.ascontiguousarray(v)).cuda().requires_grad_() for v in (a, b, c, d)]
    assert torch.autograd.gradcheck(lambda *v: solve_ad(*v, n=n, layout=layout), ts, eps=1e-6, atol=1e-5,
                                    rtol=1e-4)


def test_forward_adjoint_fp32_n1024(cuda):
    """The forward+adjoint workload (FP32, n = 1024, dominant systems, loss =
    sum(w x)) on 16384 systems; gradients of 64 of them checked in FP64."""
    from tridiagonalsolver_gb300.autograd import solve_ad

    torch = cuda
    n, batch = 1024, 16384
    g = torch.Generator(device="cuda")
    g.manual_seed(2024)

    def u(lo, hi):
        return torch.rand((batch, n), device="cuda", generator=g) * (hi - lo) + lo

    a, c, d, w = u(-1, 1), u(-1, 1), u(-1, 1), u(-1, 1)
    a[:, 0] = 0
    c[:, -1] = 0
    b = a.abs() + c.abs() + u(1, 2)
    leaves = [t.clone().requires_grad_() for t in (a, b, c, d)]
    x = solve_ad(*leaves)
    loss = (w * x).sum()
    loss.backward()
    torch.cuda.synchronize()
    idx = torch.arange(0, batch, batch // 64, device="cuda")[:64]
    host = [t.index_select(0, idx).double().cpu().numpy() for t in (a, b, c, d, w)]
    grads = [t.grad.index_select(0, idx).double().cpu().numpy() for t in leaves]
    xo = O.gtsv(*host[:4], n).reshape(64, n)
    xg = x.detach().index_select(0, idx).double().cpu().numpy()
    _, eta = O.backward_error(*host[:4], xg, n)
    assert eta <= 1e-6
    ref = O.adjoint_f64(host[0], host[1], host[2], xo, host[4], n)
    for gg, r in zip(grads, ref):
        r = r.reshape(64, n)
        scale = np.max(np.abs(r), axis=1, keepdims=True)
        assert np.max(np.abs(gg - r) / scale) <= 2e-3
    # FP64 central differences of loss_j = sum_i w_ji x_ji for a few entries
    h = 1e-6
    rng = np.random.default_rng(9)

    def loss_np(v):
        return np.sum(host[4] * O.gtsv(*v, n).reshape(64, n), axis=1)

    for k in range(4):
        for _ in range(3):
            i = int(rng.integers(1, n - 1))
            vp = [v.copy() for v in host[:4]]
            vp[k][:, i] += h
            vm = [v.copy() for v in host[:4]]
            vm[k][:, i] -= h
            fd = (loss_np(vp) - loss_np(vm)) / (2 * h)
            scale = np.max(np.abs(grads[k]), axis=1)
            assert np.max(np.abs(grads[k][:, i] - fd) / scale) <= 2e-3


def test_requires_grad_subset(cuda):
    """Only d requires a gradient: the adjoint still runs and grad_d = lambda."""
    from tridiagonalsolver_gb300.autograd import solve_ad

    torch = cuda
    n, batch = 100, 7
    a, b, c, d = inputs.nondominant(n, batch, seed=8)
    ta, tb, tc = (torch.from_numpy(v.copy()).cuda() for v in (a, b, c))
    td = torch.from_numpy(d.copy()).cuda().requires_grad_()
    w = np.random.default_rng(1).uniform(-1, 1, (batch, n))
    x = solve_ad(ta, tb, tc, td)
    (x * torch.from_numpy(w).cuda()).sum().backward()
    xo = O.gtsv(a, b, c, d, n).reshape(batch, n)
    lam = O.adjoint_f64(a, b, c, xo, w, n)[3].reshape(batch, n)
    assert np.max(np.abs(td.grad.cpu().numpy() - lam)) <= 1e-9 * np.max(np.abs(lam))


def test_solve_from_a_fresh_host_thread(cuda):
    """A thread that has made no CUDA call yet (like autograd's worker) can
    launch the TMA-fed kernels: the library binds the device context."""
    import threading

    import tridiagonalsolver_gb300 as T

    torch = cuda
    n, batch = 64, 32
    a, b, c, d = inputs.nondominant(n, batch, seed=31)
    ts = [torch.from_numpy(v.copy()).cuda() for v in (a, b, c, d)]
    piv = T.pivot_record(ts[0], n)
    torch.cuda.synchronize()
    out = {}

    def work():
        try:
            out["x"] = T.gtsv(*ts, n, pivots=piv)
            torch.cuda.synchronize()
        except Exception as e:  # reported below
            out["err"] = e

    th = threading.Thread(target=work)
    th.start()
    th.join()
    assert "err" not in out, out.get("err")
    _, eta = O.backward_error(a, b, c, d, out["x"].cpu().numpy(), n)
    assert eta <= 1e-12
