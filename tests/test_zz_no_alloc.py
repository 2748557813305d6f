"""The pivoted solve that allocates nothing (tridiag_gtsv_noalloc_*).

It exists for callers that cannot allocate device memory where they solve
(hard latency budgets, memory owned by another allocator); its scratch is a
static device array shared by all calls.  This test calls it through the C
ABI twice in a row on different systems, in each layout, and compares each
result with the existing pivoted entry point (tridiag_gtsv_*, caller-provided
workspace):
max |x_noalloc - x_gtsv| / max |x_gtsv| <= 1e-12 (FP64) / 1e-5 (FP32) per
system, and normwise backward error <= 1e-12 / 1e-6.  It also checks that a
call after the first one leaves the device's free memory unchanged, and
that a problem larger than the static array is refused, and that a call
captured in a CUDA graph replays to the direct call's bits.  The file is named to be
collected last; it passes alone and after the other tests.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from tridiagonalsolver_gb300 import inputs

pytestmark = pytest.mark.gpu

TOL = {np.float64: (1e-12, 1e-12), np.float32: (1e-5, 1e-6)}


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("layout", ["contiguous", "interleaved", "packed"])
def test_noalloc_matches_gtsv_two_calls(cuda, dt, layout):
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300._lib import LAYOUTS, SUCCESS

    lib = T.lib()
    fn = lib.tridiag_gtsv_noalloc_double if dt == np.float64 else lib.tridiag_gtsv_noalloc_single
    rel_tol, eta_tol = TOL[dt]
    n, batch = 300, 96
    es = np.dtype(dt).itemsize
    stream = cuda.cuda.current_stream().cuda_stream
    for call in range(2):
        # the second call solves different systems (another seed and
        # distribution) on the scratch the first call left behind
        if call == 0:
            a, b, c, d = (v.astype(dt) for v in inputs.dominant(n, batch, seed=41))
        else:
            a, b, c, d = (v.astype(dt) for v in inputs.reference(n, batch, seed=42)[:4])
        if layout == "packed":
            # one packed array [batch][a|b|c|d][n]; x in the d rows of a copy
            tp = cuda.from_numpy(inputs.to_packed(a, b, c, d).astype(dt)).cuda()
            x_ref = T.gtsv(tp, None, None, None, n, layout="packed")
            x_new = tp.clone()
            ptrs = (tp.data_ptr(), None, None, x_new.data_ptr() + 3 * n * es)
        else:
            host = (a, b, c, d)
            if layout == "interleaved":
                host = inputs.to_interleaved(*host)
            ta, tb, tc, td = (cuda.from_numpy(np.ascontiguousarray(v)).cuda() for v in host)
            x_ref = T.gtsv(ta, tb, tc, td, n, layout=layout)
            x_new = td.clone()
            ptrs = (ta.data_ptr(), tb.data_ptr(), tc.data_ptr(), x_new.data_ptr())
        info = cuda.full((batch,), -1, dtype=cuda.int32, device="cuda")
        st = fn(LAYOUTS[layout], *(ctypes.c_void_p(v) if v else None for v in ptrs),
                ctypes.c_void_p(info.data_ptr()), n, batch, ctypes.c_void_p(stream))
        assert st == SUCCESS
        cuda.cuda.synchronize()
        assert int(info.abs().sum()) == 0
        xr = x_ref.double().cpu().numpy()
        xn = x_new.double().cpu().numpy()
        if layout == "interleaved":
            xr, xn = xr.T, xn.T
        if layout == "packed":
            xr, xn = xr.reshape(batch, 4, n)[:, 3, :], xn.reshape(batch, 4, n)[:, 3, :]
            # the a, b, c rows of the copy are untouched
            np.testing.assert_array_equal(x_new.cpu().numpy().reshape(batch, 4, n)[:, :3, :],
                                          tp.cpu().numpy().reshape(batch, 4, n)[:, :3, :])
        xr, xn = xr.reshape(batch, n), xn.reshape(batch, n)
        rel = np.max(np.abs(xn - xr), axis=1) / np.max(np.abs(xr), axis=1)
        assert np.max(rel) <= rel_tol, (call, float(np.max(rel)))
        _, eta = O.backward_error(*(v.astype(np.float64) for v in (a, b, c, d)), xn, n)
        assert eta <= eta_tol, (call, eta)


def test_noalloc_refuses_oversized_problem(cuda):
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300._lib import ERR_WORKSPACE

    lib = T.lib()
    # 2 * n * batch * 8 bytes > 32 MiB: refused before any launch, so the
    # (never dereferenced) pointers may be small dummies
    n, batch = 4096, 1024
    p = cuda.zeros(16, dtype=cuda.float64, device="cuda")
    ptr = ctypes.c_void_p(p.data_ptr())
    st = lib.tridiag_gtsv_noalloc_double(0, ptr, ptr, ptr, ptr, None, n, batch, None)
    assert st == ERR_WORKSPACE


def test_noalloc_leaves_free_memory_unchanged(cuda):
    """After a first call on the device (which looks up the static array's
    address), further calls take no device memory: cudaMemGetInfo's free
    bytes are the same before and after."""
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300._lib import SUCCESS

    lib = T.lib()
    n, batch = 1000, 256
    a, b, c, d = (cuda.from_numpy(v.copy()).cuda() for v in inputs.nondominant(n, batch, seed=43))
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    x = d.clone()
    # warm-up: the first call of each kernel (this entry point's and torch's
    # copy) may load its module, which takes device memory once
    x.copy_(d)
    assert lib.tridiag_gtsv_noalloc_double(0, P(a), P(b), P(c), P(x), None, n, batch, None) == SUCCESS
    cuda.cuda.synchronize()
    free0, _ = cuda.cuda.mem_get_info()
    for _ in range(3):
        x.copy_(d)
        assert lib.tridiag_gtsv_noalloc_double(0, P(a), P(b), P(c), P(x), None, n, batch, None) == SUCCESS
    cuda.cuda.synchronize()
    free1, _ = cuda.cuda.mem_get_info()
    assert free1 == free0
    _, eta = O.backward_error(*(t.cpu().numpy() for t in (a, b, c, d, x)), n)
    assert eta <= 1e-12


def test_noalloc_in_a_cuda_graph(cuda):
    """After its first call the entry point can be captured: one call captured
    in a CUDA graph on a side stream, replayed on new right-hand sides copied
    into the captured buffer, gives the direct call's bits."""
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300._lib import SUCCESS

    torch = cuda
    lib = T.lib()
    n, batch = 700, 128
    a, b, c, d = (torch.from_numpy(v.copy()).cuda() for v in inputs.nondominant(n, batch, seed=44))
    d2 = torch.from_numpy(inputs.nondominant(n, batch, seed=45)[3].copy()).cuda()
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    s = torch.cuda.Stream()
    x = d.clone()
    with torch.cuda.stream(s):
        st = ctypes.c_void_p(s.cuda_stream)
        assert lib.tridiag_gtsv_noalloc_double(0, P(a), P(b), P(c), P(x), None, n, batch, st) == SUCCESS
        s.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            assert lib.tridiag_gtsv_noalloc_double(0, P(a), P(b), P(c), P(x), None, n, batch, st) == SUCCESS
        x.copy_(d2)
        g.replay()
    s.synchronize()
    want = d2.clone()
    assert lib.tridiag_gtsv_noalloc_double(0, P(a), P(b), P(c), P(want), None, n, batch, None) == SUCCESS
    torch.cuda.synchronize()
    assert torch.equal(x, want)
    _, eta = O.backward_error(*(t.cpu().numpy() for t in (a, b, c, d2, x)), n)
    assert eta <= 1e-12
