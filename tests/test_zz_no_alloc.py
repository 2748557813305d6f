"""The pivoted solve that allocates nothing (tridiag_gtsv_noalloc_*).

It exists for callers that cannot allocate device memory where they solve
(hard latency budgets, memory owned by another allocator); its scratch is a
static device array shared by all calls.  This test calls it through the C
ABI twice in a row on different systems and compares each result with the
existing pivoted entry point (tridiag_gtsv_*, caller-provided workspace):
max |x_noalloc - x_gtsv| / max |x_gtsv| <= 1e-12 (FP64) / 1e-5 (FP32) per
system, and normwise backward error <= 1e-12 / 1e-6.  It also checks that a
problem larger than the static array is refused.  The file is named to be
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
@pytest.mark.parametrize("layout", ["contiguous", "interleaved"])
def test_noalloc_matches_gtsv_two_calls(cuda, dt, layout):
    import tridiagonalsolver_gb300 as T
    from tridiagonalsolver_gb300._lib import LAYOUTS, SUCCESS

    lib = T.lib()
    fn = lib.tridiag_gtsv_noalloc_double if dt == np.float64 else lib.tridiag_gtsv_noalloc_single
    rel_tol, eta_tol = TOL[dt]
    n, batch = 300, 96
    stream = cuda.cuda.current_stream().cuda_stream
    for call in range(2):
        # the second call solves different systems (another seed and
        # distribution) on the scratch the first call left behind
        if call == 0:
            a, b, c, d = (v.astype(dt) for v in inputs.dominant(n, batch, seed=41))
        else:
            a, b, c, d = (v.astype(dt) for v in inputs.reference(n, batch, seed=42)[:4])
        host = (a, b, c, d)
        if layout == "interleaved":
            host = inputs.to_interleaved(*host)
        ta, tb, tc, td = (cuda.from_numpy(np.ascontiguousarray(v)).cuda() for v in host)
        x_ref = T.gtsv(ta, tb, tc, td, n, layout=layout)
        x_new = td.clone()
        info = cuda.full((batch,), -1, dtype=cuda.int32, device="cuda")
        st = fn(LAYOUTS[layout], ctypes.c_void_p(ta.data_ptr()), ctypes.c_void_p(tb.data_ptr()),
                ctypes.c_void_p(tc.data_ptr()), ctypes.c_void_p(x_new.data_ptr()), ctypes.c_void_p(info.data_ptr()),
                n, batch, ctypes.c_void_p(stream))
        assert st == SUCCESS
        cuda.cuda.synchronize()
        assert int(info.abs().sum()) == 0
        xr = x_ref.double().cpu().numpy()
        xn = x_new.double().cpu().numpy()
        if layout == "interleaved":
            xr, xn = xr.T, xn.T
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
