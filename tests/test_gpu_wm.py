"""GPU parity of the on-chip WM-pGE kernel (warp per system) against the
oracle and the reference's golden outputs, through the C ABI.

Tolerances: normwise backward error <= 1e-12 (FP64) / 1e-6 (FP32) on
diagonally dominant systems; max |x - x_oracle| / max |x_oracle| <= 1e-12
(FP64) / 1e-5 (FP32).
"""
import numpy as np
import pytest

from oracle import oracle as O
from tridiagonalsolver_gb300 import inputs

pytestmark = pytest.mark.gpu

ETA = {np.float64: 1e-12, np.float32: 1e-6}
FWD = {np.float64: 1e-12, np.float32: 1e-5}
WM_NAMES = {np.float32: ["WM5_shmem_single", "WM4_shmem_single", "WM5_reg_single", "WM4_reg_single"],
            np.float64: ["WM5_shmem_double", "WM4_shmem_double", "WM5_reg_double", "WM4_reg_double"]}


def _rel(x, xr):
    return np.max(np.abs(x - xr), axis=1) / np.maximum(np.max(np.abs(xr), axis=1), 1e-300)


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("n,batch", [(1, 3), (2, 5), (3, 4), (31, 7), (32, 9), (64, 9), (64, 1), (100, 33),
                                     (128, 16), (128, 3), (256, 5), (256, 70), (257, 5), (512, 64), (512, 1),
                                     (513, 8), (1000, 12), (1024, 40), (1024, 3)])
def test_wm_matches_oracle(cuda, dt, n, batch):
    import tridiagonalsolver_gb300 as T

    a, b, c, d = (v.astype(dt) for v in inputs.dominant(n, batch, seed=3 * n + batch))
    ts = [cuda.from_numpy(v.copy()).cuda() for v in (a, b, c, d)]
    T.solve(*ts, n, algo="wm")
    x = ts[3].double().cpu().numpy()
    # the reference contract: a and b untouched (c may be overwritten when a
    # shape falls back to the Thomas sweep)
    for t, v in zip(ts[:2], (a, b)):
        np.testing.assert_array_equal(t.cpu().numpy(), v)
    a64, b64, c64, d64 = (v.astype(np.float64) for v in (a, b, c, d))
    _, eta = O.backward_error(a64, b64, c64, d64, x, n)
    assert eta <= ETA[dt]
    xo = O.gtsv(a64, b64, c64, d64, n).reshape(batch, n)
    assert np.max(_rel(x, xo)) <= FWD[dt]


@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_wm_packed_layout(cuda, dt):
    import tridiagonalsolver_gb300 as T

    n, batch = 256, 10
    a, b, c, d = (v.astype(dt) for v in inputs.dominant(n, batch, seed=8))
    p = cuda.from_numpy(inputs.to_packed(a, b, c, d)).cuda()
    T.solve(p, None, None, None, n, algo="wm", layout="packed")
    x = p.double().cpu().numpy().reshape(batch, 4, n)[:, 3, :]
    _, eta = O.backward_error(*(v.astype(np.float64) for v in (a, b, c, d)), x, n)
    assert eta <= ETA[dt]


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("case", ["n128", "n512", "ref256"])
def test_wm_reference_names_vs_golden(cuda, golden, dt, case):
    import tridiagonalsolver_gb300 as T

    z = golden["f64" if dt == np.float64 else "f32"]
    ref_name = "WM3_double" if dt == np.float64 else "WM4_single"
    n = int(z[f"{case}/n"])
    xr = z[f"{case}/{ref_name}"].astype(np.float64)
    for name in WM_NAMES[dt]:
        a, b, c, d = (cuda.from_numpy(z[f"{case}/{k}"].copy()).cuda() for k in "abcd")
        T.reference_call(name, a, b, c, d, n)
        x = d.double().cpu().numpy().reshape(-1, n)
        assert np.max(_rel(x, xr)) <= FWD[dt], name


def test_wm_laplacian_kat(cuda, golden):
    import tridiagonalsolver_gb300 as T

    z = golden["kat"]
    n = z["a"].shape[1]
    ts = [cuda.from_numpy(z[k].copy()).cuda() for k in "abcd"]
    T.reference_call("WM5_reg_double", *ts, n)
    assert np.max(np.abs(ts[3].cpu().numpy() - 1.0)) < 1e-12
