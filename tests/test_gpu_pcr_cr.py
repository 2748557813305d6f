"""GPU parity of the on-chip PCR-pThomas and CR-PCR kernels against the
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
SIZES = [(1, 3), (2, 5), (3, 4), (31, 7), (32, 9), (33, 3), (64, 1), (100, 33), (128, 16), (256, 70), (257, 5),
         (512, 64), (513, 8), (1000, 12), (1024, 40)]
NAMES = {
    ("pcr", np.float32): ["PCR5_shmem_single", "PCR4_shmem_single", "PCR5_reg_single", "PCR4_reg_single"],
    ("pcr", np.float64): ["PCR5_shmem_double", "PCR4_shmem_double", "PCR5_reg_double", "PCR4_reg_double"],
    ("cr", np.float32): ["CR_single", "CR_reg4_single", "CR_reg8_single", "CR_reg16_single"],
    ("cr", np.float64): ["CR_double", "CR_reg4_double", "CR_reg8_double", "CR_reg16_double"],
}
GOLDEN = {("pcr", np.float32): "PCR4_single", ("pcr", np.float64): "PCR3_double",
          ("cr", np.float32): "CR_single", ("cr", np.float64): "CR_double"}


def _rel(x, xr):
    return np.max(np.abs(x - xr), axis=1) / np.maximum(np.max(np.abs(xr), axis=1), 1e-300)


@pytest.mark.parametrize("algo", ["pcr", "cr"])
@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("n,batch", SIZES)
def test_matches_oracle(cuda, algo, dt, n, batch):
    import tridiagonalsolver_gb300 as T

    a, b, c, d = (v.astype(dt) for v in inputs.dominant(n, batch, seed=5 * n + batch))
    ts = [cuda.from_numpy(v.copy()).cuda() for v in (a, b, c, d)]
    x = T.solve_out(*ts, n, algo=algo).double().cpu().numpy()
    # out-of-place: inputs untouched
    for t, v in zip(ts, (a, b, c, d)):
        np.testing.assert_array_equal(t.cpu().numpy(), v)
    a64, b64, c64, d64 = (v.astype(np.float64) for v in (a, b, c, d))
    _, eta = O.backward_error(a64, b64, c64, d64, x, n)
    assert eta <= ETA[dt]
    xo = O.gtsv(a64, b64, c64, d64, n).reshape(batch, n)
    assert np.max(_rel(x, xo)) <= FWD[dt]
    # in place, the reference contract
    T.solve(*ts, n, algo=algo)
    np.testing.assert_allclose(ts[3].double().cpu().numpy(), x, rtol=0, atol=0)


@pytest.mark.parametrize("algo", ["pcr", "cr"])
@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_packed_layout(cuda, algo, dt):
    import tridiagonalsolver_gb300 as T

    n, batch = 256, 10
    a, b, c, d = (v.astype(dt) for v in inputs.dominant(n, batch, seed=8))
    p = cuda.from_numpy(inputs.to_packed(a, b, c, d)).cuda()
    T.solve(p, None, None, None, n, algo=algo, layout="packed")
    x = p.double().cpu().numpy().reshape(batch, 4, n)[:, 3, :]
    _, eta = O.backward_error(*(v.astype(np.float64) for v in (a, b, c, d)), x, n)
    assert eta <= ETA[dt]


@pytest.mark.parametrize("algo", ["pcr", "cr"])
@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("case", ["n128", "n512", "ref256"])
def test_reference_names_vs_golden(cuda, golden, algo, dt, case):
    import tridiagonalsolver_gb300 as T

    z = golden["f64" if dt == np.float64 else "f32"]
    n = int(z[f"{case}/n"])
    ref = GOLDEN[(algo, dt)]
    valid = z[f"{case}/{ref}/valid"]
    xr = z[f"{case}/{ref}"].astype(np.float64)[valid]
    for name in NAMES[(algo, dt)]:
        a, b, c, d = (cuda.from_numpy(z[f"{case}/{k}"].copy()).cuda() for k in "abcd")
        if algo == "cr":
            init = getattr(T.lib(), "CR_init_" + ("double" if dt == np.float64 else "single"))
            assert init(a.data_ptr(), b.data_ptr(), c.data_ptr(), d.data_ptr(), n, a.numel() // n) == 0
        T.reference_call(name, a, b, c, d, n)
        if algo == "cr":
            T.lib().CR_final()
        x = d.double().cpu().numpy().reshape(-1, n)[valid]
        assert np.max(_rel(x, xr)) <= FWD[dt], name
        np.testing.assert_array_equal(a.cpu().numpy(), z[f"{case}/a"])
        np.testing.assert_array_equal(b.cpu().numpy(), z[f"{case}/b"])


@pytest.mark.parametrize("dt,n", [(np.float32, 512), (np.float64, 256)])
def test_pcr_tma_and_direct_paths(cuda, dt, n):
    """PCR at n = 32 x 16 (FP32) / 32 x 8 (FP64): the persistent TMA-fed
    kernel (contiguous layout; four PCR steps, the stride-16 chains solved by
    lane pairs from both ends) and the direct-load kernel (packed layout;
    five steps, one chain per lane) both meet the tolerances against the
    oracle.  a[0] and c[n-1] are not part of a system: nonzero values there
    leave each path's x exactly unchanged."""
    import tridiagonalsolver_gb300 as T

    batch = 1000
    a, b, c, d = (v.astype(dt) for v in inputs.dominant(n, batch, seed=77))
    a2, c2 = a.copy(), c.copy()
    a2[:, 0], c2[:, n - 1] = 5.0, -7.0  # outside the system
    tma, direct = [], []
    for aa, cc in ((a, c), (a2, c2)):
        ts = [cuda.from_numpy(v.copy()).cuda() for v in (aa, b, cc, d)]
        tma.append(T.solve_out(*ts, n, algo="pcr").cpu().numpy().reshape(batch, n))
        p = cuda.from_numpy(inputs.to_packed(aa, b, cc, d)).cuda()
        T.solve(p, None, None, None, n, algo="pcr", layout="packed")
        direct.append(p.cpu().numpy().reshape(batch, 4, n)[:, 3, :])
    np.testing.assert_array_equal(tma[1], tma[0])
    np.testing.assert_array_equal(direct[1], direct[0])
    a64, b64, c64, d64 = (v.astype(np.float64) for v in (a, b, c, d))
    xo = O.gtsv(a64, b64, c64, d64, n).reshape(batch, n)
    for x in (tma[0], direct[0]):
        x = x.astype(np.float64)
        _, eta = O.backward_error(a64, b64, c64, d64, x, n)
        assert eta <= ETA[dt]
        assert np.max(_rel(x, xo)) <= FWD[dt]
