"""Parity at the benchmark's full sizes, every system checked.

* Thomas FP64, n = 4096 x 4096 distinct diagonally dominant systems in the
  interleaved layout (the benchmark's configuration 1; reference algorithm
  Thomas_kernel, Tridiagonal_CUDA/tridiagonal_basic.cu:4-30, and the CPU
  Thomas, Tridiagonal_AVX512/tridiagonal_basic.cpp:6-27): normwise backward
  error <= 1e-12 for every system, and every system within
  max|x - x_oracle| / max|x_oracle| <= 1e-12 of the oracle's Thomas.
* PCR-pThomas and CR-PCR FP32, n = 512 x 32768 dominant systems (the PCR /
  CR-PCR half of configuration 2): backward error <= 1e-6 for every system,
  and every system within 1e-5 (relative to max|x|) of the golden-pinned
  oracle's PCR-pThomas (4 PCR steps, PCR4_single) and CR (7 levels,
  CR_single) in FP32.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tridiagonalsolver_gb300 import inputs

pytestmark = pytest.mark.gpu


def _rel(x, xr):
    return np.max(np.abs(x - xr), axis=1) / np.maximum(np.max(np.abs(xr), axis=1), 1e-300)


def test_thomas_fp64_interleaved_4096x4096(cuda):
    import tridiagonalsolver_gb300 as T

    n, batch = 4096, 4096
    a, b, c, d = inputs.dominant(n, batch, seed=4096)
    ts = [cuda.from_numpy(v).cuda() for v in inputs.to_interleaved(a, b, c, d)]
    x = T.solve_out(*ts, n, algo="thomas", layout="interleaved")
    xh = x.cpu().numpy().reshape(n, batch).T.copy()
    eta, worst = O.backward_error(a, b, c, d, xh, n)
    assert worst <= 1e-12, float(np.argmax(eta))
    xo = O.thomas(a, b, c, d, n).reshape(batch, n)
    assert np.max(_rel(xh, xo)) <= 1e-12


@pytest.mark.parametrize("algo,ref", [("pcr", ("pcr", 4)), ("cr", ("cr", 7))])
def test_pcr_crpcr_fp32_512x32768(cuda, algo, ref):
    import tridiagonalsolver_gb300 as T

    n, batch = 512, 32768
    a, b, c, d = (v.astype(np.float32) for v in inputs.dominant(n, batch, seed=512))
    ts = [cuda.from_numpy(v).cuda() for v in (a, b, c, d)]
    x = T.solve_out(*ts, n, algo=algo).double().cpu().numpy().reshape(batch, n)
    a64, b64, c64, d64 = (v.astype(np.float64) for v in (a, b, c, d))
    eta, worst = O.backward_error(a64, b64, c64, d64, x, n)
    assert worst <= 1e-6, float(np.argmax(eta))
    kind, arg = ref
    xo = (O.pcr(a, b, c, d, n, steps=arg) if kind == "pcr" else O.cr(a, b, c, d, n, levels=arg))
    xo = np.asarray(xo, dtype=np.float64).reshape(batch, n)
    assert np.max(_rel(x, xo)) <= 1e-5
