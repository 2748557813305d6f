"""Seeded synthetic tridiagonal systems (numpy, float64), layout 0.

The reference builds one system with MKL's MT19937 stream and replicates it
across the batch (Tridiagonal_CUDA/test.cpp:19-38, utils.cu:231-271).  MKL is
not available here, and identical systems hide per-system indexing bugs, so
every generator below draws each system independently from numpy's PCG64
with an explicit seed.  Distributions:

* ``dominant``: a, c ~ U[-1,1] with a_0 = c_{n-1} = 0,
  b_i = |a_i| + |c_i| + U[1,2], d ~ U[-1,1] (strictly diagonally dominant).
* ``nondominant``: a, b, c, d ~ U[-1,1] (a_0 = c_{n-1} = 0); needs pivoting.
* ``reference``: the reference generator's distribution (test.cpp:19-38):
  x ~ U[-1,1], a, c ~ U[-1,1], b_i = U[0,1] + max(|a_i|+|c_i|,
  |a_{i+1}|+|c_{i-1}|), d = A x; returns the manufactured x too.
* ``scaled``: a, c, d ~ U[-1,1], b_i = s_i (1 + delta)(|a_i| + |c_i|) with
  random sign s_i; delta sets the conditioning (smaller is worse).
* ``laplacian``: (-1, 2, -1) with d_0 = d_{n-1} = 1, exact x = 1 (the BPLG
  known-answer test, Tridiagonal_CUDA/third_party/BPLib/alg/BPLG/
  BPLGTridiagWM.hxx:28-46).
"""
from __future__ import annotations

import numpy as np


def _rng(seed):
    return np.random.default_rng(seed)


def _close(a, c):
    a[:, 0] = 0.0
    c[:, -1] = 0.0


def dominant(n: int, batch: int, seed: int = 0):
    g = _rng(seed)
    a = g.uniform(-1.0, 1.0, (batch, n))
    c = g.uniform(-1.0, 1.0, (batch, n))
    _close(a, c)
    b = np.abs(a) + np.abs(c) + g.uniform(1.0, 2.0, (batch, n))
    d = g.uniform(-1.0, 1.0, (batch, n))
    return a, b, c, d


def nondominant(n: int, batch: int, seed: int = 0):
    g = _rng(seed)
    a, b, c, d = (g.uniform(-1.0, 1.0, (batch, n)) for _ in range(4))
    _close(a, c)
    return a, b, c, d


def reference(n: int, batch: int, seed: int = 0):
    """(a, b, c, d, x) with d = A x computed in float64."""
    g = _rng(seed)
    a = g.uniform(-1.0, 1.0, (batch, n))
    c = g.uniform(-1.0, 1.0, (batch, n))
    x = g.uniform(-1.0, 1.0, (batch, n))
    b = g.uniform(0.0, 1.0, (batch, n))
    _close(a, c)
    s = np.abs(a) + np.abs(c)
    nxt = np.zeros_like(s)
    nxt[:, :-1] = np.abs(a[:, 1:])
    prv = np.zeros_like(s)
    prv[:, 1:] = np.abs(c[:, :-1])
    b += np.maximum(s, nxt + prv)
    d = b * x
    d[:, 1:] += a[:, 1:] * x[:, :-1]
    d[:, :-1] += c[:, :-1] * x[:, 1:]
    return a, b, c, d, x


def scaled(n: int, batch: int, delta: float, seed: int = 0):
    g = _rng(seed)
    a = g.uniform(-1.0, 1.0, (batch, n))
    c = g.uniform(-1.0, 1.0, (batch, n))
    d = g.uniform(-1.0, 1.0, (batch, n))
    _close(a, c)
    s = np.where(g.random((batch, n)) < 0.5, -1.0, 1.0)
    b = s * (1.0 + delta) * (np.abs(a) + np.abs(c))
    return a, b, c, d


def laplacian(n: int, batch: int = 1):
    a = np.full((batch, n), -1.0)
    c = np.full((batch, n), -1.0)
    b = np.full((batch, n), 2.0)
    d = np.zeros((batch, n))
    _close(a, c)
    d[:, 0] = 1.0
    d[:, -1] = 1.0
    if n == 1:
        d[:, 0] = 2.0
    return a, b, c, d


def to_interleaved(*arrs):
    """(batch, n) -> (n, batch) contiguous copies."""
    return tuple(np.ascontiguousarray(v.T) for v in arrs)


def from_interleaved(*arrs):
    return tuple(np.ascontiguousarray(v.T) for v in arrs)


def to_packed(a, b, c, d):
    """Layout 1: [batch][a|b|c|d][n]."""
    return np.ascontiguousarray(np.stack([a, b, c, d], axis=1))


def matvec(a, b, c, x):
    """A x per system (float64), layout 0 arrays of shape (batch, n)."""
    y = b * x
    y[:, 1:] += a[:, 1:] * x[:, :-1]
    y[:, :-1] += c[:, :-1] * x[:, 1:]
    return y
