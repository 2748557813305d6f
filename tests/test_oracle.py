"""The oracle against the reference's own outputs (golden fixtures), LAPACK,
the known-answer test, and finite differences.  CPU only."""
import numpy as np
import pytest

from oracle import oracle as O
from tridiagonalsolver_gb300 import inputs

# reference routine -> oracle call
CALLS = {
    "Thomas_double": lambda a, b, c, d, n: O.thomas(a, b, c, d, n),
    "Thomas_single": lambda a, b, c, d, n: O.thomas(a, b, c, d, n),
    "CR_double": lambda a, b, c, d, n: O.cr(a, b, c, d, n, levels=7),
    "CR_single": lambda a, b, c, d, n: O.cr(a, b, c, d, n, levels=7),
    "PCR3_double": lambda a, b, c, d, n: O.pcr(a, b, c, d, n, steps=3),
    "PCR2_double": lambda a, b, c, d, n: O.pcr(a, b, c, d, n, steps=2),
    "PCR4_single": lambda a, b, c, d, n: O.pcr(a, b, c, d, n, steps=4),
    "PCR3_single": lambda a, b, c, d, n: O.pcr(a, b, c, d, n, steps=3),
    "WM3_double": lambda a, b, c, d, n: O.wm(a, b, c, d, n, rounds=3, half=0),
    "WM2_double": lambda a, b, c, d, n: O.wm(a, b, c, d, n, rounds=2, half=1),
    "WM4_single": lambda a, b, c, d, n: O.wm(a, b, c, d, n, rounds=4, half=0),
    "WM3_single": lambda a, b, c, d, n: O.wm(a, b, c, d, n, rounds=3, half=1),
}


@pytest.mark.parametrize("name", sorted(CALLS))
@pytest.mark.parametrize("case", ["n128", "n512", "ref256"])
def test_oracle_bit_exact_vs_reference(golden, name, case):
    z = golden["f64" if name.endswith("double") else "f32"]
    n = int(z[f"{case}/n"])
    a, b, c, d = (z[f"{case}/{k}"] for k in "abcd")
    x_ref = z[f"{case}/{name}"]
    valid = z[f"{case}/{name}/valid"]
    x = CALLS[name](a, b, c, d, n).reshape(x_ref.shape)
    assert x.dtype == x_ref.dtype
    # bit for bit on every system the reference solved (see make_golden.py)
    np.testing.assert_array_equal(x[valid], x_ref[valid])


@pytest.mark.parametrize("tag", ["f64", "f32"])
def test_oracle_gtsv_matches_lapack(golden, tag):
    z = golden["gtsv"]
    n = int(z[f"{tag}/n"])
    a, b, c, d, xr = (z[f"{tag}/{k}"] for k in ("a", "b", "c", "d", "x"))
    x = O.gtsv(a, b, c, d, n).reshape(xr.shape)
    tol = 1e-12 if tag == "f64" else 2e-4
    scale = np.max(np.abs(xr), axis=1, keepdims=True)
    assert np.max(np.abs(x - xr) / scale) < tol
    eta, worst = O.backward_error(a, b, c, d, x, n)
    assert worst < (1e-14 if tag == "f64" else 1e-6)


def test_oracle_kat_laplacian(golden):
    z = golden["kat"]
    n = z["a"].shape[1]
    for name in ("Thomas_double", "WM3_double"):
        assert np.max(np.abs(z[name] - 1.0)) < 1e-10
    for fn in (lambda *v: O.thomas(*v, n), lambda *v: O.gtsv(*v, n), lambda *v: O.wm(*v, n, rounds=3),
               lambda *v: O.pcr(*v, n, steps=3), lambda *v: O.cr(*v, n, levels=5)):
        x = fn(z["a"], z["b"], z["c"], z["d"])
        assert np.max(np.abs(x - 1.0)) < 1e-10


def test_oracle_reference_generator_recovers_x():
    a, b, c, d, x = inputs.reference(300, 4, seed=5)
    for fn in (O.thomas, O.gtsv):
        xs = fn(a, b, c, d, 300).reshape(x.shape)
        assert np.max(np.abs(xs - x)) < 1e-13


def test_oracle_gtsv_pivots_where_thomas_fails():
    # zero leading diagonal: Thomas divides by zero, partial pivoting does not
    n = 8
    a, b, c, d = inputs.nondominant(n, 1, seed=3)
    b[0, 0] = 0.0
    x = O.gtsv(a, b, c, d, n)
    _, worst = O.backward_error(a, b, c, d, x, n)
    assert worst < 1e-15
    xt = O.thomas(a, b, c, d, n)
    assert not np.all(np.isfinite(xt))


def test_oracle_gtsv_reports_singular():
    n = 4
    z = np.zeros((1, n))
    with pytest.raises(RuntimeError):
        O.gtsv(z, z, z, np.ones((1, n)), n)


def test_oracle_adjoint_vs_finite_differences():
    n, batch = 40, 3
    a, b, c, d = inputs.nondominant(n, batch, seed=11)
    w = np.random.default_rng(12).uniform(-1, 1, (batch, n))
    x = O.gtsv(a, b, c, d, n).reshape(batch, n)
    ga, gb, gc, gd = (g.reshape(batch, n) for g in O.adjoint_f64(a, b, c, x, w, n))
    h = 1e-6

    def loss(aa, bb, cc, dd):
        return np.sum(w * O.gtsv(aa, bb, cc, dd, n).reshape(batch, n), axis=1)

    rng = np.random.default_rng(13)
    for arr_i, g in ((0, ga), (1, gb), (2, gc), (3, gd)):
        for _ in range(6):
            i = int(rng.integers(1, n - 1))
            args = [v.copy() for v in (a, b, c, d)]
            args[arr_i][:, i] += h
            lp = loss(*args)
            args[arr_i][:, i] -= 2 * h
            lm = loss(*args)
            fd = (lp - lm) / (2 * h)
            np.testing.assert_allclose(g[:, i], fd, rtol=1e-5, atol=1e-7)
    assert np.all(ga[:, 0] == 0) and np.all(gc[:, -1] == 0)


def test_oracle_backward_error_definition():
    n = 16
    a, b, c, d = inputs.dominant(n, 2, seed=1)
    x = O.gtsv(a, b, c, d, n).reshape(2, n)
    x[1, 3] += 1e-3
    eta, worst = O.backward_error(a, b, c, d, x, n)
    r = d - inputs.matvec(a, b, c, x)
    na = np.max(np.abs(a) + np.abs(b) + np.abs(c), axis=1)
    expect = np.max(np.abs(r), axis=1) / (na * np.max(np.abs(x), axis=1) + np.max(np.abs(d), axis=1))
    # system 0 is at rounding level, where the compensated residual is the
    # more accurate of the two; system 1 carries a real perturbation
    np.testing.assert_allclose(eta, expect, rtol=1e-9, atol=1e-15)
    assert eta[1] > 1e-6
    assert worst == eta.max()
