"""Generate the golden fixtures in this directory (run here, on x86-64).

    make -C oracle ref REF_ROOT=<reference checkout>   # builds oracle/_ref/libref_avx512.so from
                                   # the reference's Tridiagonal_AVX512 sources
    python tests/golden/make_golden.py

Writes:
  ref_cpu_f64.npz, ref_cpu_f32.npz -- inputs and the outputs of the
      reference's own CPU kernels (Thomas, CR, PCR-pThomas, PCR-half-pThomas,
      WM-pGE, WM-half-pGE) on seeded, per-system-distinct inputs;
  lapack_gtsv.npz -- LAPACK ?gtsv (scipy's bundled LAPACK, the algorithm of
      the reference's MKL row) on non-dominant inputs;
  kat_laplacian.npz -- the (-1, 2, -1) known-answer system (x = 1) solved by
      the reference's Thomas_double and WM3_double.

The reference FP32 PCR kernels (PCR4_single, PCR3_single) read the
uninitialised registers last_c/last_d
(Tridiagonal_AVX512/tridiagonal_s_avx512.cpp:511 and :661); a system whose
output came back non-finite is recorded with valid = False and is skipped by
the parity tests.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from oracle import oracle as O  # noqa: E402
from tridiagonalsolver_gb300 import inputs  # noqa: E402

# (reference routine, oracle call description)
ROUTINES = {
    np.float64: ["Thomas_double", "CR_double", "PCR3_double", "PCR2_double", "WM3_double", "WM2_double"],
    np.float32: ["Thomas_single", "CR_single", "PCR4_single", "PCR3_single", "WM4_single", "WM3_single"],
}
CASES = [  # (tag, n, batch, generator, seed)
    ("n128", 128, 2, "dominant", 101),
    ("n512", 512, 3, "dominant", 102),
    ("ref256", 256, 2, "reference", 103),
]


def _gen(kind, n, batch, seed):
    if kind == "reference":
        a, b, c, d, _x = inputs.reference(n, batch, seed)
        return a, b, c, d
    return getattr(inputs, kind)(n, batch, seed)


def main() -> None:
    if not O.ref_available():
        raise SystemExit("build the reference first: make -C oracle ref REF_ROOT=<reference checkout>")
    for dt, names in ROUTINES.items():
        out = {}
        tag = "f64" if dt == np.float64 else "f32"
        for case, n, batch, kind, seed in CASES:
            a, b, c, d = (v.astype(dt) for v in _gen(kind, n, batch, seed))
            for k, v in zip("abcd", (a, b, c, d)):
                out[f"{case}/{k}"] = v
            out[f"{case}/n"] = np.array(n)
            for name in names:
                x = O.ref_solve(name, a.ravel(), b.ravel(), c.ravel(), d.ravel(), n).reshape(batch, n)
                out[f"{case}/{name}"] = x
                out[f"{case}/{name}/valid"] = np.all(np.isfinite(x), axis=1)
        np.savez_compressed(HERE / f"ref_cpu_{tag}.npz", **out)
        print("wrote", HERE / f"ref_cpu_{tag}.npz")

    from scipy.linalg import lapack

    out = {}
    for dt, fn in ((np.float64, lapack.dgtsv), (np.float32, lapack.sgtsv)):
        tag = "f64" if dt == np.float64 else "f32"
        n, batch = 256, 3
        a, b, c, d = (v.astype(dt) for v in inputs.nondominant(n, batch, 104))
        xs = []
        for j in range(batch):
            _, _, _, x, info = fn(a[j, 1:].copy(), b[j].copy(), c[j, :-1].copy(), d[j].copy())
            assert info == 0
            xs.append(x)
        for k, v in zip("abcd", (a, b, c, d)):
            out[f"{tag}/{k}"] = v
        out[f"{tag}/x"] = np.stack(xs)
        out[f"{tag}/n"] = np.array(n)
    np.savez_compressed(HERE / "lapack_gtsv.npz", **out)
    print("wrote", HERE / "lapack_gtsv.npz")

    n = 64
    a, b, c, d = inputs.laplacian(n, 1)
    out = {"a": a, "b": b, "c": c, "d": d}
    for name in ("Thomas_double", "WM3_double"):
        out[name] = O.ref_solve(name, a.ravel(), b.ravel(), c.ravel(), d.ravel(), n).reshape(1, n)
    np.savez_compressed(HERE / "kat_laplacian.npz", **out)
    print("wrote", HERE / "kat_laplacian.npz")


if __name__ == "__main__":
    main()
