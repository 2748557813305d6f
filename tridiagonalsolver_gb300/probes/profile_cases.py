"""Small cases of the library's kernels for ncu captures (inputs a little
larger than L2, a few launches, one kernel family each).

    python -m tridiagonalsolver_gb300.probes.profile_cases CASE

CASE: pge64 (partitioned pivoted solve, FP64, n = 4096 x 2048 non-dominant),
pgc32 (cluster version, FP32, n = 65536 x 256 dominant), pge32 (FP32,
n = 4096 x 4096 dominant), gtsv64 (thread-per-system pivoted sweep, FP64,
n = 4096 x 1024).  Each solves its case three times.
"""
import sys

import torch

import tridiagonalsolver_gb300 as T

CASES = {"pge64": (4096, 2048, torch.float64, False), "pgc32": (65536, 256, torch.float32, True),
         "pge32": (4096, 4096, torch.float32, True), "gtsv64": (4096, 1024, torch.float64, False)}


def main(case: str) -> None:
    n, batch, dt, dominant = CASES[case]
    g = torch.Generator(device="cuda")
    g.manual_seed(3)

    def u(lo, hi):
        return torch.rand((batch, n), dtype=dt, device="cuda", generator=g) * (hi - lo) + lo

    a, b, c, d = u(-1, 1), u(-1, 1), u(-1, 1), u(-1, 1)
    if dominant:
        b = a.abs() + c.abs() + u(1, 2)
    x = torch.empty_like(d)
    for _ in range(3):
        if case == "gtsv64":
            T.gtsv(a, b, c, d, n, pivots=T.pivot_record(a, n), out=x)
        else:
            T.pge(a, b, c, d, n, out=x)
    torch.cuda.synchronize()
    print("ok", case)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "pge64")
