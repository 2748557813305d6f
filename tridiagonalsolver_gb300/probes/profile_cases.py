"""Small cases of the library's kernels for ncu captures (inputs a little
larger than L2, a few launches, one kernel family each).

    python -m tridiagonalsolver_gb300.probes.profile_cases CASE

CASE: pge64 (partitioned pivoted solve, FP64, n = 4096 x 2048 non-dominant),
pgc32 (cluster version, FP32, n = 65536 x 256 dominant), pgl64 (long
systems in chunks through gtsv, FP64, n = 65536 x 128 non-dominant), pge32 (FP32,
n = 4096 x 4096 dominant), gtsv64 (thread-per-system pivoted sweep, FP64,
n = 4096 x 1024), wmc32 (partition method without pivoting, FP32,
n = 4096 x 4096 dominant), pcr32 (PCR-pThomas, FP32, n = 512 x 32768 dominant),
block2_64 (2 x 2 block systems, FP64, interleaved,
n = 256 x 32768: the pivoted solve, then block Thomas on dominant systems),
ragged_step (the ragged workload of `bench.py --workload ragged`: three
forward + adjoint steps, then one between torch.cuda.profiler.start() and
stop(), for `ncu --profile-from-start off`).
Each other case solves its case three times.
"""
import sys

import torch

import tridiagonalsolver_gb300 as T

CASES = {"pge64": (4096, 2048, torch.float64, False), "pgc32": (65536, 256, torch.float32, True),
         "pgl64": (65536, 128, torch.float64, False),
         "wmc32": (4096, 4096, torch.float32, True), "pcr32": (512, 32768, torch.float32, True),
         "pge32": (4096, 4096, torch.float32, True), "gtsv64": (4096, 1024, torch.float64, False)}


def block2_case() -> None:
    n, batch = 256, 32768
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    src = [torch.rand(k * n * batch, dtype=torch.float64, device="cuda", generator=g) * 2 - 1 for k in (4, 4, 4, 2)]
    dom = src[1].clone().view(n, 4, batch)
    dom[:, 0] += 8
    dom[:, 3] += 8
    work = [t.clone() for t in src]
    for algo, b in (("pivoted", src[1]), ("thomas", dom.view(-1))):
        for _ in range(3):
            for w, s in zip(work, (src[0], b, src[2], src[3])):
                w.copy_(s)
            T.block2(*work, n, algo=algo, layout="interleaved")
    torch.cuda.synchronize()
    print("ok block2_64")


def ragged_step_case() -> None:
    from tridiagonalsolver_gb300 import ragged

    sizes = ragged.log_uniform_sizes(100000, 32, 65536, seed=2024)
    a, b, c, d, off, nondom = ragged.synthetic_batch(sizes, seed=2024)
    w = torch.rand_like(d) * 2 - 1
    classes = sorted({ragged.size_class(int(v)) for v in sizes})
    table, _ = ragged.autotune(classes, dtype=torch.float32, reps=1)
    plan = T.RaggedPlan(off, table=table, no_pivoting=~nondom)
    x = torch.empty_like(d)
    grads = [torch.empty_like(d) for _ in range(4)]
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        for _ in range(3):
            plan.solve(a, b, c, d, out=x, stream=s)
            plan.adjoint(a, b, c, x, w, grads=grads, stream=s)
        s.synchronize()
        torch.cuda.profiler.start()
        plan.solve(a, b, c, d, out=x, stream=s)
        plan.adjoint(a, b, c, x, w, grads=grads, stream=s)
        s.synchronize()
        torch.cuda.profiler.stop()
    print("ok ragged_step", int(off[-1]), "rows")


def main(case: str) -> None:
    if case == "block2_64":
        block2_case()
        return
    if case == "ragged_step":
        ragged_step_case()
        return
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
        elif case == "wmc32":
            T.solve_out(a, b, c, d, n, algo="partition", out=x)
        elif case == "pcr32":
            T.solve_out(a, b, c, d, n, algo="pcr", out=x)
        elif case == "pgl64":
            T.gtsv(a, b, c, d, n, out=x)
        else:
            T.pge(a, b, c, d, n, out=x)
    torch.cuda.synchronize()
    print("ok", case)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "pge64")
