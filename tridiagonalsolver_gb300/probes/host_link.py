"""Microbenchmark: host <-> device copy rates of the copy engines (page-locked
host memory, 1 GiB, 1-8 concurrent streams, each direction and both at once;
pageable host memory for comparison).

    python -m tridiagonalsolver_gb300.probes.host_link
"""
import time

import torch


def main() -> None:
    dev = torch.device("cuda")
    nbytes = 1 << 30
    for nstreams in (1, 2, 4, 8):
        h = torch.empty(nbytes // 4, dtype=torch.float32).pin_memory()
        d = torch.empty(nbytes // 4, dtype=torch.float32, device=dev)
        h2 = torch.empty(nbytes // 4, dtype=torch.float32).pin_memory()
        d2 = torch.empty(nbytes // 4, dtype=torch.float32, device=dev)
        ss = [torch.cuda.Stream() for _ in range(nstreams)]
        s2 = [torch.cuda.Stream() for _ in range(nstreams)]
        ch = nbytes // 4 // nstreams

        def timed(fn):
            for _ in range(3):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                fn()
                torch.cuda.synchronize()
                t1 = time.perf_counter()
            return t1 - t0

        def h2d():
            for k, s in enumerate(ss):
                with torch.cuda.stream(s):
                    d[k * ch:(k + 1) * ch].copy_(h[k * ch:(k + 1) * ch], non_blocking=True)

        def d2h():
            for k, s in enumerate(ss):
                with torch.cuda.stream(s):
                    h[k * ch:(k + 1) * ch].copy_(d[k * ch:(k + 1) * ch], non_blocking=True)

        def both():
            h2d()
            for k, s in enumerate(s2):
                with torch.cuda.stream(s):
                    h2[k * ch:(k + 1) * ch].copy_(d2[k * ch:(k + 1) * ch], non_blocking=True)

        print(f"streams {nstreams}: H2D {nbytes / timed(h2d) / 1e9:.0f} GB/s  D2H {nbytes / timed(d2h) / 1e9:.0f} GB/s"
              f"  both directions at once {2 * nbytes / timed(both) / 1e9:.0f} GB/s in total", flush=True)
    hp = torch.empty(nbytes // 4, dtype=torch.float32)
    d = torch.empty(nbytes // 4, dtype=torch.float32, device=dev)
    for _ in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d.copy_(hp)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
    print(f"pageable H2D {nbytes / (t1 - t0) / 1e9:.0f} GB/s")


if __name__ == "__main__":
    main()
