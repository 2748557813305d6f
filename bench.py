#!/usr/bin/env python3
"""Benchmark of the batched tridiagonal solve on GB300 (one JSON line).

Workload (the reference benchmark configuration with PCR / CR-PCR / pivoted
WM-pGE): one step solves, in sequence on one stream,
  * PCR        FP32, n = 512,  32768 diagonally dominant systems;
  * CR-PCR     FP32, n = 512,  32768 diagonally dominant systems;
  * WM-pGE with partial pivoting, FP64, n = 4096, 4096 non-dominant systems
    (a, b, c, d ~ U[-1, 1]).
Inputs are seeded synthetic arrays resident in HBM, larger than L2 in total
(671 + 268 + 268 MB); every solve is out of place (inputs untouched), so
steps are identical.  The metric is systems per second over the step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Timed region: K replays of a CUDA graph holding one step, between CUDA
events on the launching stream, a barrier and a device synchronisation on
both sides; the maximum over ranks is reported.  Under torchrun each rank
solves its own copy of the workload (weak scaling, no collective on the data
path).  Also reported: per-part times, the roofline of the dominant kernel
(algorithmic bytes / measured launch time against the measured HBM copy
bandwidth), SM clocks sampled during the timed region, an end-to-end number
through the public API with pinned host buffers, and the CPU oracle timed on
a bounded sample of the same workload.

--impl reference times the reference's CPU algorithms (the oracle's port of
Tridiagonal_AVX512's PCR-pThomas, CR and the LAPACK-style pivoted solve that
is the reference's MKL row) with all host threads on a bounded sample per
step; on x86-64 hosts that built the reference itself, PCR and CR run the
reference's own AVX-512 kernels.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "systems/s and % HBM roofline; plain vs adjoint/ragged/refined at stated rel err"
UNIT = "systems/s"
WORKLOAD = "reference config 2: PCR + CR-PCR FP32 n=512 x 32768, pivoted WM-pGE FP64 n=4096 x 4096"

PARTS = [
    # name, dtype, n, batch, distribution, algorithm of this library, reference (oracle) algorithm
    dict(name="pcr_fp32", dtype="float32", n=512, batch=32768, dist="dominant", algo="pcr", ref=("pcr", 4)),
    dict(name="crpcr_fp32", dtype="float32", n=512, batch=32768, dist="dominant", algo="cr", ref=("cr", 7)),
    dict(name="wm_pivot_fp64", dtype="float64", n=4096, batch=4096, dist="nondominant", algo="gtsv", ref=("gtsv", 0)),
]


def _measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def _traffic_table():
    """DRAM bytes per launch from the committed ncu summary (key value lines)."""
    out = {}
    p = ROOT / "profiles" / "ncu_traffic.txt"
    if p.exists():
        for line in p.read_text().splitlines():
            line = line.strip()
            if line and not line.startswith("#"):
                k, v = line.split()[:2]
                out[k] = float(v)
    return out


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 100 ms in the background."""

    FIELDS = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "100",
                 "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line.strip()))

    def mark(self, which):
        if which == "begin":
            self.t0 = time.time()
        else:
            self.t1 = time.time()

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        mhz, maxmhz, reasons = [], None, set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for t, line in self.lines:
            if self.t0 is None or not (self.t0 <= t <= (self.t1 or t)):
                continue
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                mhz.append(float(f[1]))
                maxmhz = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names[1:], f[5:9]):
                if v.lower() in ("active", "1"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(mhz) if mhz else None, "sm_max_mhz": maxmhz,
                "reasons": sorted(reasons), "samples": len(mhz)}


def make_inputs(torch, part, seed, device):
    dt = getattr(torch, part["dtype"])
    n, batch = part["n"], part["batch"]
    g = torch.Generator(device=device)
    g.manual_seed(seed)

    def u(lo, hi):
        return torch.rand((batch, n), dtype=dt, device=device, generator=g) * (hi - lo) + lo

    a, c = u(-1, 1), u(-1, 1)
    a[:, 0] = 0
    c[:, -1] = 0
    if part["dist"] == "dominant":
        b = a.abs() + c.abs() + u(1, 2)
    else:
        b = u(-1, 1)
    d = u(-1, 1)
    return [t.contiguous() for t in (a, b, c, d)]


def run_ours(args):
    import torch
    import torch.distributed as dist

    import tridiagonalsolver_gb300 as T

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    T.lib()  # fail loudly if the CUDA library is missing

    # inputs, outputs and workspaces, resident in HBM
    data = []
    for pi, part in enumerate(PARTS):
        a, b, c, d = make_inputs(torch, part, seed=1000 * rank + pi, device=dev)
        x = torch.empty_like(d)
        work = T.solve_out_workspace(a, part["n"], part["algo"])
        data.append(dict(part=part, a=a, b=b, c=c, d=d, x=x, work=work))

    stream = torch.cuda.Stream(device=dev)
    algo_used = {}

    def solve_part(item, s):
        part = item["part"]
        algo = part["algo"]
        algo_used[part["name"]] = algo
        T.solve_out(item["a"], item["b"], item["c"], item["d"], part["n"], algo=algo, out=item["x"],
                    work=item["work"], stream=s)

    def step(s):
        for item in data:
            solve_part(item, s)

    # warm-up (also allocates the library's device error word, outside capture)
    with torch.cuda.stream(stream):
        for _ in range(max(args.warmup, 3)):
            step(stream)
    stream.synchronize()

    # accuracy of this run's results on a sample of systems (FP64 oracle)
    accuracy = _accuracy(torch, data)

    # graphs: one step, and one per part (per-launch timing for the roofline)
    g_step = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g_step, stream=stream):
        step(stream)
    g_parts = []
    for item in data:
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            solve_part(item, stream)
        g_parts.append(g)
    # CUDAGraph.replay() launches on the current stream: keep it the timed one
    with torch.cuda.stream(stream):
        for _ in range(3):
            g_step.replay()
    stream.synchronize()

    sampler = ClockSampler(local)
    if rank == 0:
        sampler.start()
        time.sleep(0.6)  # let nvidia-smi start sampling
    # ---- timed region
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    sampler.mark("begin")
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        ev0.record(stream)
        for _ in range(args.steps):
            g_step.replay()
        ev1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    sampler.mark("end")
    ms_total = ev0.elapsed_time(ev1)
    if world > 1:
        t = torch.tensor([ms_total], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_total = float(t.item())
    ms_step = ms_total / args.steps

    # per-part launch times (same conditions, after the timed region)
    part_ms = []
    reps = max(10, min(args.steps, 50))
    for g in g_parts:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(reps):
                g.replay()
            e1.record(stream)
        stream.synchronize()
        part_ms.append(e0.elapsed_time(e1) / reps)
    clocks = sampler.stop() if rank == 0 else None

    # end to end through the public API: pinned host -> device, solve, device -> host
    e2e = _e2e(torch, T, data, stream, solve_part, steps=max(3, min(args.steps // 10, 20)))

    systems = sum(p["batch"] for p in PARTS)
    value = world * systems / (ms_step * 1e-3)
    if rank == 0:
        peak, peak_kind = _measured_peaks()
        traffic = _traffic_table()
        parts_out = []
        for item, ms in zip(data, part_ms):
            p = item["part"]
            s = 4 if p["dtype"] == "float32" else 8
            alg_bytes = 5 * p["n"] * p["batch"] * s
            parts_out.append(dict(
                name=p["name"], dtype=p["dtype"], n=p["n"], batch=p["batch"], dist=p["dist"],
                algorithm=algo_used[p["name"]], ms_per_launch=round(ms, 5),
                systems_per_s=p["batch"] / (ms * 1e-3), algorithmic_bytes=alg_bytes,
                hbm_gbs=round(alg_bytes / (ms * 1e-3) / 1e9, 1),
                hbm_frac=round(alg_bytes / (ms * 1e-3) / 1e9 / peak, 4),
                backward_error_max=accuracy.get(p["name"])))
        dom = max(parts_out, key=lambda r: r["ms_per_launch"])
        achieved = dom["hbm_gbs"]
        tr = traffic.get(dom["name"])
        roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": round(achieved / peak, 4), "traffic": tr, "kernel": dom["name"],
                    "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                    else "fallback 6.8 TB/s"}
        if dom["dtype"] == "float64":
            # the FP64 solve is bound by the FP64 pipe on GB300, not by HBM
            roofline["note"] = ("FP64 arithmetic bound: ~11 FP64 ops/row at ~0.5 Tops/s FP64 per GB300 "
                                "(measured, profiles/fp64_rates_microbench.txt)")
        cpu = _cpu_baseline() if (world == 1 and not args.no_cpu) else None
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded U[-1,1] systems, see config)",
            "config": {"workload": WORKLOAD, "parts": [p["name"] for p in PARTS],
                       "systems_per_step_per_gpu": systems, "l2": "inputs larger than L2 (1.2 GB per step)",
                       "timing": "CUDA graph replay of one step, CUDA events on the launching stream",
                       "parallelism": f"replicas x{world} (independent systems per GPU)"},
            "parts": parts_out, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
            "gpu_launches": args.steps * len(PARTS),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def _accuracy(torch, data, sample=16):
    """Max normwise backward error (FP64 oracle) over `sample` systems per part."""
    from oracle import oracle as O

    out = {}
    for item in data:
        p = item["part"]
        n = p["n"]
        idx = torch.linspace(0, p["batch"] - 1, sample, device=item["a"].device).long()
        arrs = [item[k].index_select(0, idx).double().cpu().numpy() for k in ("a", "b", "c", "d", "x")]
        _, worst = O.backward_error(*arrs, n)
        out[p["name"]] = float(worst)
    return out


def _e2e(torch, T, data, stream, solve_part, steps):
    host = []
    h2d = d2h = 0
    for item in data:
        hb = {k: torch.empty_like(item[k], device="cpu").pin_memory() for k in ("a", "b", "c", "d", "x")}
        for k in ("a", "b", "c", "d"):
            hb[k].copy_(item[k])
            h2d += item[k].numel() * item[k].element_size()
        d2h += item["x"].numel() * item["x"].element_size()
        host.append(hb)
    torch.cuda.synchronize()

    def one():
        for item, hb in zip(data, host):
            for k in ("a", "b", "c", "d"):
                item[k].copy_(hb[k], non_blocking=True)
            solve_part(item, stream)
            hb["x"].copy_(item["x"], non_blocking=True)

    with torch.cuda.stream(stream):
        one()
        stream.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            one()
        e1.record(stream)
        stream.synchronize()
    ms = e0.elapsed_time(e1) / steps
    systems = sum(it["part"]["batch"] for it in data)
    return {"value": systems / (ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "ms_per_step": ms, "steps": steps}


def _cpu_run_part(O, part, sample, seed=7):
    """Time the CPU algorithm of one part on `sample` systems; returns seconds."""
    import numpy as np

    from tridiagonalsolver_gb300 import inputs

    n = part["n"]
    gen = inputs.dominant if part["dist"] == "dominant" else inputs.nondominant
    dt = np.float32 if part["dtype"] == "float32" else np.float64
    a, b, c, d = (v.astype(dt) for v in gen(n, sample, seed))
    kind, arg = part["ref"]
    ref_name = None
    if O.ref_available() and kind in ("pcr", "cr"):
        ref_name = {("pcr", 4): "PCR4_single", ("cr", 7): "CR_single"}.get((kind, arg))
    t0 = time.perf_counter()
    if ref_name:
        O.ref_solve(ref_name, a, b, c, d, n)
    elif kind == "pcr":
        O.pcr(a, b, c, d, n, steps=arg)
    elif kind == "cr":
        O.cr(a, b, c, d, n, levels=arg)
    else:
        O.gtsv(a, b, c, d, n)
    return time.perf_counter() - t0, ("reference" if ref_name else "port")


def _cpu_baseline(target_s=8.0):
    """CPU oracle on a bounded sample of the step, all host threads."""
    from oracle import oracle as O

    O.set_threads(0)
    cores = O.threads()
    per = []
    kinds = set()
    # calibrate on a small sample, then size each part to ~target/3 seconds
    for part in PARTS:
        t_small, k = _cpu_run_part(O, part, max(64, cores * 8))
        rate = max(64, cores * 8) / max(t_small, 1e-6)
        sample = int(min(part["batch"], max(cores * 8, rate * target_s / len(PARTS))))
        t, k = _cpu_run_part(O, part, sample)
        kinds.add(k)
        per.append((part, sample, t))
    step_s = sum(t * part["batch"] / sample for part, sample, t in per)
    systems = sum(p["batch"] for p in PARTS)
    return {"value": systems / step_s, "unit": UNIT, "cores": cores,
            "kind": "reference" if kinds == {"reference"} else "port",
            "sample": "; ".join(f"{p['name']}: {s} of {p['batch']} systems in {t:.2f} s" for p, s, t in per)}


def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O

    O.set_threads(0)
    cores = O.threads()
    # size the per-step sample so that W + K steps take a few minutes at most
    samples = []
    for part in PARTS:
        t, _ = _cpu_run_part(O, part, max(64, cores * 8))
        rate = max(64, cores * 8) / max(t, 1e-6)
        budget = 150.0 / max(1, args.steps + args.warmup) / len(PARTS)
        samples.append(int(min(part["batch"], max(cores * 4, rate * budget))))
    for _ in range(args.warmup):
        for part, s in zip(PARTS, samples):
            _cpu_run_part(O, part, s)
    total = 0.0
    kinds = set()
    for _ in range(args.steps):
        for part, s in zip(PARTS, samples):
            t, k = _cpu_run_part(O, part, s)
            kinds.add(k)
            total += t * part["batch"] / s
    step_s = total / args.steps
    systems = sum(p["batch"] for p in PARTS)
    value = systems / step_s
    kind = "reference" if kinds == {"reference"} else "port"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded U[-1,1] systems)",
        "config": {"workload": WORKLOAD, "parts": [p["name"] for p in PARTS]},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": "; ".join(f"{p['name']}: {s} of {p['batch']} systems per step"
                                             for p, s in zip(PARTS, samples))},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
