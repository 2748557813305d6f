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

import numpy as np
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


CONFIG = {"workload": WORKLOAD, "parts": [p["name"] for p in PARTS]}  # the same in both arms


def _measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def _fp64_counts():
    """FP64 instructions per row of the FP64 kernels and the measured DFMA rate
    (key = value lines of the committed ncu summary)."""
    out = {}
    for line in (ROOT / "profiles" / "fp64_instructions.txt").read_text().splitlines():
        line = line.split("#")[0].strip()
        if "=" in line:
            k, v = line.split("=")
            out[k.strip()] = float(v)
    return out


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
        t0 = self.t0
        inside = [(t, l) for t, l in self.lines if t0 is not None and t0 <= t <= (self.t1 or t)]
        window = "timed region"
        if not inside and t0 is not None:
            # a timed region shorter than the sampling period: the samples that
            # follow it were taken while the same kernels ran again (per-part timing)
            inside = [(t, l) for t, l in self.lines if t >= t0][:3]
            window = "first samples after the timed region began (region shorter than the 100 ms period)"
        for t, line in inside:
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
                "reasons": sorted(reasons), "samples": len(mhz), "window": window}


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

    # warm-up (also allocates the library's device error word, outside capture); the
    # inputs were made on the current stream, so the solve stream waits for them
    stream.wait_stream(torch.cuda.current_stream())
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
        ms_total = max_over_ranks(torch, dist, ms_total, dev)
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
    value = job_value(world, systems, ms_step)
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
            # the FP64 solve is bound by the FP64 pipe on GB300, not by HBM: report that roofline too
            # (FP64 instructions per row and the measured DFMA rate: profiles/fp64_instructions.txt)
            roofline["compute"] = _fp64_roofline(dom["n"] * dom["batch"], dom["ms_per_launch"], "pge_fp64_ops_per_row")
            roofline["note"] = ("the pivoted FP64 solve is bound by GB300's FP64 issue rate (one FP64 warp "
                                "instruction per 80 cycles per SM sub-partition), not by HBM; see roofline.compute")
        cpu = _cpu_baseline() if (world == 1 and not args.no_cpu) else None
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded U[-1,1] systems, see config)",
            "config": CONFIG,
            "run": {"systems_per_step_per_gpu": systems, "l2": "inputs larger than L2 (1.2 GB per step)",
                    "timing": "CUDA graph replay of one step, CUDA events on the launching stream",
                    "parallelism": f"replicas x{world} (independent systems per GPU)"},
            "parts": parts_out, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
            "gpu_launches": args.steps * len(PARTS),
        }
    else:
        line = None
    if world > 1:
        dist.destroy_process_group()
    return line


def max_over_ranks(torch, dist, value: float, device) -> float:
    """The largest of every rank's value (the slowest rank's time): an
    all-reduce of one number, the same on every rank."""
    t = torch.tensor([float(value)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(world: int, systems_per_rank: int, ms_step: float) -> float:
    """Whole-job systems/s: every rank solves its own systems (replicas), the
    step lasts as long as the slowest rank's."""
    return world * systems_per_rank / (ms_step * 1e-3)


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
    """End to end through the host-buffer entry point (tridiag_solve_host_*):
    every step copies each part's a, b, c, d from page-locked host memory and
    its x back (the library streams them through device buffers in chunks,
    copies overlapping solves); the parts are issued from their own streams,
    so that one part's copies follow the previous part's without a gap, the
    part with the slowest solve per byte first (the last chunk's solve and
    copy-back are the step's tail)."""
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
    pstreams = [torch.cuda.Stream() for _ in data]

    order = sorted(range(len(data)), key=lambda i: -data[i]["a"].element_size())

    def one():
        for i in order:
            item, hb, ps = data[i], host[i], pstreams[i]
            ps.wait_stream(stream)
            part = item["part"]
            T.solve_host(hb["a"], hb["b"], hb["c"], hb["d"], part["n"], algo=part["algo"], out=hb["x"], stream=ps)
        for ps in pstreams:
            stream.wait_stream(ps)

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
    # the host results are the device path's, checked system by system on a
    # sample: the same bits, or -- where the host path's chunks of a few
    # hundred systems take another kernel than the whole batch (the pivoted
    # FP64 part: the one-CTA partitioned solve instead of the
    # thread-per-partition one) -- a normwise backward error within the
    # precision's bar, formed here in FP64
    for item, hb in zip(data, host):
        idx = torch.arange(0, item["x"].shape[0], max(1, item["x"].shape[0] // 16))
        xh = hb["x"][idx]
        if torch.equal(xh, item["x"][idx].cpu()):
            continue
        a_, b_, c_, d_ = (hb[k][idx].double() for k in ("a", "b", "c", "d"))
        x_ = xh.double()
        a_[:, 0] = 0.0
        c_[:, -1] = 0.0
        r = d_ - b_ * x_
        r[:, 1:] -= a_[:, 1:] * x_[:, :-1]
        r[:, :-1] -= c_[:, :-1] * x_[:, 1:]
        scale = (a_.abs() + b_.abs() + c_.abs()).amax(dim=1) * x_.abs().amax(dim=1) + d_.abs().amax(dim=1)
        eta = float((r.abs().amax(dim=1) / scale).max())
        bar = 1e-12 if item["x"].dtype == torch.float64 else 1e-5
        if not eta <= bar:
            raise RuntimeError(f"host-buffer solve of {item['part']['name']} differs from the device solve "
                               f"(backward error {eta:.2e})")
    systems = sum(it["part"]["batch"] for it in data)
    return {"value": systems / (ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "ms_per_step": ms, "steps": steps, "api": "tridiag_solve_host_* (chunked copies overlapping solves)"}


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
        "config": CONFIG,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": "; ".join(f"{p['name']}: {s} of {p['batch']} systems per step"
                                             for p, s in zip(PARTS, samples))},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Further workloads (--workload): the other benchmark configurations, each
# measured on its own and printed as one JSON line with the same keys.


def _graph_time(torch, stream, fn, steps, warmup):
    """Capture fn in a CUDA graph; time `steps` replays (CUDA events on the
    launching stream, synchronised on both sides); return ms per replay.  The
    inputs were made on the current stream: `stream` waits for that work first
    (otherwise buffers the caching allocator recycled from its temporaries
    could be written while those temporaries are still being read)."""
    stream.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(stream):
        for _ in range(max(warmup, 3)):
            fn()
    stream.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        fn()
    with torch.cuda.stream(stream):
        for _ in range(2):
            g.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        e0.record(stream)
        for _ in range(steps):
            g.replay()
        e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps, g


def _e2e_host(torch, T, stream, dev_abcd, dev_x, n, algo, steps, unit_count, layout="contiguous"):
    """End to end through the host-buffer entry point (tridiag_solve_host_*):
    every step copies a, b, c, d from page-locked host memory and x back,
    chunk by chunk, copies overlapping solves."""
    hin = [t.cpu().pin_memory() for t in dev_abcd]
    hx = torch.empty_like(dev_x, device="cpu").pin_memory()
    torch.cuda.synchronize()

    def one():
        T.solve_host(*hin, n, algo=algo, layout=layout, out=hx, stream=stream)

    with torch.cuda.stream(stream):
        one()
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            one()
        e1.record(stream)
        stream.synchronize()
    ms = e0.elapsed_time(e1) / steps
    if not torch.equal(hx, dev_x.cpu()):
        raise RuntimeError("host-buffer solve differs from the device solve")
    return {"value": unit_count / (ms * 1e-3), "unit": UNIT,
            "h2d_bytes_per_step": sum(t.numel() * t.element_size() for t in dev_abcd),
            "d2h_bytes_per_step": dev_x.numel() * dev_x.element_size(), "ms_per_step": ms, "steps": steps,
            "api": "tridiag_solve_host_* (chunked copies overlapping solves)"}


def _e2e_generic(torch, stream, dev_inputs, dev_outputs, fn, steps, unit_count):
    """Pinned host -> device copies of the inputs, fn, device -> host copies
    of the outputs, all inside the timed region."""
    hin = [torch.empty_like(t, device="cpu").pin_memory() for t in dev_inputs]
    hout = [torch.empty_like(t, device="cpu").pin_memory() for t in dev_outputs]
    for h, t in zip(hin, dev_inputs):
        h.copy_(t)
    torch.cuda.synchronize()

    def one():
        for t, h in zip(dev_inputs, hin):
            t.copy_(h, non_blocking=True)
        fn()
        for h, t in zip(hout, dev_outputs):
            h.copy_(t, non_blocking=True)

    with torch.cuda.stream(stream):
        one()
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            one()
        e1.record(stream)
        stream.synchronize()
    ms = e0.elapsed_time(e1) / steps
    return {"value": unit_count / (ms * 1e-3), "unit": UNIT,
            "h2d_bytes_per_step": sum(t.numel() * t.element_size() for t in dev_inputs),
            "d2h_bytes_per_step": sum(t.numel() * t.element_size() for t in dev_outputs), "ms_per_step": ms,
            "steps": steps}


def _fp64_roofline(rows, ms, key):
    """FP64 compute roofline of a kernel that does `rows` rows in `ms`, its
    instructions per row read under `key` from the committed ncu counts."""
    f64 = _fp64_counts()
    ops, peak = f64[key], f64["dfma_gops"]
    gops = rows * ops / (ms * 1e-3) / 1e9
    return {"bound": "fp64", "achieved": round(gops, 1), "peak": peak, "unit": "Gop/s", "frac": round(gops / peak, 4),
            "ops_per_row": ops, "peak_source": "measured DFMA microbenchmark (profiles/fp64_instructions.txt)"}


def _line(args, workload, value, ms_step, dtype, config, parts, roof_bytes, roof_ms, cpu, e2e, clocks, launches,
          note=None, compute=None):
    peak, peak_kind = _measured_peaks()
    achieved = roof_bytes / (roof_ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": None, "kernel": config.get("dominant", "step"),
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                else "fallback 6.8 TB/s"}
    if note:
        roofline["note"] = note
    if compute:
        roofline["compute"] = compute
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": dtype,
            "data": "synthetic (seeded, distributions of the workload)", "config": dict(config, workload=workload),
            "parts": parts, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
            "gpu_launches": launches}
    return line


def _cpu_sample(fn_sample, total_units, target_s=8.0, start=8):
    """Time fn_sample(k) (k units) growing k until ~target_s/4; extrapolate."""
    from oracle import oracle as O

    O.set_threads(0)
    k = start
    t = fn_sample(k)
    while t < target_s / 4 and k < total_units:
        k = min(total_units, k * 4)
        t = fn_sample(k)
    return k / t, k, t, O.threads()


def run_thomas_fp64(args):
    """Plain Thomas, FP64, n = 4096 x 4096 dominant systems, interleaved layout."""
    import torch

    import tridiagonalsolver_gb300 as T
    from oracle import oracle as O
    from tridiagonalsolver_gb300 import inputs

    T.lib()
    n, batch = 4096, 4096
    dev = torch.device("cuda", 0)
    g = torch.Generator(device=dev)
    g.manual_seed(11)
    u = lambda lo, hi: torch.rand((n, batch), dtype=torch.float64, device=dev, generator=g) * (hi - lo) + lo
    a, c, d = u(-1, 1), u(-1, 1), u(-1, 1)
    a[0] = 0
    c[-1] = 0
    b = a.abs() + c.abs() + u(1, 2)
    x = torch.empty_like(d)
    work = T.solve_out_workspace(a, n, "thomas", layout="interleaved")
    stream = torch.cuda.Stream(device=dev)
    step = lambda: T.solve_out(a, b, c, d, n, algo="thomas", layout="interleaved", out=x, work=work, stream=stream)
    sampler = ClockSampler(0)
    sampler.start()
    time.sleep(0.6)
    sampler.mark("begin")
    ms, _ = _graph_time(torch, stream, step, args.steps, args.warmup)
    sampler.mark("end")
    clocks = sampler.stop()
    idx = torch.arange(0, batch, batch // 16, device=dev)
    hs = [t.index_select(1, idx).T.contiguous().cpu().numpy() for t in (a, b, c, d, x)]
    _, eta = O.backward_error(*hs, n)
    e2e = _e2e_host(torch, T, stream, [a, b, c, d], x, n, "thomas", max(3, min(args.steps // 10, 10)), batch,
                    layout="interleaved")

    def cpu(k):
        aa, bb, cc, dd = inputs.dominant(n, k, seed=3)
        t0 = time.perf_counter()
        O.thomas(aa, bb, cc, dd, n)
        return time.perf_counter() - t0

    rate, k, t, cores = (None, 0, 0, 0) if args.no_cpu else _cpu_sample(cpu, batch)
    cpu_b = None if args.no_cpu else {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                                      "sample": f"{k} of {batch} systems in {t:.2f} s (reference Thomas restated)"}
    bytes_ = 5 * n * batch * 8
    return _line(args, "Thomas FP64 n=4096 x 4096, interleaved layout, dominant", batch / (ms * 1e-3), ms, "f64",
          {"n": n, "batch": batch, "layout": "interleaved",
           "dominant": "ipt_forward_kernel<double> + ipt_separator_kernel + ipt_back_kernel (partitioned Thomas)",
           "l2": "inputs larger than L2 (537 MB)"},
          [{"name": "thomas_fp64", "ms_per_launch": ms, "systems_per_s": batch / (ms * 1e-3),
            "algorithmic_bytes": bytes_, "hbm_gbs": round(bytes_ / (ms * 1e-3) / 1e9, 1),
            "backward_error_max": eta}], bytes_, ms, cpu_b, e2e, clocks,
          3 * args.steps, note="FP64 issue bound: partitioned Thomas (7 + 1 FP64 instructions per row in the end "
                               "partitions, 12 + 2 in the others); see roofline.compute",
          compute=_fp64_roofline(n * batch, ms, "ipt_fp64_ops_per_row"))


def run_plain(args):
    """Plain unpivoted solves at n = 4096 x 4096 on the dominant distribution,
    contiguous layout, out of place: the partition method (one CTA per
    system) in FP32 -- the headline of this workload -- and in FP64."""
    import torch

    import tridiagonalsolver_gb300 as T
    from oracle import oracle as O
    from tridiagonalsolver_gb300 import inputs

    T.lib()
    n, batch = 4096, 4096
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    sampler = ClockSampler(0)
    sampler.start()
    time.sleep(0.6)
    sampler.mark("begin")
    parts, keep = [], None
    for name, dt in (("partition_fp32", torch.float32), ("partition_fp64", torch.float64)):
        g = torch.Generator(device=dev)
        g.manual_seed(21)
        u = lambda lo, hi: torch.rand((batch, n), dtype=dt, device=dev, generator=g) * (hi - lo) + lo
        a, c, d = u(-1, 1), u(-1, 1), u(-1, 1)
        b = a.abs() + c.abs() + u(1, 2)
        x = torch.empty_like(d)
        work = T.solve_out_workspace(a, n, "partition")
        step = (lambda a=a, b=b, c=c, d=d, x=x, w=work:
                T.solve_out(a, b, c, d, n, algo="partition", out=x, work=w, stream=stream))
        ms, _ = _graph_time(torch, stream, step, args.steps, args.warmup)
        idx = torch.arange(0, batch, batch // 16, device=dev)
        hs = [t.index_select(0, idx).double().cpu().numpy() for t in (a, b, c, d, x)]
        _, eta = O.backward_error(*hs, n)
        es = 4 if dt == torch.float32 else 8
        alg = 5 * n * batch * es
        parts.append({"name": name, "dtype": str(dt).replace("torch.", ""), "algorithm": "partition", "n": n,
                      "batch": batch, "layout": "contiguous", "ms_per_launch": ms, "systems_per_s": batch / (ms * 1e-3),
                      "algorithmic_bytes": alg, "hbm_gbs": round(alg / (ms * 1e-3) / 1e9, 1),
                      "backward_error_max": eta})
        if keep is None:
            keep = (a, b, c, d, x, step, ms)
        else:
            del a, b, c, d, x, work, step
    sampler.mark("end")
    clocks = sampler.stop()
    a, b, c, d, x, step, ms = keep
    e2e = _e2e_host(torch, T, stream, [a, b, c, d], x, n, "partition", max(3, min(args.steps // 10, 10)), batch)

    def cpu(k):
        aa, bb, cc, dd = (v.astype(np.float32) for v in inputs.dominant(n, k, seed=3))
        t0 = time.perf_counter()
        O.thomas(aa, bb, cc, dd, n)
        return time.perf_counter() - t0

    rate, k, t, cores = (None, 0, 0, 0) if args.no_cpu else _cpu_sample(cpu, batch)
    cpu_b = None if args.no_cpu else {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                                      "sample": f"{k} of {batch} systems in {t:.2f} s (reference Thomas restated, FP32)"}
    return _line(args, "plain unpivoted solve FP32 n=4096 x 4096, contiguous, dominant (partition method)",
          batch / (ms * 1e-3), ms, "f32",
          {"n": n, "batch": batch, "layout": "contiguous", "dominant": "wmc_kernel<float>",
           "l2": "inputs larger than L2 (268 MB FP32)"},
          parts, 5 * n * batch * 4, ms, cpu_b, e2e, clocks, args.steps * 2)


def run_adjoint(args):
    """Forward + adjoint, FP32, n = 1024 x 16384 dominant, loss = sum(w x).
    Main step: the unpivoted partition method (the reference's WM-pGE
    eliminates without pivoting) forward and adjoint; the pivoted
    partitioned solve and its adjoint are timed beside it as a part."""
    import torch

    import tridiagonalsolver_gb300 as T
    from oracle import oracle as O
    from tridiagonalsolver_gb300 import inputs

    T.lib()
    n, batch = 1024, 16384
    dev = torch.device("cuda", 0)
    g = torch.Generator(device=dev)
    g.manual_seed(12)
    u = lambda lo, hi: torch.rand((batch, n), dtype=torch.float32, device=dev, generator=g) * (hi - lo) + lo
    a, c, d, w = u(-1, 1), u(-1, 1), u(-1, 1), u(-1, 1)
    a[:, 0] = 0
    c[:, -1] = 0
    b = a.abs() + c.abs() + u(1, 2)
    x = torch.empty_like(d)
    grads = [torch.empty_like(d) for _ in range(4)]
    L = T.lib()
    stream = torch.cuda.Stream(device=dev)
    P = lambda t: t.data_ptr()

    def fwd():
        T.check(L.tridiag_solve_out_single(7, 0, P(a), P(b), P(c), P(d), P(x), None, 0, n, batch,
                                           int(stream.cuda_stream)), "partition")

    def step():
        fwd()
        T.check(L.tridiag_partition_adjoint_single(0, P(a), P(b), P(c), P(x), P(w), *[P(t) for t in grads], n, batch,
                                                   int(stream.cuda_stream)), "partition adjoint")

    def fwd_piv():
        T.check(L.tridiag_pge_single(0, P(a), P(b), P(c), P(d), P(x), None, n, batch, int(stream.cuda_stream)), "pge")

    def step_piv():
        fwd_piv()
        T.check(L.tridiag_pge_adjoint_single(0, P(a), P(b), P(c), P(x), P(w), *[P(t) for t in grads], None, n, batch,
                                             int(stream.cuda_stream)), "pge adjoint")

    sampler = ClockSampler(0)
    sampler.start()
    time.sleep(0.6)
    sampler.mark("begin")
    ms, _ = _graph_time(torch, stream, step, args.steps, args.warmup)
    sampler.mark("end")
    clocks = sampler.stop()
    ms_f, _ = _graph_time(torch, stream, fwd, max(10, args.steps // 5), 3)
    idx = torch.arange(0, batch, batch // 16, device=dev)

    def accuracy():
        hs = [t.index_select(0, idx).double().cpu().numpy() for t in (a, b, c, d, x, w)]
        _, eta = O.backward_error(*hs[:5], n)
        ref = O.adjoint_f64(hs[0], hs[1], hs[2], hs[4], hs[5], n)
        gerr = max(float(np.max(np.abs(gg.index_select(0, idx).double().cpu().numpy() - r.reshape(16, n))) /
                         np.max(np.abs(r))) for gg, r in zip(grads, ref))
        return eta, gerr

    eta, gerr = accuracy()
    ms_p, _ = _graph_time(torch, stream, step_piv, max(10, args.steps // 5), 3)
    ms_pf, _ = _graph_time(torch, stream, fwd_piv, max(10, args.steps // 5), 3)
    eta_p, gerr_p = accuracy()
    e2e = _e2e_generic(torch, stream, [a, b, c, d, w], [x] + grads, step, max(3, min(args.steps // 10, 10)), batch)

    def cpu(k):
        aa, bb, cc, dd = inputs.dominant(n, k, seed=3)
        ww = np.random.default_rng(1).uniform(-1, 1, (k, n))
        t0 = time.perf_counter()
        xx = O.gtsv(aa, bb, cc, dd, n)
        O.adjoint_f64(aa, bb, cc, xx, ww, n)
        return time.perf_counter() - t0

    rate, k, t, cores = (None, 0, 0, 0) if args.no_cpu else _cpu_sample(cpu, batch)
    cpu_b = None if args.no_cpu else {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                                      "sample": f"{k} of {batch} systems forward+adjoint in {t:.2f} s (FP64 port)"}
    bytes14 = 14 * n * batch * 4
    return _line(args, "forward+adjoint FP32 WM-pGE n=1024 x 16384, dominant, loss=sum(w*x)", batch / (ms * 1e-3), ms,
          "f32", {"n": n, "batch": batch, "dominant": "wmc_kernel<float,0> forward + wmc_kernel<float,1> adjoint",
                  "algorithm": "partition method without pivoting (forward and transposed)",
                  "l2": "inputs larger than L2 (336 MB)"},
          [{"name": "forward", "ms_per_launch": ms_f, "backward_error_max": eta},
           {"name": "adjoint", "ms_per_launch": ms - ms_f, "gradient_rel_err_vs_fp64": gerr},
           {"name": "pivoted_forward_adjoint", "ms_per_step": ms_p, "forward_ms": ms_pf,
            "hbm_gbs": round(bytes14 / (ms_p * 1e-3) / 1e9, 1), "backward_error_max": eta_p,
            "gradient_rel_err_vs_fp64": gerr_p}],
          bytes14, ms, cpu_b, e2e, clocks, 2 * args.steps)


RAGGED_TABLE = ROOT / "tridiagonalsolver_gb300" / "tuned" / "ragged_fp32_gb300.json"


def _ragged_cpu_rate(O, sizes, nondom, target_s=8.0):
    """The oracle's forward + adjoint (LAPACK-style pivoted solve, FP64
    adjoint) of sampled systems of the ragged batch, one system per call on
    all host threads (a thread pool; the oracle releases the GIL).  Returns
    (systems/s, systems timed, seconds, threads)."""
    from concurrent.futures import ThreadPoolExecutor

    cores = os.cpu_count() or 1
    O.set_threads(1)

    def one(s_):
        n_ = int(sizes[s_])
        rng = np.random.default_rng(int(s_))
        aa, cc, dd, ww = (rng.uniform(-1, 1, (1, n_)) for _ in range(4))
        bb = rng.uniform(-1, 1, (1, n_)) if nondom[s_] else np.abs(aa) + np.abs(cc) + 1.5
        xx = O.gtsv(aa, bb, cc, dd, n_)
        O.adjoint_f64(aa, bb, cc, xx, ww, n_)

    k, t = 64, 0.0
    rng = np.random.default_rng(9)
    with ThreadPoolExecutor(max_workers=cores) as ex:
        while True:
            sel = rng.choice(len(sizes), min(k, len(sizes)), replace=False)
            t0 = time.perf_counter()
            list(ex.map(one, sel))
            t = time.perf_counter() - t0
            if t >= target_s / 4 or k >= len(sizes):
                break
            k *= 4
    O.set_threads(0)
    return k / t, k, t, cores


def _ragged_fp64_parts(torch, T, O, ragged, plan32, sizes, off, nondom, stream):
    """The same ragged batch in FP64, forward + adjoint: the plain FP64
    solve (a classifying FP64 plan) and the refined form (FP32 solves through
    the FP32 plan, FP64 residuals, 1 and 2 refinement steps, and 1 step plus
    1 on the systems the plan pivots); worst normwise
    backward error of x and of lambda (A^T lambda = xbar) over a sample,
    dominant and non-dominant systems apart."""
    a, b, c, d, _, _ = ragged.synthetic_batch(sizes, dtype=torch.float64, seed=2024)
    w = torch.rand_like(d) * 2 - 1
    x = torch.empty_like(d)
    grads = [torch.empty_like(d) for _ in range(4)]
    plan64 = T.RaggedPlan(off, dtype=torch.float64, classify=True)
    work = plan32.refine_workspace()
    rng = np.random.default_rng(6)
    sample = list(rng.choice(len(sizes), 24, replace=False)) + list(np.argsort(sizes)[-2:])

    def accuracy():
        worst = {True: [0.0, 0.0], False: [0.0, 0.0]}
        for s_ in sample:
            lo, hi = int(off[s_]), int(off[s_ + 1])
            ha, hb, hc, hd, hx, hw, hl = (t[lo:hi].cpu().numpy()[None] for t in (a, b, c, d, x, w, grads[3]))
            at, ct = np.zeros_like(ha), np.zeros_like(hc)
            at[:, 1:], ct[:, :-1] = hc[:, :-1], ha[:, 1:]
            ek = not nondom[s_]
            worst[ek][0] = max(worst[ek][0], O.backward_error(ha, hb, hc, hd, hx, hi - lo)[1])
            worst[ek][1] = max(worst[ek][1], O.backward_error(at, hb, ct, hw, hl, hi - lo)[1])
        return {"backward_error_max_dominant": worst[True][0], "adjoint_backward_error_max_dominant": worst[True][1],
                "backward_error_max_nondominant": worst[False][0],
                "adjoint_backward_error_max_nondominant": worst[False][1]}

    def plain():
        plan64.solve(a, b, c, d, out=x, stream=stream)
        plan64.adjoint(a, b, c, x, w, grads=grads, stream=stream)

    out = []
    ms, _ = _graph_time(torch, stream, plain, 3, 3)
    out.append(dict({"name": "FP64 forward+adjoint, plain (classifying FP64 plan)", "ms_per_step": ms,
                     "systems_per_s": len(sizes) / (ms * 1e-3),
                     "buckets": [f"class {k} v{v} x{cnt}" for k, v, cnt, _ in plan64.buckets()]}, **accuracy()))
    for iters, piv in ((1, 0), (2, 0), (1, 1)):
        def refined(iters=iters, piv=piv):
            plan32.refine(a, b, c, d, iters=iters, out=x, work=work, stream=stream, pivoted_iters=piv)
            plan32.refine_adjoint(a, b, c, x, w, iters=iters, grads=grads, work=work, stream=stream,
                                  pivoted_iters=piv)

        ms, _ = _graph_time(torch, stream, refined, 3, 3)
        steps = f"{iters} step{'s' if iters > 1 else ''}" + (", then 1 step on the pivoted systems" if piv else "")
        out.append(dict({"name": f"FP64 forward+adjoint, refined ({steps}: FP32 solves, FP64 residuals)",
                         "ms_per_step": ms, "systems_per_s": len(sizes) / (ms * 1e-3)}, **accuracy()))
    del a, b, c, d, w, x, grads, work, plan64
    torch.cuda.empty_cache()
    return out


def run_ragged(args):
    """100000 systems, n log-uniform in [32, 65536], FP32, 20% non-dominant:
    forward + adjoint through the size-class plan, the library finding per
    system (inside the timed step) which systems run without pivoting;
    variants and chunk width from the committed autotuner table (re-tuned
    here when it is absent)."""
    import torch

    import tridiagonalsolver_gb300 as T
    from oracle import oracle as O
    from tridiagonalsolver_gb300 import ragged

    T.lib()
    dev = torch.device("cuda", 0)
    sizes = ragged.log_uniform_sizes(100000, 32, 65536, seed=2024)
    a, b, c, d, off, nondom = ragged.synthetic_batch(sizes, seed=2024)
    w = torch.rand_like(d) * 2 - 1
    t0 = time.time()
    if RAGGED_TABLE.exists():
        table, utab, chunk = ragged.load_table(RAGGED_TABLE, full=True)
        tuned = f"loaded from {RAGGED_TABLE.relative_to(ROOT)}"
    else:
        classes = sorted({ragged.size_class(int(v)) for v in sizes})
        table, _ = ragged.autotune(classes, dtype=torch.float32, reps=2)
        utab, chunk, _ = ragged.autotune_unpivoted(classes, dtype=torch.float32, reps=2)
        tuned = "autotuned in this run"
    tune_s = time.time() - t0
    plan = T.RaggedPlan(off, table=table, classify=True, unpivoted_table=utab, chunk_rows=chunk)
    plan_mask = T.RaggedPlan(off, table=table, no_pivoting=~nondom)
    plan_piv = T.RaggedPlan(off, table=table)
    x = torch.empty_like(d)
    grads = [torch.empty_like(d) for _ in range(4)]
    stream = torch.cuda.Stream(device=dev)

    def step():
        plan.solve(a, b, c, d, out=x, stream=stream)
        plan.adjoint(a, b, c, x, w, grads=grads, stream=stream)

    sampler = ClockSampler(0)
    sampler.start()
    time.sleep(0.6)
    sampler.mark("begin")
    steps = max(3, min(args.steps, 20))
    ms, _ = _graph_time(torch, stream, step, steps, args.warmup)
    sampler.mark("end")
    clocks = sampler.stop()
    ms_f, _ = _graph_time(torch, stream, lambda: plan.solve(a, b, c, d, out=x, stream=stream), steps, 3)

    def step_with(p_):
        def f():
            p_.solve(a, b, c, d, out=x, stream=stream)
            p_.adjoint(a, b, c, x, w, grads=grads, stream=stream)
        return f

    ms_piv, _ = _graph_time(torch, stream, step_with(plan_piv), 3, 3)
    ms_mask, _ = _graph_time(torch, stream, step_with(plan_mask), 3, 3)
    _graph_time(torch, stream, step, 3, 3)  # leave this plan's results in x for the accuracy sample
    marks = plan.kinds()
    # (classes whose unpivoted systems the table gives a pivoted variant run as one pivoted bucket)
    piv_classes = [k_ for k_, v in utab.items() if v != 7]
    cls = np.array([ragged.size_class(int(v)) for v in sizes])
    marks_match = bool(np.array_equal(marks, ~nondom & (sizes > 64) & ~np.isin(cls, piv_classes)))
    rng = np.random.default_rng(5)
    worst = 0.0
    for s_ in list(rng.choice(len(sizes), 16, replace=False)) + list(np.argsort(sizes)[-2:]):
        lo, hi = int(off[s_]), int(off[s_ + 1])
        hs = [t[lo:hi].double().cpu().numpy()[None] for t in (a, b, c, d, x)]
        worst = max(worst, O.backward_error(*hs, hi - lo)[1])
    rows = int(off[-1])
    e2e = _e2e_generic(torch, stream, [a, b, c, d, w], [x] + grads, step, 3, len(sizes))
    fp64 = _ragged_fp64_parts(torch, T, O, ragged, plan, sizes, off, nondom, stream)
    rate, k, t, cores = (None, 0, 0, 0) if args.no_cpu else _ragged_cpu_rate(O, sizes, nondom)
    cpu_b = None if args.no_cpu else {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                                      "sample": f"{k} random systems of the batch, forward + adjoint (FP64 port), "
                                                f"{cores} threads, {t:.2f} s"}
    bk = [{"class": cl, "variant": v, "systems": cnt, "max_n": mx} for cl, v, cnt, mx in plan.buckets()]
    return _line(args, "ragged: 100000 systems, n log-uniform [32, 65536], FP32, 20% non-dominant, forward+adjoint",
                 len(sizes) / (ms * 1e-3), ms, "f32",
                 {"systems": len(sizes), "rows": rows, "buckets": bk,
                  "autotune_table": {str(k_): v for k_, v in table.items()},
                  "unpivoted_table": {str(k_): v for k_, v in utab.items()}, "chunk_rows": chunk,
                  "tuning": tuned, "tuning_seconds": round(tune_s, 1), "l2": "inputs larger than L2 (13.8 GB)",
                  "routing": "found by the library in each solve (strict row dominance checked on the staged rows); "
                             "the adjoint reuses the forward's marks",
                  "timing": "CUDA graph of the whole ragged forward+adjoint (device-side resets, one launch per "
                            "bucket, resident CTAs taking systems through atomic tickets)"},
                 [{"name": "forward (classification included)", "ms_per_launch": ms_f,
                   "backward_error_max": worst},
                  {"name": "adjoint", "ms_per_launch": ms - ms_f},
                  {"name": "forward+adjoint, every system pivoted", "ms_per_step": ms_piv},
                  {"name": "forward+adjoint, the generator's dominance passed as a mask", "ms_per_step": ms_mask},
                  {"name": "library marks", "systems_marked_unpivoted": int(marks.sum()),
                   "equal_to_generator_dominance": marks_match}] + fp64,
                 14 * rows * 4 + 16 * len(sizes), ms, cpu_b, e2e, clocks, 2 * steps * len(bk))


def run_refined(args):
    """n = 65536 x 1024, b = s (1+delta)(|a|+|c|): FP32 partitioned solve +
    FP64-residual refinement (2 steps) vs the plain FP64 solve, delta sweep."""
    import torch

    import tridiagonalsolver_gb300 as T
    from oracle import oracle as O

    T.lib()
    n, batch = 65536, 1024
    dev = torch.device("cuda", 0)
    g = torch.Generator(device=dev)
    g.manual_seed(13)
    u = lambda lo, hi: torch.rand((batch, n), dtype=torch.float64, device=dev, generator=g) * (hi - lo) + lo
    a, c, d = u(-1, 1), u(-1, 1), u(-1, 1)
    a[:, 0] = 0
    c[:, -1] = 0
    sgn = torch.where(u(0, 1) < 0.5, -1.0, 1.0)
    base_b = sgn * (a.abs() + c.abs())
    del sgn
    x = torch.empty_like(d)
    work = T.refine_workspace(a, n)
    stream = torch.cuda.Stream(device=dev)
    parts = []
    ms_main = None
    clocks = None
    idx = torch.arange(0, batch, batch // 8, device=dev)
    for delta in (1.0, 1e-2, 1e-4, 1e-6):
        b = base_b * (1 + delta)
        # the systems are diagonally dominant by construction: unpivoted FP32
        # partition solves inside the refinement; one and two refinement steps
        for iters in (1, 2):
            fn = lambda: T.refine(a, b, c, d, n, iters=iters, work=work, out=x, stream=stream, algo="partition")
            sampler = None
            if delta == 1e-6 and iters == 2:
                sampler = ClockSampler(0)
                sampler.start()
                time.sleep(0.6)
                sampler.mark("begin")
            ms, _ = _graph_time(torch, stream, fn, max(3, min(args.steps, 20)), args.warmup)
            hs = [t.index_select(0, idx).cpu().numpy() for t in (a, b, c, d, x)]
            _, eta = O.backward_error(*hs, n)
            if sampler:
                sampler.mark("end")
                clocks = sampler.stop()
                ms_main = ms
                bmain = b
                eta_main = eta
            parts.append({"name": f"refined delta={delta:g}, {iters} step{'s' if iters > 1 else ''}",
                          "ms_per_launch": ms, "systems_per_s": batch / (ms * 1e-3), "backward_error_max": eta})
    # the same refinement with pivoted FP32 solves (hardest delta)
    ms_r, _ = _graph_time(torch, stream,
                          lambda: T.refine(a, bmain, c, d, n, iters=2, work=work, out=x, stream=stream, algo="gtsv"),
                          3, 3)
    hs = [t.index_select(0, idx).cpu().numpy() for t in (a, bmain, c, d, x)]
    _, eta_r = O.backward_error(*hs, n)
    parts.append({"name": "refined with pivoted FP32 solves delta=1e-06", "ms_per_launch": ms_r,
                  "systems_per_s": batch / (ms_r * 1e-3), "backward_error_max": eta_r})
    # plain FP64 solves on the same GPU (hardest delta): partial pivoting, and
    # the unpivoted partition method
    wg = T.gtsv_workspace(a, n)
    xp = torch.empty_like(d)
    ms_p, _ = _graph_time(torch, stream, lambda: T.gtsv(a, bmain, c, d, n, work=wg, out=xp, stream=stream), 3, 3)
    hs = [t.index_select(0, idx).cpu().numpy() for t in (a, bmain, c, d, xp)]
    _, eta_p = O.backward_error(*hs, n)
    parts.append({"name": "plain FP64 pivoted solve delta=1e-06", "ms_per_launch": ms_p,
                  "systems_per_s": batch / (ms_p * 1e-3), "backward_error_max": eta_p})
    del wg
    wp = T.solve_out_workspace(a, n, "partition")
    ms_q, _ = _graph_time(torch, stream,
                          lambda: T.solve_out(a, bmain, c, d, n, algo="partition", out=xp, work=wp, stream=stream),
                          5, 3)
    hs = [t.index_select(0, idx).cpu().numpy() for t in (a, bmain, c, d, xp)]
    _, eta_q = O.backward_error(*hs, n)
    parts.append({"name": "plain FP64 partition solve (unpivoted) delta=1e-06", "ms_per_launch": ms_q,
                  "systems_per_s": batch / (ms_q * 1e-3), "backward_error_max": eta_q})
    del wp
    e2e = _e2e_generic(torch, stream, [a, bmain, c, d], [x],
                       lambda: T.refine(a, bmain, c, d, n, iters=2, work=work, out=x, stream=stream,
                                        algo="partition"), 3, batch)
    cpu_b = None
    if not args.no_cpu:
        def cpu(k):
            hs_ = [t[:k].cpu().numpy() for t in (a, bmain, c, d)]
            t0 = time.perf_counter()
            O.gtsv(*hs_, n)
            return time.perf_counter() - t0

        rate, k, t, cores = _cpu_sample(cpu, batch, start=16)
        cpu_b = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                 "sample": f"{k} of {batch} systems, plain FP64 partial pivoting, {t:.2f} s"}
    line = _line(args, "refined: FP32 WM-pGE + FP64-residual refinement, n=65536 x 1024, delta sweep",
          batch / (ms_main * 1e-3), ms_main, "f32+f64 residual",
          {"n": n, "batch": batch, "iters": 2, "fp32_solver": "partition method (unpivoted), chunked",
           "l2": "inputs larger than L2 (2.1 GB)", "headline_case": "delta=1e-6"},
          parts, 5 * n * batch * 8, ms_main, cpu_b, e2e, clocks, 7 * max(3, min(args.steps, 20)),
          note="algorithmic bytes counted as 5*n*8 (FP64 in/out), as for the plain FP64 solve; value: 2 steps "
               "at delta=1e-6")
    line["backward_error_max"] = eta_main  # of the line's own case (2 steps, delta=1e-6); each part has its own
    return line


def run_block2(args):
    """Block tridiagonal systems with 2 x 2 blocks, n = 512 block rows x 131072
    systems, interleaved layout: the pivoted solve (FP64 and FP32, U[-1,1]
    blocks) and block Thomas (FP64, block diagonally dominant).  The solve is
    in place, so every step restores the inputs from a pristine copy outside
    the timed region (as the reference's driver does) and the kernel alone is
    timed with CUDA events on its stream."""
    import torch

    import tridiagonalsolver_gb300 as T
    from oracle import oracle as O

    T.lib()
    n, batch = 512, 131072
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    parts, kernel_ms, eta_all = [], {}, {}
    sampler = ClockSampler(0)
    sampler.start()
    time.sleep(0.6)
    sampler.mark("begin")
    keep = None
    for name, dt, algo in (("pivoted_fp64", torch.float64, "pivoted"), ("thomas_fp64", torch.float64, "thomas"),
                           ("pivoted_fp32", torch.float32, "pivoted")):
        g = torch.Generator(device=dev)
        g.manual_seed(17)
        src = [torch.rand(k * n * batch, dtype=dt, device=dev, generator=g) * 2 - 1 for k in (4, 4, 4, 2)]
        if algo == "thomas":
            bv = src[1].view(n, 4, batch)
            rows = (src[0].view(n, 4, batch).abs() + src[2].view(n, 4, batch).abs() + bv.abs())
            sgn = lambda t: torch.where(t >= 0, 1.0, -1.0).to(dt)
            bv[:, 0] = sgn(bv[:, 0]) * (rows[:, 0] + rows[:, 1] + 1)
            bv[:, 3] = sgn(bv[:, 3]) * (rows[:, 2] + rows[:, 3] + 1)
        work = [t.clone() for t in src]
        info = torch.zeros(batch, dtype=torch.int32, device=dev)
        # inputs were built on the current stream (with temporaries the allocator may
        # hand to `work`): the solve stream waits for that work before touching them
        stream.wait_stream(torch.cuda.current_stream())
        times = []
        with torch.cuda.stream(stream):
            for it in range(args.warmup + args.steps):
                for w, s_ in zip(work, src):
                    w.copy_(s_)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                T.block2(*work, n, algo=algo, layout="interleaved", info=info, stream=stream)
                e1.record(stream)
                stream.synchronize()
                if it >= args.warmup:
                    times.append(e0.elapsed_time(e1))
        ms = sum(times) / len(times)
        kernel_ms[name] = ms
        # accuracy on 16 systems (FP64 residual against the inputs)
        idx = torch.arange(0, batch, batch // 16, device=dev)
        pick = lambda t, k: t.view(n * k, batch).index_select(1, idx).T.reshape(16, n, k).double().cpu().numpy()
        x = pick(work[3], 2)
        abc = [pick(t, 4).reshape(16, n, 2, 2) for t in src[:3]]
        _, eta = O.block2_backward_error(*abc, pick(src[3], 2), x, n)
        eta_all[name] = eta
        es = 8 if dt == torch.float64 else 4
        alg = 16 * n * batch * es
        parts.append({"name": name, "dtype": str(dt).replace("torch.", ""), "algorithm": algo, "n": n,
                      "batch": batch, "layout": "interleaved", "ms_per_launch": ms,
                      "systems_per_s": batch / (ms * 1e-3), "block_rows_per_s": n * batch / (ms * 1e-3),
                      "algorithmic_bytes": alg, "hbm_gbs": round(alg / (ms * 1e-3) / 1e9, 1),
                      "backward_error_max": eta, "nonzero_info": int((info != 0).sum())})
        if name == "pivoted_fp64":
            keep = (src, work, info)
        else:
            del src, work
        torch.cuda.empty_cache()
    sampler.mark("end")
    clocks = sampler.stop()
    src, work, info = keep
    for w, s_ in zip(work, src):
        w.copy_(s_)
    torch.cuda.synchronize()
    e2e_step = lambda: T.block2(*work, n, algo="pivoted", layout="interleaved", info=info, stream=stream)
    e2e = _e2e_generic(torch, stream, work, [work[3]], e2e_step, 3, batch)

    def cpu(k):
        rng = np.random.default_rng(3)
        aa, bb, cc = (rng.uniform(-1, 1, (k, n, 2, 2)) for _ in range(3))
        dd = rng.uniform(-1, 1, (k, n, 2))
        t0 = time.perf_counter()
        O.block2(aa, bb, cc, dd, n, "gbsv")
        return time.perf_counter() - t0

    rate, k, t, cores = (None, 0, 0, 0) if args.no_cpu else _cpu_sample(cpu, batch, start=64)
    cpu_b = None if args.no_cpu else {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                                      "sample": f"{k} of {batch} systems in {t:.2f} s (oracle ?gbsv restatement, FP64)"}
    ms = kernel_ms["pivoted_fp64"]
    # FP64 instructions per block row from ncu's counts (profiles/fp64_instructions.txt)
    compute = _fp64_roofline(n * batch, ms, "block2_fp64_ops_per_row")
    return _line(args, "block tridiagonal (2 x 2 blocks) pivoted FP64, n=512 x 131072, interleaved", batch / (ms * 1e-3), ms,
          "f64", {"n": n, "batch": batch, "layout": "interleaved",
                  "dominant": "block2_pivoted_kernel<double, INTERLEAVED>",
                  "l2": "inputs larger than L2 (3.8 GB FP64)", "timing": "kernel alone, inputs restored between steps"},
          parts, 16 * n * batch * 8, ms, cpu_b, e2e, clocks, 3 * args.steps,
          note="FP64 issue bound; see roofline.compute", compute=compute)


# ---------------------------------------------------------------------------
# Small cases of single kernel families for ncu captures (--profile-case NAME):
# inputs a little larger than L2 where the kernel allows, a few launches,
# each case solving three times.

PROFILE_CASES = {
    # name: (n, batch, dtype, dominant, how)
    "pge64": (4096, 2048, "float64", False, "pge"),        # partitioned pivoted solve, FP64
    "ppt64": (8192, 2048, "float64", False, "gtsv"),       # thread-per-partition pivoted solve (gtsv), FP64
    "pge32": (4096, 4096, "float32", True, "pge"),         # the same, FP32
    "pgc32": (65536, 256, "float32", True, "pge"),         # cluster version, FP32
    "pgl64": (65536, 128, "float64", False, "gtsv"),       # long systems in chunks, FP64
    "gtsv64": (4096, 1024, "float64", False, "gtsv_piv"),  # thread-per-system pivoted sweep (pivot record)
    "adj64": (4096, 1024, "float64", False, "adjoint"),    # its adjoint (AdjOp)
    "wmc32": (4096, 4096, "float32", True, "partition"),   # partition method without pivoting, FP32
    "pcr32": (512, 32768, "float32", True, "pcr"),         # PCR-pThomas at the config-2 shape
    "crpcr32": (512, 32768, "float32", True, "cr"),        # CR-PCR at the config-2 shape
    "wm32": (1024, 16384, "float32", True, "wm"),          # on-chip WM-pGE, one warp per system
    "thomas64i": (4096, 2048, "float64", True, "thomas_i"),  # Thomas FP64, interleaved (config 1 kernel)
    "thomas64c": (4096, 2048, "float64", True, "thomas_c"),  # Thomas FP64, contiguous (the Thomas_* entry points)
    "refine64": (65536, 128, "float64", True, "refine"),   # refinement pieces + chunked FP32 solves
    "factor64": (1024, 8192, "float64", False, "factor"),  # factor once / solve many
    "relayout64": (1024, 16384, "float64", True, "relayout"),  # contiguous -> interleaved transposes
    "periodic64": (1024, 8192, "float64", True, "periodic"),   # Sherman-Morrison periodic solve
}


def profile_case(name: str) -> None:
    import torch

    import tridiagonalsolver_gb300 as T

    T.lib()
    if name == "block2_64":
        n, batch = 256, 32768
        g = torch.Generator(device="cuda")
        g.manual_seed(5)
        src = [torch.rand(k * n * batch, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
               for k in (4, 4, 4, 2)]
        dom = src[1].clone().view(n, 4, batch)
        dom[:, 0] += 8
        dom[:, 3] += 8
        work = [t.clone() for t in src]
        for algo, b in (("pivoted", src[1]), ("thomas", dom.view(-1))):
            for _ in range(3):
                for w, s_ in zip(work, (src[0], b, src[2], src[3])):
                    w.copy_(s_)
                T.block2(*work, n, algo=algo, layout="interleaved")
        torch.cuda.synchronize()
        print("ok block2_64")
        return
    if name in ("ragged_long32", "ragged_long32a"):
        # long unpivoted FP32 systems of a ragged batch (the chunked partition
        # method with element-wise staging): 256 dominant systems, n in
        # [32769, 65536] (~200 MB), three solves; ragged_long32a: sizes
        # rounded up to multiples of 4, every system 16-byte aligned
        from tridiagonalsolver_gb300 import ragged

        sizes = ragged.log_uniform_sizes(256, 32769, 65536, seed=11)
        if name == "ragged_long32a":
            sizes = (sizes + 3) // 4 * 4
        a, b, c, d, off, _ = ragged.synthetic_batch(sizes, nondominant_fraction=0.0, seed=11)
        plan = T.RaggedPlan(off, no_pivoting=np.ones(len(sizes), dtype=bool))
        x = torch.empty_like(d)
        for _ in range(3):
            plan.solve(a, b, c, d, out=x)
        torch.cuda.synchronize()
        print("ok", name, plan.buckets())
        return
    if name == "ragged_refine_small":
        # the ragged refinement passes on 3000 FP64 systems, n log-uniform in [32, 65536] (~25 M rows, 1 GB):
        # one refined solve and its adjoint (1 step) through the FP32 plan, three times
        from tridiagonalsolver_gb300 import ragged

        sizes = ragged.log_uniform_sizes(3000, 32, 65536, seed=12)
        a, b, c, d, off, _ = ragged.synthetic_batch(sizes, dtype=torch.float64, seed=12)
        w = torch.rand_like(d) * 2 - 1
        plan = T.RaggedPlan(off, classify=True)
        work = plan.refine_workspace()
        x = torch.empty_like(d)
        grads = [torch.empty_like(d) for _ in range(4)]
        for _ in range(3):
            plan.refine(a, b, c, d, iters=1, out=x, work=work)
            plan.refine_adjoint(a, b, c, x, w, iters=1, grads=grads, work=work)
        torch.cuda.synchronize()
        print("ok", name, int(off[-1]), "rows")
        return
    if name == "ragged_seq64":
        # variant 9 alone: 64 non-dominant FP64 systems of 40000 rows (102 MB), three solves
        from tridiagonalsolver_gb300 import ragged

        sizes = np.full(64, 40000, dtype=np.int64)
        a, b, c, d, off, _ = ragged.synthetic_batch(sizes, dtype=torch.float64, nondominant_fraction=1.0, seed=9)
        plan = T.RaggedPlan(off, dtype=torch.float64, table={16: 9})
        x = torch.empty_like(d)
        for _ in range(3):
            plan.solve(a, b, c, d, out=x)
        torch.cuda.synchronize()
        print("ok", name, [bk for bk in plan.buckets()])
        return
    if name in ("ragged_step", "ragged64_step", "ragged_refine_step"):
        # the ragged workload (FP32; FP64 plain; FP64 refined through the FP32
        # plan, one step): three forward + adjoint steps, then one between
        # torch.cuda.profiler.start() and stop() (ncu --profile-from-start off)
        from tridiagonalsolver_gb300 import ragged

        dt = torch.float64 if name != "ragged_step" else torch.float32
        sizes = ragged.log_uniform_sizes(100000, 32, 65536, seed=2024)
        a, b, c, d, off, _ = ragged.synthetic_batch(sizes, dtype=dt, seed=2024)
        w = torch.rand_like(d) * 2 - 1
        table, utab, chunk = ragged.load_table(RAGGED_TABLE, full=True) if RAGGED_TABLE.exists() else ({}, {}, 0)
        if name == "ragged64_step":
            plan = T.RaggedPlan(off, dtype=dt, classify=True)
        else:
            plan = T.RaggedPlan(off, table=table, classify=True, unpivoted_table=utab, chunk_rows=chunk)
        x = torch.empty_like(d)
        grads = [torch.empty_like(d) for _ in range(4)]
        work = plan.refine_workspace() if name == "ragged_refine_step" else None

        def step():
            if work is not None:
                plan.refine(a, b, c, d, iters=1, out=x, work=work, stream=s_)
                plan.refine_adjoint(a, b, c, x, w, iters=1, grads=grads, work=work, stream=s_)
            else:
                plan.solve(a, b, c, d, out=x, stream=s_)
                plan.adjoint(a, b, c, x, w, grads=grads, stream=s_)

        s_ = torch.cuda.Stream()
        s_.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s_):
            for _ in range(3):
                step()
            s_.synchronize()
            torch.cuda.profiler.start()
            step()
            s_.synchronize()
            torch.cuda.profiler.stop()
        print("ok", name, int(off[-1]), "rows")
        return
    n, batch, dts, dominant, how = PROFILE_CASES[name]
    dt = getattr(torch, dts)
    g = torch.Generator(device="cuda")
    g.manual_seed(3)
    inter = how == "thomas_i"
    shape = (n, batch) if inter else (batch, n)

    def u(lo, hi):
        return torch.rand(shape, dtype=dt, device="cuda", generator=g) * (hi - lo) + lo

    a, b, c, d = u(-1, 1), u(-1, 1), u(-1, 1), u(-1, 1)
    if dominant:
        b = a.abs() + c.abs() + u(1, 2)
    x = torch.empty_like(d)
    piv = T.pivot_record(a, n) if how in ("gtsv_piv", "adjoint") else None
    fac = T.Factorization(a, b, c, n) if how == "factor" else None
    for _ in range(3):
        if how == "gtsv_piv":
            T.gtsv(a, b, c, d, n, pivots=piv, out=x)
        elif how == "adjoint":
            xf = T.gtsv(a, b, c, d, n, pivots=piv)
            T.gtsv_adjoint(a, b, c, xf, piv, d, n)
        elif how == "gtsv":
            T.gtsv(a, b, c, d, n, out=x)
        elif how in ("partition", "pcr", "cr", "wm"):
            T.solve_out(a, b, c, d, n, algo=how, out=x)
        elif how == "thomas_i":
            T.solve_out(a, b, c, d, n, algo="thomas", layout="interleaved", out=x)
        elif how == "thomas_c":
            T.solve_out(a, b, c, d, n, algo="thomas", out=x)
        elif how == "refine":
            T.refine(a, b, c, d, n, iters=2, out=x, algo="partition")
        elif how == "factor":
            fac = T.Factorization(a, b, c, n)
            fac.solve(d)
        elif how == "relayout":
            T.relayout((a, b, c, d), n, "contiguous", "interleaved")
        elif how == "periodic":
            T.periodic(a, b, c, d, n, out=x)
        else:
            T.pge(a, b, c, d, n, out=x)
    torch.cuda.synchronize()
    print("ok", name)


# ---------------------------------------------------------------------------
# GPU comparators on the benchmark's shapes: cuSPARSE gtsv2StridedBatch (the
# reference's vendor row, through its cuSparse_* entry points) and the
# reference's own CUDA kernels, built from its sources for sm_103a into
# oracle/_ref (device code only) and launched through the CUDA driver API
# with the reference's launch configurations (Tridiagonal_CUDA/
# tridiagonal_wm_pcr.cu:1433-1455, tridiagonal_basic.cu:166-190).

REF_CUBINS = [ROOT / "oracle" / "_ref" / "ref_cuda_wm_pcr.cubin", ROOT / "oracle" / "_ref" / "ref_cuda_basic.cubin"]


class RefCudaKernels:
    """The reference's kernels from the cubins in oracle/_ref: the functions
    of each module are listed through the driver (cuModuleEnumerateFunctions,
    cuFuncGetName) and found by their exported names."""

    def __init__(self):
        import ctypes
        import re

        self.ct = ctypes
        self.cu = ctypes.CDLL("libcuda.so.1")
        P, U = ctypes.c_void_p, ctypes.c_uint
        self.cu.cuModuleLoad.argtypes = [ctypes.POINTER(P), ctypes.c_char_p]
        self.cu.cuModuleGetFunctionCount.argtypes = [ctypes.POINTER(U), P]
        self.cu.cuModuleEnumerateFunctions.argtypes = [ctypes.POINTER(P), U, P]
        self.cu.cuFuncGetName.argtypes = [ctypes.POINTER(ctypes.c_char_p), P]
        self.cu.cuLaunchKernel.argtypes = [P, U, U, U, U, U, U, U, P, ctypes.POINTER(P), ctypes.POINTER(P)]
        self.funcs = {}
        for path in REF_CUBINS:
            mod = P()
            if self.cu.cuModuleLoad(ctypes.byref(mod), str(path).encode()) != 0:
                raise RuntimeError(f"cuModuleLoad failed for {path.name}")
            cnt = U()
            if self.cu.cuModuleGetFunctionCount(ctypes.byref(cnt), mod) != 0:
                raise RuntimeError("cuModuleGetFunctionCount failed")
            arr = (P * cnt.value)()
            if self.cu.cuModuleEnumerateFunctions(arr, cnt, mod) != 0:
                raise RuntimeError("cuModuleEnumerateFunctions failed")
            for f in arr:
                nm = ctypes.c_char_p()
                if self.cu.cuFuncGetName(ctypes.byref(nm), f) == 0:
                    m = re.match(r"_Z\d+(\w+?_kernel)I([fd])", nm.value.decode())
                    if m:  # e.g. WM5_reg_kernel<float, 2> -> ("WM5_reg_kernel", "f")
                        self.funcs[(m.group(1), m.group(2))] = P(f)

    def launch(self, name, dt, grid, block, ptrs, ints, stream):
        """One launch: device pointers, then int arguments (the kernels'
        (T*, ..., int n_eqt, int n_batch) signatures)."""
        ct = self.ct
        vals = [ct.c_void_p(v) for v in ptrs] + [ct.c_int(v) for v in ints]
        params = (ct.c_void_p * len(vals))(*[ct.cast(ct.pointer(v), ct.c_void_p) for v in vals])
        f = self.funcs[(name, dt)]
        rc = self.cu.cuLaunchKernel(f, grid, 1, 1, block, 1, 1, 0, ct.c_void_p(stream), params, None)
        if rc != 0:
            raise RuntimeError(f"cuLaunchKernel({name}) returned {rc}")


def _time_inplace(torch, stream, src, work, fn, reps):
    """Mean CUDA-event time of fn() over reps calls, the in-place inputs
    restored from src before each call (outside the timed interval)."""
    ms = []
    with torch.cuda.stream(stream):
        for it in range(reps + 2):
            for w, s_ in zip(work, src):
                w.copy_(s_)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            stream.synchronize()
            if it >= 2:
                ms.append(e0.elapsed_time(e1))
    return sum(ms) / len(ms)


def comparators(args):
    """GPU comparators on the benchmark's shapes, each with its time,
    systems/s (counting the systems it solves), HBM fraction over 5 n s bytes
    per solved system and the backward error of a sample of its results."""
    import torch

    import tridiagonalsolver_gb300 as T
    from oracle import oracle as O

    L = T.lib()
    dev = torch.device("cuda", 0)
    peak, _ = _measured_peaks()
    reps = max(3, min(args.steps, 10))
    default = torch.cuda.default_stream(dev)
    shapes = [("float32", 512, 32768, "dominant", "config 2, PCR / CR-PCR shape"),
              ("float64", 4096, 4096, "dominant", "config 1 shape (contiguous)"),
              ("float64", 4096, 4096, "nondominant", "config 2, pivoted WM-pGE shape")]
    try:
        ref = RefCudaKernels() if all(p.exists() for p in REF_CUBINS) else None
        ref_note = None if ref else "unavailable: the cubins built from the reference's sources are not present"
    except Exception as exc:
        ref, ref_note = None, f"unavailable: {type(exc).__name__}: {exc}"[:200]
    out = {"cusparse_gtsv2StridedBatch": [], "reference_cuda": [] if ref else ref_note}

    def record(kind, label, dts, n, batch, dist, ms, solved, x_rows, src_host, note=None):
        es = 4 if dts == "float32" else 8
        bytes_ = 5 * n * solved * es
        idx = np.linspace(0, solved - 1, 16).astype(np.int64)
        a, b, c, d = (v[idx].astype(np.float64) for v in src_host)
        _, eta = O.backward_error(a, b, c, d, x_rows[idx].astype(np.float64), n)
        rec = {"algorithm": label, "dtype": dts, "n": n, "batch": batch, "systems_solved": solved,
               "distribution": dist, "ms_per_call": round(ms, 4), "systems_per_s": solved / (ms * 1e-3),
               "hbm_gbs": round(bytes_ / (ms * 1e-3) / 1e9, 1),
               "hbm_frac": round(bytes_ / (ms * 1e-3) / 1e9 / peak, 4), "backward_error_max": eta}
        if note:
            rec["note"] = note
        out[kind].append(rec)

    for dts, n, batch, dist, what in shapes:
        dt = getattr(torch, dts)
        g = torch.Generator(device=dev)
        g.manual_seed(31)
        u = lambda lo, hi: torch.rand((batch, n), dtype=dt, device=dev, generator=g) * (hi - lo) + lo
        a, c, d = u(-1, 1), u(-1, 1), u(-1, 1)
        a[:, 0] = 0
        c[:, -1] = 0
        b = a.abs() + c.abs() + u(1, 2) if dist == "dominant" else u(-1, 1)
        src = [a, b, c, d]
        host = [t.double().cpu().numpy() for t in src]
        work = [t.clone() for t in src]
        P_ = [t.data_ptr() for t in work]
        sfx = "single" if dts == "float32" else "double"
        torch.cuda.synchronize()
        # cuSPARSE (the reference's cuSparse_* protocol: init, synchronous solves on the default stream, final)
        if getattr(L, f"cuSparse_init_{sfx}")(*P_, n, batch) == 0:
            ms = _time_inplace(torch, default, src, work, lambda: getattr(L, f"cuSparse_{sfx}")(*P_, n, batch), reps)
            record("cusparse_gtsv2StridedBatch", "gtsv2StridedBatch (CR + PCR, no pivoting)", dts, n, batch, dist,
                   ms, batch, work[3].cpu().numpy(), host, note=what)
            L.cuSparse_final()
        if ref is None:
            continue
        ks = "f" if dts == "float32" else "d"
        stream = torch.cuda.Stream(device=dev)
        cands = []
        if n <= 1024:
            # warp-per-system kernels, 2 systems per 64-thread block, grid div_ceil(batch, 2) = (batch+1)/2 - 1
            grid = (batch + 1) // 2 - 1
            cands += [("PCR5_reg_kernel", "reg PCR-pThomas (PCR5_reg)", grid, 64, grid * 2),
                      ("WM5_reg_kernel", "reg WM-pGE (WM5_reg)", grid, 64, grid * 2)]
        else:
            grid = (batch + 1) // 2 - 1
            cands += [("WM5_reg_kernel", "reg WM-pGE (WM5_reg)", grid, 64, grid * 2)]
        cands += [("Thomas_kernel", "Thomas (thread per system)", (batch - 1) // 64 + 1, 64, batch)]
        for kname, label, grid, block, solved in cands:
            if (kname, ks) not in ref.funcs:
                continue
            ms = _time_inplace(torch, stream, src, work,
                               lambda: ref.launch(kname, ks, grid, block, P_, [n, batch], stream.cuda_stream), reps)
            record("reference_cuda", label, dts, n, batch, dist, ms, solved, work[3].cpu().numpy(), host, note=what)
        if ("CR_kernel", ks) in ref.funcs and n <= 1024:
            buf = torch.empty(4 * n * batch, dtype=dt, device=dev)
            ptrs = P_[:4] + [buf.data_ptr()]
            ms = _time_inplace(torch, stream, src, work,
                               lambda: ref.launch("CR_kernel", ks, batch, 64, ptrs, [n, batch], stream.cuda_stream),
                               reps)
            record("reference_cuda", "CR (global-memory scratch)", dts, n, batch, dist, ms, batch,
                   work[3].cpu().numpy(), host, note=what)
            del buf
        del src, work, host
        torch.cuda.empty_cache()
    return out


# The other benchmark configurations, measured after the headline in the
# default run (one GPU) and reported under "configs" of its line.
OTHER_CONFIGS = [
    ("config1_thomas_fp64_interleaved", "thomas-fp64"),
    ("plain_fp32_fp64_4096x4096", "plain"),
    ("config3_forward_adjoint", "adjoint"),
    ("config4_ragged", "ragged"),
    ("config5_refined", "refined"),
]


def other_configs(args):
    """Run each other configuration's workload (20 timed steps at most, no
    CPU leg) and keep the figures of its line: systems/s, step time, HBM
    fraction of its dominant kernel, worst backward error, its parts, the
    end-to-end figure and its clocks."""
    import torch

    sub = argparse.Namespace(**vars(args))
    sub.steps = max(3, min(args.steps, 20))
    sub.no_cpu = True
    out = {}
    for key, wl in OTHER_CONFIGS:
        torch.cuda.empty_cache()
        t0 = time.time()
        try:
            ln = WORKLOADS[wl](sub)
        except Exception as exc:  # report, keep the headline
            out[key] = {"workload": wl, "error": f"{type(exc).__name__}: {exc}"[:300]}
            continue
        etas = [p.get("backward_error_max") for p in ln.get("parts", []) if p.get("backward_error_max") is not None]
        if ln.get("backward_error_max") is not None:  # a line that names its own case's error
            etas = [ln["backward_error_max"]]
        out[key] = {"workload": ln["config"]["workload"], "systems_per_s": ln["value"],
                    "ms_per_step": ln["ms_per_step"], "dtype": ln["dtype"],
                    "hbm_frac": ln["roofline"]["frac"], "achieved_gbs": ln["roofline"]["achieved"],
                    "backward_error_max": max(etas) if etas else None, "parts": ln["parts"],
                    "roofline": ln["roofline"], "e2e": ln["e2e"], "clocks": ln["clocks"],
                    "gpu_launches": ln["gpu_launches"], "steps": sub.steps, "wall_s": round(time.time() - t0, 1)}
    return out


def run_gtsv_long(args):
    """Pivoted FP64 solves of systems longer than one CTA's shared memory
    holds (U[-1,1] coefficients, non-dominant): tridiag_gtsv_double with the
    workspace tridiag_gtsv_workspace_size() asks for -- the thread-per-
    partition solve (ppt.cu) -- against the same call with the smaller
    workspace of the other paths, which takes the path these sizes took
    before (clusters of CTAs below 12288 rows, the chunked long-system solve
    from there); both graph-replayed and timed with CUDA events; the backward
    error of 16 sampled systems of each, formed in FP64 here."""
    import torch

    import tridiagonalsolver_gb300 as T

    T.lib()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    sampler = ClockSampler(0)
    sampler.start()
    time.sleep(0.6)
    sampler.mark("begin")

    def eta(a, b, c, d, x, batch):
        idx = torch.arange(0, batch, max(1, batch // 16), device=dev)
        a_, b_, c_, d_, x_ = (t.index_select(0, idx).double() for t in (a, b, c, d, x))
        a_[:, 0] = 0.0
        c_[:, -1] = 0.0
        r = d_ - b_ * x_
        r[:, 1:] -= a_[:, 1:] * x_[:, :-1]
        r[:, :-1] -= c_[:, :-1] * x_[:, 1:]
        scale = (a_.abs() + b_.abs() + c_.abs()).amax(dim=1) * x_.abs().amax(dim=1) + d_.abs().amax(dim=1)
        return float((r.abs().amax(dim=1) / scale).max())

    al = lambda v: (v + 255) // 256 * 256
    parts = []
    for n, batch in ((6144, 2048), (8192, 2048), (8192, 4096), (11000, 1536), (16384, 1024), (27648, 1024)):
        g = torch.Generator(device=dev)
        g.manual_seed(5)
        a, b, c, d = (torch.rand((batch, n), dtype=torch.float64, device=dev, generator=g) * 2 - 1 for _ in range(4))
        x, xc = torch.empty_like(d), torch.empty_like(d)
        work = T.gtsv_workspace(a, n)
        # the other paths' workspace: two n x batch arrays, the pivot words, one int per system
        small = torch.empty(2 * al(n * batch * 8) + al((n + 31) // 32 * batch * 4) + al(batch * 4),
                            dtype=torch.uint8, device=dev)
        ms_p, _ = _graph_time(torch, stream, lambda: T.gtsv(a, b, c, d, n, work=work, out=x, stream=stream),
                              args.steps, args.warmup)
        T.ppt_counts(reset=True)
        with torch.cuda.stream(stream):
            T.gtsv(a, b, c, d, n, work=work, out=x, stream=stream)
        stream.synchronize()
        counts = T.ppt_counts(reset=True)
        ms_c, _ = _graph_time(torch, stream, lambda: T.gtsv(a, b, c, d, n, work=small, out=xc, stream=stream),
                              args.steps, args.warmup)
        parts.append({"n": n, "batch": batch, "ms_thread_per_partition": round(ms_p, 4),
                      "ms_previous_path": round(ms_c, 4),
                      "previous_path": "clusters of CTAs" if n < 12288 else "chunked long-system solve",
                      "speedup": round(ms_c / ms_p, 2),
                      "systems_per_s": batch / (ms_p * 1e-3), "ppt_counts": counts,
                      "backward_error_max": max(eta(a, b, c, d, x, batch), eta(a, b, c, d, xc, batch))})
        del a, b, c, d, x, xc, work
        torch.cuda.empty_cache()
    sampler.mark("end")
    return {"workload": "gtsv-long", "metric": "systems_per_s", "unit": UNIT, "higher_is_better": True,
            "dtype": "f64", "data": "synthetic U[-1,1] (non-dominant), seed 5", "parts": parts,
            "clocks": sampler.stop(), "steps": args.steps, "warmup": args.warmup}


WORKLOADS = {"config2": None, "thomas-fp64": run_thomas_fp64, "adjoint": run_adjoint, "ragged": run_ragged,
             "refined": run_refined, "block2": run_block2, "plain": run_plain, "gtsv-long": run_gtsv_long}


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--headline-only", action="store_true",
                    help="default workload: measure configuration 2 only (no 'configs' entry)")
    ap.add_argument("--comparators", action="store_true",
                    help="time only the GPU comparators (cuSPARSE, the reference's CUDA kernels) and print them")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="config2",
                    help="config2 (default): PCR + CR-PCR FP32 and pivoted WM-pGE FP64; the others are the "
                         "remaining benchmark configurations, one JSON line each")
    ap.add_argument("--profile-case", choices=sorted(PROFILE_CASES) + ["block2_64", "ragged_step", "ragged64_step",
                                                                         "ragged_refine_step", "ragged_seq64",
                                                                         "ragged_long32", "ragged_long32a",
                                                                         "ragged_refine_small"], default=None,
                    help="run one small case of one kernel family three times (for ncu captures) and exit")
    args = ap.parse_args()
    if args.profile_case:
        profile_case(args.profile_case)
        return
    if args.comparators:
        print(json.dumps({"comparators": comparators(args)}), flush=True)
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif WORKLOADS[args.workload] is None:
        line = run_ours(args)
        if line is not None:
            if line["n_gpus"] == 1 and not args.headline_only:
                line["configs"] = other_configs(args)
                try:
                    line["comparators"] = comparators(args)
                except Exception as exc:  # report, keep the headline
                    line["comparators"] = {"error": f"{type(exc).__name__}: {exc}"[:300]}
            print(json.dumps(line), flush=True)
    else:
        print(json.dumps(WORKLOADS[args.workload](args)), flush=True)


if __name__ == "__main__":
    main()
