#!/usr/bin/env python
"""Benchmark of the banded Smith-Waterman seed extension on GB300.

Metric: BSW GCUPS (reference cells per second; a cell is one iteration of the
reference's scalar inner loop, bandedSWA.cpp:175-200) and pairs/s.  A step is
one pass of the hot path over one batch: at N=1 the 16-bit plain-launch
workload, 1,000,000 seeded synthetic pairs (query U[100,300] bp, 4% subs +
0.5% 1-5 bp indels, len1 = len2 + U[0,40], h0 ~ U[30,250], w = 100,
zdrop = 100), scored with getScores16 semantics.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`value` is measured with the inputs resident in HBM (device-resident call,
CUDA events on the library's stream); `e2e` goes through the reference-facing
C ABI call (tal_bsw_scores) with pinned host buffers, host<->device copies
inside the timed region.  Under torchrun each rank scores its own shard of
pairs (independent pairs, no collective): weak scaling.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "trans-omics-acceleration-library_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "BSW GCUPS & pairs/s, batched vs plain launch on 1 GB300 (bit-exact); p99 latency"
UNIT = "GCUPS"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="c2_16bit")
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="CPU work for the cpu_baseline sample (rank 0, N=1)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=None)
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg (profiling)")
    ap.add_argument("--pairs", type=int, default=None,
                    help="score only the first N pairs of the workload (profiling a small case)")
    ap.add_argument("--no-grouped", action="store_true",
                    help="skip the grouped-form (TAL_BSW_GROUPED) leg")
    ap.add_argument("--no-mixed", action="store_true",
                    help="skip the mixed-length plain-vs-batched comparison")
    ap.add_argument("--mixed-pairs", type=int, default=None,
                    help="pairs of the mixed-length workload (default: all 10,000,000)")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-loop section")
    ap.add_argument("--no-full-sw", action="store_true", help="skip the unbanded Smith-Waterman section")
    ap.add_argument("--no-chain", action="store_true", help="skip the anchor chaining section")
    ap.add_argument("--no-extend", action="store_true", help="skip the seed-extension section")
    ap.add_argument("--extend-reads", type=int, default=40_000,
                    help="reads (100-250 bp, 1-3 seeds each) in the seed-extension section")
    ap.add_argument("--chain-reads", type=int, default=10_000,
                    help="reads (1-10 kb, minimap2-like anchors) in the chaining section")
    ap.add_argument("--sw-pairs", type=int, default=100_000,
                    help="pairs of the unbanded Smith-Waterman workload")
    ap.add_argument("--serve-loads", type=float, nargs="+", default=[0.1, 0.3, 0.5, 0.7, 0.9])
    ap.add_argument("--serve-requests", type=int, default=300, help="requests per load point")
    ap.add_argument("--serve-plain-loads", type=float, nargs="+", default=[0.1, 0.7])
    ap.add_argument("--serve-plain-requests", type=int, default=120)
    ap.add_argument("--serve-latency-pairs", type=int, default=0,
                    help="ticks below this many pairs use the latency launches (0: library default)")
    ap.add_argument("--serve-slots", type=int, default=0, help="ticks in flight (0: library default)")
    ap.add_argument("--serve-peak", type=float, default=0.0,
                    help="pairs/s the load fractions refer to (0: the measured batched peak)")
    ap.add_argument("--serve-pool-pairs", type=int, default=3_000_000,
                    help="pairs the serving requests are drawn from")
    return ap.parse_args()


# ----------------------------------------------------------------------------- helpers
def log(msg):
    """Progress of the run on stderr (the JSON line alone goes to stdout)."""
    sys.stderr.write(f"[bench {time.strftime('%H:%M:%S')}] {msg}\n")
    sys.stderr.flush()


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    def __init__(self, backend):
        self.ws, self.rank, self.local = dist_info()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as td
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            td.init_process_group(backend=backend)
            self.td = td

    def barrier(self):
        if self.ws > 1:
            self.td.barrier()

    def max(self, v: float) -> float:
        if self.ws == 1:
            return v
        import torch
        dev = f"cuda:{self.local}" if torch.cuda.is_available() else "cpu"
        t = torch.tensor([v], dtype=torch.float64, device=dev)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v: float) -> float:
        if self.ws == 1:
            return v
        import torch
        dev = f"cuda:{self.local}" if torch.cuda.is_available() else "cpu"
        t = torch.tensor([v], dtype=torch.float64, device=dev)
        self.td.all_reduce(t, op=self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200", "-f", self.path],
                stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows),
                "power_w_max": max((float(r[3]) for r in rows
                                    if r[3].replace(".", "").isdigit()), default=None)}


def segment_configs(bsw):
    """[lanes per pair, columns per lane, max query, ring] of every segment."""
    import tal_bsw
    out = []
    while True:
        try:
            out.append(list(bsw.segment_config(len(out))))
        except tal_bsw.TalBswError:
            return out


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def workload_cells(name):
    p = os.path.join(PKG, "tal_bsw", "workload_cells.json")
    d = json.load(open(p)) if os.path.exists(p) else {}
    return d.get(name)


def profile_traffic(name):
    """dram bytes per launch of the main kernel from the committed ncu
    summary, if one covers this workload."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    d = json.load(open(p))
    e = d.get(name)
    return None if e is None else e.get("dram_bytes_per_launch")


# ---------------------------------------------------------------------- CPU baseline
def cpu_score(batch, wl, nthreads):
    """Times the CPU implementation on `batch`; returns (seconds, ref-cells,
    kind, description).  The reference itself where it was compiled on this
    host (x86 with AVX-512: getScores16 from oracle/_ref, one instance per
    thread), else the oracle's port of scalarBandedSWAWrapper (the
    reference's portable path, equal to getScores16 at e_del = e_ins = 1)."""
    import oracle
    P = wl.params()
    bits = 8 if wl.bits == 8 else 16
    if oracle.ref_available("avx512"):
        parts = np.array_split(np.arange(batch.n), nthreads)
        t = time.perf_counter()
        with cf.ThreadPoolExecutor(nthreads) as ex:
            list(ex.map(lambda ix: oracle.reference(batch.pairs[ix], batch.ref, batch.qer,
                                                    wl.w, P, mode=bits, pristine=False), parts))
        dt = time.perf_counter() - t
        _, cells = oracle.scalar(batch.pairs, batch.ref, batch.qer, wl.w, P, nthreads=nthreads)
        return dt, cells, "reference", f"getScores{bits} (AVX-512BW build of the reference)"
    t = time.perf_counter()
    _, cells = oracle.scalar(batch.pairs, batch.ref, batch.qer, wl.w, P, nthreads=nthreads)
    dt = time.perf_counter() - t
    return dt, cells, "port", "oracle port of scalarBandedSWAWrapper (bandedSWA.cpp:116-260)"


def cpu_sample(wl, seconds, nthreads, first=0):
    """A batch of the workload sized for about `seconds` of CPU work."""
    from tal_bsw import synth
    n = 2000
    probe = synth.generate(wl, n, first=first)
    dt, cells, _, _ = cpu_score(probe, wl, nthreads)
    rate = n / max(dt, 1e-3)
    n2 = int(min(wl.n_pairs, max(n, rate * seconds)))
    return synth.generate(wl, n2, first=first)


def cpu_isa():
    import platform
    m = platform.machine()
    model = ""
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                model = line.split(":", 1)[1].strip()
                break
    except OSError:
        pass
    return f"{m} {model}".strip()


# -------------------------------------------------------------------------- our arm
def run_ours(args):
    import torch
    import tal_bsw
    from tal_bsw import synth
    from tal_bsw.api import probe_int_peak

    dist = Dist("nccl")
    ws, rank, local = dist.ws, dist.rank, dist.local
    torch.cuda.set_device(local)
    wl = synth.WORKLOADS[args.workload]
    n = wl.n_pairs if not args.pairs else min(args.pairs, wl.n_pairs)
    first = rank * n                       # each rank its own shard of pairs
    b = synth.generate(wl, n, first=first)
    P = wl.params()
    bits = 8 if wl.bits == 8 else 16
    cinfo = workload_cells(wl.name)

    bsw = tal_bsw.BandedPairWiseSW(P["o_del"], P["e_del"], P["o_ins"], P["e_ins"], P["zdrop"],
                                   P["end_bonus"], None, P["a"], P["b"], 1, device=local)
    stream = torch.cuda.ExternalStream(bsw.stream)
    pairs_u8 = b.pairs.view(np.uint8).reshape(-1)
    dp = torch.from_numpy(pairs_u8.copy()).cuda()
    dr = torch.from_numpy(b.ref).cuda()
    dq = torch.from_numpy(b.qer).cuda()
    torch.cuda.synchronize()

    def step_device():
        bsw.scores_device(dp.data_ptr(), dr.data_ptr(), dr.numel(), dq.data_ptr(), dq.numel(),
                          n, wl.w, bits)

    for _ in range(max(args.warmup, 3)):
        step_device()
    kernel_cells = bsw.last_cells
    # ref-cells of this shard: counted once per workload (rank 0's shard is
    # the workload itself); other shards scale the kernel's own count
    counted = bool(cinfo) and rank == 0 and cinfo["n_pairs"] == n
    ratio = dist.max(int(cinfo["ref_cells"]) / max(kernel_cells, 1) if counted else 0.0)
    ref_cells = int(cinfo["ref_cells"]) if counted else int(kernel_cells * (ratio or 1.0))

    # ---- device-resident timed region
    clocks = ClockSampler(local)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    dist.barrier()
    torch.cuda.synchronize()
    launches0 = bsw.launch_count
    clocks.start()
    time.sleep(0.3)
    e0.record(stream)
    t0 = time.perf_counter()
    kernel_ms = 0.0
    for _ in range(args.steps):
        step_device()
        kernel_ms += bsw.last_kernel_ms     # the scoring kernel alone (events around it)
    e1.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    kernel_s = kernel_ms / 1e3 / args.steps
    launches = bsw.launch_count - launches0
    dist.barrier()
    t_step = e0.elapsed_time(e1) / 1e3 / args.steps
    t_step_max = dist.max(t_step)
    total_cells = dist.sum(float(ref_cells))
    total_pairs = n * ws
    value = total_cells / t_step_max / 1e9

    # ---- end to end through the C ABI, host buffers pinned
    log(f"device-resident: {value:.1f} GCUPS; end-to-end leg")
    if args.no_e2e:
        print(json.dumps({"value": value, "unit": UNIT, "ms_per_step": t_step_max * 1e3,
                          "pairs": n, "gpu_launches": launches}), flush=True)
        bsw.close()
        dist.close()
        return
    hp = torch.empty(pairs_u8.shape[0], dtype=torch.uint8, pin_memory=True)
    hr = torch.empty(b.ref.shape[0], dtype=torch.uint8, pin_memory=True)
    hq = torch.empty(b.qer.shape[0], dtype=torch.uint8, pin_memory=True)
    hp.numpy()[:] = pairs_u8
    hr.numpy()[:] = b.ref
    hq.numpy()[:] = b.qer
    hpairs = hp.numpy().view(tal_bsw.SEQPAIR_DTYPE)
    e2e_steps = args.e2e_steps or max(3, args.steps // 2)
    for _ in range(2):
        bsw.getScores16(hpairs, hr.numpy(), hq.numpy(), n, 1, wl.w) if bits == 16 else \
            bsw.getScores8(hpairs, hr.numpy(), hq.numpy(), n, 1, wl.w)
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        if bits == 16:
            bsw.getScores16(hpairs, hr.numpy(), hq.numpy(), n, 1, wl.w)
        else:
            bsw.getScores8(hpairs, hr.numpy(), hq.numpy(), n, 1, wl.w)
    t_e2e = (time.perf_counter() - t0) / e2e_steps
    t_e2e_max = dist.max(t_e2e)
    e2e_value = total_cells / t_e2e_max / 1e9
    lens = int(b.pairs["len1"].sum() + b.pairs["len2"].sum())
    h2d = pairs_u8.nbytes + int(b.pairs["len1"].sum()) + int(b.pairs["len2"].sum())
    d2h = pairs_u8.nbytes
    # parity guard on the timed outputs: device-resident and host paths agree
    dev_out = dp.cpu().numpy().view(tal_bsw.SEQPAIR_DTYPE)
    agree = bool((tal_bsw.outputs(dev_out) == tal_bsw.outputs(hpairs)).all())

    # ---- batched form on the same pairs (device-resident)
    log("batched form")

    def step_batched():
        bsw.scores_batched_device(dp.data_ptr(), dr.data_ptr(), dr.numel(), dq.data_ptr(), dq.numel(),
                                  n, wl.w, bits)
    for _ in range(max(args.warmup, 3)):
        step_batched()
    dist.barrier()
    torch.cuda.synchronize()
    b0 = time.perf_counter()
    for _ in range(args.steps):
        step_batched()
    torch.cuda.synchronize()
    t_batched = dist.max((time.perf_counter() - b0) / args.steps)
    batched = {"value": round(total_cells / t_batched / 1e9, 3), "unit": UNIT,
               "pairs_per_s": round(total_pairs / t_batched, 1),
               "ms_per_step": round(t_batched * 1e3, 3),
               "segments": segment_configs(bsw),
               "note": "device-resident batched call (sort into segments = length bin x band "
                       "class, one persistent launch per segment on forked streams, one CUDA "
                       "graph); segments: [lanes per pair, columns per lane, max query, row ring]; "
                       "wall time per synchronous call"}

    # ---- grouped form (the reference's SIMD groups, exact on any input) on
    # the same pairs: its speed, and how many pairs' outputs differ from the
    # per-pair kernels' (pairs whose outputs depend on their group)
    grouped = None
    if not args.no_grouped:
        log("grouped form")
        gbits = bits | tal_bsw.api.GROUPED

        def step_grouped():
            bsw.scores_device(dp.data_ptr(), dr.data_ptr(), dr.numel(), dq.data_ptr(), dq.numel(),
                              n, wl.w, gbits)
        step_grouped()
        gout = dp.cpu().numpy().view(tal_bsw.SEQPAIR_DTYPE)
        ndiff = int((tal_bsw.outputs(gout) != tal_bsw.outputs(dev_out)).any(1).sum())
        gsteps = 2
        dist.barrier()
        torch.cuda.synchronize()
        g0 = time.perf_counter()
        gk = 0.0
        for _ in range(gsteps):
            step_grouped()
            gk += bsw.last_kernel_ms
        torch.cuda.synchronize()
        t_grouped = dist.max((time.perf_counter() - g0) / gsteps)
        grouped = {"value": round(total_cells / t_grouped / 1e9, 3), "unit": UNIT,
                   "ms_per_step": round(t_grouped * 1e3, 3),
                   "kernel_ms_per_launch": round(gk / gsteps, 3),
                   "pairs_differing_from_per_pair": dist.sum(ndiff),
                   "note": "device-resident call with TAL_BSW_GROUPED (one warp per SIMD group of "
                           "the reference, wrapping int16/int8 values); wall time per synchronous "
                           "call"}

    # ---- rooflines
    hbm_peak, peak_src = measured_peaks()
    alg_bytes = lens + 56 * n + 24 * n          # bases read, SeqPair read, outputs written
    achieved = alg_bytes / (kernel_s if kernel_s > 0 else t_step) / 1e9
    dpx, i32 = probe_int_peak(local)
    int_cells_peak = dpx / 4.0                   # 8 int16 lane-ops per cell, 2 lanes per DPX op
    # reference cells per second of the scoring kernel alone (this rank)
    kernel_rate = ref_cells / kernel_s if kernel_s > 0 else value * 1e9 / ws

    result = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": max(args.warmup, 3),
        "ms_per_step": round(t_step_max * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int16", "data": "synthetic (seeded generator, no dataset)",
        "config": {"workload": f"{wl.name}: {n} pairs, query U[{wl.len_lo},{wl.len_hi}], "
                               f"w={wl.w}, zdrop={wl.zdrop}, getScores{bits} plain launch",
                   "pairs_per_step": total_pairs, "ref_cells_per_step": int(total_cells),
                   "kernel_cells_per_step": int(kernel_cells) * ws,
                   "l2": "inputs larger than L2 (no flush needed)",
                   "parallelism": f"replica shards x{ws}, no collective"},
        "pairs_per_s": round(total_pairs / t_step_max, 1),
        "wall_s_timed": round(wall, 3),
        "e2e": {"value": round(e2e_value, 3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "pairs_per_s": round(total_pairs / t_e2e_max, 1),
                "ms_per_step": round(t_e2e_max * 1e3, 3), "outputs_match_device_path": agree},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": hbm_peak,
                     "unit": "GB/s", "frac": round(achieved / hbm_peak, 5),
                     "kernel_ms_per_launch": round(kernel_s * 1e3, 3),
                     "traffic": profile_traffic(wl.name), "peak_source": peak_src,
                     "note": "integer-pipe bound kernel; see roofline_int"},
        "roofline_int": {"bound": "int (DPX 16x2)", "achieved": round(kernel_rate, 1),
                         "peak": round(int_cells_peak, 1), "unit": "cells/s",
                         "frac": round(kernel_rate / int_cells_peak, 5),
                         "peak_dpx_instr_per_s": dpx, "peak_i32_instr_per_s": i32,
                         "model": "4 DPX int16x2 instructions per cell (probe measured live)"},
        "clocks": clk,
        "batched": batched,
    }
    if grouped:
        result["grouped"] = grouped
    if not args.no_mixed:
        log("mixed-length plain vs batched")
        result["mixed"] = run_mixed(args, bsw, dist)
    if not args.no_full_sw:
        log("unbanded Smith-Waterman")
        result["full_sw"] = run_full_sw(args, dist)
    if not args.no_chain:
        log("anchor chaining")
        result["chain"] = run_chain(args, dist)
    if not args.no_extend:
        log("seed extension")
        result["extend"] = run_extend(args, dist)
    if not args.no_serving:
        log("serving loop")
        peak = result.get("mixed", {}).get("batched", {}).get("pairs_per_s")
        if args.serve_peak > 0:
            peak = args.serve_peak * dist.ws
        result["serving"] = run_serving(args, dist, peak / dist.ws if peak else None)
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        log("cpu baseline")
        nthreads = os.cpu_count() or 1
        sample = cpu_sample(wl, args.cpu_seconds, nthreads)
        dt, cells, kind, desc = cpu_score(sample, wl, nthreads)
        result["cpu_baseline"] = {"value": round(cells / dt / 1e9, 4), "unit": UNIT,
                                  "cores": nthreads, "kind": kind,
                                  "sample": f"{sample.n} of the {n} pairs (same seeded workload), "
                                            f"{desc}, {cpu_isa()}",
                                  "seconds": round(dt, 2)}
    bsw.close()
    dist.close()
    if rank == 0:
        print(json.dumps(result), flush=True)


def run_mixed(args, bsw_unused, dist):
    """The mixed-length workload (10,000,000 pairs: lognormal query lengths
    clipped to [20, 2000], bands 20/50/100 per pair, 8/16-bit routing per
    pair): plain launch vs batched form on the same device-resident pairs."""
    import torch
    import tal_bsw
    from tal_bsw import synth
    wl = synth.C3
    n = args.mixed_pairs or wl.n_pairs
    b = synth.generate(wl, n, first=dist.rank * n)
    P = wl.params()
    bsw = tal_bsw.BandedPairWiseSW(P["o_del"], P["e_del"], P["o_ins"], P["e_ins"], P["zdrop"],
                                   P["end_bonus"], None, P["a"], P["b"], 1, device=dist.local)
    dp = torch.from_numpy(b.pairs.view(np.uint8).reshape(-1).copy()).cuda()
    dr = torch.from_numpy(b.ref).cuda()
    dq = torch.from_numpy(b.qer).cuda()
    dw = torch.from_numpy(b.w.astype(np.int32)).cuda()
    del b
    out = {"workload": f"c3_mixed: {n} pairs, lognormal query (median 120, sigma 0.8) in [20,2000], "
                       "w per pair in {20,50,100}, 8/16-bit routed per pair"}
    for mode, steps in (("plain", 2), ("batched", 5)):
        def go():
            if mode == "plain":
                bsw.scores_device(dp.data_ptr(), dr.data_ptr(), dr.numel(), dq.data_ptr(), dq.numel(),
                                  n, 100, 0, dw.data_ptr())
            else:
                bsw.scores_batched_device(dp.data_ptr(), dr.data_ptr(), dr.numel(), dq.data_ptr(),
                                          dq.numel(), n, 100, 0, dw.data_ptr())
        go()
        dist.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            go()
        torch.cuda.synchronize()
        t = dist.max((time.perf_counter() - t0) / steps)
        cells = dist.sum(float(bsw.last_cells))
        out[mode] = {"pairs_per_s": round(n * dist.ws / t, 1), "ms_per_step": round(t * 1e3, 2),
                     "kernel_gcups": round(cells / t / 1e9, 2), "steps": steps}
    out["batched_over_plain_pairs_per_s"] = round(out["batched"]["pairs_per_s"] /
                                                  out["plain"]["pairs_per_s"], 2)
    bsw.close()
    return out


def run_serving(args, dist, peak_pairs_per_s):
    """The serving loop under Poisson arrivals: requests of log-uniform size in
    [1,000, 200,000] pairs drawn from the mixed-length distribution, offered at
    10-90 % of the measured batched peak, against a device pool of at most
    64 GB.  Latency of a request = its outputs in the caller's (pinned) array
    minus its scheduled arrival time.  Beside it, the same arrivals through a
    plain launch per request (one request at a time, FIFO)."""
    import threading
    import torch
    import tal_bsw
    from tal_bsw import synth
    from tal_bsw.api import BswServer, now_ns
    wl = synth.C3
    npool = args.serve_pool_pairs
    b = synth.generate(wl, npool, first=20_000_000 + dist.rank * npool)
    P = wl.params()
    bsw = tal_bsw.BandedPairWiseSW(P["o_del"], P["e_del"], P["o_ins"], P["e_ins"], P["zdrop"],
                                   P["end_bonus"], None, P["a"], P["b"], 1, device=dist.local)

    def pinned(a):
        t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
        v = t.numpy().view(a.dtype).reshape(a.shape)
        v[...] = a
        return v, t

    hp, hp_t = pinned(b.pairs)
    hr, hr_t = pinned(b.ref)
    hq, hq_t = pinned(b.qer)
    hw, hw_t = pinned(b.w.astype(np.int32))
    # expected outputs (and the autotuner's bin choices) from the batched form
    exp = b.pairs.copy()
    bsw.scores_batched(exp, b.ref, b.qer, npool, 100, wpair=b.w, bits=tal_bsw.AUTO)
    if not peak_pairs_per_s:
        t0 = time.perf_counter()
        tmp = b.pairs.copy()
        bsw.scores_batched(tmp, b.ref, b.qer, npool, 100, wpair=b.w, bits=tal_bsw.AUTO)
        peak_pairs_per_s = npool / (time.perf_counter() - t0)
    lo_n, hi_n = 1000, 200000
    mean_req = (hi_n - lo_n) / np.log(hi_n / lo_n)
    rng = np.random.default_rng(1234 + dist.rank)

    def schedule(load, nreq):
        rate = load * peak_pairs_per_s / mean_req            # requests per second
        gaps = rng.exponential(1.0 / rate, nreq)
        arrive = np.cumsum(gaps) - gaps[0]
        sizes = np.exp(rng.uniform(np.log(lo_n), np.log(hi_n), nreq)).astype(np.int64)
        starts, cur = [], int(rng.integers(0, npool))
        for s_ in sizes:
            if cur + s_ > npool:
                cur = 0
            starts.append(cur)
            cur += int(s_)
        for st_, sz_ in zip(starts, sizes):
            touched[st_:st_ + sz_] = True
        return arrive, sizes, np.array(starts)

    touched = np.zeros(npool, bool)

    def drive(submit, wait, arrive, sizes, starts):
        """Submits at the scheduled times from one thread, collects in order
        on this one; returns per-request latency (ns) and the makespan."""
        nreq = len(sizes)
        tickets = [None] * nreq
        t0 = now_ns() + 20_000_000
        sched = (t0 + arrive * 1e9).astype(np.int64)

        def submitter():
            for k in range(nreq):
                while True:
                    d = sched[k] - now_ns()
                    if d <= 0:
                        break
                    if d > 2_000_000:
                        time.sleep((d - 1_000_000) / 1e9)
                tickets[k] = submit(int(starts[k]), int(sizes[k]))
        th = threading.Thread(target=submitter)
        th.start()
        done = np.zeros(nreq, np.int64)
        for k in range(nreq):
            while tickets[k] is None:
                time.sleep(0.0002)
            done[k] = wait(tickets[k])
        th.join()
        return done - sched, done.max() - t0

    out = {"workload": f"requests of log-uniform size in [{lo_n}, {hi_n}] pairs (mean {mean_req:.0f}) "
                       f"drawn from c3_mixed ({npool} pooled pairs), Poisson arrivals",
           "batched_peak_pairs_per_s": round(peak_pairs_per_s, 1), "points": []}
    # pool: min(64 GiB, 85 % of free HBM)
    srv = BswServer(bsw, slots=args.serve_slots, latency_pairs=args.serve_latency_pairs)
    infos = {}

    def s_submit(lo, n):
        return srv.submit(hp[lo:lo + n], hr, hq, w=100, wpair=hw[lo:lo + n], bits=tal_bsw.AUTO)

    def s_wait(t):
        info = srv.poll(t, timeout_us=600_000_000)
        assert info is not None and info.status == 0, "serving request failed"
        infos[t] = info
        return info.done_ns
    # warm-up (first ticks, staging of the worker)
    drive(s_submit, s_wait, *schedule(0.3, 20))
    for load in args.serve_loads:
        log(f"serving at {load:.0%} of the batched peak")
        nreq = args.serve_requests
        arrive, sizes, starts = schedule(load, nreq)
        infos.clear()
        lat, span = drive(s_submit, s_wait, arrive, sizes, starts)
        ticks = [i.tick_requests for i in infos.values()]
        stage = np.array([[i.admit_ns - i.submit_ns, i.launch_ns - i.admit_ns, i.done_ns - i.launch_ns]
                          for i in infos.values()], np.float64) / 1e6
        out["points"].append({
            "load": load, "requests": nreq,
            "offered_pairs_per_s": round(load * peak_pairs_per_s, 1),
            "achieved_pairs_per_s": round(float(sizes.sum()) / (span / 1e9), 1),
            "p50_ms": round(float(np.percentile(lat, 50)) / 1e6, 3),
            "p99_ms": round(float(np.percentile(lat, 99)) / 1e6, 3),
            "max_ms": round(float(lat.max()) / 1e6, 3),
            "mean_tick_requests": round(float(np.mean(ticks)), 2),
            "mean_ms": {"submit_to_admit": round(float(stage[:, 0].mean()), 3),
                        "admit_to_launch": round(float(stage[:, 1].mean()), 3),
                        "launch_to_done": round(float(stage[:, 2].mean()), 3)}})
    # saturation: every request at once
    arrive, sizes, starts = schedule(1.0, args.serve_requests)
    lat, span = drive(s_submit, s_wait, np.zeros_like(arrive), sizes, starts)
    out["saturated_pairs_per_s"] = round(float(sizes.sum()) / (span / 1e9), 1)
    st = srv.stats()
    srv.close()
    out["server"] = {k: st[k] for k in ("ticks", "pairs", "max_tick_requests", "max_ticks_in_flight",
                                        "pool_bytes", "pool_peak_bytes", "failed")}
    out["outputs_match"] = bool((tal_bsw.outputs(hp[touched]) == tal_bsw.outputs(exp[touched])).all())
    out["pairs_checked"] = int(touched.sum())

    # plain launch per request: one request at a time (FIFO), pairs copied in
    # and out per request, sequences device-resident
    dr = torch.from_numpy(b.ref).cuda()
    dq = torch.from_numpy(b.qer).cuda()
    dw = torch.from_numpy(b.w.astype(np.int32)).cuda()
    dpair = torch.empty(hi_n * 56, dtype=torch.uint8, device="cuda")
    hp_u8 = hp_t
    cur = torch.cuda.current_stream()

    def p_submit(lo, n):
        return (lo, n)

    def p_wait(t):
        # copies on torch's stream (pinned blocks stay tied to a stream that
        # outlives them), the launch on the library's
        lo, n = t
        dpair[:n * 56].copy_(hp_u8[lo * 56:(lo + n) * 56], non_blocking=True)
        cur.synchronize()
        bsw.scores_device(dpair.data_ptr(), dr.data_ptr(), dr.numel(), dq.data_ptr(), dq.numel(), n,
                          100, tal_bsw.AUTO, d_w=dw.data_ptr() + 4 * lo, sync=True)
        hp_u8[lo * 56:(lo + n) * 56].copy_(dpair[:n * 56], non_blocking=True)
        cur.synchronize()
        return now_ns()
    out["plain_per_request"] = []
    for load in args.serve_plain_loads:
        log(f"plain launch per request at {load:.0%}")
        arrive, sizes, starts = schedule(load, args.serve_plain_requests)
        lat, span = drive(p_submit, p_wait, arrive, sizes, starts)
        out["plain_per_request"].append({
            "load": load, "requests": len(sizes),
            "achieved_pairs_per_s": round(float(sizes.sum()) / (span / 1e9), 1),
            "p50_ms": round(float(np.percentile(lat, 50)) / 1e6, 3),
            "p99_ms": round(float(np.percentile(lat, 99)) / 1e6, 3)})
    out["plain_outputs_match"] = bool((tal_bsw.outputs(hp[touched]) == tal_bsw.outputs(exp[touched])).all())
    bsw.close()
    return out


def run_full_sw(args, dist):
    """The unbanded Smith-Waterman scorer (PairWiseSW_16::getScores drop-in):
    GCUPS = sum of len1 * len2 (the reference driver's SW_cells) per second,
    device-resident and end to end through getScores on pinned host buffers."""
    import torch
    from tal_bsw import swdata
    from tal_bsw.sw import PairWiseSW_16
    n = args.sw_pairs
    b = swdata.generate(n, 200, 1000, bits=16, seed=31 + dist.rank)
    P = dict(match=1, mismatch=-4, open=-6, extend=-1)
    cells = b.cells
    out = {"workload": f"{n} pairs, len1 U[200,1000], len2 = len1 + U[-10,10], 4% substitutions, "
                       "match 1, mismatch -4, open -6, extend -1, PairWiseSW_16 semantics"}
    with PairWiseSW_16(P["match"], P["mismatch"], P["open"], P["extend"], device=dist.local) as sw:
        stream = torch.cuda.ExternalStream(sw.stream)
        dp = torch.from_numpy(b.pairs.view(np.uint8).reshape(-1).copy()).cuda()
        ds = torch.from_numpy(b.seqbuf).cuda()
        torch.cuda.synchronize()
        for _ in range(2):
            sw.scores_device(dp.data_ptr(), ds.data_ptr(), ds.numel(), n)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        steps = 3
        dist.barrier()
        e0.record(stream)
        for _ in range(steps):
            sw.scores_device(dp.data_ptr(), ds.data_ptr(), ds.numel(), n)
        e1.record(stream)
        torch.cuda.synchronize()
        t = dist.max(e0.elapsed_time(e1) / 1e3 / steps)
        out["device"] = {"value": round(dist.sum(cells) / t / 1e9, 2), "unit": "GCUPS",
                         "ms_per_step": round(t * 1e3, 3)}
        hp = torch.empty(b.pairs.nbytes, dtype=torch.uint8, pin_memory=True)
        hs = torch.empty(b.seqbuf.nbytes, dtype=torch.uint8, pin_memory=True)
        hp.numpy()[:] = b.pairs.view(np.uint8).reshape(-1)
        hs.numpy()[:] = b.seqbuf
        hpairs = hp.numpy().view(swdata.SW_DTYPE)
        sw.getScores(hpairs, hs.numpy(), n, 1)
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(steps):
            sw.getScores(hpairs, hs.numpy(), n, 1)
        te = dist.max((time.perf_counter() - t0) / steps)
        out["e2e"] = {"value": round(dist.sum(cells) / te / 1e9, 2), "unit": "GCUPS",
                      "ms_per_step": round(te * 1e3, 3),
                      "h2d_bytes_per_step": int(b.pairs.nbytes + b.seqbuf.nbytes),
                      "d2h_bytes_per_step": int(b.pairs.nbytes)}
        dev_scores = dp.cpu().numpy().view(swdata.SW_DTYPE)["score"]
        out["outputs_match_device_path"] = bool((dev_scores == hpairs["score"]).all())
    if dist.rank == 0 and not args.no_cpu_baseline:
        import oracle
        k = min(n, 2000)
        nth = os.cpu_count() or 1
        t0 = time.perf_counter()
        exp = oracle.sw(b.pairs[:k], b.seqbuf, b.stride, P, nthreads=nth)
        dt = time.perf_counter() - t0
        sample_cells = int((b.pairs["len1"][:k].astype(np.int64) * b.pairs["len2"][:k]).sum())
        out["cpu_baseline"] = {"value": round(sample_cells / dt / 1e9, 4), "unit": "GCUPS", "cores": nth,
                               "kind": "port", "sample": f"first {k} pairs, oracle restatement"}
        out["outputs_match_oracle_sample"] = bool((exp["score"] == hpairs["score"][:k]).all())
    return out


def run_chain(args, dist):
    """The anchor chaining DP (dp_chain::mm_dp_vectorized drop-in, the
    reference driver's parameters): predecessor evaluations (the sum over
    anchors of i - st, the reference loop's iterations) and anchors per second,
    device-resident and end to end through mm_dp_batch on pinned host buffers."""
    import torch
    from tal_bsw import chaindata
    from tal_bsw.chain import dp_chain
    b = chaindata.generate(args.chain_reads, 1000, 10000, seed=77 + dist.rank)
    P, dr, dq = chaindata.DRIVER_PARAMS, chaindata.DRIVER_DR, chaindata.DRIVER_DQ
    n = b.n
    out = {"workload": f"{b.n_reads} reads of U[1000,10000] bases, {n} anchors (span 15, one per "
                       "1-10 query bases on the true diagonal, indel drift, 30% reads with a "
                       "competing copy, 20% noise anchors), dp_chain(5000, 5000, 500, 25, 5000, "
                       "1.0, 0, 1), dr = dq = 5000"}
    with dp_chain(*P, device=dist.local) as ch:
        stream = torch.cuda.ExternalStream(ch.stream)
        da = torch.from_numpy(b.anchors.view(np.uint8).copy()).cuda()
        do = torch.from_numpy(b.offsets.copy()).cuda()
        df = torch.zeros(n, dtype=torch.int32, device="cuda")
        dp_ = torch.zeros(n, dtype=torch.int32, device="cuda")
        dv = torch.zeros(n, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()

        def step():
            ch.mm_dp_device(da.data_ptr(), do.data_ptr(), b.n_reads, dr, dq, df.data_ptr(),
                            dp_.data_ptr(), dv.data_ptr())
        for _ in range(3):
            step()
        evals = ch.last_evals
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        steps = 3
        dist.barrier()
        e0.record(stream)
        for _ in range(steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        t = dist.max(e0.elapsed_time(e1) / 1e3 / steps)
        out["device"] = {"evals_per_s": round(dist.sum(evals) / t, 1),
                         "anchors_per_s": round(dist.sum(n) / t, 1), "ms_per_step": round(t * 1e3, 3),
                         "evals_per_step": int(evals)}
        ha = torch.empty(b.anchors.nbytes, dtype=torch.uint8, pin_memory=True)
        ha.numpy()[:] = b.anchors.view(np.uint8)
        anchors_pinned = ha.numpy().view(chaindata.ANCHOR_DTYPE)
        outs_t = [torch.empty(4 * n, dtype=torch.uint8, pin_memory=True) for _ in range(3)]
        outs = (outs_t[0].numpy().view(np.uint32), outs_t[1].numpy().view(np.int32),
                outs_t[2].numpy().view(np.int32))
        ch.mm_dp_batch(anchors_pinned, b.offsets, dr, dq, out=outs)
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(steps):
            gf, gp, gv = ch.mm_dp_batch(anchors_pinned, b.offsets, dr, dq, out=outs)
        te = dist.max((time.perf_counter() - t0) / steps)
        out["e2e"] = {"evals_per_s": round(dist.sum(evals) / te, 1),
                      "anchors_per_s": round(dist.sum(n) / te, 1), "ms_per_step": round(te * 1e3, 3),
                      "h2d_bytes_per_step": int(b.anchors.nbytes + b.offsets.nbytes),
                      "d2h_bytes_per_step": int(12 * n)}
        out["outputs_match_device_path"] = bool(
            (df.cpu().numpy().view(np.uint32) == gf).all() and (dp_.cpu().numpy() == gp).all()
            and (dv.cpu().numpy() == gv).all())
    if dist.rank == 0 and not args.no_cpu_baseline:
        import oracle
        k = min(b.n_reads, 400)
        sub_o = b.offsets[:k + 1]
        sub_a = b.anchors[:int(sub_o[-1])]
        nth = os.cpu_count() or 1
        t0 = time.perf_counter()
        ef, ep, ev = oracle.chain(sub_a, sub_o, P[2], P[4], dr, dq, nthreads=nth)
        dt = time.perf_counter() - t0
        # the sample's evaluations: i - st per anchor, from the same window rule
        with dp_chain(*P, device=dist.local) as ch2:
            sf, sp, sv = ch2.mm_dp_batch(sub_a, sub_o, dr, dq)
            sample_evals = ch2.last_evals
        out["cpu_baseline"] = {"evals_per_s": round(sample_evals / dt, 1), "cores": nth, "kind": "port",
                               "sample": f"first {k} reads ({sub_a.shape[0]} anchors), oracle restatement"}
        out["outputs_match_oracle_sample"] = bool((sf == ef).all() and (sp == ep).all() and (sv == ev).all())
    return out


def run_extend(args, dist):
    """Caller-side seed extension (include/tal_extend.h) end to end on host
    buffers: seeds per second, and the cells of its two BSW batches."""
    import tal_bsw
    from tal_bsw import seeddata, synth
    from tal_bsw.extend import extend_seeds
    b = seeddata.generate(args.extend_reads, seed=55 + dist.rank)
    P = synth.C2.params()
    out = {"workload": f"{b.n_reads} reads of U[100,250] bp from a 2 Mb random reference (3% "
                       f"substitutions, 1-3 bp indels, 10% with a random tail), {b.seeds.shape[0]} "
                       "exact-match seeds, w = 100 with up to 2 band tries (BWA-MEM's loop), clipping "
                       "penalties 5 / 5, C2 scoring"}
    with tal_bsw.BandedPairWiseSW(P["o_del"], P["e_del"], P["o_ins"], P["e_ins"], P["zdrop"],
                                  P["end_bonus"], None, P["a"], P["b"], 1, device=dist.local) as bsw:
        for _ in range(2):
            extend_seeds(bsw, b.ref, b.reads, b.read_off, b.seeds, 100, 5, 5, band_tries=2)
        steps = 3
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(steps):
            got = extend_seeds(bsw, b.ref, b.reads, b.read_off, b.seeds, 100, 5, 5, band_tries=2)
        t = dist.max((time.perf_counter() - t0) / steps)
    out["e2e"] = {"seeds_per_s": round(dist.sum(b.seeds.shape[0]) / t, 1), "ms_per_step": round(t * 1e3, 3),
                  "h2d_bytes_per_step": int(b.ref.nbytes + b.reads.nbytes + b.seeds.nbytes),
                  "d2h_bytes_per_step": int(got.nbytes)}
    if dist.rank == 0 and not args.no_cpu_baseline:
        import oracle
        k = min(b.seeds.shape[0], 1500)
        t0 = time.perf_counter()
        exp = oracle.extend(b.ref, b.reads, b.read_off, b.seeds[:k], P, 100, 5, 5, band_tries=2)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"seeds_per_s": round(k / dt, 1), "cores": 1, "kind": "port",
                               "sample": f"first {k} seeds, oracle restatement (python windows, "
                                         "C BSW oracle)"}
        out["outputs_match_oracle_sample"] = bool(all((got[f][:k] == exp[f]).all()
                                                      for f in ("rb", "re", "qb", "qe", "score")))
    return out


# -------------------------------------------------------------------- reference arm
def run_reference(args):
    from tal_bsw import synth
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    wl = synth.WORKLOADS[args.workload]
    nthreads = os.cpu_count() or 1
    # each step: a bounded sample of the workload, a few seconds of CPU work
    per_step = max(1.0, min(6.0, 150.0 / max(args.steps + args.warmup, 1)))
    sample = cpu_sample(wl, per_step, nthreads)
    for _ in range(args.warmup):
        cpu_score(sample, wl, nthreads)
    tot_t, tot_c = 0.0, 0
    kind = desc = ""
    for _ in range(args.steps):
        dt, cells, kind, desc = cpu_score(sample, wl, nthreads)
        tot_t += dt
        tot_c += cells
    value = tot_c / tot_t / 1e9
    bits = 8 if wl.bits == 8 else 16
    res = {"metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": ws,
           "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": round(tot_t / args.steps * 1e3, 3), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "int16",
           "data": "synthetic (seeded generator, no dataset)", "impl": "reference",
           "config": {"workload": f"{wl.name}: {wl.n_pairs} pairs, w={wl.w}, getScores{bits}; "
                                  f"each step a {sample.n}-pair sample"},
           "pairs_per_s": round(sample.n * args.steps / tot_t, 1),
           "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": nthreads, "kind": kind,
                            "sample": f"{sample.n} pairs per step, {desc}, {cpu_isa()}"},
           "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(res), flush=True)


def main():
    import faulthandler
    faulthandler.enable()
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
