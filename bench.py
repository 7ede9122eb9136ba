#!/usr/bin/env python
"""Benchmark of the banded Smith-Waterman seed extension on GB300.

Metric: BSW GCUPS (reference cells per second; a cell is one iteration of the
reference's scalar inner loop, bandedSWA.cpp:175-200) and pairs/s, batched form
against the plain launch.  A step is one pass of the hot path over one batch:
at N=1 the mixed-length workload, 10,000,000 seeded synthetic pairs (query
length lognormal, median 120, sigma 0.8, clipped to [20, 2000]; errors
U[1%,8%]; band per pair in {20, 50, 100}; h0 U[19,250]; each pair 8- or
16-bit by the routing rule), scored by the batched form, bit-exact against the
reference's getScores8 / getScores16.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`value` is measured with the inputs resident in HBM (device-resident batched
call, CUDA events on the library's stream); `e2e` goes through the C ABI call
tal_bsw_scores_batched with pinned host buffers, host<->device copies inside
the timed region.  Under torchrun each rank scores its own shard of
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

# The batched form and the serving ticks run their segment launches on up to
# 32 forked streams; with CUDA's default of 8 hardware work queues, streams
# that share a queue serialise their launches (a 200,000-pair tick's short
# segments start only after the long ones).  Set before the CUDA context
# exists; an explicit setting in the environment wins.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

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
    ap.add_argument("--workload", default="c3_mixed")
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="CPU work for the cpu_baseline sample (rank 0, N=1)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=None)
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg (profiling)")
    ap.add_argument("--pairs", type=int, default=None,
                    help="score only the first N pairs of the workload (profiling a small case)")
    ap.add_argument("--profile-call", action="store_true",
                    help="profiling: warm up the batched call (--warmup calls), print the library's "
                         "launch counter, make one more call and exit (no timing, no JSON line)")
    ap.add_argument("--trace-tick", type=int, default=0,
                    help="serve single requests of this many c3_mixed pairs, one at a time, with the "
                         "library's segment trace on (stderr), and print each tick's time (profiling)")
    ap.add_argument("--profile-plain", action="store_true",
                    help="with --profile-call: the plain launch (tal_bsw_scores_device) instead of the batched form")
    ap.add_argument("--no-grouped", action="store_true",
                    help="skip the grouped-form (TAL_BSW_GROUPED) leg")
    ap.add_argument("--no-extras", action="store_true", help="skip the single-shape workloads")
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
def _classes(batch, wl):
    """(w, bits, indices) of each call the reference's caller would issue for
    `batch`: one band per call, 8/16-bit by the routing rule."""
    import oracle
    P = wl.params()
    n = batch.n
    warr = batch.w.astype(np.int64) if wl.w_choices else np.full(n, wl.w, np.int64)
    if wl.bits in (8, 16):
        is8 = np.full(n, wl.bits == 8)
    else:
        is8 = oracle.eligible8(batch.pairs, warr, P)
    out = []
    for wv in np.unique(warr):
        for bits in (8, 16):
            sel = np.nonzero((warr == wv) & (is8 == (bits == 8)))[0]
            if sel.size:
                out.append((int(wv), bits, sel))
    return out


def cpu_score(batch, wl, nthreads):
    """Times the CPU implementation on `batch` (one call per band / precision
    class, as the reference's caller issues them); returns (seconds,
    ref-cells, kind, description, scored pairs).  The reference itself where
    it was compiled on this host (x86 with AVX-512: getScores8/16 from
    oracle/_ref, one instance per thread), else the oracle's port of
    scalarBandedSWAWrapper (the reference's portable path, equal to
    getScores16 at e_del = e_ins = 1 and to getScores8 inside the 8-bit
    range)."""
    import oracle
    P = wl.params()
    out = batch.pairs.copy()
    cells = 0
    if oracle.ref_available("avx512"):
        t = time.perf_counter()
        for wv, bits, sel in _classes(batch, wl):
            parts = np.array_split(sel, nthreads)
            with cf.ThreadPoolExecutor(nthreads) as ex:
                res = list(ex.map(lambda ix: oracle.reference(batch.pairs[ix], batch.ref, batch.qer,
                                                              wv, P, mode=bits, pristine=False), parts))
            for ix, r in zip(parts, res):
                out[ix] = r
        dt = time.perf_counter() - t
        for wv, bits, sel in _classes(batch, wl):
            cells += oracle.scalar(batch.pairs[sel], batch.ref, batch.qer, wv, P, nthreads=nthreads)[1]
        return dt, cells, "reference", "getScores8/16 (AVX-512BW build of the reference)", out
    t = time.perf_counter()
    for wv, bits, sel in _classes(batch, wl):
        o, c = oracle.scalar(batch.pairs[sel], batch.ref, batch.qer, wv, P, nthreads=nthreads)
        out[sel] = o
        cells += c
    dt = time.perf_counter() - t
    return dt, cells, "port", "oracle port of scalarBandedSWAWrapper (bandedSWA.cpp:116-260)", out


def cpu_sample(wl, seconds, nthreads, first=0):
    """The first pairs of the workload (the generator is prefix-stable: pair k
    is the same in any batch size), about `seconds` of CPU work."""
    from tal_bsw import synth
    n = 2000
    probe = synth.generate(wl, n, first=first)
    dt = cpu_score(probe, wl, nthreads)[0]
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


def workload_desc(wl, n):
    """The workload string both arms report (same configuration)."""
    if wl.name == "c3_mixed":
        return (f"c3_mixed: {n} pairs, lognormal query (median 120, sigma 0.8) in [20,2000], "
                "errors U[1%,8%] (80% subs, 20% 1-5 bp indels), w per pair in {20,50,100}, "
                "h0 U[19,250], 8/16-bit routed per pair (getScores8 / getScores16 semantics), "
                "batched form vs plain launch")
    bits = 8 if wl.bits == 8 else 16
    return (f"{wl.name}: {n} pairs, query U[{wl.len_lo},{wl.len_hi}], w={wl.w}, zdrop={wl.zdrop}, "
            f"getScores{bits}")


# -------------------------------------------------------------------------- our arm
def run_ours(args):
    """Headline: the batched mixed-length workload (10,000,000 pairs), the
    batched form device-resident (`value`) and through tal_bsw_scores_batched
    on pinned host buffers (`e2e`), beside the plain launch on the same
    pairs; then the single-shape workloads, the grouped kernel, the sibling
    kernels, serving and the CPU baseline."""
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
    bits = wl.bits                          # 0: 8/16-bit routed per pair
    wpair = b.w.astype(np.int32) if wl.w_choices else None
    cinfo = workload_cells(wl.name)

    bsw = tal_bsw.BandedPairWiseSW(P["o_del"], P["e_del"], P["o_ins"], P["e_ins"], P["zdrop"],
                                   P["end_bonus"], None, P["a"], P["b"], 1, device=local)
    stream = torch.cuda.ExternalStream(bsw.stream)
    pairs_u8 = b.pairs.view(np.uint8).reshape(-1)
    dp = torch.from_numpy(pairs_u8.copy()).cuda()
    dr = torch.from_numpy(b.ref).cuda()
    dq = torch.from_numpy(b.qer).cuda()
    dw = torch.from_numpy(wpair).cuda() if wpair is not None else None
    dwp = dw.data_ptr() if dw is not None else None
    torch.cuda.synchronize()

    def step_batched():
        bsw.scores_batched_device(dp.data_ptr(), dr.data_ptr(), dr.numel(), dq.data_ptr(), dq.numel(),
                                  n, wl.w, bits, dwp)

    log("batched form: warm-up (autotune, graph capture)")
    for _ in range(max(args.warmup, 3)):
        step_batched()
    kernel_cells = bsw.last_cells
    flagged, regroups = bsw.last_regroup()
    counted = bool(cinfo) and rank == 0 and cinfo["n_pairs"] == n
    ratio = dist.max(int(cinfo["ref_cells"]) / max(kernel_cells, 1) if counted else 0.0)
    ref_cells = int(cinfo["ref_cells"]) if counted else int(kernel_cells * (ratio or 1.0))

    # ---- device-resident timed region (the batched form)
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
    for _ in range(args.steps):
        step_batched()
    e1.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    launches = bsw.launch_count - launches0
    dist.barrier()
    t_step = e0.elapsed_time(e1) / 1e3 / args.steps
    t_step_max = dist.max(t_step)
    total_cells = dist.sum(float(ref_cells))
    total_pairs = n * ws
    value = total_cells / t_step_max / 1e9
    gpu_out = dp.cpu().numpy().view(tal_bsw.SEQPAIR_DTYPE).copy()
    log(f"batched, device-resident: {value:.1f} GCUPS, {total_pairs / t_step_max / 1e6:.2f} M pairs/s")

    # ---- end to end through the C ABI (tal_bsw_scores_batched), pinned host buffers
    e2e = None
    if not args.no_e2e:
        hp = torch.empty(pairs_u8.shape[0], dtype=torch.uint8, pin_memory=True)
        hr = torch.empty(b.ref.shape[0], dtype=torch.uint8, pin_memory=True)
        hq = torch.empty(b.qer.shape[0], dtype=torch.uint8, pin_memory=True)
        hp.numpy()[:] = pairs_u8
        hr.numpy()[:] = b.ref
        hq.numpy()[:] = b.qer
        hw = None
        if wpair is not None:
            hw = torch.empty(n, dtype=torch.int32, pin_memory=True)
            hw.numpy()[:] = wpair
        hpairs = hp.numpy().view(tal_bsw.SEQPAIR_DTYPE)

        def step_e2e():
            bsw.scores_batched(hpairs, hr.numpy(), hq.numpy(), n, wl.w,
                               wpair=None if hw is None else hw.numpy(), bits=bits)
        e2e_steps = args.e2e_steps or max(3, args.steps // 2)
        for _ in range(2):
            step_e2e()
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            step_e2e()
        t_e2e_max = dist.max((time.perf_counter() - t0) / e2e_steps)
        h2d = pairs_u8.nbytes + b.ref.nbytes + b.qer.nbytes + (0 if wpair is None else wpair.nbytes)
        agree = bool((tal_bsw.outputs(gpu_out) == tal_bsw.outputs(hpairs)).all())
        e2e = {"value": round(total_cells / t_e2e_max / 1e9, 3), "unit": UNIT,
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(pairs_u8.nbytes),
               "pairs_per_s": round(total_pairs / t_e2e_max, 1), "ms_per_step": round(t_e2e_max * 1e3, 3),
               "steps": e2e_steps, "outputs_match_device_path": agree,
               "call": "tal_bsw_scores_batched (host buffers, pinned; copies inside the timed region)"}
        del hp, hr, hq

    # ---- plain launch (one scoring launch per call) on the same pairs
    plain = None
    if not args.no_mixed:
        log("plain launch on the same pairs")

        def step_plain():
            bsw.scores_device(dp.data_ptr(), dr.data_ptr(), dr.numel(), dq.data_ptr(), dq.numel(),
                              n, wl.w, bits, dwp)
            bsw.sync()
        step_plain()
        pflag = bsw.last_regroup()
        dist.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        psteps = 2
        for _ in range(psteps):
            step_plain()
        t_plain = dist.max((time.perf_counter() - t0) / psteps)
        pout = dp.cpu().numpy().view(tal_bsw.SEQPAIR_DTYPE)
        plain = {"value": round(total_cells / t_plain / 1e9, 3), "unit": UNIT,
                 "pairs_per_s": round(total_pairs / t_plain, 1), "ms_per_step": round(t_plain * 1e3, 2),
                 "steps": psteps, "flagged_pairs": pflag[0], "regrouped_groups": pflag[1],
                 "outputs_match_batched": bool((tal_bsw.outputs(pout) == tal_bsw.outputs(gpu_out)).all())}

    # ---- rooflines: integer pipe (DPX) and HBM
    hbm_peak, peak_src = measured_peaks()
    lens = int(b.pairs["len1"].sum() + b.pairs["len2"].sum())
    alg_bytes = lens + 56 * n + 24 * n + (4 * n if wpair is not None else 0)
    dpx, i32 = probe_int_peak(local)
    int_cells_peak = dpx / 4.0                   # 8 int16 lane-ops per cell, 2 lanes per DPX op
    cell_rate = ref_cells / t_step               # this rank, whole batched graph
    hbm_rate = alg_bytes / t_step / 1e9

    result = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": max(args.warmup, 3),
        "ms_per_step": round(t_step_max * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int16 / int8 (routed per pair), integer DP",
        "data": "synthetic (seeded generator, no dataset)",
        "config": {"workload": workload_desc(wl, wl.n_pairs), "pairs_per_step": total_pairs,
                   "ref_cells_per_step": int(total_cells), "kernel_cells_per_step": int(kernel_cells) * ws,
                   "call": "tal_bsw_scores_batched_device (device-resident), one CUDA graph per call",
                   "l2": "inputs larger than L2 (no flush needed)",
                   "cuda_device_max_connections": os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS"),
                   "parallelism": f"replica shards x{ws}, no collective"},
        "pairs_per_s": round(total_pairs / t_step_max, 1),
        "wall_s_timed": round(wall, 3),
        "exactness": {"flagged_pairs": flagged, "regrouped_groups": regroups,
                      "flag_rate": round(flagged / max(n, 1), 8),
                      "note": "pairs whose outputs could depend on their SIMD group (or outside the "
                              "per-pair kernels' exact range), re-scored in the reference's grouping "
                              "inside the timed call"},
        "gpu_launches": int(launches),
        "roofline": {"bound": "int16x2 DPX (integer pipe)", "achieved": round(cell_rate, 1),
                     "peak": round(int_cells_peak, 1), "unit": "cells/s",
                     "frac": round(cell_rate / int_cells_peak, 5),
                     "traffic": profile_traffic("c3_mixed_batched"),
                     "peak_source": "live __viaddmax_s16x2 probe (tal_bsw_probe_int_peak)",
                     "peak_dpx_instr_per_s": dpx, "peak_i32_instr_per_s": i32,
                     "model": "4 DPX int16x2 instructions per cell; achieved = reference cells / "
                              "device time of the batched call (all its launches)"},
        "roofline_hbm": {"bound": "hbm", "achieved": round(hbm_rate, 2), "peak": hbm_peak,
                         "unit": "GB/s", "frac": round(hbm_rate / hbm_peak, 6), "peak_source": peak_src,
                         "algorithmic_bytes_per_step": int(alg_bytes),
                         "traffic": profile_traffic("c3_mixed_batched")},
        "clocks": clk,
    }
    if e2e:
        result["e2e"] = e2e
    if plain:
        result["plain"] = plain
        result["batched_over_plain_pairs_per_s"] = round(result["pairs_per_s"] / plain["pairs_per_s"], 2)
    gpu_keep = gpu_out if rank == 0 else None
    del dp, dr, dq, dw, b
    torch.cuda.empty_cache()
    if not args.no_extras:
        for name in ("c1_151bp", "c1_8bit", "c2_16bit", "c4_long"):
            log(f"workload {name}")
            result[name] = run_workload(name, bsw, dist, args)
    if not args.no_grouped:
        log("grouped kernel (TAL_BSW_GROUPED) on c2_16bit")
        result["grouped"] = run_grouped(bsw, dist)
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
        peak = result["pairs_per_s"] if wl.name == "c3_mixed" else None
        if args.serve_peak > 0:
            peak = args.serve_peak * dist.ws
        result["serving"] = run_serving(args, dist, peak / dist.ws if peak else None)
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        log("cpu baseline")
        nthreads = os.cpu_count() or 1
        sample = cpu_sample(wl, args.cpu_seconds, nthreads)
        dt, cells, kind, desc, cout = cpu_score(sample, wl, nthreads)
        m = sample.n
        match = bool((tal_bsw.outputs(cout) == tal_bsw.outputs(gpu_keep[:m])).all())
        result["cpu_baseline"] = {"value": round(cells / dt / 1e9, 4), "unit": UNIT,
                                  "cores": nthreads, "kind": kind,
                                  "sample": f"the first {m} of the {n} pairs (the generator is prefix-"
                                            f"stable), {desc}, {cpu_isa()}",
                                  "pairs_per_s": round(m / dt, 1), "seconds": round(dt, 2)}
        result["outputs_match_cpu_baseline"] = match
    bsw.close()
    dist.close()
    if rank == 0:
        print(json.dumps(result), flush=True)


def run_workload(name, bsw, dist, args):
    """A single-shape workload, device-resident: the plain launch (its
    scoring kernel's time and the whole call) and the batched form, in
    GCUPS, with the pairs flagged for group re-scoring."""
    import torch
    import tal_bsw
    from tal_bsw import synth
    wl = synth.WORKLOADS[name]
    n = wl.n_pairs
    b = synth.generate(wl, n, first=dist.rank * n)
    P = wl.params()
    bits = wl.bits
    cinfo = workload_cells(name)
    w = synth.WORKLOADS[name].w
    x = tal_bsw.BandedPairWiseSW(P["o_del"], P["e_del"], P["o_ins"], P["e_ins"], P["zdrop"],
                                 P["end_bonus"], None, P["a"], P["b"], 1, device=dist.local)
    dp = torch.from_numpy(b.pairs.view(np.uint8).reshape(-1).copy()).cuda()
    dr = torch.from_numpy(b.ref).cuda()
    dq = torch.from_numpy(b.qer).cuda()
    out = {"workload": workload_desc(wl, n)}
    steps = 2 if name == "c4_long" else 5
    for mode in ("plain", "batched"):
        def go():
            if mode == "plain":
                x.scores_device(dp.data_ptr(), dr.data_ptr(), dr.numel(), dq.data_ptr(), dq.numel(), n, w, bits)
                x.sync()
            else:
                x.scores_batched_device(dp.data_ptr(), dr.data_ptr(), dr.numel(), dq.data_ptr(), dq.numel(),
                                        n, w, bits)
        for _ in range(2):
            go()
        fl = x.last_regroup()
        kcells = x.last_cells
        cells = int(cinfo["ref_cells"]) if cinfo and cinfo["n_pairs"] == n and dist.rank == 0 else kcells
        dist.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        kms = 0.0
        for _ in range(steps):
            go()
            kms += x.last_kernel_ms
        t = dist.max((time.perf_counter() - t0) / steps)
        rec = {"value": round(dist.sum(float(cells)) / t / 1e9, 2), "unit": UNIT,
               "pairs_per_s": round(n * dist.ws / t, 1), "ms_per_step": round(t * 1e3, 3),
               "flagged_pairs": fl[0], "regrouped_groups": fl[1]}
        if mode == "plain":
            rec["kernel_ms"] = round(kms / steps, 3)
            rec["kernel_gcups"] = round(cells / (kms / steps / 1e3) / 1e9, 2) if kms > 0 else None
        out[mode] = rec
    x.close()
    return out


def run_grouped(bsw_unused, dist):
    """The grouped kernel alone (TAL_BSW_GROUPED: every pair in the
    reference's SIMD groups) on the 1,000,000-pair 16-bit workload."""
    import torch
    import tal_bsw
    from tal_bsw import synth
    wl = synth.C2
    n = wl.n_pairs
    b = synth.generate(wl, n, first=dist.rank * n)
    P = wl.params()
    cinfo = workload_cells(wl.name)
    x = tal_bsw.BandedPairWiseSW(P["o_del"], P["e_del"], P["o_ins"], P["e_ins"], P["zdrop"],
                                 P["end_bonus"], None, P["a"], P["b"], 1, device=dist.local)
    dp = torch.from_numpy(b.pairs.view(np.uint8).reshape(-1).copy()).cuda()
    dr = torch.from_numpy(b.ref).cuda()
    dq = torch.from_numpy(b.qer).cuda()
    gb = 16 | tal_bsw.api.GROUPED

    def go():
        x.scores_device(dp.data_ptr(), dr.data_ptr(), dr.numel(), dq.data_ptr(), dq.numel(), n, wl.w, gb)
        x.sync()
    go()
    dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(2):
        go()
    t = dist.max((time.perf_counter() - t0) / 2)
    x.close()
    return {"workload": workload_desc(wl, n), "value": round(int(cinfo["ref_cells"]) / t / 1e9, 2),
            "unit": UNIT, "ms_per_step": round(t * 1e3, 3),
            "note": "device-resident call with TAL_BSW_GROUPED (one warp per SIMD group of the "
                    "reference for every pair); the default path runs it only for flagged pairs"}


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
            # the queueing-free floor: the largest request's service time at the
            # batched rate (the whole GPU), and with processor sharing at this load
            "p99_floor_ms": {"largest_request_at_batched_rate": round(float(sizes.max()) / peak_pairs_per_s * 1e3, 3),
                             "same_under_processor_sharing": round(float(sizes.max()) / peak_pairs_per_s * 1e3
                                                                   / max(1.0 - load, 1e-3), 3)},
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
    """The reference's CPU implementation of the path on this host's cores, on
    the same workload (`config.workload` as our arm's); each step a bounded
    sample of it (the first pairs, prefix-stable generator)."""
    from tal_bsw import synth
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    wl = synth.WORKLOADS[args.workload]
    nthreads = os.cpu_count() or 1
    per_step = max(1.0, min(6.0, 150.0 / max(args.steps + args.warmup, 1)))
    sample = cpu_sample(wl, per_step, nthreads)
    for _ in range(args.warmup):
        cpu_score(sample, wl, nthreads)
    tot_t, tot_c = 0.0, 0
    kind = desc = ""
    for _ in range(args.steps):
        dt, cells, kind, desc, _ = cpu_score(sample, wl, nthreads)
        tot_t += dt
        tot_c += cells
    value = tot_c / tot_t / 1e9
    res = {"metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": ws,
           "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": round(tot_t / args.steps * 1e3, 3), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "int16 / int8 (routed per pair), integer DP",
           "data": "synthetic (seeded generator, no dataset)", "impl": "reference",
           "config": {"workload": workload_desc(wl, wl.n_pairs), "sample_pairs_per_step": sample.n,
                      "same_config": True},
           "pairs_per_s": round(sample.n * args.steps / tot_t, 1),
           "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": nthreads, "kind": kind,
                            "sample": f"the first {sample.n} pairs of the workload per step, {desc}, "
                                      f"{cpu_isa()}"},
           "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(res), flush=True)


def profile_call(args):
    """One batched call of the workload after --warmup calls, for ncu: prints
    the launch counter before the profiled call (ncu -s) and its launches (-c)."""
    import torch
    import tal_bsw
    from tal_bsw import synth
    wl = synth.WORKLOADS[args.workload]
    n = wl.n_pairs if not args.pairs else min(args.pairs, wl.n_pairs)
    b = synth.generate(wl, n)
    P = wl.params()
    bsw = tal_bsw.BandedPairWiseSW(P["o_del"], P["e_del"], P["o_ins"], P["e_ins"], P["zdrop"],
                                   P["end_bonus"], None, P["a"], P["b"], 1, device=0)
    dp = torch.from_numpy(b.pairs.view(np.uint8).reshape(-1).copy()).cuda()
    dr = torch.from_numpy(b.ref).cuda()
    dq = torch.from_numpy(b.qer).cuda()
    dw = torch.from_numpy(b.w.astype(np.int32)).cuda() if wl.w_choices else None
    torch.cuda.synchronize()

    def call():
        if args.profile_plain:
            bsw.scores_device(dp.data_ptr(), dr.data_ptr(), dr.numel(), dq.data_ptr(), dq.numel(),
                              n, wl.w, wl.bits, None if dw is None else dw.data_ptr())
        else:
            bsw.scores_batched_device(dp.data_ptr(), dr.data_ptr(), dr.numel(), dq.data_ptr(), dq.numel(),
                                      n, wl.w, wl.bits, None if dw is None else dw.data_ptr())
        bsw.sync()
    for _ in range(args.warmup):
        call()
    l0 = bsw.launch_count
    call()
    print(f"launches before the profiled call: {l0}; in it: {bsw.launch_count - l0}; "
          f"flagged pairs / groups: {bsw.last_regroup()}", flush=True)
    bsw.close()


def trace_tick(args):
    """Single serving requests of --trace-tick C3 pairs, each alone in its tick,
    with TAL_BSW_TRACE=1: the library prints each segment launch's start / end
    (ms after the tick's fork; it synchronises the tick after its segments, so
    the request's launch-to-done time printed here is what follows them -- the
    regroup pass and the copies back)."""
    os.environ["TAL_BSW_TRACE"] = "1"
    import torch
    import tal_bsw
    from tal_bsw import synth
    from tal_bsw.api import BswServer
    n = args.trace_tick
    wl = synth.C3
    npool = max(3 * n, 1_000_000)
    b = synth.generate(wl, npool, first=20_000_000)
    P = wl.params()
    bsw = tal_bsw.BandedPairWiseSW(P["o_del"], P["e_del"], P["o_ins"], P["e_ins"], P["zdrop"],
                                   P["end_bonus"], None, P["a"], P["b"], 1, device=0)
    tmp = b.pairs.copy()
    bsw.scores_batched(tmp, b.ref, b.qer, npool, 100, wpair=b.w, bits=tal_bsw.AUTO)  # autotune

    def pinned(a):
        t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
        v = t.numpy().view(a.dtype).reshape(a.shape)
        v[...] = a
        return v, t
    hp, _hp = pinned(b.pairs)
    hr, _hr = pinned(b.ref)
    hq, _hq = pinned(b.qer)
    hw, _hw = pinned(b.w.astype(np.int32))
    srv = BswServer(bsw)
    for k in range(args.warmup + args.steps):
        lo = (k * n) % (npool - n + 1)
        t = srv.submit(hp[lo:lo + n], hr, hq, w=100, wpair=hw[lo:lo + n], bits=tal_bsw.AUTO)
        info = srv.poll(t, timeout_us=60_000_000)
        assert info is not None and info.status == 0
        if k >= args.warmup:
            sub = b.pairs[lo:lo + n]
            print(f"tick {k - args.warmup}: pairs {lo}..{lo + n}, max len2 {int(sub['len2'].max())}, "
                  f"launch -> done after the segments {(info.done_ns - info.launch_ns) / 1e6:.2f} ms",
                  file=sys.stderr, flush=True)
    srv.close()
    bsw.close()


def main():
    import faulthandler
    faulthandler.enable()
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.trace_tick:
        trace_tick(args)
    elif args.profile_call:
        profile_call(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
