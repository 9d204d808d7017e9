#!/usr/bin/env python
"""Headline benchmark: FP64 xbatched kronmult, d=6, n=4, on one GB300.

Workload (seeded synthetic, shapes and distributions of the reference's
headline configuration): 8192 X blocks and 8192 Y blocks of n^d = 4096
doubles, 131072 entries (y_idx, x_idx, a_idx[6]) with per-Y contribution
counts geometric (mean 16, shuffled), x_idx uniform, factors drawn from a pool
of 1024 4x4 matrices per dimension with entries N(0,1)/2, X ~ N(0,1).  The
entries reach the library as the reference's xbatched pointer arrays
(kronmult6_xbatched.cpp:5-13).  One step = one kronmult6_xbatched call over
all entries.  X and Y pools are 256 MiB each (> 129 MB L2), so no L2 flush is
needed between steps.

Forms: "chosen" is the library's automatic choice for (d=6, n=4, FP64) -- the
double-float split form; "plain" is native FP64.  Both are timed; the JSON
line's value is the chosen form, and its error against the plain form is
reported (the metric allows <= 1e-12).

  python bench.py [--steps K] [--warmup W] [--gpus N] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

D, NN, POOL, NBLOCKS, ENTRIES, MEAN_COUNT = 6, 4, 1024, 8192, 131072, 16
SEED = 20261203
WORKLOAD = "kronmult6_xbatched FP64 d=6 n=4, 131072 entries over 8192 X / 8192 Y blocks"
METRIC = "kronmult GFLOP/s (FP64, xbatched d=6 n=4), chosen form vs plain at <=1e-12 rel err"


def flops_per_entry(d=D, n=NN):
    return 2.0 * d * n ** (d + 1)  # kron_flops, kroncommon.hpp:204-234


def algorithmic_bytes(entries, nblocks, d=D, n=NN):
    """X block + factors + 8 pointers read per entry; each Y block read and
    written once."""
    N = n ** d
    return entries * (N * 8 + d * n * n * 8 + (d + 2) * 8) + nblocks * 2 * N * 8


def make_workload(seed=SEED, entries=ENTRIES, nblocks=NBLOCKS, pool=POOL, d=D, n=NN, ny=None):
    """nblocks X blocks and ny (default nblocks) Y blocks."""
    ny = nblocks if ny is None else ny
    rng = np.random.default_rng(seed)
    counts = rng.geometric(1.0 / MEAN_COUNT, ny).astype(np.int64)
    # adjust to exactly `entries`, keeping every count >= 1
    diff = entries - int(counts.sum())
    while diff != 0:
        idx = rng.integers(0, ny, abs(diff))
        if diff > 0:
            np.add.at(counts, idx, 1)
        else:
            for i in idx:
                if counts[i] > 1:
                    counts[i] -= 1
        diff = entries - int(counts.sum())
    y_idx = np.repeat(np.arange(ny, dtype=np.int32), counts)
    rng.shuffle(y_idx)
    x_idx = rng.integers(0, nblocks, entries, dtype=np.int32)
    a_idx = rng.integers(0, pool, (entries, d), dtype=np.int32)
    N = n ** d
    Apool = rng.standard_normal((d, pool, n, n)) / 2.0
    Xpool = rng.standard_normal((nblocks, N))
    return dict(y_idx=y_idx, x_idx=x_idx, a_idx=a_idx, Apool=Apool, Xpool=Xpool, counts=counts)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def profile_value(key):
    """A per-entry ncu counter of the headline kernel, from the committed
    profiles/kernel_counters.json (each value names the capture it comes
    from), or None."""
    p = os.path.join(ROOT, "profiles", "kernel_counters.json")
    try:
        with open(p) as f:
            v = json.load(f)["xbatched_d6n4_split"][key]
        return float(v)
    except (OSError, ValueError, KeyError, TypeError):
        return None


def profile_traffic():
    """DRAM bytes per entry of the split kernel (one full-size ncu capture)."""
    return profile_value("dram_bytes_per_entry")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        time.sleep(0.2)
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out = ""
        else:
            self.out = ""

    def summary(self):
        rows = [r for r in csv.reader(io.StringIO(self.out)) if len(r) >= 9]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for name, v in zip(names, r[5:9]):
                if v.strip() == "Active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "samples": len(rows), "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------
# CPU baseline (the oracle port of the reference's OpenMP path)
# ---------------------------------------------------------------------------

def cpu_rate(w, entries, reps=1):
    """GFLOP/s of the oracle on the first `entries` entries (best of reps)."""
    from oracle import pyoracle as po

    Y = np.zeros_like(w["Xpool"])
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        po.xbatched_idx(D, NN, w["Apool"], NN, POOL, w["Xpool"], Y, w["y_idx"][:entries],
                        w["x_idx"][:entries], w["a_idx"][:entries])
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    return entries * flops_per_entry() / best / 1e9, best


def cpu_baseline(w, budget_s=20.0):
    from oracle import pyoracle as po

    po.build(ref=False)
    cores = po.max_threads()
    rate0, t0 = cpu_rate(w, 2048)
    entries = int(min(ENTRIES, max(2048, budget_s / 2 / max(t0, 1e-6) * 2048)))
    rate, dt = cpu_rate(w, entries, reps=2)
    return {"value": round(rate, 3), "unit": "GFLOP/s", "cores": cores, "kind": "port",
            "sample": f"first {entries} of the {ENTRIES} entries, best of 2 ({dt:.2f} s each), "
                      f"oracle/kron_oracle.c OpenMP restatement of kronmult_xbatched.hpp"}


def run_reference(args):
    """--impl reference: the reference's CPU algorithm (oracle port; the
    reference's own build is x86-only here and cannot travel) on the host
    cores, same workload and metric."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle import pyoracle as po

    po.build(ref=False)
    w = make_workload()
    cores = po.max_threads()
    _, t_small = cpu_rate(w, 2048)
    per_entry = t_small / 2048
    total_budget = 150.0
    entries = int(min(ENTRIES, max(2048, total_budget / (args.steps + args.warmup) / per_entry)))
    for _ in range(args.warmup):
        cpu_rate(w, entries)
    times = []
    for _ in range(args.steps):
        _, dt = cpu_rate(w, entries)
        times.append(dt)
    t = sum(times) / len(times)
    val = entries * flops_per_entry() / t / 1e9
    line = {
        "metric": METRIC, "value": round(val, 3),
        "unit": "GFLOP/s", "impl": "reference", "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(t * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "entries_per_step": entries},
        "cpu_baseline": {"value": round(val, 3), "unit": "GFLOP/s", "cores": cores, "kind": "port",
                         "sample": f"{entries} of {ENTRIES} entries per step"},
        "e2e": {"value": round(val, 3), "unit": "GFLOP/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def run_ours(args):
    import torch

    import kronmult_gb300 as kmx

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    entries = args.entries
    if world > 1:
        # One batch of world x entries over world x 8192 Y blocks (X pool and
        # factor pool replicated), partitioned by Y-block ownership: each rank
        # runs the entries whose Y blocks it owns, against its own range of Y
        # blocks, with no collective on the data path (weak scaling: about
        # `entries` entries and 8192 Y blocks per rank).
        from kronmult_gb300.shard import plan_by_y_owner

        w = make_workload(seed=SEED, entries=entries * world, ny=NBLOCKS * world)
        shards, ranges = plan_by_y_owner(w["y_idx"], world)
        ids = np.sort(shards[rank])
        y_lo, y_hi = ranges[rank]
        w["y_idx"] = (w["y_idx"][ids] - y_lo).astype(np.int32)
        w["x_idx"] = w["x_idx"][ids]
        w["a_idx"] = w["a_idx"][ids]
        entries = len(ids)
        ny = y_hi - y_lo
    else:
        w = make_workload(seed=SEED, entries=entries)
        ny = NBLOCKS
    N = NN ** D
    dev = torch.device("cuda", local)
    Ad = torch.from_numpy(w["Apool"]).to(dev)
    Xd = torch.from_numpy(w["Xpool"]).to(dev)
    Yd = torch.zeros((ny, N), dtype=torch.float64, device=dev)
    y_idx = torch.from_numpy(w["y_idx"]).to(dev).long()
    x_idx = torch.from_numpy(w["x_idx"]).to(dev).long()
    a_idx = torch.from_numpy(w["a_idx"]).to(dev).long()
    lvl = torch.arange(D, device=dev).long()[None, :]

    def ptrs(A, X, Y):
        pA = ((lvl * POOL + a_idx) * (NN * NN * 8) + A.data_ptr()).reshape(-1).contiguous()
        pX = x_idx * (N * 8) + X.data_ptr()
        pY = y_idx * (N * 8) + Y.data_ptr()
        return pA, pX, pY

    pA, pX, pY = ptrs(Ad, Xd, Yd)
    stream = torch.cuda.current_stream()

    def step(form, Y_ptrs=pY, acc="atomic"):
        kmx.kronmult_xbatched(D, NN, pA, NN, pX, Y_ptrs, None, entries, form=form, accumulate=acc)

    def timed(form, K, W, acc="atomic"):
        for _ in range(W):
            step(form, acc=acc)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(K):
            step(form, acc=acc)
        e1.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        ms = e0.elapsed_time(e1) / K
        if dist:
            t = torch.tensor([ms], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return ms

    # plain FP64 first (untimed warm-up included), then the chosen form under clock sampling
    ms_plain = timed("plain", max(2, args.steps // 2), max(1, args.warmup // 2))
    with ClockSampler(local) as clk:
        ms = timed("auto", args.steps, args.warmup)
    clocks = clk.summary()
    kmx.check_device_status()
    # deterministic sorted-segment accumulation (sort + segment queue inside every call)
    ms_det = timed("auto", args.steps, args.warmup, acc="deterministic")
    kmx.check_device_status()
    # FP64 on the FP16 tensor cores by exact digit products
    ms_dig = timed("digits", args.steps, args.warmup)
    kmx.check_device_status()

    # accuracy: chosen vs plain on a fresh Y, and both vs the oracle on a sample
    Yc = torch.zeros_like(Yd)
    Yp = torch.zeros_like(Yd)
    _, _, pYc = ptrs(Ad, Xd, Yc)
    _, _, pYp = ptrs(Ad, Xd, Yp)
    step("auto", pYc)
    step("plain", pYp)
    torch.cuda.synchronize()
    num = torch.linalg.vector_norm(Yc - Yp, dim=1)
    den = torch.linalg.vector_norm(Yp, dim=1).clamp_min(1e-300)
    err_vs_plain = float((num / den).max().item())
    Yd1 = torch.zeros_like(Yd)
    Yd2 = torch.zeros_like(Yd)
    step("auto", ptrs(Ad, Xd, Yd1)[2], acc="deterministic")
    step("auto", ptrs(Ad, Xd, Yd2)[2], acc="deterministic")
    torch.cuda.synchronize()
    det_bitwise = bool(torch.equal(Yd1, Yd2))
    num = torch.linalg.vector_norm(Yd1 - Yp, dim=1)
    err_det_vs_plain = float((num / den).max().item())
    Yd1.zero_()
    step("digits", ptrs(Ad, Xd, Yd1)[2])
    torch.cuda.synchronize()
    num = torch.linalg.vector_norm(Yd1 - Yp, dim=1)
    err_dig_vs_plain = float((num / den).max().item())
    del Yd1, Yd2

    total_flops = args.entries * flops_per_entry() * world  # every rank's shard together
    value = total_flops / (ms * 1e-3) / 1e9
    value_plain = total_flops / (ms_plain * 1e-3) / 1e9

    # e2e through the C ABI from pinned host buffers.  Every step copies its
    # inputs host->device and its result device->host; steps are pipelined
    # over three device buffer sets and separate input, compute and output
    # streams, so step k's kernel overlaps step k+1's input copies and step
    # k-1's result copy.
    e2e = None
    if not args.no_e2e:
        Ah = torch.from_numpy(w["Apool"]).pin_memory()
        Xh = torch.from_numpy(w["Xpool"]).pin_memory()
        Yh = torch.zeros((ny, N), dtype=torch.float64).pin_memory()
        idx_h = torch.from_numpy(np.concatenate(
            [w["y_idx"], w["x_idx"], w["a_idx"].ravel()]).astype(np.int32)).pin_memory()
        # three buffer sets: step k+1's uploads need not wait for step k-1's
        # download, so slower host links do not stall the kernels
        NB = 3
        Yout = [torch.empty_like(Yh).pin_memory() for _ in range(NB)]
        bufs = [dict(A=torch.empty_like(Ad), X=torch.empty_like(Xd), Y=torch.empty_like(Yd),
                     idx=torch.empty(idx_h.numel(), dtype=torch.int32, device=dev))
                for _ in range(NB)]
        h2d = (Ah.numel() + Xh.numel() + Yh.numel()) * 8 + idx_h.numel() * 4
        d2h = Yh.numel() * 8
        # one upload and one download stream: splitting the copies over four
        # streams each measured slower on GB300 (8.2 against 6.9 ms per step:
        # the concurrent downloads slowed the kernel's step), two slower still
        NCH = 1
        s_in = [torch.cuda.Stream() for _ in range(NCH)]
        s_cmp = torch.cuda.Stream()
        s_out = [torch.cuda.Stream() for _ in range(NCH)]
        ev_out = [[torch.cuda.Event() for _ in range(NCH)] for _ in range(NB)]
        started = [False] * NB
        rows, yrows = Xh.shape[0], Yh.shape[0]
        cuts = [rows * c // NCH for c in range(NCH + 1)]
        ycuts = [yrows * c // NCH for c in range(NCH + 1)]

        cmp_events = []  # (start, end) of each timed step's device work on the compute stream

        def e2e_step(k, timed=False):
            b = k % NB
            B = bufs[b]
            ev_in = []
            for c in range(NCH):
                st = s_in[c]
                if started[b]:  # the previous download from this buffer set is done
                    for ev in ev_out[b]:
                        st.wait_event(ev)
                lo, hi = cuts[c], cuts[c + 1]
                ylo, yhi = ycuts[c], ycuts[c + 1]
                with torch.cuda.stream(st):
                    B["X"][lo:hi].copy_(Xh[lo:hi], non_blocking=True)
                    B["Y"][ylo:yhi].copy_(Yh[ylo:yhi], non_blocking=True)
                    if c == 0:
                        B["A"].copy_(Ah, non_blocking=True)
                        B["idx"].copy_(idx_h, non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(st)
                ev_in.append(ev)
            for ev in ev_in:
                s_cmp.wait_event(ev)
            with torch.cuda.stream(s_cmp):
                if timed:
                    c0 = torch.cuda.Event(enable_timing=True)
                    c0.record(s_cmp)
                idx = B["idx"]
                nb, nyb = B["X"].shape[0], B["Y"].shape[0]
                qA, qX, qY = kmx.xbatched_build(
                    D, B["A"], POOL * NN * NN, NN * NN, POOL, B["X"], N, nb, B["Y"], N, nyb,
                    idx[:entries], idx[entries:2 * entries], idx[2 * entries:], stream=s_cmp)
                kmx.kronmult_xbatched(D, NN, qA, NN, qX, qY, None, entries, stream=s_cmp)
                ev_cmp = torch.cuda.Event(enable_timing=timed)
                ev_cmp.record(s_cmp)
                if timed:
                    cmp_events.append((c0, ev_cmp))
            for c in range(NCH):
                lo, hi = ycuts[c], ycuts[c + 1]
                s_out[c].wait_event(ev_cmp)
                with torch.cuda.stream(s_out[c]):
                    Yout[b][lo:hi].copy_(B["Y"][lo:hi], non_blocking=True)
                    ev_out[b][c].record(s_out[c])
            started[b] = True

        for k in range(NB + 1):
            e2e_step(k)
        torch.cuda.synchronize()
        # host wall clock from an idle pipeline: the first upload and the last
        # download are not overlapped, so average over at least 40 steps
        K2 = max(40, args.steps)
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for k in range(K2):
            e2e_step(k, timed=True)
        torch.cuda.synchronize()
        ms_e2e = (time.perf_counter() - t0) / K2 * 1e3
        if dist:  # the slowest rank's step time
            t = torch.tensor([ms_e2e], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms_e2e = float(t.item())
        ms_e2e_dev = sum(a.elapsed_time(b) for a, b in cmp_events) / len(cmp_events)
        # the last step's result, read back on the host, against the device-resident run
        Ylast = Yout[(K2 - 1) % NB].to(dev)
        e2e_err = float((torch.linalg.vector_norm(Ylast - Yc, dim=1) /
                         torch.linalg.vector_norm(Yc, dim=1).clamp_min(1e-300)).max().item())
        del Ylast
        e2e = {"value": round(total_flops / (ms_e2e * 1e-3) / 1e9, 3), "unit": "GFLOP/s",
               "ms_per_step": round(ms_e2e, 3), "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "rel_err_vs_device_run": e2e_err,
               "device_ms_per_step": round(ms_e2e_dev, 3),
               "timing": f"host wall clock over {K2} steps, each step = H2D of pools and "
                         "index triples + device pointer build + C ABI call + D2H result; "
                         "steps pipelined over three buffer sets, one upload and one download "
                         "stream; device_ms_per_step = the pointer build and kernel alone"}

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0

    peaks, peak_kind = load_peaks()
    L = kmx.lib()
    import ctypes as C

    r64 = C.c_double(0)
    r32 = C.c_double(0)
    L.kmx_probe_fma_rate(1, C.byref(r64))
    L.kmx_probe_fma_rate(0, C.byref(r32))
    fp64_tflops = 2 * r64.value / 1e12
    fp32_tflops = 2 * r32.value / 1e12
    alg_bytes = algorithmic_bytes(entries, ny)  # this rank's launch
    achieved_gbs = alg_bytes / (ms * 1e-3) / 1e9
    tpe = profile_traffic()
    roofline = {"bound": "hbm", "achieved": round(achieved_gbs, 1), "peak": peaks["hbm_gbs"],
                "unit": "GB/s", "frac": round(achieved_gbs / peaks["hbm_gbs"], 4),
                "traffic": (round(tpe * entries) if tpe else None),
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                "algorithmic_bytes_per_launch": int(alg_bytes)}
    t_fp64 = total_flops / world / (fp64_tflops * 1e12)
    t_hbm = alg_bytes / (peaks["hbm_gbs"] * 1e9)
    north = {"definition": "max(flops / FP64 peak, bytes / HBM peak)",
             "fp64_peak_tflops_measured": round(fp64_tflops, 3),
             "fp32_peak_tflops_measured": round(fp32_tflops, 2),
             "t_fp64_ms": round(t_fp64 * 1e3, 3), "t_hbm_ms": round(t_hbm * 1e3, 3),
             "bound": "fp64" if t_fp64 > t_hbm else "hbm",
             "frac_chosen": round(max(t_fp64, t_hbm) / (ms * 1e-3), 3),
             "frac_plain": round(max(t_fp64, t_hbm) / (ms_plain * 1e-3), 3)}

    # the binding resource of the chosen form: FP32 instruction issue.  Warp-
    # instructions per entry from the committed ncu summary of the kernel;
    # peak = 4 schedulers x SMs x the SM clock sampled in the timed region.
    issue = None
    ipe = profile_value("warp_instructions_per_entry")
    sm_mhz = (clocks or {}).get("sm_mhz")
    if ipe and sm_mhz:
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        ach = ipe * entries / (ms * 1e-3)
        peak = 4.0 * sms * sm_mhz * 1e6
        issue = {"bound": "fp32 issue", "unit": "warp-instructions/s",
                 "instructions_per_entry": ipe, "achieved": float(f"{ach:.4g}"),
                 "peak": float(f"{peak:.4g}"), "frac": round(ach / peak, 3),
                 "source": "ncu smsp__inst_executed.sum of the kernel "
                           "(profiles/kernel_counters.json)"}

    cpu = None if args.no_cpu_baseline else cpu_baseline(w)
    line = {
        "metric": METRIC,
        "value": round(value, 3), "unit": "GFLOP/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "d": D, "n": NN, "entries": args.entries * world,
                   "x_blocks": NBLOCKS, "y_blocks": NBLOCKS * world, "factor_pool": POOL,
                   "accumulate": "atomic", "form_chosen": "split (double-float)",
                   "l2": "inputs larger than L2 (256 MiB X and Y pools), no flush",
                   "seed": SEED,
                   "parallelism": ("one GPU" if world == 1 else
                                   f"Y-block ownership shards of one batch x{world} "
                                   "(no data-path collective)")},
        "plain": {"value": round(value_plain, 3), "unit": "GFLOP/s", "ms_per_step": round(ms_plain, 4)},
        "deterministic": {"value": round(total_flops / (ms_det * 1e-3) / 1e9, 3), "unit": "GFLOP/s",
                          "ms_per_step": round(ms_det, 4), "bitwise_repeatable": det_bitwise,
                          "rel_err_vs_plain_atomic": err_det_vs_plain,
                          "note": "device sort by Y block + segment work queue, per call"},
        "digits": {"value": round(total_flops / (ms_dig * 1e-3) / 1e9, 3), "unit": "GFLOP/s",
                   "ms_per_step": round(ms_dig, 4), "rel_err_vs_plain": err_dig_vs_plain,
                   "note": "FP64 as base-2^9 digits, exact FP16 tensor-core products "
                           "(mma.sync), double-float pass for handed-back entries"},
        "rel_err_chosen_vs_plain": err_vs_plain,
        "roofline": roofline, "fp64_roofline": north, "issue_roofline": issue,
        "gpu_launches": args.steps, "gpu_launches_deterministic_per_step": 8, "clocks": clocks, "e2e": e2e, "cpu_baseline": cpu,
    }
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# Secondary workloads (one JSON line each; the default run is the headline).
# ---------------------------------------------------------------------------

def _selected(args, tag):
    """Whether the case with this tag runs (--cases; empty: every case)."""
    want = [c for c in getattr(args, "cases", "").split(",") if c]
    return not want or tag in want


def _events_time(torch, fn, K, W):
    for _ in range(W):
        fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(K):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / K


def _blockwise_err(torch, y, yref, rows):
    """max over blocks of the normwise relative error (blocks given as slices)."""
    worst = 0.0
    for a, b in rows:
        r = yref[a:b]
        s = r.abs().max().clamp_min(1e-300)
        num = torch.linalg.vector_norm((y[a:b] - r) / s)
        den = torch.linalg.vector_norm(r / s).clamp_min(1e-300)
        worst = max(worst, float(num / den))
    return worst


def run_mixed(args):
    """65536 instances, d ~ U{1..6}, n ~ U{2,3,4,5,6,8}, n^d <= 262144, own
    factors, X and Y ~ U[-1,1]; one kronmult_mixed call per step, a 100-call
    sequence captured as a CUDA graph and replayed."""
    import torch

    import kronmult_gb300 as kmx

    rng = np.random.default_rng(SEED + 3)
    count = args.entries if args.entries != ENTRIES else 65536
    d = rng.integers(1, 7, count)
    n = rng.choice(np.array([2, 3, 4, 5, 6, 8]), count)
    bad = n.astype(np.float64) ** d > 262144
    while bad.any():
        d[bad] = rng.integers(1, 7, bad.sum())
        n[bad] = rng.choice(np.array([2, 3, 4, 5, 6, 8]), bad.sum())
        bad = n.astype(np.float64) ** d > 262144
    N = n.astype(np.int64) ** d
    xoff = np.concatenate([[0], np.cumsum(N)[:-1]])
    nf = d.astype(np.int64)
    a_off = np.concatenate([[0], np.cumsum(nf)[:-1]])
    fsz = np.repeat(n.astype(np.int64) ** 2, nf)
    foff = np.concatenate([[0], np.cumsum(fsz)[:-1]])
    dev = torch.device("cuda")
    g = torch.Generator(device=dev).manual_seed(SEED)
    X = torch.rand(int(N.sum()), dtype=torch.float64, device=dev, generator=g) * 2 - 1
    Y = torch.rand(int(N.sum()), dtype=torch.float64, device=dev, generator=g) * 2 - 1
    F = torch.rand(int(fsz.sum()), dtype=torch.float64, device=dev, generator=g) * 2 - 1
    dims = torch.from_numpy(np.stack([d, n], 1).astype(np.int32)).to(dev)
    pA = torch.from_numpy(foff).to(dev) * 8 + F.data_ptr()
    pX = torch.from_numpy(xoff).to(dev) * 8 + X.data_ptr()
    pY = torch.from_numpy(xoff).to(dev) * 8 + Y.data_ptr()
    aoff_d = torch.from_numpy(a_off).to(dev)
    classes = sorted({(int(a), int(b)) for a, b in zip(d, n)}, key=lambda c: -(c[0] * c[1] ** (c[0] + 1)))
    W = torch.empty(2 * 262144 * 512, dtype=torch.float64, device=dev)
    flops = float((2.0 * d * n.astype(np.float64) ** (d + 1)).sum())
    res = {}
    # auto: one tuned launch per class (the default); persistent: one launch
    # over every class fed by a device work queue (generic double-float kernel)
    for name, form, engine in (("auto", "auto", None), ("plain", "plain", None),
                               ("persistent", "auto", "persistent")):
        call = lambda: kmx.kronmult_mixed(dims, pA, aoff_d, pX, pY, classes, W, form=form,
                                          engine=engine)
        ms_eager = _events_time(torch, call, max(2, args.steps // 3), 2)
        # 100-call sequence as one CUDA graph
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            with torch.cuda.graph(graph, stream=s):
                for _ in range(100):
                    kmx.kronmult_mixed(dims, pA, aoff_d, pX, pY, classes, W, form=form,
                                       engine=engine, stream=s)
        torch.cuda.current_stream().wait_stream(s)
        ms_graph = _events_time(torch, graph.replay, 2, 1) / 100
        res[name] = {"gflops_graph": round(flops / (ms_graph * 1e-3) / 1e9, 2),
                     "ms_per_call_graph": round(ms_graph, 4),
                     "gflops_eager": round(flops / (ms_eager * 1e-3) / 1e9, 2),
                     "ms_per_call_eager": round(ms_eager, 4)}
    # accuracy of the chosen form against plain FP64 on fresh Y
    Yc = torch.zeros_like(Y)
    Yp = torch.zeros_like(Y)
    kmx.kronmult_mixed(dims, pA, aoff_d, pX, torch.from_numpy(xoff).to(dev) * 8 + Yc.data_ptr(),
                       classes, W)
    kmx.kronmult_mixed(dims, pA, aoff_d, pX, torch.from_numpy(xoff).to(dev) * 8 + Yp.data_ptr(),
                       classes, W, form="plain")
    torch.cuda.synchronize()
    kmx.check_device_status()
    pick = rng.choice(count, 512, replace=False)
    err = _blockwise_err(torch, Yc, Yp, [(int(xoff[i]), int(xoff[i] + N[i])) for i in pick])
    print(json.dumps({"metric": "kronmult GFLOP/s, mixed-shape batch (one call), FP64",
                      "value": res["auto"]["gflops_graph"], "unit": "GFLOP/s", "n_gpus": 1,
                      "workload": "mixed", "instances": count, "classes": len(classes),
                      "total_gflop_per_call": round(flops / 1e9, 2),
                      "chosen": res["auto"], "plain": res["plain"],
                      "persistent_one_launch": res["persistent"],
                      "rel_err_chosen_vs_plain_512_instances": err, "data": "synthetic"}))


def run_grad(args):
    """Fused forward+backward against forward alone: d=6 n=5 batch 1024 and
    d=3 n=8 batch 4096 (FP64)."""
    import torch

    import kronmult_gb300 as kmx
    from kronmult_gb300.autograd import _grad_call, grad_workspace

    out = []
    for d, n, batch in ((6, 5, 1024), (3, 8, 4096)):
        if not _selected(args, f"{d}-{n}"):
            continue
        N = n ** d
        g = torch.Generator(device="cuda").manual_seed(SEED + d)
        A = torch.randn((batch, d, n, n), dtype=torch.float64, device="cuda", generator=g) / n ** 0.5
        X = torch.randn((batch, N), dtype=torch.float64, device="cuda", generator=g)
        G = torch.randn((batch, N), dtype=torch.float64, device="cuda", generator=g)
        Y = torch.zeros_like(X)
        dX = torch.zeros_like(X)
        dA = torch.zeros_like(A)
        W = grad_workspace(d, n, batch)
        fwd = {}
        for form in ("plain", "split"):
            fwd[form] = _events_time(torch, lambda: kmx.kronmult_batched(d, n, A, X, Y, None, batch, form=form),
                                     args.steps, 3)
        both = {}
        res = {}
        for form in ("plain", "split"):
            both[form] = _events_time(
                torch, lambda: _grad_call(d, n, A, X, G, Y, dX, dA, W, form), args.steps, 3)
            Y.zero_()
            dX.zero_()
            dA.zero_()
            _grad_call(d, n, A, X, G, Y, dX, dA, W, form)
            res[form] = (Y.clone(), dX.clone(), dA.clone())
        torch.cuda.synchronize()

        def rel(a, b):
            a, b = a.reshape(a.shape[0], -1), b.reshape(b.shape[0], -1)
            return float((torch.linalg.vector_norm(a - b, dim=1) /
                          torch.linalg.vector_norm(b, dim=1).clamp_min(1e-300)).max())

        err = max(rel(x, y) for x, y in zip(res["split"], res["plain"]))
        fl = batch * 2.0 * d * n ** (d + 1)
        out.append({"d": d, "n": n, "batch": batch, "fwd_plain_ms": round(fwd["plain"], 4),
                    "fwd_split_ms": round(fwd["split"], 4),
                    "fwd_bwd_plain_ms": round(both["plain"], 4),
                    "fwd_bwd_split_ms": round(both["split"], 4),
                    "ratio_plain_fwd_bwd_vs_plain_fwd": round(both["plain"] / fwd["plain"], 3),
                    "ratio_split_fwd_bwd_vs_plain_fwd": round(both["split"] / fwd["plain"], 3),
                    "ratio_split_fwd_bwd_vs_split_fwd": round(both["split"] / fwd["split"], 3),
                    "rel_err_split_vs_plain_fwd_bwd": err,
                    "fwd_plain_gflops": round(fl / (fwd["plain"] * 1e-3) / 1e9, 1)})
        del res
    kmx.check_device_status()
    print(json.dumps({"metric": "fused forward+backward time / forward time, FP64 data, both in "
                                f"the default form (double-float), d={out[0]['d']} "
                                f"n={out[0]['n']} batch {out[0]['batch']}",
                      "value": out[0]["ratio_split_fwd_bwd_vs_split_fwd"], "unit": "ratio",
                      "higher_is_better": False, "workload": "grad", "cases": out,
                      "data": "synthetic"}))


def run_precision(args):
    """xbatched d=4 n=8 and d=3 n=16, 262144 entries over 16384 X/Y blocks,
    geometric(16) per-Y counts, factors N(0,1)/sqrt(n), X N(0,1): FP64 forms,
    FP32- and BF16-stored forms with FP64 Y; errors against plain FP64."""
    import torch

    import kronmult_gb300 as kmx

    entries = args.entries if args.entries != ENTRIES else 262144
    nblocks = 16384
    out = []
    for d, n in ((4, 8), (3, 16)):
        N = n ** d
        rng = np.random.default_rng(SEED + 11 * n)
        counts = rng.geometric(1.0 / 16, nblocks)
        y_idx = np.repeat(np.arange(nblocks), counts)[:entries]
        if len(y_idx) < entries:
            y_idx = np.concatenate([y_idx, rng.integers(0, nblocks, entries - len(y_idx))])
        rng.shuffle(y_idx)
        x_idx = rng.integers(0, nblocks, entries)
        pool = 1024
        a_idx = rng.integers(0, pool, (entries, d))
        g = torch.Generator(device="cuda").manual_seed(SEED + n)
        A64 = torch.randn((d, pool, n, n), dtype=torch.float64, device="cuda", generator=g) / n ** 0.5
        X64 = torch.randn((nblocks, N), dtype=torch.float64, device="cuda", generator=g)
        lvl = torch.arange(d, device="cuda")[None, :]
        ai = torch.from_numpy(a_idx).cuda()
        xi = torch.from_numpy(x_idx).cuda()
        yi = torch.from_numpy(y_idx).cuda()

        def ptrs(A, X, Y):
            e = A.element_size()
            return (((lvl * pool + ai) * (n * n * e) + A.data_ptr()).reshape(-1).contiguous(),
                    xi * (N * X.element_size()) + X.data_ptr(), yi * (N * 8) + Y.data_ptr())

        fl = entries * 2.0 * d * n ** (d + 1)
        res = {}
        Yref = torch.zeros((nblocks, N), dtype=torch.float64, device="cuda")
        pA, pX, pY = ptrs(A64, X64, Yref)
        kmx.kronmult_xbatched(d, n, pA, n, pX, pY, None, entries, form="plain")
        Yacc = torch.zeros_like(Yref)
        for name in ("plain", "split", "f32", "bf16", "f32_tf32x3", "bf16_tf32x3",
                     "f32_tf32x3_det"):
            if name in ("plain", "split"):
                A, X = A64, X64
            else:
                tdt = torch.float32 if name.startswith("f32") else torch.bfloat16
                A, X = A64.to(tdt), X64.to(tdt)
            pA, pX, pY = ptrs(A, X, Yacc)
            if name in ("plain", "split"):
                call = lambda: kmx.kronmult_xbatched(d, n, pA, n, pX, pY, None, entries, form=name)
            else:
                ind = name.split("_")[0]
                fm = "tf32x3" if "tf32x3" in name else None
                acc = "deterministic" if name.endswith("_det") else None
                call = lambda: kmx.kronmult_xbatched_wide(d, n, pA, n, pX, pY, entries,
                                                          in_dtype=ind, form=fm, accumulate=acc)
            ms = _events_time(torch, call, max(3, args.steps // 2), 2)
            Yacc.zero_()
            call()
            torch.cuda.synchronize()
            s = Yref.abs().amax(dim=1, keepdim=True).clamp_min(1e-300)
            err = float((torch.linalg.vector_norm((Yacc - Yref) / s, dim=1) /
                         torch.linalg.vector_norm(Yref / s, dim=1).clamp_min(1e-300)).max())
            res[name] = {"gflops": round(fl / (ms * 1e-3) / 1e9, 1), "ms": round(ms, 4),
                         "rel_err_vs_fp64_gpu": err}
        # the FP32 entry point proper: FP32 X, factors and Y (FP32 atomics)
        A32, X32 = A64.float(), X64.float()
        Y32 = torch.zeros((nblocks, N), dtype=torch.float32, device="cuda")
        pA32 = ((lvl * pool + ai) * (n * n * 4) + A32.data_ptr()).reshape(-1).contiguous()
        pX32 = xi * (N * 4) + X32.data_ptr()
        pY32 = yi * (N * 4) + Y32.data_ptr()
        # f32_y32: the default FP32 form (each dot product rounded once, the
        # reference's float semantics); _fma: FP32 fused multiply-add
        for name, fm in (("f32_y32", None), ("f32_y32_fma", "plain"),
                         ("f32_y32_tf32x3", "tf32x3")):
            call = lambda: kmx.kronmult_xbatched(d, n, pA32, n, pX32, pY32, None, entries,
                                                 dtype=torch.float32, form=fm)
            ms = _events_time(torch, call, max(3, args.steps // 2), 2)
            Y32.zero_()
            call()
            torch.cuda.synchronize()
            Yd = Y32.double()
            s = Yref.abs().amax(dim=1, keepdim=True).clamp_min(1e-300)
            err = float((torch.linalg.vector_norm((Yd - Yref) / s, dim=1) /
                         torch.linalg.vector_norm(Yref / s, dim=1).clamp_min(1e-300)).max())
            res[name] = {"gflops": round(fl / (ms * 1e-3) / 1e9, 1), "ms": round(ms, 4),
                         "rel_err_vs_fp64_gpu": err}
        del A32, X32, Y32
        out.append({"d": d, "n": n, "entries": entries, "forms": res,
                    "f32_speedup_vs_fp64_plain": round(res["plain"]["ms"] / res["f32"]["ms"], 2),
                    "f32_speedup_vs_fp64_chosen": round(res["split"]["ms"] / res["f32"]["ms"], 2),
                    "tf32x3_speedup_vs_fp64_chosen": round(
                        res["split"]["ms"] / res["f32_tf32x3"]["ms"], 2),
                    "tf32x3_speedup_vs_f32_fma": round(res["f32"]["ms"] / res["f32_tf32x3"]["ms"], 2),
                    "tf32x3_det_speedup_vs_fp64_chosen": round(
                        res["split"]["ms"] / res["f32_tf32x3_det"]["ms"], 2)})
    kmx.check_device_status()
    print(json.dumps({"metric": "kronmult precision forms, xbatched (GFLOP/s and error vs FP64)",
                      "value": out[0]["f32_speedup_vs_fp64_chosen"], "unit": "ratio",
                      "workload": "precision", "cases": out, "data": "synthetic"}))


def run_kgemm(args):
    """kgemm_{nn,nt}_batched at the reference test's performance shapes
    (test_kgemm_nn_batched.cpp:541-553: mm = kk = n, nn = n^5) and at the
    tall-narrow transpose of the same contraction (kgemm_nt with mm = n^5,
    nn = kk = n), 16384 entries each so that C is larger than L2; alpha 1.3,
    beta 1.2.  GFLOP/s and the roofline max(flops / FP64-or-FP32 FMA peak,
    bytes / HBM peak), bytes = A + B + C read + C written."""
    import ctypes as C

    import torch

    import kronmult_gb300 as kmx

    L = kmx.lib()
    r64, r32 = C.c_double(0), C.c_double(0)
    L.kmx_probe_fma_rate(1, C.byref(r64))
    L.kmx_probe_fma_rate(0, C.byref(r32))
    hbm = float(load_peaks()[0]["hbm_gbs"]) * 1e9
    batch = 16384
    out = []
    for trans, dt in (("nn", torch.float64), ("nt", torch.float64), ("nn", torch.float32)):
        for n in (2, 3, 4, 5, 6):
            if not _selected(args, f"{trans}-{'f64' if dt == torch.float64 else 'f32'}-{n}"):
                continue
            big = n ** 5
            mm, nn, kk = (n, big, n) if trans == "nn" else (big, n, n)
            esz = 8 if dt == torch.float64 else 4
            A = torch.randn(batch * mm * kk, dtype=dt, device="cuda")
            Bm = torch.randn(batch * kk * nn, dtype=dt, device="cuda")
            Cm = torch.randn(batch * mm * nn, dtype=dt, device="cuda")
            pA = kmx.pointer_array(A, torch.arange(batch, device="cuda") * (mm * kk))
            pB = kmx.pointer_array(Bm, torch.arange(batch, device="cuda") * (kk * nn))
            pC = kmx.pointer_array(Cm, torch.arange(batch, device="cuda") * (mm * nn))
            ldA = torch.full((batch,), mm, dtype=torch.int32, device="cuda")
            ldB = torch.full((batch,), kk if trans == "nn" else nn, dtype=torch.int32, device="cuda")
            fn = kmx.kgemm_nn_batched if trans == "nn" else kmx.kgemm_nt_batched
            call = lambda: fn(mm, nn, kk, 1.3, pA, ldA, pB, ldB, 1.2, pC, ldA, batch, dtype=dt)
            ms = _events_time(torch, call, max(3, args.steps), 3)
            flops = 2.0 * mm * nn * kk * batch
            nbytes = float(esz) * batch * (mm * kk + kk * nn + 2 * mm * nn)
            peak = (r64.value if dt == torch.float64 else r32.value) * 2
            t_roof = max(flops / peak, nbytes / hbm)
            out.append({"trans": trans, "dtype": "f64" if dt == torch.float64 else "f32",
                        "mm": mm, "nn": nn, "kk": kk, "batch": batch, "ms": round(ms, 4),
                        "gflops": round(flops / (ms * 1e-3) / 1e9, 1),
                        "gbs": round(nbytes / (ms * 1e-3) / 1e9, 1),
                        "bound": "fma" if flops / peak > nbytes / hbm else "hbm",
                        "roofline_frac": round(t_roof / (ms * 1e-3), 3)})
            del A, Bm, Cm
    kmx.check_device_status()
    fr = [c["roofline_frac"] for c in out]
    print(json.dumps({"metric": "kgemm batched GFLOP/s and roofline fraction",
                      "value": round(float(np.exp(np.mean(np.log(fr)))), 3),
                      "unit": "geomean roofline fraction", "workload": "kgemm",
                      "fp64_fma_per_s": r64.value, "fp32_fma_per_s": r32.value,
                      "hbm_gbs": hbm / 1e9, "cases": out, "data": "synthetic"}))


def run_big(args):
    """Entries beyond one SM: batched FP64 d=6 n=8 (2 MB blocks, 256 entries),
    d=5 n=8 (256 KB, 2048), d=6 n=7 (0.9 MB, 512) and d=6 n=6 (0.37 MB, 1024),
    N(0,1)/sqrt(n) factors, N(0,1) X: split and plain forms on the per-mode
    kernels with the intermediate in the caller's workspace, and the split
    form without a workspace (thread-block cluster kernels)."""
    import torch

    import kronmult_gb300 as kmx

    out = []
    for d, n, batch in ((6, 8, 256), (5, 8, 2048), (6, 7, 512), (6, 6, 1024)):
        N = n ** d
        g = torch.Generator(device="cuda").manual_seed(SEED + d)
        A = torch.randn((batch, d, n, n), dtype=torch.float64, device="cuda", generator=g) / n ** 0.5
        X = torch.randn((batch, N), dtype=torch.float64, device="cuda", generator=g)
        Y = torch.zeros_like(X)
        W = torch.zeros_like(X)
        fl = batch * 2.0 * d * n ** (d + 1)
        res = {}
        for name, kw, ws in (("split", dict(form="split"), W), ("plain", dict(form="plain"), W),
                             ("split_cluster_no_workspace", dict(form="split"), None)):
            call = lambda: kmx.kronmult_batched(d, n, A, X, Y, ws, batch, **kw)
            ms = _events_time(torch, call, max(3, args.steps // 2), 2)
            res[name] = {"gflops": round(fl / (ms * 1e-3) / 1e9, 1), "ms": round(ms, 3)}
        Yr = torch.zeros_like(X)
        kmx.kronmult_batched(d, n, A, X, Yr, W, batch, form="plain")
        Y.zero_()
        kmx.kronmult_batched(d, n, A, X, Y, W, batch, form="split")
        torch.cuda.synchronize()
        err = float((torch.linalg.vector_norm(Y - Yr, dim=1) /
                     torch.linalg.vector_norm(Yr, dim=1)).max())
        out.append({"d": d, "n": n, "batch": batch, "forms": res, "rel_err_split_vs_plain": err})
        del A, X, Y, W, Yr
    kmx.check_device_status()
    print(json.dumps({"metric": "kronmult GFLOP/s, entries beyond one SM (FP64)",
                      "value": out[0]["forms"]["split"]["gflops"], "unit": "GFLOP/s",
                      "workload": "big", "cases": out, "data": "synthetic"}))


def run_small(args):
    """Small entries (the small-entry kernels' shapes): batched d=1 n=2, 4, 8,
    d=2 n=4, 8, d=3 n=4, about 256 MiB of X per call, N(0,1)/2 factors,
    N(0,1) X; FP64 plain and double-float, FP32 fused multiply-add; each with
    the fraction of HBM its algorithmic bytes ((3N + d n^2) x element size per
    entry) reach, and for FP64 plain the fraction of the FP64-pipe ceiling
    max(flops / FP64 peak, bytes / HBM peak)."""
    import ctypes as C

    import torch

    import kronmult_gb300 as kmx

    peaks, peak_kind = load_peaks()
    hbm = peaks["hbm_gbs"] * 1e9
    r64 = C.c_double(0)
    kmx.lib().kmx_probe_fma_rate(1, C.byref(r64))
    fp64 = 2 * r64.value
    out = []
    for d, n in ((1, 2), (1, 4), (1, 8), (2, 4), (2, 8), (3, 4)):
        N = n ** d
        for form in ("plain", "split", "f32"):
            if not _selected(args, f"{d}-{n}-{form}"):
                continue
            dt = torch.float32 if form == "f32" else torch.float64
            esz = 4 if form == "f32" else 8
            batch = (256 << 20) // (N * esz)
            g = torch.Generator(device="cuda").manual_seed(SEED + 10 * d + n)
            A = torch.randn((batch, d, n, n), dtype=dt, device="cuda", generator=g) / 2
            X = torch.randn((batch, N), dtype=dt, device="cuda", generator=g)
            Y = torch.zeros_like(X)
            f = "plain" if form == "f32" else form
            call = lambda: kmx.kronmult_batched(d, n, A, X, Y, None, batch, form=f)
            ms = _events_time(torch, call, max(3, args.steps // 2), 2)
            fl = batch * 2.0 * d * n ** (d + 1)
            by = batch * (3 * N + d * n * n) * esz
            row = {"d": d, "n": n, "form": form, "batch": batch,
                   "gflops": round(fl / (ms * 1e-3) / 1e9, 1), "ms": round(ms, 4),
                   "hbm_frac": round(by / (ms * 1e-3) / hbm, 3)}
            if form == "plain":
                ceil = max(fl / fp64, by / hbm)
                row["fp64_ceiling_frac"] = round(ceil / (ms * 1e-3), 3)
            out.append(row)
            del A, X, Y
    kmx.check_device_status()
    if not out:
        raise SystemExit("--cases selected no small-entry case (tags: d-n-form)")
    print(json.dumps({"metric": "HBM fraction of small entries (batched, tuned engine)",
                      "value": out[0]["hbm_frac"], "unit": "fraction of measured HBM",
                      "workload": "small", "hbm_peak_gbs": peaks["hbm_gbs"],
                      "hbm_peak_source": peak_kind, "fp64_peak_tflops_measured": round(fp64 / 1e12, 3),
                      "cases": out, "data": "synthetic"}))


def run_rect(args):
    """Shapes without a specialised kernel: rectangular factors through the
    vbatched entry point (ld = m, one X and Y block per entry) and square n
    outside {2..8, 16}; N(0,1)/sqrt(n) factors, N(0,1) X.  Split and plain
    forms on the generic per-mode kernels, and the form the library picks."""
    import torch

    import kronmult_gb300 as kmx

    cases = [
        ([4, 3, 4, 3, 4, 3], [3, 4, 3, 4, 3, 4], 65536),
        ([10, 12, 10], [12, 10, 12], 65536),
        ([32, 24], [24, 32], 65536),
        ([10] * 4, [10] * 4, 8192),
        ([12] * 3, [12] * 3, 16384),
    ]
    # beyond shared memory (25088-element blocks): intermediates in the workspace
    big = [([8, 7, 8, 7, 8], [7, 8, 7, 8, 8], 2048)]
    out = []
    for m, n, batch in cases + big:
        d = len(m)
        Nx, Ny = int(np.prod(n)), int(np.prod(m))
        g = torch.Generator(device="cuda").manual_seed(SEED + d)
        fsz = [m[l] * n[l] for l in range(d)]
        A = torch.randn(batch * sum(fsz), dtype=torch.float64, device="cuda", generator=g)
        A /= float(np.mean(n)) ** 0.5
        X = torch.randn((batch, Nx), dtype=torch.float64, device="cuda", generator=g)
        Y = torch.zeros((batch, Ny), dtype=torch.float64, device="cuda")
        offs = (np.arange(batch)[:, None] * sum(fsz) + np.cumsum([0] + fsz[:-1])[None, :]).ravel()
        pA = kmx.pointer_array(A, offs)
        pX = kmx.pointer_array(X, np.arange(batch) * Nx)
        pY = kmx.pointer_array(Y, np.arange(batch) * Ny)
        fl = batch * kmx.kron_flops(d, m, n)
        W = None
        if (m, n, batch) in big:
            sxw = max([Nx] + [int(np.prod(m[:k])) * int(np.prod(n[k:])) for k in range(1, d + 1)])
            W = torch.empty(2 * sxw * 512, dtype=torch.float64, device="cuda")  # 512 slots
        res = {}
        for name in ("split", "plain", "auto"):
            call = lambda: kmx.kronmult_vbatched(d, m, n, pA, pX, pY, W, None, batch, form=name)
            ms = _events_time(torch, call, max(3, args.steps // 2), 2)
            res[name] = {"gflops": round(fl / (ms * 1e-3) / 1e9, 1), "ms": round(ms, 3)}
        Yr = torch.zeros_like(Y)
        pYr = kmx.pointer_array(Yr, np.arange(batch) * Ny)
        kmx.kronmult_vbatched(d, m, n, pA, pX, pYr, W, None, batch, form="plain")
        Y.zero_()
        kmx.kronmult_vbatched(d, m, n, pA, pX, pY, W, None, batch, form="split")
        torch.cuda.synchronize()
        err = float((torch.linalg.vector_norm(Y - Yr, dim=1) /
                     torch.linalg.vector_norm(Yr, dim=1)).max())
        out.append({"d": d, "m": m, "n": n, "batch": batch, "forms": res,
                    "rel_err_split_vs_plain": err})
        del A, X, Y, Yr, pA, pX, pY, pYr, W
    # the five on-chip shapes mixed in one call (kmx_kronmult_vmixed), against
    # one vbatched call per shape over the same instances
    classes = [(m, n) for m, n, _ in cases]
    count = 40000
    rng = np.random.default_rng(SEED)
    cls = rng.integers(0, len(classes), count).astype(np.int32)
    fl = 0.0
    aoff, a_first, xoff, yoff = [], [], [], []
    na = nx = ny = 0
    for i in range(count):
        m, n = classes[cls[i]]
        a_first.append(len(aoff))
        for l in range(len(m)):
            aoff.append(na)
            na += m[l] * n[l]
        xoff.append(nx)
        yoff.append(ny)
        nx += int(np.prod(n))
        ny += int(np.prod(m))
    for c, (m, n) in enumerate(classes):
        fl += float((cls == c).sum()) * kmx.kron_flops(len(m), m, n)
    g = torch.Generator(device="cuda").manual_seed(SEED)
    A = torch.randn(na, dtype=torch.float64, device="cuda", generator=g) / 3.0
    X = torch.randn(nx, dtype=torch.float64, device="cuda", generator=g)
    Y = torch.zeros(ny, dtype=torch.float64, device="cuda")
    pA = kmx.pointer_array(A, aoff)
    pX = kmx.pointer_array(X, xoff)
    pY = kmx.pointer_array(Y, yoff)
    a_off = torch.tensor(a_first, dtype=torch.int64, device="cuda")
    dcls = torch.from_numpy(cls).cuda()
    per = []
    for c, (m, n) in enumerate(classes):
        idx = np.nonzero(cls == c)[0]
        per.append((len(m), m, n, len(idx),
                    kmx.pointer_array(A, [aoff[a_first[i] + l] for i in idx for l in range(len(m))]),
                    kmx.pointer_array(X, [xoff[i] for i in idx]),
                    kmx.pointer_array(Y, [yoff[i] for i in idx])))
    one = lambda: kmx.kronmult_vmixed(dcls, pA, a_off, pX, pY, classes)  # noqa: E731
    # one persistent launch over every class (device work queue)
    pers = lambda: kmx.kronmult_vmixed(dcls, pA, a_off, pX, pY, classes,  # noqa: E731
                                       engine="persistent")

    def separate():
        for d, m, n, b, qa, qx, qy in per:
            kmx.kronmult_vbatched(d, m, n, qa, qx, qy, None, 0, b)

    ms_one = _events_time(torch, one, max(3, args.steps // 2), 2)
    ms_sep = _events_time(torch, separate, max(3, args.steps // 2), 2)
    ms_pers = _events_time(torch, pers, max(3, args.steps // 2), 2)
    Y.zero_()
    pers()
    Yp = Y.clone()
    Y.zero_()
    one()
    Y1 = Y.clone()
    Y.zero_()
    separate()
    torch.cuda.synchronize()
    mixed = {"instances": count, "classes": len(classes),
             "one_call": {"gflops": round(fl / (ms_one * 1e-3) / 1e9, 1), "ms": round(ms_one, 3)},
             "per_shape_calls": {"gflops": round(fl / (ms_sep * 1e-3) / 1e9, 1),
                                 "ms": round(ms_sep, 3)},
             "persistent_one_launch": {"gflops": round(fl / (ms_pers * 1e-3) / 1e9, 1),
                                       "ms": round(ms_pers, 3)},
             "rel_err_one_vs_per_shape": float((Y1 - Y).norm() / Y.norm()),
             "rel_err_persistent_vs_per_shape": float((Yp - Y).norm() / Y.norm())}
    del A, X, Y, Y1, Yp, pA, pX, pY, per
    kmx.check_device_status()
    print(json.dumps({"metric": "kronmult GFLOP/s, shapes without a specialised kernel (FP64)",
                      "value": out[0]["forms"]["auto"]["gflops"], "unit": "GFLOP/s",
                      "workload": "rect", "cases": out, "mixed_one_call": mixed,
                      "data": "synthetic"}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--entries", type=int, default=ENTRIES)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cases", default="",
                    help="comma-separated case tags to run (grad: d-n, e.g. 3-8; kgemm: "
                         "trans-dtype-n, e.g. nn-f32-4; small: d-n-form, e.g. 2-8-split); "
                         "default: every case")
    ap.add_argument("--workload",
                    choices=["xbatched", "mixed", "grad", "precision", "kgemm", "big", "rect",
                             "small"],
                    default="xbatched")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "mixed":
        return run_mixed(args)
    if args.workload == "grad":
        return run_grad(args)
    if args.workload == "precision":
        return run_precision(args)
    if args.workload == "kgemm":
        return run_kgemm(args)
    if args.workload == "big":
        return run_big(args)
    if args.workload == "rect":
        return run_rect(args)
    if args.workload == "small":
        return run_small(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
