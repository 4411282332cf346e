#!/usr/bin/env python3
"""Benchmark of the GB300 word-based motif extraction (MoTeX hot path).

Metric: GCUPS = DP cell updates the reference computes (sum over non-skipped
ordered sequence pairs of m_i * n_j) per second.  One step = one whole-set
extraction (pack, factor dedup, all-factors x all-texts DP, quorum filter,
first-occurrence compaction) of the workload.

* value: steps on input already resident in HBM (motex_gpu_execute), device
  time from CUDA events on the engine's stream; L2 is flushed (256 MiB
  write) before every timed step.
* e2e:   the same metric through the public C ABI call motex_gpu_run with
  host buffers: host->device copy of the sequences, the extraction and the
  device->host copy of the motif list are inside the timed region.
* roofline: the factor-search DP kernel against the measured int32 issue
  peak (an add-chain probe over all pipes, run in the same process; no
  vendor figure exists for it).  The algorithmic count is 6 (Hamming) or
  17 (edit distance) integer operations per cell; packed kernels execute
  fewer per cell, so the fraction can pass 1.
* cpu_baseline: the CPU restatement of the reference path (oracle port,
  OpenMP over all host cores) on a bounded sample of the same workload.

--impl reference times that CPU implementation alone (the reference's own
libFLASM build is x86-64 only and its sources are not on the GPU host).

Extra sections of the default line: batched_vs_plain (uneven protein batch:
the whole set in one persistent launch vs the same job's static launch; the
set cut into uneven jobs, one batch call vs one motex_gpu_run per job; and
the per-pair drop-in) and serving (Poisson request stream through the
continuous-batching server vs the same arrivals served one request at a
time: p50/p99 latency, throughput).

usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from motex_gb300 import workloads as W  # noqa: E402

WORKLOADS = {
    "dna_ed": lambda s: W.dna_ed(scale=s),
    "dna_ed_k20": lambda s: W.dna_ed(scale=s, k=20, e=4),
    "dna_hd_small": lambda s: W.dna_hd_small(scale=s),
    "prot_uneven_d0": lambda s: W.prot_uneven(d=0, scale=s),
    "prot_uneven_d1": lambda s: W.prot_uneven(d=1, scale=s),
    "dna_long": lambda s: W.dna_long(scale=s),
    "structured_d1": lambda s: W.structured(scale=s, d=1),
    "structured_d0": lambda s: W.structured(scale=s, d=0),
    "structured2_d0": lambda s: W.structured2(scale=s, d=0),
    "structured2_d1": lambda s: W.structured2(scale=s, d=1),
    "dna_satellite": lambda s: W.dna_satellite(scale=s),
}
DEFAULT_WORKLOAD = "dna_ed"
# algorithmic integer operations per DP cell (one factor x one text position)
OPS_PER_CELL = {0: 6, 1: 17}
PORT = os.path.join(ROOT, "oracle", "_build", "motex_port")
REF_OMP = os.path.join(ROOT, "oracle", "_ref", "motexOMP")
REF_OMP_PORT = os.path.join(ROOT, "oracle", "_ref", "motexOMP_port")
CPU_SAMPLE_SECONDS = 12.0


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---------------------------------------------------------------- CPU side

def ensure_port():
    if not os.path.exists(PORT):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "-j8"], check=True, capture_output=True)


def cpu_binary():
    """(path, kind): the CPU implementation the baselines time, the first that
    runs on this host of
      oracle/_ref/motexOMP       the reference built from its sources, linked to
                                 its shipped libflasm.so (x86-64 only);
      oracle/_ref/motexOMP_port  the reference's own driver and writers (its
                                 unmodified sources) over the restated flasm;
      oracle/_build/motex_port   the CPU restatement of the whole path.
    The first two exist where the reference sources are (oracle/build_ref.sh)."""
    for binary, kind in ((REF_OMP, "reference"), (REF_OMP_PORT, "reference (restated flasm)")):
        if os.path.exists(binary) and os.access(binary, os.X_OK):
            try:
                subprocess.run([binary, "-h"], capture_output=True, timeout=10)
                return binary, kind
            except OSError:
                pass
    ensure_port()
    return PORT, "port"


def cpu_run(binary, wl, seqs, threads, timeout=600):
    """Run the CPU implementation on seqs; returns (cells, secs) of its own all-pairs timer."""
    with tempfile.TemporaryDirectory() as tmp:
        fa, out = os.path.join(tmp, "in.fa"), os.path.join(tmp, "out.motex")
        W.write_fasta(fa, seqs)
        args = wl.cli(fa, out) + ["-t", str(threads)]
        if wl.boxes:
            bx = os.path.join(tmp, "in.boxes")
            W.write_boxes(bx, wl.boxes)
            args[args.index("-s") + 1] = bx
        p = subprocess.run([binary] + args, capture_output=True, text=True, timeout=timeout)
        if p.returncode != 0:
            raise RuntimeError(f"{binary} failed: {p.stderr[-500:]}")
        m = re.search(r"# Run on \d+ proc\(s\) in ([0-9.]+) secs", open(out).read())
        secs = float(m.group(1))
    return ref_cells(wl, seqs), secs


def ref_cells(wl, seqs):
    """Reference DP cells of an all-pairs run: sequences shorter than the motif are skipped."""
    tml = wl.k + sum(g[0] + g[2] for g in wl.boxes)
    searched = sum(len(s) for s in seqs if len(s) >= tml)
    return searched * searched * (len(wl.boxes) + 1)


def take_symbols(seqs, total):
    """The first `total` symbols of a workload: its sequences in order, the last one cut."""
    out, left = [], total
    for s in seqs:
        if left <= 0:
            break
        out.append(s[:left])
        left -= len(out[-1])
    return out


def cpu_sample(binary, wl, threads, target_s=CPU_SAMPLE_SECONDS):
    """(sequences, description): the largest prefix of the workload, counted in
    symbols, whose CPU run takes about target_s.  The cost grows with the
    square of the symbols, so the probe starts at 20k symbols and doubles
    until a run takes a quarter of the target."""
    total = sum(map(len, wl.seqs))
    t = min(total, 20000)
    while True:
        cells, secs = cpu_run(binary, wl, take_symbols(wl.seqs, t), threads, timeout=max(120, 20 * target_s))
        if t >= total or secs >= target_s / 4:
            break
        t = min(total, t * 2)
    t2 = max(1, min(total, int(t * (target_s / max(secs, 1e-3)) ** 0.5)))
    sample = take_symbols(wl.seqs, t2)
    cut = len(sample[-1]) < len(wl.seqs[len(sample) - 1])
    desc = (f"first {t2} of {total} symbols ({len(sample)} of {len(wl.seqs)} sequences"
            + (f", the last cut to {len(sample[-1])}" if cut else "") + ")")
    return sample, desc


# ---------------------------------------------------------------- clocks

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- GPU side

def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


def traffic_record(workload):
    """DRAM bytes per DP launch from the committed ncu summary, if any."""
    try:
        with open(os.path.join(ROOT, "profiles", "dp_traffic.json")) as f:
            rec = json.load(f)
        r = rec.get(workload)
        return None if r is None else r.get("traffic")
    except (OSError, ValueError):
        return None


def executed_record(workload):
    """Executed-instruction figures of the workload's DP kernel from the
    committed one-kernel ncu summary (profiles/dp_executed.json), if any:
    thread instructions per algorithmic cell and the pipes' utilisation of
    one captured launch.  Unlike roofline.frac, these are utilisations (<= 1)."""
    try:
        with open(os.path.join(ROOT, "profiles", "dp_executed.json")) as f:
            return json.load(f).get(workload)
    except (OSError, ValueError):
        return None


def aggregate_replicas(step_s, e2e_s, cells, world):
    """Whole-job figures over `world` replicas: the slowest rank's times (max
    over ranks, host all-reduce) and the work of all ranks.  Returns
    (step_s, e2e_s, value_gcups, e2e_gcups)."""
    step_s, e2e_s = max(step_s, 1e-9), max(e2e_s, 1e-9)
    total = cells
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([step_s, e2e_s], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        w = torch.tensor([float(cells)], dtype=torch.float64)
        dist.all_reduce(w, op=dist.ReduceOp.SUM)
        step_s, e2e_s, total = float(t[0]), float(t[1]), float(w[0])
    return step_s, e2e_s, total / step_s / 1e9, total / e2e_s / 1e9


def dp_kernel_name(wl):
    """The engine's default DP kernel for the workload (bit planes B from the
    symbols present; the autotuner may pick another shape of the same kernel)."""
    if wl.boxes:
        lens = [wl.k] + [b[2] for b in wl.boxes]
        if len(wl.boxes) == 1 and max(lens) <= 32 and wl.boxes[0][1] + wl.boxes[0][2] <= 31:
            return "k_dp_struct1_swar_blk" if wl.d == 1 else "k_dp_struct1_hd"
        # the block form packs every box row of a lane in one register
        span = sum(b[1] - b[0] for b in wl.boxes) + 1
        fits = (sum(x + 1 for x in lens) - 1 <= 32) if wl.d == 1 else (len(lens) * max(lens) <= 32)
        if len(lens) <= 4 and max(lens) <= 32 and span <= 17 and fits:
            return "k_dp_structN_blk"
        return "k_dp_structN"
    if wl.k > 32:
        return "k_dp_generic"
    sigma = len(set("".join(wl.seqs)))
    B = max(2, (sigma - 1).bit_length())
    if wl.d == 1 and 4 <= wl.k <= 15:
        return f"k_dp_swar_ed (NL={min(4, 33 // (wl.k + 1))})"
    if wl.d == 0 and 5 <= wl.k <= 12 and wl.e <= 3:
        return f"k_dp_hclr (NL={3 if 6 <= wl.k <= 10 else 2})"
    if wl.d == 0 and B >= 3 and 6 <= wl.k <= 16:
        return f"k_dp_hswar (NL={32 // wl.k})"
    return "k_dp_fast"


def tuned_kernel_name(wl, shape):
    """The DP kernel of an autotuner entry (W, NL, UR): a negative NL is the
    guarded-lane Hamming form, NL > 1 a packed form, NL = 1 one factor per
    register."""
    W, NL, UR = shape
    if NL < 0:
        name = f"k_dp_hclr (NL={-NL})"
    elif NL > 1:
        name = f"k_dp_swar_ed (NL={NL})" if wl.d == 1 else f"k_dp_hswar (NL={NL})"
    else:
        name = "k_dp_fast"
    return name + " W=%d NL=%d UR=%d" % (W, abs(NL), UR)


def c_level_calls(native, ctx, jobs):
    """(batch, sequential, keep): callables that run `jobs` through the C ABI
    -- one motex_gpu_run_batch call, or one motex_gpu_run per job -- with
    argument arrays built once and every result freed unread, so that their
    time is the library's (copies, kernels, host syncs, result assembly) and
    not the Python conversion of the motif lists.  `keep` holds the arrays."""
    import ctypes as C
    lib = ctx.lib
    keep = []
    arr = (native.Job * len(jobs))()
    singles = []
    for i, (seqs, prm) in enumerate(jobs):
        bs = [s.encode() for s in seqs]
        a = (C.c_char_p * len(bs))(*bs)
        lens = (C.c_uint32 * len(bs))(*[len(b) for b in bs])
        keep.append((bs, a, lens, prm))
        arr[i] = native.Job(C.pointer(prm), a, lens, len(bs))
        singles.append((prm, a, lens, len(bs)))
    res = (native.Result * len(jobs))()
    one = native.Result()

    def check(rc):
        if rc != 0:
            raise native.MotexError(rc, lib.motex_gpu_last_error().decode())

    def batch():
        check(lib.motex_gpu_run_batch(ctx.h, arr, len(jobs), res))
        for i in range(len(jobs)):
            lib.motex_result_free(C.byref(res[i]))

    def sequential():
        for prm, a, lens, n in singles:
            check(lib.motex_gpu_run(ctx.h, C.byref(prm), a, lens, n, C.byref(one)))
            lib.motex_result_free(C.byref(one))

    return batch, sequential, keep


def batched_vs_plain(native, ctx, seed=3, sample=30, scale=1.0):
    """Uneven protein batch (-d 1 -k 10 -e 2 -q 15), batched against plain
    three ways:

    * whole: the whole set as one job through motex_gpu_run_batch (the DP as
      one persistent launch fed from the device work queue) against the same
      job through motex_gpu_run (one static-grid DP launch); DP device time
      (CUDA events) and host wall time of each;
    * jobs: the set cut into uneven jobs of 5-40 consecutive sequences, one
      motex_gpu_run_batch call against the same jobs run one after another
      through motex_gpu_run (host wall time, results compared);
    * per_pair: the per-pair drop-in (motex_gpu_extract_pair, one extraction
      launch sequence per ordered pair, the reference driver's loop) on the
      ordered pairs of the first `sample` sequences (host wall time)."""
    import random as _r
    import time as _t
    wl = W.prot_uneven(seed=seed, d=1, scale=scale)
    prm = native.make_params(wl.d, wl.k, wl.e, wl.q)
    out = {"workload": "prot_uneven_d1"}

    def best(fn, reps=3):
        t = 1e30
        for _ in range(reps):
            t0 = _t.perf_counter()
            fn()
            t = min(t, _t.perf_counter() - t0)
        return t

    # whole set: persistent batched vs the static one-job launch (results
    # compared through the Python wrapper, times taken at the C ABI)
    rb = ctx.run_batch([(wl.seqs, prm)])[0]
    rs = ctx.run(wl.seqs, prm)
    assert rb.motifs == rs.motifs, "batched and static results differ"
    wb, ws, _keep = c_level_calls(native, ctx, [(wl.seqs, prm)])
    tb, ts = best(wb), best(ws)
    cells = rb.ref_cells
    out["whole"] = {"batched_dp_gcups": round(cells / rb.dp_ms / 1e6, 1), "static_dp_gcups": round(cells / rs.dp_ms / 1e6, 1),
                    "batched_dp_ms": round(rb.dp_ms, 3), "static_dp_ms": round(rs.dp_ms, 3),
                    "batched_wall_gcups": round(cells / tb / 1e9, 1), "static_wall_gcups": round(cells / ts / 1e9, 1),
                    "dp_ratio": round(rs.dp_ms / rb.dp_ms, 3), "wall_ratio": round(ts / tb, 3)}

    # many uneven jobs: one batch call vs one motex_gpu_run per job
    rng = _r.Random(seed)
    jobs, at = [], 0
    while at < len(wl.seqs):
        n = rng.randint(5, 40)
        jobs.append((wl.seqs[at:at + n], prm))
        at += n
    rjb = ctx.run_batch(jobs)
    rjs = [ctx.run(s, p) for s, p in jobs]
    assert [r.motifs for r in rjb] == [r.motifs for r in rjs], "batched and sequential job results differ"
    jb, js_, _keep2 = c_level_calls(native, ctx, jobs)
    tjb, tjs = best(jb), best(js_)
    jcells = sum(r.ref_cells for r in rjb)
    out["jobs"] = {"jobs": len(jobs), "sequences_per_job": "5-40", "batched_gcups": round(jcells / tjb / 1e9, 1),
                   "sequential_gcups": round(jcells / tjs / 1e9, 1), "batched_ms": round(tjb * 1e3, 2),
                   "sequential_ms": round(tjs * 1e3, 2), "ratio": round(tjs / tjb, 2)}

    # per-pair drop-in
    seqs = wl.seqs[:sample]
    pcells = 0
    ctx.extract_pair(seqs[0], seqs[1], prm)
    t0 = _t.perf_counter()
    for x in seqs:
        for t in seqs:
            if len(x) >= wl.k and len(t) >= wl.k:
                ctx.extract_pair(x, t, prm)
                pcells += len(x) * len(t)
    tp = _t.perf_counter() - t0
    out["per_pair"] = {"pairs": len(seqs) ** 2, "gcups": round(pcells / tp / 1e9, 3),
                       "ratio_batched_whole_wall": round(cells / tb / (pcells / tp), 1)}
    out["note"] = ("whole: one job, batched persistent launch vs static one-job launch (dp = device DP time, "
                   "wall = host time of the C call, best of 3); jobs: one batch call vs motex_gpu_run per job "
                   "(host time of the C calls, best of 3; the small jobs take the small-job pipeline both ways); "
                   "per_pair: motex_gpu_extract_pair per ordered pair of the first "
                   f"{sample} sequences (host wall)")
    return out


def serving(native, nreq=2000, rate_hz=100.0, seed=5, max_batch=32, workers=2):
    """Poisson request stream through the continuous-batching server, and
    the same arrivals served one request at a time (plain per-request GPU
    path, FIFO).  Latency = completion - arrival."""
    import threading
    import time as _t
    stream = W.serve_stream(seed=seed, nreq=nreq, rate_hz=rate_hz)
    reqs = [(t, wl.seqs, native.make_params(wl.d, wl.k, wl.e, wl.q)) for t, wl in stream]
    cells = [sum(map(len, s)) ** 2 for _, s, _ in reqs]

    def pct(xs, q):
        xs = sorted(xs)
        return xs[min(len(xs) - 1, int(round(q / 100 * (len(xs) - 1))))]

    out = {"requests": nreq, "rate_hz": rate_hz, "max_batch": max_batch, "workers": workers}
    with native.Server(max_batch=max_batch, workers=workers) as srv:
        ids = [None] * nreq
        lat = [None] * nreq
        t0 = _t.perf_counter()

        def submitter():
            for i, (t, s, p) in enumerate(reqs):
                d = t0 + t - _t.perf_counter()
                if d > 0:
                    _t.sleep(d)
                ids[i] = srv.submit(s, p)

        th = threading.Thread(target=submitter)
        th.start()
        for i in range(nreq):
            while ids[i] is None:
                _t.sleep(0.0005)
            _, tm = srv.wait(ids[i])
            lat[i] = tm["latency_ms"]
        th.join()
        wall = _t.perf_counter() - t0
        st = srv.stats()
    out["batched"] = {"p50_ms": round(pct(lat, 50), 2), "p99_ms": round(pct(lat, 99), 2),
                      "req_per_s": round(nreq / wall, 1), "gcups": round(sum(cells) / wall / 1e9, 1),
                      "batches": st["batches"], "max_batch_seen": st["max_batch_seen"]}
    ctx = native.Context(0)
    lat2 = []
    t0 = _t.perf_counter()
    for t, s, p in reqs:
        d = t0 + t - _t.perf_counter()
        if d > 0:
            _t.sleep(d)
        ctx.run(s, p)
        lat2.append((_t.perf_counter() - t0 - t) * 1e3)
    wall2 = _t.perf_counter() - t0
    ctx.close()
    out["plain"] = {"p50_ms": round(pct(lat2, 50), 2), "p99_ms": round(pct(lat2, 99), 2),
                    "req_per_s": round(nreq / wall2, 1), "gcups": round(sum(cells) / wall2 / 1e9, 1)}
    return out


def workload_config(args, wl, world, l2):
    """The `config` object of both arms: the workload, its sizes and switches."""
    return {"workload": args.workload, "scale": args.scale, "alphabet": wl.alphabet, "num_seqs": len(wl.seqs),
            "total_len": sum(len(s) for s in wl.seqs), "d": wl.d, "k": wl.k, "e": wl.e, "q": wl.q,
            "boxes": [list(b) for b in wl.boxes], "ref_cells": ref_cells(wl, wl.seqs),
            "parallelism": f"replicas{world}", "l2": l2}


def run_gpu(args, rank, world, local_rank):
    import ctypes as C
    import torch
    from motex_gb300 import native

    torch.cuda.set_device(local_rank)
    wl = WORKLOADS[args.workload](args.scale)
    prm = native.make_params(wl.d, wl.k, wl.e, wl.q, wl.Q, wl.n, wl.N, wl.boxes)
    ctx = native.Context(local_rank)
    lib = ctx.lib
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local_rank}")

    def dist_barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    # ---- value: device-resident steps
    ctx.load(wl.seqs, prm)
    for _ in range(args.warmup):
        ctx.execute()
    first = ctx.fetch()
    dist_barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local_rank)
    sampler.start()
    launches0 = ctx.launches
    dev_ms, dp_ms, wall = [], [], []
    results = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.execute()
        wall.append(time.perf_counter() - t0)
        r = ctx.fetch()
        dev_ms.append(r.device_ms)
        dp_ms.append(r.dp_ms)
        results.append(r.motifs)
    launches = ctx.launches - launches0
    torch.cuda.synchronize()
    dist_barrier()
    clocks = sampler.stop()
    assert all(m == first.motifs for m in results), "non-deterministic result across steps"

    # ---- e2e: public C ABI with host buffers
    bs = [s.encode() for s in wl.seqs]
    arr = (C.c_char_p * len(bs))(*bs)
    lens = (C.c_uint32 * len(bs))(*[len(b) for b in bs])
    res = native.Result()
    e2e_wall = []
    e2e_warm = 1                      # the resident-input warm-up above already warmed the context
    for i in range(e2e_warm + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rc = lib.motex_gpu_run(ctx.h, C.byref(prm), arr, lens, len(bs), C.byref(res))
        dt = time.perf_counter() - t0
        if rc != 0:
            raise native.MotexError(rc, lib.motex_gpu_last_error().decode())
        count = res.count
        lib.motex_result_free(C.byref(res))
        if i >= e2e_warm:
            e2e_wall.append(dt)
    assert count == len(first.motifs)

    total = sum(len(b) for b in bs)
    h2d = total + 2 * 4 * (len(bs) + 1) + (len(bs) + 1) + 256
    d2h = 12 * count + 256 * 4 + 8

    # ---- aggregate over ranks (replicas)
    cells = first.ref_cells
    step_s, e2e_s, value, e2e = aggregate_replicas(sum(dev_ms) / 1e3, sum(e2e_wall), cells * args.steps, world)

    # ---- roofline of the DP kernel
    lop3, iadd, popc = native.probe_int_peak(local_rank)
    total_pos = sum(len(s) for s in wl.seqs)
    alg_ops = first.unique_words * total_pos * OPS_PER_CELL[wl.d]
    dp_s = statistics.mean(dp_ms) / 1e3
    achieved = alg_ops / dp_s / 1e12 if dp_s > 0 else 0.0
    tr = traffic_record(args.workload)
    kernel = dp_kernel_name(wl)
    if not wl.boxes and wl.k <= 32:
        # the launch shape the autotuner settled on for this key, if it tuned
        sigma = len(set("".join(wl.seqs)))
        shape = native.tune_lookup(max(2, (sigma - 1).bit_length()), wl.k, wl.e, wl.d)
        if shape:
            kernel = tuned_kernel_name(wl, shape)
    roofline = {"bound": "int32_alu", "kernel": kernel, "achieved": round(achieved, 3),
                "peak": round(iadd, 3), "unit": "Tops/s", "frac": round(achieved / iadd, 4) if iadd else None,
                "peak_source": "measured int32 add throughput, all pipes (motex_probe_int_peak), same run",
                "lop3_pipe_peak": round(lop3, 3), "popc_peak": round(popc, 3),
                "ops_per_cell": OPS_PER_CELL[wl.d], "cells_per_launch": first.unique_words * total_pos,
                "dp_ms": round(dp_s * 1e3, 3), "dp_cells_per_s": round(first.unique_words * total_pos / dp_s, 1),
                "traffic": tr,
                "note": "algorithmic ops per cell; SWAR lanes (2-4 cells per instruction) and the shared Eq "
                        "table execute fewer, so frac can exceed 1; `executed` gives the measured utilisations"}
    ex = executed_record(args.workload)
    if ex:
        roofline["executed"] = ex
    if wl.d == 0 and not wl.boxes and dp_s > 0 and popc and not kernel.startswith("k_dp_hclr"):
        # plain Hamming runs one population count per cell (the guarded-lane
        # form none): its second roof
        popc_rate = first.unique_words * total_pos / dp_s / 1e12
        roofline.update(popc_achieved=round(popc_rate, 3), popc_frac=round(popc_rate / popc, 4))

    extras = {}
    if rank == 0 and not args.no_extras and args.scale == 1.0:
        extras["batched_vs_plain"] = batched_vs_plain(native, ctx)
        extras["serving"] = serving(native, nreq=args.serve_requests)
        # a rate both arms sustain (the one-at-a-time arm serves about 90
        # requests/s): latency is then service time, not queue growth
        extras["serving"]["at_40hz"] = serving(native, nreq=max(100, args.serve_requests * 2 // 5), rate_hz=40.0)
    out = {
        "metric": "GCUPS (reference DP cell updates per second), whole-set word-based motif extraction",
        "value": round(value, 2), "unit": "GCUPS", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(step_s * 1e3 / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32 bit-vector (integer)", "data": "synthetic (seeded generator)",
        "config": workload_config(args, wl, world, "flushed (256 MiB write) before every step"),
        "run": {"unique_words": first.unique_words, "motifs": len(first.motifs),
                "host_wall_ms_per_step": round(1e3 * statistics.mean(wall), 3)},
        "e2e": {"value": round(e2e, 2), "unit": "GCUPS", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": round(e2e_s * 1e3 / args.steps, 3)},
        "gpu_launches": launches,
        "roofline": roofline,
        "clocks": clocks,
        "measured_peaks": {k: measured_peaks().get(k) for k in ("hbm_gbs", "bf16_tflops")},
    }
    out.update(extras)
    ctx.close()
    return out, wl


def run_reference(args, world):
    """Reference arm: the CPU implementation of the path, all host threads."""
    wl = WORKLOADS[args.workload](args.scale)
    binary, kind = cpu_binary()
    threads = os.cpu_count() or 1
    sample, sample_desc = cpu_sample(binary, wl, threads, target_s=8.0)
    for _ in range(args.warmup):
        cpu_run(binary, wl, sample, threads)
    cells_t, secs_t = 0, 0.0
    for _ in range(args.steps):
        c, s = cpu_run(binary, wl, sample, threads)
        cells_t += c
        secs_t += s
    val = cells_t / secs_t / 1e9
    desc = sample_desc
    return {
        "impl": "reference", "metric": "GCUPS (reference DP cell updates per second), whole-set word-based motif extraction",
        "value": round(val, 3), "unit": "GCUPS", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(secs_t * 1e3 / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "integer", "data": "synthetic (seeded generator)",
        "config": workload_config(args, wl, world, "not applicable (CPU run, host caches)"),
        "run": {"host_threads": threads},
        "cpu_baseline": {"value": round(val, 3), "unit": "GCUPS", "cores": threads, "kind": kind, "sample": desc},
        "e2e": {"value": round(val, 3), "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scale", type=float, default=1.0,
                    help="shrink the workload (profiling captures only; 1.0 = the benchmark size)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=2000,
                    help="requests in the serving stream (Poisson arrivals, 100/s)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batched-vs-plain and serving sections")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args, world)), flush=True)
        return

    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
    out, wl = run_gpu(args, rank, world, local_rank)
    if rank == 0:
        if not args.no_cpu_baseline:
            binary, kind = cpu_binary()
            threads = os.cpu_count() or 1
            sample, desc = cpu_sample(binary, wl, threads)
            cells, secs = cpu_run(binary, wl, sample, threads)
            out["cpu_baseline"] = {"value": round(cells / secs / 1e9, 3), "unit": "GCUPS", "cores": threads,
                                   "kind": kind, "sample": f"{desc}, {secs:.1f} s"}
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
