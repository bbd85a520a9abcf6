#!/usr/bin/env python3
"""Benchmark: terminals/s of the batched persistent derivation engine.

Workload (one step): the 4096-building procedural city (Quad footprints on a
64 x 64 grid, seed 1234; Extrude, ComponentSplit, Repeat floors/tiles,
IfSizeLess, window Subdivide) derived in one pga_derive call -> 5,856,274
instanced terminals (375 MB of 64-byte records, larger than the 129 MB L2;
L2 is also flushed with a 256 MB write before every timed step).

schedule: before timing, the engine knobs are autotuned on this workload
         (operatorgraph_gb300/autotune.py, 64 candidates); the fastest drives
         the timed engine ("batched + autotuned").
value  : terminals/s with axioms and grammar resident in HBM (CUDA events on
         the launching stream around pga_derive).
e2e    : the same through the C ABI with host buffers (pga_derive_to_host):
         pinned-host -> device copy of the axioms, derivation in axiom ranges,
         device -> pinned-host copy of every terminal record overlapped with
         the next range's derivation, all inside the timed region.
roofline: algorithmic bytes of the derivation kernel (64 B per terminal
         written + 48 B per axiom read) / kernel time, against the measured
         HBM copy bandwidth.
extra  : the plain one-grammar-per-launch GPU form on the same city, the
         Menger sponge at depth 5, the LBVH over the city's terminals, the
         facades with tape + adjoint, and the 65,536-axiom mixed batch, also
         as one graph-captured differentiable step (derivation with the tape,
         LBVH over the device-side count, loss gradient, adjoint).

`--impl reference` times the reference's own CPU derivation (oracle/_ref,
built from the reference sources) on the same workload, sharded by axiom
ranges over all host cores.

Synthetic data: every input is generated from fixed seeds.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from operatorgraph_gb300 import grammar as G  # noqa: E402
from operatorgraph_gb300 import scenes  # noqa: E402

METRIC = "terminals/s (batched persistent derivation, 4096-building city)"
UNIT = "terminals/s"
WORKLOAD = {"workload": "city-4096 (64x64 grid, seed 1234, Repeat anchor-to-start)", "axioms": 4096,
            "terminals": 5856274, "l2": "256 MB flush before each timed step; outputs 375 MB > L2"}


def read_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def read_profile_traffic(name):
    """Per-launch DRAM bytes recorded from an ncu capture under profiles/."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.strip().startswith("traffic_bytes_per_launch:"):
            return float(line.split(":", 1)[1].split()[0])
    return None


class ClockSampler:
    """nvidia-smi samples (200 ms) during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
            return self
        return self

    def _read(self):
        # nvidia-smi's own timestamp, not the arrival time: its output through a
        # pipe is block-buffered and can arrive long after the sample was taken.
        import datetime

        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                try:
                    t = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                except ValueError:
                    t = time.time()
                self.samples.append([t] + parts[1:])

    def mark(self, start, end):
        self.window = (start, end)

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.3)  # one more period, so that a sample follows the timed region
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=5)

    def summary(self):
        """Median SM clock and throttle reasons of the samples taken while the
        timed steps ran (a sample arrives within one 200 ms period)."""
        lo, hi = getattr(self, "window", (0.0, float("inf")))
        inside = [s[1:] for s in self.samples if lo <= s[0] <= hi + 0.25]
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(s[0]) for s in inside if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in inside if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in inside for k in range(4) if s[3 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(inside)}


def host_info():
    try:
        cores = len(os.sched_getaffinity(0))
    except AttributeError:
        cores = os.cpu_count()
    model = ""
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                model = line.split(":", 1)[1].strip()
                break
    except OSError:
        pass
    import platform

    return cores, f"{platform.machine()} {model}".strip()


# ------------------------------------------------------------- CPU reference


def ref_harness_available():
    import oracle

    if os.path.exists(oracle.REF_HARNESS):
        return oracle.REF_HARNESS
    return oracle.build_ref()


def run_reference_sharded(batch, shards, repeats=1):
    """Runs the reference's CPU evaluator on `shards` axiom ranges in parallel
    processes, each timing `repeats` execute() calls and writing no terminal
    file.  Returns (terminals, per-shard lists of execute() seconds, wall
    seconds of the whole call including process start and the batch files)."""
    harness = ref_harness_available()
    tmp = tempfile.mkdtemp()
    ax = batch["axioms"]
    parts = np.array_split(np.arange(len(ax)), shards)
    procs = []
    t0 = time.perf_counter()
    for k, idx in enumerate(parts):
        bf = os.path.join(tmp, f"b{k}.bin")
        G.write_batch_file(bf, batch["entries"], ax[idx])
        procs.append(subprocess.Popen([harness, bf, os.path.join(tmp, f"t{k}.bin"), str(repeats),
                                       "--axiom-base", str(int(idx[0]) if len(idx) else 0), "--no-output"],
                                      stdout=subprocess.PIPE, text=True))
    total, per = 0, []
    for p in procs:
        out, _ = p.communicate()
        d = json.loads(out.strip().splitlines()[-1])
        total += d["terminals"]
        per.append(d["all_seconds"])
    wall = time.perf_counter() - t0
    return total, per, wall


def cpu_baseline_single(batch):
    """The reference's own CPU evaluator, 1 thread, on a bounded sample."""
    cores, model = host_info()
    try:
        ref_harness_available()
        n, secs, _ = run_reference_sharded(batch, 1, repeats=3)
        return {"value": n / statistics.median(secs[0]), "unit": UNIT, "cores": 1, "kind": "reference",
                "sample": f"full city-4096 ({n} terminals), median of 3 execute() calls, 1 thread, {model}"}
    except Exception:
        import oracle

        t0 = time.perf_counter()
        t = oracle.derive(G.DEFAULT_PROCS, batch["entries"], batch["axioms"])
        secs = time.perf_counter() - t0
        return {"value": len(t) / secs, "unit": UNIT, "cores": 1, "kind": "port",
                "sample": f"full city-4096 ({len(t)} terminals), oracle restatement, 1 thread, {model}"}


def max_over_ranks(ms, device):
    """The largest of every rank's `ms` (the job is as slow as its slowest
    replica); `ms` itself when there is one rank."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return ms
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    batch = scenes.city(4096)
    cores, model = host_info()
    kind = "reference"
    try:
        ref_harness_available()
    except Exception:
        kind = "port"
    if kind == "port":
        print(json.dumps({"impl": "reference", "unavailable": "reference CPU evaluator could not be built here"}))
        return
    # One process per host core, each timing warmup + steps execute() calls on
    # its axiom range.  The shards run side by side, so the job's timed steps
    # take as long as the slowest shard's timed execute() calls together.
    total, per, wall = run_reference_sharded(batch, cores, repeats=args.warmup + args.steps)
    mean = max(sum(sh[args.warmup:]) for sh in per) / args.steps
    value = total / mean
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": mean * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": WORKLOAD, "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                             "sample": f"full city-4096 per step in {cores} axiom shards, one process per core; "
                                       f"the slowest shard's execute() time per step (no file output), {model}"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_incl_process_start_s": wall, "wall_steps": args.warmup + args.steps}
    print(json.dumps(line))


# ------------------------------------------------------------------ GPU arm


def our_arm(args):
    import torch

    from operatorgraph_gb300 import autotune
    from operatorgraph_gb300 import build as B
    from operatorgraph_gb300.engine import Engine, load_library

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    if not B.up_to_date():
        B.build()
    load_library()
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream()

    batch = scenes.city(4096)
    n_ax = len(batch["axioms"])
    cap = 6_000_000
    # Schedule autotuning (the reference's per-grammar schedule search): the
    # fastest knob set on this workload drives the timed engine.
    if args.schedule:
        best = {k: int(v) for k, v in (kv.split("=") for kv in args.schedule.split(","))}
        tuned_ms, tuning, default_ms = None, [], None
    else:
        best, tuned_ms, tuning = autotune.tune(batch, cap, node_capacity=1 << 22, runs=5)
        default_ms = next((r["ms"] for r in tuning if autotune.is_default(r["config"])), None)
    eng = Engine(batch["entries"], node_capacity=1 << 22, max_terminals=cap, **best)
    d_ax = torch.from_numpy(batch["axioms"].view(np.uint8).copy()).to(dev)
    out = torch.empty((cap, 64), dtype=torch.uint8, device=dev)
    count = torch.zeros(1, dtype=torch.int64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def step():
        eng.derive_raw(d_ax.data_ptr(), n_ax, None, out.data_ptr(), cap, count.data_ptr())

    for _ in range(max(args.warmup, 3)):
        step()
    rep = eng.report()
    assert rep["status"] == 0, rep
    n_term = int(count.item())
    assert n_term == WORKLOAD["terminals"], n_term

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize()

    # ---- device-resident timing (value, roofline)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clocks:
        time.sleep(1.0)  # let the sampler start
        barrier()
        t_start = time.time()
        for k in range(args.steps):
            flush.fill_(k & 0xFF)
            evs[k][0].record(stream)
            step()
            evs[k][1].record(stream)
        barrier()
        clocks.mark(t_start, time.time())
    step_ms = [a.elapsed_time(b) for a, b in evs]
    ms = max_over_ranks(sum(step_ms) / len(step_ms), dev)
    value = world * n_term / (ms * 1e-3)

    # ---- end to end through the C ABI with host buffers: pga_derive_to_host
    # copies the pinned host axioms in, derives in axiom ranges and copies each
    # range's terminals back to pinned host memory while the next one derives.
    h_ax = torch.from_numpy(batch["axioms"].view(np.uint8).copy()).pin_memory()
    h_out = torch.empty((cap, 64), dtype=torch.uint8).pin_memory()

    def e2e_step():
        n, _ = eng.derive_to_host(h_ax.data_ptr(), n_ax, h_out.data_ptr(), cap)
        return n

    for _ in range(3):
        e2e_step()
    # Each call returns when the host buffer holds the terminals, so a step is
    # timed by the host clock around it.  The value is the median step (a step
    # that waits on the host -- another process, a page fault -- is an outlier
    # of a few ms); the mean, min and max are reported beside it.
    e2e_steps = max(1, min(args.steps, 20))
    barrier()
    e2e_times = []
    for _ in range(e2e_steps):
        h0 = time.perf_counter()
        n_host = e2e_step()
        e2e_times.append((time.perf_counter() - h0) * 1e3)
    barrier()
    e2e_ms = max_over_ranks(statistics.median(e2e_times), dev)
    assert n_host == n_term
    e2e_value = world * n_term / (e2e_ms * 1e-3)

    # The same with one launch, then one copy of the whole output (for comparison).
    h_cnt = torch.empty(1, dtype=torch.int64).pin_memory()
    d_ax2 = torch.empty_like(d_ax)

    def single_step():
        d_ax2.copy_(h_ax, non_blocking=True)
        eng.derive_raw(d_ax2.data_ptr(), n_ax, None, out.data_ptr(), cap, count.data_ptr())
        h_cnt.copy_(count, non_blocking=True)
        h_out[:n_term].copy_(out[:n_term], non_blocking=True)

    single_step()
    torch.cuda.synchronize()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    for _ in range(e2e_steps):
        single_step()
    s1.record(stream)
    torch.cuda.synchronize()
    single_ms = s0.elapsed_time(s1) / e2e_steps

    line = None
    if rank == 0:
        peak, peak_kind = read_peaks()
        alg_bytes = 64.0 * n_term + 48.0 * n_ax
        achieved = alg_bytes / (ms * 1e-3) / 1e9
        traffic = read_profile_traffic("k_derive_persistent_city4096.md")
        extra = extras(eng, batch, out, n_term, dev, stream, flush)
        # the batching gain over the one-grammar-per-launch form (same engine, same schedule)
        extra["batched_over_plain"] = value / world / extra["plain_city_terminals_per_s"]
        cores, model = host_info()
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": WORKLOAD,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h_ax.numel()),
                    "d2h_bytes_per_step": int(n_term * 64), "ms_per_step": e2e_ms, "steps": e2e_steps,
                    "mean_ms": statistics.fmean(e2e_times), "min_ms": min(e2e_times), "max_ms": max(e2e_times),
                    "api": "pga_derive_to_host (pinned host buffers)", "single_launch_then_copy_ms": single_ms},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "kernel": "k_derive_persistent", "algorithmic_bytes": alg_bytes},
            "schedule": {"autotuned": best, "candidates": len(tuning), "tuned_ms": tuned_ms,
                         "default_ms": default_ms},
            "gpu_launches": args.steps,
            "clocks": clocks.summary(),
            "extra": extra,
            "cpu_baseline": cpu_baseline_single(batch),
            "host": {"cores": cores, "cpu": model},
        }
    eng.release()
    if line is not None:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def step_order(n_ax, mout, count, dev, schedule, runs=3):
    """The level order for the differentiable mixed step: times the
    tape-recording derivation plus the adjoint of the scalar batch (eagerly,
    CUDA events) with the derivation's dynamic chunks off and on (the adjoint
    hands out its wide levels dynamically either way), keeps the faster.  The
    forward-only autotune times derivations without the tape.  Returns
    (dynamic_chunks, {False: ms, True: ms})."""
    import torch

    from operatorgraph_gb300.engine import Engine

    mx = scenes.mixed(n_ax)
    mcap = mout.shape[0]
    d_mx = torch.from_numpy(mx["axioms"].view(np.uint8).copy()).to(dev)
    g_sz = torch.empty((n_ax, 3), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()
    times = {}
    for dyn in (False, True):
        knobs = dict(schedule or {}, group_axioms=True, dynamic_chunks=dyn)
        eng = Engine(mx["entries"], node_capacity=1 << 28, max_terminals=mcap, record_tape=True, **knobs)
        ts = []
        for k in range(runs + 1):
            a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            eng.derive_raw(d_mx.data_ptr(), n_ax, None, mout.data_ptr(), mcap, count.data_ptr())
            eng.adjoint_raw(mout.data_ptr(), None, 0, g_sz.data_ptr(), stream=stream, grad_stride=16)
            z.record(stream)
            torch.cuda.synchronize()
            if k:
                ts.append(a.elapsed_time(z))
        assert eng.report()["status"] == 0
        eng.release()
        times[dyn] = statistics.median(ts)
    return times[True] < times[False], times


def mixed_step(n_ax, mout, count, dev, n_expected, blocks=True, schedule=None):
    """The mixed batch as one differentiable step captured in one CUDA graph:
    derivation with the tape recorded, LBVH over all its terminals (the leaf
    count read on the device, pga_lbvh_build_counted), and the adjoint for the
    loss L = |M|^2 / 2, whose dL/dM = M the adjoint reads in place from the
    terminal records (pga_adjoint_strided, stride 16 floats).  blocks=True:
    to every DynParam and axiom size, on the batch with parameter blocks
    (scenes.mixed(blocks=True): each building's floor height, tile width and
    window wall widths, each sponge's split factors; the same terminals as the
    scalar batch); blocks=False: to the axiom sizes of the scalar batch.  The
    axioms are seeded grouped by root entry.  `schedule`: engine knobs (the
    mixed batch's autotuned schedule, dynamic chunks included), else the
    defaults.  The parts are also timed one by one, eagerly.  Keys are prefixed
    mixed65536_step_ (blocks) or mixed65536_sizes_step_."""
    import torch

    from operatorgraph_gb300.engine import Engine

    res = {}
    mx = scenes.mixed(n_ax, blocks=blocks)
    mcap = mout.shape[0]
    knobs = dict(schedule or {})
    knobs["group_axioms"] = True
    et = Engine(mx["entries"], node_capacity=1 << 28, max_terminals=mcap, record_tape=True,
                block_stride=mx["block_stride"], **knobs)
    d_mx = torch.from_numpy(mx["axioms"].view(np.uint8).copy()).to(dev)
    d_blk = torch.from_numpy(mx["blocks"]).to(dev) if blocks else torch.zeros(1, dtype=torch.float32, device=dev)
    g_blk = torch.empty_like(d_blk)
    blk_ptr = d_blk.data_ptr() if blocks else None
    gblk_ptr = g_blk.data_ptr() if blocks else None
    n_blocks = n_ax if blocks else 0
    g_sz = torch.empty((n_ax, 3), dtype=torch.float32, device=dev)
    m_rows = mout.view(torch.float32).view(mcap, 16)
    # LBVH bounds: the box of the terminal centres of a first derivation, one
    # metre wider on every side.
    et.derive_raw(d_mx.data_ptr(), n_ax, blk_ptr, mout.data_ptr(), mcap, count.data_ptr())
    torch.cuda.synchronize()
    rep = et.report()
    assert rep["status"] == 0, rep
    n = int(count.item())
    assert n == n_expected, (n, n_expected)
    c = m_rows[:n][:, [3, 7, 11]]
    lo, hi = c.amin(dim=0).double().cpu().numpy() - 1.0, c.amax(dim=0).double().cpu().numpy() + 1.0
    del c
    bounds = tuple(float(v) for v in lo) + tuple(float(v) for v in hi)
    n_items = int(rep["nodes"])
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())

    def step(st, marks=None):
        def mark(k):
            if marks is not None:
                marks[k].record(st)

        mark(0)
        et.derive_raw(d_mx.data_ptr(), n_ax, blk_ptr, mout.data_ptr(), mcap, count.data_ptr(), stream=st)
        mark(1)
        bv = et.lbvh(mout, mcap, bounds, stream=st, count=count)
        mark(2)
        et.adjoint_raw(mout.data_ptr(), gblk_ptr, n_blocks, g_sz.data_ptr(), stream=st, grad_stride=16)
        mark(3)
        return bv

    seg = []
    with torch.cuda.stream(s):
        for it in range(5):
            marks = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
            bv = step(s, marks)
            s.synchronize()
            if it >= 2:
                seg.append([marks[k].elapsed_time(marks[k + 1]) for k in range(3)])
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    rep = et.report()
    assert rep["status"] == 0, rep
    assert int(count.item()) == n
    keys = bv["keys"][:n] ^ (-(1 << 63))  # sign bit flipped: signed order = the keys' unsigned order
    assert bool((keys[1:] >= keys[:-1]).all()), "LBVH keys not sorted"
    del bv, keys
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        bv = step(torch.cuda.current_stream())
    ts = []
    for it in range(6):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        g.replay()
        b.record()
        torch.cuda.synchronize()
        if it >= 2:
            ts.append(a.elapsed_time(b))
    rep = et.report()
    assert rep["status"] == 0, rep
    assert int(count.item()) == n
    assert bool(torch.isfinite(g_sz).all()) and float(g_sz.abs().max()) > 0
    if blocks:
        assert bool(torch.isfinite(g_blk).all()) and float(g_blk.abs().max()) > 0
    names = ("derive_tape", "lbvh", "adjoint")
    med = [statistics.median(x[k] for x in seg) for k in range(3)]
    n_par = int(d_blk.numel()) if blocks else 0
    # Algorithmic bytes, counted two ways.  This bench's count: derivation 64 B
    # per terminal, its 8-B tape link and 48 B per axiom; LBVH 204 B per leaf
    # (the 64-B record read, 52 B of tree written, four radix passes over 12-B
    # key/value pairs read and written); adjoint per terminal 48 + 8 B, per
    # item 2 x 64 + 2 x 24 B, 4 B per parameter and axiom size.  The
    # reference-path formulas: B_fwd = 64 T + 32 A, B_lbvh = 108 T,
    # B_adj = 112 T + 140 N + 4 P.
    parts = [72.0 * n + 48.0 * n_ax, 204.0 * n, 56.0 * n + 176.0 * n_items + 4.0 * (n_par + 3 * n_ax)]
    parts_8d = [64.0 * n + 32.0 * n_ax, 108.0 * n, 112.0 * n + 140.0 * n_items + 4.0 * (n_par + 3 * n_ax)]
    pre = "mixed65536_step_" if blocks else "mixed65536_sizes_step_"
    peak, _ = read_peaks()
    step_ms = statistics.median(ts)
    res[pre + "graph_ms"] = step_ms
    res[pre + "items"] = n_items
    res[pre + "params"] = n_par
    res[pre + "segments_ms"] = {k: v for k, v in zip(names, med)}
    res[pre + "segments_gbs"] = {k: b / (v * 1e-3) / 1e9 for k, b, v in zip(names, parts, med)}
    res[pre + "bytes"] = sum(parts)
    res[pre + "gbs"] = sum(parts) / (step_ms * 1e-3) / 1e9
    res[pre + "roofline_frac"] = res[pre + "gbs"] / peak
    res[pre + "bytes_formula"] = sum(parts_8d)
    res[pre + "roofline_frac_formula"] = sum(parts_8d) / (step_ms * 1e-3) / 1e9 / peak
    # the forward + adjoint step alone (no LBVH), by the formulas
    fa_ms = med[0] + med[2]
    res[pre + "fwd_adjoint_ms"] = fa_ms
    res[pre + "fwd_adjoint_roofline_frac_formula"] = (parts_8d[0] + parts_8d[2]) / (fa_ms * 1e-3) / 1e9 / peak
    res[pre + "lbvh_bounds"] = [round(v, 3) for v in bounds]
    res[pre + "schedule"] = knobs
    del g, bv
    et.release()
    return res


def c4_step(f, dev):
    """Differentiable facade fitting (1024 facades, 16 parameters each): the
    target is the same trees with every parameter moved by N(0, 0.02) and
    clamped so no branch flips; one step is the forward derivation through
    torch.autograd, the SSE of terminal centres and extents matched by path,
    and the backward pass (the adjoint), then an Adam update.  Timed with CUDA
    events around whole steps."""
    import torch

    from operatorgraph_gb300.autograd import PathTarget, axioms_tensor, derive_transforms
    from operatorgraph_gb300.engine import Engine

    n_f = len(f["axioms"]) * 384
    ef = Engine(f["entries"], node_capacity=1 << 20, max_terminals=1 << 20, block_stride=f["block_stride"],
                record_tape=True)
    d_ax = axioms_tensor(f["axioms"], dev)
    sizes = torch.tensor(f["axioms"]["size"], dtype=torch.float32, device=dev)
    tb = torch.tensor(scenes.facade_target_params(f["blocks"]), dtype=torch.float32, device=dev)
    Mt, pt = derive_transforms(ef, d_ax, tb, sizes, n_f)
    target = PathTarget(Mt, pt)
    blocks = torch.tensor(f["blocks"], dtype=torch.float32, device=dev, requires_grad=True)
    opt = torch.optim.Adam([blocks], lr=2e-3)

    def step():
        opt.zero_grad()
        M, paths = derive_transforms(ef, d_ax, blocks, sizes, n_f)
        loss = target.sse(M, paths, check=False)
        loss.backward()
        opt.step()
        return loss.detach()

    losses = [float(step()) for _ in range(3)]
    ts = []
    for _ in range(10):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record()
        loss = step()
        b.record()
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
        losses.append(float(loss))
    M, paths = derive_transforms(ef, d_ax, blocks.detach(), sizes, n_f)
    target.sse(M, paths, check=True)  # still the target's trees
    ef.release()
    return {"facades1024_c4_step_ms": statistics.median(ts), "facades1024_c4_loss_first": losses[0],
            "facades1024_c4_loss_last": losses[-1], "facades1024_c4_steps": len(losses)}


def extras(eng, batch, out, n_term, dev, stream, flush):
    """Plain GPU form, Menger depth 5 and LBVH timings (reported beside the headline)."""
    import torch

    from operatorgraph_gb300.engine import Engine

    res = {}
    n_ax = len(batch["axioms"])
    d_ax = torch.from_numpy(batch["axioms"].view(np.uint8).copy()).to(dev)
    count = torch.zeros(1, dtype=torch.int64, device=dev)
    peak, _ = read_peaks()
    # The one-grammar-per-launch GPU form: pga_derive_per_axiom, one persistent
    # launch per axiom (4,096 launches, the batched kernel and schedule, each
    # axiom's records appended on the device), enqueued back to back with no
    # host read-back; timed eagerly and as one captured CUDA graph, CUDA
    # events over 5 repeats each.  The batched/plain ratio uses the faster.
    def per_axiom(st):
        eng.derive_raw(d_ax.data_ptr(), n_ax, None, out.data_ptr(), out.shape[0], count.data_ptr(), stream=st,
                       plain="per_axiom")

    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        per_axiom(side)  # allocates the staging buffer
        side.synchronize()
        assert int(count.item()) == n_term and eng.report(side)["status"] == 0
        ts = []
        for _ in range(5):
            flush.fill_(5)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(side)
            per_axiom(side)
            b.record(side)
            side.synchronize()
            ts.append(a.elapsed_time(b))
    torch.cuda.current_stream().wait_stream(side)
    res["plain_per_axiom_eager_ms"] = statistics.median(ts)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        per_axiom(torch.cuda.current_stream())
    ts = []
    for _ in range(5):
        flush.fill_(6)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        g.replay()
        b.record(stream)
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
    assert int(count.item()) == n_term
    del g
    res["plain_per_axiom_graph_ms"] = statistics.median(ts)
    plain_ms = min(res["plain_per_axiom_eager_ms"], res["plain_per_axiom_graph_ms"])
    res["plain_city_terminals_per_s"] = n_term / (plain_ms * 1e-3)
    res["plain_city_roofline_frac"] = (64.0 * n_term + 48.0 * n_ax) / (plain_ms * 1e-3) / 1e9 / peak
    res["plain_form"] = "pga_derive_per_axiom: one persistent launch per axiom, no host read-back"
    # The naive form for comparison: pga_derive_plain, one launch per level of
    # each axiom with the level size read back to the host (one timed call).
    eng.derive_raw(d_ax.data_ptr(), n_ax, None, out.data_ptr(), out.shape[0], count.data_ptr(), plain=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    eng.derive_raw(d_ax.data_ptr(), n_ax, None, out.data_ptr(), out.shape[0], count.data_ptr(), plain=True)
    torch.cuda.synchronize()
    assert int(count.item()) == n_term
    res["naive_host_driven_terminals_per_s"] = n_term / (time.perf_counter() - t0)
    # Restore the batched output for the LBVH below.
    eng.derive_raw(d_ax.data_ptr(), n_ax, None, out.data_ptr(), out.shape[0], count.data_ptr())
    torch.cuda.synchronize()
    # LBVH over the city's terminals.
    bounds = (-50.0, -50.0, -1.0, 3250.0, 3250.0, 400.0)
    for _ in range(2):
        eng.lbvh(out, n_term, bounds)
    ts = []
    for _ in range(5):
        flush.fill_(1)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        eng.lbvh(out, n_term, bounds)
        b.record(stream)
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
    lb = statistics.median(ts)
    res["lbvh_city_ms"] = lb
    res["lbvh_city_leaves_per_s"] = n_term / (lb * 1e-3)
    # Menger sponge, depth 5 (3.2M terminals), one axiom in one launch.
    m = scenes.menger(0.005)
    em = Engine(m["entries"], node_capacity=1 << 22, max_terminals=4_000_000)
    d_m = torch.from_numpy(m["axioms"].view(np.uint8).copy()).to(dev)
    for _ in range(3):
        em.derive_raw(d_m.data_ptr(), 1, None, out.data_ptr(), out.shape[0], count.data_ptr())
    ts = []
    for _ in range(5):
        flush.fill_(2)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        em.derive_raw(d_m.data_ptr(), 1, None, out.data_ptr(), out.shape[0], count.data_ptr())
        b.record(stream)
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
    assert int(count.item()) == 3_200_000
    res["menger_d5_ms"] = statistics.median(ts)
    res["menger_d5_terminals_per_s"] = 3.2e6 / (res["menger_d5_ms"] * 1e-3)
    # Its LBVH over all 3.2M terminals (30-bit Morton codes on the unit-cube bounds).
    ts = []
    for it in range(6):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        em.lbvh(out, 3_200_000, (-0.5, -0.5, -0.5, 0.5, 0.5, 0.5), stream=stream)
        b.record(stream)
        torch.cuda.synchronize()
        if it >= 2:
            ts.append(a.elapsed_time(b))
    res["lbvh_menger_d5_ms"] = statistics.median(ts)
    res["menger_d5_with_lbvh_ms"] = res["menger_d5_ms"] + res["lbvh_menger_d5_ms"]
    em.release()
    # Facades (1024 axioms x 16 block parameters, 393,216 terminals): derivation
    # with the tape recorded, then the adjoint to the block parameters and sizes.
    f = scenes.facades(1024)
    ef = Engine(f["entries"], node_capacity=1 << 20, max_terminals=1 << 20, block_stride=f["block_stride"],
                record_tape=True)
    d_f = torch.from_numpy(f["axioms"].view(np.uint8).copy()).to(dev)
    d_blk = torch.from_numpy(f["blocks"]).to(dev)
    n_f = 1024 * 384
    g_term = torch.randn((n_f, 12), dtype=torch.float32, device=dev)
    g_blk = torch.empty_like(d_blk)
    g_sz = torch.empty((1024, 3), dtype=torch.float32, device=dev)
    fw, bw = [], []
    for it in range(8):
        flush.fill_(3)
        a, b, c = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        a.record(stream)
        ef.derive_raw(d_f.data_ptr(), 1024, d_blk.data_ptr(), out.data_ptr(), out.shape[0], count.data_ptr())
        b.record(stream)
        ef.adjoint_raw(g_term.data_ptr(), g_blk.data_ptr(), 1024, g_sz.data_ptr())
        c.record(stream)
        torch.cuda.synchronize()
        if it >= 3:
            fw.append(a.elapsed_time(b))
            bw.append(b.elapsed_time(c))
    assert int(count.item()) == n_f
    res["facades1024_forward_tape_ms"] = statistics.median(fw)
    res["facades1024_adjoint_ms"] = statistics.median(bw)
    # Algorithmic bytes of the adjoint: per terminal the 48-B gradient and the
    # 64-B record's tape link (8 B); per queued item its 64-B record read twice
    # (replay of the parent and of itself) and 24 B of gradient written and read;
    # per parameter and axiom size 4 B written.
    n_items = ef.report()["nodes"]
    adj_bytes = n_f * (48 + 8) + n_items * (2 * 64 + 2 * 24) + 4 * (d_blk.numel() + 3 * 1024)
    peak, _ = read_peaks()
    res["facades1024_adjoint_items"] = int(n_items)
    res["facades1024_adjoint_gbs"] = adj_bytes / (res["facades1024_adjoint_ms"] * 1e-3) / 1e9
    res["facades1024_adjoint_roofline_frac"] = res["facades1024_adjoint_gbs"] / peak
    res["facades1024_fwd_adjoint_step_ms"] = res["facades1024_forward_tape_ms"] + res["facades1024_adjoint_ms"]
    ef.release()
    res.update(c4_step(f, dev))
    del out
    # The mixed batch: 65,536 axioms (40 % Menger depth 1-3, 40 % city
    # buildings, 20 % random grammars), about 152M terminals in one launch.
    # The axioms are interleaved by kind; the engine seeds them grouped by root
    # entry (PGA_FLAG_GROUP_AXIOMS).  The index-order time is kept beside it.
    mx = scenes.mixed(65536)
    mcap = 160_000_000
    d_mx = torch.from_numpy(mx["axioms"].view(np.uint8).copy()).to(dev)
    mout = torch.empty((mcap, 64), dtype=torch.uint8, device=dev)
    # Schedule: a sweep of the split knobs and of the rule-to-warp grouping
    # (axioms grouped by root entry), against the engine's defaults.
    from operatorgraph_gb300 import autotune

    mspace = {"sub_item": (4, 8), "narrow_sub_item": (0, 2), "items_per_lane": (1,), "blocks_per_sm": (0,),
              "dynamic_chunks": (False, True)}
    mbest, mms, mres = autotune.tune(mx, mcap, node_capacity=1 << 27, space=mspace, runs=3)
    res["mixed65536_schedule"] = mbest
    res["mixed65536_default_ms"] = next((r["ms"] for r in mres if autotune.is_default(r["config"])), None)
    res["mixed65536_index_order_ms"] = min(r["ms"] for r in mres
                                           if r["ms"] is not None and not r["config"]["group_axioms"])
    em = Engine(mx["entries"], node_capacity=1 << 27, max_terminals=mcap, **mbest)
    em.derive_raw(d_mx.data_ptr(), 65536, None, mout.data_ptr(), mcap, count.data_ptr())
    rep = em.report()
    assert rep["status"] == 0, rep
    em.release()
    n_mx = int(count.item())
    res["mixed65536_terminals"] = n_mx
    res["mixed65536_ms"] = mms
    res["mixed65536_terminals_per_s"] = n_mx / (res["mixed65536_ms"] * 1e-3)
    dyn, order_ms = step_order(len(mx["axioms"]), mout, count, dev, mbest)
    res["mixed65536_step_order_ms"] = {"static": order_ms[False], "dynamic": order_ms[True]}
    sched = dict(mbest, dynamic_chunks=dyn)
    res.update(mixed_step(len(mx["axioms"]), mout, count, dev, n_mx, blocks=True, schedule=sched))
    res.update(mixed_step(len(mx["axioms"]), mout, count, dev, n_mx, blocks=False, schedule=sched))
    del mout
    # Forest: 4096 trees (Rotate with arbitrary angles, Replicate, Translate,
    # Scale: the general-frame kernels), about 13.4M terminals in one launch.
    fo = scenes.forest(4096)
    fcap = 14_000_000
    # The forest's forks have four children and its first levels are narrow:
    # a short autotune over the split knobs (the city's sweep, reduced).
    from operatorgraph_gb300 import autotune

    fbest, fms, fres = autotune.tune(fo, fcap, node_capacity=1 << 23, runs=3,
                                     space={"sub_item": (1, 2, 4, 8), "narrow_sub_item": (0, 1), "items_per_lane": (1,),
                                            "blocks_per_sm": (0,), "dynamic_chunks": (False, True)})
    res["forest4096_schedule"] = fbest
    res["forest4096_tuned_ms"] = fms
    res["forest4096_default_ms"] = next((r["ms"] for r in fres if autotune.is_default(r["config"])), None)
    eo = Engine(fo["entries"], node_capacity=1 << 23, max_terminals=fcap, **fbest)
    d_fo = torch.from_numpy(fo["axioms"].view(np.uint8).copy()).to(dev)
    fout = torch.empty((fcap, 64), dtype=torch.uint8, device=dev)
    ts = []
    for it in range(7):
        flush.fill_(3)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        eo.derive_raw(d_fo.data_ptr(), 4096, None, fout.data_ptr(), fcap, count.data_ptr())
        b.record(stream)
        torch.cuda.synchronize()
        if it >= 2:
            ts.append(a.elapsed_time(b))
    rep = eo.report()
    assert rep["status"] == 0, rep
    n_fo = int(count.item())
    res["forest4096_terminals"] = n_fo
    res["forest4096_ms"] = statistics.median(ts)
    res["forest4096_terminals_per_s"] = n_fo / (res["forest4096_ms"] * 1e-3)
    res["forest4096_roofline_frac"] = 64.0 * n_fo / (res["forest4096_ms"] * 1e-3) / 1e9 / peak
    eo.release()
    del fout
    # Triangle meshes of the city (walls, windows and roofs as triangle-mesh
    # terminals: 5.86M quads): pga_generate_meshes alone, from derived records.
    cm = scenes.city(4096, meshes=True)
    ec = Engine(cm["entries"], node_capacity=1 << 22, max_terminals=6_000_000)
    d_cm = torch.from_numpy(cm["axioms"].view(np.uint8).copy()).to(dev)
    cout = torch.empty((6_000_000, 64), dtype=torch.uint8, device=dev)
    ec.derive_raw(d_cm.data_ptr(), 4096, None, cout.data_ptr(), 6_000_000, count.data_ptr())
    torch.cuda.synchronize()
    n_cm = int(count.item())
    caps = [(4 * n_cm, 6 * n_cm)] * 3
    vbufs = [torch.empty((mv, 48), dtype=torch.uint8, device=dev) for mv, _ in caps]
    ibufs = [torch.empty((mi,), dtype=torch.int32, device=dev) for _, mi in caps]
    table = np.array([(0, 0, mv, mi, v.data_ptr(), i.data_ptr()) for (mv, mi), v, i in zip(caps, vbufs, ibufs)],
                     dtype=G.MESH_DT)
    d_table = torch.from_numpy(table.view(np.uint8).copy()).to(dev)
    ts = []
    for it in range(8):
        d_table.view(-1, 32)[:, :8].zero_()  # numVertices, numIndices
        flush.fill_(4)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ec.generate_meshes_raw(cout.data_ptr(), n_cm, d_table.data_ptr(), 3, stream)
        b.record(stream)
        torch.cuda.synchronize()
        if it >= 3:
            ts.append(a.elapsed_time(b))
    rep = ec.report()
    assert rep["status"] == 0, rep
    nv = int(d_table.cpu().numpy().view(G.MESH_DT)["numVertices"].sum())
    assert nv == 4 * n_cm, (nv, n_cm)
    mesh_bytes = 64.0 * n_cm + 48.0 * nv + 4.0 * 1.5 * nv
    res["city_meshes_quads"] = n_cm
    res["city_meshes_ms"] = statistics.median(ts)
    res["city_meshes_gbs"] = mesh_bytes / (res["city_meshes_ms"] * 1e-3) / 1e9
    res["city_meshes_roofline_frac"] = res["city_meshes_gbs"] / peak
    ec.release()
    del cout, vbufs, ibufs
    # Two-phase derivation with colliders (scenes.collisions: 4096 buildings and
    # 4096 billboards stored in phase 0, 65,536 turned trees tested against
    # them in phase 1): the whole pga_derive, host round trip and collider
    # LBVH between the phases included.
    co = scenes.collisions(4096, 65536, 4096, rotate=True)
    ek = Engine(co["entries"], node_capacity=1 << 20, max_terminals=1 << 20)
    d_co = torch.from_numpy(co["axioms"].view(np.uint8).copy()).to(dev)
    kout = torch.empty((1 << 20, 64), dtype=torch.uint8, device=dev)
    ts = []
    for it in range(6):
        t0 = time.perf_counter()
        ek.derive_raw(d_co.data_ptr(), len(co["axioms"]), None, kout.data_ptr(), 1 << 20, count.data_ptr())
        torch.cuda.synchronize()
        if it >= 2:
            ts.append((time.perf_counter() - t0) * 1e3)
    rep = ek.report()
    assert rep["status"] == 0, rep
    res["collisions_trees"] = 65536
    res["collisions_terminals"] = int(count.item())
    res["collisions_ms"] = statistics.median(ts)
    res["collisions_trees_per_s"] = 65536 / (res["collisions_ms"] * 1e-3)
    ek.release()
    del kout
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--schedule", default="",
                    help="fixed engine knobs instead of autotuning, e.g. sub_item=16,narrow_sub_item=2")
    args = ap.parse_args()
    if args.impl == "reference":
        reference_arm(args)
    else:
        our_arm(args)


if __name__ == "__main__":
    main()
