"""Per-grammar schedule autotuner for the batched engine.

The reference picks a schedule per grammar offline: its operator-graph
analyzer partitions the grammar and a Windows auto-tuner compiles and times
each candidate (src/compiler, src/analyzer; MSBuild per schedule).  Here the
schedule is a handful of engine knobs, so tuning is a timed sweep at run time:

  subItem        children per queued work item (parallelism vs item traffic)
  narrowSubItem  the same for levels narrower than the grid
  itemsPerLane   work items a lane takes per warp chunk
  blocksPerSM    resident blocks per SM of the persistent launch
  groupAxioms    rule-to-warp grouping: seed the axioms grouped by root entry
                 (PGA_FLAG_GROUP_AXIOMS); searched only for batches whose
                 axioms use more than one root entry
  dynamicChunks  the last quarter of each wide level's items from a shared
                 counter instead of the static grid-stride order
                 (PGA_FLAG_DYNAMIC_CHUNKS): pays where items differ in cost

Every candidate derives the batch `runs` times (CUDA events, after a warm-up);
a candidate whose derivation reports a non-OK status (e.g. the finer splits
overflow the item arena) is discarded.  The result is the fastest candidate's
configuration, ready for Engine(**config).

Threads per block is not a knob: every kernel is compiled for 256 (its block
scans and the output compaction's shared-memory tables are sized for it), and
the persistent kernel's 128 registers fix the warps per SM at 16 whatever the
block size; the grid's shape is searched through blocksPerSM.

`size_capacities` sizes the item arena and the terminal capacity from one
counting derivation (statuses report the full counts, so an undersized first
guess is grown and retried), and `tune_cached` keeps the best schedule on disk
per (rule table, batch signature, GPU name, library version).
"""
import argparse
import hashlib
import itertools
import json
import os
import statistics

import numpy as np

DEFAULT_SPACE = {
    "sub_item": (4, 8, 16),
    "narrow_sub_item": (0, 2, 4),  # 0: same as sub_item
    "items_per_lane": (1, 2),
    "blocks_per_sm": (0, 1),      # 0: occupancy maximum
    "dynamic_chunks": (False, True),
}


# The engine's built-in defaults, as a point of the space.
DEFAULT_CONFIG = {"sub_item": 8, "narrow_sub_item": 0, "items_per_lane": 1, "blocks_per_sm": 0, "dynamic_chunks": False}


def is_default(config):
    """Whether `config` is the engine's default schedule: every knob of
    DEFAULT_CONFIG at its default (a knob the config leaves out counts as
    default) and no axiom grouping."""
    return (all(config.get(k, v) == v for k, v in DEFAULT_CONFIG.items())
            and not config.get("group_axioms", False))


def space_for(batch, space=None):
    """The search space for `batch`: `space` (default DEFAULT_SPACE), plus the
    axiom grouping knob when the batch's axioms use more than one root entry
    (a one-grammar batch gains nothing from it)."""
    sp = dict(DEFAULT_SPACE if space is None else space)
    if batch is not None and "group_axioms" not in sp and len(np.unique(np.asarray(batch["axioms"]["entry"]))) > 1:
        sp["group_axioms"] = (False, True)
    return sp


def candidates(space=None):
    """All knob combinations of `space` (dict name -> values), duplicates removed."""
    space = dict(DEFAULT_SPACE if space is None else space)
    names = sorted(space)
    seen, out = set(), []
    for values in itertools.product(*(space[n] for n in names)):
        c = dict(zip(names, values))
        if c.get("narrow_sub_item", 0) == c.get("sub_item", 0):
            c["narrow_sub_item"] = 0
        key = tuple(sorted(c.items()))
        if key not in seen:
            seen.add(key)
            out.append(c)
    return out


def select(results):
    """The fastest successful result: (config, ms), or raises if none succeeded."""
    ok = [r for r in results if r["status"] == 0 and r["ms"] is not None]
    if not ok:
        raise RuntimeError("autotune: no candidate configuration derived the batch")
    best = min(ok, key=lambda r: (r["ms"], r["index"]))
    return best["config"], best["ms"]


def measure(batch, config, capacity, node_capacity, runs=5, warmup=2):
    """Median milliseconds of pga_derive on `batch` with engine knobs `config`,
    and the device status of the last run."""
    import torch

    from .engine import Engine

    eng = Engine(batch["entries"], node_capacity=node_capacity, max_terminals=capacity,
                 block_stride=batch.get("block_stride", 0), **config)
    try:
        d_ax = torch.from_numpy(np.ascontiguousarray(batch["axioms"]).view(np.uint8).copy()).cuda()
        d_blk = None
        if batch.get("blocks") is not None:
            d_blk = torch.from_numpy(np.asarray(batch["blocks"], np.float32)).cuda()
        out = torch.empty((capacity, 64), dtype=torch.uint8, device="cuda")
        count = torch.zeros(1, dtype=torch.int64, device="cuda")
        n_ax = len(batch["axioms"])
        stream = torch.cuda.current_stream()

        def run():
            eng.derive_raw(d_ax.data_ptr(), n_ax, None if d_blk is None else d_blk.data_ptr(), out.data_ptr(),
                           capacity, count.data_ptr())

        for _ in range(warmup):
            run()
        status = eng.report()["status"]
        if status != 0:
            return None, status
        ts = []
        for _ in range(runs):
            a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            run()
            z.record(stream)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(z))
        return statistics.median(ts), eng.report()["status"]
    finally:
        eng.release()


def tune(batch, capacity, node_capacity=1 << 22, space=None, runs=5, measure_fn=None):
    """Times every candidate of `space` on `batch`; returns (best config, best ms, all results)."""
    measure_fn = measure_fn or (lambda cfg: measure(batch, cfg, capacity, node_capacity, runs=runs))
    results = []
    for i, cfg in enumerate(candidates(space_for(batch, space))):
        ms, status = measure_fn(cfg)
        results.append({"index": i, "config": cfg, "ms": ms, "status": int(status)})
    best, ms = select(results)
    return best, ms, results


def size_capacities(batch, node_capacity=1 << 20, max_terminals=1 << 20, margin=0.05, limit=1 << 31, config=None):
    """Item-arena and terminal capacities for `batch`: derives it once with
    the given capacities, doubling whichever the device status says was too
    small (the counts keep counting past it), then returns the counts plus
    `margin`: {"node_capacity": ..., "max_terminals": ...}."""
    import torch

    from .engine import Engine

    config = dict(config or {})
    d_ax = torch.from_numpy(np.ascontiguousarray(batch["axioms"]).view(np.uint8).copy()).cuda()
    d_blk = None
    if batch.get("blocks") is not None:
        d_blk = torch.from_numpy(np.asarray(batch["blocks"], np.float32)).cuda()
    count = torch.zeros(1, dtype=torch.int64, device="cuda")
    while True:
        eng = Engine(batch["entries"], node_capacity=node_capacity, max_terminals=max_terminals,
                     block_stride=batch.get("block_stride", 0), **config)
        out = torch.empty((max_terminals, 64), dtype=torch.uint8, device="cuda")
        try:
            eng.derive_raw(d_ax.data_ptr(), len(batch["axioms"]), None if d_blk is None else d_blk.data_ptr(),
                           out.data_ptr(), max_terminals, count.data_ptr())
            rep = eng.report()
        finally:
            eng.release()
        del out
        if rep["status"] == 1 and node_capacity < limit:  # queue overflow
            node_capacity *= 2
            continue
        if rep["status"] == 2 and max_terminals < limit:  # output overflow: the report holds the full count
            max_terminals = max(2 * max_terminals, int(rep["terminals"]))
            continue
        if rep["status"] != 0:
            raise RuntimeError(f"size_capacities: device status {rep['status']}")
        grow = lambda x: int(min(limit, max(1024, x * (1.0 + margin))))
        return {"node_capacity": grow(rep["nodes"]), "max_terminals": grow(rep["terminals"])}


def schedule_key(batch, gpu_name, library_version=""):
    """Cache key of a batch's schedule: the rule table's bytes, the batch's
    signature (axiom count and the histogram of root entries), the GPU name and
    the library version."""
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(batch["entries"]).view(np.uint8).tobytes())
    ax = np.asarray(batch["axioms"])
    roots, counts = np.unique(np.asarray(ax["entry"]), return_counts=True)
    h.update(np.asarray([len(ax)], np.int64).tobytes() + roots.astype(np.int64).tobytes() +
             counts.astype(np.int64).tobytes())
    h.update(gpu_name.encode() + b"|" + library_version.encode())
    return h.hexdigest()[:32]


def default_cache_dir():
    return os.environ.get("PGA_SCHEDULE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "pga_gb300")


def tune_cached(batch, capacity, node_capacity=1 << 22, space=None, runs=5, cache_dir=None, gpu_name=None,
                library_version=None, measure_fn=None):
    """tune() with the best schedule kept on disk per schedule_key: a hit
    returns (config, ms, [] , True) without timing anything; a miss tunes,
    stores and returns (config, ms, results, False)."""
    if gpu_name is None or library_version is None:
        import torch

        from .engine import load_library

        gpu_name = gpu_name or torch.cuda.get_device_name()
        library_version = library_version or load_library().pga_version().decode()
    cache_dir = cache_dir or default_cache_dir()
    path = os.path.join(cache_dir, schedule_key(batch, gpu_name, library_version) + ".json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return d["config"], d["ms"], [], True
    best, ms, results = tune(batch, capacity, node_capacity, space=space, runs=runs, measure_fn=measure_fn)
    os.makedirs(cache_dir, exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump({"config": best, "ms": ms, "gpu": gpu_name, "version": library_version}, f)
    os.replace(tmp, path)
    return best, ms, results, False


def main(argv=None):
    from . import runner

    ap = argparse.ArgumentParser(description="Tune the batched engine's knobs for a scene")
    ap.add_argument("--scene", default="city", choices=["city", "menger", "facades", "mixed"])
    ap.add_argument("--n", type=int, default=0)
    ap.add_argument("--capacity", type=int, default=8_000_000)
    ap.add_argument("--nodes", type=int, default=1 << 22)
    ap.add_argument("--runs", type=int, default=5)
    args = ap.parse_args(argv)
    batch, _ = runner.make_scene(args.scene, args.n)
    best, ms, results = tune(batch, args.capacity, args.nodes, runs=args.runs)
    print(json.dumps({"scene": args.scene, "best": best, "ms": ms, "results": results}))


if __name__ == "__main__":
    main()
