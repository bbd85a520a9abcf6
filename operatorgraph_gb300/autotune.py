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

Every candidate derives the batch `runs` times (CUDA events, after a warm-up);
a candidate whose derivation reports a non-OK status (e.g. the finer splits
overflow the item arena) is discarded.  The result is the fastest candidate's
configuration, ready for Engine(**config).
"""
import argparse
import itertools
import json
import statistics

import numpy as np

DEFAULT_SPACE = {
    "sub_item": (4, 8, 16),
    "narrow_sub_item": (0, 2, 4),  # 0: same as sub_item
    "items_per_lane": (1, 2),
    "blocks_per_sm": (0, 1),      # 0: occupancy maximum
}


# The engine's built-in defaults, as a point of the space.
DEFAULT_CONFIG = {"sub_item": 8, "narrow_sub_item": 0, "items_per_lane": 1, "blocks_per_sm": 0}


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
