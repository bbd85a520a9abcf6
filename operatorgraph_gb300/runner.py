"""Command-line runner for the synthetic scenes (the role of the reference's
test_runner app, src/test_runner/TestRunnerApp.cpp:303-345: derive a scene a
number of times and log timings).

    python -m operatorgraph_gb300.runner --scene city --runs 5 [--plain | --per-axiom] [--lbvh] [--step]
                                         [--meshes] [--blocks]

Prints one JSON line: terminals, per-run milliseconds (CUDA events) and the
device report of the last run.  --meshes (city) makes walls, windows and roofs
triangle-mesh terminals and runs pga_generate_meshes after each derivation;
--blocks (mixed) gives the axioms parameter blocks (scenes.mixed(blocks=True));
--per-axiom derives with one persistent launch per axiom.  --step runs the differentiable step after
each derivation (made with the tape recorded): the LBVH over the device-side
terminal count, then the adjoint to the block parameters and axiom sizes for
L = |M|^2 / 2, reading dL/dM = M in place from the terminal records
(pga_adjoint_strided, stride 16 floats), each part timed.
"""
import argparse
import json
import statistics

import numpy as np

from . import scenes


def make_scene(name, n, meshes=False, blocks=False):
    if name == "city":
        return scenes.city(n or 4096, meshes=meshes), (-50.0, -50.0, -1.0, 3250.0, 3250.0, 400.0)
    if name == "menger":
        return scenes.menger({1: 0.5, 2: 0.15, 3: 0.05, 4: 0.015, 5: 0.005}[n or 5]), (-0.5, -0.5, -0.5, 0.5, 0.5, 0.5)
    if name == "facades":
        return scenes.facades(n or 1024), (-1.0, -1.0, -1.0, 70.0, 2.0, 70.0)
    if name == "mixed":
        return scenes.mixed(n or 65536, blocks=blocks), (-50.0, -50.0, -110.0, 13000.0, 13000.0, 400.0)
    raise SystemExit(f"unknown scene {name}")


def main(argv=None):
    import torch

    from .engine import Engine

    ap = argparse.ArgumentParser()
    ap.add_argument("--scene", default="city", choices=["city", "menger", "facades", "mixed"])
    ap.add_argument("--n", type=int, default=0, help="axioms (city/facades/mixed) or depth (menger)")
    ap.add_argument("--runs", type=int, default=3)
    ap.add_argument("--plain", action="store_true", help="plain one-grammar-per-launch form")
    ap.add_argument("--lbvh", action="store_true", help="also build the LBVH after each derivation")
    ap.add_argument("--step", action="store_true",
                    help="differentiable step: tape, LBVH over the device count, dL/dM = M, adjoint")
    ap.add_argument("--capacity", type=int, default=0)
    ap.add_argument("--nodes", type=int, default=1 << 22)
    ap.add_argument("--sub-item", type=int, default=0, help="children per work item (engine default 8)")
    ap.add_argument("--items-per-lane", type=int, default=0, help="work items per lane per chunk (default 2)")
    ap.add_argument("--narrow-sub-item", type=int, default=0,
                    help="children per work item queued from levels narrower than the grid (default subItem)")
    ap.add_argument("--blocks-per-sm", type=int, default=0, help="cap on resident blocks per SM (0: occupancy)")
    ap.add_argument("--group", action="store_true", help="seed the axioms grouped by root entry")
    ap.add_argument("--dynamic", action="store_true",
                    help="the last quarter of each level's items from a shared counter (PGA_FLAG_DYNAMIC_CHUNKS)")
    ap.add_argument("--per-axiom", action="store_true", help="one persistent launch per axiom (pga_derive_per_axiom)")
    ap.add_argument("--meshes", action="store_true", help="city: triangle-mesh terminals, then pga_generate_meshes")
    ap.add_argument("--blocks", action="store_true", help="mixed: per-axiom parameter blocks")
    args = ap.parse_args(argv)

    b, bounds = make_scene(args.scene, args.n, meshes=args.meshes, blocks=args.blocks)
    cap = args.capacity or 8_000_000
    eng = Engine(b["entries"], node_capacity=args.nodes, max_terminals=cap, block_stride=b["block_stride"],
                 sub_item=args.sub_item, items_per_lane=args.items_per_lane, blocks_per_sm=args.blocks_per_sm,
                 narrow_sub_item=args.narrow_sub_item, record_tape=args.step, group_axioms=args.group,
                 dynamic_chunks=args.dynamic)
    dev = torch.device("cuda", torch.cuda.current_device())
    d_ax = torch.from_numpy(b["axioms"].view(np.uint8).copy()).to(dev)
    d_blk = None if b["blocks"] is None else torch.from_numpy(np.asarray(b["blocks"], np.float32)).to(dev)
    out = torch.empty((cap, 64), dtype=torch.uint8, device=dev)
    count = torch.zeros(1, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream()
    n_ax = len(b["axioms"])
    if args.step:
        g_sz = torch.empty((n_ax, 3), dtype=torch.float32, device=dev)
        g_blk = None if d_blk is None else torch.empty_like(d_blk)
        n_blk = 0 if d_blk is None else d_blk.numel() // max(b["block_stride"], 1)
    times, lb, steps, mesh_ms = [], [], [], []
    form = "per_axiom" if args.per_axiom else args.plain
    for _ in range(args.runs):
        a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        eng.derive_raw(d_ax.data_ptr(), len(b["axioms"]), None if d_blk is None else d_blk.data_ptr(),
                       out.data_ptr(), cap, count.data_ptr(), plain=form)
        z.record(stream)
        torch.cuda.synchronize()
        times.append(a.elapsed_time(z))
        if args.lbvh:
            n = int(count.item())
            a.record(stream)
            eng.lbvh(out, n, bounds)
            z.record(stream)
            torch.cuda.synchronize()
            lb.append(a.elapsed_time(z))
        if args.meshes:
            n = int(count.item())
            a.record(stream)
            eng.generate_meshes(out, n, [(4 * n, 6 * n)] * 3)
            z.record(stream)
            torch.cuda.synchronize()
            mesh_ms.append(a.elapsed_time(z))
        if args.step:
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            ev[0].record(stream)
            eng.lbvh(out, cap, bounds, stream=stream, count=count)
            ev[1].record(stream)
            eng.adjoint_raw(out.data_ptr(), None if g_blk is None else g_blk.data_ptr(), n_blk, g_sz.data_ptr(),
                            stream=stream, grad_stride=16)
            ev[2].record(stream)
            torch.cuda.synchronize()
            steps.append({"lbvh_ms": ev[0].elapsed_time(ev[1]), "adjoint_ms": ev[1].elapsed_time(ev[2])})
    rep = eng.report()
    lv = {}
    if not args.plain and not args.per_axiom:
        starts, nanos = eng.levels()
        nanos = nanos.astype(np.int64)
        d = np.diff(nanos) / 1e3
        lv = {"level_nodes": np.diff(starts.astype(np.int64)).tolist(),
              "seed_us": round(float(d[0]), 2), "level_us": d[1:-1].round(2).tolist(),
              "compact_us": round(float(d[-1]), 2)}
    res = {"scene": args.scene, "n": args.n, "plain": args.plain, "sub_item": args.sub_item,
           "items_per_lane": args.items_per_lane, "narrow_sub_item": args.narrow_sub_item,
           "terminals": int(count.item()),
           "ms": times, "ms_median": statistics.median(times), "report": rep, **lv}
    if lb:
        res["lbvh_ms"] = lb
    if mesh_ms:
        res["meshes_ms"] = mesh_ms
    if steps:
        res["step"] = steps
    print(json.dumps(res))
    eng.release()


if __name__ == "__main__":
    main()
