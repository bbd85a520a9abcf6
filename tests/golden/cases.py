"""Grammar batches with golden outputs produced by the reference's own evaluator.

Each case is (name, batch) where batch is a scenes-style dict.  The fixtures
(tests/golden/<name>.npz) are written by make_golden.py, which runs the
reference's SinglePhaseEvaluator (oracle/_ref/ref_harness) on each batch.
"""
import numpy as np

from operatorgraph_gb300 import grammar as G
from operatorgraph_gb300 import scenes
from operatorgraph_gb300.grammar import DispatchTable, Entry, Parameter, rand, scalar, shape_attr


def _single(table, axioms, name):
    return {"entries": table, "axioms": axioms, "blocks": None, "block_stride": 0, "name": name}


def edge_repeat(mode, ext):
    """Box Repeat with relative/absolute extents feeding a Subdivide<DynParams>
    whose factors read the seed and a random range (the in-place quirk of
    Subdivide.cuh:220-235), two axioms, one with a seed >= 1."""
    tab = DispatchTable([
        Entry(G.BOX_REPEAT, [scalar(0), scalar(ext), scalar(mode)], [(1, 0)]),
        Entry(G.BOX_SUBDIVIDE, [scalar(1), rand(-2, -1), Parameter(G.PT_SHAPE_ATTR, (15,)), scalar(-1), scalar(0.1)],
              [(2, 0), (3, 0), (2, 0), (3, 0)]),
        Entry(G.BOX_GENERATE, [scalar(0)], []),
        Entry(G.BOX_REPEAT, [scalar(2), scalar(0.7), scalar(mode)], [(2, 0)]),
    ]).to_array()
    ax = G.make_axioms(2)
    ax["size"] = [(2.5, 3.0, 1.9), (1.0, 4.0, 0.3)]
    ax["seed"] = [0.5, 1.7]
    return _single(tab, ax, f"edge_repeat_m{mode}_{str(ext).replace('-', 'n').replace('.', 'p')}")


def edge_static_zero():
    """Static 3-pair Subdivide with a zero factor (skipped, Subdivide.cuh:49-67)
    and an absolute factor, on a Quad, with Extrude and IfSizeLess chains."""
    tab = DispatchTable([
        Entry(G.QUAD_SUBDIVIDE3, [scalar(1), scalar(0.5), scalar(0), scalar(-2)], [(1, 0), (2, 0), (1, 0)]),
        Entry(G.QUAD_EXTRUDE, [scalar(1), scalar(0.75)], [(3, 0)]),
        Entry(G.QUAD_GENERATE, [scalar(1)], []),
        Entry(G.BOX_IF_SIZE_LESS, [scalar(1), shape_attr(12)], [(4, 0), (5, 0)]),
        Entry(G.BOX_GENERATE, [scalar(2)], []),
        Entry(G.BOX_COMPONENT_SPLIT, [], [(2, 0), (6, 0), (2, 0)]),
        Entry(G.QUAD_DISCARD, [], []),
    ]).to_array()
    ax = G.make_axioms(3)
    ax["shape"] = G.SHAPE_QUAD
    ax["size"] = [(1.0, 3.0, 1.0), (0.6, 1.0, 1.0), (2.0, 5.0, 1.0)]
    ax["position"] = [(0, 0, 0), (3, -2, 1), (-4, 5, -6)]
    ax["seed"] = 0.25
    ax["custom"] = [1.0, 2.0, 3.0]
    return _single(tab, ax, "edge_static_zero")


def random_small():
    tab = scenes.random_grammars(1, seed=99)[0]
    ax = G.make_axioms(1)
    ax["shape"] = G.SHAPE_BOX
    ax["seed"] = 0.5
    return _single(tab, ax, "random_grammar")


def cases():
    out = [
        ("menger_d1", scenes.menger(0.5)),
        ("menger_d2", scenes.menger(0.15)),
        ("menger_d3", scenes.menger(0.05)),
        ("menger_d3_dsl", scenes.menger(0.111)),
        ("building_start", scenes.building(mode=G.ANCHOR_TO_START)),
        ("building_end", scenes.building(mode=G.ANCHOR_TO_END)),
        ("building_fill", scenes.building(mode=G.ADJUST_TO_FILL)),
        ("city_16", scenes.city(16)),
        ("facades_2", scenes.facades(2)),
        ("edge_static_zero", edge_static_zero()),
        ("random_grammar", random_small()),
    ]
    for mode in (0, 1, 2):
        for ext in (-0.3, 0.7):
            b = edge_repeat(mode, ext)
            out.append((b["name"], b))
    return out


def canonical(terminals, num_entries=None):
    """Order-free, path-free form: -0 -> +0, entry index folded into the base
    table for per-axiom table copies, sorted by bit pattern."""
    t = terminals.copy()
    t["m"] = t["m"] + np.float32(0)
    t["path"] = 0
    if num_entries is not None:
        e = t["rule"] & 0xFFFFFF
        t["rule"] = (t["rule"] & 0xFF000000) | (e % num_entries)
    return G.sort_terminals(t)


def digest(canon):
    import hashlib

    return hashlib.sha256(np.ascontiguousarray(canon).tobytes()).hexdigest()
