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


def affine_mix():
    """Translate, Scale and RandomRule<DynParams> (Translate.cuh, Scale.cuh,
    RandomRule.cuh:121-150) on both shapes: a seed-driven choice between a
    translated, absolutely / relatively scaled box split into faces and a
    scaled subdivision; a custom-attribute choice among three weights that do
    not sum to one; a zero first weight (picked when the chance is exactly 0,
    since the accumulated probability is then 0 <= 0); a chance from a random
    range; seeds with fractional part 0 and near 1."""
    tab = DispatchTable([
        Entry(G.BOX_RANDOM_RULE, [shape_attr(15), scalar(0.5), scalar(0.5)], [(1, 0), (4, 0)]),       # 0
        Entry(G.BOX_TRANSLATE, [scalar(1.0), scalar(-2.0), scalar(0.5)], [(2, 0)]),                    # 1
        Entry(G.BOX_SCALE, [scalar(-0.8), scalar(-1), scalar(2.0)], [(3, 0)]),                         # 2
        Entry(G.BOX_COMPONENT_SPLIT, [], [(6, 0), (11, 0), (7, 0)]),                                   # 3
        Entry(G.BOX_SCALE, [scalar(-1.0666), scalar(-1), scalar(-1.1333)], [(5, 0)]),                  # 4
        Entry(G.BOX_SUBDIVIDE, [scalar(1), scalar(-1), scalar(-3)], [(9, 0), (10, 0)]),                # 5
        Entry(G.QUAD_RANDOM_RULE, [shape_attr(16), scalar(0.333), scalar(0.333), scalar(0.334)],
              [(8, 0), (12, 0), (13, 0)]),                                                              # 6
        Entry(G.QUAD_RANDOM_RULE, [rand(0.0, 1.0), scalar(0.0), scalar(1.0)], [(12, 0), (13, 0)]),     # 7
        Entry(G.QUAD_TRANSLATE, [scalar(0), scalar(0.1666), scalar(-0.25)], [(14, 0)]),                # 8
        Entry(G.BOX_GENERATE, [scalar(0)], []),                                                        # 9
        Entry(G.BOX_RANDOM_RULE, [shape_attr(15), scalar(0.0), scalar(2.0), scalar(1.0)],
              [(9, 0), (15, 0), (16, 0)]),                                                              # 10
        Entry(G.QUAD_DISCARD, [], []),                                                                 # 11
        Entry(G.QUAD_GENERATE, [scalar(1)], []),                                                       # 12
        Entry(G.QUAD_SCALE, [scalar(0.5), scalar(-0.5), scalar(1)], [(12, 0)]),                        # 13
        Entry(G.QUAD_GENERATE, [scalar(2)], []),                                                       # 14
        Entry(G.BOX_TRANSLATE, [G.exp(("a", 12), ("s", 0.5), ("op", G.OPT_MULTI)), scalar(0), scalar(0)],
              [(17, 0)]),                                                                               # 15
        Entry(G.BOX_SCALE, [scalar(3), scalar(-2), scalar(-0.5)], [(9, 0)]),                           # 16
        Entry(G.BOX_GENERATE, [scalar(3)], []),                                                        # 17
    ]).to_array()
    ax = G.make_axioms(10)
    ax["size"] = [(2.0, 3.0, 1.5), (1.0, 1.0, 1.0), (4.0, 2.0, 0.5), (0.7, 5.0, 2.2), (3.0, 3.0, 3.0),
                  (1.5, 0.5, 2.5), (2.5, 4.5, 1.0), (0.9, 1.1, 1.3), (1.2, 0.8, 2.0), (2.0, 1.0, 1.0)]
    ax["position"] = [(0, 0, 0), (5, 0, 0), (0, 5, 0), (-3, 2, 1), (1, -4, 7), (2, 2, -2), (-6, -1, 3), (4, 4, 4),
                      (-2, 6, 0), (3, -3, 3)]
    ax["seed"] = [0.25, 0.75, 2.0, 0.999, 1.5, 3.0, 0.5, 1.6, 0.6, 0.0]
    ax["custom"] = [0.1, 0.5, 0.9, 0.333, 0.666, 1.0, 0.0, 2.7, 0.4, 0.2]
    # the last two axioms start inside the grammar: a box at the three-way
    # choice and a quad at the choice whose first weight is zero
    ax["entry"][8] = 10
    ax["entry"][9] = 7
    ax["shape"][9] = G.SHAPE_QUAD
    return _single(tab, ax, "affine_mix")


def rotate_mix():
    """Rotate (Rotate.cuh:24-41, rotateXYZ in matrix.h:876-888) and
    Replicate<DynParams> (Replicate.cuh:95-110): a box replicated into an
    unrotated copy, a copy turned 90 degrees about y then split, and a copy
    turned by arbitrary angles about all three axes then split into faces; a
    face rotated again, translated along its rotated axes, scaled and
    extruded; a quad replicated into three turned copies; chained rotations
    whose matrices are general (not signed permutations)."""
    tab = DispatchTable([
        Entry(G.BOX_REPLICATE, [], [(1, 0), (2, 0), (4, 0)]),                                        # 0
        Entry(G.BOX_GENERATE, [scalar(0)], []),                                                      # 1
        Entry(G.BOX_ROTATE, [scalar(0), scalar(90), scalar(0)], [(3, 0)]),                           # 2
        Entry(G.BOX_SUBDIVIDE, [scalar(0), scalar(-1), scalar(-2)], [(1, 0), (5, 0)]),               # 3
        Entry(G.BOX_ROTATE, [scalar(30), scalar(-47.5), scalar(12.25)], [(6, 0)]),                   # 4
        Entry(G.BOX_ROTATE, [scalar(0), scalar(0), scalar(-37)], [(1, 0)]),                          # 5
        Entry(G.BOX_COMPONENT_SPLIT, [], [(7, 0), (11, 0), (12, 0)]),                                # 6
        Entry(G.QUAD_ROTATE, [scalar(0), scalar(0), scalar(45)], [(8, 0)]),                          # 7
        Entry(G.QUAD_TRANSLATE, [scalar(0.5), G.exp(("a", 13), ("s", 0.5), ("op", G.OPT_MULTI)), scalar(-0.25)],
              [(9, 0)]),                                                                              # 8
        Entry(G.QUAD_SCALE, [scalar(-0.5), scalar(2), scalar(1)], [(10, 0)]),                        # 9
        Entry(G.QUAD_EXTRUDE, [scalar(0), scalar(0.75)], [(13, 0)]),                                 # 10
        Entry(G.QUAD_DISCARD, [], []),                                                               # 11
        Entry(G.QUAD_REPLICATE, [], [(14, 0), (15, 0), (16, 0)]),                                    # 12
        Entry(G.BOX_REPEAT, [scalar(1), scalar(-0.3), scalar(2)], [(5, 0)]),                         # 13
        Entry(G.QUAD_GENERATE, [scalar(1)], []),                                                     # 14
        Entry(G.QUAD_ROTATE, [scalar(90), scalar(90), scalar(0)], [(14, 0)]),                        # 15
        Entry(G.QUAD_ROTATE, [scalar(-132.63), scalar(18.95), scalar(180)], [(17, 0)]),              # 16
        Entry(G.QUAD_IF_SIZE_LESS, [scalar(0), scalar(1.5)], [(14, 0), (18, 0)]),                    # 17
        Entry(G.QUAD_SUBDIVIDE, [scalar(0), scalar(-1), scalar(-1)], [(19, 0), (19, 0)]),            # 18
        Entry(G.QUAD_ROTATE, [scalar(0), scalar(-94.74), scalar(0)], [(20, 0)]),                     # 19
        Entry(G.QUAD_GENERATE, [scalar(2)], []),                                                     # 20
    ]).to_array()
    ax = G.make_axioms(5)
    ax["size"] = [(2.0, 3.0, 1.5), (1.0, 1.0, 1.0), (4.0, 2.0, 0.5), (0.7, 5.0, 2.2), (3.3, 1.9, 2.8)]
    ax["position"] = [(0, 0, 0), (5, -1, 2), (-7.25, 5, 0.5), (-3, 2, 1), (100, -40, 7)]
    ax["seed"] = [0.25, 0.75, 1.5, 0.999, 2.5]
    ax["custom"] = [0.1, 0.5, 0.9, 0.333, 0.666]
    return _single(tab, ax, "rotate_mix")


def random_static_mix():
    """The static RandomRule<Chance, Pair<weight, next>...> (RandomRule.cuh:33-99):
    two, three and four pairs on both shapes; weights summed right to left;
    shares that do not reach one (the last pair is then taken anyway); a zero
    first weight (never taken, unlike the DynParams form, which takes it at
    chance 0); chances from the seed, the custom attribute and a random range;
    64 axioms whose seeds include 0, values just below 1 and values >= 1."""
    tab = DispatchTable([
        Entry(G.BOX_RANDOM_RULE3, [shape_attr(15), scalar(0.333), scalar(0.333), scalar(0.333)],
              [(1, 0), (2, 0), (3, 0)]),                                                                   # 0
        Entry(G.BOX_GENERATE, [scalar(0)], []),                                                           # 1
        Entry(G.BOX_COMPONENT_SPLIT, [], [(4, 0), (5, 0), (6, 0)]),                                       # 2
        Entry(G.BOX_RANDOM_RULE4, [shape_attr(16), scalar(0.1), scalar(0.2), scalar(0.3), scalar(0.15)],
              [(1, 0), (7, 0), (8, 0), (9, 0)]),                                                          # 3
        Entry(G.QUAD_RANDOM_RULE2, [shape_attr(15), scalar(0.0), scalar(1.0)], [(10, 0), (11, 0)]),      # 4
        Entry(G.QUAD_DISCARD, [], []),                                                                    # 5
        Entry(G.QUAD_RANDOM_RULE3, [rand(0.0, 1.0), scalar(2.0), scalar(0.0), scalar(1.0)],
              [(10, 0), (11, 0), (12, 0)]),                                                               # 6
        Entry(G.BOX_GENERATE, [scalar(1)], []),                                                           # 7
        Entry(G.BOX_GENERATE, [scalar(2)], []),                                                           # 8
        Entry(G.BOX_GENERATE, [scalar(3)], []),                                                           # 9
        Entry(G.QUAD_GENERATE, [scalar(4)], []),                                                          # 10
        Entry(G.QUAD_GENERATE, [scalar(5)], []),                                                          # 11
        Entry(G.QUAD_RANDOM_RULE4, [shape_attr(16), scalar(0.25), scalar(0.25), scalar(0.25), scalar(0.25)],
              [(10, 0), (11, 0), (13, 0), (11, 0)]),                                                      # 12
        Entry(G.QUAD_GENERATE, [scalar(6)], []),                                                          # 13
    ]).to_array()
    rng = np.random.default_rng(17)
    n = 64
    ax = G.make_axioms(n)
    ax["size"] = rng.uniform(0.5, 3.0, (n, 3)).astype(np.float32)
    ax["position"] = rng.uniform(-20, 20, (n, 3)).astype(np.float32)
    seeds = rng.uniform(0.0, 3.0, n).astype(np.float32)
    seeds[:8] = [0.0, 1.0, 0.333, 0.666, 0.999, np.nextafter(np.float32(1), np.float32(0)), 2.0, 0.3329999]
    ax["seed"] = seeds
    custom = rng.uniform(0.0, 1.0, n).astype(np.float32)
    custom[:6] = [0.0, 0.1, 0.3, 0.6, 0.75, np.nextafter(np.float32(1), np.float32(0))]
    ax["custom"] = custom
    return _single(tab, ax, "random_static_mix")


def if_swap_mix():
    """If<Expression, True, False> (If.cuh:22-49) and SwapSize (SwapSize.cuh:20-38):
    conditions from comparisons of the size and the seed, a logical and, a
    plain shape attribute (nonzero is true) and scalars; SwapSize as a cyclic
    permutation, a swap, and with a repeated axis, on both shapes."""
    gt = G.OPT_GT
    tab = DispatchTable([
        Entry(G.BOX_IF, [G.exp(("a", 12), ("s", 1.5), ("op", gt))], [(1, 0), (4, 0)]),                 # 0
        Entry(G.BOX_SWAP_SIZE, [scalar(1), scalar(2), scalar(0)], [(2, 0)]),                            # 1
        Entry(G.BOX_SUBDIVIDE, [scalar(0), scalar(-1), scalar(-1)], [(3, 0), (5, 0)]),                  # 2
        Entry(G.BOX_GENERATE, [scalar(0)], []),                                                         # 3
        Entry(G.BOX_COMPONENT_SPLIT, [], [(6, 0), (7, 0), (8, 0)]),                                     # 4
        Entry(G.BOX_IF, [shape_attr(15)], [(9, 0), (3, 0)]),                                            # 5
        Entry(G.QUAD_SWAP_SIZE, [scalar(1), scalar(0), scalar(2)], [(10, 0)]),                          # 6
        Entry(G.QUAD_DISCARD, [], []),                                                                  # 7
        Entry(G.QUAD_IF, [G.exp(("a", 13), ("s", 1.0), ("op", gt), ("a", 15), ("s", 0.5), ("op", gt),
                                ("op", G.OPT_AND))], [(11, 0), (12, 0)]),                               # 8
        Entry(G.BOX_SWAP_SIZE, [scalar(2), scalar(2), scalar(1)], [(3, 0)]),                            # 9
        Entry(G.QUAD_GENERATE, [scalar(1)], []),                                                        # 10
        Entry(G.QUAD_IF, [scalar(0)], [(7, 0), (13, 0)]),                                               # 11
        Entry(G.QUAD_EXTRUDE, [scalar(0), scalar(0.5)], [(14, 0)]),                                     # 12
        Entry(G.QUAD_GENERATE, [scalar(2)], []),                                                        # 13
        Entry(G.BOX_IF, [scalar(1)], [(9, 0), (3, 0)]),                                                 # 14
    ]).to_array()
    rng = np.random.default_rng(23)
    n = 12
    ax = G.make_axioms(n)
    ax["size"] = rng.uniform(0.5, 3.0, (n, 3)).astype(np.float32)
    ax["position"] = rng.uniform(-20, 20, (n, 3)).astype(np.float32)
    ax["seed"] = rng.uniform(0.0, 1.0, n).astype(np.float32)
    ax["seed"][:2] = 0.0
    return _single(tab, ax, "if_swap_mix")


def mesh_mix():
    """Triangle-mesh terminals (Generate<false, 0, mesh>, GenerationFunctions.cuh:41-153,
    ShapeGenerator.cuh:377-512, 671-708): boxes and quads into three meshes,
    beside instanced terminals; unrotated, right-angle and arbitrary rotations
    (the general-frame kernels); a face extruded to a box; a degenerate quad of
    zero width (its normal is NaN in the reference too)."""
    tab = DispatchTable([
        Entry(G.BOX_REPLICATE, [], [(1, 0), (2, 0), (4, 0), (9, 0)]),                                 # 0
        Entry(G.BOX_GENERATE_MESH, [scalar(0)], []),                                                  # 1
        Entry(G.BOX_ROTATE, [scalar(0), scalar(90), scalar(0)], [(3, 0)]),                            # 2
        Entry(G.BOX_COMPONENT_SPLIT, [], [(5, 0), (6, 0), (7, 0)]),                                   # 3
        Entry(G.BOX_ROTATE, [scalar(17.5), scalar(-33), scalar(61.25)], [(8, 0)]),                    # 4
        Entry(G.QUAD_GENERATE_MESH, [scalar(1)], []),                                                 # 5
        Entry(G.QUAD_GENERATE, [scalar(2)], []),                                                      # 6
        Entry(G.QUAD_EXTRUDE, [scalar(0), scalar(0.4)], [(1, 0)]),                                    # 7
        Entry(G.BOX_SUBDIVIDE, [scalar(1), scalar(-1), scalar(-2)], [(1, 0), (3, 0)]),                # 8
        Entry(G.BOX_SCALE, [scalar(0), scalar(-1), scalar(-1)], [(10, 0)]),                           # 9
        Entry(G.BOX_COMPONENT_SPLIT, [], [(11, 0), (11, 0), (11, 0)]),                                # 10
        Entry(G.QUAD_GENERATE_MESH, [scalar(2)], []),                                                 # 11
    ]).to_array()
    ax = G.make_axioms(3)
    ax["size"] = [(1.0, 2.0, 3.0), (0.5, 0.25, 4.0), (3.3, 1.7, 2.9)]
    ax["position"] = [(0, 0, 0), (10, 5, -3), (-7.5, 2.25, 100)]
    ax["seed"] = [0.1, 0.5, 0.9]
    return _single(tab, ax, "mesh_mix")


def rich_random(seed, depth=5, n_axioms=4, affine=False, rotate=False, more=False, meshes=False):
    """A random grammar over all eight operators and both shapes: a DAG of
    rules `depth` levels deep (rules of a level reused with some probability),
    with scalar, random-range, shape-attribute and expression parameters,
    relative / absolute / zero Subdivide factors, the three Repeat modes with
    relative and absolute extents, ComponentSplit, Extrude from the custom
    attribute, IfSizeLess on scalars and expressions, constant and random
    terminal indices.  Seeds >= 1 and custom attributes vary per axiom.
    With affine=True the grammar also draws Translate, Scale and RandomRule
    rules, with rotate=True also Rotate and Replicate rules, with more=True also
    If and SwapSize rules, with meshes=True half of the terminal rules are
    triangle-mesh Generates (the defaults draw exactly the grammars they always
    drew)."""
    rng = np.random.default_rng(seed)
    BOX, QUAD = G.SHAPE_BOX, G.SHAPE_QUAD
    GEN = {BOX: G.BOX_GENERATE, QUAD: G.QUAD_GENERATE}
    GEN_MESH = {BOX: G.BOX_GENERATE_MESH, QUAD: G.QUAD_GENERATE_MESH}
    DIS = {BOX: G.BOX_DISCARD, QUAD: G.QUAD_DISCARD}
    SUB = {BOX: G.BOX_SUBDIVIDE, QUAD: G.QUAD_SUBDIVIDE}
    SUB3 = {BOX: G.BOX_SUBDIVIDE3, QUAD: G.QUAD_SUBDIVIDE3}
    REP = {BOX: G.BOX_REPEAT, QUAD: G.QUAD_REPEAT}
    IFL = {BOX: G.BOX_IF_SIZE_LESS, QUAD: G.QUAD_IF_SIZE_LESS}
    TRA = {BOX: G.BOX_TRANSLATE, QUAD: G.QUAD_TRANSLATE}
    SCA = {BOX: G.BOX_SCALE, QUAD: G.QUAD_SCALE}
    RRU = {BOX: G.BOX_RANDOM_RULE, QUAD: G.QUAD_RANDOM_RULE}
    ROT = {BOX: G.BOX_ROTATE, QUAD: G.QUAD_ROTATE}
    REPL = {BOX: G.BOX_REPLICATE, QUAD: G.QUAD_REPLICATE}
    IFX = {BOX: G.BOX_IF, QUAD: G.QUAD_IF}
    SWP = {BOX: G.BOX_SWAP_SIZE, QUAD: G.QUAD_SWAP_SIZE}
    entries = []
    made = {}

    def add(e):
        entries.append(e)
        return len(entries) - 1

    def axis(kind):
        return scalar(int(rng.integers(0, 3 if kind == BOX else 2)))

    def rel_factor():
        u = rng.random()
        if u < 0.6:
            return scalar(-float(rng.uniform(0.5, 2.0)))
        if u < 0.8:
            return rand(-2.0, -0.5)
        return G.exp(("a", 12 + int(rng.integers(0, 2))), ("s", -float(rng.uniform(0.2, 1.0))), ("op", G.OPT_MULTI))

    def make(kind, level):
        key = (kind, level)
        if made.get(key) and rng.random() < 0.3:
            return made[key][int(rng.integers(0, len(made[key])))]
        if level >= depth or rng.random() < 0.1:
            if rng.random() < 0.15:
                e = add(Entry(DIS[kind], [], []))
            else:
                tidx = scalar(int(rng.integers(0, 4))) if rng.random() < 0.8 else rand(0.0, 3.9)
                gen = GEN_MESH[kind] if meshes and rng.random() < 0.5 else GEN[kind]
                e = add(Entry(gen, [tidx], []))
            made.setdefault(key, []).append(e)
            return e
        ops = ["sub", "sub3", "rep", "ifl"] + (["cs"] if kind == BOX else ["ext"])
        if affine:
            ops += ["tr", "sc", "rr"]
        if rotate:
            ops += ["rot", "repl"]
        if more:
            ops += ["if", "swap"]
        op = ops[int(rng.integers(0, len(ops)))]
        if op == "sub":
            k = int(rng.integers(2, 5))
            factors = [rel_factor() for _ in range(k)]
            if rng.random() < 0.3:
                factors[int(rng.integers(0, k))] = scalar(0.02)
            succ = [(make(kind, level + 1), 0) for _ in range(k)]
            e = add(Entry(SUB[kind], [axis(kind)] + factors, succ))
        elif op == "sub3":
            factors = [rel_factor() for _ in range(3)]
            if rng.random() < 0.4:
                factors[int(rng.integers(0, 3))] = scalar(0.0)
            succ = [(make(kind, level + 1), 0) for _ in range(3)]
            e = add(Entry(SUB3[kind], [axis(kind)] + factors, succ))
        elif op == "rep":
            ext = scalar(-float(rng.uniform(0.2, 0.5))) if rng.random() < 0.7 else scalar(float(rng.uniform(0.3, 0.8)))
            e = add(Entry(REP[kind], [axis(kind), ext, scalar(int(rng.integers(0, 3)))], [(make(kind, level + 1), 0)]))
        elif op == "ifl":
            size = scalar(float(rng.uniform(0.1, 1.0))) if rng.random() < 0.7 else G.exp(
                ("a", 12 + int(rng.integers(0, 2))), ("s", 0.5), ("op", G.OPT_MULTI))
            e = add(Entry(IFL[kind], [axis(kind), size], [(make(kind, level + 1), 0), (make(kind, level + 1), 0)]))
        elif op == "cs":
            e = add(Entry(G.BOX_COMPONENT_SPLIT, [],
                          [(make(QUAD, level + 1), 0), (make(QUAD, level + 1), 0), (make(QUAD, level + 1), 0)]))
        elif op == "tr":
            v = [scalar(float(rng.uniform(-2.0, 2.0))) if rng.random() < 0.7 else rand(-1.0, 1.0) for _ in range(3)]
            if rng.random() < 0.3:
                v[int(rng.integers(0, 3))] = G.exp(("a", 12), ("s", 0.5), ("op", G.OPT_MULTI))
            e = add(Entry(TRA[kind], v, [(make(kind, level + 1), 0)]))
        elif op == "sc":
            v = []
            for _ in range(3):
                u = rng.random()
                v.append(scalar(-float(rng.uniform(0.5, 1.5))) if u < 0.6 else
                         (scalar(float(rng.uniform(0.2, 3.0))) if u < 0.8 else scalar(-1)))
            e = add(Entry(SCA[kind], v, [(make(kind, level + 1), 0)]))
        elif op == "rr":
            u = rng.random()
            chance = shape_attr(15) if u < 0.4 else (shape_attr(16) if u < 0.7 else rand(0.0, 1.0))
            k = int(rng.integers(2, 5))
            weights = [scalar(float(rng.uniform(0.1, 1.0))) for _ in range(k)]
            if rng.random() < 0.2:
                weights[int(rng.integers(0, k))] = scalar(0.0)
            e = add(Entry(RRU[kind], [chance] + weights, [(make(kind, level + 1), 0) for _ in range(k)]))
        elif op == "rot":
            ang = [scalar(float(rng.choice([0.0, 90.0, -90.0, 180.0]))) if rng.random() < 0.4 else
                   scalar(round(float(rng.uniform(-180.0, 180.0)), 2)) for _ in range(3)]
            e = add(Entry(ROT[kind], ang, [(make(kind, level + 1), 0)]))
        elif op == "if":
            u = rng.random()
            if u < 0.5:
                cond = G.exp(("a", 12 + int(rng.integers(0, 2))), ("s", float(rng.uniform(0.3, 1.5))),
                             ("op", G.OPT_GT if rng.random() < 0.5 else G.OPT_LT))
            elif u < 0.8:
                cond = G.exp(("a", 15), ("s", 0.5), ("op", G.OPT_GEQ))
            else:
                cond = scalar(float(rng.integers(0, 2)))
            e = add(Entry(IFX[kind], [cond], [(make(kind, level + 1), 0), (make(kind, level + 1), 0)]))
        elif op == "swap":
            axes = [scalar(int(rng.integers(0, 3))) for _ in range(3)]
            e = add(Entry(SWP[kind], axes, [(make(kind, level + 1), 0)]))
        elif op == "repl":
            k = int(rng.integers(2, 4))
            e = add(Entry(REPL[kind], [], [(make(kind, level + 1), 0) for _ in range(k)]))
        else:  # ext
            u = rng.random()
            extent = scalar(float(rng.uniform(0.2, 2.0))) if u < 0.5 else (shape_attr(16) if u < 0.8 else rand(0.3, 1.5))
            e = add(Entry(G.QUAD_EXTRUDE, [scalar(1), extent], [(make(BOX, level + 1), 0)]))
        made.setdefault(key, []).append(e)
        return e

    root_kind = BOX if rng.random() < 0.6 else QUAD
    root = make(root_kind, 0)
    tab = DispatchTable(entries).to_array()
    ax = G.make_axioms(n_axioms)
    ax["shape"] = root_kind
    ax["entry"] = root
    ax["size"] = rng.uniform(0.5, 4.0, (n_axioms, 3)).astype(np.float32)
    if root_kind == QUAD:
        ax["size"][:, 2] = 1.0
    ax["position"] = rng.uniform(-10.0, 10.0, (n_axioms, 3)).astype(np.float32)
    ax["seed"] = rng.uniform(0.0, 3.0, n_axioms).astype(np.float32)
    ax["custom"] = rng.uniform(0.5, 3.0, n_axioms).astype(np.float32)
    name = "rich_mesh" if meshes else (
        "rich_more" if more else ("rich_rotate" if rotate else ("rich_affine" if affine else "rich_random")))
    return _single(tab, ax, f"{name}_{seed}")


# Seeds of rich_random() with golden fixtures: seeds among the first sixty
# whose grammar derives without error (the reference throws on, e.g., a
# Subdivide whose absolute factors exceed the size) and that together use
# every operator, both shapes and every parameter kind.
RICH_SEEDS = (3, 5, 6, 8, 20, 26, 29, 32, 36, 38, 53, 58)

# Seeds of rich_random(affine=True) with golden fixtures: together they use
# Translate, Scale and RandomRule on both shapes, with every chance kind.
AFFINE_SEEDS = (2, 3, 5, 12, 13, 19, 27, 29, 49, 58)

# Seeds of rich_random(affine=True, rotate=True) with golden fixtures: together
# they use Rotate (right angles and arbitrary ones) and Replicate on both
# shapes, mixed with every other operator.
ROTATE_SEEDS = (3, 6, 8, 13, 24, 47, 58, 71, 73, 75)

# Seeds of rich_random(affine=True, more=True) with golden fixtures: together
# they use If (expression, attribute and scalar conditions) and SwapSize on
# both shapes.
MORE_SEEDS = (0, 3, 4, 18, 19, 20, 34, 47, 49, 50)

# Seeds of rich_random(affine=True, rotate=True, more=True, meshes=True) with
# golden fixtures, meshes included: boxes and quads into up to four meshes,
# rotated and not.
MESH_SEEDS = (3, 8, 13, 15, 24, 26, 29, 34, 36, 39)


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
    for seed in RICH_SEEDS:
        b = rich_random(seed)
        out.append((b["name"], b))
    out.append(("affine_mix", affine_mix()))
    for seed in AFFINE_SEEDS:
        b = rich_random(seed, affine=True)
        out.append((b["name"], b))
    out.append(("rotate_mix", rotate_mix()))
    out.append(("random_static_mix", random_static_mix()))
    out.append(("forest_4", scenes.forest(4)))
    out.append(("if_swap_mix", if_swap_mix()))
    for seed in MORE_SEEDS:
        b = rich_random(seed, affine=True, more=True)
        out.append((b["name"], b))
    out.append(("mesh_mix", mesh_mix()))
    for seed in MESH_SEEDS:
        b = rich_random(seed, affine=True, rotate=True, more=True, meshes=True)
        out.append((b["name"], b))
    for seed in ROTATE_SEEDS:
        b = rich_random(seed, affine=True, rotate=True)
        out.append((b["name"], b))
    return out


def mesh_digest(vertices, indices):
    """Digest of a generated mesh's faces, order-free (grammar.mesh_faces)."""
    import hashlib

    return hashlib.sha256(np.ascontiguousarray(G.mesh_faces(vertices, indices)).tobytes()).hexdigest()


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


def canonical_paths(terminals, num_entries=None):
    """Order-free form WITH derivation-path hashes: -0 -> +0, entry index
    folded into the base table, sorted by path hash (the paths of one batch
    are distinct, so the order is total)."""
    t = terminals.copy()
    t["m"] = t["m"] + np.float32(0)
    if num_entries is not None:
        e = t["rule"] & 0xFFFFFF
        t["rule"] = (t["rule"] & 0xFF000000) | (e % num_entries)
    return G.sort_terminals(t, by_path=True)


def digest(canon):
    import hashlib

    return hashlib.sha256(np.ascontiguousarray(canon).tobytes()).hexdigest()
