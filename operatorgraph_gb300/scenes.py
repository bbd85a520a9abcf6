"""Synthetic grammar batches (seeded) for the benchmark and parity workloads.

All use the generic procedure list (grammar.DEFAULT_PROCS).  Each function
returns a dict with ``entries`` (ENTRY_DT array), ``axioms`` (AXIOM_DT array),
``blocks`` (float32 array or None) and ``block_stride``.

* menger(threshold): the reference's Menger sponge scene
  (src/test_runner/MengerSponge.cuh:28-45) on one unit box at the origin.
  Threshold 0.05 -> depth 3 (8,000 terminals), 0.005 -> depth 5 (3.2M).
* city(n): Quad footprints on a 64-wide grid (pitch 50 m), widths and depths
  U[10, 40] m, heights LogN(ln 30, 0.5) clamped to [6, 300] m, drawn from
  numpy default_rng(seed) in the order w, d, h.  Extrude to the height
  (custom attribute, PT_SHAPE_ATTR 16), ComponentSplit, facades Repeat along Y
  (3.0 m) and X (2.5 m), IfSizeLess(X, 1.2){Discard | Window}, windows
  Subdivide X {0.2 | -1 | 0.2}.  Walls, windows and roofs are instanced
  terminals.  Footprints lie in the XY plane; buildings rise along +Z.
* facades(n): unit boxes with 16 per-axiom continuous parameters (8 split
  ratios U[0.1, 0.9], 8 extents U[0.5, 2.0], default_rng(seed)) used as
  relative Subdivide factors along Y and X; 8 x 8 cells, each ComponentSplit
  into 4 sides (IfSizeLess guard) and a top halved along X: 384 terminals.
* random_grammars(): 64-rule random grammars (branching U{2..6}, IfSizeLess
  thresholds U[0.01, 0.2], Discard probability 0.15, depth cap 12).
* mixed(n): 40 % Menger (depth 1-3), 40 % city buildings, 20 % random grammars
  (16 generated grammars shared by the random axioms); with blocks=True the
  buildings' and sponges' continuous parameters come from per-axiom blocks.
* collisions(...): a two-phase scene for Collider / IfCollides: in phase 0
  buildings (boxes, tag 1) and billboards (quads, tag 2) store themselves and
  emit terminals; trees (boxes, optionally turned) wait for phase 1, where a
  tree that overlaps a building is discarded, one that overlaps a billboard
  becomes terminal 2 and a free one terminal 3.
* forest(n): n trees on a 64-wide grid (pitch 40 m), boxes 2 x 16 x 2 m
  turned by a per-tree angle about y; a trunk and a crown that forks into
  three branches (Replicate) turned 35 degrees out and 0 / 120 / 240 degrees
  around the stem, each 0.6 of its parent's size, until a branch is shorter
  than 0.5 m (a leaf).  Rotate with arbitrary angles: the general-frame
  kernels.
"""
import math

import numpy as np

from . import grammar as G
from .grammar import DispatchTable, Entry, block, scalar, shape_attr


def _batch(entries, axioms, blocks=None, block_stride=0, name=""):
    return {"entries": entries, "axioms": axioms, "blocks": blocks, "block_stride": block_stride, "name": name}


def menger_table(threshold, blocks=False):
    """The Menger sponge dispatch table (MengerSponge.cuh:35-45) on generic codes.
    blocks=True reads the three relative factors of every split from the
    axiom's parameter block, slots 0..2 (value -1 each gives the sponge)."""
    S3, DIS, IFL, GEN = G.BOX_SUBDIVIDE3, G.BOX_DISCARD, G.BOX_IF_SIZE_LESS, G.BOX_GENERATE
    rel = [block(0), block(1), block(2)] if blocks else [scalar(-1), scalar(-1), scalar(-1)]
    return DispatchTable([
        Entry(IFL, [scalar(0), scalar(threshold)], [(1, 0), (2, 0)]),   # 0 A
        Entry(GEN, [scalar(0)], []),                                     # 1 B (terminal)
        Entry(S3, [scalar(0)] + rel, [(3, 0), (7, 0), (3, 0)]),          # 2 SubX
        Entry(S3, [scalar(1)] + rel, [(4, 0), (5, 0), (4, 0)]),          # 3 SubY
        Entry(S3, [scalar(2)] + rel, [(0, 0), (0, 0), (0, 0)]),          # 4 SubZ
        Entry(S3, [scalar(2)] + rel, [(0, 0), (6, 0), (0, 0)]),          # 5 ZDiscard
        Entry(DIS, [], []),                                              # 6
        Entry(S3, [scalar(1)] + rel, [(5, 0), (8, 0), (5, 0)]),          # 7 YDiscard
        Entry(DIS, [], []),                                              # 8
    ]).to_array()


def menger(threshold=0.05, n=1, seed=0.5):
    ax = G.make_axioms(n)
    ax["seed"] = seed
    ax["custom"] = seed
    ax["shape"] = G.SHAPE_BOX
    ax["entry"] = 0
    if n > 1:
        cols = int(math.ceil(math.sqrt(n)))
        i = np.arange(n)
        ax["position"][:, 0] = 1.5 * (i % cols)
        ax["position"][:, 2] = 1.5 * (i // cols)
    return _batch(menger_table(threshold), ax, name=f"menger(threshold={threshold})")


def building_table(mode=G.ANCHOR_TO_START, meshes=False, blocks=False):
    """One city building: Extrude -> ComponentSplit -> Repeat Y -> Repeat X -> IfSizeLess -> Subdivide.
    meshes=True makes the walls, windows and roofs triangle-mesh terminals
    (meshes 0, 1, 2) instead of instanced ones.  blocks=True reads the floor
    height, the tile width and the window's two wall widths from the axiom's
    parameter block, slots 0..3 (3.0, 2.5, 0.2, 0.2 give the city)."""
    gen = G.QUAD_GENERATE_MESH if meshes else G.QUAD_GENERATE
    floor, tile = (block(0), block(1)) if blocks else (scalar(3.0), scalar(2.5))
    wl, wr = (block(2), block(3)) if blocks else (scalar(0.2), scalar(0.2))
    return DispatchTable([
        Entry(G.QUAD_EXTRUDE, [scalar(1), shape_attr(16)], [(1, 0)]),                      # 0 extrude to height
        Entry(G.BOX_COMPONENT_SPLIT, [], [(9, 0), (7, 0), (2, 0)]),                       # 1 top, bottom, sides
        Entry(G.QUAD_REPEAT, [scalar(1), floor, scalar(mode)], [(3, 0)]),                 # 2 floors
        Entry(G.QUAD_REPEAT, [scalar(0), tile, scalar(mode)], [(4, 0)]),                  # 3 tiles
        Entry(G.QUAD_IF_SIZE_LESS, [scalar(0), scalar(1.2)], [(7, 0), (5, 0)]),           # 4 narrow tile?
        Entry(G.QUAD_SUBDIVIDE, [scalar(0), wl, scalar(-1), wr],
              [(8, 0), (6, 0), (8, 0)]),                                                  # 5 window
        Entry(gen, [scalar(1)], []),                                                      # 6 window terminal
        Entry(G.QUAD_DISCARD, [], []),                                                    # 7
        Entry(gen, [scalar(0)], []),                                                      # 8 wall terminal
        Entry(gen, [scalar(2)], []),                                                      # 9 roof terminal
    ]).to_array()


def building(w=25.0, d=20.0, h=31.0, mode=G.ANCHOR_TO_START):
    ax = G.make_axioms(1)
    ax["size"] = (w, d, 1.0)
    ax["seed"] = 0.5
    ax["custom"] = h
    ax["shape"] = G.SHAPE_QUAD
    return _batch(building_table(mode), ax, name="building")


def city_axioms(n=4096, seed=1234, cols=64, pitch=50.0):
    rng = np.random.default_rng(seed)
    w = rng.uniform(10.0, 40.0, n)
    d = rng.uniform(10.0, 40.0, n)
    h = np.clip(rng.lognormal(math.log(30.0), 0.5, n), 6.0, 300.0)
    ax = G.make_axioms(n)
    i = np.arange(n)
    ax["position"][:, 0] = pitch * (i % cols)
    ax["position"][:, 1] = pitch * (i // cols)
    ax["size"][:, 0] = w
    ax["size"][:, 1] = d
    ax["size"][:, 2] = 1.0
    ax["custom"] = h
    ax["seed"] = 0.5
    ax["shape"] = G.SHAPE_QUAD
    ax["entry"] = 0
    return ax


def city(n=4096, seed=1234, mode=G.ANCHOR_TO_START, meshes=False):
    return _batch(building_table(mode, meshes), city_axioms(n, seed), name=f"city({n})")


FACADE_STRIDE = 16


def facade_table():
    BLK = [block(k) for k in range(16)]
    return DispatchTable([
        Entry(G.BOX_SUBDIVIDE, [scalar(1)] + BLK[0:8], [(1, 0)] * 8),        # 0 eight bands along Y
        Entry(G.BOX_SUBDIVIDE, [scalar(0)] + BLK[8:16], [(2, 0)] * 8),       # 1 eight cells along X
        Entry(G.BOX_COMPONENT_SPLIT, [], [(3, 0), (4, 0), (5, 0)]),          # 2 top, bottom, sides
        Entry(G.QUAD_SUBDIVIDE, [scalar(0), scalar(-1), scalar(-1)], [(6, 0), (6, 0)]),  # 3 top halves
        Entry(G.QUAD_DISCARD, [], []),                                       # 4
        Entry(G.QUAD_IF_SIZE_LESS, [scalar(0), scalar(0.01)], [(4, 0), (6, 0)]),          # 5 side guard
        Entry(G.QUAD_GENERATE, [scalar(0)], []),                             # 6 terminal
    ]).to_array()


def facade_params(n=1024, seed=7):
    rng = np.random.default_rng(seed)
    ratios = rng.uniform(0.1, 0.9, (n, 8))
    extents = rng.uniform(0.5, 2.0, (n, 8))
    # Negative factors are relative shares (Subdivide.cuh:196-205).
    return np.concatenate([-ratios, -extents], axis=1).astype(np.float32)


def facades(n=1024, seed=7):
    ax = G.make_axioms(n)
    cols = int(math.ceil(math.sqrt(n)))
    i = np.arange(n)
    ax["position"][:, 0] = 2.0 * (i % cols)
    ax["position"][:, 2] = 2.0 * (i // cols)
    ax["seed"] = 0.5
    ax["shape"] = G.SHAPE_BOX
    ax["entry"] = 0
    blocks = facade_params(n, seed).reshape(-1)
    return _batch(facade_table(), ax, blocks, FACADE_STRIDE, name=f"facades({n})")


def facade_target_params(params, seed=8, sigma=0.02):
    """Target parameters: each parameter perturbed by N(0, sigma), clamped so the
    relative factors keep their sign (no branch or count can change)."""
    rng = np.random.default_rng(seed)
    p = params.reshape(-1, FACADE_STRIDE).astype(np.float64)
    q = p + rng.normal(0.0, sigma, p.shape)
    q = np.minimum(q, -0.05)
    return q.astype(np.float32).reshape(-1)


def random_grammar_table(rng, num_rules=64, depth_cap=12):
    """A random grammar of `num_rules` rules arranged in `depth_cap` levels.

    Rule r (two entries): IfSizeLess(axis, t ~ U[0.01, 0.2]) { terminal |
    Subdivide<DynParams>(axis', k ~ U{2..6} relative factors) }, each child slot a
    Discard with probability 0.15, else a rule of the next level (a terminal at
    the last level).
    """
    levels = np.sort(rng.integers(0, depth_cap, num_rules))
    levels[0] = 0
    levels = np.sort(levels)
    by_level = [np.nonzero(levels == L)[0] for L in range(depth_cap)]
    GEN, DIS = 2 * num_rules, 2 * num_rules + 1
    entries = [None] * (2 * num_rules + 2)
    for r in range(num_rules):
        L = levels[r]
        axis_t = int(rng.integers(0, 3))
        thr = float(rng.uniform(0.01, 0.2))
        entries[2 * r] = Entry(G.BOX_IF_SIZE_LESS, [scalar(axis_t), scalar(thr)], [(GEN, 0), (2 * r + 1, 0)])
        k = int(rng.integers(2, 7))
        axis_s = int(rng.integers(0, 3))
        factors = [scalar(-float(rng.uniform(0.5, 1.5))) for _ in range(k)]
        succ = []
        nxt = [i for i in range(L + 1, depth_cap) if len(by_level[i])]
        for _ in range(k):
            if rng.random() < 0.15:
                succ.append((DIS, 0))
            elif not nxt:
                succ.append((GEN, 0))
            else:
                cand = by_level[nxt[0]]
                succ.append((2 * int(cand[rng.integers(0, len(cand))]), 0))
        entries[2 * r + 1] = Entry(G.BOX_SUBDIVIDE, [scalar(axis_s)] + factors, succ)
    entries[GEN] = Entry(G.BOX_GENERATE, [scalar(3)], [])
    entries[DIS] = Entry(G.BOX_DISCARD, [], [])
    return DispatchTable(entries).to_array()


def random_grammars(num_grammars=16, seed=99):
    rng = np.random.default_rng(seed)
    tables = [random_grammar_table(rng) for _ in range(num_grammars)]
    return tables


MIXED_STRIDE = 4


def mixed(n=65536, seed=99, menger_depths=(1, 2, 3), num_random_grammars=16, blocks=False):
    """Heterogeneous batch: 40 % Menger, 40 % buildings, 20 % random grammars.

    The random axioms share `num_random_grammars` generated grammars (16 by
    default; one grammar per random axiom would be 13,107 x 130 dispatch-table
    entries).  blocks=True gives every axiom a parameter block of
    MIXED_STRIDE floats: a building reads its floor height, tile width and
    window wall widths from it, a Menger sponge its split factors (the values
    are the scalar grammars' own, so the terminals are the same); random
    grammars read none.  The adjoint then reaches those DynParams."""
    rng = np.random.default_rng(seed)
    thresholds = {1: 0.5, 2: 0.15, 3: 0.05, 4: 0.015, 5: 0.005}
    menger_tables = [menger_table(thresholds[d], blocks=blocks) for d in menger_depths]
    rand_tables = random_grammars(num_random_grammars, seed)
    tables = menger_tables + [building_table(blocks=blocks)] + rand_tables
    entries, offs = G.concat_tables(tables)
    kind = rng.choice(3, size=n, p=[0.4, 0.4, 0.2])
    ax = G.make_axioms(n)
    cols = int(math.ceil(math.sqrt(n)))
    i = np.arange(n)
    ax["position"][:, 0] = 50.0 * (i % cols)
    ax["position"][:, 1] = 50.0 * (i // cols)
    ax["seed"] = 0.5
    city_ax = city_axioms(n, seed + 1, cols=cols)
    depth_pick = rng.integers(0, len(menger_depths), n)
    rand_pick = rng.integers(0, num_random_grammars, n)
    b_off = offs[len(menger_tables)]
    for j in range(n):
        if kind[j] == 0:
            ax[j]["shape"] = G.SHAPE_BOX
            ax[j]["entry"] = offs[depth_pick[j]]
            ax[j]["size"] = (1.0, 1.0, 1.0)
        elif kind[j] == 1:
            ax[j]["shape"] = G.SHAPE_QUAD
            ax[j]["entry"] = b_off
            ax[j]["size"] = city_ax[j]["size"]
            ax[j]["custom"] = city_ax[j]["custom"]
        else:
            ax[j]["shape"] = G.SHAPE_BOX
            ax[j]["entry"] = offs[len(menger_tables) + 1 + rand_pick[j]]
            ax[j]["size"] = (1.0, 1.0, 1.0)
    if not blocks:
        return _batch(entries, ax, name=f"mixed({n})")
    blk = np.zeros((n, MIXED_STRIDE), np.float32)
    blk[kind == 0] = (-1.0, -1.0, -1.0, 0.0)
    blk[kind == 1] = (3.0, 2.5, 0.2, 0.2)
    ax["block"] = np.arange(n)
    return _batch(entries, ax, blk.reshape(-1), MIXED_STRIDE, name=f"mixed({n}, blocks)")


def forest_table(angles=(0.0, 22.5, 45.0, 67.5)):
    """Tree grammar with Rotate / Replicate / Translate / Scale / IfSizeLess;
    entries 0..len(angles)-1 are the roots, one per base angle about y."""
    k = len(angles)
    half = G.exp(("a", 13), ("s", 0.5), ("op", G.OPT_MULTI))  # half the branch length
    # entries after the roots
    TRUNK, CROWN, BRANCH, LEAF, FORK = k, k + 1, k + 2, k + 3, k + 4
    entries = [Entry(G.BOX_ROTATE, [scalar(0), scalar(a), scalar(0)], [(k + 5, 0)]) for a in angles]
    rest = [
        Entry(G.BOX_SCALE, [scalar(-0.5), scalar(-0.5), scalar(-0.5)], [(k + 9, 0)]),        # TRUNK
        Entry(G.BOX_TRANSLATE, [scalar(0), half, scalar(0)], [(BRANCH, 0)]),                  # CROWN
        Entry(G.BOX_IF_SIZE_LESS, [scalar(1), scalar(0.5)], [(LEAF, 0), (FORK, 0)]),         # BRANCH
        Entry(G.BOX_GENERATE, [scalar(1)], []),                                               # LEAF
        Entry(G.BOX_REPLICATE, [], [(k + 6, 0), (k + 7, 0), (k + 8, 0), (TRUNK, 0)]),         # FORK
        Entry(G.BOX_REPLICATE, [], [(TRUNK, 0), (CROWN, 0)]),                                 # k + 5: tree
    ]
    for i, yaw in enumerate((0.0, 120.0, 240.0)):
        # k + 6 + 3 i: turn around the stem, tilt out, shrink, move up by half the new length
        rest.append(Entry(G.BOX_ROTATE, [scalar(0), scalar(yaw), scalar(35)], [(k + 10 + 2 * i, 0)]))
    rest.append(Entry(G.BOX_GENERATE, [scalar(0)], []))                                       # k + 9: trunk piece
    for i in range(3):
        rest.append(Entry(G.BOX_SCALE, [scalar(-0.6), scalar(-0.6), scalar(-0.6)], [(k + 11 + 2 * i, 0)]))
        rest.append(Entry(G.BOX_TRANSLATE, [scalar(0), half, scalar(0)], [(BRANCH, 0)]))
    # fix the three forks' successors (k + 6 .. k + 8 point at k + 10, 12, 14)
    return DispatchTable(entries + rest).to_array()


def forest(n=4096, seed=4321, cols=64, pitch=40.0):
    angles = (0.0, 22.5, 45.0, 67.5)
    rng = np.random.default_rng(seed)
    ax = G.make_axioms(n)
    i = np.arange(n)
    ax["position"][:, 0] = (i % cols) * pitch
    ax["position"][:, 2] = (i // cols) * pitch
    ax["size"] = (2.0, 16.0, 2.0)
    ax["entry"] = rng.integers(0, len(angles), n)
    ax["seed"] = rng.uniform(0.0, 1.0, n).astype(np.float32)
    return _batch(forest_table(angles), ax, name=f"forest({n})")


TREE_TURNS = ((0.0, 30.0, 0.0), (10.0, -47.5, 12.25), (0.0, 45.0, 90.0), (-20.0, 0.0, 33.0))


def collision_table(rotate=True):
    """The two-phase grammar of collisions(); successors (entry, phase).
    Trees enter at entry 6 (rotate=False: a size swap instead of a turn) or,
    with rotate=True, at 12..15, turned by TREE_TURNS."""
    tree_yaw = 30.0 if rotate else 90.0
    turns = [Entry(G.BOX_ROTATE, [scalar(x), scalar(y), scalar(z)], [(7, 1)]) for x, y, z in TREE_TURNS]
    return DispatchTable([
        Entry(G.BOX_COLLIDER, [scalar(1)], [(1, 0)]),                                    # 0 building
        Entry(G.BOX_COMPONENT_SPLIT, [], [(2, 0), (3, 0), (2, 0)]),                      # 1
        Entry(G.QUAD_GENERATE, [scalar(0)], []),                                         # 2 roof / wall
        Entry(G.QUAD_DISCARD, [], []),                                                   # 3
        Entry(G.QUAD_COLLIDER, [scalar(2)], [(5, 0)]),                                   # 4 billboard
        Entry(G.QUAD_GENERATE, [scalar(1)], []),                                         # 5
        Entry(G.BOX_ROTATE if rotate else G.BOX_SWAP_SIZE,
              [scalar(0), scalar(tree_yaw), scalar(0)] if rotate else [scalar(0), scalar(1), scalar(2)],
              [(7, 1)]),                                                                 # 6 tree: waits for phase 1
        Entry(G.BOX_IF_COLLIDES, [scalar(1)], [(8, 1), (9, 1)]),                         # 7 building?
        Entry(G.BOX_DISCARD, [], []),                                                    # 8
        Entry(G.BOX_IF_COLLIDES, [scalar(2)], [(10, 1), (11, 1)]),                       # 9 billboard?
        Entry(G.BOX_GENERATE, [scalar(2)], []),                                          # 10
        Entry(G.BOX_GENERATE, [scalar(3)], []),                                          # 11
    ] + (turns if rotate else [])).to_array()


def collisions(n_buildings=64, n_trees=512, n_boards=96, seed=77, rotate=True):
    rng = np.random.default_rng(seed)
    n = n_buildings + n_boards + n_trees
    ax = G.make_axioms(n)
    area = 40.0 * math.sqrt(n_buildings)
    b = slice(0, n_buildings)
    ax["entry"][b] = 0
    ax["shape"][b] = G.SHAPE_BOX
    ax["size"][b] = np.stack([rng.uniform(5, 15, n_buildings), rng.uniform(8, 40, n_buildings),
                              rng.uniform(5, 15, n_buildings)], 1)
    ax["position"][b] = np.stack([rng.uniform(0, area, n_buildings), ax["size"][b][:, 1] * 0.5,
                                  rng.uniform(0, area, n_buildings)], 1)
    q = slice(n_buildings, n_buildings + n_boards)
    ax["entry"][q] = 4
    ax["shape"][q] = G.SHAPE_QUAD
    ax["size"][q] = np.stack([rng.uniform(4, 12, n_boards), rng.uniform(2, 6, n_boards), np.ones(n_boards)], 1)
    ax["position"][q] = np.stack([rng.uniform(0, area, n_boards), rng.uniform(1, 4, n_boards),
                                  rng.uniform(0, area, n_boards)], 1)
    t = slice(n_buildings + n_boards, n)
    ax["entry"][t] = rng.integers(12, 16, n_trees) if rotate else 6
    ax["shape"][t] = G.SHAPE_BOX
    ax["size"][t] = np.stack([rng.uniform(1, 4, n_trees), rng.uniform(3, 9, n_trees), rng.uniform(1, 4, n_trees)], 1)
    ax["position"][t] = np.stack([rng.uniform(0, area, n_trees), ax["size"][t][:, 1] * 0.5,
                                  rng.uniform(0, area, n_trees)], 1)
    ax["seed"] = rng.uniform(0, 1, n).astype(np.float32)
    return _batch(collision_table(rotate), ax, name=f"collisions({n_buildings}, {n_trees}, {n_boards})")
