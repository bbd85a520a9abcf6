"""The .pga front end (operatorgraph_gb300/dsl.py).

Grammars written in the reference's language are parsed and lowered to
dispatch tables; the oracle derives them and the results are compared with the
same grammars built as data (scenes.py).  Rule order and names differ, so
entry indices and path hashes differ: transforms, terminal indices and custom
attributes are compared as multisets.
"""
import os

import numpy as np
import pytest

import oracle
from operatorgraph_gb300 import dsl
from operatorgraph_gb300 import grammar as G
from operatorgraph_gb300 import scenes

MENGER = """
axiom Box Cube;
terminal Piece (1, 0);

// a cube larger than the threshold is split into 3 x 3 x 3 and loses its centre cross
Cube = IfSizeLess(X, 0.111) { Piece | SplitX };
SplitX = SubDiv(X) { -1: SplitY | -1: HoleY | -1: SplitY };
SplitY = SubDiv(Y) { -1: SplitZ | -1: HoleZ | -1: SplitZ };
SplitZ = SubDiv(Z) { -1: Cube | -1: Cube | -1: Cube };
HoleY = SubDiv(Y) { -1: HoleZ | -1: Discard() | -1: HoleZ };
HoleZ = SubDiv(Z) { -1: Cube | -1: Discard() | -1: Cube };
"""

BUILDING = """
axiom Quad Lot;
terminal Wall (1, 0);
terminal Window (1, 1);
terminal Roof (1, 2);

Lot = Extrude(Y, ShapeCustomAttribute()) CompSplit() { Roof | Discard() | Repeat(Y, 3, %(mode)s) Floor };
Floor = Repeat(X, 2.5, %(mode)s) Tile;
Tile = IfSizeLess(X, 1.2) { Discard() | SubDiv(X) { 0.2: Wall | -1: Window | 0.2: Wall } };
"""


def _multiset(t):
    key = np.concatenate([(t["m"] + np.float32(0)).view(np.uint32), (t["rule"] >> 24)[:, None],
                          t["custom"].view(np.uint32)[:, None]], axis=1)
    return key[np.lexsort(key.T[::-1])]


def test_menger_from_pga_matches_the_data_table():
    b = dsl.load(MENGER)
    ref = scenes.menger(0.111)
    b["axioms"]["seed"] = ref["axioms"]["seed"]
    b["axioms"]["custom"] = ref["axioms"]["custom"]
    got = oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"])
    want = oracle.derive(G.DEFAULT_PROCS, ref["entries"], ref["axioms"])
    assert len(got) == len(want) == 8000
    assert (_multiset(got) == _multiset(want)).all()
    assert len(np.unique(got["path"])) == len(got)


@pytest.mark.parametrize("mode", ["ANCHOR_TO_START", "ANCHOR_TO_END", "ADJUST_TO_FILL"])
def test_building_from_pga_matches_the_data_table(mode):
    b = dsl.load(BUILDING % {"mode": mode})
    ref = scenes.building(w=25.3, d=19.7, h=31.0, mode=dsl.MODES[mode])
    for f in ("size", "position", "seed", "custom"):
        b["axioms"][f] = ref["axioms"][f]
    got = oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"])
    want = oracle.derive(G.DEFAULT_PROCS, ref["entries"], ref["axioms"])
    assert len(got) == len(want) > 1000
    assert (_multiset(got) == _multiset(want)).all()


def test_expression_arguments_use_the_reference_packing():
    g = dsl.parse("axiom Box A; terminal T (1, 0); A = SubDiv(X) { Exp(ShapeSize(Y) * -0.5): T | -1: T };")
    entries, _ = dsl.lower(g)
    p = entries[0]["parameters"][1]
    want = G.exp(("a", 13), ("s", -0.5), ("op", G.OPT_MULTI))
    assert int(p["type"]) == G.PT_EXP
    assert (p["value"][: len(want.values)] == np.array(want.values, np.float32)).all()


def test_a_rule_used_on_both_shapes_is_lowered_per_shape():
    g = dsl.parse("""axiom Box A; terminal T (1, 0);
                     A = CompSplit() { Piece | Piece | Discard() };
                     Piece = SubDiv(X) { -1: T | -1: T };""")
    entries, roots = dsl.lower(g)
    codes = sorted(int(e["operatorCode"]) for e in entries)
    assert G.QUAD_SUBDIVIDE in codes and G.QUAD_GENERATE in codes and G.BOX_COMPONENT_SPLIT in codes


@pytest.mark.parametrize("text, words", [
    ("axiom Box A; A = SetAsDynamicConvexRightPrism((0, 0.5), (-0.5, -0.5), (0.5, -0.5)) B; B = Discard();",
     ["SetAsDynamicConvexRightPrism", "'A'"]),
    ("axiom Box A; terminal T (1, 0); A = Scale(-1, 2) T;", ["Scale", "three"]),
    ("axiom Box A; terminal T (1, 0); A = RandomRule() { 0.5: T | 0.5: T };", ["RandomRule", "chance"]),
    ("axiom Box A; A = SubDiv(X) { -1: Nowhere };", ["unknown symbol", "Nowhere"]),
    ("axiom Box A;\nA = SubDiv(X) { -1 Discard() };", ["line 2", "':'"]),
    ("axiom Box A; terminal T (2, 3); A = T;", ["generation function 2"]),
])
def test_errors_name_the_problem(text, words):
    with pytest.raises(dsl.DslError) as e:
        dsl.lower(dsl.parse(text))
    for w in words:
        assert w in str(e.value)


AFFINE = """
axiom Box Tower;
terminal Block (1, 0);
terminal Roof (1, 1);
terminal Panel (1, 2);

Tower = RandomRule(ShapeSeed()) { 0.5: Narrow | 0.5: Body };
Narrow = SubDiv(Y) { -1: Body | 2: Scale(-0.8, -1, -0.8) Body };
Body = Translate(0.5, 0, Exp(ShapeSize(X) * -0.25)) CompSplit() { Roof | Discard() | Face };
Face = RandomRule(ShapeCustomAttribute()) { 0.3: Scale(1.5, -0.5, 1) Panel | 0.7: Extrude(0.2) Block };
"""


def _affine_table():
    """AFFINE built as data with the same rules in a different order."""
    from operatorgraph_gb300.grammar import DispatchTable, Entry, scalar, shape_attr

    return DispatchTable([
        Entry(G.BOX_RANDOM_RULE, [shape_attr(15), scalar(0.5), scalar(0.5)], [(1, 0), (3, 0)]),
        Entry(G.BOX_SUBDIVIDE, [scalar(1), scalar(-1), scalar(2)], [(3, 0), (2, 0)]),
        Entry(G.BOX_SCALE, [scalar(-0.8), scalar(-1), scalar(-0.8)], [(3, 0)]),
        Entry(G.BOX_TRANSLATE, [scalar(0.5), scalar(0), G.exp(("a", 12), ("s", -0.25), ("op", G.OPT_MULTI))],
              [(4, 0)]),
        Entry(G.BOX_COMPONENT_SPLIT, [], [(5, 0), (6, 0), (7, 0)]),
        Entry(G.QUAD_GENERATE, [scalar(1)], []),
        Entry(G.QUAD_DISCARD, [], []),
        Entry(G.QUAD_RANDOM_RULE, [shape_attr(16), scalar(0.3), scalar(0.7)], [(8, 0), (10, 0)]),
        Entry(G.QUAD_SCALE, [scalar(1.5), scalar(-0.5), scalar(1)], [(9, 0)]),
        Entry(G.QUAD_GENERATE, [scalar(2)], []),
        Entry(G.QUAD_EXTRUDE, [scalar(0), scalar(0.2)], [(11, 0)]),
        Entry(G.BOX_GENERATE, [scalar(0)], []),
    ]).to_array()


def test_translate_scale_random_rule_from_pga_match_the_data_table():
    b = dsl.load(AFFINE, n_axioms=12)
    rng = np.random.default_rng(4)
    b["axioms"]["size"] = rng.uniform(1.0, 5.0, (12, 3)).astype(np.float32)
    b["axioms"]["position"] = rng.uniform(-20, 20, (12, 3)).astype(np.float32)
    b["axioms"]["seed"] = rng.uniform(0.0, 3.0, 12).astype(np.float32)
    b["axioms"]["custom"] = rng.uniform(0.0, 1.0, 12).astype(np.float32)
    ax = b["axioms"].copy()
    ax["entry"] = 0
    got = oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"])
    want = oracle.derive(G.DEFAULT_PROCS, _affine_table(), ax)
    assert len(got) == len(want) > 12
    assert (_multiset(got) == _multiset(want)).all()
    kinds = set((got["rule"] >> 24).tolist())
    assert len(kinds) == 3  # blocks (box), roofs and panels (quads) all chosen somewhere


def _scene_lots(name, n, rng):
    """(sizes, positions, seeds) of n lots as the reference's test-runner scene
    for the grammar builds them (src/test_runner/*.cuh AxiomTraits): the
    grammars' absolute splits and extents are written for those sizes, and the
    reference evaluator throws on lots they do not fit."""
    seed = rng.uniform(0.0, 1.0, n).astype(np.float32)
    if name == "mc_skyscraper":  # MC_Skyscrapers.cuh:88-101
        side = (np.round(2 * seed) + 2) * 5
        size = np.stack([side, (np.round(3 * seed) + 2) * 15, side], 1)
    elif name.startswith("3d_tree"):  # 3DTree_*.cuh: 16 x 16 x 16
        size = np.full((n, 3), 16.0)
    elif name == "mc_spaceship":  # MC_Spaceship.cuh
        size = np.tile([5.0, 4.5, 8.0], (n, 1))
    elif name == "commercial":  # Commercial.cuh
        size = np.tile([30.0, 45.0, 30.0], (n, 1))
    else:  # MengerSponge.cuh: unit cubes
        size = np.ones((n, 3))
    pos = rng.uniform(-200, 200, (n, 3)).astype(np.float32)
    return size.astype(np.float32), pos, seed


# The reference grammars this engine derives (every operator they use is one of
# its operators) and the smallest terminal count expected for 12 lots.
FROM_FILE = {"menger_sponge_3": 96_000, "mc_skyscraper": 1000, "3d_tree_4_3": 1000, "3d_tree_8_3": 100_000,
             "3d_tree_12_2": 50_000, "mc_spaceship": 100, "commercial": 1000}


@pytest.mark.parametrize("name", sorted(FROM_FILE))
def test_reference_grammar_from_its_file_matches_the_reference_evaluator(name, tmp_path):
    """A grammar the reference's interpreter ships, lowered from its .pga file
    and derived by the oracle, gives the reference evaluator's terminals on the
    same table bit for bit, for 12 lots whose seeds and custom attributes reach
    the grammar's random choices.  Run where the reference sources are present;
    no grammar file is copied into this repository."""
    path = os.path.join(oracle.REFERENCE_ROOT, "src", "interpreter", "grammars", name, "grammar.pga")
    if not os.path.isfile(path) or not os.path.isfile(oracle.REF_HARNESS):
        pytest.skip("reference sources or the reference evaluator not present")
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import cases as C

    b = dsl.load(open(path).read(), n_axioms=12)
    rng = np.random.default_rng(11)
    size, pos, seed = _scene_lots(name, 12, rng)
    b["axioms"]["size"] = size
    b["axioms"]["position"] = pos
    b["axioms"]["seed"] = seed
    b["axioms"]["custom"] = rng.uniform(0.0, 1.0, 12).astype(np.float32)
    bf, tf = str(tmp_path / "b.bin"), str(tmp_path / "t.bin")
    G.write_batch_file(bf, b["entries"], b["axioms"])
    oracle.run_reference(bf, tf)
    ref = G.read_terminal_file(tf)
    got = oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"])
    assert len(got) == len(ref) >= FROM_FILE[name]
    assert C.digest(C.canonical(got)) == C.digest(C.canonical(ref))
    if name == "mc_skyscraper":
        assert len(set((got["rule"] >> 24).tolist())) >= 8  # columns, walls, windows, roofs


def test_reference_grammar_files_parse():
    """Every grammar the reference's interpreter ships parses; the ones that use
    only this engine's operators lower and derive, the others name the
    operator they need."""
    root = os.path.join(oracle.REFERENCE_ROOT, "src", "interpreter", "grammars")
    if not os.path.isdir(root):
        pytest.skip("reference sources not present")
    names = sorted(os.listdir(root))
    assert len(names) >= 9
    lowered = 0
    for name in names:
        path = os.path.join(root, name, "grammar.pga")
        g = dsl.parse(open(path).read())
        assert g["axioms"] and g["rules"], name
        try:
            entries, roots = dsl.lower(g)
        except dsl.DslError as err:
            assert "not supported" in str(err), (name, str(err))
            continue
        ax = G.make_axioms(1)
        ax["shape"], ax["entry"] = roots[0]
        ax["size"] = _scene_lots(name, 1, np.random.default_rng(0))[0]
        n = len(oracle.derive(G.DEFAULT_PROCS, entries, ax))
        assert n > 0
        if name.startswith("menger_sponge"):
            assert n == 8000  # the depth-3 sponge of a unit cube
        lowered += 1
    assert lowered >= len(FROM_FILE)


@pytest.mark.gpu
def test_pga_grammar_on_the_gpu():
    pytest.importorskip("torch")
    from operatorgraph_gb300 import build as B
    from operatorgraph_gb300.engine import Engine, terminals_to_numpy

    B.build()
    b = dsl.load(BUILDING % {"mode": "ANCHOR_TO_END"}, n_axioms=16)
    b["axioms"] = scenes.city_axioms(16)
    b["axioms"]["entry"] = dsl.lower(dsl.parse(BUILDING % {"mode": "ANCHOR_TO_END"}))[1][0][1]
    ref = oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"])
    eng = Engine(b["entries"], node_capacity=1 << 20, max_terminals=1 << 20)
    out, n, rep = eng.execute(b["axioms"], capacity=len(ref))
    got = terminals_to_numpy(out, n)
    eng.release()
    assert n == len(ref)
    ka = np.sort(got.view(np.uint8).reshape(n, 64).view(np.dtype((np.void, 64))).ravel())
    kb = np.sort(ref.view(np.uint8).reshape(n, 64).view(np.dtype((np.void, 64))).ravel())
    assert (ka == kb).all()
