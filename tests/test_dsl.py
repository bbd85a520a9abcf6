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
    ("axiom Box A; A = Translate(0, 1, 0) B; B = Discard();", ["Translate", "'A'"]),
    ("axiom Box A; A = SubDiv(X) { -1: Nowhere };", ["unknown symbol", "Nowhere"]),
    ("axiom Box A;\nA = SubDiv(X) { -1 Discard() };", ["line 2", "':'"]),
    ("axiom Box A; terminal T (0, 3); A = T;", ["instanced"]),
])
def test_errors_name_the_problem(text, words):
    with pytest.raises(dsl.DslError) as e:
        dsl.lower(dsl.parse(text))
    for w in words:
        assert w in str(e.value)


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
        ax["size"] = 1.0
        n = len(oracle.derive(G.DEFAULT_PROCS, entries, ax))
        assert n > 0
        if name.startswith("menger_sponge"):
            assert n == 8000  # the depth-3 sponge of a unit cube
        lowered += 1
    assert lowered >= 1


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
