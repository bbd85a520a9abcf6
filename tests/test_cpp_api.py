"""The C++ operator API (include/pga/core.hpp, include/pga/engine.hpp).

Grammars written in the reference's template syntax (tests/cpp/lower_scenes.cpp)
are lowered to rule tables by a g++-built program; the oracle derives them and
the results are compared with the same grammars built as data.  Dynamic
procedure lists keep entry indices, so terminals match bit for bit including
path hashes; statically chained grammars add entries, so their transforms,
rules' terminal indices and custom attributes are compared as multisets.
"""
import shutil
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle
from operatorgraph_gb300 import grammar as G
from operatorgraph_gb300 import scenes

ROOT = Path(__file__).resolve().parents[1]


def _compile(src, out, extra=()):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"), str(src), "-o",
           str(out), *extra]
    subprocess.run(cmd, check=True, capture_output=True, text=True)


def _read_scenes(path):
    data = path.read_bytes()
    off, out = 0, {}

    def u32():
        nonlocal off
        v = struct.unpack_from("<I", data, off)[0]
        off += 4
        return v

    while off < len(data):
        n = u32()
        name = data[off:off + n].decode()
        off += n
        np_ = u32()
        if np_ == 0xFFFFFFFF:
            m = u32()
            out[name] = data[off:off + m].decode()
            off += m
            continue
        procs = np.frombuffer(data, G.PROC_DT, np_, off).copy()
        off += np_ * G.PROC_DT.itemsize
        ne = u32()
        entries = np.frombuffer(data, G.ENTRY_DT, ne, off).copy()
        off += ne * G.ENTRY_DT.itemsize
        out[name] = (procs, entries, u32())
    return out


@pytest.fixture(scope="module")
def lowered(tmp_path_factory):
    d = tmp_path_factory.mktemp("cpp")
    exe = d / "lower_scenes"
    _compile(ROOT / "tests" / "cpp" / "lower_scenes.cpp", exe)
    subprocess.run([str(exe), str(d / "out.bin")], check=True)
    return _read_scenes(d / "out.bin")


def _derive(procs, entries, axioms):
    return oracle.derive(procs, entries, axioms)


def _multiset(t):
    key = np.concatenate([t["m"].view(np.uint32), (t["rule"] >> 24)[:, None], t["custom"].view(np.uint32)[:, None]],
                         axis=1)
    return key[np.lexsort(key.T[::-1])]


def _same_bits(a, b):
    assert len(a) == len(b)
    ka = np.sort(a.view(np.uint8).reshape(len(a), -1).view(np.dtype((np.void, 64))).ravel())
    kb = np.sort(b.view(np.uint8).reshape(len(b), -1).view(np.dtype((np.void, 64))).ravel())
    assert (ka == kb).all()


def test_dynamic_menger_lowers_to_the_same_table(lowered):
    procs, entries, nuser = lowered["menger"]
    ref = scenes.menger_table(0.05)
    assert nuser == len(ref) == len(entries)
    for e, r in zip(entries, ref):
        pe, pr = procs[e["operatorCode"]], G.DEFAULT_PROCS[r["operatorCode"]]
        assert (pe["op"], pe["shape"], pe["numChildren"]) == (pr["op"], pr["shape"], pr["numChildren"])
        assert e["numParameters"] == r["numParameters"] and e["numSuccessors"] == r["numSuccessors"]
        k = int(r["numParameters"])
        assert (e["parameters"][:k] == r["parameters"][:k]).all()
        s = int(r["numSuccessors"])
        assert (e["successors"]["entryIndex"][:s] == r["successors"]["entryIndex"][:s]).all()
    b = scenes.menger(0.05)
    _same_bits(_derive(procs, entries, b["axioms"]), _derive(G.DEFAULT_PROCS, ref, b["axioms"]))


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_dynamic_building_is_bit_exact(lowered, mode):
    procs, entries, _ = lowered[f"building_dyn_m{mode}"]
    b = scenes.building(mode=mode)
    _same_bits(_derive(procs, entries, b["axioms"]), _derive(G.DEFAULT_PROCS, b["entries"], b["axioms"]))


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_static_chain_building_matches(lowered, mode):
    procs, entries, nuser = lowered[f"building_static_m{mode}"]
    assert nuser == 1 and len(entries) == 12  # the chain became 11 more entries
    b = scenes.building(w=25.3, d=19.7, h=31.0, mode=mode)
    got = _derive(procs, entries, b["axioms"])
    want = _derive(G.DEFAULT_PROCS, b["entries"], b["axioms"])
    assert len(got) == len(want) > 1000
    assert (_multiset(got) == _multiset(want)).all()
    assert len(np.unique(got["path"])) == len(got)


def test_expression_parameters_evaluate_like_scalars(lowered):
    procs, entries, _ = lowered["building_exp"]
    kinds = {int(p["type"]) for e in entries for p in e["parameters"][: e["numParameters"]]}
    assert G.PT_EXP in kinds
    b = scenes.building(w=25.3, d=19.7, h=31.0)
    got = _derive(procs, entries, b["axioms"])
    want = _derive(G.DEFAULT_PROCS, b["entries"], b["axioms"])
    assert (_multiset(got) == _multiset(want)).all()


def test_static_calls_follow_the_table(lowered):
    procs, entries, _ = lowered["menger_calls"]
    b = scenes.menger(0.05)
    _same_bits(_derive(procs, entries, b["axioms"]), _derive(G.DEFAULT_PROCS, scenes.menger_table(0.05), b["axioms"]))


def test_static_random_rule_with_dynamic_pairs_is_bit_exact(lowered):
    """RandomRule<DynParam<0>, Pair<DynParam<k>, DCall<k-1>>...> lowers to the
    static-form operator with the entry's chance, weights and successors: the
    same table as the golden random_static_mix case (whose fixture came from
    the reference's evaluator), so the terminals match bit for bit."""
    import sys

    sys.path.insert(0, str(ROOT / "tests" / "golden"))
    import cases as C

    procs, entries, nuser = lowered["random_static_dyn"]
    b = C.random_static_mix()
    assert nuser == len(entries) == len(b["entries"])
    assert {int(p["op"]) for p in procs} >= {G.OP_RANDOM_RULE_STATIC, G.OP_COMPONENT_SPLIT}
    _same_bits(_derive(procs, entries, b["axioms"]), _derive(G.DEFAULT_PROCS, b["entries"], b["axioms"]))


def _rotate_static_table():
    """tests/cpp/lower_scenes.cpp rotate_static built as data."""
    from operatorgraph_gb300.grammar import DispatchTable, Entry, scalar

    return DispatchTable([
        Entry(G.BOX_REPLICATE, [], [(1, 0), (2, 0), (5, 0)]),                                      # 0
        Entry(G.BOX_GENERATE, [scalar(0)], []),                                                    # 1
        Entry(G.BOX_ROTATE, [scalar(0), scalar(90), scalar(0)], [(3, 0)]),                         # 2
        Entry(G.BOX_SUBDIVIDE, [scalar(0), scalar(-1), scalar(-2)], [(1, 0), (4, 0)]),             # 3
        Entry(G.BOX_ROTATE, [scalar(0), scalar(0), scalar(-37)], [(1, 0)]),                        # 4
        Entry(G.BOX_ROTATE, [scalar(30), scalar(-47.5), scalar(12.25)], [(6, 0)]),                 # 5
        Entry(G.BOX_COMPONENT_SPLIT, [], [(7, 0), (12, 0), (13, 0)]),                              # 6
        Entry(G.QUAD_ROTATE, [scalar(0), scalar(0), scalar(45)], [(8, 0)]),                        # 7
        Entry(G.QUAD_TRANSLATE, [scalar(0.5), G.exp(("a", 13), ("s", 0.5), ("op", G.OPT_MULTI)), scalar(-0.25)],
              [(9, 0)]),                                                                            # 8
        Entry(G.QUAD_SCALE, [scalar(-0.5), scalar(2), scalar(1)], [(10, 0)]),                      # 9
        Entry(G.QUAD_EXTRUDE, [scalar(0), scalar(0.75)], [(11, 0)]),                               # 10
        Entry(G.BOX_GENERATE, [scalar(0)], []),                                                    # 11
        Entry(G.QUAD_DISCARD, [], []),                                                             # 12
        Entry(G.QUAD_REPLICATE, [], [(14, 0), (15, 0)]),                                           # 13
        Entry(G.QUAD_GENERATE, [scalar(1)], []),                                                   # 14
        Entry(G.QUAD_ROTATE, [scalar(90), scalar(90), scalar(0)], [(14, 0)]),                      # 15
    ]).to_array()


def test_static_rotate_replicate_chain_matches(lowered):
    procs, entries, nuser = lowered["rotate_static"]
    assert nuser == 1 and len(entries) > 10
    ax = G.make_axioms(6)
    rng = np.random.default_rng(5)
    ax["size"] = rng.uniform(1.0, 4.0, (6, 3)).astype(np.float32)
    ax["position"] = rng.uniform(-10, 10, (6, 3)).astype(np.float32)
    got = _derive(procs, entries, ax)
    want = _derive(G.DEFAULT_PROCS, _rotate_static_table(), ax)
    assert len(got) == len(want) == 6 * 12  # copy, 2 pieces, top, 4 sides x 2
    assert (_multiset(got) == _multiset(want)).all()


def test_static_if_swap_size_chain_matches(lowered):
    from operatorgraph_gb300.grammar import DispatchTable, Entry, scalar

    procs, entries, _ = lowered["if_swap_static"]
    tab = DispatchTable([
        Entry(G.BOX_IF, [G.exp(("a", 12), ("s", 1.5), ("op", G.OPT_GT))], [(1, 0), (3, 0)]),
        Entry(G.BOX_SWAP_SIZE, [scalar(1), scalar(2), scalar(0)], [(2, 0)]),
        Entry(G.BOX_GENERATE, [scalar(0)], []),
        Entry(G.BOX_SUBDIVIDE, [scalar(0), scalar(-1), scalar(-1)], [(2, 0), (4, 0)]),
        Entry(G.BOX_SWAP_SIZE, [scalar(0), scalar(2), scalar(1)], [(5, 0)]),
        Entry(G.BOX_GENERATE, [scalar(1)], []),
    ]).to_array()
    ax = G.make_axioms(8)
    rng = np.random.default_rng(9)
    ax["size"] = rng.uniform(0.5, 3.0, (8, 3)).astype(np.float32)
    got = _derive(procs, entries, ax)
    want = _derive(G.DEFAULT_PROCS, tab, ax)
    assert len(got) == len(want) > 8
    assert (_multiset(got) == _multiset(want)).all()


def test_mesh_generates_lower_to_the_mesh_operator(lowered):
    """Generate<false, 0, ...> lowers to PGA_OP_GENERATE_MESH; the oracle's
    meshes of the lowered table equal those of the same grammar built as data."""
    from operatorgraph_gb300.grammar import DispatchTable, Entry, scalar

    procs, entries, _ = lowered["mesh_terminals"]
    assert G.OP_GENERATE_MESH in {int(p["op"]) for p in procs}
    tab = DispatchTable([
        Entry(G.BOX_REPLICATE, [], [(1, 0), (2, 0)]),
        Entry(G.BOX_GENERATE_MESH, [scalar(0)], []),
        Entry(G.BOX_COMPONENT_SPLIT, [], [(3, 0), (4, 0), (5, 0)]),
        Entry(G.QUAD_GENERATE_MESH, [scalar(1)], []),
        Entry(G.QUAD_DISCARD, [], []),
        Entry(G.QUAD_GENERATE, [scalar(2)], []),
    ]).to_array()
    ax = G.make_axioms(3)
    ax["size"] = [(1.0, 2.0, 3.0), (2.5, 0.5, 1.5), (4.0, 4.0, 0.25)]
    t_got, m_got = oracle.derive_meshes(procs, entries, ax)
    t_want, m_want = oracle.derive_meshes(G.DEFAULT_PROCS, tab, ax)
    assert (_multiset(t_got) == _multiset(t_want)).all()
    assert len(m_got) == len(m_want) == 2
    for (v, i), (w, j) in zip(m_got, m_want):
        assert np.array_equal(G.mesh_faces(v, i).view(np.uint32), G.mesh_faces(w, j).view(np.uint32))


def test_unsupported_forms_are_lowering_errors(lowered):
    assert "generation function 2" in lowered["bad_generation_function"]
    assert "DynParam<0>" in lowered["bad_dynparam"]


@pytest.mark.gpu
def test_evaluator_runs_the_menger_grammar(tmp_path):
    """Evaluator<ProcedureList> through libpga_gb300.so on the GPU, against the oracle."""
    from operatorgraph_gb300 import build as B

    B.build()
    lib_dir = Path(B.LIB).parent
    cuda = Path("/usr/local/cuda")
    exe = tmp_path / "evaluator_menger"
    _compile(ROOT / "tests" / "cpp" / "evaluator_menger.cpp", exe,
             ["-I", str(cuda / "include"), "-L", str(lib_dir), "-lpga_gb300", f"-Wl,-rpath,{lib_dir}",
              "-L", str(cuda / "lib64"), "-lcudart", f"-Wl,-rpath,{cuda / 'lib64'}"])
    res = subprocess.run([str(exe), str(tmp_path / "t.bin")], check=True, capture_output=True, text=True)
    n, count, overflow = (int(v) for v in res.stdout.split())
    assert n == count == 8000
    assert overflow == 2  # PGA_ERR_OUTPUT_OVERFLOW
    got = np.fromfile(tmp_path / "t.bin", G.TERMINAL_DT)
    b = scenes.menger(0.05)
    _same_bits(got, _derive(G.DEFAULT_PROCS, scenes.menger_table(0.05), b["axioms"]))
