"""The oracle (CPU restatement) pinned against the reference's own outputs.

The golden fixtures were produced by the reference's SinglePhaseEvaluator
(tests/golden/make_golden.py); the known answers below are the reference's
probe values for the Menger sponge.  No GPU needed.
"""
import glob
import os

import numpy as np
import pytest

import oracle
from operatorgraph_gb300 import grammar as G
from operatorgraph_gb300 import scenes

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


def load_case(path):
    z = np.load(path)
    b = {"entries": z["entries"].view(G.ENTRY_DT), "axioms": z["axioms"].view(G.AXIOM_DT)}
    b["blocks"] = z["blocks"] if "blocks" in z else None
    b["block_stride"] = int(z["block_stride"]) if "block_stride" in z else 0
    return b, z


def canonical(t, num_entries=None):
    import sys

    sys.path.insert(0, os.path.join(HERE, "golden"))
    import cases

    return cases.canonical(t, num_entries), cases.digest


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_matches_reference_golden(path):
    b, z = load_case(path)
    t = oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"], b["blocks"], b["block_stride"])
    n_base = len(b["entries"]) if b["blocks"] is not None else None
    canon, digest = canonical(t, n_base)
    assert len(t) == int(z["count"])
    if "terminals" in z:
        ref = z["terminals"].view(G.TERMINAL_DT)
        assert np.array_equal(canon["m"].view(np.uint32), ref["m"].view(np.uint32))
        assert np.array_equal(canon["rule"], ref["rule"])
        assert np.array_equal(canon["custom"], ref["custom"])
        assert np.array_equal(np.sort(t["path"]), z["paths"]), "path hashes differ from the reference's"
    assert digest(canon) == str(z["digest"])
    # the records with their derivation-path hashes, as the instrumented
    # reference derived them (each path names the same record in both)
    import cases

    assert digest(cases.canonical_paths(t, n_base)) == str(z["digest_path"]), "records by path differ"


@pytest.mark.parametrize("path", [p for p in GOLDEN if "mesh_counts" in np.load(p)],
                         ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_meshes_match_reference_golden(path):
    """Triangle meshes: the restatement's vertices (positions, normals, uvs)
    and triangles against the reference's GenerationFunction<.., 0> output, as
    order-free faces, mesh by mesh."""
    import sys

    sys.path.insert(0, os.path.join(HERE, "golden"))
    import cases

    b, z = load_case(path)
    _, meshes = oracle.derive_meshes(G.DEFAULT_PROCS, b["entries"], b["axioms"], b["blocks"], b["block_stride"])
    counts = z["mesh_counts"]
    assert len(meshes) == len(counts)
    for m, ((v, i), (nv, ni), dg) in enumerate(zip(meshes, counts, z["mesh_digests"])):
        assert (len(v), len(i)) == (nv, ni), m
        assert cases.mesh_digest(v, i) == str(dg), m


def test_golden_fixtures_present():
    assert len(GOLDEN) >= 15


def test_menger_depth5_known_answer():
    """Reference probe: threshold 0.005 -> 3,200,000 terminals, checksum 13169.1925,
    first terminal (FIFO order) at (-0.497942358)^3 with size 0.00411522621."""
    b = scenes.menger(0.005)
    t = oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"])
    assert len(t) == 3_200_000
    # The probe summed the float expression M14 + 2 M24 + 3 M34 + M11 into a double.
    m = t["m"]
    per = ((m[:, 3] + np.float32(2) * m[:, 7]) + np.float32(3) * m[:, 11]) + m[:, 0]
    checksum = per.astype(np.float64).sum()
    assert abs(checksum - 13169.1925) < 1e-3
    corner = np.isclose(t["m"][:, 3], -0.497942358) & np.isclose(t["m"][:, 7], -0.497942358) & \
        np.isclose(t["m"][:, 11], -0.497942358)
    assert corner.sum() == 1
    assert np.isclose(t["m"][corner][0, 0], 0.00411522621)


def test_city_4096_count():
    """The 4096-building city (seed 1234) gives 5,856,274 terminals on the
    reference's evaluator (measured with oracle/_ref)."""
    b = scenes.city(4096)
    t = oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"])
    assert len(t) == 5_856_274


def test_path_hashes_unique():
    b = scenes.city(64)
    t = oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"])
    assert len(np.unique(t["path"])) == len(t)


def test_errors_match_reference_behaviour():
    """Subdivide<DynParams> with absolute factors larger than the shape throws in
    the reference (Subdivide.cuh:208-216); Repeat with extent 0 throws
    (Repeat.cuh:75-83); a shape of the wrong type is rejected (CPUEvaluator.h:64-68)."""
    from operatorgraph_gb300.grammar import DispatchTable, Entry, scalar

    bad_sub = DispatchTable([Entry(G.BOX_SUBDIVIDE, [scalar(0), scalar(5.0), scalar(-1)], [(1, 0), (1, 0)]),
                             Entry(G.BOX_GENERATE, [scalar(0)], [])]).to_array()
    with pytest.raises(oracle.OracleError) as e:
        oracle.derive(G.DEFAULT_PROCS, bad_sub, G.make_axioms(1))
    assert e.value.status == 5
    bad_rep = DispatchTable([Entry(G.BOX_REPEAT, [scalar(0), scalar(0.0), scalar(0)], [(1, 0)]),
                             Entry(G.BOX_GENERATE, [scalar(0)], [])]).to_array()
    with pytest.raises(oracle.OracleError) as e:
        oracle.derive(G.DEFAULT_PROCS, bad_rep, G.make_axioms(1))
    assert e.value.status == 5
    mismatch = DispatchTable([Entry(G.QUAD_GENERATE, [scalar(0)], [])]).to_array()
    with pytest.raises(oracle.OracleError) as e:
        oracle.derive(G.DEFAULT_PROCS, mismatch, G.make_axioms(1))  # Box axiom into a Quad procedure
    assert e.value.status == 4


def _check_lbvh_structure(nodes, lp, n):
    """Each internal node has two children, every node but the root one parent,
    every leaf is reached exactly once and node ranges are contiguous."""
    seen_leaf = np.zeros(n, np.int64)
    seen_int = np.zeros(n - 1, np.int64)
    lo = np.zeros(n - 1, np.int64)
    hi = np.zeros(n - 1, np.int64)
    order = []
    stack = [0]
    while stack:
        i = stack.pop()
        order.append(i)
        for c in nodes[i, 1:]:
            if c >= 0:
                seen_leaf[c] += 1
                assert lp[c] == i
            else:
                seen_int[-c] += 1
                assert nodes[-c, 0] == i
                stack.append(-c)
    assert (seen_leaf == 1).all() and (seen_int[1:] == 1).all() and seen_int[0] == 0
    for i in reversed(order):
        rng = []
        for c in nodes[i, 1:]:
            rng.append((c, c) if c >= 0 else (lo[-c], hi[-c]))
        assert rng[0][1] + 1 == rng[1][0]
        lo[i], hi[i] = rng[0][0], rng[1][1]
    assert lo[0] == 0 and hi[0] == n - 1


@pytest.mark.parametrize("scene", ["menger", "city"])
def test_oracle_lbvh_invariants(scene):
    b = scenes.menger(0.05) if scene == "menger" else scenes.city(16)
    t = oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"])
    bounds = (-0.5, -0.5, -0.5, 0.5, 0.5, 0.5) if scene == "menger" else (-50, -50, -1, 800, 100, 400)
    nodes, lp, aabb, lt, keys = oracle.lbvh(t, bounds)
    n = len(t)
    _check_lbvh_structure(nodes, lp, n)
    assert np.all(keys[1:] >= keys[:-1])
    assert sorted(lt.tolist()) == list(range(n))
    # Every internal box contains its children's boxes; the root contains every terminal centre.
    c = np.stack([t["m"][:, 3], t["m"][:, 7], t["m"][:, 11]], 1)
    assert np.all(c >= aabb[0, :3] - 1e-6) and np.all(c <= aabb[0, 3:] + 1e-6)
    for i in range(n - 1):
        for ch in nodes[i, 1:]:
            if ch < 0:
                assert np.all(aabb[-ch, :3] >= aabb[i, :3]) and np.all(aabb[-ch, 3:] <= aabb[i, 3:])


def _spread10(v):
    v = v.astype(np.uint32)
    v = (v | (v << np.uint32(16))) & np.uint32(0x030000FF)
    v = (v | (v << np.uint32(8))) & np.uint32(0x0300F00F)
    v = (v | (v << np.uint32(4))) & np.uint32(0x030C30C3)
    v = (v | (v << np.uint32(2))) & np.uint32(0x09249249)
    return v


def test_oracle_lbvh_leaf_order_is_morton_then_path_then_index():
    """The LBVH's leaf order, pinned independently of the restatement's C++:
    30-bit Morton codes of the terminal centres (FP32 (c - min) / size * 1023,
    truncated, clamped at 0), then the full derivation-path hash, then the
    terminal index; keys morton << 34 | path >> 30.  Synthetic records with
    many shared centres, shared top path bits and repeated paths, so every
    tie-break level decides somewhere."""
    n = 20_000
    rng = np.random.default_rng(3)
    rec = np.zeros(n, G.TERMINAL_DT)
    m = rng.uniform(-0.5, 0.5, (n, 12)).astype(np.float32)
    m[:, [3, 7, 11]] = rng.uniform(-9.0, 9.0, (n, 3)).astype(np.float32)
    shared = rng.choice(n, n // 2, replace=False)
    m[np.ix_(shared, [3, 7, 11])] = rng.uniform(-9.0, 9.0, (40, 3)).astype(np.float32)[rng.integers(0, 40, n // 2)]
    paths = rng.integers(0, 2**64, size=n, dtype=np.uint64)
    top = rng.choice(n, n // 4, replace=False)
    paths[top] = (paths[top] & np.uint64((1 << 54) - 1)) | np.uint64(0x155 << 54)  # shared top 10 bits
    dst, src = rng.choice(n, n // 20, replace=False), rng.choice(n, n // 20, replace=False)
    paths[dst] = paths[src]
    m[np.ix_(dst, [3, 7, 11])] = m[np.ix_(src, [3, 7, 11])]  # equal keys and equal paths
    rec["m"] = m
    rec["path"] = paths
    bounds = np.array([-10.0, -10.0, -10.0, 10.0, 10.0, 10.0], np.float32)
    _, _, _, lt, keys = oracle.lbvh(rec, tuple(float(v) for v in bounds))
    size = bounds[3:] - bounds[:3]
    code = np.zeros(n, np.uint32)
    for k, col in enumerate((3, 7, 11)):
        nc = (m[:, col] - bounds[k]) / size[k]
        q = nc * np.float32(1023.0)
        v = np.where(q > 0, np.minimum(q, np.float32(4294967040.0)), 0).astype(np.uint32)
        code |= _spread10(v) << np.uint32(k)
    want_keys = (code.astype(np.uint64) << np.uint64(34)) | (paths >> np.uint64(30))
    order = np.lexsort((np.arange(n), paths, code))  # last key is the primary one
    assert np.array_equal(lt.astype(np.int64), order), "leaf order differs"
    assert np.array_equal(keys, want_keys[order]), "keys differ"
    assert int((code[order][1:] == code[order][:-1]).sum()) > n // 4
    assert int((paths[order][1:] == paths[order][:-1]).sum()) > 100


def test_phases_defer_and_collide():
    """Multi-phase semantics of the restatement: a shape reaching a rule of a
    later phase waits for it; IfCollides in phase 1 sees the colliders stored
    in phase 0 (and none stored in its own phase); edges into one entry that
    name different phases are rejected."""
    from operatorgraph_gb300.grammar import DispatchTable, Entry, scalar

    tab = DispatchTable([
        Entry(G.BOX_COLLIDER, [scalar(5)], [(1, 0)]),                  # 0: store with tag 5
        Entry(G.BOX_GENERATE, [scalar(0)], []),                        # 1
        Entry(G.BOX_IF_COLLIDES, [scalar(5)], [(3, 1), (4, 1)]),       # 2: phase-0 test (sees nothing yet)
        Entry(G.BOX_GENERATE, [scalar(1)], []),                        # 3 hit
        Entry(G.BOX_REPLICATE, [], [(5, 1)]),                          # 4 miss: retry in phase 1
        Entry(G.BOX_IF_COLLIDES, [scalar(5)], [(6, 1), (7, 1)]),       # 5
        Entry(G.BOX_GENERATE, [scalar(2)], []),                        # 6 hit in phase 1
        Entry(G.BOX_GENERATE, [scalar(3)], []),                        # 7
    ]).to_array()
    ax = G.make_axioms(3)
    ax["entry"] = [0, 2, 2]
    ax["size"] = 1.0
    ax["position"] = [(0, 0, 0), (0.5, 0, 0), (5, 0, 0)]  # axiom 1 overlaps the collider, axiom 2 does not
    t = oracle.derive(G.DEFAULT_PROCS, tab, ax)
    tidx = sorted(((t["rule"] >> 24) & 0x7F).tolist())
    assert tidx == [0, 2, 3]
    bad = DispatchTable([Entry(G.BOX_REPLICATE, [], [(1, 0), (1, 1)]), Entry(G.BOX_GENERATE, [scalar(0)], [])]).to_array()
    with pytest.raises(oracle.OracleError) as e:
        oracle.derive(G.DEFAULT_PROCS, bad, G.make_axioms(1))
    assert e.value.status == 5
