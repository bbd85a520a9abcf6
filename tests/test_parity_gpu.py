"""GPU parity: the CUDA engine against the reference's golden outputs and the
oracle, through the C ABI.

Bar: terminal count, rule ids, custom attributes, derivation-path hashes and
transforms bit-exact (the derivation is written with round-to-nearest
intrinsics and no FMA, so the FP32 transforms match to the bit, well inside
the 1e-5 relative tolerance the target allows); Morton keys, LBVH topology and
boxes bit-exact.  Multisets are compared after sorting (queue order is free).
"""
import glob
import os

import numpy as np
import pytest

import oracle
from operatorgraph_gb300 import grammar as G
from operatorgraph_gb300 import scenes

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
REL_TOL = 1e-5  # FP32 transform tolerance of the target; observed error is 0


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from operatorgraph_gb300 import build as B

    B.build()
    torch.cuda.set_device(0)


def _engine(entries, **kw):
    from operatorgraph_gb300.engine import Engine

    kw.setdefault("node_capacity", 1 << 20)
    kw.setdefault("max_terminals", 1 << 20)
    return Engine(entries, **kw)


def _run(b, plain=False, capacity=None, **kw):
    from operatorgraph_gb300.engine import terminals_to_numpy

    ref_n = None
    if capacity is None:
        ref_n = len(oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"], b["blocks"], b["block_stride"]))
        capacity = max(ref_n, 1)
    eng = _engine(b["entries"], block_stride=b["block_stride"], **kw)
    out, n, rep = eng.execute(b["axioms"], blocks=b["blocks"], capacity=capacity, plain=plain)
    torch.cuda.synchronize()
    got = terminals_to_numpy(out, n)
    return eng, out, got, rep


def _assert_same(got, ref):
    assert len(got) == len(ref)
    a, c = G.sort_terminals(got, by_path=True), G.sort_terminals(ref, by_path=True)
    assert np.array_equal(a["path"], c["path"]), "derivation-path hashes differ"
    assert np.array_equal(a["rule"], c["rule"]), "rule ids differ"
    assert np.array_equal(a["custom"].view(np.uint32), c["custom"].view(np.uint32))
    am, cm = a["m"] + np.float32(0), c["m"] + np.float32(0)
    denom = np.maximum(np.abs(cm), 1e-30)
    assert np.max(np.abs(am - cm) / denom) <= REL_TOL
    assert np.array_equal(am.view(np.uint32), cm.view(np.uint32)), "transforms not bit-exact"


def _load(path):
    z = np.load(path)
    b = {"entries": z["entries"].view(G.ENTRY_DT), "axioms": z["axioms"].view(G.AXIOM_DT)}
    b["blocks"] = z["blocks"] if "blocks" in z else None
    b["block_stride"] = int(z["block_stride"]) if "block_stride" in z else 0
    return b, z


@pytest.mark.parametrize("form", ["persistent", "queued", "plain", "grouped", "per_axiom"])
@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_golden_case(path, form):
    """persistent: the batched launch (leaf children expanded in place);
    queued: the same with every branching child queued (PGA_FLAG_NO_INLINE);
    plain: one axiom and one launch per level;
    grouped: the batched launch with the axioms seeded grouped by root entry
    (PGA_FLAG_GROUP_AXIOMS);
    per_axiom: one persistent launch per axiom, appended on the device."""
    import sys

    sys.path.insert(0, os.path.join(HERE, "golden"))
    import cases

    b, z = _load(path)
    plain = {"plain": True, "per_axiom": "per_axiom"}.get(form, False)
    eng, out, got, rep = _run(b, plain=plain, no_inline=form == "queued", group_axioms=form == "grouped")
    assert rep["status"] == 0
    n_base = len(b["entries"]) if b["blocks"] is not None else None
    canon = cases.canonical(got, n_base)
    assert len(got) == int(z["count"])
    assert cases.digest(canon) == str(z["digest"]), "differs from the reference's own output"
    assert cases.digest(cases.canonical_paths(got, n_base)) == str(z["digest_path"]), \
        "records by derivation path differ from the reference's own output"
    ref = oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"], b["blocks"], b["block_stride"])
    _assert_same(got, ref)
    if "mesh_counts" in z:
        # triangle meshes from the derived records (pga_generate_meshes)
        counts = z["mesh_counts"]
        meshes = eng.generate_meshes(out, len(got), [(int(nv), int(ni)) for nv, ni in counts])
        for m, ((v, i, nv, ni), (rv, ri), dg) in enumerate(zip(meshes, counts, z["mesh_digests"])):
            assert (nv, ni) == (rv, ri), m
            assert cases.mesh_digest(v.cpu().numpy(), i.cpu().numpy().view(np.uint32)) == str(dg), m
    eng.release()


@pytest.mark.parametrize("name", ["menger_d5", "city_4096", "facades_1024", "random_16", "city_4096_queued",
                                  "city_4096_dynamic"])
def test_full_size_bit_exact(name):
    """_queued: leaf children queued as work items; _dynamic: the last quarter
    of each wide level's items from the shared counter (the city's deepest
    level has ~0.4M items, above the four rounds of chunks the flag needs)."""
    kw = {"no_inline": True} if name.endswith("_queued") else {}
    if name.endswith("_dynamic"):
        kw = {"dynamic_chunks": True}
    name = name.replace("_queued", "").replace("_dynamic", "")
    if name == "menger_d5":
        b = scenes.menger(0.005)
    elif name == "city_4096":
        b = scenes.city(4096)
    elif name == "facades_1024":
        b = scenes.facades(1024)
    else:
        tabs = scenes.random_grammars(16)
        entries, offs = G.concat_tables(tabs)
        ax = G.make_axioms(64)
        ax["seed"] = 0.5
        ax["entry"] = [offs[i % 16] for i in range(64)]
        b = {"entries": entries, "axioms": ax, "blocks": None, "block_stride": 0}
    ref = oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"], b["blocks"], b["block_stride"])
    eng, out, got, rep = _run(b, capacity=len(ref), node_capacity=1 << 23, max_terminals=1 << 23, **kw)
    assert rep["status"] == 0
    _assert_same(got, ref)
    eng.release()


@pytest.mark.parametrize("scene", ["menger_d3", "building", "city_16", "menger_d5"])
def test_lbvh_bit_exact(scene):
    if scene == "menger_d3":
        b, bounds = scenes.menger(0.05), (-0.5, -0.5, -0.5, 0.5, 0.5, 0.5)
    elif scene == "menger_d5":
        b, bounds = scenes.menger(0.005), (-0.5, -0.5, -0.5, 0.5, 0.5, 0.5)
    elif scene == "building":
        b, bounds = scenes.building(), (-20, -20, -1, 20, 20, 40)
    else:
        b, bounds = scenes.city(16), (-50, -50, -1, 800, 100, 400)
    eng, out, got, rep = _run(b, node_capacity=1 << 23, max_terminals=1 << 23)
    n = len(got)
    bv = eng.lbvh(out, n, bounds)
    torch.cuda.synchronize()
    nodes, lp, aabb, lt, keys = oracle.lbvh(got, bounds)
    assert np.array_equal(bv["keys"].cpu().numpy().view(np.uint64), keys), "Morton keys differ"
    assert np.array_equal(bv["leafTerminal"].cpu().numpy().view(np.uint32), lt), "leaf order differs"
    assert np.array_equal(bv["nodes"].cpu().numpy(), nodes), "topology differs"
    assert np.array_equal(bv["leafParents"].cpu().numpy().view(np.uint32), lp)
    assert np.array_equal(bv["aabbs"].cpu().numpy().view(np.uint32), aabb.view(np.uint32)), "boxes differ"
    eng.release()


def test_repeat_runs_are_identical_as_multisets():
    b = scenes.city(256)
    eng, out, got1, _ = _run(b)
    out2, n2, _ = eng.execute(b["axioms"], capacity=len(got1))
    got2 = G.sort_terminals(
        out2[:n2].cpu().numpy().reshape(-1).view(G.TERMINAL_DT), by_path=True)
    assert np.array_equal(G.sort_terminals(got1, by_path=True).view(np.uint8), got2.view(np.uint8))
    eng.release()


def test_empty_batch():
    b = scenes.menger(0.05)
    eng = _engine(b["entries"])
    ax = torch.empty(0, dtype=torch.uint8, device="cuda")
    out, n, rep = eng.execute(ax, capacity=16)
    assert n == 0 and rep["status"] == 0
    eng.release()


def test_all_discarded():
    from operatorgraph_gb300.grammar import DispatchTable, Entry, scalar

    tab = DispatchTable([Entry(G.BOX_SUBDIVIDE, [scalar(0), scalar(-1), scalar(-1)], [(1, 0), (1, 0)]),
                         Entry(G.BOX_DISCARD, [], [])]).to_array()
    b = {"entries": tab, "axioms": G.make_axioms(100), "blocks": None, "block_stride": 0}
    eng, out, got, rep = _run(b, capacity=16)
    assert len(got) == 0 and rep["status"] == 0


def test_output_overflow_reports_status():
    from operatorgraph_gb300.engine import PgaError

    b = scenes.menger(0.05)
    eng = _engine(b["entries"])
    with pytest.raises(PgaError) as e:
        eng.execute(b["axioms"], capacity=100)
    assert e.value.status == 2
    # The engine and the context stay usable.
    out, n, rep = eng.execute(b["axioms"], capacity=8000)
    assert n == 8000
    eng.release()


def test_queue_overflow_reports_status():
    b = scenes.menger(0.05)
    eng = _engine(b["entries"], node_capacity=8)
    out, n, rep = eng.execute(b["axioms"], capacity=8000, check=False)
    assert rep["status"] == 1
    eng.release()


@pytest.mark.parametrize("kind", ["bad_param", "bad_opcode", "depth"])
def test_device_errors_are_statuses(kind):
    from operatorgraph_gb300.grammar import DispatchTable, Entry, scalar

    if kind == "bad_param":  # Repeat extent 0 (Repeat.cuh:75-83 traps on the GPU)
        tab = DispatchTable([Entry(G.BOX_REPEAT, [scalar(0), scalar(0.0), scalar(0)], [(1, 0)]),
                             Entry(G.BOX_GENERATE, [scalar(0)], [])]).to_array()
        want = 5
    elif kind == "bad_opcode":  # successor outside the table
        tab = DispatchTable([Entry(G.BOX_SUBDIVIDE, [scalar(0), scalar(-1)], [(7, 0)])]).to_array()
        want = 4
    else:  # an IfSizeLess cycle never reaches a branching rule
        tab = DispatchTable([Entry(G.BOX_IF_SIZE_LESS, [scalar(0), scalar(5.0)], [(0, 0), (0, 0)])]).to_array()
        want = 9
    eng = _engine(tab)
    for plain in (False, True):
        out, n, rep = eng.execute(G.make_axioms(4), capacity=64, plain=plain, check=False)
        assert rep["status"] == want
    eng.release()


def test_bounded_barrier_timeout_is_a_status():
    """With a spin limit of 1 the grid barrier gives up at once: the launch
    ends with PGA_ERR_TIMEOUT (or completes when every block arrived before the
    others polled), never a hang."""
    b = scenes.menger(0.05)
    eng = _engine(b["entries"], spin_limit=1)
    out, n, rep = eng.execute(b["axioms"], capacity=8000, check=False)
    assert rep["status"] in (0, 3)
    eng.release()
    eng = _engine(b["entries"])
    out, n, rep = eng.execute(b["axioms"], capacity=8000)
    assert n == 8000
    eng.release()


def test_derive_is_graph_capturable():
    """pga_derive (a state reset plus one cooperative launch on the caller's
    stream) captured in a CUDA graph and replayed gives the same terminals."""
    import torch

    b = scenes.city(64)
    eng = _engine(b["entries"])
    d_ax = torch.from_numpy(b["axioms"].view(np.uint8).copy()).cuda()
    cap = 200_000
    out = torch.zeros((cap, 64), dtype=torch.uint8, device="cuda")
    count = torch.zeros(1, dtype=torch.int64, device="cuda")
    want, n, _ = eng.execute(b["axioms"], capacity=cap)
    want = want[:n].cpu().numpy().copy()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):  # warm-up outside the capture
        eng.derive_raw(d_ax.data_ptr(), len(b["axioms"]), None, out.data_ptr(), cap, count.data_ptr(), stream=s)
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        eng.derive_raw(d_ax.data_ptr(), len(b["axioms"]), None, out.data_ptr(), cap, count.data_ptr(),
                       stream=torch.cuda.current_stream())
    for _ in range(3):
        out.zero_()
        count.zero_()
        g.replay()
        torch.cuda.synchronize()
        assert int(count.item()) == n
        got = out[:n].cpu().numpy()
        ka = np.sort(got.view(np.dtype((np.void, 64))).ravel())
        kb = np.sort(want.view(np.dtype((np.void, 64))).ravel())
        assert (ka == kb).all()
    assert eng.report()["status"] == 0
    eng.release()


def test_grouped_axioms_give_the_same_records():
    """PGA_FLAG_GROUP_AXIOMS on a batch mixing Menger, buildings and random
    grammars (4,096 axioms, interleaved): the same records, bit for bit, as
    the index-order launch, and the order really changes."""
    b = scenes.mixed(4096)
    ref, got = None, None
    for group in (False, True):
        eng = _engine(b["entries"], node_capacity=1 << 23, max_terminals=12_000_000, group_axioms=group)
        out, n, rep = eng.execute(b["axioms"], capacity=12_000_000)
        assert rep["status"] == 0
        rec = out[:n].cpu().numpy().copy()
        if group:
            got = rec
        else:
            ref = rec
        eng.release()
    assert len(got) == len(ref)
    assert not np.array_equal(got, ref), "grouping left the output order unchanged"
    ka = np.sort(got.view(np.dtype((np.void, 64))).ravel())
    kb = np.sort(ref.view(np.dtype((np.void, 64))).ravel())
    assert (ka == kb).all()


def test_mixed_65536_full_size_bit_exact():
    """The C5 mix at full size (65,536 axioms: Menger depths 1-3, city buildings,
    random grammars; about 152M terminals) in one launch, against the oracle run
    in 16 axiom shards of 4,096, each hashing its root paths from its first
    axiom's index in the whole batch.  Every oracle record is looked up by its
    derivation-path hash among the launch's records (sorted by path on the
    device) and compared field by field: transform bits (up to the sign of
    zero), rule, custom attribute.  Counts add up and paths are unique, so the
    two multisets are equal record for record."""
    import torch

    b = scenes.mixed(65536)
    cap = 160_000_000
    eng = _engine(b["entries"], node_capacity=1 << 27, max_terminals=cap)
    out, n, rep = eng.execute(b["axioms"], capacity=cap)
    assert rep["status"] == 0
    rows = out[:n].view(torch.int64).view(n, 8)
    paths, perm = torch.sort(rows[:, 7])
    assert bool((paths[1:] != paths[:-1]).all()), "path hashes not unique"
    total = 0
    for lo in range(0, 65536, 4096):
        t = oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"][lo:lo + 4096], axiom_base=lo)
        total += len(t)
        ref = torch.from_numpy(t.view(np.uint8).reshape(-1, 64)).cuda()
        del t
        rp = ref.view(torch.int64).view(-1, 8)[:, 7]
        pos = torch.searchsorted(paths, rp).clamp_(max=n - 1)
        assert bool((paths[pos] == rp).all()), f"shard {lo}: path hashes missing from the launch"
        got = out[perm[pos]]
        gm, rm = got.view(torch.float32).view(-1, 16)[:, :12], ref.view(torch.float32).view(-1, 16)[:, :12]
        assert bool((gm == rm).all()), f"shard {lo}: transforms differ"
        gi, ri = got.view(torch.int32).view(-1, 16)[:, 12:14], ref.view(torch.int32).view(-1, 16)[:, 12:14]
        assert bool((gi == ri).all()), f"shard {lo}: rule or custom attribute differs"
        del ref, rp, pos, got, gm, rm, gi, ri
    assert total == n
    eng.release()


@pytest.mark.parametrize("scene", ["city_4096", "mixed_4096"])
def test_lbvh_full_size_bit_exact(scene):
    """The LBVH over every terminal of the full city (5.86M leaves; 30-bit
    Morton cells of 3.2 m hold many terminals, so 85% of neighbouring sorted
    keys share their Morton code and are ordered by sub-cell code and path)
    and of a 4,096-axiom mix (9.4M leaves, 93% shared) against the
    restatement: keys, leaf order, topology, leaf parents and boxes bit for
    bit."""
    if scene == "city_4096":
        b, bounds = scenes.city(4096), (-50.0, -50.0, -1.0, 3250.0, 3250.0, 400.0)
    else:
        b = scenes.mixed(4096)
        bounds = None
    eng, out, got, rep = _run(b, node_capacity=1 << 24, max_terminals=1 << 24)
    assert rep["status"] == 0
    n = len(got)
    if bounds is None:
        c = np.stack([got["m"][:, 3], got["m"][:, 7], got["m"][:, 11]], 1)
        bounds = tuple(float(v) for v in c.min(0) - 1.0) + tuple(float(v) for v in c.max(0) + 1.0)
    nodes, lp, aabb, lt, keys = oracle.lbvh(got, bounds)
    runs = int((keys[1:] >> 34 == keys[:-1] >> 34).sum())
    assert runs > n // 4, "the scene should share Morton codes"
    bv = eng.lbvh(out, n, bounds)
    torch.cuda.synchronize()
    assert np.array_equal(bv["keys"].cpu().numpy().view(np.uint64), keys), "Morton keys differ"
    assert np.array_equal(bv["leafTerminal"].cpu().numpy().view(np.uint32), lt), "leaf order differs"
    assert np.array_equal(bv["nodes"].cpu().numpy(), nodes), "topology differs"
    assert np.array_equal(bv["leafParents"].cpu().numpy().view(np.uint32), lp)
    assert np.array_equal(bv["aabbs"].cpu().numpy().view(np.uint32), aabb.view(np.uint32)), "boxes differ"
    eng.release()


@pytest.mark.parametrize("counted", [False, True])
def test_lbvh_tie_runs_bit_exact(counted):
    """Terminals that share a Morton cell and their path hash's top 10 bits
    share the sorted part of the key, so their order comes from the tie ranks:
    200,000 synthetic records, half of them at 250 shared centres; groups of 2
    to 48 records (and one of 3,000) at one centre whose path hashes share
    their top 10 bits (runs inside and across the 64-key windows of the
    ranking warps, and one far longer); a tenth with a path hash and centre
    copied from another record (equal keys, then equal paths: ordered by
    terminal index); a third of them quads.  Keys, leaf order, topology,
    parents and boxes against the restatement bit for bit, built over the host
    count and over a device count with padding."""
    from operatorgraph_gb300.engine import Engine

    n, cap = 200_000, 200_000 + (4096 if counted else 0)
    rng = np.random.default_rng(5)
    rec = np.zeros(n, G.TERMINAL_DT)
    m = rng.uniform(-0.5, 0.5, (n, 12)).astype(np.float32)
    centres = rng.uniform(-9.0, 9.0, (250, 3)).astype(np.float32)
    m[:, [3, 7, 11]] = rng.uniform(-9.0, 9.0, (n, 3)).astype(np.float32)
    shared = rng.choice(n, n // 2, replace=False)
    m[np.ix_(shared, [3, 7, 11])] = centres[rng.integers(0, 250, len(shared))]
    paths = rng.integers(0, 2**64, size=n, dtype=np.uint64)
    grouped = rng.permutation(n)
    at = 0
    for size in [3000] + [int(x) for x in rng.integers(2, 49, 400)]:
        g = grouped[at:at + size]
        at += size
        m[np.ix_(g, [3, 7, 11])] = rng.uniform(-9.0, 9.0, 3).astype(np.float32)
        top = np.uint64(int(rng.integers(0, 1024)) << 54)
        paths[g] = top | (paths[g] & np.uint64((1 << 54) - 1))
    dst, src = rng.choice(n, n // 10, replace=False), rng.choice(n, n // 10, replace=False)
    paths[dst] = paths[src]
    m[np.ix_(dst, [3, 7, 11])] = m[np.ix_(src, [3, 7, 11])]  # same centre and path: equal keys
    rec["m"] = m
    rec["rule"] = np.where(rng.random(n) < 1 / 3, np.uint32(1 << 31), np.uint32(0)) | rng.integers(0, 64, n).astype(np.uint32)
    rec["path"] = paths
    bounds = (-10.0, -10.0, -10.0, 10.0, 10.0, 10.0)
    nodes, lp, aabb, lt, keys = oracle.lbvh(rec, bounds)
    _, runs = np.unique(keys >> np.uint64(24), return_counts=True)
    assert runs.max() >= 2500 and int(runs[runs > 1].sum()) > 20_000, "the records should make tie runs"
    assert int((keys[1:] == keys[:-1]).sum()) > 100, "some keys should be equal"
    out = torch.zeros((cap, 64), dtype=torch.uint8, device="cuda")
    out[:n] = torch.from_numpy(rec.view(np.uint8).reshape(n, 64).copy()).cuda()
    eng = Engine(scenes.building()["entries"], node_capacity=1 << 16, max_terminals=cap)
    if counted:
        bv = eng.lbvh(out, cap, bounds, count=torch.tensor([n], dtype=torch.int64, device="cuda"))
    else:
        bv = eng.lbvh(out, n, bounds)
    torch.cuda.synchronize()
    k = bv["keys"].cpu().numpy().view(np.uint64)
    assert np.array_equal(k[:n], keys), "Morton keys differ"
    assert np.array_equal(bv["leafTerminal"][:n].cpu().numpy().view(np.uint32), lt), "leaf order differs"
    assert np.array_equal(bv["nodes"][: n - 1].cpu().numpy(), nodes), "topology differs"
    assert np.array_equal(bv["leafParents"][:n].cpu().numpy().view(np.uint32), lp)
    assert np.array_equal(bv["aabbs"][: n - 1].cpu().numpy().view(np.uint32), aabb.view(np.uint32)), "boxes differ"
    eng.release()


@pytest.mark.parametrize("scene", ["city_4096", "menger_d3"])
def test_derive_to_host_matches_device_derive(scene):
    """pga_derive_to_host (host axioms in, host terminals out, derived in axiom
    ranges whose copies overlap the next range's derivation) gives the same
    terminal records as one pga_derive, path hashes included."""
    b = scenes.city(4096) if scene == "city_4096" else scenes.menger(0.05)
    ref = oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"])
    cap = len(ref) + 4096
    eng = _engine(b["entries"], node_capacity=1 << 23, max_terminals=1 << 23)
    h_ax = torch.from_numpy(b["axioms"].view(np.uint8).copy()).pin_memory()
    h_out = torch.empty((cap, 64), dtype=torch.uint8).pin_memory()
    for _ in range(2):  # staging is allocated on the first call and reused on the second
        h_out.zero_()
        n, st = eng.derive_to_host(h_ax.data_ptr(), len(b["axioms"]), h_out.data_ptr(), cap)
        assert st == 0 and n == len(ref)
        _assert_same(h_out[:n].numpy().reshape(-1).view(G.TERMINAL_DT), ref)
    out, n2, _ = eng.execute(b["axioms"], capacity=cap)
    assert n2 == n
    eng.release()


def test_per_axiom_form_matches_batched_in_a_graph():
    """pga_derive_per_axiom on 256 city buildings: eagerly and captured in a
    CUDA graph (256 launches and appends, no host read-back), the same records
    as pga_derive in axiom order; then an output overflow is a status."""
    b = scenes.city(256)
    ref = oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"])
    cap = len(ref)
    eng = _engine(b["entries"])
    d_ax = torch.from_numpy(b["axioms"].view(np.uint8).copy()).cuda()
    out = torch.zeros((cap, 64), dtype=torch.uint8, device="cuda")
    count = torch.zeros(1, dtype=torch.int64, device="cuda")
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        eng.derive_raw(d_ax.data_ptr(), len(b["axioms"]), None, out.data_ptr(), cap, count.data_ptr(), stream=s,
                       plain="per_axiom")
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    assert eng.report()["status"] == 0 and int(count.item()) == cap
    from operatorgraph_gb300.engine import terminals_to_numpy

    got = terminals_to_numpy(out, cap)
    _assert_same(got, ref)
    # axiom order: each axiom's records follow the previous axiom's
    want_first = oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"][:1])
    _assert_same(got[:len(want_first)], want_first)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        eng.derive_raw(d_ax.data_ptr(), len(b["axioms"]), None, out.data_ptr(), cap, count.data_ptr(),
                       stream=torch.cuda.current_stream(), plain="per_axiom")
    out.zero_()
    count.zero_()
    g.replay()
    torch.cuda.synchronize()
    assert eng.report()["status"] == 0 and int(count.item()) == cap
    _assert_same(terminals_to_numpy(out, cap), ref)
    del g
    out2, n, rep = eng.execute(b["axioms"], capacity=cap // 2, plain="per_axiom", check=False)
    assert rep["status"] == 2 and n == cap
    eng.release()


def test_derive_to_host_reports_overflow():
    from operatorgraph_gb300.engine import PgaError

    b = scenes.city(256)
    eng = _engine(b["entries"])
    h_ax = torch.from_numpy(b["axioms"].view(np.uint8).copy()).pin_memory()
    h_out = torch.empty((1000, 64), dtype=torch.uint8).pin_memory()
    n, st = eng.derive_to_host(h_ax.data_ptr(), len(b["axioms"]), h_out.data_ptr(), 1000, check=False)
    assert st == 2 and n > 1000
    with pytest.raises(PgaError):
        eng.derive_to_host(h_ax.data_ptr(), len(b["axioms"]), h_out.data_ptr(), 1000)
    eng.release()


def test_city_meshes_match_the_oracle():
    """pga_generate_meshes on 64 city buildings with triangle-mesh terminals
    (walls, windows, roofs: about 90k quads in three meshes) against the
    oracle's meshes, face for face, bit for bit; then with too little space
    (PGA_ERR_OUTPUT_OVERFLOW) and too few meshes (PGA_ERR_BAD_PARAM)."""
    from operatorgraph_gb300.engine import PgaError

    b = scenes.city(64, meshes=True)
    _, meshes_ref = oracle.derive_meshes(G.DEFAULT_PROCS, b["entries"], b["axioms"])
    eng, out, got, rep = _run(b)
    assert rep["status"] == 0
    caps = [(len(v), len(i)) for v, i in meshes_ref]
    meshes = eng.generate_meshes(out, len(got), caps)
    for (v, i, nv, ni), (rv, ri) in zip(meshes, meshes_ref):
        assert (nv, ni) == (len(rv), len(ri))
        a = G.mesh_faces(v.cpu().numpy(), i.cpu().numpy().view(np.uint32))
        c = G.mesh_faces(rv, ri)
        assert np.array_equal(a.view(np.uint32), c.view(np.uint32))
    with pytest.raises(PgaError) as e:
        eng.generate_meshes(out, len(got), [(nv // 2, ni // 2) for nv, ni in caps])
    assert e.value.status == 2
    eng.release()
    eng, out, got, rep = _run(b)
    with pytest.raises(PgaError) as e:
        eng.generate_meshes(out, len(got), caps[:2])
    assert e.value.status == 5
    eng.release()


def test_forest_general_frames_bit_exact():
    """256 trees of the forest scene (Rotate with arbitrary angles, Replicate,
    Translate, Scale, IfSizeLess: the general-frame kernels, 840k terminals)
    in the persistent, queued and plain forms against the oracle, bit for bit
    including path hashes."""
    from operatorgraph_gb300.engine import terminals_to_numpy

    b = scenes.forest(256)
    ref = oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"])
    assert len(ref) == 256 * 3281
    for form in ("persistent", "queued", "plain"):
        eng = _engine(b["entries"], no_inline=form == "queued")
        out, n, rep = eng.execute(b["axioms"], capacity=len(ref), plain=form == "plain")
        assert rep["status"] == 0, (form, rep)
        _assert_same(terminals_to_numpy(out, n), ref)
        eng.release()


@pytest.mark.parametrize("affine,rotate,more", [(False, False, False), (True, False, False), (True, True, False),
                                               (True, False, True)],
                         ids=["split_ops", "with_affine_ops", "with_rotate_ops", "with_if_swap_ops"])
def test_rich_random_grammars_fuzz(affine, rotate, more):
    """120 more seeds of the rich random grammar generator (all operators, both
    shapes, every parameter kind; with_affine_ops adds Translate, Scale and
    RandomRule, with_rotate_ops also Rotate and Replicate, which run the
    general-frame kernels, with_if_swap_ops If and SwapSize), each derived by
    the batched engine with leaf
    children in place, with every child queued, and in the plain form, and
    compared bit for bit with the oracle.  Seeds the oracle rejects (grammars
    the reference would throw on) are skipped; statuses must then agree."""
    import sys

    sys.path.insert(0, os.path.join(HERE, "golden"))
    import cases

    from operatorgraph_gb300.engine import terminals_to_numpy

    checked = 0
    for seed in range(1000, 1120):
        b = cases.rich_random(seed, affine=affine, rotate=rotate, more=more)
        try:
            ref = oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"])
        except oracle.OracleError as err:
            eng = _engine(b["entries"])
            _, _, rep = eng.execute(b["axioms"], capacity=1 << 16, check=False)
            assert rep["status"] == err.status, (seed, rep["status"], err.status)
            eng.release()
            continue
        if len(ref) > 200_000:
            continue
        for form in ("persistent", "queued", "plain"):
            eng = _engine(b["entries"], no_inline=form == "queued")
            out, n, rep = eng.execute(b["axioms"], capacity=max(len(ref), 1), plain=form == "plain")
            assert rep["status"] == 0, (seed, form, rep)
            if len(ref) == 0:
                assert n == 0, (seed, form, n)
            else:
                _assert_same(terminals_to_numpy(out, n), ref)
            eng.release()
        checked += 1
    assert checked >= 100
