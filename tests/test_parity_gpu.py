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


@pytest.mark.parametrize("form", ["persistent", "queued", "plain", "grouped"])
@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_golden_case(path, form):
    """persistent: the batched launch (leaf children expanded in place);
    queued: the same with every branching child queued (PGA_FLAG_NO_INLINE);
    plain: one axiom and one launch per level;
    grouped: the batched launch with the axioms seeded grouped by root entry
    (PGA_FLAG_GROUP_AXIOMS)."""
    import sys

    sys.path.insert(0, os.path.join(HERE, "golden"))
    import cases

    b, z = _load(path)
    eng, out, got, rep = _run(b, plain=form == "plain", no_inline=form == "queued", group_axioms=form == "grouped")
    assert rep["status"] == 0
    n_base = len(b["entries"]) if b["blocks"] is not None else None
    canon = cases.canonical(got, n_base)
    assert len(got) == int(z["count"])
    assert cases.digest(canon) == str(z["digest"]), "differs from the reference's own output"
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


@pytest.mark.parametrize("name", ["menger_d5", "city_4096", "facades_1024", "random_16", "city_4096_queued"])
def test_full_size_bit_exact(name):
    kw = {"no_inline": True} if name.endswith("_queued") else {}
    name = name.replace("_queued", "")
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


def test_mixed_65536_full_size_properties():
    """The C5 mix at full size (65,536 axioms: Menger depths 1-3, city buildings,
    random grammars; about 152M terminals) in one launch, against the oracle run
    in axiom shards: the exact count, the exact histogram of emitting rules
    (entry, mesh index, shape), float64 sums of every transform component, and
    unique path hashes.  Bit-exact per-record parity is covered on the smaller
    cases; here the shard runs renumber the axioms, so path hashes differ."""
    import torch

    b = scenes.mixed(65536)
    want_n, want_sum, want_rules = 0, np.zeros(12), {}
    for lo in range(0, 65536, 4096):
        t = oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"][lo:lo + 4096])
        want_n += len(t)
        want_sum += t["m"].astype(np.float64).sum(axis=0)
        r, c = np.unique(t["rule"], return_counts=True)
        for k, v in zip(r.tolist(), c.tolist()):
            want_rules[k] = want_rules.get(k, 0) + v
        del t
    cap = want_n + (1 << 20)
    eng = _engine(b["entries"], node_capacity=1 << 27, max_terminals=cap)
    out, n, rep = eng.execute(b["axioms"], capacity=cap)
    assert rep["status"] == 0 and n == want_n
    got_sum = torch.zeros(12, dtype=torch.float64, device="cuda")
    rules, paths = [], []
    for lo in range(0, n, 1 << 23):
        chunk = out[lo:min(n, lo + (1 << 23))]
        f = chunk.view(torch.float32).view(-1, 16)
        got_sum += f[:, :12].double().sum(dim=0)
        rules.append(chunk.view(torch.int32).view(-1, 16)[:, 12])
        paths.append(chunk.view(torch.int64).view(-1, 8)[:, 7])
    r, c = torch.unique(torch.cat(rules), return_counts=True)
    got_rules = {int(k) & 0xFFFFFFFF: int(v) for k, v in zip(r.cpu().tolist(), c.cpu().tolist())}
    assert got_rules == want_rules
    np.testing.assert_allclose(got_sum.cpu().numpy(), want_sum, rtol=1e-9, atol=1e-3)
    assert torch.unique(torch.cat(paths)).numel() == n
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
