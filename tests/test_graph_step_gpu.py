"""The LBVH over a device-side leaf count, and the whole differentiable step
(derivation, LBVH over its terminals, loss gradient, adjoint) in one CUDA graph.

pga_lbvh_build_counted reads the leaf count the derivation wrote on the device,
so nothing is read back to the host between the steps and the four of them
replay as one graph.  Bar: the counted build gives the oracle's Morton keys,
leaf order, topology and boxes bit for bit, with all-ones padding keys past the
count; graph replays give the eager run's terminal multiset and LBVH bit for
bit (leaf order compared through the records it points at, since the output
order of a derivation is free) and its gradients to FP32 accumulation order.
"""
import ctypes

import numpy as np
import pytest

import oracle
from operatorgraph_gb300 import grammar as G
from operatorgraph_gb300 import scenes

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from operatorgraph_gb300 import build as B

    B.build()
    torch.cuda.set_device(0)


def _engine(b, **kw):
    from operatorgraph_gb300.engine import Engine

    kw.setdefault("node_capacity", 1 << 22)
    kw.setdefault("max_terminals", 1 << 22)
    return Engine(b["entries"], block_stride=b["block_stride"], **kw)


def _bounds_of(m):
    c = m[:, [3, 7, 11]].astype(np.float64)
    lo, hi = c.min(axis=0) - 1.0, c.max(axis=0) + 1.0
    return tuple(float(v) for v in lo) + tuple(float(v) for v in hi)


@pytest.mark.parametrize("scene", ["menger_d3", "city_16"])
def test_lbvh_counted_matches_the_oracle(scene):
    from operatorgraph_gb300.engine import terminals_to_numpy

    b = scenes.menger(0.05) if scene == "menger_d3" else scenes.city(16)
    eng = _engine(b)
    n_ref = len(oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"], b["blocks"], b["block_stride"]))
    cap = n_ref + 1000
    out, n, rep = eng.execute(b["axioms"], blocks=b["blocks"], capacity=cap)
    assert n == n_ref and rep["status"] == 0
    got = terminals_to_numpy(out, n)
    bounds = _bounds_of(got["m"])
    count = torch.tensor([n], dtype=torch.int64, device="cuda")
    bv = eng.lbvh(out, cap, bounds, count=count)
    torch.cuda.synchronize()
    nodes, lp, aabb, lt, keys = oracle.lbvh(got, bounds)
    k = bv["keys"].cpu().numpy().view(np.uint64)
    assert np.array_equal(k[:n], keys), "Morton keys differ"
    assert (k[n:] == np.uint64(0xFFFFFFFFFFFFFFFF)).all(), "padding keys are not all ones"
    assert np.array_equal(bv["leafTerminal"][:n].cpu().numpy().view(np.uint32), lt), "leaf order differs"
    assert np.array_equal(bv["nodes"][: n - 1].cpu().numpy(), nodes), "topology differs"
    assert np.array_equal(bv["leafParents"][:n].cpu().numpy().view(np.uint32), lp)
    assert np.array_equal(bv["aabbs"][: n - 1].cpu().numpy().view(np.uint32), aabb.view(np.uint32)), "boxes differ"
    eng.release()


@pytest.mark.parametrize("leaves", [0, 1])
def test_lbvh_counted_below_two_leaves_builds_no_tree(leaves):
    """A count below 2 leaves the tree arrays as they were."""
    from operatorgraph_gb300.engine import PgaBounds, PgaLbvh, load_library

    b = scenes.building()
    eng = _engine(b)
    out, n, _ = eng.execute(b["axioms"], capacity=4096)
    cap = 64
    sentinel = -7
    arrays = {
        "nodes": torch.full((cap - 1, 3), sentinel, dtype=torch.int32, device="cuda"),
        "leafParents": torch.full((cap,), sentinel, dtype=torch.int32, device="cuda"),
        "aabbs": torch.full((cap - 1, 6), float(sentinel), dtype=torch.float32, device="cuda"),
        "leafTerminal": torch.full((cap,), sentinel, dtype=torch.int32, device="cuda"),
        "keys": torch.zeros(cap, dtype=torch.int64, device="cuda"),
    }
    lb = PgaLbvh(*(arrays[k].data_ptr() for k in ("nodes", "leafParents", "aabbs", "leafTerminal", "keys")))
    pb = PgaBounds((ctypes.c_float * 3)(-50, -50, -50), (ctypes.c_float * 3)(50, 50, 50))
    count = torch.tensor([leaves], dtype=torch.int64, device="cuda")
    st = load_library().pga_lbvh_build_counted(eng.handle, out.data_ptr(), count.data_ptr(), cap, ctypes.byref(pb),
                                               ctypes.byref(lb), None)
    assert st == 0
    torch.cuda.synchronize()
    for k in ("nodes", "leafParents", "leafTerminal"):
        assert (arrays[k] == sentinel).all(), f"{k} written for {leaves} leaves"
    assert (arrays["aabbs"] == float(sentinel)).all()
    assert (arrays["keys"][leaves:].cpu().numpy().view(np.uint64) == np.uint64(0xFFFFFFFFFFFFFFFF)).all()
    eng.release()


def test_counted_capacity_is_checked():
    from operatorgraph_gb300.engine import PgaBounds, PgaLbvh, load_library

    b = scenes.building()
    eng = _engine(b, max_terminals=1 << 12, node_capacity=1 << 14)
    t = torch.zeros((1 << 13, 64), dtype=torch.uint8, device="cuda")
    count = torch.zeros(1, dtype=torch.int64, device="cuda")
    lb = PgaLbvh(t.data_ptr(), t.data_ptr(), t.data_ptr(), t.data_ptr(), t.data_ptr())
    pb = PgaBounds((ctypes.c_float * 3)(0, 0, 0), (ctypes.c_float * 3)(1, 1, 1))
    L = load_library()
    for cap in (1, (1 << 12) + 1):
        assert L.pga_lbvh_build_counted(eng.handle, t.data_ptr(), count.data_ptr(), cap, ctypes.byref(pb),
                                        ctypes.byref(lb), None) != 0
    assert L.pga_lbvh_build_counted(eng.handle, t.data_ptr(), None, 16, ctypes.byref(pb), ctypes.byref(lb), None) != 0
    eng.release()


class _Step:
    """Buffers and calls of one differentiable step on a tape-recording engine:
    derive, LBVH over the derived count, dL/dM = M for L = |M|^2 / 2 (a torch
    kernel on the step's own output rows), adjoint to blocks and sizes."""

    def __init__(self, b, cap, bounds):
        self.b, self.cap, self.bounds = b, cap, bounds
        self.eng = _engine(b, record_tape=True, node_capacity=1 << 20, max_terminals=cap)
        self.n_ax = len(b["axioms"])
        self.d_ax = torch.from_numpy(b["axioms"].view(np.uint8).copy()).cuda()
        self.d_blk = torch.from_numpy(b["blocks"]).cuda()
        self.out = torch.zeros((cap, 64), dtype=torch.uint8, device="cuda")
        self.count = torch.zeros(1, dtype=torch.int64, device="cuda")
        self.g_term = torch.zeros((cap, 12), dtype=torch.float32, device="cuda")
        self.g_blk = torch.zeros_like(self.d_blk)
        self.g_sz = torch.zeros((self.n_ax, 3), dtype=torch.float32, device="cuda")
        self.bv = None

    def run(self, stream):
        e = self.eng
        e.derive_raw(self.d_ax.data_ptr(), self.n_ax, self.d_blk.data_ptr(), self.out.data_ptr(), self.cap,
                     self.count.data_ptr(), stream=stream)
        self.bv = e.lbvh(self.out, self.cap, self.bounds, stream=stream, count=self.count)
        self.g_term.copy_(self.out.view(torch.float32).view(self.cap, 16)[:, :12])
        e.adjoint_raw(self.g_term.data_ptr(), self.g_blk.data_ptr(), len(self.b["blocks"]) // max(
            self.b["block_stride"], 1), self.g_sz.data_ptr(), stream=stream)

    def snapshot(self):
        n = int(self.count.item())
        rec = self.out[:n].cpu().numpy().copy()
        lt = self.bv["leafTerminal"][:n].cpu().numpy().astype(np.int64)
        return {
            "n": n,
            "records": np.sort(rec.view(np.dtype((np.void, 64))).ravel()),
            "keys": self.bv["keys"][:n].cpu().numpy().copy(),
            "nodes": self.bv["nodes"][: n - 1].cpu().numpy().copy(),
            "leafParents": self.bv["leafParents"][:n].cpu().numpy().copy(),
            "aabbs": self.bv["aabbs"][: n - 1].cpu().numpy().copy(),
            "sortedRecords": rec[lt],
            "gBlocks": self.g_blk.cpu().numpy().astype(np.float64),
            "gSizes": self.g_sz.cpu().numpy().astype(np.float64),
        }


def _close(a, b, what):
    scale = max(float(np.abs(b).max()), 1e-30)
    assert float(np.abs(a - b).max()) <= 1e-5 * scale, f"{what} differ beyond FP32 accumulation order"


def test_derive_lbvh_adjoint_in_one_graph():
    b = scenes.facades(64)
    n_ref = len(oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"], b["blocks"], b["block_stride"]))
    cap = n_ref + 4096
    probe = _engine(b)
    out, n, _ = probe.execute(b["axioms"], blocks=b["blocks"], capacity=cap)
    from operatorgraph_gb300.engine import terminals_to_numpy

    bounds = _bounds_of(terminals_to_numpy(out, n)["m"])
    probe.release()
    step = _Step(b, cap, bounds)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):  # eager run, also the warm-up before the capture
        step.run(s)
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    assert step.eng.report()["status"] == 0
    want = step.snapshot()
    assert want["n"] == n_ref
    assert np.abs(want["gBlocks"]).max() > 0 and np.abs(want["gSizes"]).max() > 0
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        step.run(torch.cuda.current_stream())
    for _ in range(3):
        step.out.zero_()
        step.count.zero_()
        step.g_blk.fill_(1.0)
        step.g_sz.fill_(1.0)
        g.replay()
        torch.cuda.synchronize()
        got = step.snapshot()
        assert got["n"] == want["n"]
        assert (got["records"] == want["records"]).all(), "terminal multiset differs"
        for k in ("keys", "nodes", "leafParents"):
            assert np.array_equal(got[k], want[k]), f"LBVH {k} differs"
        assert np.array_equal(got["aabbs"].view(np.uint32), want["aabbs"].view(np.uint32)), "LBVH boxes differ"
        assert np.array_equal(got["sortedRecords"], want["sortedRecords"]), "leaf order differs"
        _close(got["gBlocks"], want["gBlocks"], "block gradients")
        _close(got["gSizes"], want["gSizes"], "size gradients")
    assert step.eng.report()["status"] == 0
    step.eng.release()


def test_adjoint_with_grouped_axioms_matches_index_order():
    """The adjoint after a PGA_FLAG_GROUP_AXIOMS derivation (a mixed batch of
    Menger, buildings and random grammars): the same axiom-size gradients as
    after the index-order derivation, to FP32 accumulation order.  The loss is
    L = |M|^2 / 2, so dL/dM = M for whatever order the records come in."""
    from operatorgraph_gb300.engine import Engine

    b = scenes.mixed(512)
    grads = []
    for group in (False, True):
        eng = Engine(b["entries"], node_capacity=1 << 21, max_terminals=2_000_000, record_tape=True,
                     group_axioms=group)
        d_ax = torch.from_numpy(b["axioms"].view(np.uint8).copy()).cuda()
        out = torch.zeros((2_000_000, 64), dtype=torch.uint8, device="cuda")
        count = torch.zeros(1, dtype=torch.int64, device="cuda")
        eng.derive_raw(d_ax.data_ptr(), len(b["axioms"]), None, out.data_ptr(), out.shape[0], count.data_ptr())
        g_term = out.view(torch.float32).view(-1, 16)[:, :12].contiguous()
        g_sz = torch.zeros((len(b["axioms"]), 3), dtype=torch.float32, device="cuda")
        eng.adjoint_raw(g_term.data_ptr(), None, 0, g_sz.data_ptr())
        torch.cuda.synchronize()
        assert eng.report()["status"] == 0
        grads.append(g_sz.cpu().numpy().astype(np.float64))
        eng.release()
    assert np.abs(grads[0]).max() > 0
    _close(grads[1], grads[0], "axiom-size gradients")


def test_dynamic_chunks_give_the_same_records_and_gradients():
    """PGA_FLAG_DYNAMIC_CHUNKS on a batch whose widest levels take the dynamic
    path (a 4,096-axiom mix: levels of up to ~2M work items, above the four
    rounds of 77,824-item chunks the flag needs): the same terminal records as
    the static order (as a multiset, bit for bit) and, after the tape-recording
    derivation, the same axiom-size gradients to FP32 accumulation order."""
    from operatorgraph_gb300.engine import Engine

    b = scenes.mixed(4096)
    cap = 10_000_000
    d_ax = torch.from_numpy(b["axioms"].view(np.uint8).copy()).cuda()
    out = torch.zeros((cap, 64), dtype=torch.uint8, device="cuda")
    count = torch.zeros(1, dtype=torch.int64, device="cuda")
    records, grads = [], []
    for dynamic in (False, True):
        eng = Engine(b["entries"], node_capacity=1 << 23, max_terminals=cap, dynamic_chunks=dynamic)
        eng.derive_raw(d_ax.data_ptr(), len(b["axioms"]), None, out.data_ptr(), cap, count.data_ptr())
        torch.cuda.synchronize()
        rep = eng.report()
        assert rep["status"] == 0 and rep["max_level_nodes"] >= 4 * 77_824
        n = int(count.item())
        records.append(np.sort(out[:n].cpu().numpy().view(np.dtype((np.void, 64))).ravel()))
        eng.release()
        eng = Engine(b["entries"], node_capacity=1 << 23, max_terminals=cap, record_tape=True, dynamic_chunks=dynamic)
        eng.derive_raw(d_ax.data_ptr(), len(b["axioms"]), None, out.data_ptr(), cap, count.data_ptr())
        g_sz = torch.zeros((len(b["axioms"]), 3), dtype=torch.float32, device="cuda")
        eng.adjoint_raw(out.data_ptr(), None, 0, g_sz.data_ptr(), grad_stride=16)
        torch.cuda.synchronize()
        assert eng.report()["status"] == 0
        grads.append(g_sz.cpu().numpy().astype(np.float64))
        eng.release()
    assert len(records[0]) == len(records[1]) and (records[0] == records[1]).all()
    assert np.abs(grads[0]).max() > 0
    _close(grads[1], grads[0], "axiom-size gradients")


@pytest.mark.parametrize("blocks", [False, True])
def test_wide_adjoint_matches_the_standard_one(blocks):
    """Engines of at least 8M terminals of capacity launch the adjoint with 3
    (block build: 4) blocks per SM, smaller ones the standard kernel: on a
    2,048-axiom mix (~4.7M terminals) an engine of 9M capacity and one of 6M
    derive the same terminals and must give the same block and size gradients
    to FP32 accumulation order."""
    from operatorgraph_gb300.engine import Engine

    b = scenes.mixed(2048, blocks=blocks)
    d_ax = torch.from_numpy(b["axioms"].view(np.uint8).copy()).cuda()
    d_blk = torch.from_numpy(b["blocks"]).cuda() if blocks else None
    grads, counts = [], []
    for cap in (9_000_000, 6_000_000):
        eng = Engine(b["entries"], node_capacity=1 << 23, max_terminals=cap, record_tape=True,
                     block_stride=b["block_stride"])
        out = torch.zeros((cap, 64), dtype=torch.uint8, device="cuda")
        count = torch.zeros(1, dtype=torch.int64, device="cuda")
        eng.derive_raw(d_ax.data_ptr(), len(b["axioms"]), None if d_blk is None else d_blk.data_ptr(), out.data_ptr(),
                       cap, count.data_ptr())
        g_sz = torch.zeros((len(b["axioms"]), 3), dtype=torch.float32, device="cuda")
        g_blk = torch.zeros_like(d_blk) if blocks else None
        eng.adjoint_raw(out.data_ptr(), None if g_blk is None else g_blk.data_ptr(),
                        len(b["axioms"]) if blocks else 0, g_sz.data_ptr(), grad_stride=16)
        torch.cuda.synchronize()
        assert eng.report()["status"] == 0
        counts.append(int(count.item()))
        grads.append((g_sz.cpu().numpy().astype(np.float64),
                      None if g_blk is None else g_blk.cpu().numpy().astype(np.float64)))
        eng.release()
        del out
    assert counts[0] == counts[1] and 6_000_000 > counts[0] > 3_000_000
    assert np.abs(grads[0][0]).max() > 0
    _close(grads[0][0], grads[1][0], "axiom-size gradients")
    if blocks:
        assert np.abs(grads[0][1]).max() > 0
        _close(grads[0][1], grads[1][1], "block gradients")


def test_strided_gradient_read_in_place_matches_a_copy():
    """pga_adjoint_strided reading dL/dM = M straight from the 16-float terminal
    records gives the gradients of pga_adjoint on a 12-float copy; a stride
    below 12 is rejected."""
    from operatorgraph_gb300.engine import load_library

    b = scenes.facades(64)
    eng = _engine(b, record_tape=True, node_capacity=1 << 20, max_terminals=1 << 20)
    d_ax = torch.from_numpy(b["axioms"].view(np.uint8).copy()).cuda()
    d_blk = torch.from_numpy(b["blocks"]).cuda()
    out = torch.zeros((1 << 20, 64), dtype=torch.uint8, device="cuda")
    count = torch.zeros(1, dtype=torch.int64, device="cuda")
    eng.derive_raw(d_ax.data_ptr(), 64, d_blk.data_ptr(), out.data_ptr(), out.shape[0], count.data_ptr())
    rows = out.view(torch.float32).view(-1, 16)
    res = []
    for stride in (12, 16):
        g_term = rows[:, :12].contiguous() if stride == 12 else rows
        g_blk = torch.zeros_like(d_blk)
        g_sz = torch.zeros((64, 3), dtype=torch.float32, device="cuda")
        eng.adjoint_raw(g_term.data_ptr(), g_blk.data_ptr(), 64, g_sz.data_ptr(), grad_stride=stride)
        torch.cuda.synchronize()
        assert eng.report()["status"] == 0
        res.append((g_blk.cpu().numpy().astype(np.float64), g_sz.cpu().numpy().astype(np.float64)))
    assert np.abs(res[0][0]).max() > 0
    _close(res[1][0], res[0][0], "block gradients")
    _close(res[1][1], res[0][1], "size gradients")
    assert load_library().pga_adjoint_strided(eng.handle, rows.data_ptr(), 11, None, 0, None, None) != 0
    eng.release()
