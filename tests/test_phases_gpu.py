"""Multi-phase derivation with Collider and IfCollides on the GPU.

The scenes.collisions() grammar stores buildings (boxes, tag 1) and billboards
(quads, tag 2) in phase 0 and tests trees (boxes, turned by general rotations
or not) against them in phase 1.  The engine runs one persistent launch per
phase and builds an LBVH over the colliders between them; its terminals must
equal the oracle's (which tests every stored collider) bit for bit, path
hashes included.  The collision predicate itself is pinned against the
reference's Collision::check in tests/test_collision.py.
"""
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


def _same(got, ref):
    assert len(got) == len(ref)
    a, c = G.sort_terminals(got, by_path=True), G.sort_terminals(ref, by_path=True)
    assert np.array_equal(a["path"], c["path"])
    assert np.array_equal(a["rule"], c["rule"])
    assert np.array_equal((a["m"] + np.float32(0)).view(np.uint32), (c["m"] + np.float32(0)).view(np.uint32))


@pytest.mark.parametrize("rotate", [False, True], ids=["frame_codes", "general_frames"])
@pytest.mark.parametrize("size", [(64, 512, 96), (1024, 16384, 1024)], ids=["small", "large"])
def test_collision_scene_matches_the_oracle(rotate, size):
    from operatorgraph_gb300.engine import Engine, terminals_to_numpy

    b = scenes.collisions(*size, rotate=rotate)
    ref = oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"])
    kinds = np.bincount((ref["rule"] >> 24) & 0x7F, minlength=4)
    assert kinds[2] > 0 and kinds[3] > 0 and kinds[3] < size[1]  # some trees hit billboards, some buildings
    eng = Engine(b["entries"], node_capacity=1 << 20, max_terminals=1 << 20)
    out, n, rep = eng.execute(b["axioms"], capacity=len(ref))
    assert rep["status"] == 0 and rep["terminals"] == len(ref)
    _same(terminals_to_numpy(out, n), ref)
    # the same engine again (phases, colliders and buffers start over)
    out, n, rep = eng.execute(b["axioms"], capacity=len(ref))
    _same(terminals_to_numpy(out, n), ref)
    eng.release()


def test_multi_phase_needs_the_batched_derivation():
    from operatorgraph_gb300.engine import Engine, PgaError

    b = scenes.collisions(rotate=False)
    eng = Engine(b["entries"], node_capacity=1 << 16, max_terminals=1 << 16)
    with pytest.raises(PgaError) as e:
        eng.execute(b["axioms"], capacity=4096, plain=True)
    assert e.value.status == 7
    eng.release()


def test_inconsistent_phases_are_rejected():
    from operatorgraph_gb300.engine import Engine, PgaError
    from operatorgraph_gb300.grammar import DispatchTable, Entry, scalar

    tab = DispatchTable([
        Entry(G.BOX_REPLICATE, [], [(1, 0), (1, 1)]),  # entry 1 reached in phase 0 and in phase 1
        Entry(G.BOX_GENERATE, [scalar(0)], []),
    ]).to_array()
    with pytest.raises(PgaError) as e:
        Engine(tab)
    assert e.value.status == 5


def test_collider_and_deferral_overflow_are_statuses():
    """More colliders or deferred shapes than the engine holds (both bounded by
    nodeCapacity) end the derivation with PGA_ERR_QUEUE_OVERFLOW, not a fault."""
    from operatorgraph_gb300.engine import Engine, PgaError

    b = scenes.collisions(64, 512, 96, rotate=False)
    eng = Engine(b["entries"], node_capacity=128, max_terminals=1 << 16)
    with pytest.raises(PgaError) as e:
        eng.execute(b["axioms"], capacity=1 << 16)
    assert e.value.status == 1
    eng.release()
