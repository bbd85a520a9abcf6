"""Schedule autotuner: candidate space and selection on CPU (fake timings),
one real sweep on the GPU whose winner must still derive bit-exactly."""
import numpy as np
import pytest

import oracle
from operatorgraph_gb300 import autotune as A
from operatorgraph_gb300 import grammar as G
from operatorgraph_gb300 import scenes


def test_candidates_cover_the_space_without_duplicates():
    c = A.candidates({"sub_item": (4, 8), "narrow_sub_item": (0, 4, 8), "items_per_lane": (1,)})
    keys = {tuple(sorted(x.items())) for x in c}
    assert len(keys) == len(c)
    # narrow == sub is the same schedule as narrow = 0
    assert {"sub_item": 4, "narrow_sub_item": 0, "items_per_lane": 1} in c
    assert {"sub_item": 4, "narrow_sub_item": 4, "items_per_lane": 1} not in c
    assert len(c) == 4  # (4,0) (4,8) (8,0) (8,4)


def test_tune_picks_the_fastest_successful_candidate():
    space = {"sub_item": (4, 8, 16), "items_per_lane": (1, 2)}
    fake = {(4, 1): (0.30, 1), (8, 1): (0.31, 0), (16, 1): (0.29, 2), (4, 2): (0.35, 0), (8, 2): (0.33, 0),
            (16, 2): (0.40, 0)}

    def measure(cfg):
        ms, st = fake[(cfg["sub_item"], cfg["items_per_lane"])]
        return (ms if st == 0 else None), st

    best, ms, results = A.tune(None, 0, space=space, measure_fn=measure)
    assert best == {"sub_item": 8, "items_per_lane": 1} and ms == pytest.approx(0.31)
    assert len(results) == 6 and sum(r["status"] != 0 for r in results) == 2


def test_grouping_is_searched_only_for_batches_of_several_root_entries():
    one = A.space_for(scenes.city(16))
    assert "group_axioms" not in one and one == A.DEFAULT_SPACE
    mixed = A.space_for(scenes.mixed(64), {"sub_item": (4, 8)})
    assert mixed == {"sub_item": (4, 8), "group_axioms": (False, True)}
    assert len(A.candidates(mixed)) == 4


def test_default_schedule_is_recognised_with_or_without_optional_knobs():
    assert A.is_default(dict(A.DEFAULT_CONFIG))
    assert A.is_default({"sub_item": 8, "narrow_sub_item": 0, "items_per_lane": 1, "blocks_per_sm": 0})
    assert A.is_default(dict(A.DEFAULT_CONFIG, group_axioms=False))
    assert not A.is_default(dict(A.DEFAULT_CONFIG, group_axioms=True))
    assert not A.is_default(dict(A.DEFAULT_CONFIG, dynamic_chunks=True))
    assert not A.is_default(dict(A.DEFAULT_CONFIG, sub_item=4))


def test_schedule_cache_round_trip(tmp_path):
    """tune_cached tunes on a miss, stores the winner under the key of (rule
    table, batch signature, GPU, version), and returns it untimed on a hit; a
    different GPU name or batch is a different key."""
    b = scenes.city(16)
    calls = []

    def measure(cfg):
        calls.append(cfg)
        return 0.3 + 0.01 * cfg["sub_item"], 0

    kw = dict(space={"sub_item": (4, 8)}, cache_dir=str(tmp_path), gpu_name="GB300", library_version="x",
              measure_fn=measure)
    best, ms, res, hit = A.tune_cached(b, 0, **kw)
    assert not hit and best == {"sub_item": 4} and len(calls) == 2
    best2, ms2, res2, hit2 = A.tune_cached(b, 0, **kw)
    assert hit2 and best2 == best and ms2 == ms and len(calls) == 2
    assert A.schedule_key(b, "GB300", "x") != A.schedule_key(b, "B200", "x")
    assert A.schedule_key(b, "GB300", "x") != A.schedule_key(scenes.city(32), "GB300", "x")
    kw["gpu_name"] = "B200"
    A.tune_cached(b, 0, **kw)
    assert len(calls) == 4


def test_tune_fails_loudly_when_nothing_runs():
    with pytest.raises(RuntimeError):
        A.tune(None, 0, space={"sub_item": (8,)}, measure_fn=lambda cfg: (None, 1))


@pytest.mark.gpu
def test_tuned_schedule_derives_the_same_terminals():
    torch = pytest.importorskip("torch")
    from operatorgraph_gb300 import build as B
    from operatorgraph_gb300.engine import Engine

    B.build()
    b = scenes.city(256)
    want = oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"])
    cap = len(want) + 4096
    best, ms, results = A.tune(b, cap, node_capacity=1 << 20, runs=2,
                               space={"sub_item": (4, 8), "narrow_sub_item": (0, 2), "items_per_lane": (1, 2)})
    assert ms > 0 and len(results) == 8
    eng = Engine(b["entries"], node_capacity=1 << 20, max_terminals=cap, **best)
    out, n, _ = eng.execute(b["axioms"], capacity=cap)
    got = out[:n].cpu().numpy()
    eng.release()
    ka = np.sort(got.view(np.dtype((np.void, 64))).ravel())
    kb = np.sort(want.view(np.uint8).reshape(len(want), 64).view(np.dtype((np.void, 64))).ravel())
    assert n == len(want) and (ka == kb).all()
    assert torch.cuda.is_available()


@pytest.mark.gpu
def test_capacities_are_sized_from_a_counting_derivation():
    """size_capacities grows undersized capacities from the statuses' counts;
    the result derives the batch with no overflow and little slack."""
    pytest.importorskip("torch")
    from operatorgraph_gb300 import build as B

    B.build()
    b = scenes.city(256)
    want = len(oracle.derive(G.DEFAULT_PROCS, b["entries"], b["axioms"]))
    caps = A.size_capacities(b, node_capacity=1 << 10, max_terminals=1 << 10)
    assert want <= caps["max_terminals"] <= 1.06 * want + 1024
    assert caps["node_capacity"] >= 1024
    from operatorgraph_gb300.engine import Engine

    eng = Engine(b["entries"], **caps)
    out, n, rep = eng.execute(b["axioms"], capacity=caps["max_terminals"])
    assert rep["status"] == 0 and n == want
    eng.release()
