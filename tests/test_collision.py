"""The collision predicate of IfCollides: the restated separating-axis test
(oracle.collide) against the reference's own Collision::check
(include/pga/core/Collision.cuh, run by oracle/_ref/ref_harness --collide) on
random box / quad pairs and on pairs that touch exactly, and against the
committed fixture tests/golden/collision/pairs.npz (written by
tests/golden/make_collision_golden.py from the reference), which the GPU test
uses too."""
import os
import sys

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_collision_golden as MC  # noqa: E402


def test_restated_predicate_matches_the_committed_reference_results():
    z = np.load(os.path.join(HERE, "golden", "collision", "pairs.npz"))
    pairs = z["pairs"].view(oracle.PAIR_DT).reshape(-1)
    ref = z["hits"].astype(bool)
    got = oracle.collide(pairs)
    assert len(got) == len(ref) >= 20000
    assert (got == ref).all(), int((got != ref).sum())
    assert 0.05 < ref.mean() < 0.95  # both outcomes well represented


@pytest.mark.parametrize("seed", [11, 12])
def test_restated_predicate_matches_the_reference_live(seed, tmp_path):
    if not os.path.isfile(oracle.REF_HARNESS):
        pytest.skip("reference evaluator not built")
    pairs = MC.pairs(seed, 5000)
    assert (oracle.collide(pairs) == oracle.collide_reference(pairs, str(tmp_path))).all()
