#!/usr/bin/env python3
"""Writes tests/golden/collision/pairs.npz: box / quad pairs and the results of
the reference's own collision predicate on them (Collision::check,
include/pga/core/Collision.cuh, through oracle/_ref/ref_harness --collide).

Pairs: random general rotations (rotateXYZ of uniform angles), signed
permutations, and pairs placed to touch exactly along a face axis or to miss by
one float step; kinds box/box, box/quad, quad/box, quad/quad.

Usage: python tests/golden/make_collision_golden.py   (needs oracle/_ref built)
"""
import math
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402


def _rotation(rng):
    if rng.random() < 0.35:
        R = np.eye(3)[:, rng.permutation(3)] * rng.choice([-1.0, 1.0], 3)
        return R.astype(np.float32)
    a, b, g = rng.uniform(-math.pi, math.pi, 3)
    sa, sb, sg, ca, cb, cg = math.sin(a), math.sin(b), math.sin(g), math.cos(a), math.cos(b), math.cos(g)
    return np.array([[cb * cg, cg * sa * sb - ca * sg, ca * cg * sb + sa * sg],
                     [cb * sg, ca * cg + sa * sb * sg, -cg * sa + ca * sb * sg],
                     [-sb, cb * sa, ca * cb]], np.float32)


def pairs(seed, n):
    rng = np.random.default_rng(seed)
    P = np.zeros(n, oracle.PAIR_DT)
    for k in range(n):
        kinds = rng.integers(0, 2, 2)
        P["kind"][k] = kinds
        touch = rng.random() < 0.25
        models, sizes = [], []
        for side in range(2):
            R = np.eye(3, dtype=np.float32)[:, rng.permutation(3)] if touch else _rotation(rng)
            s = rng.uniform(0.25, 3.0, 3).astype(np.float32)
            if kinds[side] == 1:
                s[2] = 1.0
            c = rng.uniform(-2.0, 2.0, 3).astype(np.float32)
            models.append(np.concatenate([R, c[:, None]], axis=1))
            sizes.append(s)
        if touch:
            # put B against A along A's world axis `ax`: centre distance = the
            # two half-extents along it (A's and B's axes are permutations)
            ax = int(rng.integers(0, 3))
            ha = sizes[0][np.argmax(np.abs(models[0][ax, :3]))] * np.float32(0.5)
            hb = sizes[1][np.argmax(np.abs(models[1][ax, :3]))] * np.float32(0.5)
            d = np.float32(ha + hb)
            if rng.random() < 0.5:
                d = np.nextafter(d, np.float32(np.inf))  # a hair apart
            models[1][:, 3] = models[0][:, 3]
            models[1][ax, 3] = np.float32(models[0][ax, 3] + d)
        P["ma"][k], P["sa"][k] = models[0].reshape(-1), sizes[0]
        P["mb"][k], P["sb"][k] = models[1].reshape(-1), sizes[1]
    return P


def main():
    P = pairs(2024, 24000)
    hits = oracle.collide_reference(P, tempfile.mkdtemp())
    np.savez_compressed(os.path.join(HERE, "collision", "pairs.npz"), pairs=P.view(np.uint8).reshape(len(P), -1),
                        hits=hits.astype(np.uint8))
    print(f"{len(P)} pairs, {int(hits.sum())} overlapping")


if __name__ == "__main__":
    main()
