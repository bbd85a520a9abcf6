#!/usr/bin/env python3
"""Writes tests/golden/<case>.npz from the reference's own evaluator.

Runs oracle/_ref/ref_harness (the reference's SinglePhaseEvaluator, built by
oracle/make_ref.py from the reference sources) on every case of cases.py and
stores: the grammar batch, the terminal count, a SHA-256 digest and checksum
of the canonical (sorted, path-free) terminal records, a second digest of the
records WITH their derivation-path hashes (sorted by path; the harness takes
the hashes from the reference's own child-creation call sites, see
oracle/make_ref.py), and -- for cases of at most 2,000 terminals -- the
canonical records themselves and the sorted path hashes.  For grammars with
triangle-mesh terminals it also stores each mesh's vertex and index counts and
the digest of its order-free faces (cases.mesh_digest).

Usage: python tests/golden/make_golden.py [case-name-prefix ...]   (needs oracle/_ref built)
With prefixes, only the matching cases are (re)written.
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

import oracle  # noqa: E402
from operatorgraph_gb300 import grammar as G  # noqa: E402

import cases as C  # noqa: E402

FULL_LIMIT = 2000


def main():
    tmp = tempfile.mkdtemp()
    only = sys.argv[1:]
    for name, b in C.cases():
        if only and not any(name.startswith(p) for p in only):
            continue
        entries, axioms = b["entries"], b["axioms"]
        n_base = None
        if b["blocks"] is not None:
            entries, axioms = G.expand_blocks(entries, axioms, b["blocks"], b["block_stride"])
            n_base = len(b["entries"])
        bf, tf = os.path.join(tmp, "b.bin"), os.path.join(tmp, "t.bin")
        if os.path.exists(tf + ".mesh"):
            os.remove(tf + ".mesh")
        G.write_batch_file(bf, entries, axioms)
        info = oracle.run_reference(bf, tf, entry_mod=n_base)
        ref = G.read_terminal_file(tf)
        meshes = G.read_mesh_file(tf + ".mesh") if os.path.exists(tf + ".mesh") else []
        canon = C.canonical(ref, n_base)
        m = canon["m"].astype(np.float64)
        checksum = float((m[:, 3] + 2 * m[:, 7] + 3 * m[:, 11] + m[:, 0]).sum())
        payload = dict(entries=b["entries"].view(np.uint8), axioms=b["axioms"].view(np.uint8),
                       count=np.int64(len(ref)), digest=np.array(C.digest(canon)), checksum=np.float64(checksum),
                       digest_path=np.array(C.digest(C.canonical_paths(ref, n_base))))
        if b["blocks"] is not None:
            payload["blocks"] = b["blocks"]
            payload["block_stride"] = np.int64(b["block_stride"])
        if len(ref) <= FULL_LIMIT:
            payload["terminals"] = canon.view(np.uint8)
            payload["paths"] = np.sort(ref["path"])
        if meshes:
            payload["mesh_counts"] = np.array([(len(v), len(i)) for v, i in meshes], np.int64)
            payload["mesh_digests"] = np.array([C.mesh_digest(v, i) for v, i in meshes])
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **payload)
        print(f"{name}: {len(ref)} terminals, checksum {checksum:.6f}, reference {info['seconds']:.6f} s")


if __name__ == "__main__":
    main()
