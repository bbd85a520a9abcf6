"""The oracle package: CPU restatement of the reference's derivation path.

Test infrastructure only.  Only tests/, __graft_entry__.smoke() and the
cpu_baseline / reference legs of bench.py may import it, as the checker or as
the timed CPU baseline; the product (operatorgraph_gb300) never does.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_HARNESS = os.path.join(HERE, "_ref", "ref_harness")
from .make_ref import REFERENCE_ROOT  # noqa: E402  (where the reference sources are read, if present)

_lib = None


def build(verbose=False):
    """Compile the restatement (plain g++, -ffp-contract=off)."""
    src = os.path.join(HERE, "pga_oracle.cpp")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", src, "-o", LIB_PATH]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return LIB_PATH


def build_ref(ref_root=REFERENCE_ROOT):
    """Build oracle/_ref (the reference's own evaluator); returns the path or None."""
    script = os.path.join(HERE, "make_ref.py")
    try:
        subprocess.check_call(["python3", script, ref_root], stdout=subprocess.DEVNULL)
    except (subprocess.CalledProcessError, OSError):
        return None
    return REF_HARNESS if os.path.exists(REF_HARNESS) else None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "pga_oracle.cpp")):
            build()
        L = ctypes.CDLL(LIB_PATH)
        vp, u32, u64 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64
        L.oracle_derive.argtypes = [vp, u32, vp, u32, vp, u32, vp, u32, vp, u64, vp, vp]
        L.oracle_derive.restype = ctypes.c_int
        L.oracle_derive_base.argtypes = [vp, u32, vp, u32, vp, u32, vp, u32, vp, u64, vp, vp, u64]
        L.oracle_derive_base.restype = ctypes.c_int
        L.oracle_derive_f64.argtypes = [vp, u32, vp, u32, vp, u32, vp, u32, vp, vp, vp, u64, vp]
        L.oracle_derive_f64.restype = ctypes.c_int
        L.oracle_lbvh.argtypes = [vp, u64, vp, vp, vp, vp, vp, vp]
        L.oracle_lbvh.restype = ctypes.c_int
        L.oracle_mesh_count.restype = u32
        L.oracle_collide.argtypes = [vp, u64, vp]
        L.oracle_mesh_sizes.argtypes = [u32, vp, vp]
        L.oracle_mesh_copy.argtypes = [u32, vp, vp]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class OracleError(RuntimeError):
    def __init__(self, status, detail=0):
        super().__init__(f"oracle status {status} (detail {detail})")
        self.status = status
        self.detail = detail


def derive(procs, entries, axioms, blocks=None, block_stride=0, capacity=None, axiom_base=0):
    """Terminals of the batch (PgaTerminal records, derivation order).
    axiom_base: index of the batch's first axiom in a larger batch, so a shard
    gives the records (path hashes included) the whole batch gives for it."""
    from operatorgraph_gb300.grammar import TERMINAL_DT

    L = lib()
    procs = np.ascontiguousarray(procs)
    entries = np.ascontiguousarray(entries)
    axioms = np.ascontiguousarray(axioms)
    blk = None if blocks is None else np.ascontiguousarray(blocks, dtype=np.float32)
    cnt = np.zeros(1, np.uint64)
    det = np.zeros(1, np.int32)
    if capacity is None:
        st = L.oracle_derive_base(_ptr(procs), len(procs), _ptr(entries), len(entries), _ptr(axioms), len(axioms),
                                  _ptr(blk), block_stride, None, 0, _ptr(cnt), _ptr(det), axiom_base)
        if st not in (0, 2):
            raise OracleError(st, int(det[0]))
        capacity = int(cnt[0])
    out = np.zeros(max(capacity, 1), dtype=TERMINAL_DT)
    st = L.oracle_derive_base(_ptr(procs), len(procs), _ptr(entries), len(entries), _ptr(axioms), len(axioms),
                              _ptr(blk), block_stride, _ptr(out), capacity, _ptr(cnt), _ptr(det), axiom_base)
    if st != 0:
        raise OracleError(st, int(det[0]))
    return out[: int(cnt[0])]


def derive_meshes(procs, entries, axioms, blocks=None, block_stride=0):
    """Terminals and the triangle meshes of the triangle-mesh terminals:
    (terminals, [(vertices [nv, 12] float32, indices [ni] uint32) per mesh])."""
    terms = derive(procs, entries, axioms, blocks, block_stride)
    L = lib()
    out = []
    nv, ni = np.zeros(1, np.uint32), np.zeros(1, np.uint32)
    for m in range(L.oracle_mesh_count()):
        L.oracle_mesh_sizes(m, _ptr(nv), _ptr(ni))
        v = np.zeros((int(nv[0]), 12), np.float32)
        i = np.zeros(int(ni[0]), np.uint32)
        L.oracle_mesh_copy(m, _ptr(v), _ptr(i))
        out.append((v, i))
    return terms, out


PAIR_DT = np.dtype([("kind", "<u4", (2,)), ("ma", "<f4", (12,)), ("sa", "<f4", (3,)), ("mb", "<f4", (12,)),
                    ("sb", "<f4", (3,))])


def collide(pairs):
    """The restated collision predicate on PAIR_DT records (bool array)."""
    pairs = np.ascontiguousarray(pairs, dtype=PAIR_DT)
    out = np.zeros(len(pairs), np.uint8)
    lib().oracle_collide(_ptr(pairs), len(pairs), _ptr(out))
    return out.astype(bool)


def collide_reference(pairs, tmpdir):
    """The reference's Collision::check on the same records (oracle/_ref)."""
    pairs = np.ascontiguousarray(pairs, dtype=PAIR_DT)
    pf, of = os.path.join(tmpdir, "pairs.bin"), os.path.join(tmpdir, "hits.bin")
    pairs.tofile(pf)
    r = subprocess.run([REF_HARNESS, "--collide", pf, of], capture_output=True, text=True, timeout=600)
    if r.returncode != 0:
        raise RuntimeError(f"ref_harness --collide failed ({r.returncode}): {r.stderr.strip()}")
    return np.fromfile(of, np.uint8).astype(bool)


def derive_f64(procs, entries, axioms, blocks64=None, block_stride=0, axiom_sizes64=None, capacity=None):
    """Double-precision derivation: (M[n,12] float64, path[n] uint64)."""
    L = lib()
    procs = np.ascontiguousarray(procs)
    entries = np.ascontiguousarray(entries)
    axioms = np.ascontiguousarray(axioms)
    blk = None if blocks64 is None else np.ascontiguousarray(blocks64, dtype=np.float64)
    sz = None if axiom_sizes64 is None else np.ascontiguousarray(axiom_sizes64, dtype=np.float64)
    cnt = np.zeros(1, np.uint64)
    if capacity is None:
        st = L.oracle_derive_f64(_ptr(procs), len(procs), _ptr(entries), len(entries), _ptr(axioms), len(axioms),
                                 _ptr(blk), block_stride, _ptr(sz), None, None, 0, _ptr(cnt))
        if st not in (0, 2):
            raise OracleError(st)
        capacity = int(cnt[0])
    M = np.zeros((max(capacity, 1), 12), np.float64)
    P = np.zeros(max(capacity, 1), np.uint64)
    st = L.oracle_derive_f64(_ptr(procs), len(procs), _ptr(entries), len(entries), _ptr(axioms), len(axioms),
                             _ptr(blk), block_stride, _ptr(sz), _ptr(M), _ptr(P), capacity, _ptr(cnt))
    if st != 0:
        raise OracleError(st)
    n = int(cnt[0])
    return M[:n], P[:n]


def lbvh(terminals, bounds):
    """(nodes[n-1,3] int32, leafParents[n], aabbs[n-1,6], leafTerminal[n], keys[n])."""
    L = lib()
    t = np.ascontiguousarray(terminals)
    n = len(t)
    b = np.ascontiguousarray(np.asarray(bounds, np.float32).reshape(6))
    nodes = np.zeros((n - 1, 3), np.int32)
    lp = np.zeros(n, np.uint32)
    aabb = np.zeros((n - 1, 6), np.float32)
    lt = np.zeros(n, np.uint32)
    keys = np.zeros(n, np.uint64)
    st = L.oracle_lbvh(_ptr(t), n, _ptr(b), _ptr(nodes), _ptr(lp), _ptr(aabb), _ptr(lt), _ptr(keys))
    if st != 0:
        raise OracleError(st)
    return nodes, lp, aabb, lt, keys


def run_reference(batch_file, out_file, repeats=1, timeout=600, axiom_base=0, entry_mod=None, write_output=True):
    """Run the reference's own evaluator (oracle/_ref); returns its JSON summary.

    axiom_base: index of the batch's first axiom in a larger batch (root path
    hashes); entry_mod: entries per table copy when the batch gives each axiom
    its own copy of one table (child path hashes use the shared table's
    indices); write_output=False times execute() without writing the terminal
    file."""
    import json

    if not os.path.exists(REF_HARNESS):
        raise FileNotFoundError(REF_HARNESS)
    cmd = [REF_HARNESS, batch_file, out_file, str(repeats)]
    if axiom_base:
        cmd += ["--axiom-base", str(int(axiom_base))]
    if entry_mod:
        cmd += ["--entry-mod", str(int(entry_mod))]
    if not write_output:
        cmd += ["--no-output"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"ref_harness failed ({r.returncode}): {r.stderr.strip()}")
    return json.loads(r.stdout.strip().splitlines()[-1])
