"""Grammar-as-data: the reference's dispatch-table format, in numpy.

Mirrors PGA::DispatchTable / DispatchTable::Entry / Parameter / Successor
(include/pga/core/DispatchTable.h:16-106) and the POD DispatchTableEntry
(include/pga/core/DispatchTableEntry.h:8-36).  Values are given as Python
floats (doubles) and narrowed to float32 exactly like
DispatchTable::Parameter::fill (DispatchTable.h:27-35, static_cast<float>).

The numpy record layouts are byte-identical to the C structs of
include/pga_gb300.h (PgaEntry, PgaProc, PgaAxiom, PgaTerminal).
"""
import struct

import numpy as np

MAX_PARAMS = 17
MAX_VALUES = 16
MAX_SUCC = 20

# PGA::ParameterType (include/pga/core/ParameterType.h) plus the per-axiom block type.
PT_SCALAR, PT_RAND, PT_SHAPE_ATTR, PT_EXP, PT_VEC2, PT_VEC4 = 0, 1, 2, 3, 4, 5
PT_BLOCK = 16

# PgaOperator
OP_SUBDIVIDE, OP_SUBDIVIDE_STATIC, OP_REPEAT, OP_COMPONENT_SPLIT = 0, 1, 2, 3
OP_EXTRUDE, OP_IF_SIZE_LESS, OP_GENERATE, OP_DISCARD = 4, 5, 6, 7
OP_TRANSLATE, OP_SCALE, OP_RANDOM_RULE, OP_ROTATE, OP_REPLICATE, OP_RANDOM_RULE_STATIC = 8, 9, 10, 11, 12, 13
OP_IF, OP_SWAP_SIZE, OP_GENERATE_MESH, OP_COLLIDER, OP_IF_COLLIDES = 14, 15, 16, 17, 18
OP_NAMES = ["Subdivide", "SubdivideStatic", "Repeat", "ComponentSplit", "Extrude", "IfSizeLess", "Generate", "Discard",
            "Translate", "Scale", "RandomRule", "Rotate", "Replicate", "RandomRuleStatic", "If", "SwapSize",
            "GenerateMesh", "Collider", "IfCollides"]

SHAPE_BOX, SHAPE_QUAD = 0, 1

# PGA::RepeatMode (include/pga/core/RepeatMode.h)
ANCHOR_TO_START, ANCHOR_TO_END, ADJUST_TO_FILL = 0, 1, 2

# Operator codes of the generic procedure list (pga_default_procs()).
BOX_SUBDIVIDE, QUAD_SUBDIVIDE = 0, 1
BOX_SUBDIVIDE3, QUAD_SUBDIVIDE3 = 2, 3
BOX_REPEAT, QUAD_REPEAT = 4, 5
BOX_COMPONENT_SPLIT, QUAD_EXTRUDE = 6, 7
BOX_IF_SIZE_LESS, QUAD_IF_SIZE_LESS = 8, 9
BOX_GENERATE, QUAD_GENERATE = 10, 11
BOX_DISCARD, QUAD_DISCARD = 12, 13
BOX_TRANSLATE, QUAD_TRANSLATE = 14, 15
BOX_SCALE, QUAD_SCALE = 16, 17
BOX_RANDOM_RULE, QUAD_RANDOM_RULE = 18, 19
BOX_ROTATE, QUAD_ROTATE = 20, 21
BOX_REPLICATE, QUAD_REPLICATE = 22, 23
# RandomRule<DynParam<0>, Pair<DynParam<k>, DCall<k-1>>...> with 2, 3 and 4 pairs (the static form)
BOX_RANDOM_RULE2, QUAD_RANDOM_RULE2, BOX_RANDOM_RULE3, QUAD_RANDOM_RULE3, BOX_RANDOM_RULE4, QUAD_RANDOM_RULE4 = range(24, 30)
BOX_IF, QUAD_IF = 30, 31
BOX_SWAP_SIZE, QUAD_SWAP_SIZE = 32, 33
BOX_GENERATE_MESH, QUAD_GENERATE_MESH = 34, 35  # Generate<false, 0, DynParam<0>>: triangle-mesh terminals
# Collider<DynParam<0> tag, DCall<0>> and IfCollides<DynParam<0> tag, DCall<0>, DCall<1>> (multi-phase tables;
# the reference evaluates them on the GPU only, so the reference harness has no procedures for them)
BOX_COLLIDER, QUAD_COLLIDER, BOX_IF_COLLIDES, QUAD_IF_COLLIDES = 36, 37, 38, 39

PARAM_DT = np.dtype([("type", "<i4"), ("value", "<f4", (MAX_VALUES,))])
SUCC_DT = np.dtype([("entryIndex", "<i4"), ("phaseIndex", "<i4")])
ENTRY_DT = np.dtype([
    ("operatorCode", "<i4"), ("numParameters", "<u4"), ("numSuccessors", "<u4"), ("reserved", "<u4"),
    ("parameters", PARAM_DT, (MAX_PARAMS,)), ("successors", SUCC_DT, (MAX_SUCC,)),
])
PROC_DT = np.dtype([("op", "<u4"), ("shape", "<u4"), ("numChildren", "<u4"), ("numThreads", "<u4")])
AXIOM_DT = np.dtype([
    ("position", "<f4", (3,)), ("seed", "<f4"), ("size", "<f4", (3,)), ("custom", "<f4"),
    ("entry", "<u4"), ("shape", "<u4"), ("block", "<u4"), ("flags", "<u4"),
])
TERMINAL_DT = np.dtype([("m", "<f4", (12,)), ("rule", "<u4"), ("custom", "<f4"), ("path", "<u8")])
# PgaVertex / PgaTriangleMesh (the reference's TriangleMeshData layouts).
VERTEX_DT = np.dtype([("position", "<f4", (4,)), ("normal", "<f4", (3,)), ("uv", "<f4", (2,)), ("pad", "<f4", (3,))])
MESH_DT = np.dtype([("numVertices", "<u4"), ("numIndices", "<u4"), ("maxNumVertices", "<u4"), ("maxNumIndices", "<u4"),
                    ("vertices", "<u8"), ("indices", "<u8")])
assert ENTRY_DT.itemsize == 1332 and AXIOM_DT.itemsize == 48 and TERMINAL_DT.itemsize == 64
assert VERTEX_DT.itemsize == 48 and MESH_DT.itemsize == 32

# The generic procedure list: (operator, shape, numChildren) per operator code.
DEFAULT_PROCS = np.array([
    (OP_SUBDIVIDE, SHAPE_BOX, 0, 1), (OP_SUBDIVIDE, SHAPE_QUAD, 0, 1),
    (OP_SUBDIVIDE_STATIC, SHAPE_BOX, 3, 1), (OP_SUBDIVIDE_STATIC, SHAPE_QUAD, 3, 1),
    (OP_REPEAT, SHAPE_BOX, 0, 1), (OP_REPEAT, SHAPE_QUAD, 0, 1),
    (OP_COMPONENT_SPLIT, SHAPE_BOX, 0, 1), (OP_EXTRUDE, SHAPE_QUAD, 0, 1),
    (OP_IF_SIZE_LESS, SHAPE_BOX, 0, 1), (OP_IF_SIZE_LESS, SHAPE_QUAD, 0, 1),
    (OP_GENERATE, SHAPE_BOX, 0, 1), (OP_GENERATE, SHAPE_QUAD, 0, 1),
    (OP_DISCARD, SHAPE_BOX, 0, 1), (OP_DISCARD, SHAPE_QUAD, 0, 1),
    (OP_TRANSLATE, SHAPE_BOX, 0, 1), (OP_TRANSLATE, SHAPE_QUAD, 0, 1),
    (OP_SCALE, SHAPE_BOX, 0, 1), (OP_SCALE, SHAPE_QUAD, 0, 1),
    (OP_RANDOM_RULE, SHAPE_BOX, 0, 1), (OP_RANDOM_RULE, SHAPE_QUAD, 0, 1),
    (OP_ROTATE, SHAPE_BOX, 0, 1), (OP_ROTATE, SHAPE_QUAD, 0, 1),
    (OP_REPLICATE, SHAPE_BOX, 0, 1), (OP_REPLICATE, SHAPE_QUAD, 0, 1),
    (OP_RANDOM_RULE_STATIC, SHAPE_BOX, 2, 1), (OP_RANDOM_RULE_STATIC, SHAPE_QUAD, 2, 1),
    (OP_RANDOM_RULE_STATIC, SHAPE_BOX, 3, 1), (OP_RANDOM_RULE_STATIC, SHAPE_QUAD, 3, 1),
    (OP_RANDOM_RULE_STATIC, SHAPE_BOX, 4, 1), (OP_RANDOM_RULE_STATIC, SHAPE_QUAD, 4, 1),
    (OP_IF, SHAPE_BOX, 0, 1), (OP_IF, SHAPE_QUAD, 0, 1),
    (OP_SWAP_SIZE, SHAPE_BOX, 0, 1), (OP_SWAP_SIZE, SHAPE_QUAD, 0, 1),
    (OP_GENERATE_MESH, SHAPE_BOX, 0, 1), (OP_GENERATE_MESH, SHAPE_QUAD, 0, 1),
    (OP_COLLIDER, SHAPE_BOX, 0, 1), (OP_COLLIDER, SHAPE_QUAD, 0, 1),
    (OP_IF_COLLIDES, SHAPE_BOX, 0, 1), (OP_IF_COLLIDES, SHAPE_QUAD, 0, 1),
], dtype=PROC_DT)


class Parameter:
    """DispatchTable::Parameter: a type and up to 16 values (doubles)."""

    def __init__(self, type=PT_SCALAR, values=(0.0,)):
        self.type = int(type)
        self.values = [float(v) for v in values]
        if len(self.values) > MAX_VALUES:
            raise ValueError("values.size() > MaxNumParameterValues")


class Successor:
    def __init__(self, entryIndex=-1, phaseIndex=0):
        self.entryIndex = int(entryIndex)
        self.phaseIndex = int(phaseIndex)


class Entry:
    """DispatchTable::Entry: operator code, parameters and successors."""

    def __init__(self, operatorCode, parameters=(), successors=()):
        self.operatorCode = int(operatorCode)
        self.parameters = [p if isinstance(p, Parameter) else Parameter(*p) for p in parameters]
        self.successors = [s if isinstance(s, Successor) else Successor(*s) for s in successors]
        if len(self.parameters) > MAX_PARAMS:
            raise ValueError("parameters.size() > MaxNumParameters")
        if len(self.successors) > MAX_SUCC:
            raise ValueError("successors.size() > MaxNumSuccessors")


class DispatchTable:
    def __init__(self, entries=()):
        self.entries = list(entries)

    def __len__(self):
        return len(self.entries)

    def to_array(self):
        """Like DispatchTable::toDispatchTableEntriesPtr (DispatchTable.h:98-104)."""
        arr = np.zeros(len(self.entries), dtype=ENTRY_DT)
        arr["successors"]["entryIndex"] = -1
        arr["successors"]["phaseIndex"] = -1
        for i, e in enumerate(self.entries):
            arr[i]["operatorCode"] = e.operatorCode
            arr[i]["numParameters"] = len(e.parameters)
            arr[i]["numSuccessors"] = len(e.successors)
            for k, p in enumerate(e.parameters):
                arr[i]["parameters"][k]["type"] = p.type
                vals = np.zeros(MAX_VALUES, dtype=np.float32)
                vals[: len(p.values)] = np.array(p.values, dtype=np.float64).astype(np.float32)
                arr[i]["parameters"][k]["value"] = vals
            for k, s in enumerate(e.successors):
                arr[i]["successors"][k]["entryIndex"] = s.entryIndex
                arr[i]["successors"][k]["phaseIndex"] = s.phaseIndex
        return arr


def scalar(v):
    return Parameter(PT_SCALAR, (v,))


def shape_attr(i):
    return Parameter(PT_SHAPE_ATTR, (i,))


def rand(lo, hi):
    return Parameter(PT_RAND, (lo, hi))


def block(slot):
    return Parameter(PT_BLOCK, (slot,))


# Operand kinds and operations of expression parameters
# (include/pga/core/OperandType.h, OperationType.h).
ORT_SCALAR, ORT_RAND, ORT_SHAPE_ATTR, ORT_OP = 0, 1, 2, 3
OPT_ADD, OPT_SUB, OPT_DIV, OPT_MULTI, OPT_EQ, OPT_NEQ, OPT_LT, OPT_GT, OPT_LEQ, OPT_GEQ, OPT_AND, OPT_OR = range(12)


def _pack_operand(kind, x):
    """One program word: the operand kind in the top two bits, the value's
    float32 bits shifted right by two below (PackUtils::packOperand, PackUtils.h:18-23)."""
    r = int(np.float32(x).view(np.uint32))
    return float(np.uint32((r >> 2) | (kind << 30)).view(np.float32))


def exp(*program):
    """Expression parameter (PT_EXP) from a postfix program of tokens:
    ("s", value) scalar, ("a", index) shape attribute, ("op", OPT_*) binary
    operation.  value[0] = program length, value[1..] = the packed words
    (Parameters.cuh:459-483)."""
    words = []
    for tok in program:
        kind, v = tok
        words.append(_pack_operand({"s": ORT_SCALAR, "a": ORT_SHAPE_ATTR, "op": ORT_OP}[kind], float(v)))
    if len(words) + 1 > MAX_VALUES:
        raise ValueError("expression longer than a parameter holds")
    return Parameter(PT_EXP, [float(len(words))] + words)


def make_axioms(n):
    a = np.zeros(n, dtype=AXIOM_DT)
    a["size"] = 1.0
    a["block"] = np.arange(n, dtype=np.uint32)
    return a


def concat_tables(tables):
    """Concatenate entry arrays, rebasing successor indices; returns (array, offsets)."""
    offsets, parts, base = [], [], 0
    for t in tables:
        t = t.copy()
        succ = t["successors"]["entryIndex"]
        succ[succ >= 0] += base
        t["successors"]["entryIndex"] = succ
        offsets.append(base)
        parts.append(t)
        base += len(t)
    return np.concatenate(parts), offsets


def write_batch_file(path, entries, axioms):
    """Grammar-batch file read by oracle/_ref/ref_harness and the oracle CLI."""
    entries = np.ascontiguousarray(entries, dtype=ENTRY_DT)
    axioms = np.ascontiguousarray(axioms, dtype=AXIOM_DT)
    with open(path, "wb") as f:
        f.write(b"PGAB" + struct.pack("<III", 1, len(entries), len(axioms)))
        f.write(entries.tobytes())
        f.write(axioms.tobytes())


def read_terminal_file(path):
    with open(path, "rb") as f:
        head = f.read(16)
        assert head[:4] == b"PGAT", head
        (n,) = struct.unpack("<Q", head[8:16])
        return np.frombuffer(f.read(n * TERMINAL_DT.itemsize), dtype=TERMINAL_DT).copy()


def expand_blocks(entries, axioms, blocks, block_stride):
    """Realise per-axiom parameter blocks as per-axiom copies of the table.

    PGA_PT_BLOCK has no counterpart in the reference; for the reference's own
    evaluator a batch with blocks becomes one table copy per axiom, with the
    block values written in as PT_SCALAR and the axiom rooted in its copy.
    """
    n_e = len(entries)
    out, ax = [], axioms.copy()
    for i, a in enumerate(axioms):
        t = entries.copy()
        p = t["parameters"]
        is_blk = p["type"] == PT_BLOCK
        slots = p["value"][..., 0].astype(np.int64)
        vals = blocks[int(a["block"]) * block_stride + slots]
        p["value"][..., 0] = np.where(is_blk, vals, p["value"][..., 0])
        p["type"] = np.where(is_blk, PT_SCALAR, p["type"])
        t["parameters"] = p
        succ = t["successors"]["entryIndex"]
        succ[succ >= 0] += i * n_e
        t["successors"]["entryIndex"] = succ
        out.append(t)
        ax[i]["entry"] = a["entry"] + i * n_e
    return np.concatenate(out), ax


def sort_terminals(t, by_path=False):
    """Canonical order for multiset comparison (queue order is free)."""
    if by_path:
        return t[np.argsort(t["path"], kind="stable")]
    m = t["m"].view(np.uint32)
    keys = [t["custom"].view(np.uint32), t["rule"]] + [m[:, i] for i in range(11, -1, -1)]
    return t[np.lexsort(keys)]


def mesh_faces(vertices, indices):
    """Faces of a generated triangle mesh as an order-free array: for each run
    of 6 indices (v, v+1, v+2, v, v+2, v+3) the 4 vertices' 12 floats (PgaVertex
    without padding; -0 -> +0), checked against that pattern; sorted by bytes.
    vertices: [nv, 12] float32 (PgaVertex layout), indices: [ni] integers."""
    v = np.asarray(vertices, np.float32).reshape(-1, 12)[:, :9] + np.float32(0)
    v = np.where(np.isnan(v), np.float32(np.nan), v).astype(np.float32)  # one NaN pattern (degenerate faces)
    idx = np.asarray(indices).astype(np.int64).reshape(-1, 6)
    base = idx[:, 0]
    want = base[:, None] + np.array([0, 1, 2, 0, 2, 3])
    assert (idx == want).all(), "index pattern of a face"
    assert base.size == 0 or (base.min() >= 0 and base.max() + 3 < len(v)), "face vertex out of range"
    faces = v[base[:, None] + np.arange(4)].reshape(len(base), 36)
    key = np.ascontiguousarray(faces).view(np.dtype((np.void, 36 * 4))).ravel()
    return faces[np.argsort(key, kind="stable")]


def read_mesh_file(path):
    """Meshes written by the reference harness: per mesh (vertices [nv, 12]
    float32, indices [ni] uint32)."""
    out = []
    with open(path, "rb") as f:
        head = f.read(8)
        assert head[:4] == b"PGAM", head
        n = int(np.frombuffer(head[4:], "<u4")[0])
        for _ in range(n):
            nv, ni = np.frombuffer(f.read(8), "<u4")
            v = np.frombuffer(f.read(int(nv) * 48), np.float32).reshape(-1, 12)
            i = np.frombuffer(f.read(int(ni) * 4), "<u4")
            out.append((v, i))
    return out
