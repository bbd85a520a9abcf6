"""Python side of the C ABI (include/pga_gb300.h) over ctypes.

`Engine` mirrors the reference's evaluator interface
(PGA::GPU::SinglePhaseEvaluator, include/pga/core/GPUEvaluator.cuh:475-536):
``initialize`` (here: the constructor, from a dispatch table), ``execute``
(derive a batch of axioms) and ``release``.  Device memory and streams come
from PyTorch; the work itself runs in libpga_gb300.so.  There is no CPU
fallback: without the compiled library every call raises.
"""
import ctypes
import os

import numpy as np

from . import grammar as G

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("PGA_LIB") or os.path.join(HERE, "libpga_gb300.so")

STATUS = {
    0: "PGA_OK", 1: "PGA_ERR_QUEUE_OVERFLOW", 2: "PGA_ERR_OUTPUT_OVERFLOW", 3: "PGA_ERR_TIMEOUT",
    4: "PGA_ERR_BAD_OPCODE", 5: "PGA_ERR_BAD_PARAM", 6: "PGA_ERR_CUDA", 7: "PGA_ERR_INVALID_ARGUMENT",
    8: "PGA_ERR_NO_TAPE", 9: "PGA_ERR_DEPTH", 10: "PGA_ERR_INTERNAL",
}

# Every symbol include/pga_gb300.h declares.
EXPORTS = ["pga_version", "pga_last_error", "pga_default_procs", "pga_engine_create", "pga_engine_destroy",
           "pga_derive", "pga_derive_plain", "pga_engine_sync_report", "pga_engine_levels", "pga_lbvh_build",
           "pga_lbvh_build_counted", "pga_lbvh_build_static", "pga_adjoint", "pga_adjoint_strided",
           "pga_derive_to_host", "pga_generate_meshes", "pga_derive_per_axiom"]


class PgaError(RuntimeError):
    def __init__(self, status, message=""):
        self.status = int(status)
        super().__init__(f"{STATUS.get(self.status, self.status)}: {message}")


class PgaProc(ctypes.Structure):
    _fields_ = [("op", ctypes.c_uint32), ("shape", ctypes.c_uint32), ("numChildren", ctypes.c_uint32),
                ("numThreads", ctypes.c_uint32)]


class PgaRuleTable(ctypes.Structure):
    _fields_ = [("procs", ctypes.c_void_p), ("numProcs", ctypes.c_uint32), ("entries", ctypes.c_void_p),
                ("numEntries", ctypes.c_uint32)]


class PgaEngineConfig(ctypes.Structure):
    _fields_ = [("nodeCapacity", ctypes.c_uint64), ("maxTerminals", ctypes.c_uint64),
                ("blockStride", ctypes.c_uint32), ("threadsPerBlock", ctypes.c_uint32),
                ("blocksPerSM", ctypes.c_uint32), ("recordTape", ctypes.c_uint32), ("spinLimit", ctypes.c_uint32),
                ("maxLevels", ctypes.c_uint32), ("flags", ctypes.c_uint32), ("subItem", ctypes.c_uint32),
                ("itemsPerLane", ctypes.c_uint32), ("narrowSubItem", ctypes.c_uint32)]


class PgaDeriveReport(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("detail", ctypes.c_int32), ("terminals", ctypes.c_uint64),
                ("nodes", ctypes.c_uint64), ("levels", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("maxLevelNodes", ctypes.c_uint64)]


class PgaBounds(ctypes.Structure):
    _fields_ = [("min", ctypes.c_float * 3), ("max", ctypes.c_float * 3)]


class PgaLbvh(ctypes.Structure):
    _fields_ = [("nodes", ctypes.c_void_p), ("leafParents", ctypes.c_void_p), ("aabbs", ctypes.c_void_p),
                ("leafTerminal", ctypes.c_void_p), ("keys", ctypes.c_void_p)]


_lib = None


PGA_FLAG_NO_INLINE = 1  # PgaEngineConfig.flags: queue leaf children instead of expanding them in place
PGA_FLAG_GROUP_AXIOMS = 2  # seed the axioms grouped by root entry (same records, another output order)
PGA_FLAG_DYNAMIC_CHUNKS = 4  # the last quarter of each level's items from a shared counter (another output order)


def load_library(path=LIB_PATH):
    """Loads libpga_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise PgaError(6, f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    L = ctypes.CDLL(path)
    vp, u32, u64 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64
    L.pga_version.restype = ctypes.c_char_p
    L.pga_last_error.restype = ctypes.c_char_p
    L.pga_default_procs.argtypes = [ctypes.POINTER(u32)]
    L.pga_default_procs.restype = ctypes.POINTER(PgaProc)
    L.pga_engine_create.argtypes = [ctypes.POINTER(PgaRuleTable), ctypes.POINTER(PgaEngineConfig), ctypes.POINTER(vp)]
    L.pga_engine_destroy.argtypes = [vp]
    for name in ("pga_derive", "pga_derive_plain", "pga_derive_per_axiom"):
        getattr(L, name).argtypes = [vp, vp, u32, vp, vp, u64, vp, vp]
    L.pga_engine_sync_report.argtypes = [vp, vp, ctypes.POINTER(PgaDeriveReport)]
    L.pga_lbvh_build.argtypes = [vp, vp, u64, ctypes.POINTER(PgaBounds), ctypes.POINTER(PgaLbvh), vp]
    L.pga_lbvh_build_counted.argtypes = [vp, vp, vp, u64, ctypes.POINTER(PgaBounds), ctypes.POINTER(PgaLbvh), vp]
    L.pga_adjoint.argtypes = [vp, vp, vp, u32, vp, vp]
    L.pga_adjoint_strided.argtypes = [vp, vp, u32, vp, u32, vp, vp]
    L.pga_engine_levels.argtypes = [vp, vp, vp, vp, u32, ctypes.POINTER(u32)]
    L.pga_lbvh_build_static.argtypes = [vp, u64, ctypes.POINTER(PgaBounds), ctypes.POINTER(PgaLbvh), vp]
    L.pga_derive_to_host.argtypes = [vp, vp, u32, vp, vp, u64, ctypes.POINTER(u64), vp]
    L.pga_generate_meshes.argtypes = [vp, vp, u64, vp, u32, vp]
    for name in EXPORTS[3:]:
        getattr(L, name).restype = ctypes.c_int
    _lib = L
    return L


def last_error():
    return load_library().pga_last_error().decode()


def _check(status, what=""):
    if status != 0:
        raise PgaError(status, f"{what}: {last_error()}")


def _stream_handle(stream):
    import torch

    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


def _dev(arr_or_tensor):
    """Device copy (torch uint8) of a numpy record array, or the tensor itself."""
    import torch

    if isinstance(arr_or_tensor, torch.Tensor):
        return arr_or_tensor
    a = np.ascontiguousarray(arr_or_tensor)
    return torch.from_numpy(a.view(np.uint8).reshape(-1).copy()).cuda()


class Engine:
    """A dispatch table lowered to the device, plus all of its work storage."""

    def __init__(self, entries, procs=None, node_capacity=1 << 22, max_terminals=1 << 22, block_stride=0,
                 record_tape=False, blocks_per_sm=0, spin_limit=0, max_levels=0, sub_item=0, items_per_lane=0,
                 narrow_sub_item=0, no_inline=False, group_axioms=False, dynamic_chunks=False):
        L = load_library()
        self.entries = np.ascontiguousarray(entries, dtype=G.ENTRY_DT)
        self.procs = np.ascontiguousarray(G.DEFAULT_PROCS if procs is None else procs, dtype=G.PROC_DT)
        table = PgaRuleTable(self.procs.ctypes.data, len(self.procs), self.entries.ctypes.data, len(self.entries))
        self.config = PgaEngineConfig(node_capacity, max_terminals, block_stride, 256, blocks_per_sm,
                                      1 if record_tape else 0, spin_limit, max_levels,
                                      (PGA_FLAG_NO_INLINE if no_inline else 0)
                                      | (PGA_FLAG_GROUP_AXIOMS if group_axioms else 0)
                                      | (PGA_FLAG_DYNAMIC_CHUNKS if dynamic_chunks else 0), sub_item,
                                      items_per_lane, narrow_sub_item)
        h = ctypes.c_void_p()
        _check(L.pga_engine_create(ctypes.byref(table), ctypes.byref(self.config), ctypes.byref(h)),
               "pga_engine_create")
        self.handle = h
        self.block_stride = block_stride

    # -- raw C-ABI calls on device pointers ------------------------------------------------
    def derive_raw(self, d_axioms, n_axioms, d_blocks, d_out, capacity, d_count, stream=None, plain=False):
        """pga_derive; plain=True: pga_derive_plain (host-driven levels), plain="per_axiom":
        pga_derive_per_axiom (one persistent launch per axiom, no host read-back)."""
        L = load_library()
        name = {False: "pga_derive", True: "pga_derive_plain", "per_axiom": "pga_derive_per_axiom"}[plain]
        fn = getattr(L, name)
        _check(fn(self.handle, d_axioms, n_axioms, d_blocks, d_out, capacity, d_count, _stream_handle(stream)), name)

    def derive_to_host(self, h_axioms, n_axioms, h_out, capacity, d_blocks=None, stream=None, check=True):
        """pga_derive_to_host on host pointers (pinned memory is fastest); returns (count, status)."""
        n = ctypes.c_uint64()
        st = load_library().pga_derive_to_host(self.handle, h_axioms, n_axioms, d_blocks, h_out, capacity,
                                                ctypes.byref(n), _stream_handle(stream))
        if check:
            _check(st, "pga_derive_to_host")
        return n.value, st

    def report(self, stream=None):
        rep = PgaDeriveReport()
        st = load_library().pga_engine_sync_report(self.handle, _stream_handle(stream), ctypes.byref(rep))
        return {"status": st, "detail": rep.detail, "terminals": rep.terminals, "nodes": rep.nodes,
                "levels": rep.levels, "max_level_nodes": rep.maxLevelNodes}

    def levels(self, stream=None, capacity=4096):
        """Per-level node ranges and device clocks of the last pga_derive.

        Returns (starts, nanos): starts[l] is the first item of level l; nanos[0]
        the launch start, nanos[l + 1] the time level l's range was fixed and
        nanos[-1] the launch end."""
        L = load_library()
        starts = np.zeros(capacity, np.uint64)
        nanos = np.zeros(capacity + 2, np.uint64)
        n = ctypes.c_uint32()
        _check(L.pga_engine_levels(self.handle, _stream_handle(stream), starts.ctypes.data, nanos.ctypes.data,
                                   capacity + 2, ctypes.byref(n)), "pga_engine_levels")
        k = min(n.value, capacity)
        return starts[:k], nanos[: k + 2]

    # -- convenience on torch tensors --------------------------------------------------------
    def execute(self, axioms, blocks=None, capacity=None, plain=False, out=None, stream=None, check=True):
        """Derives `axioms` (AXIOM_DT array or device uint8 tensor); returns (terminals, count, report)."""
        import torch

        d_ax = _dev(axioms)
        n_ax = d_ax.numel() // G.AXIOM_DT.itemsize
        d_blk = None
        if blocks is not None:
            d_blk = blocks if isinstance(blocks, torch.Tensor) else torch.from_numpy(
                np.ascontiguousarray(blocks, np.float32)).cuda()
        if out is None:
            out = torch.empty((capacity, G.TERMINAL_DT.itemsize), dtype=torch.uint8, device="cuda")
        capacity = out.shape[0]
        count = torch.zeros(1, dtype=torch.int64, device="cuda")
        self.derive_raw(d_ax.data_ptr(), n_ax, None if d_blk is None else d_blk.data_ptr(), out.data_ptr(), capacity,
                        count.data_ptr(), stream, plain)
        rep = self.report(stream)
        if check and rep["status"] != 0:
            raise PgaError(rep["status"], f"device status (detail {rep['detail']})")
        n = int(count.item())
        if check and n > capacity:
            raise PgaError(2, f"{n} terminals > capacity {capacity}")
        return out, n, rep

    def lbvh(self, terminals, n, bounds, stream=None, count=None):
        """Builds the LBVH over terminals[:n]; returns a dict of device tensors.

        With `count` (a device int64 tensor holding the leaf count, such as the
        one derive wrote), n is the capacity: the tree covers the first
        min(count, n) terminals and nothing is read back to the host
        (pga_lbvh_build_counted), so the call can be captured in a CUDA graph.
        """
        import torch

        L = load_library()
        dev = "cuda"
        res = {
            "nodes": torch.empty((n - 1, 3), dtype=torch.int32, device=dev),
            "leafParents": torch.empty(n, dtype=torch.int32, device=dev),
            "aabbs": torch.empty((n - 1, 6), dtype=torch.float32, device=dev),
            "leafTerminal": torch.empty(n, dtype=torch.int32, device=dev),
            "keys": torch.empty(n, dtype=torch.int64, device=dev),
        }
        b = np.asarray(bounds, np.float32).reshape(6)
        pb = PgaBounds((ctypes.c_float * 3)(*b[:3]), (ctypes.c_float * 3)(*b[3:]))
        out = PgaLbvh(res["nodes"].data_ptr(), res["leafParents"].data_ptr(), res["aabbs"].data_ptr(),
                      res["leafTerminal"].data_ptr(), res["keys"].data_ptr())
        if count is None:
            _check(L.pga_lbvh_build(self.handle, terminals.data_ptr(), n, ctypes.byref(pb), ctypes.byref(out),
                                    _stream_handle(stream)), "pga_lbvh_build")
        else:
            _check(L.pga_lbvh_build_counted(self.handle, terminals.data_ptr(), count.data_ptr(), n, ctypes.byref(pb),
                                            ctypes.byref(out), _stream_handle(stream)), "pga_lbvh_build_counted")
        return res

    def generate_meshes_raw(self, d_terminals, n, d_meshes, num_meshes, stream=None):
        _check(load_library().pga_generate_meshes(self.handle, d_terminals, n, d_meshes, num_meshes,
                                                  _stream_handle(stream)), "pga_generate_meshes")

    def generate_meshes(self, terminals, n, capacities, stream=None):
        """Triangle meshes of the triangle-mesh terminals among terminals[:n]
        (a device tensor of records).  capacities: (maxNumVertices,
        maxNumIndices) per mesh.  Returns, per mesh, (vertices [numVertices, 12]
        float32 tensor in PgaVertex layout, indices uint32-as-int32 tensor,
        numVertices, numIndices) after a synchronize; statuses raise."""
        import torch

        bufs, rows = [], []
        for mv, mi in capacities:
            v = torch.zeros((max(mv, 1), 12), dtype=torch.float32, device="cuda")
            i = torch.zeros(max(mi, 1), dtype=torch.int32, device="cuda")
            bufs.append((v, i))
            rows.append((0, 0, mv, mi, v.data_ptr(), i.data_ptr()))
        table = np.array(rows, dtype=G.MESH_DT)
        d_table = torch.from_numpy(table.view(np.uint8).copy()).to("cuda")
        self.generate_meshes_raw(terminals.data_ptr(), n, d_table.data_ptr(), len(rows), stream)
        torch.cuda.synchronize()
        rep = self.report(stream)
        if rep["status"] != 0:
            raise PgaError(rep["status"], f"pga_generate_meshes: {STATUS.get(rep['status'])} (detail {rep['detail']})")
        counts = d_table.cpu().numpy().view(G.MESH_DT)
        out = []
        for (v, i), c in zip(bufs, counts):
            nv, ni = int(c["numVertices"]), int(c["numIndices"])
            out.append((v[:nv], i[:ni], nv, ni))
        return out

    def adjoint_raw(self, d_grad_terminals, d_grad_params, num_blocks, d_grad_sizes, stream=None, grad_stride=12):
        """pga_adjoint (grad_stride 12) or pga_adjoint_strided: dL/dm of terminal t at
        d_grad_terminals + t * grad_stride floats."""
        L = load_library()
        if grad_stride == 12:
            _check(L.pga_adjoint(self.handle, d_grad_terminals, d_grad_params, num_blocks, d_grad_sizes,
                                 _stream_handle(stream)), "pga_adjoint")
        else:
            _check(L.pga_adjoint_strided(self.handle, d_grad_terminals, grad_stride, d_grad_params, num_blocks,
                                         d_grad_sizes, _stream_handle(stream)), "pga_adjoint_strided")

    def release(self):
        if getattr(self, "handle", None):
            load_library().pga_engine_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass


def terminals_to_numpy(out, n):
    return out[:n].cpu().numpy().reshape(-1).view(G.TERMINAL_DT).copy()
