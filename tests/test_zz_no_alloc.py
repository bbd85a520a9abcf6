"""pga_lbvh_build_static: the LBVH build for callers that cannot allocate.

Some callers of this library cannot allocate device memory when they need a
hierarchy -- their device-memory budget was handed out in full at start-up, or
the allocator belongs to the host application they run in.  The static entry
point takes only inputs and outputs and draws all of its scratch from a fixed
device array inside the library.  These tests make the start-up call (n = 0)
and then call it through the C ABI three times in a row (the array keeps the
previous call's contents; the last call at exactly the leaf limit) and
compare every output with pga_lbvh_build's, bit for bit -- the tolerance the
other LBVH tests use.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from operatorgraph_gb300 import scenes
from operatorgraph_gb300.engine import PgaBounds, PgaLbvh


def _bounds(b):
    b = np.asarray(b, np.float32)
    return PgaBounds((ctypes.c_float * 3)(*b[:3]), (ctypes.c_float * 3)(*b[3:]))


def test_static_rejects_too_many_leaves_without_a_gpu():
    from operatorgraph_gb300 import build as B
    from operatorgraph_gb300 import engine

    B.build()
    L = engine.load_library()
    dummy = ctypes.c_void_p(16)
    out = PgaLbvh(dummy, dummy, dummy, dummy, dummy)
    st = L.pga_lbvh_build_static(dummy, 65537, ctypes.byref(_bounds((0, 0, 0, 1, 1, 1))), ctypes.byref(out), None)
    assert st == 7
    assert b"65536" in L.pga_last_error()


@pytest.mark.gpu
def test_static_matches_engine_lbvh_twice_in_a_row():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from operatorgraph_gb300 import build as B
    from operatorgraph_gb300 import engine
    from operatorgraph_gb300.engine import Engine

    B.build()
    torch.cuda.set_device(0)
    L = engine.load_library()
    # the start-up call: n = 0 loads the module and looks the array up, nothing else
    assert L.pga_lbvh_build_static(None, 0, None, None, None) == 0, L.pga_last_error()
    cases = [(scenes.menger(0.05), (-0.5, -0.5, -0.5, 0.5, 0.5, 0.5)),
             (scenes.building(), (-20.0, -20.0, -1.0, 20.0, 20.0, 40.0)),
             ("limit", (-10.0, -10.0, -10.0, 10.0, 10.0, 10.0))]
    for b, bounds in cases:
        if isinstance(b, str):
            # exactly PGA_LBVH_STATIC_MAX_LEAVES synthetic records: the carve of
            # the fixed array (radix-sort temp included) must fit at the limit
            from operatorgraph_gb300 import grammar as G

            n = 65536
            rng = np.random.default_rng(11)
            rec = np.zeros(n, G.TERMINAL_DT)
            m = rng.uniform(-0.5, 0.5, (n, 12)).astype(np.float32)
            m[:, [3, 7, 11]] = rng.uniform(-9.0, 9.0, (n, 3)).astype(np.float32)
            m[: n // 4, [3, 7, 11]] = np.round(m[: n // 4, [3, 7, 11]])  # duplicate centres: ties
            rec["m"] = m
            rec["path"] = rng.permutation(np.arange(n, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15))
            out = torch.from_numpy(rec.view(np.uint8).copy()).cuda().view(n, 64)
            eng = Engine(scenes.menger(0.05)["entries"], node_capacity=1 << 16, max_terminals=1 << 17)
        else:
            eng = Engine(b["entries"], node_capacity=1 << 16, max_terminals=1 << 16)
            out, n, _ = eng.execute(b["axioms"], capacity=1 << 14)
        want = eng.lbvh(out, n, bounds)
        torch.cuda.synchronize()
        got = {
            "nodes": torch.empty((n - 1, 3), dtype=torch.int32, device="cuda"),
            "leafParents": torch.empty(n, dtype=torch.int32, device="cuda"),
            "aabbs": torch.empty((n - 1, 6), dtype=torch.float32, device="cuda"),
            "leafTerminal": torch.empty(n, dtype=torch.int32, device="cuda"),
            "keys": torch.empty(n, dtype=torch.int64, device="cuda"),
        }
        lb = PgaLbvh(got["nodes"].data_ptr(), got["leafParents"].data_ptr(), got["aabbs"].data_ptr(),
                     got["leafTerminal"].data_ptr(), got["keys"].data_ptr())
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        st = L.pga_lbvh_build_static(ctypes.c_void_p(out.data_ptr()), n, ctypes.byref(_bounds(bounds)),
                                     ctypes.byref(lb), stream)
        assert st == 0, L.pga_last_error()
        torch.cuda.synchronize()
        for k in want:
            a = want[k].cpu().numpy().view(np.uint32)
            c = got[k].cpu().numpy().view(np.uint32)
            assert np.array_equal(a, c), f"{k} differs from pga_lbvh_build"
        eng.release()
