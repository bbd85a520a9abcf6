"""The C-ABI library builds for sm_103a, loads and exports every declared symbol.

No GPU is needed: nothing here launches a kernel.
"""
import os
import re

import pytest

from operatorgraph_gb300 import build as B
from operatorgraph_gb300 import engine
from operatorgraph_gb300 import grammar as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "pga_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(pga_\w+)\(", text, re.M)))


@pytest.fixture(scope="module")
def lib():
    B.build()
    return engine.load_library()


def test_header_declares_the_abi():
    assert declared_symbols() == sorted(engine.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_version_and_default_procs(lib):
    import ctypes

    assert b"sm_103a" in lib.pga_version()
    n = ctypes.c_uint32()
    p = lib.pga_default_procs(ctypes.byref(n))
    assert n.value == len(G.DEFAULT_PROCS)
    for i in range(n.value):
        assert (p[i].op, p[i].shape, p[i].numChildren) == tuple(int(v) for v in G.DEFAULT_PROCS[i])[:3]


def test_struct_layouts_match_header():
    import ctypes

    assert ctypes.sizeof(engine.PgaEngineConfig) == 56
    assert ctypes.sizeof(engine.PgaDeriveReport) == 40
    assert G.ENTRY_DT.itemsize == 1332 and G.AXIOM_DT.itemsize == 48 and G.TERMINAL_DT.itemsize == 64


def test_null_arguments_rejected_without_gpu(lib):
    import ctypes

    h = ctypes.c_void_p()
    assert lib.pga_engine_create(None, None, ctypes.byref(h)) == 7
    assert b"null" in lib.pga_last_error()
