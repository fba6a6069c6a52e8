"""The C ABI library: it loads without a GPU and exports every entry point that
include/ptl_codegen.h declares; its code tables equal the reference's."""
from __future__ import annotations

import ctypes
import os
import re
import zlib

import numpy as np
import pytest

from conftest import ROOT, manifest


def declared_functions():
    with open(os.path.join(ROOT, "include", "ptl_codegen.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(ptl_[a-z_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built_cuda):
    from ptilopsis_gb300 import codegen
    lib = ctypes.CDLL(codegen.LIB_PATH)
    names = declared_functions()
    assert "ptl_generator_create" in names and len(names) >= 10
    for name in names:
        assert hasattr(lib, name), name


def test_code_tables_equal_reference(built_cuda):
    from ptilopsis_gb300 import code_table
    for w, (n, c) in manifest()["tables"].items():
        t = code_table(int(w))
        assert len(t) == n, w
        assert zlib.crc32(np.ascontiguousarray(t, np.uint32).tobytes()) == c, w


def test_no_cpu_fallback_without_library(monkeypatch, built_cuda):
    """Without the CUDA library the package refuses instead of computing on the CPU."""
    import pytest
    from ptilopsis_gb300 import codegen
    monkeypatch.setattr(codegen, "_lib", None)
    monkeypatch.setattr(codegen, "LIB_PATH", "/nonexistent/libptl_gb300.so")
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        codegen.lib()


def test_argument_checks_need_no_device(built_cuda):
    """Arguments the C ABI refuses before touching a device: status BAD_ARGUMENT (7)."""
    import ctypes
    import numpy as np
    from ptilopsis_gb300 import PtlError, depth_order
    from ptilopsis_gb300.codegen import lib
    with pytest.raises(PtlError) as e:
        depth_order(np.array([3, -1, 2], np.int32))  # keys are depths, never negative
    assert e.value.status == 7
    L = lib()
    assert L.ptl_depth_order(None, 4, None, 0) == 7
    count = ctypes.c_size_t()
    assert L.ptl_compile(None, 0, None, 0, ctypes.byref(count)) == 7
