"""ctypes binding for the oracle's CPU restatement (oracle/port, built into
oracle/_port/libptlport.so).

Test infrastructure only: imported by tests, __graft_entry__.smoke() and bench.py's
CPU-baseline leg, never by the product.  The restatement is plain C++ and builds on
any host, including the aarch64 GPU machines where the reference itself (AVX2) cannot.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from .refbind import Ast, BUF_NAMES, RefResult

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_port", "libptlport.so")

TABLE_NAMES = ["node_size", "has_instr", "has_output", "parent_arg_idx", "get_output",
               "instr", "instr_constant", "operand", "instr_jt", "pareas_to_rv"]


class _Buf(ctypes.Structure):
    _fields_ = [("p", ctypes.POINTER(ctypes.c_uint32)), ("n", ctypes.c_size_t)]


class _Result(ctypes.Structure):
    _fields_ = [("bufs", _Buf * len(BUF_NAMES)), ("stage_ns", ctypes.c_uint64 * 7)]


class PortError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


_lib = None


def build(quiet: bool = True) -> bool:
    src = os.path.join(HERE, "port")
    newest = max(os.path.getmtime(os.path.join(src, f)) for f in os.listdir(src))
    if os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest:
        return True
    res = subprocess.run(["make", "-C", src], capture_output=quiet)
    return res.returncode == 0 and os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) and not build():
            raise RuntimeError("oracle restatement could not be built: " + LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        u8p = ctypes.POINTER(ctypes.c_uint8)
        i32p = ctypes.POINTER(ctypes.c_int32)
        u32p = ctypes.POINTER(ctypes.c_uint32)
        L.ptlport_compile.argtypes = [u8p, u8p, i32p, i32p, i32p, u32p, ctypes.c_size_t, ctypes.c_size_t,
                                      ctypes.c_int, ctypes.POINTER(_Result), ctypes.c_char_p, ctypes.c_size_t]
        L.ptlport_compile.restype = ctypes.c_int
        L.ptlport_compile_scalar.argtypes = L.ptlport_compile.argtypes
        L.ptlport_compile_scalar.restype = ctypes.c_int
        L.ptlport_free_result.argtypes = [ctypes.POINTER(_Result)]
        L.ptlport_depth_sort.argtypes = [i32p, ctypes.c_size_t, u32p]
        L.ptlport_table.argtypes = [ctypes.c_int, u32p]
        L.ptlport_table.restype = ctypes.c_size_t
        L.ptlport_flatten.argtypes = [ctypes.c_size_t, u8p, u8p, i32p, i32p, u32p, u8p, u8p, i32p, i32p, i32p, u32p,
                                      i32p, ctypes.POINTER(ctypes.c_size_t)]
        L.ptlport_flatten.restype = ctypes.c_int
        _lib = L
    return _lib


def compile_ast(ast: Ast, snapshots: bool = False, scalar: bool = False) -> RefResult:
    """The restatement of rv_generator_avx (one worker thread), or with scalar=True of
    the scalar generator rv_generator_st (src/codegen/rv_generator.cpp:227-1736)."""
    L = lib()
    a = [np.ascontiguousarray(ast.type, np.uint8), np.ascontiguousarray(ast.rtype, np.uint8),
         np.ascontiguousarray(ast.parent, np.int32), np.ascontiguousarray(ast.depth, np.int32),
         np.ascontiguousarray(ast.child_idx, np.int32), np.ascontiguousarray(ast.data, np.uint32)]
    ptrs = [a[0].ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), a[1].ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
            a[2].ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), a[3].ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
            a[4].ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), a[5].ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))]
    r = _Result()
    err = ctypes.create_string_buffer(1024)
    fn = L.ptlport_compile_scalar if scalar else L.ptlport_compile
    rc = fn(*ptrs, ast.n, int(ast.max_depth), int(snapshots), ctypes.byref(r), err, 1024)
    if rc != 0:
        raise PortError(rc, "oracle restatement: " + err.value.decode())
    try:
        out = RefResult(stage_ns=list(r.stage_ns))
        for i, name in enumerate(BUF_NAMES):
            b = r.bufs[i]
            if b.p:
                out.bufs[name] = (np.ctypeslib.as_array(b.p, shape=(b.n,)).copy() if b.n
                                  else np.zeros(0, np.uint32))
        return out
    finally:
        L.ptlport_free_result(ctypes.byref(r))


def flatten(type_, rtype, parent, child_idx, data):
    """DepthTree construction (pareas-ast/src/codegen/depthtree.cpp:11-100) from a
    parent-pointer tree in any node order: returns (Ast in post-order, order) with
    order[v] = v's post-order index; raises PortError for arrays that are not one tree."""
    L = lib()
    a = [np.ascontiguousarray(type_, np.uint8), np.ascontiguousarray(rtype, np.uint8),
         np.ascontiguousarray(parent, np.int32), np.ascontiguousarray(child_idx, np.int32),
         np.ascontiguousarray(data, np.uint32)]
    n = a[0].shape[0]
    o = [np.empty(n, np.uint8), np.empty(n, np.uint8), np.empty(n, np.int32), np.empty(n, np.int32),
         np.empty(n, np.int32), np.empty(n, np.uint32)]
    order = np.empty(n, np.int32)
    md = ctypes.c_size_t(0)
    p = lambda x, t: x.ctypes.data_as(ctypes.POINTER(t))
    u8, i32, u32 = ctypes.c_uint8, ctypes.c_int32, ctypes.c_uint32
    rc = L.ptlport_flatten(n, p(a[0], u8), p(a[1], u8), p(a[2], i32), p(a[3], i32), p(a[4], u32),
                           p(o[0], u8), p(o[1], u8), p(o[2], i32), p(o[3], i32), p(o[4], i32), p(o[5], u32),
                           p(order, i32), ctypes.byref(md))
    if rc != 0:
        raise PortError(rc, "oracle flatten: the arrays are not one tree")
    return Ast(type=o[0], rtype=o[1], parent=o[2], depth=o[3], child_idx=o[4], data=o[5],
               max_depth=int(md.value)), order


def depth_sort(keys: np.ndarray) -> np.ndarray:
    """libstdc++ std::sort's permutation of iota(n) ordered by keys."""
    L = lib()
    k = np.ascontiguousarray(keys, np.int32)
    out = np.empty(k.shape[0], np.uint32)
    L.ptlport_depth_sort(k.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), k.shape[0],
                         out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
    return out


def table(which: int) -> np.ndarray:
    L = lib()
    n = L.ptlport_table(which, None)
    out = np.empty(n, np.uint32)
    L.ptlport_table(which, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
    return out
