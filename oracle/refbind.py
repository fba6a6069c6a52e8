"""ctypes binding for oracle/_ref/libptlref.so -- the reference code generator built from
the reference's own sources by oracle/ref/Makefile.

Test infrastructure only: imported by tests and by the fixture script under
tests/golden/, never by the product.  The library exists only where the reference
tree is mounted and the host is x86-64 (the reference is written against AVX2).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libptlref.so")


def ref_root() -> str:
    """The reference source tree: $PTL_REFERENCE_ROOT, else the REF default of the build
    recipe (oracle/ref/Makefile), which is where the reference is mounted for the build."""
    env = os.environ.get("PTL_REFERENCE_ROOT")
    if env:
        return env
    res = subprocess.run(["make", "-s", "--no-print-directory", "-C", os.path.join(HERE, "ref"), "print-ref"],
                         capture_output=True, text=True)
    return res.stdout.strip() if res.returncode == 0 else ""


BUF_NAMES = [
    "out_words", "fn_start", "fn_end", "fn_size", "fn_id",
    "pre_type", "pre_rtype", "pre_data",
    "cnt_size", "cnt_loc", "cnt_fn_id", "cnt_fn_start", "cnt_fn_end", "cnt_fn_size",
    "gen_instr", "gen_rd", "gen_rs1", "gen_rs2", "gen_jt",
    "opt_used",
    "ra_instr", "ra_rd", "ra_rs1", "ra_rs2", "ra_jt", "ra_fn_start", "ra_fn_end", "ra_fn_size",
    "fj_instr", "fj_rd", "fj_rs1", "fj_rs2", "fj_jt", "fj_fn_start", "fj_fn_end", "fj_fn_size",
]
STAGES = ["preprocess", "isn_cnt", "isn_gen", "optimize", "regalloc", "fix_jumps", "postprocess"]


class _Tree(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_size_t), ("max_depth", ctypes.c_size_t),
        ("type", ctypes.POINTER(ctypes.c_uint8)), ("rtype", ctypes.POINTER(ctypes.c_uint8)),
        ("parent", ctypes.POINTER(ctypes.c_int32)), ("depth", ctypes.POINTER(ctypes.c_int32)),
        ("child_idx", ctypes.POINTER(ctypes.c_int32)), ("data", ctypes.POINTER(ctypes.c_uint32)),
    ]


class _Buf(ctypes.Structure):
    _fields_ = [("p", ctypes.POINTER(ctypes.c_uint32)), ("n", ctypes.c_size_t)]


class _Result(ctypes.Structure):
    _fields_ = [("bufs", _Buf * len(BUF_NAMES)), ("stage_ns", ctypes.c_uint64 * 7),
                ("threads_used", ctypes.c_int)]


@dataclass
class Ast:
    """A flattened post-order AST in the reference's DepthTree layout."""
    type: np.ndarray       # u8 Pareas NodeType
    rtype: np.ndarray      # u8 Pareas DataType
    parent: np.ndarray     # i32
    depth: np.ndarray      # i32
    child_idx: np.ndarray  # i32
    data: np.ndarray       # u32
    max_depth: int = 0

    @property
    def n(self) -> int:
        return int(self.type.shape[0])


@dataclass
class RefResult:
    bufs: dict = field(default_factory=dict)
    stage_ns: list = field(default_factory=list)
    threads_used: int = 1

    @property
    def words(self) -> np.ndarray:
        return self.bufs["out_words"]


_lib = None


def build(ref_root: str | None = None, quiet: bool = True) -> bool:
    """Compile the reference into oracle/_ref (make rebuilds only what changed; where the
    reference tree is absent an existing build is used as it is).

    Returns False where there is neither a build nor a reference tree on an x86-64 host."""
    ref_root = ref_root or ref_root_cached()
    if not ref_root or not os.path.isdir(ref_root) or os.uname().machine not in ("x86_64", "AMD64"):
        return os.path.exists(LIB_PATH)
    cmd = ["make", "-C", os.path.join(HERE, "ref"), f"REF={ref_root}", f"-j{os.cpu_count() or 4}"]
    res = subprocess.run(cmd, capture_output=quiet)
    return res.returncode == 0 and os.path.exists(LIB_PATH)


_root = None


def ref_root_cached() -> str:
    global _root
    if _root is None:
        _root = ref_root()
    return _root


def available() -> bool:
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        if not available():
            raise RuntimeError("reference oracle library not built: " + LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        L.ptlref_parse_file.argtypes = [ctypes.c_char_p, ctypes.POINTER(_Tree), ctypes.c_char_p, ctypes.c_size_t]
        L.ptlref_parse_file.restype = ctypes.c_int
        L.ptlref_free_tree.argtypes = [ctypes.POINTER(_Tree)]
        L.ptlref_compile.argtypes = [ctypes.POINTER(_Tree), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_uint32, ctypes.c_int, ctypes.POINTER(_Result),
                                     ctypes.c_char_p, ctypes.c_size_t]
        L.ptlref_compile.restype = ctypes.c_int
        L.ptlref_free_result.argtypes = [ctypes.POINTER(_Result)]
        L.ptlref_compile_scalar.argtypes = [ctypes.POINTER(_Tree), ctypes.c_int, ctypes.POINTER(_Result),
                                            ctypes.c_char_p, ctypes.c_size_t]
        L.ptlref_compile_scalar.restype = ctypes.c_int
        u8p, i32p, u32p = (ctypes.POINTER(ctypes.c_uint8), ctypes.POINTER(ctypes.c_int32),
                           ctypes.POINTER(ctypes.c_uint32))
        L.ptlref_flatten.argtypes = [ctypes.c_size_t, u8p, u8p, i32p, i32p, u32p, ctypes.POINTER(_Tree)]
        L.ptlref_flatten.restype = ctypes.c_int
        _lib = L
    return _lib


def _np(ptr, n, dtype):
    if n == 0:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


def parse_file(path: str) -> Ast:
    L = lib()
    t = _Tree()
    err = ctypes.create_string_buffer(1024)
    rc = L.ptlref_parse_file(path.encode(), ctypes.byref(t), err, 1024)
    if rc != 0:
        raise RuntimeError(f"reference front end failed on {path}: {err.value.decode()}")
    try:
        return Ast(type=_np(t.type, t.n, np.uint8), rtype=_np(t.rtype, t.n, np.uint8),
                   parent=_np(t.parent, t.n, np.int32), depth=_np(t.depth, t.n, np.int32),
                   child_idx=_np(t.child_idx, t.n, np.int32), data=_np(t.data, t.n, np.uint32),
                   max_depth=int(t.max_depth))
    finally:
        L.ptlref_free_tree(ctypes.byref(t))


def flatten(type_, rtype, parent, child_idx, data) -> Ast:
    """The reference's DepthTree constructor on the pointer tree (ASTNode) that a
    parent-pointer tree in any node order describes (one tree required)."""
    L = lib()
    a = [np.ascontiguousarray(type_, np.uint8), np.ascontiguousarray(rtype, np.uint8),
         np.ascontiguousarray(parent, np.int32), np.ascontiguousarray(child_idx, np.int32),
         np.ascontiguousarray(data, np.uint32)]
    p = lambda x, t: x.ctypes.data_as(ctypes.POINTER(t))
    t = _Tree()
    rc = L.ptlref_flatten(a[0].shape[0], p(a[0], ctypes.c_uint8), p(a[1], ctypes.c_uint8), p(a[2], ctypes.c_int32),
                          p(a[3], ctypes.c_int32), p(a[4], ctypes.c_uint32), ctypes.byref(t))
    if rc != 0:
        raise RuntimeError("reference flatten failed")
    try:
        return Ast(type=_np(t.type, t.n, np.uint8), rtype=_np(t.rtype, t.n, np.uint8),
                   parent=_np(t.parent, t.n, np.int32), depth=_np(t.depth, t.n, np.int32),
                   child_idx=_np(t.child_idx, t.n, np.int32), data=_np(t.data, t.n, np.uint32),
                   max_depth=int(t.max_depth))
    finally:
        L.ptlref_free_tree(ctypes.byref(t))


def compile_ast(ast: Ast, threads: int = 1, sync: int = 0, altblock: int = 0,
                mininstr: int = 0, snapshots: bool = False) -> RefResult:
    L = lib()
    keep = [np.ascontiguousarray(ast.type, np.uint8), np.ascontiguousarray(ast.rtype, np.uint8),
            np.ascontiguousarray(ast.parent, np.int32), np.ascontiguousarray(ast.depth, np.int32),
            np.ascontiguousarray(ast.child_idx, np.int32), np.ascontiguousarray(ast.data, np.uint32)]
    t = _Tree()
    t.n = ast.n
    t.max_depth = int(ast.max_depth)
    t.type = keep[0].ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
    t.rtype = keep[1].ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
    t.parent = keep[2].ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    t.depth = keep[3].ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    t.child_idx = keep[4].ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    t.data = keep[5].ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
    r = _Result()
    err = ctypes.create_string_buffer(1024)
    rc = L.ptlref_compile(ctypes.byref(t), threads, sync, altblock, mininstr, int(snapshots),
                          ctypes.byref(r), err, 1024)
    if rc != 0:
        raise RuntimeError("reference generator failed: " + err.value.decode())
    try:
        out = RefResult(stage_ns=list(r.stage_ns), threads_used=r.threads_used)
        for i, name in enumerate(BUF_NAMES):
            b = r.bufs[i]
            if b.p:
                out.bufs[name] = _np(b.p, b.n, np.uint32)
        return out
    finally:
        L.ptlref_free_result(ctypes.byref(r))


def compile_ast_scalar(ast: Ast, snapshots: bool = False) -> RefResult:
    """The reference's scalar generator (rv_generator_st, src/codegen/rv_generator.cpp:
    129-1736; the -s flag) on the tree, with the same snapshot names as compile_ast."""
    L = lib()
    keep = [np.ascontiguousarray(ast.type, np.uint8), np.ascontiguousarray(ast.rtype, np.uint8),
            np.ascontiguousarray(ast.parent, np.int32), np.ascontiguousarray(ast.depth, np.int32),
            np.ascontiguousarray(ast.child_idx, np.int32), np.ascontiguousarray(ast.data, np.uint32)]
    t = _Tree()
    t.n = ast.n
    t.max_depth = int(ast.max_depth)
    t.type = keep[0].ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
    t.rtype = keep[1].ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
    t.parent = keep[2].ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    t.depth = keep[3].ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    t.child_idx = keep[4].ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    t.data = keep[5].ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
    r = _Result()
    err = ctypes.create_string_buffer(1024)
    rc = L.ptlref_compile_scalar(ctypes.byref(t), int(snapshots), ctypes.byref(r), err, 1024)
    if rc != 0:
        raise RuntimeError("reference scalar generator failed: " + err.value.decode())
    try:
        out = RefResult(stage_ns=list(r.stage_ns), threads_used=1)
        for i, name in enumerate(BUF_NAMES):
            b = r.bufs[i]
            if b.p:
                out.bufs[name] = _np(b.p, b.n, np.uint32)
        return out
    finally:
        L.ptlref_free_result(ctypes.byref(r))


def to_asm(words) -> str:
    """The reference's rv_generator::to_asm text of the words."""
    L = lib()
    w = np.ascontiguousarray(words, np.uint32)
    fn = L.ptlref_to_asm
    fn.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t]
    fn.restype = ctypes.c_size_t
    n = fn(w.ctypes.data, w.shape[0], None, 0)
    buf = ctypes.create_string_buffer(n + 1)
    fn(w.ctypes.data, w.shape[0], buf, n)
    return buf.raw[:n].decode()


def disassemble(words, start_addr: int = 0, func_starts=()) -> str:
    """The reference's rvdisasm::disassemble listing of the words."""
    L = lib()
    w = np.ascontiguousarray(words, np.uint32)
    f = np.ascontiguousarray(func_starts, np.uint64)
    fn = L.ptlref_disassemble
    fn.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_size_t,
                   ctypes.c_char_p, ctypes.c_size_t]
    fn.restype = ctypes.c_size_t
    n = fn(w.ctypes.data, w.shape[0], start_addr, f.ctypes.data, f.shape[0], None, 0)
    buf = ctypes.create_string_buffer(n + 1)
    fn(w.ctypes.data, w.shape[0], start_addr, f.ctypes.data, f.shape[0], buf, n)
    return buf.raw[:n].decode()

