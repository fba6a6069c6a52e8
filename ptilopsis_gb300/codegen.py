"""Python mirror of the reference code generator's interface, over the C ABI of
include/ptl_codegen.h (libptl_gb300.so).

The reference (TypeA2/Ptilopsis) is driven as

    DepthTree tree(ast);                                   // pareas-ast flattening
    rv_generator_avx gen(tree, threads, sync, altblock, mininstr);
    gen.process(profile);
    gen.get_instructions();  gen.to_binary(os);

(src/main.cpp:119-157).  Here:

    gen = RvGenerator(tree)          # tree: DepthTree of numpy arrays or CUDA tensors
    gen.process(profile=True)
    gen.get_instructions()           # np.uint32 words, identical to the reference's
    gen.to_binary(stream)

There is no CPU fallback: if the CUDA library is missing or no GPU is visible,
constructing a generator raises.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from typing import BinaryIO, Optional

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libptl_gb300.so")

# ptl_status (include/ptl_codegen.h)
STATUS = {0: "OK", 1: "INVALID_AST", 2: "UNSUPPORTED", 3: "OOM", 4: "ADMISSION_DENIED",
          5: "DEVICE_TIMEOUT", 6: "CUDA_ERROR", 7: "BAD_ARGUMENT"}

STAGES = ["preprocess", "isn_cnt", "isn_gen", "optimize", "regalloc", "fix_jumps", "postprocess"]

# Snapshot slots of ptl_generator_snapshot: the reference generator's arrays after each
# stage (same order as the oracle harness).  Slots the GPU pipeline does not keep
# (the intermediate fix_jumps arrays, fused with postprocess) are absent.
SNAPSHOTS = {
    "out_words": 0, "fn_start": 1, "fn_end": 2, "fn_size": 3, "fn_id": 4,
    "pre_type": 5, "pre_rtype": 6, "pre_data": 7,
    "cnt_size": 8, "cnt_loc": 9, "cnt_fn_id": 10, "cnt_fn_start": 11, "cnt_fn_end": 12, "cnt_fn_size": 13,
    "gen_instr": 14, "gen_rd": 15, "gen_rs1": 16, "gen_rs2": 17, "gen_jt": 18,
    "opt_used": 19,
    "ra_instr": 20, "ra_rd": 21, "ra_rs1": 22, "ra_rs2": 23, "ra_jt": 24,
    "ra_fn_start": 25, "ra_fn_end": 26, "ra_fn_size": 27,
    "depth_order_pos": 40, "registers": 41,
}


class PtlError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


@dataclass
class DepthTree:
    """The flattened AST of pareas-ast (subprojects/pareas-ast/include/codegen/
    depthtree.hpp:12-59): six parallel arrays in post-order, root last."""
    type: object        # u8 Pareas NodeType
    rtype: object       # u8 Pareas DataType
    parent: object      # i32
    depth: object       # i32
    child_idx: object   # i32
    data: object        # u32
    max_depth: int

    def __setattr__(self, name, value):
        # a replaced array or max_depth makes the cached C view (_view) stale
        self.__dict__.pop("_ptl_view", None)
        object.__setattr__(self, name, value)

    @property
    def n(self) -> int:
        return int(self.type.shape[0])

    @property
    def on_device(self) -> bool:
        return bool(getattr(self.type, "is_cuda", False))

    def to(self, device) -> "DepthTree":
        """Copy the arrays to a torch device (for device-resident compiles)."""
        import torch
        conv = {"type": torch.uint8, "rtype": torch.uint8, "parent": torch.int32,
                "depth": torch.int32, "child_idx": torch.int32, "data": torch.int32}
        out = {}
        for k, dt in conv.items():
            a = getattr(self, k)
            if isinstance(a, np.ndarray):
                a = torch.from_numpy(a.view(np.int32) if k == "data" else a)
            out[k] = a.to(device=device, dtype=dt).contiguous()
        return DepthTree(max_depth=self.max_depth, **out)

    def numpy(self) -> "DepthTree":
        def host(a, dt):
            if isinstance(a, np.ndarray):
                return np.ascontiguousarray(a, dt)
            return np.ascontiguousarray(a.cpu().numpy()).view(dt) if dt == np.uint32 else np.ascontiguousarray(a.cpu().numpy(), dt)
        return DepthTree(host(self.type, np.uint8), host(self.rtype, np.uint8), host(self.parent, np.int32),
                         host(self.depth, np.int32), host(self.child_idx, np.int32), host(self.data, np.uint32),
                         self.max_depth)

    def nbytes(self) -> int:
        return self.n * 18


class _AstView(ctypes.Structure):
    _fields_ = [("n", ctypes.c_size_t), ("max_depth", ctypes.c_size_t),
                ("type", ctypes.c_void_p), ("rtype", ctypes.c_void_p), ("parent", ctypes.c_void_p),
                ("depth", ctypes.c_void_p), ("child_idx", ctypes.c_void_p), ("data", ctypes.c_void_p),
                ("on_device", ctypes.c_int)]


_lib = None


def library_path() -> str:
    return LIB_PATH


def lib():
    """Load libptl_gb300.so; raises when it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"GB300 code generator library missing ({LIB_PATH}); run "
                               "ptilopsis_gb300.build.build_all() -- there is no CPU fallback")
        L = ctypes.CDLL(LIB_PATH)
        vp, sz, u32p = ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_uint32)
        L.ptl_generator_create.argtypes = [ctypes.POINTER(_AstView), ctypes.c_int, ctypes.POINTER(vp)]
        L.ptl_generator_create_scalar.argtypes = [ctypes.POINTER(_AstView), ctypes.c_int, ctypes.POINTER(vp)]
        L.ptl_generator_process.argtypes = [vp, ctypes.c_int]
        L.ptl_generator_upload.argtypes = [vp, ctypes.POINTER(_AstView)]
        L.ptl_kernel_launches.argtypes = []
        L.ptl_kernel_launches.restype = ctypes.c_uint64
        L.ptl_generator_instructions.argtypes = [vp, ctypes.POINTER(u32p), ctypes.POINTER(sz)]
        L.ptl_generator_copy_instructions.argtypes = [vp, u32p, sz, ctypes.POINTER(sz)]
        L.ptl_generator_device_instructions.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(sz)]
        L.ptl_generator_function_table.argtypes = [vp, ctypes.POINTER(u32p), ctypes.POINTER(u32p),
                                                   ctypes.POINTER(u32p), ctypes.POINTER(u32p), ctypes.POINTER(sz)]
        L.ptl_generator_stage_ns.argtypes = [vp, ctypes.POINTER(ctypes.c_uint64)]
        L.ptl_generator_last_error.argtypes = [vp]
        L.ptl_generator_last_error.restype = ctypes.c_char_p
        L.ptl_generator_destroy.argtypes = [vp]
        L.ptl_generator_destroy.restype = None
        L.ptl_generator_snapshot.argtypes = [vp, ctypes.c_int, u32p, sz, ctypes.POINTER(sz)]
        L.ptl_compile.argtypes = [ctypes.POINTER(_AstView), ctypes.c_int, u32p, sz, ctypes.POINTER(sz)]
        L.ptl_depth_order.argtypes = [ctypes.c_void_p, sz, ctypes.c_void_p, ctypes.c_int]
        L.ptl_depth_order.restype = ctypes.c_int
        L.ptl_code_table.argtypes = [ctypes.c_int, u32p]
        L.ptl_code_table.restype = ctypes.c_size_t
        L.ptl_device_info.argtypes = [ctypes.c_int, ctypes.c_char_p, sz, ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        for fn in ("ptl_generator_create", "ptl_generator_create_scalar", "ptl_generator_process", "ptl_generator_upload", "ptl_generator_instructions", "ptl_generator_copy_instructions",
                   "ptl_generator_device_instructions", "ptl_generator_function_table",
                   "ptl_generator_stage_ns", "ptl_generator_snapshot", "ptl_compile", "ptl_device_info"):
            getattr(L, fn).restype = ctypes.c_int
        _lib = L
    return _lib


def _ptr(a) -> int:
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()


_FIELDS = (("type", np.dtype(np.uint8)), ("rtype", np.dtype(np.uint8)), ("parent", np.dtype(np.int32)),
           ("depth", np.dtype(np.int32)), ("child_idx", np.dtype(np.int32)), ("data", np.dtype(np.uint32)))


def _view(tree: DepthTree, keep: list) -> _AstView:
    """The C view of a tree.  It is kept on the tree until one of its fields is assigned
    (DepthTree.__setattr__ drops it): a view holds pointers, not contents."""
    cached = tree.__dict__.get("_ptl_view")
    if cached is not None:
        keep.append(cached)
        return cached[1]
    arrs = (tree.type, tree.rtype, tree.parent, tree.depth, tree.child_idx, tree.data)
    on_dev = tree.on_device
    held, ptrs = [], []
    for a, (_, dt) in zip(arrs, _FIELDS):
        if on_dev:
            ptrs.append(a.data_ptr())
        else:
            if not (type(a) is np.ndarray and a.dtype == dt and a.flags.c_contiguous):
                a = np.ascontiguousarray(a, dt)
            ptrs.append(a.__array_interface__["data"][0])
        held.append(a)
    v = _AstView(int(arrs[0].shape[0]), int(tree.max_depth), *ptrs, 1 if on_dev else 0)
    entry = (arrs, v, tree.max_depth, held)
    tree.__dict__["_ptl_view"] = entry
    keep.append(entry)
    return v


def code_table(which: int) -> np.ndarray:
    """The generator's code tables in the reference's flat layouts (ptl_code_table)."""
    L = lib()
    n = L.ptl_code_table(which, None)
    out = np.empty(n, np.uint32)
    L.ptl_code_table(which, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
    return out


class RvGenerator:
    """GPU counterpart of rv_generator_avx (include/codegen/rv_generator_avx.hpp:26-148);
    with scalar=True, of the single-threaded rv_generator_st (include/codegen/
    rv_generator.hpp:82-100, the -s flag of src/main.cpp), whose output differs."""

    def __init__(self, tree: DepthTree, device: int = 0, scalar: bool = False):
        self._lib = lib()
        self._h = ctypes.c_void_p()
        keep: list = []
        view = _view(tree, keep)
        create = self._lib.ptl_generator_create_scalar if scalar else self._lib.ptl_generator_create
        st = create(ctypes.byref(view), device, ctypes.byref(self._h))
        if st != 0:
            raise PtlError(st, "ptl_generator_create_scalar" if scalar else "ptl_generator_create")
        self.n = tree.n
        self.scalar = scalar

    def _check(self, st: int, what: str) -> None:
        if st != 0:
            msg = self._lib.ptl_generator_last_error(self._h)
            raise PtlError(st, f"{what}: {msg.decode() if msg else ''}")

    def upload(self, tree: DepthTree) -> None:
        """Rebinds the generator to another tree, reusing its device memory."""
        keep: list = []
        view = _view(tree, keep)
        self._check(self._lib.ptl_generator_upload(self._h, ctypes.byref(view)), "upload")
        self.n = tree.n

    def process(self, profile: bool = False, to_host: bool = True, row0_hash: bool = False,
                serial: bool = False) -> None:
        """rv_generator_avx::process.  to_host=False leaves the words on the device;
        row0_hash=True takes the register allocator's general row-0 lookup, serial=True
        the scalar generator's serial register allocation (both: same output)."""
        flags = (1 if profile else 0) | (0 if to_host else 2) | (4 if row0_hash else 0) | (8 if serial else 0)
        self._check(self._lib.ptl_generator_process(self._h, flags), "process")

    def get_instructions(self) -> np.ndarray:
        # A copy of the generator's host words.  (Fetching from the device straight into a
        # new array was slower: the device's stores fault the new array's pages in one by
        # one, while the generator's buffer keeps its pages from call to call.)
        p = ctypes.POINTER(ctypes.c_uint32)()
        n = ctypes.c_size_t()
        self._check(self._lib.ptl_generator_instructions(self._h, ctypes.byref(p), ctypes.byref(n)), "instructions")
        if n.value == 0:
            return np.zeros(0, np.uint32)
        return np.ctypeslib.as_array(p, shape=(n.value,)).copy()

    def device_instructions(self):
        """(device pointer, count) of the output words."""
        p = ctypes.c_void_p()
        n = ctypes.c_size_t()
        self._check(self._lib.ptl_generator_device_instructions(self._h, ctypes.byref(p), ctypes.byref(n)), "device words")
        return p.value, n.value

    def function_table(self) -> dict:
        ptrs = [ctypes.POINTER(ctypes.c_uint32)() for _ in range(4)]
        n = ctypes.c_size_t()
        self._check(self._lib.ptl_generator_function_table(self._h, *[ctypes.byref(p) for p in ptrs], ctypes.byref(n)),
                    "function table")
        names = ["starts", "ends", "sizes", "ids"]
        return {k: (np.ctypeslib.as_array(p, shape=(n.value,)).copy() if n.value else np.zeros(0, np.uint32))
                for k, p in zip(names, ptrs)}

    def stage_ns(self) -> list:
        ns = (ctypes.c_uint64 * 7)()
        self._check(self._lib.ptl_generator_stage_ns(self._h, ns), "stage_ns")
        return list(ns)

    def snapshot(self, name: str) -> np.ndarray:
        which = SNAPSHOTS[name]
        n = ctypes.c_size_t()
        self._check(self._lib.ptl_generator_snapshot(self._h, which, None, 0, ctypes.byref(n)), "snapshot size")
        out = np.empty(n.value, np.uint32)
        if n.value:
            self._check(self._lib.ptl_generator_snapshot(self._h, which, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                                         n.value, ctypes.byref(n)), "snapshot")
        return out

    def to_binary(self, stream: BinaryIO) -> None:
        """rv_generator::to_binary (src/codegen/rv_generator.cpp:116-119): raw
        little-endian 32-bit words."""
        stream.write(self.get_instructions().astype("<u4").tobytes())

    def to_asm(self) -> str:
        """rv_generator::to_asm (src/codegen/rv_generator.cpp:121-127): one line per word."""
        return to_asm(self.get_instructions())

    def to_elf(self) -> bytes:
        """The words and function table as an ELF64 RISC-V relocatable object
        (ptl_write_elf; the reference writes raw words only)."""
        t = self.function_table()
        return to_elf(self.get_instructions(), t["starts"], t["ends"])

    def close(self) -> None:
        if self._h:
            self._lib.ptl_generator_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def compile_tree(tree: DepthTree, device: int = 0, profile: bool = False, scalar: bool = False) -> np.ndarray:
    with RvGenerator(tree, device, scalar=scalar) as gen:
        gen.process(profile=profile)
        return gen.get_instructions()


def depth_order(keys, device: int = 0) -> np.ndarray:
    """isn_gen's depth order on its own (ptl_depth_order): pos[i] is i's position in
    libstdc++'s std::sort of iota(n) by keys (non-negative), from the GPU's emulation."""
    k = np.ascontiguousarray(keys, np.int32)
    pos = np.empty(k.shape[0], np.uint32)
    st = lib().ptl_depth_order(k.ctypes.data, k.shape[0], pos.ctypes.data, device)
    if st != 0:
        raise PtlError(st, "ptl_depth_order")
    return pos


def kernel_launches() -> int:
    """Kernel launches issued by the library so far in this process."""
    return int(lib().ptl_kernel_launches())


def device_info(device: int = 0) -> Optional[dict]:
    L = lib()
    name = ctypes.create_string_buffer(256)
    sm, ma, mi = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    if L.ptl_device_info(device, name, 256, ctypes.byref(sm), ctypes.byref(ma), ctypes.byref(mi)) != 0:
        return None
    return {"name": name.value.decode(), "sm_count": sm.value, "cc": (ma.value, mi.value)}


def _text(fn, *args) -> str:
    n = ctypes.c_size_t()
    st = fn(*args, None, 0, ctypes.byref(n))
    if st != 0:
        raise PtlError(st, fn.__name__)
    buf = ctypes.create_string_buffer(n.value + 1)
    st = fn(*args, buf, n.value, ctypes.byref(n))
    if st != 0:
        raise PtlError(st, fn.__name__)
    return buf.raw[:n.value].decode()


def to_asm(words) -> str:
    """The words as RISC-V assembly, one instruction per line (ptl_to_asm)."""
    L = lib()
    w = np.ascontiguousarray(words, np.uint32)
    L.ptl_to_asm.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t,
                             ctypes.POINTER(ctypes.c_size_t)]
    L.ptl_to_asm.restype = ctypes.c_int
    return _text(L.ptl_to_asm, w.ctypes.data, w.shape[0])


def disassemble(words, start_addr: int = 0, func_starts=()) -> str:
    """The coloured listing of the words with indices, addresses, bytes and function
    labels at the word indices in func_starts (ptl_disassemble)."""
    L = lib()
    w = np.ascontiguousarray(words, np.uint32)
    f = np.ascontiguousarray(func_starts, np.uint64)
    L.ptl_disassemble.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint64, ctypes.c_void_p,
                                  ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
    L.ptl_disassemble.restype = ctypes.c_int
    return _text(L.ptl_disassemble, w.ctypes.data, w.shape[0], start_addr, f.ctypes.data, f.shape[0])


def to_elf(words, func_starts, func_ends) -> bytes:
    """An ELF64 little-endian RISC-V relocatable object: .text holds the words, and
    function k of the table (starts/ends in words, address order) is the global
    function symbol "func<k>" (ptl_write_elf)."""
    L = lib()
    w = np.ascontiguousarray(words, np.uint32)
    s = np.ascontiguousarray(func_starts, np.uint32)
    e = np.ascontiguousarray(func_ends, np.uint32)
    if s.shape != e.shape:
        raise ValueError("func_starts and func_ends differ in length")
    vp = ctypes.c_void_p
    L.ptl_write_elf.argtypes = [vp, ctypes.c_size_t, vp, vp, ctypes.c_size_t, vp, ctypes.c_size_t,
                                ctypes.POINTER(ctypes.c_size_t)]
    L.ptl_write_elf.restype = ctypes.c_int
    n = ctypes.c_size_t()
    args = (w.ctypes.data, w.shape[0], s.ctypes.data, e.ctypes.data, s.shape[0])
    st = L.ptl_write_elf(*args, None, 0, ctypes.byref(n))
    if st != 0:
        raise PtlError(st, "ptl_write_elf")
    buf = (ctypes.c_uint8 * max(n.value, 1))()
    st = L.ptl_write_elf(*args, ctypes.addressof(buf), n.value, ctypes.byref(n))
    if st != 0:
        raise PtlError(st, "ptl_write_elf")
    return bytes(buf)[:n.value]


class _TreeView(ctypes.Structure):
    _fields_ = [("n", ctypes.c_size_t), ("type", ctypes.c_void_p), ("rtype", ctypes.c_void_p),
                ("parent", ctypes.c_void_p), ("child_idx", ctypes.c_void_p), ("data", ctypes.c_void_p),
                ("on_device", ctypes.c_int)]


class _TreeOut(ctypes.Structure):
    _fields_ = [("type", ctypes.c_void_p), ("rtype", ctypes.c_void_p), ("parent", ctypes.c_void_p),
                ("depth", ctypes.c_void_p), ("child_idx", ctypes.c_void_p), ("data", ctypes.c_void_p),
                ("order", ctypes.c_void_p), ("max_depth", ctypes.c_size_t), ("on_device", ctypes.c_int)]


def flatten(type_, rtype, parent, child_idx, data, device: int = 0):
    """The DepthTree of a parent-pointer tree given in any node order (ptl_flatten on the
    GPU; the reference builds it from its pointer tree, pareas-ast/src/codegen/
    depthtree.cpp:11-100).  parent[v] is -1 for the root; child_idx[v] is v's place among
    its parent's children.  Returns (DepthTree in post-order, order) with order[v] = v's
    post-order index; raises PtlError (INVALID_AST) for arrays that are not one tree.
    With CUDA tensors in, the result stays on their device (a DepthTree of CUDA tensors
    that RvGenerator compiles without a host round trip)."""
    L = lib()
    L.ptl_flatten.argtypes = [ctypes.POINTER(_TreeView), ctypes.POINTER(_TreeOut), ctypes.c_int, ctypes.c_void_p]
    L.ptl_flatten.restype = ctypes.c_int
    if getattr(type_, "is_cuda", False):
        return _flatten_device(L, type_, rtype, parent, child_idx, data)
    a = [np.ascontiguousarray(type_, np.uint8), np.ascontiguousarray(rtype, np.uint8),
         np.ascontiguousarray(parent, np.int32), np.ascontiguousarray(child_idx, np.int32),
         np.ascontiguousarray(data, np.uint32)]
    n = a[0].shape[0]
    if any(x.shape[0] != n for x in a):
        raise ValueError("the five arrays must have one length")
    o = [np.empty(n, np.uint8), np.empty(n, np.uint8), np.empty(n, np.int32), np.empty(n, np.int32),
         np.empty(n, np.int32), np.empty(n, np.uint32), np.empty(n, np.int32)]
    v = _TreeView(n, *(x.ctypes.data for x in a), 0)
    r = _TreeOut(*(x.ctypes.data for x in o), 0, 0)
    st = L.ptl_flatten(ctypes.byref(v), ctypes.byref(r), device, None)
    if st != 0:
        raise PtlError(st, "ptl_flatten: the arrays are not one tree" if st == 1 else "ptl_flatten")
    tree = DepthTree(type=o[0], rtype=o[1], parent=o[2], depth=o[3], child_idx=o[4], data=o[5],
                     max_depth=int(r.max_depth))
    return tree, o[6]


def _flatten_device(L, type_, rtype, parent, child_idx, data):
    import torch
    dev = type_.device
    a = [type_.to(torch.uint8).contiguous(), rtype.to(dev, torch.uint8).contiguous(),
         parent.to(dev, torch.int32).contiguous(), child_idx.to(dev, torch.int32).contiguous(),
         (data.view(torch.int32) if data.dtype == torch.uint32 else data.to(dev, torch.int32)).contiguous()]
    n = int(a[0].shape[0])
    if any(int(x.shape[0]) != n for x in a):
        raise ValueError("the five arrays must have one length")
    dts = (torch.uint8, torch.uint8, torch.int32, torch.int32, torch.int32, torch.int32, torch.int32)
    o = [torch.empty(n, dtype=dt, device=dev) for dt in dts]
    v = _TreeView(n, *(x.data_ptr() for x in a), 1)
    r = _TreeOut(*(x.data_ptr() for x in o), 0, 1)
    stream = torch.cuda.current_stream(dev).cuda_stream
    st = L.ptl_flatten(ctypes.byref(v), ctypes.byref(r), dev.index or 0, ctypes.c_void_p(stream))
    if st != 0:
        raise PtlError(st, "ptl_flatten: the arrays are not one tree" if st == 1 else "ptl_flatten")
    tree = DepthTree(type=o[0], rtype=o[1], parent=o[2], depth=o[3], child_idx=o[4], data=o[5],
                     max_depth=int(r.max_depth))
    return tree, o[6]
