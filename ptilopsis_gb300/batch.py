"""Batched compilation and the compile server (ptl_batch_* / ptl_server_* of
include/ptl_codegen.h).

Neither exists in the reference, which compiles one tree per process.  A batch goes
through the batched pipeline (one launch per stage step for all its programs); the server
runs a pool of worker threads in libptl_gb300.so, each owning a generator with a resident
device arena and its own stream, so compiles overlap on the GPU.  Every program's output is
identical to compiling it alone.
"""
from __future__ import annotations

import ctypes
import json
import os
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

from .codegen import DepthTree, PtlError, _AstView, _view, device_info, lib

_u32p = ctypes.POINTER(ctypes.c_uint32)


def _bind(L):
    if getattr(L, "_ptl_batch_bound", False):
        return L
    vp, sz, u64 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint64
    L.ptl_batch_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp)]
    L.ptl_batch_compile.argtypes = [vp, ctypes.POINTER(_AstView), sz]
    L.ptl_batch_status.argtypes = [vp, sz]
    L.ptl_batch_words.argtypes = [vp, sz, ctypes.POINTER(_u32p), ctypes.POINTER(sz)]
    L.ptl_batch_function_table.argtypes = [vp, sz] + [ctypes.POINTER(_u32p)] * 4 + [ctypes.POINTER(sz)]
    L.ptl_batch_elapsed_ns.argtypes = [vp]
    L.ptl_batch_elapsed_ns.restype = u64
    L.ptl_batch_stage_ns.argtypes = [vp, ctypes.POINTER(u64)]
    L.ptl_batch_sizes.argtypes = [vp, sz, ctypes.POINTER(u64)]
    L.ptl_batch_host_ns.argtypes = [vp, ctypes.POINTER(u64)]
    L.ptl_batch_copied_bytes.argtypes = [vp, ctypes.POINTER(u64), ctypes.POINTER(u64)]
    L.ptl_batch_last_error.argtypes = [vp]
    L.ptl_batch_last_error.restype = ctypes.c_char_p
    L.ptl_batch_set_tiles.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32]
    L.ptl_batch_tiles.argtypes = [vp, ctypes.POINTER(ctypes.c_uint32)]
    L.ptl_batch_set_regalloc_share.argtypes = [vp, ctypes.c_double]
    L.ptl_batch_set_scalar.argtypes = [vp, ctypes.c_int]
    L.ptl_batch_device_ns.argtypes = [vp]
    L.ptl_batch_device_ns.restype = u64
    L.ptl_batch_depth_sort_ns.argtypes = [vp]
    L.ptl_batch_depth_sort_ns.restype = u64
    L.ptl_batch_destroy.argtypes = [vp]
    L.ptl_batch_destroy.restype = None
    L.ptl_server_create.argtypes = [ctypes.c_int, ctypes.c_int, u64, ctypes.POINTER(vp)]
    L.ptl_server_submit.argtypes = [vp, ctypes.POINTER(_AstView), ctypes.POINTER(u64)]
    L.ptl_server_submit_flags.argtypes = [vp, ctypes.POINTER(_AstView), ctypes.c_uint32, ctypes.POINTER(u64)]
    L.ptl_server_poll.argtypes = [vp, u64, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    L.ptl_server_result.argtypes = [vp, u64, ctypes.POINTER(_u32p), ctypes.POINTER(sz)] + \
        [ctypes.POINTER(_u32p)] * 4 + [ctypes.POINTER(sz)]
    L.ptl_server_times.argtypes = [vp, u64, ctypes.POINTER(u64)]
    L.ptl_server_release.argtypes = [vp, u64]
    L.ptl_server_error.argtypes = [vp, u64]
    L.ptl_server_error.restype = ctypes.c_char_p
    L.ptl_server_stats.argtypes = [vp, ctypes.POINTER(u64)]
    L.ptl_server_memory.argtypes = [vp, ctypes.POINTER(u64)]
    L.ptl_server_destroy.argtypes = [vp]
    L.ptl_server_destroy.restype = None
    L.ptl_clock_ns.argtypes = []
    L.ptl_clock_ns.restype = u64
    for fn in ("ptl_batch_create", "ptl_batch_compile", "ptl_batch_status", "ptl_batch_words", "ptl_batch_stage_ns",
               "ptl_batch_copied_bytes", "ptl_batch_sizes", "ptl_batch_host_ns", "ptl_batch_set_tiles", "ptl_batch_tiles",
               "ptl_batch_set_regalloc_share", "ptl_batch_set_scalar",
               "ptl_batch_function_table", "ptl_server_create", "ptl_server_submit", "ptl_server_submit_flags", "ptl_server_poll",
               "ptl_server_result", "ptl_server_times", "ptl_server_release", "ptl_server_stats", "ptl_server_memory"):
        getattr(L, fn).restype = ctypes.c_int
    L._ptl_batch_bound = True
    return L


def _arr(p, n) -> np.ndarray:
    if n == 0:
        return np.zeros(0, np.uint32)
    return np.ctypeslib.as_array(p, shape=(n,)).copy()


@dataclass
class Compiled:
    words: np.ndarray
    table: dict  # starts, ends, sizes, ids


def clock_ns() -> int:
    """The monotonic clock of the server's request times."""
    return int(_bind(lib()).ptl_clock_ns())


# ---- tile-size autotuning
ELEM_TILES = (1024, 2048, 4096, 8192)   # candidates for the element-wise stages
SWEEP_TILES = (512, 1024, 2048)         # candidates for the optimize sweeps


def autotune_cache_path() -> str:
    """Where tuned tile sizes are kept (PTL_AUTOTUNE_CACHE overrides)."""
    return os.environ.get("PTL_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "ptilopsis_gb300", "autotune.json"))


def _device_key(device: int) -> str:
    d = device_info(device) or {"name": "unknown", "sm_count": 0, "cc": (0, 0)}
    return f"{d['name']}|sm_{d['cc'][0]}{d['cc'][1]}|{d['sm_count']}SM"


def cached_tiles(device: int = 0) -> Optional[tuple]:
    """(element tile, sweep tile) tuned earlier for this device, or None."""
    try:
        with open(autotune_cache_path()) as f:
            e = json.load(f).get(_device_key(device))
        return (int(e["elem_tile"]), int(e["sweep_tile"])) if e else None
    except (OSError, ValueError, KeyError, TypeError):
        return None


def autotune(trees: Sequence[DepthTree], device: int = 0, workers: int = 8, reps: int = 2, save: bool = True) -> dict:
    """Chooses the tile sizes of the batched pipeline by measurement: the element-wise
    tile first (sweep tile at its default), then the sweep tile with that choice; each
    candidate is timed as the best of `reps` compiles of `trees` (device time of all
    stages, CUDA events).  With save, the choice is cached for this device."""
    def timed(b, e, w):
        b.set_tiles(e, w)
        best = None
        for _ in range(reps):
            b.compile(trees)
            t = sum(b.stage_ns()) / 1e6
            best = t if best is None else min(best, t)
        return best

    with BatchCompiler(device, workers, tiles=None) as b:
        b.compile(trees)  # arenas and code paths
        elem = {e: timed(b, e, 1024) for e in ELEM_TILES}
        e_best = min(elem, key=elem.get)
        sweep = {w: (elem[e_best] if w == 1024 else timed(b, e_best, w)) for w in SWEEP_TILES}
        w_best = min(sweep, key=sweep.get)
    out = {"elem_tile": e_best, "sweep_tile": w_best, "ms_by_elem_tile": elem, "ms_by_sweep_tile": sweep,
           "programs": len(trees), "nodes": int(sum(t.n for t in trees)), "device": _device_key(device)}
    if save:
        path = autotune_cache_path()
        try:
            with open(path) as f:
                table = json.load(f)
        except (OSError, ValueError):
            table = {}
        table[out["device"]] = {k: out[k] for k in ("elem_tile", "sweep_tile", "programs", "nodes")}
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            json.dump(table, f, indent=1)
    return out


class BatchCompiler:
    """Compiles many programs per call through the batched pipeline (one launch per stage
    step for the whole batch); `workers` host threads gather the inputs.  tiles: "cached"
    applies this device's autotuned tile sizes when there are some, None keeps the
    defaults, a pair (element tile, sweep tile) sets them."""

    def __init__(self, device: int = 0, workers: int = 8, tiles="cached", scalar: bool = False):
        self._lib = _bind(lib())
        self._h = ctypes.c_void_p()
        st = self._lib.ptl_batch_create(device, workers, ctypes.byref(self._h))
        if st != 0:
            raise PtlError(st, "ptl_batch_create")
        if scalar:
            self.set_scalar(True)
        choice = cached_tiles(device) if isinstance(tiles, str) and tiles == "cached" else tiles
        if choice:
            self.set_tiles(*choice)

    def set_tiles(self, elem_tile: int, sweep_tile: int) -> None:
        st = self._lib.ptl_batch_set_tiles(self._h, elem_tile, sweep_tile)
        if st != 0:
            raise PtlError(st, f"ptl_batch_set_tiles({elem_tile}, {sweep_tile})")

    def set_scalar(self, on: bool) -> None:
        """True: the following compiles give the scalar generator's output (the
        reference's -s, RvGenerator(scalar=True) one program at a time)."""
        st = self._lib.ptl_batch_set_scalar(self._h, 1 if on else 0)
        if st != 0:
            raise PtlError(st, "ptl_batch_set_scalar")

    def set_regalloc_share(self, share: float) -> None:
        """Part of the device's resident blocks the persistent register-allocation launch
        may take (default 1); less leaves room for batches compiled beside this one."""
        st = self._lib.ptl_batch_set_regalloc_share(self._h, float(share))
        if st != 0:
            raise PtlError(st, f"ptl_batch_set_regalloc_share({share})")

    def tiles(self) -> tuple:
        v = (ctypes.c_uint32 * 2)()
        self._lib.ptl_batch_tiles(self._h, v)
        return int(v[0]), int(v[1])

    def compile(self, trees: Sequence[DepthTree], check: bool = True) -> None:
        """Compiles the trees (host arrays); results via result(k).  With check=False a
        program's own failure is left to status(k)."""
        # the view array is kept while the same trees (with the same cached views) come back
        cached = getattr(self, "_views", None)
        if (cached is not None and len(cached[0]) == len(trees)
                and all(t.__dict__.get("_ptl_view") is e for t, e in zip(trees, cached[0]))):
            views = cached[1]
        else:
            keep: list = []
            views = (_AstView * len(trees))(*[_view(t, keep) for t in trees])
            self._views = (keep, views)
        self._n = len(trees)
        st = self._lib.ptl_batch_compile(self._h, views, len(trees))
        if st != 0 and (check or self._batch_failed()):
            raise PtlError(st, "ptl_batch_compile: " + (self._lib.ptl_batch_last_error(self._h) or b"").decode())

    def _batch_failed(self) -> bool:
        return bool(self._lib.ptl_batch_last_error(self._h))

    def status(self, k: int) -> int:
        return int(self._lib.ptl_batch_status(self._h, k))

    def stage_ns(self) -> list:
        ns = (ctypes.c_uint64 * 7)()
        self._lib.ptl_batch_stage_ns(self._h, ns)
        return list(ns)

    def device_ns(self) -> int:
        """Device time of the last compile from its inputs on the device to its outputs
        complete (before the output copy)."""
        return int(self._lib.ptl_batch_device_ns(self._h))

    def depth_sort_ns(self) -> int:
        """Device time of the last compile's depth sort (part of the isn_gen stage)."""
        return int(self._lib.ptl_batch_depth_sort_ns(self._h))

    def sizes(self, k: int) -> dict:
        """Program k's nodes and word counts after isn_gen, regalloc and fix_jumps."""
        v = (ctypes.c_uint64 * 4)()
        st = self._lib.ptl_batch_sizes(self._h, k, v)
        if st != 0:
            raise PtlError(st, f"ptl_batch_sizes({k})")
        return {"n": int(v[0]), "W": int(v[1]), "W2": int(v[2]), "W3": int(v[3])}

    def host_ns(self) -> dict:
        """Host-side parts of the last compile: input gather, input copy, output copy."""
        v = (ctypes.c_uint64 * 3)()
        self._lib.ptl_batch_host_ns(self._h, v)
        return {"gather_ns": int(v[0]), "h2d_ns": int(v[1]), "d2h_ns": int(v[2])}

    def copied_bytes(self) -> tuple:
        a, b = ctypes.c_uint64(), ctypes.c_uint64()
        self._lib.ptl_batch_copied_bytes(self._h, ctypes.byref(a), ctypes.byref(b))
        return int(a.value), int(b.value)

    def elapsed_ns(self) -> int:
        return int(self._lib.ptl_batch_elapsed_ns(self._h))

    def words(self, k: int) -> np.ndarray:
        p, n = _u32p(), ctypes.c_size_t()
        st = self._lib.ptl_batch_words(self._h, k, ctypes.byref(p), ctypes.byref(n))
        if st != 0:
            raise PtlError(st, f"ptl_batch_words({k})")
        return _arr(p, n.value)

    def function_table(self, k: int) -> dict:
        ptrs = [_u32p() for _ in range(4)]
        n = ctypes.c_size_t()
        st = self._lib.ptl_batch_function_table(self._h, k, *[ctypes.byref(p) for p in ptrs], ctypes.byref(n))
        if st != 0:
            raise PtlError(st, f"ptl_batch_function_table({k})")
        return {name: _arr(p, n.value) for name, p in zip(("starts", "ends", "sizes", "ids"), ptrs)}

    def result(self, k: int) -> Compiled:
        return Compiled(self.words(k), self.function_table(k))

    def close(self) -> None:
        if self._h:
            self._lib.ptl_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class CompileServer:
    """Continuous-batching compile server: `slots` batched-pipeline lanes, admission against
    a device-memory budget (bytes)."""

    def __init__(self, device: int = 0, slots: int = 2, memory_budget: int = 120 << 30):
        self._lib = _bind(lib())
        self._h = ctypes.c_void_p()
        self._held = {}  # ticket -> the arrays a borrowed request refers to
        st = self._lib.ptl_server_create(device, slots, memory_budget, ctypes.byref(self._h))
        if st != 0:
            raise PtlError(st, "ptl_server_create")

    def submit(self, tree: DepthTree, copy: bool = True, scalar: bool = False) -> int:
        """Queues a host tree.  copy=False lends the tree's arrays to the server instead of
        copying them (the server keeps a reference until release(ticket)); scalar=True asks
        for the scalar generator's output (the reference's -s)."""
        keep: list = []
        view = _view(tree, keep)
        t = ctypes.c_uint64()
        flags = (0 if copy else 1) | (2 if scalar else 0)
        st = self._lib.ptl_server_submit_flags(self._h, ctypes.byref(view), flags, ctypes.byref(t))
        if st != 0:
            raise PtlError(st, "ptl_server_submit")
        if not copy:
            self._held[int(t.value)] = keep
        return int(t.value)

    def poll(self, ticket: int, wait: bool = False) -> bool:
        done = ctypes.c_int()
        st = self._lib.ptl_server_poll(self._h, ticket, 1 if wait else 0, ctypes.byref(done))
        if st != 0:
            why = (self._lib.ptl_server_error(self._h, ticket) or b"").decode()
            raise PtlError(st, f"request {ticket}" + (f": {why}" if why else ""))
        return bool(done.value)

    def result(self, ticket: int) -> Compiled:
        self.poll(ticket, wait=True)
        p, n = _u32p(), ctypes.c_size_t()
        ptrs = [_u32p() for _ in range(4)]
        f = ctypes.c_size_t()
        st = self._lib.ptl_server_result(self._h, ticket, ctypes.byref(p), ctypes.byref(n),
                                         *[ctypes.byref(q) for q in ptrs], ctypes.byref(f))
        if st != 0:
            raise PtlError(st, f"request {ticket}")
        return Compiled(_arr(p, n.value), {name: _arr(q, f.value)
                                           for name, q in zip(("starts", "ends", "sizes", "ids"), ptrs)})

    def times(self, ticket: int) -> tuple:
        """(submitted, started, finished) in clock_ns() time."""
        t = (ctypes.c_uint64 * 3)()
        st = self._lib.ptl_server_times(self._h, ticket, t)
        if st != 0:
            raise PtlError(st, f"request {ticket}")
        return int(t[0]), int(t[1]), int(t[2])

    def release(self, ticket: int) -> None:
        if self._lib.ptl_server_release(self._h, ticket) == 0:
            self._held.pop(ticket, None)

    def stats(self) -> dict:
        s = (ctypes.c_uint64 * 5)()
        self._lib.ptl_server_stats(self._h, s)
        return {"completed": int(s[0]), "nodes": int(s[1]), "queued": int(s[2]), "bytes_in_flight": int(s[3]),
                "batches": int(s[4])}

    def memory(self) -> dict:
        """Device memory of the lanes: held (bytes their arenas hold now), charged (what
        admission counts now), peak_charged (largest charge after a compile), budget."""
        m = (ctypes.c_uint64 * 4)()
        self._lib.ptl_server_memory(self._h, m)
        return {"held": int(m[0]), "charged": int(m[1]), "peak_charged": int(m[2]), "budget": int(m[3])}

    def close(self) -> None:
        if self._h:
            self._lib.ptl_server_destroy(self._h)
            self._h = ctypes.c_void_p()
        self._held.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def shard_programs(sizes: Sequence[int], world: int) -> List[List[int]]:
    """Splits a set of independent programs over `world` GPUs by size: longest first,
    each to the GPU with the fewest nodes so far (ties to the lower rank).  Programs
    share nothing, so the shards need no exchange; every GPU compiles its own list, in
    the order given (ascending program index).  Deterministic, so every rank computes
    the same split without communicating."""
    if world < 1:
        raise ValueError("world must be at least 1")
    order = sorted(range(len(sizes)), key=lambda k: (-int(sizes[k]), k))
    load = [0] * world
    shards: List[List[int]] = [[] for _ in range(world)]
    for k in order:
        r = min(range(world), key=lambda i: (load[i], i))
        shards[r].append(k)
        load[r] += int(sizes[k])
    return [sorted(x) for x in shards]


def compile_many(trees: Sequence[DepthTree], device: int = 0, workers: int = 8) -> List[Compiled]:
    with BatchCompiler(device, workers) as b:
        b.compile(trees)
        return [b.result(k) for k in range(len(trees))]
