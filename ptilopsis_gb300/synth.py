"""Seeded synthetic Pareas programs (libptlsynth.so, csrc/synth/ptl_synth.h).

Workload presets follow the benchmark configurations of this project:

  c0  one small program: 16 functions, ~20k nodes, expression depth <= 6, 30% float
  c1  one large program: 2,048 functions, lognormal body sizes (median 1k nodes,
      sigma 1.5) clipped to ~4M nodes in total, nesting <= 64, a quarter of the
      functions holding more than 31 live values at once
  c2  one huge program: 32,768 functions, lognormal (median 1.5k, sigma 1.2) clipped
      to ~64M nodes, expression depth <= 12, 50% float
  c3  4,096 independent programs, 1k..500k nodes each (lognormal, about 258M nodes in
      total), 4..512 functions
  c4  compile requests for the server: 80% U[1k, 10k] nodes, 20% lognormal in
      [100k, 2M]

Seeds: 0x50544C00 + config index; program k of c3 uses seed ^ k.
"""
from __future__ import annotations

import ctypes
import math
import os
from dataclasses import dataclass, fields

import numpy as np

from .codegen import DepthTree

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libptlsynth.so")

SEEDS = {"c0": 0x50544C00, "c1": 0x50544C01, "c2": 0x50544C02, "c3": 0x50544C03, "c4": 0x50544C04}


class _Params(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_uint64), ("n_functions", ctypes.c_uint32),
                ("median_fn_nodes", ctypes.c_double), ("sigma", ctypes.c_double),
                ("min_fn_nodes", ctypes.c_uint32), ("max_fn_nodes", ctypes.c_uint32),
                ("max_expr_depth", ctypes.c_uint32), ("float_frac", ctypes.c_double),
                ("max_nesting", ctypes.c_uint32), ("spill_frac", ctypes.c_double),
                ("emit_source", ctypes.c_int)]


class _Prog(ctypes.Structure):
    _fields_ = [("n", ctypes.c_size_t), ("max_depth", ctypes.c_size_t),
                ("type", ctypes.POINTER(ctypes.c_uint8)), ("rtype", ctypes.POINTER(ctypes.c_uint8)),
                ("parent", ctypes.POINTER(ctypes.c_int32)), ("depth", ctypes.POINTER(ctypes.c_int32)),
                ("child_idx", ctypes.POINTER(ctypes.c_int32)), ("data", ctypes.POINTER(ctypes.c_uint32)),
                ("source", ctypes.c_char_p), ("source_len", ctypes.c_size_t)]


@dataclass
class SynthParams:
    seed: int = SEEDS["c0"]
    n_functions: int = 16
    median_fn_nodes: float = 1250.0
    sigma: float = 0.0
    min_fn_nodes: int = 16
    max_fn_nodes: int = 0
    max_expr_depth: int = 6
    float_frac: float = 0.30
    max_nesting: int = 8
    spill_frac: float = 0.0
    emit_source: bool = False


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"synthetic generator library missing ({LIB_PATH}); run ptilopsis_gb300.build.build_all()")
        L = ctypes.CDLL(LIB_PATH)
        L.ptl_synth_generate.argtypes = [ctypes.POINTER(_Params), ctypes.POINTER(_Prog)]
        L.ptl_synth_generate.restype = ctypes.c_int
        L.ptl_synth_free.argtypes = [ctypes.POINTER(_Prog)]
        L.ptl_synth_free.restype = None
        _lib = L
    return _lib


def generate(params: SynthParams, with_source: bool = False):
    """Returns a DepthTree (and the source text when with_source)."""
    L = lib()
    p = _Params()
    for f in fields(SynthParams):
        v = getattr(params, f.name)
        setattr(p, f.name, int(v) if isinstance(v, bool) else v)
    p.emit_source = 1 if (with_source or params.emit_source) else 0
    out = _Prog()
    if L.ptl_synth_generate(ctypes.byref(p), ctypes.byref(out)) != 0:
        raise RuntimeError("synthetic generator failed")
    try:
        n = out.n

        def arr(ptr, dt):
            return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dt, copy=True)

        tree = DepthTree(arr(out.type, np.uint8), arr(out.rtype, np.uint8), arr(out.parent, np.int32),
                         arr(out.depth, np.int32), arr(out.child_idx, np.int32), arr(out.data, np.uint32),
                         int(out.max_depth))
        src = out.source.decode() if (p.emit_source and out.source) else None
    finally:
        L.ptl_synth_free(ctypes.byref(out))
    return (tree, src) if with_source else tree


def config_params(name: str, scale: float = 1.0, program: int = 0) -> SynthParams:
    """Parameters of a preset; scale < 1 shrinks the function count (tests)."""
    seed = SEEDS[name]
    if name == "c0":
        return SynthParams(seed=seed)
    if name == "c1":
        return SynthParams(seed=seed, n_functions=max(8, int(2048 * scale)), median_fn_nodes=1000.0, sigma=1.5,
                           max_fn_nodes=7000, max_nesting=64, spill_frac=0.25)
    if name == "c2":
        return SynthParams(seed=seed, n_functions=max(8, int(32768 * scale)), median_fn_nodes=1500.0, sigma=1.2,
                           max_fn_nodes=4000, max_expr_depth=12, float_frac=0.5, max_nesting=64)
    if name == "c3":
        # program k: total size lognormal (median 22k nodes, sigma 1.6) clipped to [1k, 500k]
        # -- a mean of about 63k, 258M nodes over 4,096 programs -- in 4..512 functions whose
        # sizes are lognormal (sigma 0.5) with that mean
        rng = np.random.default_rng(seed ^ program)
        total = float(np.clip(np.exp(math.log(22000.0) + 1.6 * rng.standard_normal()), 1000, 500000))
        nf = int(np.clip(total / 600.0, 4, 512))
        return SynthParams(seed=seed ^ program, n_functions=nf, median_fn_nodes=total / nf / math.exp(0.125),
                           sigma=0.5, max_nesting=32)
    if name == "c4":
        rng = np.random.default_rng(seed ^ program)
        if rng.random() < 0.8:
            total = float(rng.uniform(1000, 10000))
        else:
            total = float(np.clip(np.exp(math.log(300000.0) + 0.8 * rng.standard_normal()), 100000, 2000000))
        nf = int(np.clip(total / 800.0, 2, 1024))
        return SynthParams(seed=seed ^ program, n_functions=nf, median_fn_nodes=total / nf, sigma=0.6,
                           max_nesting=32)
    raise KeyError(name)


def config_tree(name: str, scale: float = 1.0, program: int = 0) -> DepthTree:
    return generate(config_params(name, scale, program))
