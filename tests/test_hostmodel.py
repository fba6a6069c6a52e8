"""The GPU algorithm, run on the CPU through the host model build of the same stage
functions, against the oracle -- stage by stage.  This is the CPU-side check of the
parallel formulations (depth-order emulation, priority writes, in-place optimize
fixpoint, lock-step lane-0 register allocation, serial path) before they run on a GPU."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import load_fixture, manifest, tree_to_ast

SLOTS = {"out_words": 0, "fn_start": 1, "fn_end": 2, "fn_size": 3, "fn_id": 4, "pre_type": 5, "pre_rtype": 6,
         "pre_data": 7, "cnt_size": 8, "cnt_loc": 9, "cnt_fn_id": 10, "cnt_fn_start": 11, "cnt_fn_end": 12,
         "cnt_fn_size": 13, "gen_instr": 14, "gen_rd": 15, "gen_rs1": 16, "gen_rs2": 17, "gen_jt": 18,
         "opt_used": 19, "ra_instr": 20, "ra_rd": 21, "ra_rs1": 22, "ra_rs2": 23, "ra_jt": 24,
         "ra_fn_start": 25, "ra_fn_end": 26, "ra_fn_size": 27}


class _Buf(ctypes.Structure):
    _fields_ = [("p", ctypes.POINTER(ctypes.c_uint32)), ("n", ctypes.c_size_t)]


_hm = None


def hostmodel():
    global _hm
    if _hm is None:
        from ptilopsis_gb300 import build as b
        L = ctypes.CDLL(b.build_hostmodel())
        L.ptlhm_compile.restype = ctypes.c_int
        L.ptlhm_compile_mode.restype = ctypes.c_int
        L.ptlhm_set_scalar_serial.argtypes = [ctypes.c_int]
        L.ptlhm_set_scalar_serial.restype = None
        L.ptlhm_depth_sort.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
        L.ptlhm_depth_sort.restype = None
        _hm = L
    return _hm


def hm_compile(ast):
    L = hostmodel()
    nb = 48
    bufs = (_Buf * nb)()
    err = (ctypes.c_uint32 * 3)()
    arrs = [np.ascontiguousarray(ast.type, np.uint8), np.ascontiguousarray(ast.rtype, np.uint8),
            np.ascontiguousarray(ast.parent, np.int32), np.ascontiguousarray(ast.depth, np.int32),
            np.ascontiguousarray(ast.child_idx, np.int32), np.ascontiguousarray(ast.data, np.uint32)]
    rc = L.ptlhm_compile(*[ctypes.c_void_p(a.ctypes.data) for a in arrs], ctypes.c_size_t(ast.n),
                         ctypes.c_size_t(ast.max_depth), bufs, nb, err)
    out = {}
    for k in range(nb):
        if bufs[k].p:
            out[k] = np.ctypeslib.as_array(bufs[k].p, shape=(bufs[k].n,)).copy() if bufs[k].n else np.zeros(0, np.uint32)
    L.ptlhm_free(bufs, nb)
    return rc, list(err), out


def assert_stages_equal(ast):
    from oracle import portbind
    ref = portbind.compile_ast(ast, snapshots=True)
    rc, err, got = hm_compile(ast)
    assert rc == 0, f"host model error {err}"
    for name, slot in SLOTS.items():
        np.testing.assert_array_equal(got[slot], ref.bufs[name], err_msg=name)


@pytest.mark.parametrize("fx", [f["name"] for f in manifest()["fixtures"]])
def test_hostmodel_fixture(built, fx):
    ast, _ = load_fixture(fx)
    assert_stages_equal(ast)


@pytest.mark.parametrize("seed", [0x50544C00, 0x50544C20, 0x50544C21])
def test_hostmodel_synthetic_c0(built, seed):
    from ptilopsis_gb300.synth import SynthParams, generate
    assert_stages_equal(tree_to_ast(generate(SynthParams(seed=seed))))


def test_hostmodel_spilling_program(built):
    """Lognormal bodies, deep nesting and >31-live chains (the large-program shape)."""
    from ptilopsis_gb300.synth import config_params, generate
    assert_stages_equal(tree_to_ast(generate(config_params("c1", scale=24 / 2048))))


def test_hostmodel_many_small_functions(built):
    """Hundreds of functions: many groups of 8, lane-0 chains interleaved."""
    from ptilopsis_gb300.synth import SynthParams, generate
    tree = generate(SynthParams(seed=0x50544C30, n_functions=300, median_fn_nodes=60.0, sigma=0.9, max_nesting=6))
    assert_stages_equal(tree_to_ast(tree))


def test_hostmodel_float_heavy(built):
    from ptilopsis_gb300.synth import SynthParams, generate
    tree = generate(SynthParams(seed=0x50544C31, n_functions=40, median_fn_nodes=500.0, sigma=1.0,
                                max_expr_depth=12, float_frac=0.5))
    assert_stages_equal(tree_to_ast(tree))


@pytest.mark.parametrize("mode", ["random", "sorted", "reversed", "periodic", "few"])
def test_depth_order_emulation_equals_std_sort(built, mode):
    from oracle import portbind
    L = hostmodel()
    rng = np.random.default_rng(hash(mode) & 0xFFFF)
    for case in range(48):
        # up to 8,192 keys one block sorts the array; above, partition rounds come first
        n = int(rng.integers(1, 6000)) if case < 40 else int(rng.integers(8193, 80000))
        kmax = int(rng.integers(1, 80))
        if mode == "random":
            keys = rng.integers(0, kmax, n)
        elif mode == "sorted":
            keys = np.sort(rng.integers(0, kmax, n))
        elif mode == "reversed":
            keys = np.sort(rng.integers(0, kmax, n))[::-1]
        elif mode == "periodic":
            keys = np.arange(n) % kmax
        else:
            keys = rng.integers(0, 2, n)
        keys = np.ascontiguousarray(keys, np.int32)
        want = portbind.depth_sort(keys)
        got = np.empty(n, np.uint32)
        L.ptlhm_depth_sort(keys.ctypes.data, n, got.ctypes.data)
        np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("k", [1, 64])
def test_hostmodel_symbol_cache_sizes(built, k):
    """The lane-0 symbol cache gives the same result with one entry and with many."""
    from ptilopsis_gb300.synth import config_params, generate
    L = hostmodel()
    L.ptlhm_set_cache_entries(ctypes.c_uint32(k))
    try:
        assert_stages_equal(tree_to_ast(generate(config_params("c1", scale=40 / 2048))))
        ast, _ = load_fixture("pareas_basic_3_in")
        assert_stages_equal(ast)
    finally:
        L.ptlhm_set_cache_entries(ctypes.c_uint32(4))


@pytest.mark.parametrize("hashed", [False, True])
def test_hostmodel_row0_lookup_modes(built, hashed):
    """Row-0 membership by recorded definition position and by hashing row 0 agree."""
    from ptilopsis_gb300.synth import config_params, generate
    L = hostmodel()
    L.ptlhm_set_hashed(ctypes.c_int(1 if hashed else 0))
    try:
        assert_stages_equal(tree_to_ast(generate(config_params("c1", scale=40 / 2048))))
        for name in ("pareas_basic_3_in", "comp_all_ptl", "arith1_ptl"):
            ast, _ = load_fixture(name)
            assert_stages_equal(ast)
    finally:
        L.ptlhm_set_hashed(ctypes.c_int(0))


def test_packed_gen_tables_decode_to_the_code_tables(built):
    """isn_gen reads each node type's four slots from one packed 16-byte record; every
    field must fit and decode to the table it was packed from."""
    assert hostmodel().ptlhm_gen_desc_ok() == 1
