"""Bit-exactness at the sizes the measurements are quoted on, through the C ABI.

* The reference's larger Pareas inputs (basic/4-5, funclen/1-8, shape/3-6): every stage
  array the GPU keeps against the CRCs of the reference's own run (one worker thread),
  alone and all fourteen in one batch.  The deep shape/* trees exercise the register
  allocator's lane-0 coupling (rv_generator_avx.cpp:1245-1320, 1400-1413).
* The whole large-program workload (4.3M nodes, 2,048 functions, a quarter of them
  spilling) and the whole huge-program workload (64M nodes, 32,768 functions, 4,096
  lane-0 groups): words and function table against the oracle, plain and batched.
"""
from __future__ import annotations

import zlib

import numpy as np
import pytest

from conftest import ast_to_tree, load_large, manifest_large, tree_to_ast

pytestmark = pytest.mark.gpu

GPU_SNAPSHOTS = ["pre_type", "pre_rtype", "pre_data", "cnt_size", "cnt_loc", "cnt_fn_id", "cnt_fn_start",
                 "cnt_fn_end", "cnt_fn_size", "gen_instr", "gen_rd", "gen_rs1", "gen_rs2", "gen_jt", "opt_used",
                 "ra_instr", "ra_rd", "ra_rs1", "ra_rs2", "ra_jt", "ra_fn_start", "ra_fn_end", "ra_fn_size",
                 "out_words", "fn_start", "fn_end", "fn_size", "fn_id"]
TABLE = (("starts", "fn_start"), ("ends", "fn_end"), ("sizes", "fn_size"), ("ids", "fn_id"))
LARGE = [f["name"] for f in manifest_large()["fixtures"]]


def crc(a) -> int:
    return zlib.crc32(np.ascontiguousarray(a, np.uint32).tobytes())


def _first_difference(got, want) -> str:
    n = min(len(got), len(want))
    d = np.flatnonzero(got[:n] != want[:n])
    at = int(d[0]) if len(d) else n
    return f"lengths {len(got)} vs {len(want)}, first difference at {at}"


@pytest.mark.parametrize("fx", LARGE)
def test_gpu_large_input_matches_reference(built_cuda, fx):
    from ptilopsis_gb300 import RvGenerator
    ast, entry = load_large(fx)
    with RvGenerator(ast_to_tree(ast)) as gen:
        gen.process()
        snaps = {k: gen.snapshot(k) for k in GPU_SNAPSHOTS}
    bad = [k for k in GPU_SNAPSHOTS
           if len(snaps[k]) != entry["snapshots"][k][0] or crc(snaps[k]) != entry["snapshots"][k][1]]
    if bad:  # name the first differing position against the oracle (pinned to the same CRCs)
        from oracle import portbind
        ref = portbind.compile_ast(ast, snapshots=True)
        pytest.fail(f"{fx}: {bad[0]} differs from the reference ({_first_difference(snaps[bad[0]], ref.bufs[bad[0]])});"
                    f" differing arrays: {bad}")


def test_gpu_large_inputs_batched_match_reference(built_cuda):
    from ptilopsis_gb300.batch import BatchCompiler
    trees, entries = [], []
    for fx in LARGE:
        ast, entry = load_large(fx)
        trees.append(ast_to_tree(ast))
        entries.append(entry)
    with BatchCompiler(workers=8) as b:
        b.compile(trees)
        for fx, entry, k in zip(LARGE, entries, range(len(trees))):
            res = b.result(k)
            assert len(res.words) == entry["words"] and crc(res.words) == entry["snapshots"]["out_words"][1], fx
            for key, snap in TABLE:
                assert crc(res.table[key]) == entry["snapshots"][snap][1], (fx, key)


def _check_against_oracle(tree, label):
    from oracle import portbind
    from ptilopsis_gb300 import RvGenerator
    from ptilopsis_gb300.batch import BatchCompiler
    ref = portbind.compile_ast(tree_to_ast(tree))
    with RvGenerator(tree) as gen:
        gen.process()
        words = gen.get_instructions()
        table = gen.function_table()
    assert np.array_equal(words, ref.words), f"{label} plain: {_first_difference(words, ref.words)}"
    for key, snap in TABLE:
        np.testing.assert_array_equal(table[key], ref.bufs[snap], err_msg=f"{label} plain {key}")
    del words, table
    with BatchCompiler(workers=8) as b:
        b.compile([tree])
        res = b.result(0)
        assert np.array_equal(res.words, ref.words), f"{label} batched: {_first_difference(res.words, ref.words)}"
        for key, snap in TABLE:
            np.testing.assert_array_equal(res.table[key], ref.bufs[snap], err_msg=f"{label} batched {key}")
    return len(ref.words)


def test_gpu_whole_large_program_matches_oracle(built_cuda):
    from ptilopsis_gb300.synth import config_tree
    tree = config_tree("c1")
    assert tree.n > 4_000_000
    _check_against_oracle(tree, "4.3M-node program")


def test_gpu_whole_huge_program_matches_oracle(built_cuda):
    """64M nodes; the oracle takes about two minutes on one core."""
    from ptilopsis_gb300.synth import config_tree
    tree = config_tree("c2")
    assert tree.n > 60_000_000
    _check_against_oracle(tree, "64M-node program")
