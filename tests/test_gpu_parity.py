"""GPU parity through the C ABI: the CUDA pipeline against the reference's golden
outputs and against the oracle, stage by stage, on the same inputs.  Integer work:
the bar is bit-exact."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import ast_to_tree, load_fixture, load_synth_golden, manifest, tree_to_ast

pytestmark = pytest.mark.gpu

STAGE_SNAPSHOTS = ["pre_type", "pre_rtype", "pre_data", "cnt_size", "cnt_loc", "cnt_fn_id", "cnt_fn_start",
                   "cnt_fn_end", "cnt_fn_size", "gen_instr", "gen_rd", "gen_rs1", "gen_rs2", "gen_jt", "opt_used",
                   "ra_instr", "ra_rd", "ra_rs1", "ra_rs2", "ra_jt", "ra_fn_start", "ra_fn_end", "ra_fn_size",
                   "out_words", "fn_start", "fn_end", "fn_size", "fn_id"]


def gpu_compile(tree, snapshots=False):
    from ptilopsis_gb300 import RvGenerator
    with RvGenerator(tree) as gen:
        gen.process(profile=True)
        words = gen.get_instructions()
        table = gen.function_table()
        snaps = {k: gen.snapshot(k) for k in STAGE_SNAPSHOTS} if snapshots else {}
    return words, table, snaps


def assert_matches_oracle(tree):
    from oracle import portbind
    ref = portbind.compile_ast(tree_to_ast(tree), snapshots=True)
    words, table, snaps = gpu_compile(tree, snapshots=True)
    for name in STAGE_SNAPSHOTS:
        np.testing.assert_array_equal(snaps[name], ref.bufs[name], err_msg=name)
    np.testing.assert_array_equal(words, ref.words)
    return words


@pytest.mark.parametrize("fx", [f["name"] for f in manifest()["fixtures"]])
def test_gpu_matches_reference_golden(built_cuda, fx):
    ast, gold = load_fixture(fx)
    words, table, _ = gpu_compile(ast_to_tree(ast))
    np.testing.assert_array_equal(words, gold["words"])
    for k, g in (("starts", "fn_start"), ("ends", "fn_end"), ("sizes", "fn_size"), ("ids", "fn_id")):
        np.testing.assert_array_equal(table[k], gold[g], err_msg=k)


@pytest.mark.parametrize("entry", manifest()["synthetic"], ids=lambda e: e["name"])
def test_gpu_matches_reference_golden_synthetic(built_cuda, entry):
    from ptilopsis_gb300.synth import SynthParams, generate
    words, _, _ = gpu_compile(generate(SynthParams(seed=entry["seed"])))
    np.testing.assert_array_equal(words, load_synth_golden(entry["name"])["words"])


@pytest.mark.parametrize("fx", [f["name"] for f in manifest()["fixtures"]])
def test_gpu_stages_match_oracle_fixture(built_cuda, fx):
    ast, _ = load_fixture(fx)
    assert_matches_oracle(ast_to_tree(ast))


@pytest.mark.parametrize("seed", [0x50544C00, 0x50544C40, 0x50544C41])
def test_gpu_stages_match_oracle_synthetic(built_cuda, seed):
    from ptilopsis_gb300.synth import SynthParams, generate
    assert_matches_oracle(generate(SynthParams(seed=seed)))


def test_gpu_spilling_program(built_cuda):
    from ptilopsis_gb300.synth import config_params, generate
    assert_matches_oracle(generate(config_params("c1", scale=96 / 2048)))


@pytest.mark.parametrize("scale", [96 / 2048, 0.1])
def test_gpu_row0_hash_path_equals_definition_path(built_cuda, scale):
    """The register allocator's two row-0 lookups (recorded definition position, and
    the hash of row 0 taken when a virtual register has two definitions) agree."""
    from ptilopsis_gb300 import RvGenerator
    from ptilopsis_gb300.synth import config_params, generate
    tree = generate(config_params("c1", scale=scale))
    with RvGenerator(tree) as gen:
        gen.process()
        fast = gen.get_instructions()
        gen.process(row0_hash=True)
        np.testing.assert_array_equal(gen.get_instructions(), fast)


def test_gpu_many_functions(built_cuda):
    from ptilopsis_gb300.synth import SynthParams, generate
    assert_matches_oracle(generate(SynthParams(seed=0x50544C42, n_functions=2000, median_fn_nodes=80.0,
                                               sigma=1.0, max_nesting=8)))


@pytest.mark.parametrize("n_functions", [9000, 32768, 33000])
def test_gpu_cluster_lane0_pass(built_cuda, n_functions):
    """More than 1,024 lane-0 groups: the lane-0 pass runs on a thread-block cluster
    (one slot per thread up to 4,096 groups -- 32,768 functions fill 8 CTAs of 512 --
    two per thread above).  Plain pipeline with both row-0 lookups, and the batched
    pipeline with a small program beside it, all against the oracle."""
    from oracle import portbind
    from ptilopsis_gb300 import RvGenerator
    from ptilopsis_gb300.batch import BatchCompiler
    from ptilopsis_gb300.synth import SynthParams, generate
    tree = generate(SynthParams(seed=0x50544C60 + n_functions, n_functions=n_functions, median_fn_nodes=40.0,
                                sigma=1.0, max_nesting=6, spill_frac=0.25))
    small = generate(SynthParams(seed=0x50544C44))
    ref = portbind.compile_ast(tree_to_ast(tree))
    ref_small = portbind.compile_ast(tree_to_ast(small))
    with RvGenerator(tree) as gen:
        gen.process()
        np.testing.assert_array_equal(gen.get_instructions(), ref.words)
        np.testing.assert_array_equal(gen.function_table()["starts"], ref.bufs["fn_start"])
        gen.process(row0_hash=True)
        np.testing.assert_array_equal(gen.get_instructions(), ref.words)
    with BatchCompiler(workers=8) as b:
        b.compile([small, tree])
        np.testing.assert_array_equal(b.result(0).words, ref_small.words)
        np.testing.assert_array_equal(b.result(1).words, ref.words)
        np.testing.assert_array_equal(b.result(1).table["starts"], ref.bufs["fn_start"])


def test_gpu_cluster_and_one_block_lane0_passes_agree(built_cuda):
    """The lane-0 pass of a program with 1,125 lane-0 groups on a cluster (the default)
    and in one block of 1,024 threads (PTL_RA_ONE_BLOCK=1, the pass a device that cannot
    place the cluster takes) give the same words, plain and batched.  The environment is
    read once per process, so the one-block run is a child process."""
    import json
    import os
    import subprocess
    import sys
    from ptilopsis_gb300 import RvGenerator
    from ptilopsis_gb300.synth import SynthParams, generate
    params = dict(seed=0x50544C60 + 9000, n_functions=9000, median_fn_nodes=40.0, sigma=1.0, max_nesting=6,
                  spill_frac=0.25)
    with RvGenerator(generate(SynthParams(**params))) as gen:
        gen.process()
        want = gen.get_instructions()
    code = f"""
import json, sys, zlib
sys.path.insert(0, {os.path.dirname(os.path.dirname(os.path.abspath(__file__)))!r})
from ptilopsis_gb300 import RvGenerator
from ptilopsis_gb300.batch import BatchCompiler
from ptilopsis_gb300.synth import SynthParams, generate
t = generate(SynthParams(**{params!r}))
with RvGenerator(t) as g:
    g.process()
    w = g.get_instructions()
with BatchCompiler(workers=4) as b:
    b.compile([t])
    wb = b.result(0).words
print(json.dumps([len(w), zlib.crc32(w.tobytes()), len(wb), zlib.crc32(wb.tobytes())]))
"""
    env = dict(os.environ, PTL_RA_ONE_BLOCK="1")
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    import zlib
    n, c, nb, cb = json.loads(out.stdout.strip().splitlines()[-1])
    assert (n, c) == (len(want), zlib.crc32(want.tobytes())), "plain, one block"
    assert (nb, cb) == (len(want), zlib.crc32(want.tobytes())), "batched, one block"


def test_gpu_float_heavy_deep_expressions(built_cuda):
    from ptilopsis_gb300.synth import config_params, generate
    assert_matches_oracle(generate(config_params("c2", scale=64 / 32768)))


def test_gpu_device_resident_input_equals_host_input(built_cuda):
    import torch
    from ptilopsis_gb300.synth import SynthParams, generate
    tree = generate(SynthParams(seed=0x50544C43))
    host_words, _, _ = gpu_compile(tree)
    dev_words, _, _ = gpu_compile(tree.to(torch.device("cuda", 0)))
    np.testing.assert_array_equal(host_words, dev_words)


def test_gpu_process_is_repeatable_and_upload_rebinds(built_cuda):
    from oracle import portbind
    from ptilopsis_gb300 import RvGenerator
    from ptilopsis_gb300.synth import SynthParams, generate
    a = generate(SynthParams(seed=0x50544C44))
    b = generate(SynthParams(seed=0x50544C45, n_functions=40, median_fn_nodes=900.0, sigma=1.0))
    with RvGenerator(a) as gen:
        gen.process()
        w1 = gen.get_instructions()
        gen.process()
        np.testing.assert_array_equal(gen.get_instructions(), w1)
        gen.upload(b)
        gen.process()
        np.testing.assert_array_equal(gen.get_instructions(), portbind.compile_ast(tree_to_ast(b)).words)
        gen.upload(a)
        gen.process()
        np.testing.assert_array_equal(gen.get_instructions(), w1)


def test_gpu_rejects_malformed_tree(built_cuda):
    from ptilopsis_gb300 import PtlError, RvGenerator
    from ptilopsis_gb300.synth import SynthParams, generate
    tree = generate(SynthParams(seed=0x50544C46, n_functions=2, median_fn_nodes=50.0))
    bad = ast_to_tree(tree_to_ast(tree))
    bad.parent = bad.parent.copy()
    bad.parent[3] = 1  # a parent before its child breaks post-order
    with RvGenerator(bad) as gen:
        with pytest.raises(PtlError) as e:
            gen.process()
    assert e.value.status == 1
    # a declared max_depth that no node reaches leaves a depth level empty
    empty = ast_to_tree(tree_to_ast(tree))
    empty.max_depth = empty.max_depth + 1
    with RvGenerator(empty) as gen:
        with pytest.raises(PtlError) as e:
            gen.process()
    assert e.value.status == 1 and "not all populated" in str(e.value)


def test_gpu_large_program_against_oracle(built_cuda):
    """A quarter of the large-program workload (~1M nodes), words and function table."""
    from oracle import portbind
    from ptilopsis_gb300.synth import config_params, generate
    tree = generate(config_params("c1", scale=0.25))
    ref = portbind.compile_ast(tree_to_ast(tree))
    words, table, _ = gpu_compile(tree)
    np.testing.assert_array_equal(words, ref.words)
    np.testing.assert_array_equal(table["starts"], ref.bufs["fn_start"])


def _program_by_size(lo, hi):
    from ptilopsis_gb300.synth import config_params, generate
    for k in range(64):
        t = generate(config_params("c3", program=k))
        if lo <= t.n <= hi:
            return t
    raise AssertionError(f"no program of {lo}..{hi} nodes")


@pytest.mark.parametrize("case", ["one_block", "rounds_then_blocks", "equal_key_ranges"])
def test_gpu_depth_order_equals_std_sort(built_cuda, case):
    """isn_gen's depth order (libstdc++ std::sort of node ids by depth) against the
    oracle's std::sort: a program of at most 8,192 nodes (one block sorts it), one above
    that (partition rounds, then blocks), and a 1M-node program whose depth levels hold
    tens of thousands of nodes each (ranges of equal keys finished in closed form)."""
    from oracle import portbind
    from ptilopsis_gb300 import RvGenerator
    from ptilopsis_gb300.synth import config_params, generate
    if case == "one_block":
        tree = _program_by_size(1000, 8192)
    elif case == "rounds_then_blocks":
        tree = _program_by_size(8193, 200_000)
    else:
        tree = generate(config_params("c1", scale=0.25))
    perm = portbind.depth_sort(np.ascontiguousarray(tree.depth, np.int32))
    want = np.empty(tree.n, np.uint32)
    want[perm] = np.arange(tree.n, dtype=np.uint32)
    with RvGenerator(tree) as gen:
        gen.process()
        got = gen.snapshot("depth_order_pos")
    np.testing.assert_array_equal(got[:tree.n], want)


def _adversarial_keys(kind: str, n: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    if kind == "all_equal":
        return np.full(n, 7, np.int32)
    if kind == "one_low":  # all equal but one smaller key, somewhere
        k = np.full(n, 9, np.int32)
        k[rng.integers(n)] = 3
        return k
    if kind == "mostly_one":  # 99% one value, the rest spread below and above it
        k = np.full(n, 20, np.int32)
        idx = rng.choice(n, size=max(1, n // 100), replace=False)
        k[idx] = rng.integers(0, 41, size=idx.size)
        return k
    if kind == "two_alternating":
        return (np.arange(n) % 2).astype(np.int32) + 5
    if kind == "few_sorted":
        return np.sort(rng.integers(0, 4, size=n)).astype(np.int32)
    if kind == "few_reversed":
        return np.sort(rng.integers(0, 4, size=n))[::-1].astype(np.int32).copy()
    return rng.integers(0, 60, size=n).astype(np.int32)  # "depth_like"


@pytest.mark.parametrize("kind", ["all_equal", "one_low", "mostly_one", "two_alternating", "few_sorted",
                                  "few_reversed", "depth_like"])
@pytest.mark.parametrize("n", [17, 8192, 8193, 50_000, 300_000])
def test_gpu_depth_order_adversarial_keys(built_cuda, kind, n):
    """The depth-order emulation on key sets that stress the partition rounds' pair-count
    bound and the closed forms (one value, one outlier, a 1% sprinkle, alternation, few
    values sorted either way), at sizes for one leaf, one block, and rounds then blocks:
    every position against the oracle's std::sort."""
    from oracle import portbind
    from ptilopsis_gb300 import depth_order
    keys = _adversarial_keys(kind, n, seed=n ^ len(kind))
    perm = portbind.depth_sort(keys)
    want = np.empty(n, np.uint32)
    want[perm] = np.arange(n, dtype=np.uint32)
    np.testing.assert_array_equal(depth_order(keys), want)


def test_gpu_copy_instructions_into_caller_buffer(built_cuda):
    """ptl_generator_copy_instructions: a null buffer sets the count, a short one is
    refused, and after a process that left the words on the device (and after one that
    brought them to the host) the copy equals get_instructions."""
    import ctypes
    from ptilopsis_gb300 import RvGenerator
    from ptilopsis_gb300.synth import SynthParams, generate
    tree = generate(SynthParams(seed=0x50544C45))
    with RvGenerator(tree) as gen:
        L, h = gen._lib, gen._h
        for to_host in (False, True):
            gen.process(to_host=to_host)
            n = ctypes.c_size_t()
            assert L.ptl_generator_copy_instructions(h, None, 0, ctypes.byref(n)) == 0
            assert n.value > 0
            buf = np.zeros(n.value, np.uint32)
            ptr = buf.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
            assert L.ptl_generator_copy_instructions(h, ptr, n.value - 1, ctypes.byref(n)) != 0
            assert L.ptl_generator_copy_instructions(h, ptr, n.value, ctypes.byref(n)) == 0
            np.testing.assert_array_equal(buf, gen.get_instructions(), err_msg=f"to_host={to_host}")
