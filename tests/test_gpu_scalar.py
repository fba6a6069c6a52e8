"""The scalar generator's semantics on the GPU (RvGenerator(scalar=True), the C ABI's
ptl_generator_create_scalar): every stage array and the output against the reference's
scalar generator (rv_generator_st, the -s flag) on the fixtures, the c0 seeds and
seeded programs of the batched workload -- CRCs of the reference's arrays
(tests/golden/manifest_scalar.json) and its stored words.  Bit-exact."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import ast_to_tree, crc32, load_fixture, load_scalar_case, manifest, manifest_scalar

pytestmark = pytest.mark.gpu

GPU_SNAPSHOTS = ["pre_type", "pre_rtype", "pre_data", "cnt_size", "cnt_loc", "cnt_fn_id", "cnt_fn_start",
                 "cnt_fn_end", "cnt_fn_size", "gen_instr", "gen_rd", "gen_rs1", "gen_rs2", "gen_jt", "opt_used",
                 "ra_instr", "ra_rd", "ra_rs1", "ra_rs2", "ra_jt", "ra_fn_start", "ra_fn_end", "ra_fn_size",
                 "out_words", "fn_start", "fn_end", "fn_size", "fn_id"]
CASES = [e["name"] for e in manifest_scalar()["fixtures"]]


def _crc(name, a):
    if name == "opt_used":  # the reference's flags are bools
        a = (a != 0).astype(np.uint32)
    return [int(len(a)), crc32(a)]


@pytest.mark.parametrize("name", CASES)
def test_gpu_scalar_matches_reference(built_cuda, name):
    from ptilopsis_gb300 import RvGenerator
    entry = next(e for e in manifest_scalar()["fixtures"] if e["name"] == name)
    ast, gold = load_scalar_case(entry)
    with RvGenerator(ast_to_tree(ast), scalar=True) as gen:
        gen.process(profile=True)
        words = gen.get_instructions()
        table = gen.function_table()
        for k in GPU_SNAPSHOTS:
            assert _crc(k, gen.snapshot(k)) == entry["snapshots"][k], f"{name}: {k}"
    assert [len(words), crc32(words)] == entry["snapshots"]["out_words"]
    if gold is not None:
        np.testing.assert_array_equal(words, gold["out_words"])
        np.testing.assert_array_equal(table["starts"], gold["fn_start"])
        np.testing.assert_array_equal(table["ends"], gold["fn_end"])
        np.testing.assert_array_equal(table["sizes"], gold["fn_size"])
        np.testing.assert_array_equal(table["ids"], gold["fn_id"])


def test_gpu_scalar_and_avx_generators_side_by_side(built_cuda):
    """Generators of both kinds on one device, interleaved, each giving its own
    reference's words (no state leaks between the kinds)."""
    from ptilopsis_gb300 import RvGenerator
    fx = "many_args_in"
    ast, gold = load_fixture(fx)
    entry = next(e for e in manifest_scalar()["fixtures"] if e["name"] == fx)
    _, sgold = load_scalar_case(entry)
    tree = ast_to_tree(ast)
    with RvGenerator(tree) as a, RvGenerator(tree, scalar=True) as s:
        for _ in range(2):
            a.process()
            s.process()
            np.testing.assert_array_equal(a.get_instructions(), gold["words"])
            np.testing.assert_array_equal(s.get_instructions(), sgold["out_words"])
    assert not np.array_equal(gold["words"], sgold["out_words"])


def test_gpu_scalar_cli(built_cuda, tmp_path):
    import os
    import subprocess
    import sys
    from ptilopsis_gb300 import to_asm
    from ptilopsis_gb300.cli import save_tree
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    fx = manifest()["fixtures"][0]["name"]
    ast, _ = load_fixture(fx)
    entry = next(e for e in manifest_scalar()["fixtures"] if e["name"] == fx)
    _, sgold = load_scalar_case(entry)
    save_tree(ast_to_tree(ast), tmp_path / "prog.npz")
    env = {**os.environ, "PYTHONPATH": root}
    r = subprocess.run([sys.executable, "-m", "ptilopsis_gb300", "prog.npz", "-s"], cwd=tmp_path, env=env,
                       capture_output=True)
    assert r.returncode == 0, r.stderr
    np.testing.assert_array_equal(np.fromfile(tmp_path / "c.out", "<u4"), sgold["out_words"])
    r = subprocess.run([sys.executable, "-m", "ptilopsis_gb300", "prog.npz", "-s", "-S", "-o", "-"], cwd=tmp_path,
                       env=env, capture_output=True)
    assert r.returncode == 0 and r.stdout.decode() == to_asm(sgold["out_words"])


def test_gpu_scalar_rejects_malformed_tree(built_cuda):
    from ptilopsis_gb300 import PtlError, RvGenerator
    from ptilopsis_gb300.synth import SynthParams, generate
    from conftest import tree_to_ast
    tree = generate(SynthParams(seed=0x50544C46, n_functions=2, median_fn_nodes=50.0))
    bad = ast_to_tree(tree_to_ast(tree))
    bad.parent = bad.parent.copy()
    bad.parent[3] = 1  # a parent before its child breaks post-order
    with RvGenerator(bad, scalar=True) as gen:
        with pytest.raises(PtlError) as e:
            gen.process()
    assert e.value.status == 1


@pytest.mark.parametrize("name", [n for n in CASES if not n.startswith("c3_")] + ["c3_program_0", "c3_program_22"])
def test_gpu_scalar_serial_order_equals_reference(built_cuda, name):
    """The serial register-allocation kernel (the reference's order over all functions,
    which programs whose functions name each other's words need) gives the reference's
    words on every program."""
    from ptilopsis_gb300 import RvGenerator
    entry = next(e for e in manifest_scalar()["fixtures"] if e["name"] == name)
    ast, _ = load_scalar_case(entry)
    with RvGenerator(ast_to_tree(ast), scalar=True) as gen:
        gen.process(serial=True)
        words = gen.get_instructions()
        for k in ("ra_instr", "ra_rd", "ra_rs1", "ra_rs2", "ra_jt"):
            assert _crc(k, gen.snapshot(k)) == entry["snapshots"][k], f"{name}: {k}"
    assert [len(words), crc32(words)] == entry["snapshots"]["out_words"]


@pytest.mark.parametrize("case", ["c1_quarter", "c3_large"])
def test_gpu_scalar_against_oracle_at_scale(built_cuda, case):
    """Programs larger than the committed cases against the oracle's restatement of the
    scalar generator: a quarter of the 4.3M-node spilling configuration, and the largest
    of the first 256 batched-workload programs."""
    from oracle import portbind
    from ptilopsis_gb300 import RvGenerator
    from ptilopsis_gb300.synth import config_params, generate
    from conftest import tree_to_ast
    if case == "c1_quarter":
        tree = generate(config_params("c1", scale=0.25))
    else:
        sizes = [(generate(config_params("c3", program=k)).n, k) for k in range(0, 256, 16)]
        tree = generate(config_params("c3", program=max(sizes)[1]))
    ref = portbind.compile_ast(tree_to_ast(tree), snapshots=True, scalar=True)
    with RvGenerator(tree, scalar=True) as gen:
        gen.process()
        np.testing.assert_array_equal(gen.get_instructions(), ref.words)
        t = gen.function_table()
        np.testing.assert_array_equal(t["starts"], ref.bufs["fn_start"])
        np.testing.assert_array_equal(t["sizes"], ref.bufs["fn_size"])
        for k in ("gen_instr", "gen_rd", "ra_instr", "ra_rs1"):
            np.testing.assert_array_equal(gen.snapshot(k), ref.bufs[k], err_msg=k)


@pytest.mark.parametrize("fx", [e["name"] for e in __import__("conftest").manifest_scalar_large()["fixtures"]])
def test_gpu_scalar_matches_reference_on_large_inputs(built_cuda, fx):
    from conftest import load_large, manifest_scalar_large
    from ptilopsis_gb300 import RvGenerator
    entry = next(e for e in manifest_scalar_large()["fixtures"] if e["name"] == fx)
    ast, _ = load_large(fx)
    with RvGenerator(ast_to_tree(ast), scalar=True) as gen:
        gen.process()
        words = gen.get_instructions()
        for k in ("gen_instr", "gen_rs1", "ra_instr", "ra_rd", "ra_rs1", "ra_rs2", "fn_start", "fn_size"):
            assert _crc(k, gen.snapshot(k)) == entry["snapshots"][k], f"{fx}: {k}"
    assert [len(words), crc32(words)] == entry["snapshots"]["out_words"]


def test_gpu_scalar_batch_matches_reference(built_cuda):
    """Every committed scalar case (fixtures, c0 seeds, batched-workload programs) in one
    batch with the scalar switch on: each program's words and function table equal the
    reference's scalar run (CRCs), the same as through the one-program API."""
    from ptilopsis_gb300.batch import BatchCompiler
    entries = manifest_scalar()["fixtures"]
    trees = [ast_to_tree(load_scalar_case(e)[0]) for e in entries]
    with BatchCompiler(workers=4, scalar=True) as b:
        b.compile(trees)
        for k, e in enumerate(entries):
            res = b.result(k)
            assert [len(res.words), crc32(res.words)] == e["snapshots"]["out_words"], e["name"]
            for key, snap in (("starts", "fn_start"), ("ends", "fn_end"), ("sizes", "fn_size"), ("ids", "fn_id")):
                assert [len(res.table[key]), crc32(res.table[key])] == e["snapshots"][snap], (e["name"], key)


def test_gpu_scalar_batch_large_inputs(built_cuda):
    """The reference's larger Pareas inputs with scalar goldens, all in one scalar batch."""
    from conftest import load_large, manifest_scalar_large
    from ptilopsis_gb300.batch import BatchCompiler
    entries = manifest_scalar_large()["fixtures"]
    trees = [ast_to_tree(load_large(e["name"])[0]) for e in entries]
    with BatchCompiler(workers=8, scalar=True) as b:
        b.compile(trees)
        for k, e in enumerate(entries):
            w = b.result(k).words
            assert [len(w), crc32(w)] == e["snapshots"]["out_words"], e["name"]


def test_gpu_scalar_batch_equals_plain_and_switches(built_cuda):
    """Synthetic programs (spilling ones, one with a function too long for a warp's
    symbol bytes, which takes the tile form on its own) in one scalar batch equal the
    plain scalar generator; the same compiler then compiles them with the AVX
    generator's semantics and back, each equal to the matching plain generator."""
    from ptilopsis_gb300 import RvGenerator
    from ptilopsis_gb300.batch import BatchCompiler
    from ptilopsis_gb300.synth import SynthParams, config_params, generate
    rng = np.random.default_rng(0x50544C70)
    trees = [generate(SynthParams(seed=0x50544C70 + k, n_functions=int(rng.integers(1, 40)),
                                  median_fn_nodes=float(rng.integers(40, 900)), sigma=0.8,
                                  max_nesting=int(rng.integers(2, 12)), spill_frac=0.25 if k % 3 == 0 else 0.0))
             for k in range(24)]
    trees.append(generate(SynthParams(seed=0x50544C90, n_functions=2, median_fn_nodes=16000.0, max_nesting=4)))
    trees += [generate(config_params("c3", program=k)) for k in (3, 8)]

    def plain(t, scalar):
        with RvGenerator(t, scalar=scalar) as g:
            g.process()
            return g.get_instructions(), g.function_table()

    want_s = [plain(t, True) for t in trees]
    want_a = [plain(t, False) for t in trees]
    with RvGenerator(trees[24], scalar=True) as g:  # its longest function passes the warp form's cap
        g.process(profile=True)
        assert int(np.max(g.snapshot("cnt_fn_size"))) > 12288
    with BatchCompiler(workers=6) as b:
        for mode, want in ((True, want_s), (False, want_a), (True, want_s)):
            b.set_scalar(mode)
            b.compile(trees)
            for k, (w, tab) in enumerate(want):
                res = b.result(k)
                np.testing.assert_array_equal(res.words, w, err_msg=f"scalar={mode} program {k}")
                for key in ("starts", "ends", "sizes", "ids"):
                    np.testing.assert_array_equal(res.table[key], tab[key], err_msg=f"scalar={mode} {k} {key}")
