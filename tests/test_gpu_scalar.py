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
