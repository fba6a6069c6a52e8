"""Pins the oracle (the CPU restatement in oracle/port) to the reference.

Where the reference is built here (x86-64 with the reference tree), the restatement is
compared stage by stage with the reference itself; everywhere, it is compared with the
golden outputs the reference produced (tests/golden, made by make_golden.py)."""
from __future__ import annotations

import glob
import os
import zlib

import numpy as np
import pytest

from conftest import load_fixture, load_synth_golden, manifest, reference_available, tree_to_ast

STAGE_BUFS = ["pre_type", "pre_rtype", "pre_data", "cnt_size", "cnt_loc", "cnt_fn_id", "cnt_fn_start",
              "cnt_fn_end", "cnt_fn_size", "gen_instr", "gen_rd", "gen_rs1", "gen_rs2", "gen_jt", "opt_used",
              "ra_instr", "ra_rd", "ra_rs1", "ra_rs2", "ra_jt", "ra_fn_start", "ra_fn_end", "ra_fn_size",
              "fj_instr", "fj_rd", "fj_rs1", "fj_rs2", "fj_jt", "fj_fn_start", "fj_fn_end", "fj_fn_size",
              "out_words", "fn_start", "fn_end", "fn_size", "fn_id"]


def crc(a):
    return zlib.crc32(np.ascontiguousarray(a, np.uint32).tobytes())


@pytest.mark.parametrize("fx", [f["name"] for f in manifest()["fixtures"]])
def test_port_matches_golden_fixture(built, fx):
    from oracle import portbind
    ast, gold = load_fixture(fx)
    res = portbind.compile_ast(ast, snapshots=True)
    np.testing.assert_array_equal(res.words, gold["words"])
    for k in ("fn_start", "fn_end", "fn_size", "fn_id"):
        np.testing.assert_array_equal(res.bufs[k], gold[k])
    # every intermediate array, through the CRCs of the reference's snapshots
    snaps = next(f for f in manifest()["fixtures"] if f["name"] == fx)["snapshots"]
    for name, (length, c) in snaps.items():
        assert len(res.bufs[name]) == length, name
        assert crc(res.bufs[name]) == c, name


@pytest.mark.parametrize("entry", manifest()["synthetic"], ids=lambda e: e["name"])
def test_port_matches_golden_synthetic(built, entry):
    from oracle import portbind
    from ptilopsis_gb300.synth import SynthParams, generate
    tree = generate(SynthParams(seed=entry["seed"]))
    assert tree.n == entry["n"]
    res = portbind.compile_ast(tree_to_ast(tree), snapshots=True)
    gold = load_synth_golden(entry["name"])
    np.testing.assert_array_equal(res.words, gold["words"])
    for name, (length, c) in entry["snapshots"].items():
        assert len(res.bufs[name]) == length and crc(res.bufs[name]) == c, name


def test_port_tables_match_reference_tables(built):
    from oracle import portbind
    for w, (n, c) in manifest()["tables"].items():
        t = portbind.table(int(w))
        assert len(t) == n and crc(t) == c, portbind.TABLE_NAMES[int(w)]


REF_INPUTS = ["basic/1.in", "basic/3.in", "basic/5.in", "funclen/1.in", "funclen/8.in"]


@pytest.mark.parametrize("rel", REF_INPUTS)
def test_port_matches_reference_stage_by_stage(built, rel):
    if not reference_available():
        pytest.skip("reference not buildable on this host")
    from oracle import portbind, refbind
    ast = refbind.parse_file(os.path.join(refbind.ref_root_cached(), "testfiles/pareas", rel))
    ref = refbind.compile_ast(ast, snapshots=True)
    port = portbind.compile_ast(ast, snapshots=True)
    for name in STAGE_BUFS:
        np.testing.assert_array_equal(port.bufs[name], ref.bufs[name], err_msg=name)


@pytest.mark.parametrize("seed", [0x50544C10 + k for k in range(4)])
def test_port_matches_reference_on_synthetic(built, seed):
    if not reference_available():
        pytest.skip("reference not buildable on this host")
    from oracle import portbind, refbind
    from ptilopsis_gb300.synth import SynthParams, generate
    tree = generate(SynthParams(seed=seed, n_functions=24, median_fn_nodes=600.0, sigma=1.0, spill_frac=0.3,
                                max_nesting=24))
    ast = tree_to_ast(tree)
    ref = refbind.compile_ast(ast, snapshots=True)
    port = portbind.compile_ast(ast, snapshots=True)
    for name in STAGE_BUFS:
        np.testing.assert_array_equal(port.bufs[name], ref.bufs[name], err_msg=name)


def test_depth_sort_is_libstdcxx_sort(built):
    """The oracle's depth order is std::sort's; the golden words depend on it."""
    from oracle import portbind
    keys = np.array([3, 1, 2, 1, 3, 0, 2, 1, 1, 2, 0, 3, 1, 2, 2, 1, 0, 3, 1, 1, 2, 2], np.int32)
    perm = portbind.depth_sort(keys)
    assert np.all(np.diff(keys[perm]) >= 0)
    assert sorted(perm.tolist()) == list(range(len(keys)))


@pytest.mark.parametrize("fx", [f["name"] for f in __import__("conftest").manifest_large()["fixtures"]])
def test_port_matches_reference_on_large_inputs(built, fx):
    """The reference's larger Pareas inputs (basic/4-5, funclen/1-8, shape/3-6; deep
    shape/* trees exercise the lane-0 coupling of register allocation): every one of the
    36 stage arrays of the restatement against the CRCs of the reference's own run."""
    from conftest import load_large
    from oracle import portbind
    ast, entry = load_large(fx)
    res = portbind.compile_ast(ast, snapshots=True)
    assert len(res.words) == entry["words"]
    for name, (length, c) in entry["snapshots"].items():
        assert len(res.bufs[name]) == length and crc(res.bufs[name]) == c, name


# ---------------------------------------------------------------- scalar generator
@pytest.mark.parametrize("name", [e["name"] for e in __import__("conftest").manifest_scalar()["fixtures"]])
def test_port_scalar_matches_reference_snapshots(built, name):
    """The restatement of the scalar generator (rv_generator_st, the -s flag): all 36
    stage arrays against the CRCs of the reference's scalar run (manifest_scalar.json)."""
    from conftest import load_scalar_case, manifest_scalar
    from oracle import portbind
    entry = next(e for e in manifest_scalar()["fixtures"] if e["name"] == name)
    ast, gold = load_scalar_case(entry)
    res = portbind.compile_ast(ast, snapshots=True, scalar=True)
    for k, (length, c) in entry["snapshots"].items():
        a = res.bufs[k]
        if k == "opt_used":  # the reference's flags are bools
            a = (a != 0).astype(np.uint32)
        assert len(a) == length and crc(a) == c, k
    if gold is not None:
        np.testing.assert_array_equal(res.words, gold["out_words"])


@pytest.mark.parametrize("seed", [0x50544C10 + k for k in range(3)])
def test_port_scalar_matches_reference_on_synthetic(built, seed):
    if not reference_available():
        pytest.skip("reference not buildable on this host")
    from oracle import portbind, refbind
    from ptilopsis_gb300.synth import SynthParams, generate
    tree = generate(SynthParams(seed=seed, n_functions=24, median_fn_nodes=600.0, sigma=1.0, spill_frac=0.3,
                                max_nesting=24, float_frac=0.4))
    ast = tree_to_ast(tree)
    ref = refbind.compile_ast_scalar(ast, snapshots=True)
    port = portbind.compile_ast(ast, snapshots=True, scalar=True)
    for name in STAGE_BUFS:
        a = port.bufs[name]
        b = ref.bufs[name]
        if name == "opt_used":
            a, b = (a != 0), (b != 0)
        np.testing.assert_array_equal(a, b, err_msg=name)


@pytest.mark.parametrize("fx", [e["name"] for e in __import__("conftest").manifest_scalar_large()["fixtures"]])
def test_port_scalar_matches_reference_on_large_inputs(built, fx):
    """The scalar restatement on the reference's larger Pareas inputs: every stage array
    against the CRCs of the reference's scalar run (minutes per input there)."""
    from conftest import load_large, manifest_scalar_large
    from oracle import portbind
    entry = next(e for e in manifest_scalar_large()["fixtures"] if e["name"] == fx)
    ast, _ = load_large(fx)
    res = portbind.compile_ast(ast, snapshots=True, scalar=True)
    assert len(res.words) == entry["words"]
    for k, (length, c) in entry["snapshots"].items():
        a = res.bufs[k]
        if k == "opt_used":
            a = (a != 0).astype(np.uint32)
        assert len(a) == length and crc(a) == c, k
