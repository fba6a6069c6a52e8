"""The scalar generator's semantics (the reference's rv_generator_st, the -s flag of
src/main.cpp) on the CPU: the host model build of the GPU stage functions in scalar mode
against the CRCs of every stage array the reference's scalar generator produced
(tests/golden/manifest_scalar.json, made by make_golden.py --scalar), with the register
allocation in both of its GPU forms (one thread per function, and the reference's
serial order that programs whose functions name each other's words take)."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import crc32, load_scalar_case, manifest_scalar
from test_hostmodel import SLOTS, _Buf, hostmodel


def hm_compile_scalar(ast, serial: bool = False):
    L = hostmodel()
    L.ptlhm_set_scalar_serial(1 if serial else 0)
    nb = 48
    bufs = (_Buf * nb)()
    err = (ctypes.c_uint32 * 3)()
    arrs = [np.ascontiguousarray(ast.type, np.uint8), np.ascontiguousarray(ast.rtype, np.uint8),
            np.ascontiguousarray(ast.parent, np.int32), np.ascontiguousarray(ast.depth, np.int32),
            np.ascontiguousarray(ast.child_idx, np.int32), np.ascontiguousarray(ast.data, np.uint32)]
    try:
        rc = L.ptlhm_compile_mode(*[ctypes.c_void_p(a.ctypes.data) for a in arrs], ctypes.c_size_t(ast.n),
                                  ctypes.c_size_t(ast.max_depth), bufs, nb, err, ctypes.c_int(1))
    finally:
        L.ptlhm_set_scalar_serial(0)
    out = {}
    for k in range(nb):
        if bufs[k].p:
            out[k] = np.ctypeslib.as_array(bufs[k].p, shape=(bufs[k].n,)).copy() if bufs[k].n else np.zeros(0, np.uint32)
    L.ptlhm_free(bufs, nb)
    return rc, list(err), out


def snapshot_crc(name: str, a: np.ndarray) -> list:
    if name == "opt_used":  # the reference's flags are bools
        a = (a != 0).astype(np.uint32)
    return [int(len(a)), crc32(a)]


def assert_matches_reference(entry, got):
    for name, slot in SLOTS.items():
        want = entry["snapshots"].get(name)
        if want is None:
            continue
        assert snapshot_crc(name, got[slot]) == want, f"{entry['name']}: {name}"


CASES = [e["name"] for e in manifest_scalar()["fixtures"]]


@pytest.mark.parametrize("name", CASES)
def test_scalar_hostmodel_matches_reference_stages(built, name):
    entry = next(e for e in manifest_scalar()["fixtures"] if e["name"] == name)
    ast, gold = load_scalar_case(entry)
    rc, err, got = hm_compile_scalar(ast)
    assert rc == 0, f"host model error {err}"
    assert_matches_reference(entry, got)
    if gold is not None:
        np.testing.assert_array_equal(got[SLOTS["out_words"]], gold["out_words"])
        np.testing.assert_array_equal(got[SLOTS["fn_start"]], gold["fn_start"])


@pytest.mark.parametrize("name", [n for n in CASES if not n.startswith("c3_")] + ["c3_program_0", "c3_program_22"])
def test_scalar_serial_order_matches_reference(built, name):
    """The serial register allocation gives the reference's output for every program,
    not only for the ones that need it."""
    entry = next(e for e in manifest_scalar()["fixtures"] if e["name"] == name)
    ast, _ = load_scalar_case(entry)
    rc, err, got = hm_compile_scalar(ast, serial=True)
    assert rc == 0, f"host model error {err}"
    assert_matches_reference(entry, got)


def test_scalar_output_differs_from_the_avx_generator(built):
    """The two generators are distinct: on the fixture with many arguments the scalar
    output is not the AVX output (the reference's -s flag changes the program)."""
    from conftest import load_fixture
    from test_hostmodel import hm_compile
    ast, gold = load_fixture("many_args_in")
    rc, _, scalar = hm_compile_scalar(ast)
    assert rc == 0
    rc, _, avx = hm_compile(ast)
    assert rc == 0
    np.testing.assert_array_equal(avx[0], gold["words"])
    assert len(scalar[0]) != len(avx[0]) or not np.array_equal(scalar[0], avx[0])
