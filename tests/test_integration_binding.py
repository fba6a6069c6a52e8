"""The reference-side binding (include/rv_generator_gb300.hpp) compiles against the
reference's own headers, links with the reference's objects and libptl_gb300.so, and
runs the reference's main-program sequence (front end, DepthTree, process, to_asm,
to_binary).  Needs the reference tree and an x86-64 host (the reference is written
against AVX2); where a GPU is visible the words must equal the reference's golden words,
elsewhere the generator must refuse with the C ABI's status in the exception text."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_fixture, reference_available


def test_reference_binding_builds_and_runs(built_cuda, tmp_path):
    if not reference_available():
        pytest.skip("reference not buildable on this host")
    from oracle import refbind
    root = refbind.ref_root_cached()
    res = subprocess.run(["make", "-C", os.path.join(ROOT, "oracle", "ref"), f"REF={root}", "binding"],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
    exe = os.path.join(ROOT, "oracle", "_ref", "binding_check")
    src = os.path.join(root, "testfiles", "pareas", "basic", "1.in")
    out_s, out_b = tmp_path / "out.S", tmp_path / "out.bin"
    run = subprocess.run([exe, src, str(out_s), str(out_b)], capture_output=True, text=True, timeout=300)
    try:
        import torch
        gpu = torch.cuda.is_available()
    except ImportError:
        gpu = False
    if gpu:
        assert run.returncode == 0, run.stderr
        _, gold = load_fixture("pareas_basic_1_in")
        np.testing.assert_array_equal(np.fromfile(out_b, dtype="<u4"), gold["words"])
        assert out_s.read_text() == refbind.to_asm(gold["words"])
        csv = run.stdout.strip().splitlines()
        assert csv[0] == "preprocess,isn_cnt,isn_gen,optimize,regalloc,fix_jumps,postprocess"
        assert len(csv[1].split(",")) == 7
    else:
        assert run.returncode == 3, run.stdout + run.stderr
        assert "ptl_generator_create: status 6" in run.stderr  # PTL_CUDA_ERROR: no device
    # the scalar generator through the same binding (the reference's -s)
    run = subprocess.run([exe, "-s", src, str(out_s), str(out_b)], capture_output=True, text=True, timeout=300)
    if gpu:
        assert run.returncode == 0, run.stderr
        ref = refbind.compile_ast_scalar(refbind.parse_file(src))
        np.testing.assert_array_equal(np.fromfile(out_b, dtype="<u4"), ref.bufs["out_words"])
    else:
        assert run.returncode == 3, run.stdout + run.stderr
        assert "ptl_generator_create_scalar: status 6" in run.stderr
