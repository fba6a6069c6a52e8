"""The command line (ptilopsis_gb300.cli, mirroring the reference's src/main.cpp): its
argument handling and profiling format on the CPU; a compile of a golden fixture through
it on the GPU, binary and assembly, against the reference's words and to_asm text."""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ast_to_tree, load_fixture, manifest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(args, cwd, stdin=None):
    return subprocess.run([sys.executable, "-m", "ptilopsis_gb300", *args], cwd=cwd, input=stdin,
                          capture_output=True, env={**os.environ, "PYTHONPATH": ROOT})


def test_cli_arguments_and_profile_format(tmp_path):
    from ptilopsis_gb300.cli import load_tree, profile_csv, save_tree
    r = _run(["--help"], tmp_path)
    assert r.returncode == 0 and b"-S" in r.stdout
    r = _run([str(tmp_path / "missing.npz")], tmp_path)
    assert r.returncode == 1 and b"Failed to open file" in r.stderr
    r = _run(["-s", "x.npz"], tmp_path)  # -s (the scalar generator) is accepted
    assert r.returncode == 1 and b"Failed to open file" in r.stderr
    assert profile_csv(["a", "b", "c"], [1, 22, 333]) == "a,b,c\n1,22,333\n"
    ast, _ = load_fixture(manifest()["fixtures"][0]["name"])
    tree = ast_to_tree(ast)
    save_tree(tree, tmp_path / "t.npz")
    back = load_tree(tmp_path / "t.npz")
    for f in ("type", "rtype", "parent", "depth", "child_idx", "data"):
        np.testing.assert_array_equal(getattr(back, f), getattr(tree, f))
    assert back.max_depth == tree.max_depth


@pytest.mark.gpu
def test_cli_compiles_like_the_reference(built_cuda, tmp_path):
    from ptilopsis_gb300 import STAGES, to_asm
    from ptilopsis_gb300.cli import save_tree
    fx = manifest()["fixtures"][0]["name"]
    ast, golden = load_fixture(fx)
    save_tree(ast_to_tree(ast), tmp_path / "prog.npz")
    r = _run(["prog.npz", "-p"], tmp_path)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.decode().splitlines()
    assert lines[0] == ",".join(STAGES) and len(lines[1].split(",")) == len(STAGES)
    np.testing.assert_array_equal(np.fromfile(tmp_path / "c.out", "<u4"), golden["words"])
    r = _run(["prog.npz", "-S"], tmp_path)
    assert r.returncode == 0, r.stderr
    assert (tmp_path / "prog.s").read_text() == to_asm(golden["words"])
    from ptilopsis_gb300 import to_elf
    r = _run(["prog.npz", "--elf", "prog.o"], tmp_path)
    assert r.returncode == 0, r.stderr
    assert (tmp_path / "prog.o").read_bytes() == to_elf(golden["words"], golden["fn_start"], golden["fn_end"])
    r = _run(["-", "-S", "-o", "-"], tmp_path, stdin=(tmp_path / "prog.npz").read_bytes())
    assert r.returncode == 0 and r.stdout.decode() == to_asm(golden["words"])
    # the parser's tree in a shuffled node order, flattened on the GPU before the compile
    from ptilopsis_gb300.cli import save_unordered
    t = ast_to_tree(ast)
    perm = np.random.default_rng(7).permutation(t.n)
    par = np.where(t.parent >= 0, perm[np.maximum(t.parent, 0)], -1)
    arrs = []
    for x in (t.type, t.rtype, par, t.child_idx, t.data):
        y = np.empty_like(x)
        y[perm] = x
        arrs.append(y)
    save_unordered(*arrs, tmp_path / "unordered.npz")
    r = _run(["unordered.npz", "-o", "u.out"], tmp_path)
    assert r.returncode == 0, r.stderr
    np.testing.assert_array_equal(np.fromfile(tmp_path / "u.out", "<u4"), golden["words"])
