"""The synthetic program generator against the reference front end: the source text it
prints, parsed by pareas-ast, must give exactly the arrays it emits."""
from __future__ import annotations

import os
import tempfile
import zlib

import numpy as np
import pytest

from conftest import manifest, reference_available


@pytest.mark.parametrize("seed", range(6))
def test_generator_matches_front_end(built, seed):
    if not reference_available():
        pytest.skip("reference front end not buildable on this host")
    from oracle import refbind
    from ptilopsis_gb300.synth import SynthParams, generate
    tree, src = generate(SynthParams(seed=seed, n_functions=5, median_fn_nodes=180.0, sigma=0.7, max_nesting=6,
                                     spill_frac=0.2), with_source=True)
    with tempfile.NamedTemporaryFile("w", suffix=".ptl", delete=False) as f:
        f.write(src)
        path = f.name
    try:
        ast = refbind.parse_file(path)
    finally:
        os.unlink(path)
    for k in ("type", "rtype", "parent", "depth", "child_idx", "data"):
        np.testing.assert_array_equal(getattr(tree, k), getattr(ast, k), err_msg=k)
    assert tree.max_depth == ast.max_depth


def test_generator_is_deterministic(built):
    """A seed names one program on every host (golden tree CRCs were made on x86-64)."""
    from ptilopsis_gb300.synth import SynthParams, generate
    for e in manifest()["synthetic"]:
        t = generate(SynthParams(seed=e["seed"]))
        assert t.n == e["n"]
        got = [zlib.crc32(t.type.astype(np.uint32).tobytes()), zlib.crc32(t.parent.view(np.uint32).tobytes()),
               zlib.crc32(t.data.tobytes())]
        assert got == e["tree_crc"]


def test_post_order_invariants(built):
    from ptilopsis_gb300.synth import config_params, generate
    t = generate(config_params("c1", scale=32 / 2048))
    n = t.n
    assert t.parent[-1] == -1 and t.child_idx[-1] == -1 and t.depth[-1] == 0
    idx = np.arange(n - 1)
    assert np.all(t.parent[:-1] > idx)
    assert np.all(t.depth[:-1] == t.depth[t.parent[:-1]] + 1)
    assert t.max_depth == int(t.depth.max())
