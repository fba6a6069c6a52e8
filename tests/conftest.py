"""Shared test setup: the gpu marker, library builds and fixture loading."""
from __future__ import annotations

import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def built():
    """Builds the native libraries in-tree (no-op when up to date)."""
    from ptilopsis_gb300 import build as b
    from oracle import portbind
    b.build_synth()
    b.build_hostmodel()
    assert portbind.build(), "oracle restatement failed to build"
    return True


@pytest.fixture(scope="session")
def built_cuda(built):
    from ptilopsis_gb300 import build as b
    b.build_cuda()
    return True


def manifest() -> dict:
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)


def load_fixture(name: str):
    """(Ast, golden dict) of a committed fixture."""
    from oracle.refbind import Ast
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    ast = Ast(type=z["type"], rtype=z["rtype"], parent=z["parent"], depth=z["depth"], child_idx=z["child_idx"],
              data=z["data"], max_depth=int(z["max_depth"]))
    return ast, {k: z[k] for k in ("words", "fn_start", "fn_end", "fn_size", "fn_id")}


def load_synth_golden(name: str) -> dict:
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


def tree_to_ast(tree):
    from oracle.refbind import Ast
    return Ast(type=tree.type, rtype=tree.rtype, parent=tree.parent, depth=tree.depth, child_idx=tree.child_idx,
               data=tree.data, max_depth=tree.max_depth)


def ast_to_tree(ast):
    from ptilopsis_gb300 import DepthTree
    return DepthTree(ast.type, ast.rtype, ast.parent, ast.depth, ast.child_idx, ast.data, ast.max_depth)


def reference_available() -> bool:
    from oracle import refbind
    return refbind.build()


def manifest_large() -> dict:
    with open(os.path.join(GOLDEN, "manifest_large.json")) as f:
        return json.load(f)


_large_cache: dict = {}


def load_large(name: str):
    """(Ast, manifest entry) of one of the reference's larger Pareas inputs, decoded from
    tests/golden/large and checked against the CRCs of the tree the reference front end
    built (tests/golden/codec.py)."""
    if name not in _large_cache:
        if GOLDEN not in sys.path:
            sys.path.insert(0, GOLDEN)
        import codec
        from oracle.refbind import Ast
        entry = next(e for e in manifest_large()["fixtures"] if e["name"] == name)
        with open(os.path.join(GOLDEN, "large", name + ".tree.xz"), "rb") as f:
            arrs = codec.decode(f.read())
        got = codec.tree_crcs(*arrs)
        assert got == entry["tree_crcs"], f"{name}: decoded tree differs from the reference front end's"
        ast = Ast(*arrs, max_depth=entry["max_depth"])
        _large_cache.clear()  # one large tree at a time
        _large_cache[name] = (ast, entry)
    return _large_cache[name]


def manifest_scalar() -> dict:
    with open(os.path.join(GOLDEN, "manifest_scalar.json")) as f:
        return json.load(f)


def crc32(a) -> int:
    import zlib
    return zlib.crc32(np.ascontiguousarray(a, np.uint32).tobytes())


def load_scalar_case(entry: dict):
    """(Ast, golden outputs or None) of a scalar-generator case of manifest_scalar.json:
    a committed fixture's tree, or a seeded program regenerated and checked against the
    CRCs of the tree the reference compiled.  Outputs are stored for the fixtures and
    the c0 seeds; the workload programs keep CRCs only."""
    if "fixture" in entry:
        ast, _ = load_fixture(entry["fixture"])
    else:
        from ptilopsis_gb300.synth import SynthParams, config_params, generate
        prm = SynthParams(seed=entry["seed"]) if "seed" in entry else config_params("c3", program=entry["c3_program"])
        ast = tree_to_ast(generate(prm))
    got = [crc32(np.asarray(ast.type, np.uint32)), crc32(np.asarray(ast.parent).view(np.uint32)), crc32(ast.data)]
    assert got == entry["tree_crcs"], f"{entry['name']}: tree differs from the one the reference compiled"
    z = np.load(os.path.join(GOLDEN, "scalar_words.npz"))
    key = entry["name"] + ".out_words"
    if key not in z.files:
        return ast, None
    return ast, {k: z[f"{entry['name']}.{k}"] for k in ("out_words", "fn_start", "fn_end", "fn_size", "fn_id")}


def manifest_scalar_large() -> dict:
    """The scalar generator's stage CRCs on the larger Pareas inputs it finished
    (make_golden.py --scalar-large); their trees are those of manifest_large.json."""
    with open(os.path.join(GOLDEN, "manifest_scalar_large.json")) as f:
        return json.load(f)
