"""AST flattening: a parent-pointer tree in any node order into the reference's DepthTree
(pareas-ast/src/codegen/depthtree.cpp:11-100).  The oracle's restatement is pinned
against the reference's own DepthTree constructor (built from its sources) and against
the post-order trees the generator tests use; the GPU (ptl_flatten) is checked against
the oracle on shuffled trees, degenerate shapes and malformed inputs."""
from __future__ import annotations

import numpy as np
import pytest

FIELDS = ("type", "rtype", "parent", "depth", "child_idx", "data")


def shuffled(tree, seed):
    """The tree's nodes in a random order: (type, rtype, parent, child_idx, data) and the
    permutation (old index -> new index)."""
    rng = np.random.default_rng(seed)
    n = tree.n
    perm = rng.permutation(n)
    par = np.where(tree.parent >= 0, perm[np.maximum(tree.parent, 0)], -1).astype(np.int32)
    out = []
    for x in (tree.type, tree.rtype, par, tree.child_idx, tree.data):
        y = np.empty_like(x)
        y[perm] = x
        out.append(y)
    return out, perm


def synth_tree(seed, fns=12, median=300.0):
    from ptilopsis_gb300.synth import SynthParams, generate
    return generate(SynthParams(seed=seed, n_functions=fns, median_fn_nodes=median))


def chain(n):
    """A path of n nodes (the deepest shape): node k's parent is k+1."""
    parent = np.arange(1, n + 1, dtype=np.int32)
    parent[-1] = -1
    child = np.zeros(n, np.int32)
    child[-1] = -1
    return (np.full(n, 3, np.uint8), np.full(n, 2, np.uint8), parent, child, np.arange(n, dtype=np.uint32))


def star(k):
    """A root with k leaf children, the root first and the leaves in reverse order."""
    n = k + 1
    parent = np.zeros(n, np.int32)
    parent[0] = -1
    child = np.zeros(n, np.int32)
    child[0] = -1
    child[1:] = np.arange(k - 1, -1, -1, dtype=np.int32)
    return (np.full(n, 7, np.uint8), np.full(n, 1, np.uint8), parent, child, np.arange(n, dtype=np.uint32) * 3)


def assert_tree(got, want, msg=""):
    for f in FIELDS:
        np.testing.assert_array_equal(getattr(got, f), getattr(want, f), err_msg=f"{msg} {f}")
    assert int(got.max_depth) == int(want.max_depth), msg


# ---------------------------------------------------------------- oracle (CPU)
def test_oracle_flatten_restores_post_order():
    from oracle import portbind
    for seed in range(4):
        t = synth_tree(0x50544E00 + seed)
        arrs, perm = shuffled(t, seed)
        ast, order = portbind.flatten(*arrs)
        assert_tree(ast, t, f"seed {seed}")
        np.testing.assert_array_equal(order[perm], np.arange(t.n))


def test_oracle_flatten_pinned_to_reference():
    from oracle import portbind, refbind
    if not refbind.available():
        pytest.skip("reference oracle not built here")
    cases = [shuffled(synth_tree(0x50544E10 + s, fns=20), s)[0] for s in range(3)] + [chain(300), star(500)]
    for k, arrs in enumerate(cases):
        assert_tree(portbind.flatten(*arrs)[0], refbind.flatten(*arrs), f"case {k}")


def _fixture_cases():
    """The reference front end's own DepthTrees (committed fixtures, built by the
    reference's DepthTree constructor), each given in a seeded random node order."""
    from conftest import ast_to_tree, load_fixture, manifest
    out = []
    for k, fx in enumerate(manifest()["fixtures"]):
        ast, _ = load_fixture(fx["name"])
        tree = ast_to_tree(ast)
        out.append((fx["name"], tree, shuffled(tree, 0x50544E60 + k)[0]))
    return out


def test_oracle_flatten_pinned_to_reference_fixtures():
    """Runs anywhere: the restatement rebuilds exactly the trees the reference built."""
    from oracle import portbind
    for name, tree, arrs in _fixture_cases():
        assert_tree(portbind.flatten(*arrs)[0], tree, name)


def test_oracle_flatten_rejects_malformed():
    from oracle import portbind
    base = list(star(5))
    for name, edit in [("two roots", lambda a: a[2].__setitem__(3, -1)),
                       ("parent out of range", lambda a: a[2].__setitem__(2, 99)),
                       ("child index taken twice", lambda a: a[3].__setitem__(2, int(a[3][1]))),
                       ("child index out of range", lambda a: a[3].__setitem__(1, 5)),
                       ("cycle", lambda a: (a[2].__setitem__(1, 2), a[2].__setitem__(2, 1)))]:
        arrs = [x.copy() for x in base]
        edit(arrs)
        with pytest.raises(portbind.PortError):
            portbind.flatten(*arrs)


# ---------------------------------------------------------------- GPU
@pytest.mark.gpu
def test_gpu_flatten_equals_oracle(built_cuda):
    from oracle import portbind
    from ptilopsis_gb300 import flatten
    cases = [shuffled(synth_tree(0x50544E20 + s, fns=4 + 9 * s), s)[0] for s in range(4)]
    cases += [chain(1), chain(5000), star(70000), shuffled(synth_tree(0x50544E30, fns=600, median=900.0), 9)[0]]
    for k, arrs in enumerate(cases):
        want, want_order = portbind.flatten(*arrs)
        got, order = flatten(*arrs)
        assert_tree(got, want, f"case {k} ({arrs[0].shape[0]} nodes)")
        np.testing.assert_array_equal(order, want_order, err_msg=f"case {k} order")


@pytest.mark.gpu
def test_gpu_flatten_reference_fixtures(built_cuda):
    from ptilopsis_gb300 import flatten
    for name, tree, arrs in _fixture_cases():
        assert_tree(flatten(*arrs)[0], tree, name)


@pytest.mark.gpu
def test_gpu_flatten_then_compile(built_cuda):
    """Flattening a shuffled tree and compiling it gives the words of the original."""
    from ptilopsis_gb300 import compile_tree, flatten
    t = synth_tree(0x50544E40, fns=40)
    arrs, _ = shuffled(t, 3)
    flat, _ = flatten(*arrs)
    np.testing.assert_array_equal(compile_tree(flat), compile_tree(t))


@pytest.mark.gpu
def test_gpu_flatten_rejects_malformed(built_cuda):
    from ptilopsis_gb300 import PtlError, flatten
    base = list(star(5))
    for name, edit in [("two roots", lambda a: a[2].__setitem__(3, -1)),
                       ("no root", lambda a: a[2].__setitem__(0, 1)),
                       ("parent out of range", lambda a: a[2].__setitem__(2, 99)),
                       ("child index taken twice", lambda a: a[3].__setitem__(2, int(a[3][1]))),
                       ("child index out of range", lambda a: a[3].__setitem__(1, 5)),
                       ("cycle", lambda a: (a[2].__setitem__(1, 2), a[2].__setitem__(2, 1)))]:
        arrs = [x.copy() for x in base]
        edit(arrs)
        with pytest.raises(PtlError) as e:
            flatten(*arrs)
        assert e.value.status == 1, name


@pytest.mark.gpu
def test_gpu_flatten_on_device_then_compile(built_cuda):
    """Device arrays in, a device DepthTree out, compiled from device memory: the words of
    the original tree, with no host copy of the flattened arrays."""
    import torch
    from ptilopsis_gb300 import RvGenerator, compile_tree, flatten
    t = synth_tree(0x50544E50, fns=30)
    arrs, perm = shuffled(t, 4)
    dev = [torch.from_numpy(x.view(np.int32) if x.dtype == np.uint32 else x).cuda() for x in arrs]
    flat, order = flatten(*dev)
    assert flat.on_device and int(flat.max_depth) == int(t.max_depth)
    assert_tree(flat.numpy(), t, "device flatten")
    np.testing.assert_array_equal(order.cpu().numpy()[perm], np.arange(t.n))
    with RvGenerator(flat) as g:
        g.process()
        np.testing.assert_array_equal(g.get_instructions(), compile_tree(t))
