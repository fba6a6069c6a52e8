"""Batched compilation and the compile server through the C ABI: every program's output
equals compiling it alone with a plain generator, and the oracle for the small ones."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import tree_to_ast

pytestmark = pytest.mark.gpu


def _programs(count, seed0=0x50544C60, max_fns=24):
    from ptilopsis_gb300.synth import SynthParams, generate
    rng = np.random.default_rng(seed0)
    out = []
    for k in range(count):
        out.append(generate(SynthParams(seed=seed0 + k, n_functions=int(rng.integers(1, max_fns)),
                                        median_fn_nodes=float(rng.integers(40, 900)), sigma=0.8,
                                        max_nesting=int(rng.integers(2, 12)), spill_frac=0.2 if k % 3 == 0 else 0.0)))
    return out


def _alone(tree):
    from ptilopsis_gb300 import RvGenerator
    with RvGenerator(tree) as g:
        g.process()
        return g.get_instructions(), g.function_table()


def _assert_same(res, words, table, msg):
    np.testing.assert_array_equal(res.words, words, err_msg=msg)
    for k in ("starts", "ends", "sizes", "ids"):
        np.testing.assert_array_equal(res.table[k], table[k], err_msg=f"{msg} {k}")


def test_batch_equals_alone_and_oracle(built_cuda):
    from oracle import portbind
    from ptilopsis_gb300.batch import BatchCompiler
    trees = _programs(48)
    with BatchCompiler(workers=6) as b:
        b.compile(trees)
        for k, t in enumerate(trees):
            res = b.result(k)
            w, tab = _alone(t)
            _assert_same(res, w, tab, f"program {k}")
            if k % 4 == 0:
                np.testing.assert_array_equal(res.words, portbind.compile_ast(tree_to_ast(t)).words, err_msg=f"oracle {k}")
        # a second call on the same workers (arenas reused, other sizes)
        trees2 = _programs(17, seed0=0x50544C90, max_fns=60)
        b.compile(trees2)
        for k, t in enumerate(trees2):
            w, tab = _alone(t)
            _assert_same(b.result(k), w, tab, f"second call, program {k}")


def test_batch_uneven_sizes(built_cuda):
    """Large and tiny programs in one call (largest-first scheduling)."""
    from ptilopsis_gb300.batch import BatchCompiler
    from ptilopsis_gb300.synth import config_params, generate
    trees = [generate(config_params("c3", program=k)) for k in (1, 5)] + _programs(12, seed0=0x50544CA0)
    trees = [t for t in trees if t.n <= 400_000]
    with BatchCompiler(workers=4) as b:
        b.compile(trees)
        for k, t in enumerate(trees):
            w, tab = _alone(t)
            _assert_same(b.result(k), w, tab, f"program {k} ({t.n} nodes)")


@pytest.mark.parametrize("copy", [True, False])
def test_server_results_same_alone_and_in_the_mix(built_cuda, copy):
    """Requests compiled in the server's batches equal each tree compiled alone, whether
    the server copies a request's arrays or borrows them (PTL_SUBMIT_BORROW)."""
    from ptilopsis_gb300.batch import CompileServer
    trees = _programs(40, seed0=0x50544CB0)
    alone = [_alone(t) for t in trees]
    with CompileServer(slots=6, memory_budget=8 << 30) as srv:
        tickets = [srv.submit(t, copy=copy) for t in trees]
        for k, tk in enumerate(tickets):
            _assert_same(srv.result(tk), *alone[k], f"request {k}")
            s, st, d = srv.times(tk)
            assert s <= st <= d
            srv.release(tk)
        assert srv.stats()["completed"] == len(trees)


def test_server_budget_admission(built_cuda):
    """A budget that fits one request at a time still completes every request correctly;
    a request larger than the whole budget is refused at submit."""
    from ptilopsis_gb300 import PtlError
    from ptilopsis_gb300.batch import CompileServer
    trees = _programs(10, seed0=0x50544CC0)
    alone = [_alone(t) for t in trees]
    budget = (64 << 20) + 288 * max(t.n for t in trees)  # one compile in flight at a time
    with CompileServer(slots=4, memory_budget=budget) as srv:
        tickets = [srv.submit(t) for t in trees]
        for k, tk in enumerate(tickets):
            _assert_same(srv.result(tk), *alone[k], f"request {k}")
        from ptilopsis_gb300.synth import SynthParams, generate
        big = generate(SynthParams(seed=0x50544CD0, n_functions=100, median_fn_nodes=900.0))
        assert 288 * big.n + (64 << 20) > budget
        with pytest.raises(PtlError) as e:
            srv.submit(big)
        assert e.value.status == 4  # PTL_ADMISSION_DENIED


def test_server_device_memory_stays_within_budget(built_cuda):
    """The lanes' resident arenas count against the budget: with a budget a few batches
    wide, the device memory the server holds -- by its own account and by the device's
    free memory, sampled every millisecond -- stays within it while a mix of small and
    large requests (the serving size mix) runs on four lanes, and every result is exact."""
    import threading
    import time
    import torch
    from ptilopsis_gb300.batch import CompileServer
    from ptilopsis_gb300.synth import config_params, generate
    trees = [generate(config_params("c4", program=k)) for k in range(48)]
    assert max(t.n for t in trees) > 100_000 and min(t.n for t in trees) < 10_000
    budget = 2 << 30
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(0)[0]
    peak, held_max, stop = [0], [0], threading.Event()
    with CompileServer(slots=4, memory_budget=budget) as srv:
        def sampler():
            while not stop.is_set():
                peak[0] = max(peak[0], free0 - torch.cuda.mem_get_info(0)[0])
                held_max[0] = max(held_max[0], srv.memory()["held"])
                time.sleep(0.001)
        th = threading.Thread(target=sampler, daemon=True)
        th.start()
        for rnd in range(2):  # two rounds: arenas kept from the first must be charged in the second
            tickets = [srv.submit(t, copy=False) for t in trees]
            outs = [srv.result(tk) for tk in tickets]
            for tk in tickets:
                srv.release(tk)
        stop.set()
        th.join()
        mem = srv.memory()
    assert mem["peak_charged"] <= budget and held_max[0] <= budget, (mem, held_max[0])
    assert peak[0] <= budget + (128 << 20), f"device memory {peak[0] / 2**30:.2f} GiB over a {budget / 2**30} GiB budget"
    for k in range(0, len(trees), 6):
        w, tab = _alone(trees[k])
        _assert_same(outs[k], w, tab, f"request {k}")


def test_batch_program_failure_is_isolated(built_cuda):
    """A malformed tree fails alone (INVALID_AST); the other programs of the batch are
    still exact."""
    from conftest import ast_to_tree
    from ptilopsis_gb300.batch import BatchCompiler
    trees = _programs(9, seed0=0x50544CE0)
    bad = ast_to_tree(tree_to_ast(trees[4]))
    bad.parent = bad.parent.copy()
    bad.parent[3] = 1  # a parent before its child breaks post-order
    trees[4] = bad
    with BatchCompiler(workers=4) as b:
        b.compile(trees, check=False)
        assert b.status(4) == 1
        for k, t in enumerate(trees):
            if k == 4:
                continue
            assert b.status(k) == 0
            w, tab = _alone(t)
            _assert_same(b.result(k), w, tab, f"program {k}")


def test_batch_fixtures_and_serial_path(built_cuda):
    """The reference's fixtures in one batch, including the program whose functions share
    symbols (serial register allocation), against the golden words."""
    from conftest import ast_to_tree, load_fixture, manifest
    from ptilopsis_gb300.batch import BatchCompiler
    names = [f["name"] for f in manifest()["fixtures"]]
    trees, golds = [], []
    for nm in names:
        ast, gold = load_fixture(nm)
        trees.append(ast_to_tree(ast))
        golds.append(gold)
    with BatchCompiler(workers=4) as b:
        b.compile(trees)
        for k, nm in enumerate(names):
            res = b.result(k)
            np.testing.assert_array_equal(res.words, golds[k]["words"], err_msg=nm)
            np.testing.assert_array_equal(res.table["starts"], golds[k]["fn_start"], err_msg=nm)


def test_batch_tile_sizes_leave_results_unchanged(built_cuda, tmp_path, monkeypatch):
    """Every tile size the autotuner may pick gives the same words as the defaults; sizes
    the kernels do not take are refused; a tuned choice is cached per device and applied
    by the next compiler."""
    from ptilopsis_gb300 import PtlError
    from ptilopsis_gb300.batch import BatchCompiler, autotune, cached_tiles
    trees = _programs(12, seed0=0x50544CF0)
    with BatchCompiler(workers=4, tiles=None) as b:
        b.compile(trees)
        want = [b.words(k) for k in range(len(trees))]
        for elem, sweep in ((256, 512), (2048, 2048), (8192, 1024), (65536, 512)):
            b.set_tiles(elem, sweep)
            assert b.tiles() == (elem, sweep)
            b.compile(trees)
            for k in range(len(trees)):
                np.testing.assert_array_equal(b.words(k), want[k], err_msg=f"tiles {elem}/{sweep}, program {k}")
        for bad in ((1000, 1024), (128, 1024), (1024, 4096)):
            with pytest.raises(PtlError):
                b.set_tiles(*bad)
    monkeypatch.setenv("PTL_AUTOTUNE_CACHE", str(tmp_path / "autotune.json"))
    got = autotune(trees[:4], reps=1)
    assert cached_tiles() == (got["elem_tile"], got["sweep_tile"])
    with BatchCompiler(workers=2) as b:
        assert b.tiles() == (got["elem_tile"], got["sweep_tile"])


def _misaligned(tree):
    """The same tree with every array starting one element past a 16-byte boundary."""
    import dataclasses
    out = {}
    for f in ("type", "rtype", "parent", "depth", "child_idx", "data"):
        a = np.ascontiguousarray(getattr(tree, f))
        buf = np.empty(a.shape[0] + 16, a.dtype)
        off = 1
        while (buf[off:].ctypes.data % 16) == 0:
            off += 1
        buf[off:off + a.shape[0]] = a
        out[f] = buf[off:off + a.shape[0]]
        assert out[f].ctypes.data % 16 != 0
    return dataclasses.replace(tree, **out)


def test_batch_input_paths_agree(built_cuda, monkeypatch):
    """The inputs reach the device either by a kernel reading the caller's arrays (where
    the device reads pageable host memory; arrays off a 16-byte boundary take the byte
    path) or through pinned memory (PTL_HOST_GATHER=1); both give the same words."""
    from ptilopsis_gb300.batch import BatchCompiler
    trees = _programs(10, seed0=0x50544D00)
    odd = [_misaligned(t) if k % 2 else t for k, t in enumerate(trees)]
    with BatchCompiler(workers=4) as b:
        b.compile(trees)
        want = [b.words(k) for k in range(len(trees))]
        b.compile(odd)
        for k in range(len(trees)):
            np.testing.assert_array_equal(b.words(k), want[k], err_msg=f"program {k}, misaligned inputs")
    monkeypatch.setenv("PTL_HOST_GATHER", "1")
    with BatchCompiler(workers=4) as b:
        b.compile(odd)
        for k in range(len(trees)):
            np.testing.assert_array_equal(b.words(k), want[k], err_msg=f"program {k}, pinned gather")


def test_batch_poisoned_arenas(built_cuda, monkeypatch):
    """Arrays the stages write in full are not zeroed between compiles.  With
    PTL_POISON_ARENAS=1 their bytes are filled with 0xA5 before every compile (only the
    pads are cleared), so a stage that read one of them before writing it would change
    the words: every program still equals its plain compile, over two calls of different
    sizes and an invalid program."""
    from conftest import ast_to_tree
    from ptilopsis_gb300.batch import BatchCompiler
    monkeypatch.setenv("PTL_POISON_ARENAS", "1")
    first = _programs(12, seed0=0x50544D40)
    second = _programs(7, seed0=0x50544D60, max_fns=40)
    bad = ast_to_tree(tree_to_ast(second[2]))
    bad.max_depth = bad.max_depth + 1  # a depth with no node
    second[2] = bad
    with BatchCompiler(workers=4) as b:
        for trees in (first, second):
            b.compile(trees, check=False)
            for k, t in enumerate(trees):
                if t is bad:
                    assert b.status(k) == 1  # INVALID_AST
                    continue
                assert b.status(k) == 0
                w, tab = _alone(t)
                _assert_same(b.result(k), w, tab, f"program {k} ({t.n} nodes)")


def test_batch_regalloc_share_and_device_window(built_cuda):
    """A smaller share of resident blocks for the regalloc launch changes no word; the
    device window of a compile is positive and within its wall time."""
    from ptilopsis_gb300 import PtlError
    from ptilopsis_gb300.batch import BatchCompiler
    trees = _programs(10, seed0=0x50544DA0)
    with BatchCompiler(workers=4) as b:
        b.compile(trees)
        want = [b.words(k).copy() for k in range(len(trees))]
        for share in (0.5, 0.1):
            b.set_regalloc_share(share)
            b.compile(trees)
            for k in range(len(trees)):
                np.testing.assert_array_equal(b.words(k), want[k], err_msg=f"share {share} program {k}")
            assert 0 < b.device_ns() <= b.elapsed_ns()
        with pytest.raises(PtlError):
            b.set_regalloc_share(0.0)


def test_server_scalar_and_avx_requests_in_the_mix(built_cuda):
    """Requests for the scalar generator (PTL_SUBMIT_SCALAR) and for the AVX generator
    submitted interleaved to one server: batches hold one kind each, and every result
    equals the plain generator of its kind."""
    from ptilopsis_gb300 import RvGenerator
    from ptilopsis_gb300.batch import CompileServer
    trees = _programs(24, seed0=0x50544DE0)
    kinds = [k % 3 == 1 for k in range(len(trees))]
    with CompileServer(device=0, slots=3, memory_budget=8 << 30) as srv:
        tickets = [srv.submit(t, scalar=sc) for t, sc in zip(trees, kinds)]
        outs = [srv.result(t) for t in tickets]
        for t in tickets:
            srv.release(t)
    for k, (t, sc) in enumerate(zip(trees, kinds)):
        with RvGenerator(t, scalar=sc) as g:
            g.process()
            _assert_same(outs[k], g.get_instructions(), g.function_table(), f"request {k} scalar={sc}")
