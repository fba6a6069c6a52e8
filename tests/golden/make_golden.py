"""Regenerates the golden fixtures of tests/golden from the reference itself.

Run in the x86-64 build container, where the reference tree is mounted and
oracle/ref/Makefile has built it into oracle/_ref:

    python tests/golden/make_golden.py            # small fixtures, synthetic seeds, tables
    python tests/golden/make_golden.py --large    # the reference's larger Pareas inputs
    python tests/golden/make_golden.py --scalar   # the scalar generator (rv_generator_st)
    python tests/golden/make_golden.py --scalar-large   # ... on the larger Pareas inputs

For each fixture it stores the DepthTree the reference front end (pareas-ast) builds
from one of the reference's own Pareas test inputs, and what the reference generator
(rv_generator_avx with one worker thread) produces from it: the output words, the
function table, and a CRC32 of every intermediate array.  Seeded synthetic programs
store only the outputs (their trees are regenerated from the seed).  The code tables
are stored as CRC32s of the reference's constexpr arrays.  --scalar runs the reference's
scalar generator (rv_generator_st, the -s flag) on the same trees and on seeded programs
of the batched workload's shape, and stores the outputs of the first two kinds in
scalar_words.npz and the CRCs of every stage array in manifest_scalar.json.
"""
from __future__ import annotations

import json
import os
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import refbind  # noqa: E402

REF = refbind.ref_root_cached()
FIXTURES = [
    "testfiles/pareas/basic/1.in",
    "testfiles/pareas/basic/2.in",
    "testfiles/pareas/basic/3.in",
    "testfiles/arith1.ptl",
    "testfiles/basic1.ptl",
    "testfiles/comp0.ptl",
    "testfiles/comp1.ptl",
    "testfiles/comp_all.ptl",
    "testfiles/many_args.in",
]
SYNTH_SEEDS = [0x50544C00, 0x50544C00 + 1, 0x50544C00 + 2]


def crc(a: np.ndarray) -> int:
    return zlib.crc32(np.ascontiguousarray(a, np.uint32).tobytes())


def table_crcs() -> dict:
    import ctypes
    L = refbind.lib()
    L.ptlref_table.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_uint32)]
    L.ptlref_table.restype = ctypes.c_size_t
    out = {}
    for w in range(10):
        n = L.ptlref_table(w, None)
        a = np.empty(n, np.uint32)
        L.ptlref_table(w, a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
        out[str(w)] = [int(n), crc(a)]
    return out


# The reference's larger Pareas inputs (testfiles/pareas; basic/6,7 and shape/1,2 are not
# shipped).  Their trees are kept in the compact form of codec.py, their outputs as CRCs:
# the reference takes minutes per shape/* input at one worker thread, the restatement and
# the GPU a second, so the tests recompute the outputs and compare CRCs.
LARGE = (["basic/4", "basic/5"] + [f"funclen/{i}" for i in range(1, 9)] + [f"shape/{i}" for i in range(3, 7)])


def _large_one(rel: str) -> dict:
    import time
    sys.path.insert(0, HERE)
    import codec
    t0 = time.time()
    ast = refbind.parse_file(os.path.join(REF, "testfiles/pareas", rel + ".in"))
    res = refbind.compile_ast(ast, threads=1, snapshots=True)
    name = "pareas_" + rel.replace("/", "_")
    with open(os.path.join(HERE, "large", name + ".tree.xz"), "wb") as f:
        f.write(codec.encode(ast.type, ast.rtype, ast.parent, ast.data))
    return {"name": name, "source": f"testfiles/pareas/{rel}.in", "n": int(ast.n), "max_depth": int(ast.max_depth),
            "tree_crcs": codec.tree_crcs(ast.type, ast.rtype, ast.parent, ast.depth, ast.child_idx, ast.data),
            "words": int(len(res.words)), "n_funcs": int(len(res.bufs["fn_id"])),
            "snapshots": {k: [int(len(v)), crc(v)] for k, v in res.bufs.items()},
            "reference_s": round(time.time() - t0, 1)}


def main_large() -> None:
    import multiprocessing as mp
    if not refbind.build(REF):
        raise SystemExit("the reference could not be built here (needs the reference tree on x86-64)")
    os.makedirs(os.path.join(HERE, "large"), exist_ok=True)
    # longest first (shape/* run minutes in the reference's register allocation)
    order = sorted(LARGE, key=lambda r: (not r.startswith("shape"), r))
    with mp.get_context("spawn").Pool(max(1, min(len(order), (os.cpu_count() or 2) - 1))) as pool:
        entries = {}
        for e in pool.imap_unordered(_large_one, order):
            entries[e["name"]] = e
            print(f"{e['source']}: {e['n']} nodes -> {e['words']} words ({e['reference_s']} s)", flush=True)
    out = {"fixtures": [entries["pareas_" + r.replace("/", "_")] for r in LARGE]}
    with open(os.path.join(HERE, "manifest_large.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)


def main() -> None:
    if not refbind.build(REF):
        raise SystemExit("the reference could not be built here (needs the reference tree on x86-64)")
    manifest = {"fixtures": [], "synthetic": [], "tables": table_crcs()}
    for rel in FIXTURES:
        ast = refbind.parse_file(os.path.join(REF, rel))
        res = refbind.compile_ast(ast, snapshots=True)
        name = rel.replace("testfiles/", "").replace("/", "_").replace(".", "_")
        np.savez_compressed(os.path.join(HERE, name + ".npz"),
                            type=ast.type, rtype=ast.rtype, parent=ast.parent, depth=ast.depth,
                            child_idx=ast.child_idx, data=ast.data, max_depth=np.int64(ast.max_depth),
                            words=res.bufs["out_words"], fn_start=res.bufs["fn_start"], fn_end=res.bufs["fn_end"],
                            fn_size=res.bufs["fn_size"], fn_id=res.bufs["fn_id"])
        snaps = {k: [int(len(v)), crc(v)] for k, v in res.bufs.items()}
        manifest["fixtures"].append({"name": name, "source": rel, "n": int(ast.n), "words": int(len(res.words)),
                                     "snapshots": snaps})
        print(f"{rel}: {ast.n} nodes -> {len(res.words)} words")

    from ptilopsis_gb300.synth import SynthParams, generate
    for seed in SYNTH_SEEDS:
        tree = generate(SynthParams(seed=seed))
        ast = refbind.Ast(tree.type, tree.rtype, tree.parent, tree.depth, tree.child_idx, tree.data, tree.max_depth)
        res = refbind.compile_ast(ast, snapshots=True)
        name = f"synth_c0_{seed:08x}"
        np.savez_compressed(os.path.join(HERE, name + ".npz"), words=res.bufs["out_words"],
                            fn_start=res.bufs["fn_start"], fn_end=res.bufs["fn_end"], fn_size=res.bufs["fn_size"],
                            fn_id=res.bufs["fn_id"])
        manifest["synthetic"].append({"name": name, "seed": seed, "n": int(ast.n),
                                      "tree_crc": [crc(tree.type.astype(np.uint32)), crc(tree.parent.view(np.uint32)),
                                                   crc(tree.data)],
                                      "words": int(len(res.words)),
                                      "snapshots": {k: [int(len(v)), crc(v)] for k, v in res.bufs.items()}})
        print(f"synthetic seed {seed:#x}: {ast.n} nodes -> {len(res.words)} words")
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)


# Seeded programs of the batched workload (program k of config c3) for the scalar
# generator, the ones of at most SCALAR_C3_MAX_NODES nodes among the first SCALAR_C3.
SCALAR_C3 = 24
SCALAR_C3_MAX_NODES = 60000


def main_scalar() -> None:
    if not refbind.build(REF):
        raise SystemExit("the reference could not be built here (needs the reference tree on x86-64)")
    from ptilopsis_gb300.synth import SynthParams, config_params, generate
    cases = []
    for rel in FIXTURES:
        name = rel.replace("testfiles/", "").replace("/", "_").replace(".", "_")
        cases.append((name, {"fixture": name}, refbind.parse_file(os.path.join(REF, rel))))
    for seed in SYNTH_SEEDS:
        t = generate(SynthParams(seed=seed))
        cases.append((f"synth_c0_{seed:08x}", {"seed": seed},
                      refbind.Ast(t.type, t.rtype, t.parent, t.depth, t.child_idx, t.data, t.max_depth)))
    for k in range(SCALAR_C3):
        t = generate(config_params("c3", program=k))
        if t.n > SCALAR_C3_MAX_NODES:
            continue
        cases.append((f"c3_program_{k}", {"c3_program": k},
                      refbind.Ast(t.type, t.rtype, t.parent, t.depth, t.child_idx, t.data, t.max_depth)))
    words = {}
    manifest = {"fixtures": []}
    for name, origin, ast in cases:
        res = refbind.compile_ast_scalar(ast, snapshots=True)
        if "c3_program" not in origin:  # the seeded workload programs keep CRCs only
            for k in ("out_words", "fn_start", "fn_end", "fn_size", "fn_id"):
                words[f"{name}.{k}"] = res.bufs[k]
        manifest["fixtures"].append({"name": name, **origin, "n": int(ast.n), "words": int(len(res.bufs["out_words"])),
                                     "tree_crcs": [crc(np.asarray(ast.type, np.uint32)),
                                                   crc(np.asarray(ast.parent).view(np.uint32)), crc(ast.data)],
                                     "snapshots": {k: [int(len(v)), crc(v)] for k, v in res.bufs.items()}})
        print(f"{name}: {ast.n} nodes -> {len(res.bufs['out_words'])} words (scalar generator)")
    np.savez_compressed(os.path.join(HERE, "scalar_words.npz"), **words)
    with open(os.path.join(HERE, "manifest_scalar.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)


def _scalar_large_one(rel: str) -> dict:
    import time
    sys.path.insert(0, HERE)
    import codec
    name = "pareas_" + rel.replace("/", "_")
    with open(os.path.join(HERE, "large", name + ".tree.xz"), "rb") as f:
        arrs = codec.decode(f.read())
    entry = next(e for e in json.load(open(os.path.join(HERE, "manifest_large.json")))["fixtures"] if e["name"] == name)
    ast = refbind.Ast(*arrs, max_depth=entry["max_depth"])
    t0 = time.time()
    res = refbind.compile_ast_scalar(ast, snapshots=True)
    return {"name": name, "words": int(len(res.bufs["out_words"])),
            "snapshots": {k: [int(len(v)), crc(v)] for k, v in res.bufs.items()},
            "reference_s": round(time.time() - t0, 1)}


def main_scalar_large() -> None:
    """The scalar generator on the larger Pareas inputs (their trees as committed under
    large/), as many as finish: its register allocation copies every function's register
    state at every step, so the reference takes minutes per 100k nodes.  Each result is
    written as it arrives."""
    import multiprocessing as mp
    if not refbind.build(REF):
        raise SystemExit("the reference could not be built here (needs the reference tree on x86-64)")
    path = os.path.join(HERE, "manifest_scalar_large.json")
    out = {"fixtures": []}
    with mp.get_context("spawn").Pool(max(1, (os.cpu_count() or 2) - 1)) as pool:
        for e in pool.imap_unordered(_scalar_large_one, LARGE):
            out["fixtures"].append(e)
            out["fixtures"].sort(key=lambda x: x["name"])
            with open(path, "w") as f:
                json.dump(out, f, indent=1, sort_keys=True)
            print(f"{e['name']}: {e['words']} words ({e['reference_s']} s)", flush=True)


if __name__ == "__main__":
    if "--large" in sys.argv[1:]:
        main_large()
    elif "--scalar-large" in sys.argv[1:]:
        main_scalar_large()
    elif "--scalar" in sys.argv[1:]:
        main_scalar()
    else:
        main()
