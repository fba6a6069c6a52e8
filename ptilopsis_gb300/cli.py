"""Command line of the reference (src/main.cpp:35-157) over the GPU generator.

    python -m ptilopsis_gb300 <infile> [-S] [-o <outfile>] [-dp] [-t <threads>] [-m <sync>] [-b] [-i <mininstr>]

The reference reads Pareas source and flattens it with its front end; the GPU generator's
boundary is the flattened tree, so <infile> is a DepthTree saved as .npz (arrays type,
rtype, parent, depth, child_idx, data and the scalar max_depth, as save_tree writes
them), or - for the same bytes on stdin.  A file without depth and max_depth holds the
parser's tree in any node order (parent -1 for the root, child_idx the place among the
parent's children; save_unordered writes it): it is flattened on the GPU first
(ptl_flatten, the reference's DepthTree construction).  Output as the reference writes it: raw 32-bit
words (to_binary) to ./c.out, or with -S assembly text (to_asm) to <infile stem>.s; -o -
writes to stdout.  -p prints the reference's profiling CSV (stage names, then
nanoseconds; src/codegen/rv_generator.cpp:150-162) with the GPU's per-stage device times.
--elf <file> also writes the program as an ELF64 RISC-V relocatable object (an option the
reference does not have; ptl_write_elf).  -t, -m, -b and -i set how the reference
schedules its CPU threads; they are accepted and have no effect here.  -s selects the
scalar generator's semantics (rv_generator_st, main.cpp:123-124), also on the GPU.
"""
from __future__ import annotations

import argparse
import io
import os
import sys
from typing import List, Optional

import numpy as np

FIELDS = ("type", "rtype", "parent", "depth", "child_idx", "data")


def save_tree(tree, path_or_file) -> None:
    """Writes a DepthTree as the .npz the command line reads."""
    np.savez(path_or_file, max_depth=np.int64(tree.max_depth),
             **{f: np.ascontiguousarray(getattr(tree, f)) for f in FIELDS})


UNORDERED = ("type", "rtype", "parent", "child_idx", "data")


def save_unordered(type_, rtype, parent, child_idx, data, path_or_file) -> None:
    """Writes a parser's tree in any node order (no depth) as the .npz the command line
    flattens before compiling."""
    np.savez(path_or_file, type=np.ascontiguousarray(type_, np.uint8), rtype=np.ascontiguousarray(rtype, np.uint8),
             parent=np.ascontiguousarray(parent, np.int32), child_idx=np.ascontiguousarray(child_idx, np.int32),
             data=np.ascontiguousarray(data, np.uint32))


def load_tree(path_or_file, device: int = 0):
    from .codegen import DepthTree
    z = np.load(path_or_file)
    dt = {"type": np.uint8, "rtype": np.uint8, "parent": np.int32, "depth": np.int32, "child_idx": np.int32,
          "data": np.uint32}
    if "depth" not in z.files:
        from .codegen import flatten
        return flatten(*(np.ascontiguousarray(z[f], dt[f]) for f in UNORDERED), device=device)[0]
    return DepthTree(max_depth=int(z["max_depth"]), **{f: np.ascontiguousarray(z[f], dt[f]) for f in FIELDS})


def _parser() -> argparse.ArgumentParser:
    ap = argparse.ArgumentParser(prog="ptilopsis_gb300", description="GB300 RISC-V code generator (drop-in for "
                                 "Ptilopsis' rv_generator_avx)")
    ap.add_argument("infile", help="flattened tree (.npz from save_tree), - for stdin")
    ap.add_argument("-S", dest="asm", action="store_true", help="output assembly instead of machine code")
    ap.add_argument("-o", dest="outfile", help="output filename (default: ./c.out, or <infile>.s with -S; - for stdout)")
    ap.add_argument("-d", "--debug", action="store_true", help="print tree and output sizes")
    ap.add_argument("-s", "--simple", action="store_true", help="use the scalar generator's semantics")
    ap.add_argument("-f", "--tree", action="store_true", help="print tree info")
    ap.add_argument("-t", "--threads", type=int, default=-1, help="accepted for compatibility; no effect")
    ap.add_argument("-m", "--sync", type=int, default=0, help="accepted for compatibility; no effect")
    ap.add_argument("-b", "--altblock", action="store_true", help="accepted for compatibility; no effect")
    ap.add_argument("-i", "--mininstr", type=int, default=0, help="accepted for compatibility; no effect")
    ap.add_argument("-p", "--profile", action="store_true", help="profiling CSV to stdout")
    ap.add_argument("--device", type=int, default=0, help="CUDA device")
    ap.add_argument("--elf", dest="elf", help="also write an ELF64 RISC-V relocatable object (one symbol per function)")
    return ap


def profile_csv(stage_names: List[str], stage_ns: List[int]) -> str:
    """The reference's -p output: the names, then the nanoseconds, comma-separated."""
    return ",".join(stage_names) + "\n" + ",".join(str(int(v)) for v in stage_ns) + "\n"


def main(argv: Optional[List[str]] = None) -> int:
    args = _parser().parse_args(argv)
    if args.infile == "-":
        src = io.BytesIO(sys.stdin.buffer.read())
    elif not os.path.exists(args.infile):
        print(f"Failed to open file {args.infile}", file=sys.stderr)
        return 1
    else:
        src = args.infile
    tree = load_tree(src, device=args.device)
    outfile = args.outfile
    if outfile is None:
        outfile = (os.path.splitext(os.path.basename(args.infile))[0] + ".s") if args.asm else "c.out"

    from .codegen import STAGES, RvGenerator
    with RvGenerator(tree, device=args.device, scalar=args.simple) as gen:
        gen.process(profile=True)
        if args.profile:
            sys.stdout.write(profile_csv(STAGES, gen.stage_ns()))
            sys.stdout.flush()
        if args.debug or args.tree:
            words = gen.get_instructions()
            print(f"Number of nodes: {tree.n}\nMax depth: {tree.max_depth}\nOutput words: {len(words)}")
        if args.elf:
            with open(args.elf, "wb") as f:
                f.write(gen.to_elf())
        if outfile == "-":
            if args.asm:
                sys.stdout.write(gen.to_asm())
            else:
                gen.to_binary(sys.stdout.buffer)
            sys.stdout.flush()
        elif args.asm:
            with open(outfile, "w") as f:
                f.write(gen.to_asm())
        else:
            with open(outfile, "wb") as f:
                gen.to_binary(f)
    return 0
