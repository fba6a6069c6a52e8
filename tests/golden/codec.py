"""Compact storage of the large fixture trees (test infrastructure).

A post-order DepthTree is fully determined by each node's type, result type, data and
number of children: in post-order a node's children are the last subtrees completed
before it, so a stack rebuilds parent and child index, and depth follows from the
parents (pareas-ast/src/codegen/depthtree.cpp:52-100 emits exactly this order).  The
four arrays are stored as an lzma-compressed .npz; the manifest keeps a CRC32 of each of
the six full arrays, and decoding checks them, so a decoded tree is the tree the
reference front end built.
"""
from __future__ import annotations

import io
import lzma
import zlib

import numpy as np


def crc(a) -> int:
    return zlib.crc32(np.ascontiguousarray(a).tobytes())


def tree_crcs(type_, rtype, parent, depth, child_idx, data) -> dict:
    return {"type": crc(np.asarray(type_, np.uint8)), "rtype": crc(np.asarray(rtype, np.uint8)),
            "parent": crc(np.asarray(parent, np.int32)), "depth": crc(np.asarray(depth, np.int32)),
            "child_idx": crc(np.asarray(child_idx, np.int32)), "data": crc(np.asarray(data, np.uint32))}


def encode(type_, rtype, parent, data) -> bytes:
    n = len(type_)
    par = np.asarray(parent, np.int64)
    nch = np.bincount(par[par >= 0], minlength=n)
    dt = np.uint8 if nch.max(initial=0) < 256 else (np.uint16 if nch.max() < 65536 else np.uint32)
    buf = io.BytesIO()
    np.savez(buf, type=np.asarray(type_, np.uint8), rtype=np.asarray(rtype, np.uint8), nch=nch.astype(dt),
             data=np.asarray(data, np.uint32))
    return lzma.compress(buf.getvalue(), preset=9 | lzma.PRESET_EXTREME)


def decode(blob: bytes):
    """(type, rtype, parent, depth, child_idx, data) of an encoded post-order tree."""
    z = np.load(io.BytesIO(lzma.decompress(blob)))
    type_, rtype, nch, data = z["type"], z["rtype"], z["nch"], z["data"]
    n = len(type_)
    parent = np.full(n, -1, np.int32)
    child_idx = np.full(n, -1, np.int32)
    stack: list[int] = []
    for i, k in enumerate(nch.tolist()):
        if k:
            kids = stack[-k:]
            del stack[-k:]
            parent[kids] = i
            child_idx[kids] = np.arange(k, dtype=np.int32)
        stack.append(i)
    if len(stack) != 1:
        raise ValueError(f"encoded tree has {len(stack)} roots")
    # parents have larger indices than their children: one pass from the root down
    depth = np.zeros(n, np.int32)
    par = parent.tolist()
    dl = depth.tolist()
    for i in range(n - 2, -1, -1):
        dl[i] = dl[par[i]] + 1
    depth = np.asarray(dl, np.int32)
    return type_, rtype, parent, depth, child_idx, data
