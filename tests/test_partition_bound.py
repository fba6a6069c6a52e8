"""The facts the GPU's partition rounds rely on, checked on the CPU against a direct
restatement of the Hoare partition's stop lists (libstdc++ __unguarded_partition after the
median move): with A the L-stop positions (keys >= pivot, from the left) and B the R-stop
positions (keys <= pivot, from the right), K = #{k: A[k] < B[k]} is at most
max(L-stops before x, R-stops from x on) at every position x, so the tile starts give a
bound from the tile counts alone; and the K swapped pairs touch disjoint positions (every
A[k] lies left of every B[k'])."""
from __future__ import annotations

import numpy as np


def stops(keys, pivot):
    pos = np.arange(1, keys.shape[0])  # the pivot sits at 0
    body = keys[1:]
    A = pos[body >= pivot]
    B = pos[body <= pivot][::-1]
    m = min(A.shape[0], B.shape[0])
    K = int(np.count_nonzero(A[:m] < B[:m]))
    return A, B, K


def tile_bound(keys, pivot, tile):
    body = keys[1:]
    isL = (body >= pivot).astype(np.int64)
    isR = (body <= pivot).astype(np.int64)
    nL, nR = int(isL.sum()), int(isR.sum())
    bound = nL  # the end of the range
    for t0 in range(0, body.shape[0], tile):
        bound = min(bound, max(int(isL[:t0].sum()), nR - int(isR[:t0].sum())))
    return bound


def test_pair_count_bound_and_disjoint_swaps():
    rng = np.random.default_rng(0x50544F10)
    for case in range(300):
        n = int(rng.integers(3, 3000))
        distinct = int(rng.integers(1, 60))
        keys = rng.integers(0, distinct, n)
        if case % 3 == 0:  # depth-like: one dominant value
            keys[rng.random(n) < 0.7] = int(rng.integers(0, distinct))
        pivot = int(np.median(keys[[1, n // 2, n - 1]]))  # some key of the range
        keys[0] = pivot
        A, B, K = stops(keys, pivot)
        for tile in (1, 7, 64, 2048):
            assert K <= tile_bound(keys, pivot, tile), (case, tile)
        if K:
            assert A[K - 1] < B[K - 1] and A[:K].max() < B[:K].min(), case
