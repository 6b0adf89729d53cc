"""The wall search reads one list per particle cell: the triangles whose cell box
(clamped to the grid), grown by one cell when it is not empty, holds the cell
(k_bin_count / k_bin_fill).  That list must be the union of the plain box lists of the
cell's 27 neighbours (the candidate set of a 27-cell search), each triangle once.
Checked here on random triangles over a small grid, including ones partly or wholly
outside it."""
import itertools

import numpy as np


def box_cells(lo, hi, cs, G, grow):
    # tri_cell_box: conversion toward zero (f2i), then clamped to the grid
    i0 = np.maximum(np.trunc(lo / cs).astype(int), 0)
    i1 = np.minimum(np.trunc(hi / cs).astype(int), G - 1)
    if (i0 > i1).any():
        return set()
    if grow:
        i0 = np.maximum(i0 - 1, 0)
        i1 = np.minimum(i1 + 1, G - 1)
    return set(itertools.product(*(range(a, b + 1) for a, b in zip(i0, i1))))


def test_halo_lists_equal_union_of_neighbour_box_lists():
    rng = np.random.default_rng(3)
    G = np.array([7, 6, 5])
    cs = 1.0
    tris = []
    for _ in range(300):
        c = rng.uniform(-1.5, G + 0.5)
        tris.append(c + rng.normal(0, rng.choice([0.2, 0.8, 2.0]), (3, 3)))
    plain = {c: set() for c in itertools.product(*(range(g) for g in G))}
    halo = {c: [] for c in plain}
    for t, v in enumerate(tris):
        lo, hi = v.min(0), v.max(0)
        for c in box_cells(lo, hi, cs, G, False):
            plain[c].add(t)
        for c in box_cells(lo, hi, cs, G, True):
            halo[c].append(t)
    for c in plain:
        union = set()
        for d in itertools.product((-1, 0, 1), repeat=3):
            n = tuple(np.add(c, d))
            if all(0 <= n[a] < G[a] for a in range(3)):
                union |= plain[n]
        assert sorted(halo[c]) == sorted(union), c
        assert len(halo[c]) == len(set(halo[c]))
    assert sum(len(v) for v in halo.values()) > sum(len(v) for v in plain.values())
