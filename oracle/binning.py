"""CPU oracle of the plan's bin permutation (TEST INFRASTRUCTURE ONLY).

The reference has no binning step: its Triton kernels walk the points in
their original order (``functional/_interp/grid.py:169-520``). The GPU plan
instead sorts (point, tile) pairs so that each CTA owns one output tile. This
restates, independently of the CUDA code, which pairs exist and their order:

* taps of each axis follow the reference window (``axis_taps`` in
  ``oracle.interp``: ``lower = ceil(x - W/2)``, taps ``lower + k`` with
  ``|d| <= W/2`` and, for Kaiser-Bessel, ``|d| <= 1``; zero padding drops
  taps outside ``[0, N)``, circular padding wraps them);
* tiles are 8^3 in 3D, 16 x 16 in 2D and 512 in 1D (clipped to the grid),
  numbered ``(t0 * nt1 + t1) * nt2 + t2`` over internal dims padded to 3;
* a point pairs with every tile that one of its valid taps lands in (the
  product of the distinct tiles per axis, at most 3 per axis); its home pair
  is the tile of its first valid tap on every axis;
* points with a non-finite coordinate or one beyond 2^24 in magnitude have no
  pairs (the GPU treats them as having no taps);
* pairs are ordered by ``key = 2 * tile + (0 if home else 1)`` and, for equal
  keys, by point index (a stable sort of the pairs in point order).

Plans of the 8-entry gridding also list (point, block) pairs for output
blocks of 4 x 4 x 4 cells (3D) or 8 x 8 cells (2D) (``block_pairs``): a point
pairs with every block that one of its valid taps lands in, keyed
``(b0 * nb1 + b1) * nb2 + b2``,
in point order within a block. Each pair is stored as
``point | (i0 | i1 << 1 | i2 << 2) << 29``, i_e the index of the block among
the point's blocks along dim e in window order.
"""

from __future__ import annotations

import math

import numpy as np
import torch

from .interp import axis_taps

__all__ = ["tile_shape", "plan_pairs", "block_pairs"]


def tile_shape(grid_size):
    nd = len(grid_size)
    N = (1,) * (3 - nd) + tuple(int(n) for n in grid_size)
    T = {3: (8, 8, 8), 2: (1, 16, 16), 1: (1, 1, 512)}[nd]
    T = tuple(min(t, n) for t, n in zip(T, N))
    nt = tuple(-(-n // t) for n, t in zip(N, T))
    return N, T, nt


def plan_pairs(locs: torch.Tensor, grid_size, width, kernel: str = "kaiser_bessel", pad_mode: str = "circular"):
    """(keys, points): the sorted pair keys and the point index of each pair."""
    nd = len(grid_size)
    N, T, nt = tile_shape(grid_size)
    x = locs.reshape(-1, nd).to(torch.float32)
    P = x.shape[0]
    widths = width if isinstance(width, (tuple, list)) else (width,) * nd
    ok = torch.isfinite(x).all(-1) & (x.abs() < 16777216.0).all(-1)
    tiles = []  # per internal dim: [P, 3] distinct tiles in order of first appearance, -1 = none
    for e in range(3):
        if e < 3 - nd:
            t = torch.full((P, 3), -1, dtype=torch.int64)
            t[:, 0] = 0
            tiles.append(t)
            continue
        a = e - (3 - nd)
        g, _, valid = axis_taps(x[:, a], float(widths[a]), kernel, torch.float32)
        if pad_mode == "zero":
            valid = valid & (g >= 0) & (g < N[e])
        pos = torch.remainder(g, N[e]) if pad_mode == "circular" else g
        tl = torch.div(pos, T[e], rounding_mode="floor")
        out = torch.full((P, 3), -1, dtype=torch.int64)
        cnt = torch.zeros(P, dtype=torch.int64)
        for k in range(g.shape[1]):
            tk = tl[:, k]
            seen = (out == tk[:, None]).any(-1)
            add = valid[:, k] & ~seen & (cnt < 3)
            idx = torch.nonzero(add).flatten()
            out[idx, cnt[idx]] = tk[idx]
            cnt = cnt + add.to(torch.int64)
        tiles.append(out)
    keys, pts = [], []
    pidx = torch.arange(P)
    for i0 in range(3):
        for i1 in range(3):
            for i2 in range(3):
                t0, t1, t2 = tiles[0][:, i0], tiles[1][:, i1], tiles[2][:, i2]
                m = ok & (t0 >= 0) & (t1 >= 0) & (t2 >= 0)
                # a point has pairs only if every axis has a valid tap
                m = m & (tiles[0][:, 0] >= 0) & (tiles[1][:, 0] >= 0) & (tiles[2][:, 0] >= 0)
                lin = (t0 * nt[1] + t1) * nt[2] + t2
                nonhome = 0 if (i0, i1, i2) == (0, 0, 0) else 1
                keys.append((2 * lin + nonhome)[m])
                pts.append(pidx[m])
    keys = torch.cat(keys).numpy()
    pts = torch.cat(pts).numpy()
    order = np.lexsort((pts, keys))
    return keys[order], pts[order]


def block_pairs(locs: torch.Tensor, grid_size, width, kernel: str = "kaiser_bessel", pad_mode: str = "circular"):
    """(keys, entries) of the block lists: every (point, block) pair for
    blocks of 4 x 4 x 4 cells (3D) or 8 x 8 cells (2D), sorted by block key
    and, within a block, by point index; entries as stored by the plan (point
    index and the block's index per internal dim; a 2D grid's leading
    internal dim has one block)."""
    nd = len(grid_size)
    assert nd in (2, 3)
    N = (1,) * (3 - nd) + tuple(int(n) for n in grid_size)
    edge = (4, 4, 4) if nd == 3 else (1, 8, 8)
    nb = tuple(-(-n // b) for n, b in zip(N, edge))
    x = locs.reshape(-1, nd).to(torch.float32)
    P = x.shape[0]
    widths = width if isinstance(width, (tuple, list)) else (width,) * nd
    ok = torch.isfinite(x).all(-1) & (x.abs() < 16777216.0).all(-1)
    blocks = []  # per internal dim: [P, 3] distinct blocks, -1 = none
    for e in range(3):
        if e < 3 - nd:
            t = torch.full((P, 3), -1, dtype=torch.int64)
            t[:, 0] = 0
            blocks.append(t)
            continue
        a = e - (3 - nd)
        g, _, valid = axis_taps(x[:, a], float(widths[a]), kernel, torch.float32)
        if pad_mode == "zero":
            valid = valid & (g >= 0) & (g < N[e])
        pos = torch.remainder(g, N[e]) if pad_mode == "circular" else g
        bl = torch.div(pos, edge[e], rounding_mode="floor")
        out = torch.full((P, 3), -1, dtype=torch.int64)
        cnt = torch.zeros(P, dtype=torch.int64)
        for k in range(g.shape[1]):
            bk = bl[:, k]
            seen = (out == bk[:, None]).any(-1)
            add = valid[:, k] & ~seen & (cnt < 3)
            idx = torch.nonzero(add).flatten()
            out[idx, cnt[idx]] = bk[idx]
            cnt = cnt + add.to(torch.int64)
        blocks.append(out)
    keys, pts, sels = [], [], []
    pidx = torch.arange(P)
    for i0 in range(3):
        for i1 in range(3):
            for i2 in range(3):
                b0, b1, b2 = blocks[0][:, i0], blocks[1][:, i1], blocks[2][:, i2]
                m = ok & (b0 >= 0) & (b1 >= 0) & (b2 >= 0)
                keys.append(((b0 * nb[1] + b1) * nb[2] + b2)[m])
                pts.append(pidx[m])
                sels.append(torch.full((int(m.sum()),), i0 | i1 << 1 | i2 << 2, dtype=torch.int64))
    keys = torch.cat(keys).numpy()
    pts = torch.cat(pts).numpy()
    sels = torch.cat(sels).numpy()
    order = np.lexsort((pts, keys))  # by block, then by point
    return keys[order], pts[order] | (sels[order] << 29)
