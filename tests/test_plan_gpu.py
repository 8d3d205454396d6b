"""The plan's bin permutation, bit-exact against the CPU oracle
(oracle/binning.py): every (point, tile) pair, ordered by tile, home pairs
first, then by point index; and in 2D and 3D the (point, block) lists of the
gridding, ordered by block, then by point index, with their work items and
split blocks. Sizes large enough for the multi-CTA scans."""

import numpy as np
import pytest
import torch

from oracle import binning as OB

from torchlinops_gb300 import interp

pytestmark = pytest.mark.gpu
DEV = "cuda"

CASES = [
    ((40, 36, 48), 60000, "circular"),
    ((40, 36, 45), 60000, "zero"),
    ((200, 150), 50000, "circular"),
    ((5000,), 40000, "zero"),
]


def _entries(plan) -> np.ndarray:
    off, n = int(plan.info.off_entries), int(plan.info.n_entries)
    return plan.buffer[off:off + 4 * n].view(torch.int32).cpu().numpy()


@pytest.mark.parametrize("grid_size,npts,pad", CASES)
def test_plan_permutation_is_bit_exact(grid_size, npts, pad):
    gen = torch.Generator().manual_seed(npts + len(grid_size))
    n = torch.tensor(grid_size, dtype=torch.float32)
    locs = torch.rand(npts, len(grid_size), generator=gen) * (n + 6) - 3  # past both edges
    locs[:500] = torch.randint(0, 30, (500, len(grid_size)), generator=gen).float()  # exact integers
    locs[500:520, 0] = float("nan")  # no taps
    keys, pts = OB.plan_pairs(locs, grid_size, 4.0, "kaiser_bessel", pad)
    plan = interp.get_plan(locs.to(DEV), grid_size, 4.0, "kaiser_bessel", pad, 6.99666)
    got = _entries(plan)
    assert got.shape == pts.shape
    assert np.array_equal(got, pts)
    # home pairs: one per point with taps
    assert int(plan.info.n_home) == int((keys % 2 == 0).sum())


BLOCK_CASES = [c for c in CASES if len(c[0]) == 3] + [((200, 144), 50000, "circular"), ((190, 150), 40000, "zero")]


@pytest.mark.parametrize("grid_size,npts,pad", BLOCK_CASES)
def test_block_lists_are_bit_exact(grid_size, npts, pad):
    gen = torch.Generator().manual_seed(npts + 7)
    nd = len(grid_size)
    n = torch.tensor(grid_size, dtype=torch.float32)
    locs = torch.rand(npts, nd, generator=gen) * (n + 6) - 3
    locs[:500] = torch.randint(0, 30, (500, nd), generator=gen).float()  # exact integers: 5 taps
    locs[500:520, 1] = float("inf")
    locs[520:6520] = 10 + 2 * torch.rand(6000, nd, generator=gen)  # dense blocks, split into parts
    keys, pts = OB.block_pairs(locs, grid_size, 4.0, "kaiser_bessel", pad)
    plan = interp.get_plan(locs.to(DEV), grid_size, 4.0, "kaiser_bessel", pad, 6.99666)
    info = plan.info
    assert int(info.n_blk_entries) == len(pts) and int(info.n_blk_items) > 0
    off = int(info.off_blk_entries)
    got = plan.buffer[off:off + 4 * len(pts)].view(torch.int32).cpu().numpy().astype(np.int64) & 0xFFFFFFFF
    assert np.array_equal(got, pts)  # point index and block index per dim
    # work items: each block's entries exactly once, split into parts of at most 256
    items = plan.buffer[int(info.off_blk_items):int(info.off_blk_items) + 16 * int(info.n_blk_items)]
    items = items.view(torch.int32).reshape(-1, 4).cpu().numpy()
    full = items[items[:, 1] < items[:, 2]]
    assert (full[:, 2] - full[:, 1]).max() <= 256
    cover = np.zeros(len(pts), dtype=np.int64)
    for b, s0, s1, _ in full:
        assert np.all(keys[s0:s1] == b)
        cover[s0:s1] += 1
    assert np.all(cover == 1)
    # split blocks: listed by falling part count; their partial slots are the
    # parts' slots, each used once
    nsp = int(info.n_blk_split)
    if nsp > 0:
        off_sp = int(info.off_blk_split)
        sp = plan.buffer[off_sp:off_sp + 16 * nsp].view(torch.int32).reshape(-1, 4).cpu().numpy()
        assert np.all(np.diff(sp[:, 2]) <= 0)
        slots = np.concatenate([np.arange(a, a + c) for a, c in zip(sp[:, 1], sp[:, 2])])
        assert np.array_equal(np.sort(slots), np.arange(int(info.n_blk_partials)))
        parts = items[items[:, 3] >= 0]
        assert np.array_equal(np.sort(parts[:, 3]), np.arange(int(info.n_blk_partials)))
    assert nsp > 0
    # empty runs and non-empty items together name every block once
    nb = int(np.prod([-(-s // (4 if nd == 3 else 8)) for s in grid_size]))
    named = np.zeros(nb, dtype=np.int64)
    for b, s0, s1, w in items:
        if s0 == s1:
            named[b:b - w] += 1
        elif w < 0 or s0 == keys.searchsorted(b):
            named[b] += 1
    assert np.all(named == 1)
