"""The plan's bin permutation, bit-exact against the CPU oracle
(oracle/binning.py): every (point, tile) pair, ordered by tile, home pairs
first, then by point index. Sizes large enough for the multi-CTA scans."""

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
