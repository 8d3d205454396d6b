"""The oracle's own CPU checks that no golden fixture covers: the float64 CG
and the bin-permutation restatement (structure and invariants)."""

import numpy as np
import torch

from oracle import binning as OB
from oracle import cg as OCG


def test_float64_cg_solves_spd():
    gen = torch.Generator().manual_seed(0)
    n = 80
    Q, _ = torch.linalg.qr(torch.randn(n, n, dtype=torch.float64, generator=gen))
    M = (Q * torch.logspace(0, 3, n, dtype=torch.float64)) @ Q.T
    xt = torch.randn(n, dtype=torch.float64, generator=gen)
    x, it = OCG.cg(lambda v: M @ v, M @ xt, rtol=1e-12)
    assert it <= 3 * n  # finite precision: a few sweeps past n at condition 1e3
    assert torch.linalg.vector_norm(x - xt) / torch.linalg.vector_norm(xt) < 1e-8


def test_binning_invariants():
    gen = torch.Generator().manual_seed(1)
    locs = torch.rand(3000, 3, generator=gen) * 40 - 4
    keys, pts = OB.plan_pairs(locs, (32, 32, 32), 4.0)
    assert np.all(np.diff(keys) >= 0)  # sorted by key
    same = np.diff(keys) == 0
    assert np.all(np.diff(pts)[same] > 0)  # stable: point order inside a key
    home = keys % 2 == 0
    assert len(np.unique(pts[home])) == home.sum() == 3000  # one home pair per point (circular)
    # a W=4 window spans at most 2 tiles of 8 per axis: at most 8 pairs per point
    assert np.bincount(pts).max() <= 8
    assert 2.0 < len(keys) / 3000 < 4.0
