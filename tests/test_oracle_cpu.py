"""The oracle's own CPU checks that no golden fixture covers: the float64 CG,
the bin-permutation restatement (structure and invariants), and FP64
identities of the interpolation, block and NUFFT restatements (adjoint
pairs, linearity, the Toeplitz normal against the explicit normal)."""

import numpy as np
import pytest
import torch

from oracle import binning as OB
from oracle import blocks as OBL
from oracle import cg as OCG
from oracle import interp as OI
from oracle import nufft as ON


def _vdot(a, b):
    return complex(torch.vdot(a.flatten().to(torch.complex128), b.flatten().to(torch.complex128)))


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


def test_block_list_invariants():
    gen = torch.Generator().manual_seed(2)
    locs = torch.rand(3000, 3, generator=gen) * 40 - 4
    keys, ent = OB.block_pairs(locs, (32, 32, 32), 4.0)
    pts = ent & ((1 << 29) - 1)
    assert np.all(np.diff(keys) >= 0)
    same = np.diff(keys) == 0
    assert np.all(np.diff(pts)[same] > 0)  # point order inside a block
    # a window of 4 (5 at exact integers) taps meets at most 2 blocks of 4 per axis
    assert np.bincount(pts).max() <= 8 and (ent >> 29).max() <= 7
    assert 4.5 < len(keys) / 3000 < 6.0  # 1.75^3 = 5.36 blocks per point on average
    # every point's blocks contain its taps: one block holds its first tap on each axis
    kt, pt = OB.plan_pairs(locs, (32, 32, 32), 4.0)
    assert np.array_equal(np.unique(pts), np.unique(pt))


@pytest.mark.parametrize("pad", ["circular", "zero"])
def test_block_list_invariants_2d(pad):
    """2D blocks of 8 x 8 cells: a W = 4 window (5 taps at exact integers)
    meets at most 2 blocks per axis, so at most 4 per point, 1.9 on average
    for uniform points; the leading internal dim has one block (selector bit
    0 clear); every point with a valid tap has at least one block."""
    gen = torch.Generator().manual_seed(3)
    locs = torch.rand(4000, 2, generator=gen) * 70 - 3
    locs[:200] = torch.randint(0, 64, (200, 2), generator=gen).float()
    keys, ent = OB.block_pairs(locs, (64, 64), 4.0, pad_mode=pad)
    pts, sel = ent & ((1 << 29) - 1), ent >> 29
    assert np.all(np.diff(keys) >= 0)
    same = np.diff(keys) == 0
    assert np.all(np.diff(pts)[same] > 0)
    assert np.bincount(pts).max() <= 4 and np.all(sel & 1 == 0) and sel.max() <= 6
    assert keys.max() < 64 and 1.5 < len(keys) / len(np.unique(pts)) < 2.4
    kt, pt = OB.plan_pairs(locs, (64, 64), 4.0, pad_mode=pad)
    assert np.array_equal(np.unique(pts), np.unique(pt))


@pytest.mark.parametrize("shape", [(37,), (19, 23), (9, 10, 11)])
@pytest.mark.parametrize("kernel,norm", [("kaiser_bessel", 1), ("spline", 1), ("kaiser_bessel", 2)])
@pytest.mark.parametrize("pad", ["circular", "zero"])
def test_interp_oracle_adjoint_pair(shape, kernel, norm, pad):
    """<ungrid(x), y> = <x, grid(y)> in FP64, points anywhere including the
    edges (wrapped or cut) and exact-integer coordinates."""
    gen = torch.Generator().manual_seed(len(shape) * 10 + norm)
    nd = len(shape)
    locs = torch.rand(200, nd, generator=gen, dtype=torch.float64) * torch.tensor(shape, dtype=torch.float64)
    locs[:10] = torch.floor(locs[:10])
    x = torch.randn(2, *shape, dtype=torch.complex128, generator=gen)
    y = torch.randn(2, 200, dtype=torch.complex128, generator=gen)
    beta = OI.nufft_beta(4.0, 1.25)
    fx = OI.ungrid(x, locs, 4.0, kernel, norm, pad, beta, dtype=torch.float64)
    gy = OI.grid(y, locs, shape, 4.0, kernel, norm, pad, beta, dtype=torch.float64)
    lhs, rhs = _vdot(fx, y), _vdot(x, gy)
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


@pytest.mark.parametrize("shape,block,stride", [((15, 14), (3, 4), (2, 3)), ((10, 9, 8), (4, 3, 2), (2, 2, 2)), ((20,), (5,), (5,))])
def test_blocks_oracle_adjoint_pair_and_masking(shape, block, stride):
    """<unfold(x), y> = <x, fold(y)> exactly in FP64 (sums of products), with
    and without a mask; the mask keeps exactly its entries."""
    gen = torch.Generator().manual_seed(sum(shape))
    x = torch.randn(3, *shape, dtype=torch.float64, generator=gen)
    u = OBL.unfold(x, block, stride)
    y = torch.randn(u.shape, dtype=torch.float64, generator=gen)
    assert abs(float((u * y).sum() - (x * OBL.fold(y, shape, block, stride)).sum())) < 1e-10
    mask = torch.rand(block, generator=gen) > 0.4
    um = OBL.unfold(x, block, stride, mask)
    assert torch.equal(um, u[..., mask])
    ym = torch.randn(um.shape, dtype=torch.float64, generator=gen)
    assert abs(float((um * ym).sum() - (x * OBL.fold(ym, shape, block, stride, mask)).sum())) < 1e-10


@pytest.mark.parametrize("shape", [(16, 16), (12, 14), (8, 8, 8)])
def test_nufft_oracle_adjoint_pair(shape):
    gen = torch.Generator().manual_seed(len(shape) + shape[-1])
    locs = (torch.rand(120, len(shape), generator=gen, dtype=torch.float64) - 0.5) * torch.tensor(shape,
                                                                                                  dtype=torch.float64)
    x = torch.randn(*shape, dtype=torch.complex128, generator=gen)
    y = torch.randn(120, dtype=torch.complex128, generator=gen)
    lhs = _vdot(ON.nufft(x, locs), y)
    rhs = _vdot(x, ON.nufft_adjoint(y, locs, shape))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


def test_toeplitz_oracle_against_the_explicit_normal():
    """At sizes where 1.25 N is a whole number of cells the Toeplitz normal is
    the explicit nufft_adjoint(nufft(x)) up to the interpolation error of
    both (about 1%); linear in x; a point weighting w gives the explicit
    nufft_adjoint(w * nufft(x)) to the same accuracy."""
    gen = torch.Generator().manual_seed(5)
    shape = (16, 16)
    locs = (torch.rand(300, 2, generator=gen, dtype=torch.float64) - 0.5) * 16
    x = torch.randn(*shape, dtype=torch.complex128, generator=gen)
    z = torch.randn(*shape, dtype=torch.complex128, generator=gen)
    K = ON.toeplitz_kernel(locs, shape)
    t = ON.toeplitz_normal(x, K, shape)
    e = ON.nufft_adjoint(ON.nufft(x, locs), locs, shape)
    assert float((t - e).norm() / e.norm()) < 0.03
    lin = ON.toeplitz_normal(2 * x - 3j * z, K, shape)
    assert torch.allclose(lin, 2 * t - 3j * ON.toeplitz_normal(z, K, shape), rtol=1e-12, atol=1e-12)
    w = torch.rand(300, generator=gen, dtype=torch.float64) + 0.5
    tw = ON.toeplitz_normal(x, ON.toeplitz_kernel(locs, shape, weight=w), shape)
    ew = ON.nufft_adjoint(w * ON.nufft(x, locs), locs, shape)
    assert float((tw - ew).norm() / ew.norm()) < 0.03
