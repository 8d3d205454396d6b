"""The NUFFT's Toeplitz normal operator, ``NUFFT(..., toeplitz=True).normal(inner)``
(reference linops/nufft.py:226-239, 395-568):

* the PSF kernel and the operator applied to an image against the reference's
  own outputs (tests/golden/toeplitz.npz, written by tests/golden/make_golden.py)
  and the FP64 oracle, with and without a diagonal weighting of the points,
  for a batched image and for the odd-padding case in which the reference's
  rescaled points and larger grid disagree by one cell;
* at 24^3 with 3,000 points: the embedding against the explicit normal
  operator (about 1% apart in FP64 too: both carry the interpolation error),
  the exact adjoint pair, and batch entries sharing the kernel.
"""

import numpy as np
import pytest
import torch

from conftest import GOLDEN, rel_l2, to_torch
from oracle import nufft as ON

from torchlinops_gb300 import linops

pytestmark = pytest.mark.gpu
DEV = "cuda"
TOL = 1e-5
TOEPLITZ = {"2d": (16, 16), "2d_batch_dcf": (12, 16), "2d_odd_pad": (12, 14), "3d": (8, 8, 8)}


@pytest.mark.parametrize("name", sorted(TOEPLITZ))
def test_toeplitz_matches_reference(name):
    d = np.load(f"{GOLDEN}/toeplitz.npz")
    shape = TOEPLITZ[name]
    locs = torch.from_numpy(d[f"{name}_locs"])
    x = to_torch(d[f"{name}_x"], True)
    w = torch.from_numpy(d[f"{name}_dcf"]) if f"{name}_dcf" in d.files else None
    A = linops.NUFFT(locs.to(DEV), shape, toeplitz=True)
    T = A.normal(None if w is None else linops.Diagonal(w.to(DEV)))
    assert isinstance(T, linops.ToeplitzNormal)
    assert rel_l2(T.kernel.cpu(), to_torch(d[f"{name}_kernel"], True)) < TOL
    y = T(x.to(DEV)).cpu()
    assert y.shape == x.shape
    assert rel_l2(y, to_torch(d[f"{name}_normal"], True)) < TOL
    K64 = ON.toeplitz_kernel(locs, shape, weight=w)
    assert rel_l2(T.kernel.cpu(), K64) < TOL
    assert rel_l2(y, ON.toeplitz_normal(x, K64, shape)) < TOL


def test_toeplitz_normal_against_the_explicit_normal():
    gen = torch.Generator().manual_seed(3)
    shape = (24, 24, 24)
    locs = ((torch.rand(3000, 3, generator=gen) - 0.5) * 24).to(DEV)
    x = torch.randn(2, *shape, dtype=torch.complex64, generator=gen).to(DEV)
    v = torch.randn(2, *shape, dtype=torch.complex64, generator=gen).to(DEV)
    A = linops.NUFFT(locs, shape, toeplitz=True)
    T = A.N
    assert isinstance(T, linops.ToeplitzNormal) and A.N is T
    tx = T(x)
    ex = linops.NUFFT(locs, shape).N(x)
    assert rel_l2(tx.cpu(), ex.cpu()) < 0.03
    # T.H is the exact adjoint (the kernel is not real: 2x grids are even)
    lhs = torch.vdot(tx.flatten().to(torch.complex128), v.flatten().to(torch.complex128))
    rhs = torch.vdot(x.flatten().to(torch.complex128), T.H(v).flatten().to(torch.complex128))
    assert abs(complex(lhs - rhs)) <= 1e-5 * abs(complex(lhs))
    assert rel_l2(T(x[1:]).cpu(), tx[1:].cpu()) < 1e-6
