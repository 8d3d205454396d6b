"""Parity at the benchmark sizes: whole outputs against the oracle, and size-independent properties.

* 3D interpolation at the headline workload (256^3 x 8 coils complex64,
  2^21 points in a 1/r^2 ball, KB W=4): the whole ungrid and the whole grid
  against the oracle (float32, 1e-5 relative L2) with their FP64 errors, the
  adjoint identity in float64, linearity of gridding, bit-identical repeats,
  and the dense centre against FP64.
* ArrayToBlocks / BlocksToArray at 16 x 160^3 complex64, block 8^3, stride
  4: the whole unfold against Tensor.unfold, the whole fold of random blocks
  against the oracle (bit-exact), and fold(unfold(x)) against x added to
  itself once per covering block, in the same order (bit-exact).
"""

import math

import pytest
import torch

from conftest import rel_l2
from oracle import blocks as OB
from oracle import interp as OI

import torchlinops_gb300 as T

pytestmark = pytest.mark.gpu
DEV = "cuda"
N, C, P = 256, 8, 1 << 21


@pytest.fixture(scope="module")
def interp_case():
    g = torch.Generator().manual_seed(0)
    r = torch.rand(P, generator=g) * (N / 2)
    u = torch.randn(P, 3, generator=g)
    locs = (N / 2 + r[:, None] * u / u.norm(dim=-1, keepdim=True)).to(torch.float32)
    gd = torch.Generator(device=DEV).manual_seed(1)
    img = torch.randn(C, N, N, N, dtype=torch.complex64, device=DEV, generator=gd)
    vals = torch.randn(C, P, dtype=torch.complex64, device=DEV, generator=gd)
    beta = OI.nufft_beta(4.0, 1.25)
    return locs, locs.to(DEV), img, vals, beta


def test_fullsize_adjoint_identity_and_determinism(interp_case):
    locs_h, locs, img, vals, beta = interp_case
    kp = dict(beta=beta)
    y = T.ungrid(img, locs, 4.0, kernel_params=kp)
    g1 = T.grid(vals, locs, (N, N, N), 4.0, kernel_params=kp)
    lhs = torch.vdot(y.flatten().to(torch.complex128), vals.flatten().to(torch.complex128))
    rhs = torch.vdot(img.flatten().to(torch.complex128), g1.flatten().to(torch.complex128))
    assert abs(complex(lhs - rhs)) / abs(complex(lhs)) < 1e-5
    g2 = T.grid(vals, locs, (N, N, N), 4.0, kernel_params=kp)
    assert torch.equal(g1, g2)  # fixed summation order, no atomics
    del g2
    # linearity: grid(2 v1 + v2) = 2 grid(v1) + grid(v2)
    v2 = torch.roll(vals, 1, dims=0)
    g3 = T.grid(2 * vals + v2, locs, (N, N, N), 4.0, kernel_params=kp)
    ref = 2 * g1 + T.grid(v2, locs, (N, N, N), 4.0, kernel_params=kp)
    num = torch.linalg.vector_norm((g3 - ref).flatten().to(torch.complex128))
    assert float(num / torch.linalg.vector_norm(ref.flatten().to(torch.complex128))) < 1e-6


def test_fullsize_ungrid_matches_oracle_whole(interp_case):
    """The whole 8 x 2^21 ungrid against the oracle (the reference's torch
    path restated, float32) at 1e-5 relative L2, with its FP64 error beside."""
    locs_h, locs, img, vals, beta = interp_case
    y = T.ungrid(img, locs, 4.0, kernel_params=dict(beta=beta)).cpu()
    img_h = img.cpu()
    ref = OI.ungrid(img_h, locs_h, 4.0, beta=beta)
    e32 = rel_l2(y, ref)
    ref64 = OI.ungrid(img_h.to(torch.complex128), locs_h, 4.0, beta=beta, dtype=torch.float64)
    e64 = rel_l2(y.to(torch.complex128), ref64)
    print(f"ungrid 256^3 x 8 x 2^21: rel. L2 vs float32 oracle {e32:.3e}, vs FP64 oracle {e64:.3e}")
    assert e32 < 1e-5
    assert e64 < 1e-5


def test_fullsize_grid_matches_oracle_whole(interp_case):
    """The whole 8 x 256^3 grid against the oracle at 1e-5 relative L2, with
    its FP64 error beside."""
    locs_h, locs, img, vals, beta = interp_case
    g = T.grid(vals, locs, (N, N, N), 4.0, kernel_params=dict(beta=beta)).cpu()
    vals_h = vals.cpu()
    ref = OI.grid(vals_h, locs_h, (N, N, N), 4.0, beta=beta)
    e32 = rel_l2(g, ref)
    del ref
    ref64 = OI.grid(vals_h.to(torch.complex128), locs_h, (N, N, N), 4.0, beta=beta, dtype=torch.float64)
    e64 = rel_l2(g.to(torch.complex128), ref64)
    print(f"grid 256^3 x 8 x 2^21: rel. L2 vs float32 oracle {e32:.3e}, vs FP64 oracle {e64:.3e}")
    assert e32 < 1e-5
    assert e64 < 1e-5


def test_fullsize_grid_dense_centre_vs_fp64(interp_case):
    """The hottest voxels (tens of thousands of points pile onto each cell of
    the centre tile): the GPU's error against the FP64 oracle stays at the
    level of one float32 rounding per cell, and no worse than the float32
    oracle's own sequential sum (parts of at most 256 points per block
    accumulated in fp32, then a compensated sum of the parts)."""
    locs_h, locs, img, vals, beta = interp_case
    g = T.grid(vals, locs, (N, N, N), 4.0, kernel_params=dict(beta=beta))
    c = torch.tensor((128.0, 128.0, 128.0))
    pts = torch.nonzero((locs_h - c).abs().max(dim=-1).values < 6).flatten()
    v = vals[:, pts].cpu()
    sl = (slice(None),) + tuple(slice(124, 132) for _ in range(3))
    ref64 = OI.grid(v.to(torch.complex128), locs_h[pts], (N, N, N), 4.0, beta=beta, dtype=torch.float64)[sl]
    ref32 = OI.grid(v, locs_h[pts], (N, N, N), 4.0, beta=beta)[sl]
    e_gpu = rel_l2(g[sl].cpu().to(torch.complex128), ref64)
    e_f32 = rel_l2(ref32.to(torch.complex128), ref64)
    print(f"dense centre: {pts.numel()} points, rel. L2 vs FP64: GPU {e_gpu:.3e}, float32 oracle {e_f32:.3e}")
    assert e_gpu < 2e-6
    assert e_gpu <= max(e_f32, 5e-7)


def test_fullsize_unfold_fold():
    """16 x 160^3 complex64, block 8^3, stride 4: the whole unfold against
    Tensor.unfold (the same elements as the reference's unfold), the whole
    fold of random blocks against the oracle's fold (same summation order:
    bit-exact), and fold(unfold(x)) against x added once per covering block."""
    B, S, shape = (8, 8, 8), (4, 4, 4), (16, 160, 160, 160)
    gd = torch.Generator(device=DEV).manual_seed(3)
    x = torch.randn(shape, dtype=torch.complex64, device=DEV, generator=gd)
    y = T.unfold(x, B, S)
    nb = tuple((s - b) // st + 1 for s, b, st in zip(shape[1:], B, S))
    assert tuple(y.shape) == (16, *nb, *B)
    assert torch.equal(y, x.unfold(1, 8, 4).unfold(2, 8, 4).unfold(3, 8, 4))
    z = T.fold(y, shape[1:], B, S)
    del y
    # every element is added once per covering block, starting from zero, in
    # ascending block order: the same float additions as acc += x, cnt times
    cnt = torch.ones(shape[1:], device=DEV)
    for d in range(3):
        i = torch.arange(shape[1 + d], device=DEV)
        lo = torch.clamp(torch.div(i - 8, 4, rounding_mode="floor") + 1, min=0)
        hi = torch.clamp(torch.div(i, 4, rounding_mode="floor"), max=nb[d] - 1)
        c = (hi - lo + 1).to(torch.float32)
        cnt = cnt * c.reshape([-1 if k == d else 1 for k in range(3)])
    acc = torch.zeros_like(x)
    for k in range(int(cnt.max())):
        acc = torch.where(cnt > k, acc + x, acc)
    assert torch.equal(z, acc)
    assert torch.equal(T.fold(T.unfold(x, B, S), shape[1:], B, S), z)  # deterministic
    del acc, z, x
    # random blocks (not the unfold of an array): the whole fold, bit-exact
    yr = torch.randn((16, *nb, *B), dtype=torch.complex64, device=DEV, generator=gd)
    zr = T.fold(yr, shape[1:], B, S).cpu()
    ref = OB.fold(yr.cpu(), shape[1:], B, S)
    assert torch.equal(zr, ref)
