"""The differentiable 2D NUFFT at the multi-slice workload: 32 slices x 8 coils
of a 256^2 complex64 image (padded 320^2) on a golden-angle radial trajectory
of 402 spokes x 512 readouts (spoke k at angle k pi (sqrt 5 - 1) / 2,
readouts (j - 256) / 2, N(0, 0.1) jitter per coordinate), through the
functional ``nufft`` with autograd:

* the forward values and the image gradient (the adjoint NUFFT of the
  cotangent) against the float32 mirror of the reference's operations and
  the FP64 oracle on two of the 256 batch entries;
* the trajectory gradient against FP64 central differences on sampled
  points, and against the FP64 autograd restatement of the interpolation on
  more points; both sum over all 256 batch entries.
"""

import math

import pytest
import torch

from conftest import rel_l2
from oracle import interp as OI
from oracle import nufft as ON

from torchlinops_gb300 import linops

pytestmark = pytest.mark.gpu
DEV = "cuda"
S, C, N, SPOKES, READ = 32, 8, 256, 402, 512


def golden_angle_radial(gen):
    k = torch.arange(SPOKES, dtype=torch.float64)
    ang = k * math.pi * (math.sqrt(5.0) - 1.0) / 2.0
    r = (torch.arange(READ, dtype=torch.float64) - READ // 2) * (N / READ)
    locs = torch.stack([r[None, :] * torch.cos(ang[:, None]), r[None, :] * torch.sin(ang[:, None])], dim=-1)
    locs = locs + 0.1 * torch.randn(locs.shape, generator=gen, dtype=torch.float64)
    return locs.to(torch.float32)  # [402, 512, 2]


@pytest.fixture(scope="module")
def case():
    gen = torch.Generator().manual_seed(4)
    locs = golden_angle_radial(gen)
    img = torch.randn(S, C, N, N, dtype=torch.complex64, generator=gen)
    a = torch.randn(S, C, SPOKES, READ, dtype=torch.complex64, generator=gen)
    x = img.to(DEV).requires_grad_(True)
    L = locs.to(DEV).requires_grad_(True)
    y = linops.nufft(x, L)
    (a.to(DEV).conj() * y).real.sum().backward()
    return dict(locs=locs, img=img, a=a, y=y.detach().cpu(), gimg=x.grad.cpu(), glocs=L.grad.cpu())


def test_forward_and_image_gradient_vs_oracle(case):
    """Against the float32 mirror of the reference's operations (the parity
    bar, 1e-5) and the FP64 oracle. At this size the FP64 error is set by the
    float32 interpolation coordinates, which the reference computes the same
    way: scaled into [0, 320) their ulp is about 3e-5 grid units."""
    locs, img, a = case["locs"], case["img"], case["a"]
    assert case["y"].shape == (S, C, SPOKES, READ)
    for s, c in ((0, 0), (17, 5)):
        assert rel_l2(case["y"][s, c], ON.nufft(img[s, c], locs, dtype=torch.float32)) < 1e-5
        assert rel_l2(case["y"][s, c], ON.nufft(img[s, c], locs)) < 1e-4
        # d/d conj(img) of Re<a, F img> is F^H a
        assert rel_l2(case["gimg"][s, c], ON.nufft_adjoint(a[s, c], locs, (N, N), dtype=torch.float32)) < 1e-5
        assert rel_l2(case["gimg"][s, c], ON.nufft_adjoint(a[s, c], locs, (N, N))) < 1e-4


def _trajectory_objective(kspace, a_p, x, sf):
    """sum_b Re(conj(a_b) y_b(x)) for one point x (user units), FP64."""
    padded = (int(N * 1.25),) * 2
    g = ON.prep_locs(x[None], (N, N), padded)
    y = OI.ungrid(kspace, g, 4.0, beta=OI.nufft_beta(4.0, 1.25), dtype=torch.float64)[:, 0] / sf
    return float((a_p.conj() * y).real.sum())


def test_trajectory_gradient_vs_fp64(case):
    locs, img, a = case["locs"], case["img"], case["a"]
    padded = (int(N * 1.25),) * 2
    sf = ON.scale_factor((N, N), padded, 4.0)
    K = ON.kspace(img.reshape(S * C, N, N), 2)  # [256, 320, 320] complex128
    A = a.reshape(S * C, SPOKES * READ).to(torch.complex128)
    flat = locs.reshape(-1, 2)
    G = case["glocs"].reshape(-1, 2).double()
    beta = OI.nufft_beta(4.0, 1.25)
    # FP64 autograd restatement of the interpolation, chained through the
    # locations' rescaling (d grid / d user = Np / N)
    idx = torch.randperm(flat.shape[0], generator=torch.Generator().manual_seed(5))[:300]
    g = ON.prep_locs(flat[idx].double(), (N, N), padded)
    ref = OI.grad_locs_interp(K, A[:, idx] / sf, g, 4.0, beta=beta) * (padded[0] / N)
    assert rel_l2(G[idx], ref) < 1e-4
    # central differences on points away from tap boundaries
    h = 1e-3
    checked = 0
    for p in idx[:40].tolist():
        x = flat[p].double()
        gx = ON.prep_locs(torch.stack([x - h, x + h]), (N, N), padded)
        same = True
        for e in range(2):
            _, _, ok = OI.axis_taps(gx[:, e], 4.0, "kaiser_bessel", torch.float64)
            lo = torch.ceil(gx[:, e] - 2.0)
            same = same and torch.equal(ok[0], ok[1]) and bool(lo[0] == lo[1])
        if not same:
            continue
        for e in range(2):
            d = torch.zeros(2, dtype=torch.float64)
            d[e] = h
            fd = (_trajectory_objective(K, A[:, p], x + d, sf) - _trajectory_objective(K, A[:, p], x - d, sf)) / (2 * h)
            assert abs(float(G[p, e]) - fd) <= 1e-3 * max(1.0, abs(fd)), (p, e, float(G[p, e]), fd)
        checked += 1
    assert checked >= 20
