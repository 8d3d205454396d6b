"""NUFFT chain, operator algebra (.H, .N, @) and the float64 CG on the GPU."""

import math

import numpy as np
import pytest
import torch

from conftest import GOLDEN, rel_l2, to_torch

import torchlinops_gb300 as T
from torchlinops_gb300 import alg, linops

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.mark.parametrize("name", ["2d", "3d"])
def test_functional_nufft_matches_reference(name):
    d = np.load(f"{GOLDEN}/nufft.npz")
    x = to_torch(d[f"{name}_x"], True).to(DEV)
    locs = torch.from_numpy(d[f"{name}_locs"]).to(DEV)
    y = to_torch(d[f"{name}_y"], True).to(DEV)
    shape = tuple(x.shape[-locs.shape[-1]:])
    fwd = linops.nufft(x, locs)
    adj = linops.nufft_adjoint(y, locs, shape)
    assert rel_l2(fwd.cpu(), to_torch(d[f"{name}_fwd"], True)) < 1e-5
    assert rel_l2(adj.cpu(), to_torch(d[f"{name}_adj"], True)) < 1e-5


def _nudft(x, locs):
    """Exact type-2 NUDFT in float64 (centred), small problems only."""
    shape = x.shape[-locs.shape[-1]:]
    grids = torch.meshgrid(*(torch.arange(s, dtype=torch.float64) - s // 2 for s in shape), indexing="ij")
    phase = sum(l[:, None] * g.reshape(1, -1) / s for l, g, s in zip(locs.double().T, grids, shape))
    E = torch.exp(-2j * math.pi * phase)
    return (x.reshape(*x.shape[: -len(shape)], -1).to(torch.complex128) @ E.T) / math.sqrt(math.prod(shape))


def test_nufft_linop_approximates_nudft():
    gen = torch.Generator().manual_seed(1)
    shape = (32, 32)
    locs = torch.rand(500, 2, generator=gen) * 32 - 16
    x = torch.randn(2, *shape, dtype=torch.complex64, generator=gen)
    A = linops.NUFFT(locs.to(DEV), shape, oversamp=1.25, width=4.0)
    y = A(x.to(DEV)).cpu()
    ref = _nudft(x, locs)
    assert rel_l2(y, ref) < 2e-2  # NUFFT approximation error at oversampling 1.25, width 4


def test_nufft_adjoint_normal_identities():
    gen = torch.Generator().manual_seed(2)
    shape = (24, 24, 24)
    locs = (torch.rand(4000, 3, generator=gen) * 24 - 12).to(DEV)
    A = linops.NUFFT(locs, shape)
    x = torch.randn(3, *shape, dtype=torch.complex64, generator=gen).to(DEV)
    y = torch.randn(3, 4000, dtype=torch.complex64, generator=gen).to(DEV)
    Ax, AHy = A(x), A.H(y)
    lhs = torch.vdot(Ax.flatten().to(torch.complex128), y.flatten().to(torch.complex128))
    rhs = torch.vdot(x.flatten().to(torch.complex128), AHy.flatten().to(torch.complex128))
    assert abs(lhs - rhs) / abs(lhs) < 1e-5
    torch.testing.assert_close(A.N(x), A.H(A(x)), rtol=1e-5, atol=1e-5)
    B = A.H @ A
    torch.testing.assert_close(B(x), A.N(x), rtol=1e-5, atol=1e-5)


def test_array_to_blocks_linop():
    mask = torch.zeros(3, 3, 3, dtype=torch.bool)
    mask[1] = True
    A = linops.ArrayToBlocks((15, 15, 15), (3, 3, 3), (1, 1, 1), mask)
    x = torch.randn(2, 15, 15, 15, device=DEV)
    y = torch.randn(2, 13, 13, 13, 9, device=DEV)
    lhs = torch.vdot(A(x).flatten().double(), y.flatten().double())
    rhs = torch.vdot(x.flatten().double(), A.H(y).flatten().double())
    assert abs(lhs - rhs) / abs(lhs) < 1e-4  # float32 outputs, cancelling sum
    torch.testing.assert_close(A.N(x), A.H(A(x)))
    assert isinstance(A.H, linops.BlocksToArray)


def test_dot64_matches_float64():
    gen = torch.Generator().manual_seed(3)
    x = torch.randn(1_000_003, dtype=torch.complex64, generator=gen)
    y = torch.randn(1_000_003, dtype=torch.complex64, generator=gen)
    d = alg.dot64(x.to(DEV), y.to(DEV)).cpu()
    ref = torch.vdot(x.to(torch.complex128), y.to(torch.complex128))
    assert abs(complex(d[0], d[1]) - complex(ref)) / abs(complex(ref)) < 1e-12
    d2 = alg.dot64(x.to(DEV), y.to(DEV)).cpu()
    assert torch.equal(d, d2)


def test_cg_float64_scalars_solve_spd_system():
    gen = torch.Generator().manual_seed(4)
    n = 256
    Q, _ = torch.linalg.qr(torch.randn(n, n, dtype=torch.complex128, generator=gen))
    ev = torch.logspace(0, 3, n, dtype=torch.float64)
    M = (Q * ev) @ Q.conj().T
    Mc = M.to(torch.complex64).to(DEV)
    xt = torch.randn(n, dtype=torch.complex64, generator=gen).to(DEV)
    b = Mc @ xt
    x, info = alg.cg_solve(lambda v: Mc @ v, b, rtol=1e-5, max_iters=1000)
    assert info.converged and info.true_rel_residual < 2e-5
    # reference signature still works
    x2 = alg.conjugate_gradients(lambda v: Mc @ v, b, max_num_iters=600, disable_tracking=True)
    assert float(alg.norm64((b - Mc @ x2).contiguous())) / float(alg.norm64(b)) < 1e-4


def test_cg_on_nufft_normal_equations():
    gen = torch.Generator().manual_seed(5)
    shape = (32, 32, 32)
    locs = (torch.rand(60000, 3, generator=gen) * 32 - 16).to(DEV)
    A = linops.NUFFT(locs, shape)
    xt = torch.randn(*shape, dtype=torch.complex64, generator=gen).to(DEV)
    lam = 1e-2
    N = lambda v: A.N(v) + lam * v  # noqa: E731
    b = N(xt)
    x, info = alg.cg_solve(N, b, rtol=1e-4, max_iters=300)
    assert info.converged and info.true_rel_residual < 2e-4
    # flexible PCG with a fixed diagonal preconditioner converges too
    x2, info2 = alg.cg_solve(N, b, rtol=1e-4, max_iters=300, M=lambda r: r * 0.5)
    assert info2.converged and info2.true_rel_residual < 2e-4


@pytest.mark.parametrize("learned", [False, True])
def test_cg_true_residual_decides_convergence(learned):
    """A solve whose recursive residual reaches rtol while its true residual
    does not is not converged: it continues as plain CG from its iterate. The
    operator here changes after the iterations of the first solve (as an
    operator whose rounding drifts would), so the recursive residual belongs
    to a different system than the final check."""
    gen = torch.Generator().manual_seed(9)
    n = 512
    d1 = (torch.rand(n, generator=gen) * 9 + 1).to(DEV)
    d2 = d1 * (1 + 0.01 * torch.randn(n, generator=gen).to(DEV))
    b = torch.randn(n, dtype=torch.complex64, generator=gen).to(DEV)
    M = (lambda r: (r / d1).to(r.dtype)) if learned else None
    _, first = alg.cg_solve(lambda v: d1 * v, b, rtol=1e-4, max_iters=200, M=M)
    assert first.converged and first.restarts == 0
    calls = [0]

    def A(v):  # d1 for the iterations of the first solve, d2 from the final check on
        calls[0] += 1
        return (d1 if calls[0] <= first.iters else d2) * v

    x, info = alg.cg_solve(A, b, rtol=1e-4, max_iters=200, M=M)
    assert info.restarts >= 1
    assert info.converged and info.true_rel_residual <= 1e-4
    assert float(alg.norm64((b - d2 * x).contiguous())) / float(alg.norm64(b)) <= 1e-4


def test_cg_matches_float64_oracle():
    """alg.cg_solve (float32 vectors, float64 scalars) against textbook CG in
    float64 on the CPU (oracle/cg.py): the same solution to 1e-4."""
    from oracle import cg as OCG

    gen = torch.Generator().manual_seed(8)
    n = 200
    Q, _ = torch.linalg.qr(torch.randn(n, n, dtype=torch.complex128, generator=gen))
    M = (Q * torch.logspace(0, 2, n, dtype=torch.float64)) @ Q.conj().T
    xt = torch.randn(n, dtype=torch.complex128, generator=gen)
    b = M @ xt
    ref, it = OCG.cg(lambda v: M @ v, b, rtol=1e-10)
    Mc = M.to(torch.complex64).to(DEV)
    x, info = alg.cg_solve(lambda v: Mc @ v, b.to(torch.complex64).to(DEV), rtol=1e-6, max_iters=2000)
    assert info.converged
    assert rel_l2(x.cpu(), ref) < 1e-4


@pytest.mark.parametrize("im,padded", [((24, 20, 18), (30, 25, 23)), ((16, 15), (20, 19)), ((33,), (41,))])
def test_pad_shift_and_crop_shift_match_torch(im, padded):
    """pad_shift = ifftshift(pad(maps * apod * x)), crop_shift its adjoint
    with fftshift, against torch on odd and even sizes."""
    gen = torch.Generator().manual_seed(len(im) + padded[0])
    nd = len(im)
    dims = tuple(range(-nd, 0))
    x = torch.randn(*im, dtype=torch.complex64, generator=gen)
    maps = torch.randn(3, *im, dtype=torch.complex64, generator=gen)
    apod = torch.rand(*im, generator=gen) + 0.5
    pad = linops.pad_to_size(im, padded)
    ref = torch.fft.ifftshift(torch.nn.functional.pad(maps * apod * x, pad), dim=dims)
    got = linops.pad_shift(x.to(DEV), im, padded, maps=maps.to(DEV), apod=apod.to(DEV)).cpu()
    torch.testing.assert_close(got, ref, rtol=1e-6, atol=1e-6)  # same values, products rounded in another order
    assert torch.equal(got == 0, ref == 0)  # the same zero padding
    z = torch.randn(3, *padded, dtype=torch.complex64, generator=gen)
    sl = tuple(linops.crop_slice_from_pad(pad))
    back = (maps.conj() * apod * torch.fft.fftshift(z, dim=dims)[(slice(None),) + sl]).sum(0)
    add = torch.randn(*im, dtype=torch.complex64, generator=gen)
    gotb = linops.crop_shift(z.to(DEV), im, padded, maps=maps.to(DEV), apod=apod.to(DEV), alpha=0.5,
                             add=add.to(DEV), beta=2.0).cpu()
    torch.testing.assert_close(gotb, 0.5 * back + 2.0 * add, rtol=1e-5, atol=1e-5)
    # with the k-space modulation, an uncentred fftn of the pad is the centred
    # cfftn (fftshift . fftn . ifftshift) of the padded image, and the crop
    # of an uncentred ifftn is the crop of the centred cifftn
    xm = linops.pad_shift(x.to(DEV), im, padded, maps=maps.to(DEV), apod=apod.to(DEV), modulate=True)
    k = torch.fft.fftn(xm, dim=dims, norm="ortho").cpu()
    kref = torch.fft.fftshift(torch.fft.fftn(ref, dim=dims, norm="ortho"), dim=dims)
    torch.testing.assert_close(k, kref, rtol=1e-5, atol=1e-5)
    G = torch.randn(3, *padded, dtype=torch.complex64, generator=gen)
    cif = torch.fft.fftshift(torch.fft.ifftn(torch.fft.ifftshift(G, dim=dims), dim=dims, norm="ortho"), dim=dims)
    backm = (maps.conj() * apod * cif[(slice(None),) + sl]).sum(0)
    gotm = linops.crop_shift(torch.fft.ifftn(G.to(DEV), dim=dims, norm="ortho"), im, padded, maps=maps.to(DEV),
                             apod=apod.to(DEV), modulate=True).cpu()
    torch.testing.assert_close(gotm, backm, rtol=1e-5, atol=1e-5)
    # adjoint pair without maps
    y = torch.randn(*padded, dtype=torch.complex64, generator=gen)
    lhs = torch.vdot(linops.pad_shift(x.to(DEV), im, padded, apod=apod.to(DEV)).cpu().flatten(), y.flatten())
    rhs = torch.vdot(x.flatten(), linops.crop_shift(y.to(DEV), im, padded, apod=apod.to(DEV)).cpu().flatten())
    assert abs(complex(lhs) - complex(rhs)) / abs(complex(lhs)) < 1e-5


@pytest.mark.parametrize("im,padded", [((10, 12), (13, 15)), ((6, 7, 8), (8, 9, 10))])
def test_pad_shift_and_crop_shift_gradients_match_torch(im, padded):
    """Autograd through pad_shift (x) and crop_shift (z and add) against torch
    autograd of the unfused ops, with coil maps and apodization."""
    gen = torch.Generator().manual_seed(3 + len(im))
    nd = len(im)
    dims = tuple(range(-nd, 0))
    x = torch.randn(2, *im, dtype=torch.complex64, generator=gen)
    maps = torch.randn(3, *im, dtype=torch.complex64, generator=gen)
    apod = torch.rand(*im, generator=gen) + 0.5
    a = torch.randn(2, 3, *padded, dtype=torch.complex64, generator=gen)
    pad = linops.pad_to_size(im, padded)
    xr = x.clone().requires_grad_(True)
    ref = torch.fft.ifftshift(torch.nn.functional.pad(maps[None] * apod * xr[:, None], pad), dim=dims)
    (a.conj() * ref).real.sum().backward()
    xg = x.to(DEV).requires_grad_(True)
    out = linops.pad_shift(xg, im, padded, maps=maps.to(DEV), apod=apod.to(DEV))
    (a.to(DEV).conj() * out).real.sum().backward()
    torch.testing.assert_close(xg.grad.cpu(), xr.grad, rtol=1e-5, atol=1e-5)
    # the modulated pad through an uncentred fftn against torch's cfftn
    xr2 = x.clone().requires_grad_(True)
    ref2 = torch.fft.ifftshift(torch.nn.functional.pad(maps[None] * apod * xr2[:, None], pad), dim=dims)
    k2 = torch.fft.fftshift(torch.fft.fftn(ref2, dim=dims, norm="ortho"), dim=dims)
    (a.conj() * k2).real.sum().backward()
    xg2 = x.to(DEV).requires_grad_(True)
    outm = linops.pad_shift(xg2, im, padded, maps=maps.to(DEV), apod=apod.to(DEV), modulate=True)
    (a.to(DEV).conj() * torch.fft.fftn(outm, dim=dims, norm="ortho")).real.sum().backward()
    torch.testing.assert_close(xg2.grad.cpu(), xr2.grad, rtol=1e-5, atol=1e-5)
    z = torch.randn(2, 3, *padded, dtype=torch.complex64, generator=gen)
    add = torch.randn(2, *im, dtype=torch.complex64, generator=gen)
    b = torch.randn(2, *im, dtype=torch.complex64, generator=gen)
    sl = (slice(None), slice(None)) + tuple(linops.crop_slice_from_pad(pad))
    zr, ar = z.clone().requires_grad_(True), add.clone().requires_grad_(True)
    back = 0.5 * (maps.conj() * apod * torch.fft.fftshift(zr, dim=dims)[sl]).sum(1) + 2.0 * ar
    (b.conj() * back).real.sum().backward()
    zg, ag = z.to(DEV).requires_grad_(True), add.to(DEV).requires_grad_(True)
    got = linops.crop_shift(zg, im, padded, maps=maps.to(DEV), apod=apod.to(DEV), alpha=0.5, add=ag, beta=2.0)
    (b.to(DEV).conj() * got).real.sum().backward()
    torch.testing.assert_close(zg.grad.cpu(), zr.grad, rtol=1e-5, atol=1e-5)
    torch.testing.assert_close(ag.grad.cpu(), ar.grad, rtol=1e-6, atol=1e-6)


def test_sense_normal_matches_unfused_operator():
    """The fused SENSE normal operator equals sum_c conj(S_c) F^H F (S_c x)
    built from the NUFFT linop and torch elementwise ops."""
    from torchlinops_gb300 import mri

    n = 20
    locs = mri.radial_trajectory_3d(100, 40, n, DEV)
    maps = mri.gaussian_coil_maps_3d(3, n, device=DEV)
    A = mri.SenseNormal(locs, maps, lam=1e-2, normalise=False)
    gen = torch.Generator().manual_seed(3)
    x = torch.randn(n, n, n, dtype=torch.complex64, generator=gen).to(DEV)
    ref = (maps.conj() * A.F.N(maps * x)).sum(0) + 1e-2 * x
    assert rel_l2(A(x).cpu(), ref.cpu()) < 1e-5
