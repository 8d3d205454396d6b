"""Tensor-core 3^3 convolution kernels (BF16 operands, FP32 accumulation) and
the learned preconditioner's gradients, against the float64 CPU oracle.

Inputs are bfloat16 values, so products are exact in float32 and the only
error left is float32 accumulation: 1e-5 relative L2 for float32 outputs.
bfloat16 outputs are compared after rounding the oracle the same way.
"""

import pytest
import torch

from conftest import rel_l2
from oracle import conv as OC

from torchlinops_gb300 import _ext
from torchlinops_gb300 import precond as P

pytestmark = pytest.mark.gpu
DEV = "cuda"
SHAPES = [(1, 1, 1), (3, 4, 70), (6, 5, 64), (9, 7, 130)]


def _rand(shape, gen, scale=1.0):
    return (torch.randn(*shape, generator=gen) * scale).to(torch.bfloat16)


@pytest.mark.parametrize("shape", SHAPES + [(2, 3, 128), (3, 2, 300)])
def test_conv_forward_float32_out(shape):
    """The tcgen05 kernel: 128-voxel row tiles (W = 128 exactly one tile, 300
    a ragged last tile), halos from TMA with zero fill."""
    gen = torch.Generator().manual_seed(sum(shape))
    x, w = _rand((*shape, 16), gen), _rand((27, 16, 16), gen, 0.2)
    _ext.device_status(clear=True)
    y = P.conv3d(x.to(DEV), w.to(DEV), _ext.TLGB_CONV_PLAIN, out_f32=True).cpu()
    assert _ext.device_status() == 0  # no bounded wait gave up
    ref = OC.conv3d(x, w)
    assert rel_l2(y.double(), ref) < 1e-5


@pytest.mark.parametrize("shape", SHAPES[1:])
def test_conv_forward_relu_and_mask_bf16(shape):
    gen = torch.Generator().manual_seed(3 + sum(shape))
    x, w = _rand((*shape, 16), gen), _rand((27, 16, 16), gen, 0.2)
    aux = _rand((*shape, 16), gen)
    y = P.conv3d(x.to(DEV), w.to(DEV), _ext.TLGB_CONV_RELU).cpu()
    ref = torch.relu(OC.conv3d(x, w)).to(torch.bfloat16)
    assert (y.float() - ref.float()).abs().max() <= ref.float().abs().max() * 2**-7
    ym = P.conv3d(x.to(DEV), w.to(DEV), _ext.TLGB_CONV_MASK, aux=aux.to(DEV), out_f32=True).cpu()
    refm = OC.conv3d(x, w) * (aux.double() > 0)
    assert rel_l2(ym.double(), refm) < 1e-5


@pytest.mark.parametrize("shape", SHAPES)
def test_conv_data_gradient_is_flipped_forward(shape):
    gen = torch.Generator().manual_seed(7 + sum(shape))
    gy, w = _rand((*shape, 16), gen), _rand((27, 16, 16), gen, 0.2)
    gx = P.conv3d(gy.to(DEV), P.flip_weights(w.to(DEV)), _ext.TLGB_CONV_PLAIN, out_f32=True).cpu()
    assert rel_l2(gx.double(), OC.conv3d_dgrad(gy, w)) < 1e-5


@pytest.mark.parametrize("shape", SHAPES)
def test_conv_weight_gradient(shape):
    gen = torch.Generator().manual_seed(11 + sum(shape))
    x, gy = _rand((*shape, 16), gen), _rand((*shape, 16), gen)
    dw = P.conv3d_wgrad(x.to(DEV), gy.to(DEV))
    assert rel_l2(dw.cpu().double(), OC.conv3d_wgrad(x, gy)) < 1e-5
    assert torch.equal(dw, P.conv3d_wgrad(x.to(DEV), gy.to(DEV)))  # fixed summation order


def test_pack_unpack():
    gen = torch.Generator().manual_seed(5)
    z = torch.complex(torch.randn(4, 5, 6, generator=gen), torch.randn(4, 5, 6, generator=gen))
    s = torch.tensor([0.5])
    p = P.pack(z.to(DEV), s.to(DEV)).cpu()
    assert torch.equal(p[..., 0], (z.real * 0.5).to(torch.bfloat16))
    assert torch.equal(p[..., 1], (z.imag * 0.5).to(torch.bfloat16))
    assert torch.count_nonzero(p[..., 2:].float()) == 0
    q = P.pack(z.to(DEV), s.to(DEV), hilo=True).cpu().float()
    two = q[..., 0] + q[..., 2]  # a two-term split: 16 significant bits
    assert torch.allclose(two, z.real * 0.5, rtol=2**-15, atol=0)
    assert torch.count_nonzero(q[..., 4:]) == 0
    y = torch.randn(4, 5, 6, 16, generator=gen)
    u = P.unpack(y.to(DEV), z.to(DEV), torch.tensor([2.0]).to(DEV), 1.0).cpu()
    torch.testing.assert_close(u, 2.0 * torch.complex(y[..., 0], y[..., 1]) + z)


def test_conv_rejects_bad_inputs():
    x = torch.zeros(2, 2, 2, 8, dtype=torch.bfloat16, device=DEV)
    with pytest.raises(ValueError):
        P.conv3d(x, torch.zeros(27, 16, 16, dtype=torch.bfloat16, device=DEV))
    with pytest.raises(RuntimeError):
        P.conv3d(torch.zeros(2, 2, 2, 16, dtype=torch.bfloat16), torch.zeros(27, 16, 16, dtype=torch.bfloat16))


def test_network_gradients_match_cpu_autograd():
    """Gradients of L = |M(r) - e|^2/|e|^2 w.r.t. the free parameters from the
    GPU kernels vs CPU autograd through the float64 oracle network with the
    same bf16 rounding. The GPU backward also rounds the propagated gradients
    to bfloat16, so the agreement is to bf16 precision."""
    gen = torch.Generator().manual_seed(9)
    shape = (10, 12, 14)
    r = torch.complex(torch.randn(*shape, generator=gen), torch.randn(*shape, generator=gen))
    e = torch.complex(torch.randn(*shape, generator=gen), torch.randn(*shape, generator=gen))
    M = P.CNNPreconditioner(DEV, seed=3, init="random", c0=0.7)
    loss, (g1, g2, gs) = M.loss_and_grads((r.to(DEV), e.to(DEV)), kind="mse")
    v1 = M.v1.detach().cpu().double().requires_grad_(True)
    v2 = M.v2.detach().cpu().double().requires_grad_(True)
    skip = torch.tensor(0.7, dtype=torch.float64, requires_grad=True)
    ref = OC.network_loss(r.to(torch.complex128), e.to(torch.complex128), v1, v2, skip)
    ref.backward()
    assert abs(float(loss) - float(ref.detach())) / float(ref.detach()) < 1e-3
    assert rel_l2(g1.cpu().double(), v1.grad) < 3e-2
    assert rel_l2(g2.cpu().double(), v2.grad) < 3e-2
    assert abs(float(gs) - float(skip.grad)) / abs(float(skip.grad)) < 3e-2
    z = M(r.to(DEV)).cpu()
    zr = OC.network(r.to(torch.complex128), v1.detach(), v2.detach(), 0.7)
    assert rel_l2(z.to(torch.complex128), zr) < 1e-3


def test_preconditioner_is_symmetric_positive_definite_and_complex_linear():
    gen = torch.Generator().manual_seed(4)
    shape = (12, 10, 14)
    M = P.CNNPreconditioner(DEV, seed=2, init="random", c0=0.05)
    x, y = (torch.complex(torch.randn(*shape, generator=gen), torch.randn(*shape, generator=gen)).to(DEV) for _ in range(2))
    # M is homogeneous, so <M x, y> = <x, M y> holds for the linear map r -> M(r) at fixed |r|:
    # compare on a pair with equal norms
    y = y * (torch.linalg.vector_norm(x) / torch.linalg.vector_norm(y))
    a = torch.vdot(M(x).flatten(), y.flatten())
    b = torch.vdot(x.flatten(), M(y).flatten())
    assert abs(complex(a) - complex(b)) / abs(complex(a)) < 2e-2  # bf16 activations
    assert float(torch.real(torch.vdot(x.flatten(), M(x).flatten()))) > 0
    z1 = M(1j * x)
    assert rel_l2(z1.cpu(), (1j * M(x)).cpu()) < 1e-2


def test_laplacian_warm_start_is_exact():
    """The warm start is M = c0 I - lap (7-point, zero boundary) up to bf16."""
    import torch.nn.functional as F

    gen = torch.Generator().manual_seed(6)
    shape = (9, 11, 13)
    r = torch.complex(torch.randn(*shape, generator=gen), torch.randn(*shape, generator=gen))
    M = P.CNNPreconditioner(DEV, init="laplacian", c0=0.02, noise=0.0)
    k = torch.zeros(1, 1, 3, 3, 3, dtype=torch.float64)
    k[0, 0, 1, 1, 1] = 6.0
    for d in [(0, 1, 1), (2, 1, 1), (1, 0, 1), (1, 2, 1), (1, 1, 0), (1, 1, 2)]:
        k[0, 0][d] = -1.0
    lap = lambda t: F.conv3d(t.double()[None, None], k, padding=1)[0, 0]  # noqa: E731
    # N^T N with N = forward differences and zero padding is the 7-point
    # operator with zero boundary except on the first plane of each axis,
    # where the difference below the volume is missing: compare away from it
    ref = 0.02 * r.to(torch.complex128) + torch.complex(lap(r.real), lap(r.imag))
    z = M(r.to(DEV)).cpu().to(torch.complex128)
    inner = (slice(1, None),) * 3
    assert rel_l2(z[inner], ref[inner]) < 5e-3
