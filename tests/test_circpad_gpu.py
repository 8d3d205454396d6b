"""Circular padding and the Convolution linop's circular mode on the GPU,
against the reference's own outputs (tests/golden/circpad_cases.npz): the
pad bit-exact (a copy), the adjoint and the convolution within float32
rounding, autograd pairs, determinism and the errors."""

import pytest
import torch

from conftest import load_cases, rel_l2, to_torch
from oracle import circpad as OC

import torchlinops_gb300 as T
from torchlinops_gb300 import linops

pytestmark = pytest.mark.gpu
DEV = "cuda"
CASES = load_cases("circpad_cases.npz")


@pytest.mark.parametrize("case", sorted(CASES))
def test_circpad_matches_reference_golden(case):
    rec = CASES[case]
    m = rec["meta"]
    cplx = m["complex"]
    if "padding" in m:
        x = to_torch(rec["x"], cplx).to(DEV)
        y = T.circular_pad(x, m["padding"])
        assert torch.equal(y.cpu(), to_torch(rec["pad"], cplx))
        z = to_torch(rec["z"], cplx).to(DEV)
        adj = T.circular_pad_adjoint(z, m["padding"])
        assert rel_l2(adj.cpu(), to_torch(rec["adj"], cplx)) < 1e-6
        assert torch.equal(adj, T.circular_pad_adjoint(z, m["padding"]))  # fixed order
    else:
        A = linops.Convolution(to_torch(rec["kernel"], cplx).to(DEV), padding_mode="circular")
        assert rel_l2(A(to_torch(rec["x"], cplx).to(DEV)).cpu(), to_torch(rec["fwd"], cplx)) < 1e-5
        assert rel_l2(A.H(to_torch(rec["z"], cplx).to(DEV)).cpu(), to_torch(rec["adj"], cplx)) < 1e-5


def test_circpad_large_and_adjoint_identity():
    """16 x 160^3 complex64 padded by (4, 4) per dim (the block workload's
    array), against the oracle; <A x, y> = <x, A^H y> in float64."""
    g = torch.Generator(device=DEV).manual_seed(5)
    x = torch.randn(16, 160, 160, 160, dtype=torch.complex64, device=DEV, generator=g)
    pad = (4, 4, 4, 4, 4, 4)
    y = T.circular_pad(x, pad)
    assert torch.equal(y[0].cpu(), OC.circular_pad(x[0].cpu(), pad))
    w = torch.randn(y.shape, dtype=torch.complex64, device=DEV, generator=g)
    aw = T.circular_pad_adjoint(w, pad)
    assert rel_l2(aw[1].cpu(), OC.circular_pad_adjoint(w[1].cpu().to(torch.complex128), pad)) < 1e-6
    lhs = torch.vdot(y.flatten().to(torch.complex128), w.flatten().to(torch.complex128))
    rhs = torch.vdot(x.flatten().to(torch.complex128), aw.flatten().to(torch.complex128))
    assert abs(complex(lhs - rhs)) / abs(complex(lhs)) < 1e-6


def test_circpad_autograd_and_dtypes():
    g = torch.Generator().manual_seed(6)
    x = torch.randn(3, 7, 9, dtype=torch.float64, generator=g).to(DEV).requires_grad_(True)
    pad = (2, 3, 1, 0)
    y = T.circular_pad(x, pad)
    gy = torch.randn(y.shape, dtype=torch.float64, generator=g).to(DEV)
    (gx,) = torch.autograd.grad(y, x, gy)
    assert torch.equal(gx, T.circular_pad_adjoint(gy, pad))
    assert torch.equal(T.circular_pad(torch.arange(12, device=DEV).reshape(3, 4), (1, 2)).cpu(),
                       OC.circular_pad(torch.arange(12).reshape(3, 4), (1, 2)))
    b = torch.rand(5, 6, generator=g).to(torch.bfloat16).to(DEV)
    assert torch.equal(T.circular_pad(b, (2, 2, 1, 1)).cpu(), OC.circular_pad(b.cpu(), (2, 2, 1, 1)))


def test_circpad_errors():
    x = torch.ones(4, 5, device=DEV)
    with pytest.raises(ValueError, match="even length"):
        T.circular_pad(x, (1, 2, 3))
    with pytest.raises(ValueError, match="wraps around at most once"):
        T.circular_pad(x, (6, 0))
    with pytest.raises(RuntimeError, match="CUDA tensors only"):
        T.circular_pad(torch.ones(4, 5), (1, 1))
