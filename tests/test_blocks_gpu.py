"""Parity of the CUDA unfold / fold kernels with the reference (bit-exact)."""

import pytest
import torch

from conftest import load_cases, to_torch
from oracle import blocks as OB

import torchlinops_gb300 as T

pytestmark = pytest.mark.gpu
DEV = "cuda"
BLOCKS = load_cases("blocks_cases.npz")


@pytest.mark.parametrize("case", sorted(BLOCKS))
def test_blocks_match_reference_bit_exact(case):
    rec = BLOCKS[case]
    m = rec["meta"]
    cplx = "complex" in m["dtype"]
    x = to_torch(rec["x"], cplx).to(DEV)
    y = to_torch(rec["y"], cplx).to(DEV)
    u = T.array_to_blocks(x, tuple(m["block"]), tuple(m["stride"]))
    f = T.blocks_to_array(y, tuple(m["shape"]), tuple(m["block"]), tuple(m["stride"]))
    assert torch.equal(u.cpu(), to_torch(rec["unfold"], cplx))
    # the fold sums in the reference's block order: equal bit for bit
    assert torch.equal(f.cpu(), to_torch(rec["fold"], cplx))
    if "mask" in rec:
        mask = torch.from_numpy(rec["mask"])
        ym = to_torch(rec["ym"], cplx).to(DEV)
        um = T.array_to_blocks(x, tuple(m["block"]), tuple(m["stride"]), mask)
        fm = T.blocks_to_array(ym, tuple(m["shape"]), tuple(m["block"]), tuple(m["stride"]), mask)
        assert torch.equal(um.cpu(), to_torch(rec["unfold_masked"], cplx))
        assert torch.equal(fm.cpu(), to_torch(rec["fold_masked"], cplx))


@pytest.mark.parametrize(
    "shape,block,stride,dtype",
    [
        ((3, 40, 40, 40), (8, 8, 8), (4, 4, 4), torch.complex64),
        ((2, 37, 29, 31), (7, 5, 6), (3, 2, 5), torch.float32),
        ((4, 120, 120, 120), (10, 10, 10), (10, 10, 10), torch.complex64),
        ((2, 1025), (25,), (25,), torch.float64),
        ((5, 64, 80), (16, 8), (4, 8), torch.complex128),
        # even innermost block, stride and extent: the paired fold, with
        # uncovered trailing elements (f64) and a stride not dividing the block (f32)
        ((2, 30, 34, 42), (4, 6, 8), (2, 4, 6), torch.float64),
        ((3, 50, 64), (6, 10), (2, 4), torch.float32),
        ((2, 18, 20, 22), (3, 4, 6), (3, 2, 2), torch.complex64),
    ],
)
def test_blocks_random_against_oracle(shape, block, stride, dtype):
    gen = torch.Generator().manual_seed(sum(shape))
    x = torch.randn(shape, generator=gen, dtype=torch.float64).to(dtype) if not dtype.is_complex else torch.randn(shape, generator=gen, dtype=dtype)
    u = T.unfold(x.to(DEV), block, stride)
    assert torch.equal(u.cpu(), OB.unfold(x, block, stride))
    y = torch.randn(u.shape, generator=gen, dtype=torch.float64).to(dtype) if not dtype.is_complex else torch.randn(u.shape, generator=gen, dtype=dtype)
    f = T.fold(y.to(DEV), shape[-len(block):], block, stride)
    ref = OB.fold(y, shape[-len(block):], block, stride)
    assert torch.equal(f.cpu(), ref)


def test_fold_is_deterministic_and_adjoint():
    gen = torch.Generator().manual_seed(9)
    x = torch.randn(2, 48, 48, 48, dtype=torch.complex64, generator=gen).to(DEV)
    u = T.unfold(x, (8, 8, 8), (4, 4, 4))
    y = torch.randn(u.shape, dtype=torch.complex64, generator=gen).to(DEV)
    a = T.fold(y, (48, 48, 48), (8, 8, 8), (4, 4, 4))
    b = T.fold(y, (48, 48, 48), (8, 8, 8), (4, 4, 4))
    assert torch.equal(a, b)
    lhs = torch.vdot(u.flatten().to(torch.complex128), y.flatten().to(torch.complex128))
    rhs = torch.vdot(x.flatten().to(torch.complex128), a.flatten().to(torch.complex128))
    assert abs(lhs - rhs) / abs(lhs) < 1e-6


def test_output_buffer_reuse():
    """reference _unfold/tests/test_fold_unfold_output_buffer.py."""
    x = torch.randn(2, 20, 20, device=DEV)
    buf = torch.full((2, 9, 9, 4, 4), 7.0, device=DEV)
    y = T.unfold(x, (4, 4), (2, 2), output=buf)
    assert y.data_ptr() == buf.data_ptr()
    assert torch.equal(y.cpu(), OB.unfold(x.cpu(), (4, 4), (2, 2)))
    obuf = torch.full((2, 20, 20), 3.0, device=DEV)
    z = T.fold(y, (20, 20), (4, 4), (2, 2), output=obuf)
    assert z.data_ptr() == obuf.data_ptr()
    assert torch.equal(z.cpu(), OB.fold(y.cpu(), (20, 20), (4, 4), (2, 2)))
    with pytest.raises(ValueError):
        T.unfold(x, (4, 4), (2, 2), output=buf.double())


def test_norm_weights_round_trip():
    w = T.get_norm_weights((33, 43), (7, 7), (2, 2), device=DEV)
    x = torch.randn(2, 33, 43, dtype=torch.complex64, device=DEV)
    x2 = (1.0 / w.clamp(min=1e-6)) * T.fold(T.unfold(x, (7, 7), (2, 2)), (33, 43), (7, 7), (2, 2))
    covered = w > 0
    torch.testing.assert_close(x2[:, covered], x[:, covered])


def test_autograd_unfold_fold():
    x = torch.randn(1, 15, 15, 15, device=DEV, requires_grad=True)
    mask = torch.zeros(3, 3, 3, dtype=torch.bool)
    mask[1, 1, :] = True
    mask[0, 1, 1] = True
    y = T.array_to_blocks(x, (3, 3, 3), (1, 1, 1), mask)
    y.sum().backward()
    ref = T.get_norm_weights((15, 15, 15), (3, 3, 3), (1, 1, 1), mask, device=DEV)
    assert torch.equal(x.grad[0], ref)


def test_errors_match_reference():
    with pytest.raises(ValueError):
        T.unfold(torch.randn(4, 4, device=DEV), (8, 8), (1, 1))  # no block fits
    with pytest.raises(RuntimeError):
        T.fold(torch.randn(3, 3, 2, 2, device=DEV), (5, 5), (2, 2), (1, 1))  # wrong block grid
