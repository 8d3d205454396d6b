"""Sampling at integer locations on the GPU against the reference's own
outputs (tests/golden/index_cases.npz, bit-exact) and the oracle: gather,
deterministic scatter-add with collisions, negative indices, broadcast and
sliced indices, integer values, autograd, the bounds error, and a large
case repeated bit for bit."""

import pytest
import torch

from conftest import load_cases, to_torch
from oracle import index as OX

import torchlinops_gb300 as T

pytestmark = pytest.mark.gpu
DEV = "cuda"
CASES = load_cases("index_cases.npz")


@pytest.mark.parametrize("case", sorted(CASES))
def test_index_matches_reference_golden(case):
    rec = CASES[case]
    m = rec["meta"]
    cplx = "complex" in m["dtype"]
    idx = tuple(torch.from_numpy(rec[f"idx{d}"]).to(DEV) for d in range(m["ndim"]) if f"idx{d}" in rec)
    if "vals" in rec:
        out = T.index_adjoint(to_torch(rec["vals"], cplx).to(DEV), idx, m["grid"])
        assert torch.equal(out.cpu(), to_torch(rec["out"], cplx))  # same summation order: bit-exact
    if "fwd" in rec:
        gv = to_torch(rec["grid_vals"], cplx).to(DEV)
        if "slices" in m:
            sl = tuple(slice(*s) for s in m["slices"])
            got = T.index(gv, sl)
        else:
            got = T.index(gv, idx)
        assert torch.equal(got.cpu(), to_torch(rec["fwd"], cplx))


def test_index_adjoint_large_deterministic_and_exact():
    """2^20 samples with many collisions into a 64^3 grid, 4 complex batch
    entries: equal to the oracle's sequential index_add_ bit for bit, and
    identical on repeat."""
    g = torch.Generator().manual_seed(11)
    n, m = 64, 1 << 20
    idx = tuple(torch.randint(-n, n, (m,), generator=g) for _ in range(3))
    # a dense corner: 1/8 of the samples pile onto 8 cells
    for i in idx:
        i[: m // 8] = torch.randint(0, 2, (m // 8,), generator=g)
    vals = torch.complex(torch.randn(4, m, generator=g), torch.randn(4, m, generator=g))
    ref = OX.index_adjoint(vals, idx, (n, n, n))
    idx_d = tuple(i.to(DEV) for i in idx)
    out1 = T.index_adjoint(vals.to(DEV), idx_d, (n, n, n))
    out2 = T.index_adjoint(vals.to(DEV), idx_d, (n, n, n))
    assert torch.equal(out1, out2)
    assert torch.equal(out1.cpu(), ref)
    # the gather is a copy
    img = torch.randn(4, n, n, n, generator=g)
    assert torch.equal(T.index(img.to(DEV), idx_d).cpu(), OX.index(img, idx))


def test_index_autograd_is_the_adjoint_pair():
    g = torch.Generator().manual_seed(12)
    idx = (torch.randint(0, 9, (300,), generator=g).to(DEV), torch.randint(0, 7, (300,), generator=g).to(DEV))
    x = torch.randn(2, 9, 7, generator=g).to(DEV).requires_grad_(True)
    y = T.index(x, idx)
    gy = torch.randn(2, 300, generator=g).to(DEV)
    (gx,) = torch.autograd.grad(y, x, gy)
    assert torch.equal(gx, T.index_adjoint(gy, idx, (9, 7)))
    v = torch.randn(2, 300, generator=g).to(DEV).requires_grad_(True)
    z = T.index_adjoint(v, idx, (9, 7))
    gz = torch.randn(2, 9, 7, generator=g).to(DEV)
    (gv,) = torch.autograd.grad(z, v, gz)
    assert torch.equal(gv, T.index(gz, idx))


def test_index_errors_match_reference():
    with pytest.raises(IndexError, match=r"Out-of-bounds index for grid of shape \(3, 5\): idx\[1\]"):
        T.index_adjoint(torch.ones(3, device=DEV), (torch.tensor([0, 1, 2], device=DEV),
                                                     torch.tensor([0, 5, 1], device=DEV)), (3, 5))
    with pytest.raises(IndexError, match=r"\(4,\): idx\[0\]"):
        T.index_adjoint(torch.ones(2, device=DEV), (torch.tensor([0, -5], device=DEV),), (4,))
    with pytest.raises(ValueError, match="cannot be indexed"):
        T.index(torch.ones(4, device=DEV), (torch.tensor([0], device=DEV),) * 2)
    with pytest.raises(ValueError, match="should correspond"):
        T.index_adjoint(torch.ones(2, 5, device=DEV), (torch.tensor([0, 1, 2], device=DEV),), (4,))


@pytest.mark.parametrize("name", ["2d", "3d"])
def test_nufft_sampling_mode_matches_reference(name):
    """The NUFFT's "sampling" mode (reference linops/nufft.py:185-200): the
    reference's own forward and adjoint (tests/golden/nufft_sampling.npz)."""
    import numpy as np

    from conftest import GOLDEN, rel_l2
    from torchlinops_gb300 import linops

    d = np.load(f"{GOLDEN}/nufft_sampling.npz")
    locs = torch.from_numpy(d[f"{name}_locs"]).to(DEV)
    x = to_torch(d[f"{name}_x"], True).to(DEV)
    A = linops.NUFFT(locs, tuple(x.shape[1:]), mode="sampling")
    assert rel_l2(A(x).cpu(), to_torch(d[f"{name}_fwd"], True)) < 1e-5
    z = to_torch(d[f"{name}_z"], True).to(DEV)
    assert rel_l2(A.H(z).cpu(), to_torch(d[f"{name}_adj"], True)) < 1e-5
