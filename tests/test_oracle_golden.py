"""The oracle is pinned against golden vectors produced by the reference itself."""

import numpy as np
import pytest
import torch

from conftest import GOLDEN, load_cases, rel_l2, to_torch
from oracle import blocks as OB
from oracle import interp as OI

INTERP = load_cases("interp_cases.npz")
BLOCKS = load_cases("blocks_cases.npz")


def test_kernel_values_match_reference():
    k = np.load(f"{GOLDEN}/kernels.npz")
    x = torch.from_numpy(k["x"])
    for key in k.files:
        if key.startswith("kb_"):
            beta = float(key[3:])
            ref = torch.from_numpy(k[key])
            got = OI.kaiser_bessel(x, beta)
            finite = torch.isfinite(ref)
            assert torch.equal(finite, torch.isfinite(got))
            torch.testing.assert_close(got[finite], ref[finite], rtol=2e-6, atol=0)
    torch.testing.assert_close(OI.spline(x), torch.from_numpy(k["spline"]), rtol=0, atol=0)


def test_known_kb_values():
    beta = OI.nufft_beta(4.0, 1.25)
    assert abs(beta - 6.99666) < 1e-5
    one = OI.kaiser_bessel(torch.tensor([1.0, -1.0], dtype=torch.float64), beta)
    assert torch.all(one == 1.0)
    assert torch.isnan(OI.kaiser_bessel(torch.tensor([1.01]), beta)).all()
    assert abs(OI.kaiser_bessel(torch.tensor([0.0], dtype=torch.float64), beta).item() - 168.07) < 0.01


@pytest.mark.parametrize("case", sorted(INTERP))
def test_interp_oracle_matches_reference(case):
    rec = INTERP[case]
    m = rec["meta"]
    cplx = m["complex"]
    locs = torch.from_numpy(rec["locs"])
    img = to_torch(rec["img"], cplx)
    pts = to_torch(rec["pts"], cplx)
    w = m["width"] if not isinstance(m["width"], list) else tuple(m["width"])
    kw = dict(kernel=m["kernel"], norm=1, pad_mode=m["pad_mode"], beta=m["beta"])
    fwd = OI.ungrid(img, locs, w, **kw)
    adj = OI.grid(pts, locs, m["grid_size"], w, **kw)
    ref_fwd = to_torch(rec["fwd"], cplx)
    ref_adj = to_torch(rec["adj"], cplx)
    assert fwd.shape == ref_fwd.shape and adj.shape == ref_adj.shape
    assert rel_l2(fwd, ref_fwd) < 2e-6
    assert rel_l2(adj, ref_adj) < 2e-6
    # the float64 oracle agrees with the reference's float32 arithmetic
    fwd64 = OI.ungrid(img, locs, w, dtype=torch.float64, **kw)
    assert rel_l2(fwd64, ref_fwd) < 1e-5


def test_config1_oracle():
    d = np.load(f"{GOLDEN}/config1_interp2d.npz")
    locs = torch.from_numpy(d["locs"])
    img = to_torch(d["img"], True)
    pts = to_torch(d["pts"], True)
    beta = float(d["beta"])
    fwd = OI.ungrid(img, locs, 4.0, beta=beta)
    adj = OI.grid(pts, locs, (64, 64), 4.0, beta=beta)
    assert rel_l2(fwd, to_torch(d["fwd"], True)) < 2e-6
    assert rel_l2(adj, to_torch(d["adj"], True)) < 2e-6


def test_exact_integer_location():
    d = np.load(f"{GOLDEN}/edge_intloc.npz")
    for tag, cplx in (("r", False), ("c", True)):
        dt = torch.complex64 if cplx else torch.float32
        vals = torch.arange(1, 9).to(dt)
        locs = torch.tensor([[4.0]])
        fwd = OI.ungrid(vals, locs, 4.0)
        adj = OI.grid(torch.tensor([[1.0]]).to(dt), locs, (8,), 4.0)
        torch.testing.assert_close(fwd, to_torch(d[f"fwd_{tag}"], cplx), rtol=1e-6, atol=0)
        torch.testing.assert_close(adj, to_torch(d[f"adj_{tag}"], cplx), rtol=1e-6, atol=0)
        # 5 taps at an exact integer (the outer two have weight KB(1) = 1)
        assert int((adj != 0).sum()) == 5


@pytest.mark.parametrize("case", sorted(BLOCKS))
def test_blocks_oracle_matches_reference(case):
    rec = BLOCKS[case]
    m = rec["meta"]
    cplx = "complex" in m["dtype"]
    x = to_torch(rec["x"], cplx)
    y = to_torch(rec["y"], cplx)
    assert torch.equal(OB.unfold(x, m["block"], m["stride"]), to_torch(rec["unfold"], cplx))
    assert torch.equal(OB.fold(y, m["shape"], m["block"], m["stride"]), to_torch(rec["fold"], cplx))
    if "mask" in rec:
        mask = torch.from_numpy(rec["mask"])
        ym = to_torch(rec["ym"], cplx)
        assert torch.equal(OB.unfold(x, m["block"], m["stride"], mask), to_torch(rec["unfold_masked"], cplx))
        assert torch.equal(OB.fold(ym, m["shape"], m["block"], m["stride"], mask), to_torch(rec["fold_masked"], cplx))


def test_get_nblocks_known_answers():
    # get_nblocks doctests, reference _unfold/nblocks.py:15-26
    assert OB.get_nblocks((5, 5), (3, 3), (1, 1)) == (3, 3)
    assert OB.get_nblocks((5, 5), (3, 3), (2, 2)) == (2, 2)
    assert OB.get_nblocks((6, 6), (3, 3), (2, 2)) == (2, 2)
    assert OB.get_nblocks((7, 7), (3, 3), (2, 2)) == (3, 3)
    assert OB.get_nblocks((10, 10), (8, 8), (4, 4)) == (1, 1)


def test_norm_weights_round_trip():
    # reference _unfold/tests/test_adjoint.py:61-81
    w = OB.norm_weights((15, 15), (3, 3), (1, 1))
    x = torch.randn(1, 15, 15, generator=torch.Generator().manual_seed(3))
    x2 = (1.0 / w.clamp(min=1e-6)) * OB.fold(OB.unfold(x, (3, 3), (1, 1)), (15, 15), (3, 3), (1, 1))
    torch.testing.assert_close(x, x2)


@pytest.mark.parametrize("name", ["2d", "3d"])
def test_nufft_oracle_matches_reference_golden(name):
    """The NUFFT oracle (float32 mirror and FP64) against the reference's own
    functional nufft / nufft_adjoint outputs (tests/golden/make_golden.py)."""
    from oracle import nufft as ON

    d = np.load(f"{GOLDEN}/nufft.npz")
    x = to_torch(d[f"{name}_x"], True)
    y = to_torch(d[f"{name}_y"], True)
    locs = torch.from_numpy(d[f"{name}_locs"])
    fwd = to_torch(d[f"{name}_fwd"], True)
    adj = to_torch(d[f"{name}_adj"], True)
    for dtype, tol in ((torch.float32, 2e-6), (torch.float64, 1e-5)):
        assert rel_l2(ON.nufft(x, locs, dtype=dtype), fwd) < tol
        assert rel_l2(ON.nufft_adjoint(y, locs, tuple(x.shape[-locs.shape[-1]:]), dtype=dtype), adj) < tol


TOEPLITZ = {"2d": (16, 16), "2d_batch_dcf": (12, 16), "2d_odd_pad": (12, 14), "3d": (8, 8, 8)}


@pytest.mark.parametrize("name", sorted(TOEPLITZ))
def test_toeplitz_oracle_matches_reference_golden(name):
    """The Toeplitz PSF kernel and normal operator of the oracle (float32
    mirror and FP64) against the reference's NUFFT(toeplitz=True).normal(inner)
    and toeplitz_psf outputs, including a diagonal point weighting with a
    batched image and the odd-padding case whose rescaled points and larger
    grid disagree by one cell."""
    from oracle import nufft as ON

    d = np.load(f"{GOLDEN}/toeplitz.npz")
    shape = TOEPLITZ[name]
    locs = torch.from_numpy(d[f"{name}_locs"])
    x = to_torch(d[f"{name}_x"], True)
    w = torch.from_numpy(d[f"{name}_dcf"]) if f"{name}_dcf" in d.files else None
    kern = to_torch(d[f"{name}_kernel"], True)
    normal = to_torch(d[f"{name}_normal"], True)
    for dtype, tol in ((torch.float32, 2e-6), (torch.float64, 1e-5)):
        K = ON.toeplitz_kernel(locs, shape, weight=w, dtype=dtype)
        assert rel_l2(K, kern) < tol
        assert rel_l2(ON.toeplitz_normal(x, K, shape), normal) < tol


INDEX = load_cases("index_cases.npz")


def _index_case(rec):
    m = rec["meta"]
    cplx = "complex" in m["dtype"]
    idx = tuple(torch.from_numpy(rec[f"idx{d}"]) for d in range(m["ndim"]) if f"idx{d}" in rec)
    return m, cplx, idx


@pytest.mark.parametrize("case", sorted(INDEX))
def test_index_oracle_matches_reference(case):
    """oracle.index against the reference's own index / index_adjoint: bit-exact
    (the CPU index_add_ sums each cell's samples in ascending order)."""
    from oracle import index as OX

    rec = INDEX[case]
    m, cplx, idx = _index_case(rec)
    if "vals" in rec:
        out = OX.index_adjoint(to_torch(rec["vals"], cplx), idx, m["grid"])
        assert torch.equal(out, to_torch(rec["out"], cplx))
    if "fwd" in rec and idx:
        assert torch.equal(OX.index(to_torch(rec["grid_vals"], cplx), idx), to_torch(rec["fwd"], cplx))


def test_index_oracle_bounds_error():
    from oracle import index as OX

    with pytest.raises(IndexError, match=r"idx\[1\]"):
        OX.index_adjoint(torch.ones(3), (torch.tensor([0, 1, 2]), torch.tensor([0, 5, 1])), (3, 5))


CIRC = load_cases("circpad_cases.npz")


@pytest.mark.parametrize("case", sorted(CIRC))
def test_circpad_oracle_matches_reference(case):
    """oracle.circpad against the reference's circular_pad (bit-exact: copies),
    its autograd adjoint and its Convolution linop in circular mode."""
    from oracle import circpad as OC

    rec = CIRC[case]
    m = rec["meta"]
    cplx = m["complex"]
    if "padding" in m:
        x = to_torch(rec["x"], cplx)
        assert torch.equal(OC.circular_pad(x, m["padding"]), to_torch(rec["pad"], cplx))
        adj = OC.circular_pad_adjoint(to_torch(rec["z"], cplx), m["padding"])
        assert rel_l2(adj, to_torch(rec["adj"], cplx)) < 1e-6
    else:
        k = to_torch(rec["kernel"], cplx)
        assert rel_l2(OC.conv_circular(k, to_torch(rec["x"], cplx)), to_torch(rec["fwd"], cplx)) < 1e-6
        assert rel_l2(OC.conv_circular(k, to_torch(rec["z"], cplx), adjoint=True), to_torch(rec["adj"], cplx)) < 1e-6
