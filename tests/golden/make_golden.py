"""Generate golden vectors by running the reference itself (torchlinops 0.7.4).

Run in a container that has the reference source:

    python tests/golden/make_golden.py --ref <torch-named-linops checkout>/src

(or set ``TORCHLINOPS_SRC`` to that directory instead of passing ``--ref``).

It imports the reference's functional API with a no-op ``jaxtyping`` stub
(``tests/golden/_stubs``) and runs its pure-torch CPU path (``ungrid_torch``,
``grid_torch``, ``_unfold_torch``, ``_fold_torch``, ``kaiser_bessel_torch``)
on small seeded inputs, writing ``tests/golden/*.npz``. ``toeplitz.npz`` comes
from its linops: ``NUFFT(..., toeplitz=True).normal(inner)`` and
``toeplitz_psf`` (``--only toeplitz`` rewrites just that file). The fixtures
are the parity pins for the oracle (``tests/test_oracle_golden.py``) and, on
the GPU, for the CUDA kernels (``tests/test_interp_gpu.py``,
``tests/test_blocks_gpu.py``, ``tests/test_linops_gpu.py``,
``tests/test_toeplitz_gpu.py``).
"""

from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))

NUFFT_BETA = float(np.pi * (((4.0 / 1.25) * (1.25 - 0.5)) ** 2 - 0.8) ** 0.5)


def _np(t: torch.Tensor) -> np.ndarray:
    t = t.detach().cpu()
    if t.is_complex():
        return torch.view_as_real(t.contiguous()).numpy()
    return t.numpy()


def _rand(shape, is_complex, gen):
    if is_complex:
        re = torch.randn(shape, generator=gen)
        im = torch.randn(shape, generator=gen)
        return torch.complex(re, im)
    return torch.randn(shape, generator=gen)


INTERP_SPECS = {
    # name: (batch N, grid_size, locs batch, width) -- shapes of the
    # reference fixtures in _interp/tests/conftest.py
    "small1d": ((2,), (10,), (20,), 4.0),
    "small2d": ((2, 2), (10, 8), (9,), 4.0),
    "tiny2d": ((2,), (2, 2), (1,), 2.0),
    "small3d": ((1, 1), (10, 8, 9), (3, 5), 4.0),
    "medium1d": ((2, 2), (24,), (6, 11), 4.0),
    "medium2d": ((2, 2), (124, 125), (3, 19), 4.0),
    "medium3d": ((1,), (33, 35, 37), (3, 19), 4.0),
    "aniso3d": ((3,), (12, 9, 14), (40,), (4.0, 3.0, 5.5)),
}

KERNELS = [
    ("kaiser_bessel", {"beta": 1.0}),
    ("kaiser_bessel", {"beta": NUFFT_BETA}),
    ("spline", {}),
]


def make_interp(F, out_dir):
    cases = {}
    seed = 0
    for name, (N, gsz, lbs, width) in INTERP_SPECS.items():
        small = not name.startswith("medium")
        kerns = KERNELS if small else [KERNELS[1]]
        dtypes = [False, True] if small else [True]
        for kname, kparams in kerns:
            for pad in ("circular", "zero"):
                for cplx in dtypes:
                    seed += 1
                    gen = torch.Generator().manual_seed(seed)
                    ndim = len(gsz)
                    # points range past both edges so wrap / zero-pad paths are hit
                    lo, hi = (-2.5, 2.5) if small else (0.0, 0.0)
                    locs = torch.stack(
                        [torch.rand(lbs, generator=gen) * (g + hi - lo) + lo for g in gsz], -1
                    ).to(torch.float32)
                    if small:
                        # a few exact integer and half-integer coordinates
                        flat = locs.reshape(-1, ndim)
                        flat[0] = torch.tensor([float(g // 2) for g in gsz])
                        if flat.shape[0] > 1:
                            flat[1] = torch.tensor([float(g // 2) + 0.5 for g in gsz])
                    img = _rand((*N, *gsz), cplx, gen)
                    pts = _rand((*N, *lbs), cplx, gen)
                    w = width if isinstance(width, float) else tuple(width)
                    fwd = F.interpolate(img, locs, w, kernel=kname, norm=1, pad_mode=pad, kernel_params=dict(kparams))
                    adj = F.interpolate_adjoint(
                        pts, locs, gsz, w, kernel=kname, norm=1, pad_mode=pad, kernel_params=dict(kparams)
                    )
                    key = f"{name}-{kname}-{kparams.get('beta', 0):.5f}-{pad}-{'c' if cplx else 'r'}"
                    meta = dict(
                        spec=name,
                        N=list(N),
                        grid_size=list(gsz),
                        locs_batch=list(lbs),
                        width=list(width) if isinstance(width, tuple) else width,
                        kernel=kname,
                        beta=kparams.get("beta", 1.0),
                        pad_mode=pad,
                        complex=cplx,
                        norm=1,
                    )
                    cases[key] = dict(
                        meta=json.dumps(meta),
                        locs=_np(locs),
                        img=_np(img),
                        pts=_np(pts),
                        fwd=_np(fwd),
                        adj=_np(adj),
                    )
    np.savez_compressed(os.path.join(out_dir, "interp_cases.npz"), **_flatten(cases))
    return len(cases)


def make_config1(F, out_dir):
    """Plain 2D Interpolate forward+adjoint: grid 64x64 c64, 4096 pts, KB W=4, seed 0."""
    gen = torch.Generator().manual_seed(0)
    img = torch.complex(torch.randn(64, 64, generator=gen), torch.randn(64, 64, generator=gen))
    locs = (torch.rand(4096, 2, generator=gen) * 64).to(torch.float32)
    pts = torch.complex(torch.randn(4096, generator=gen), torch.randn(4096, generator=gen))
    kp = dict(beta=NUFFT_BETA)
    fwd = F.interpolate(img, locs, 4.0, kernel="kaiser_bessel", kernel_params=dict(kp))
    adj = F.interpolate_adjoint(pts, locs, (64, 64), 4.0, kernel="kaiser_bessel", kernel_params=dict(kp))
    np.savez_compressed(
        os.path.join(out_dir, "config1_interp2d.npz"),
        locs=_np(locs),
        img=_np(img),
        pts=_np(pts),
        fwd=_np(fwd),
        adj=_np(adj),
        beta=np.float64(NUFFT_BETA),
    )


def make_edgecases(F, out_dir):
    """Exact integer location (reference _interp/tests/test_edgecases.py:16-65)."""
    out = {}
    for cplx in (False, True):
        dt = torch.complex64 if cplx else torch.float32
        vals = torch.arange(1, 9).to(dt)
        locs = torch.tensor([[4.0]])
        fwd = F.ungrid(vals, locs, width=4.0, kernel="kaiser_bessel")
        gv = torch.tensor([[1.0]]).to(dt)
        adj = F.grid(gv, locs, (8,), width=4.0, kernel="kaiser_bessel")
        tag = "c" if cplx else "r"
        out[f"fwd_{tag}"] = _np(fwd)
        out[f"adj_{tag}"] = _np(adj)
    np.savez_compressed(os.path.join(out_dir, "edge_intloc.npz"), **out)


def make_nufft(F, out_dir):
    """Functional NUFFT / adjoint (functional/_nufft.py:16-112), 2D and 3D."""
    out = {}
    for name, shape, npts, batch in (("2d", (24, 20), 300, (2,)), ("3d", (12, 10, 14), 400, (1,))):
        gen = torch.Generator().manual_seed(len(name) * 31 + npts)
        x = torch.complex(torch.randn(*batch, *shape, generator=gen), torch.randn(*batch, *shape, generator=gen))
        locs = torch.stack([torch.rand(npts, generator=gen) * s - s / 2 for s in shape], -1).to(torch.float32)
        y = torch.complex(torch.randn(*batch, npts, generator=gen), torch.randn(*batch, npts, generator=gen))
        out[f"{name}_x"] = _np(x)
        out[f"{name}_locs"] = _np(locs)
        out[f"{name}_y"] = _np(y)
        out[f"{name}_fwd"] = _np(F.nufft(x, locs, oversamp=1.25, width=4.0))
        out[f"{name}_adj"] = _np(F.nufft_adjoint(y, locs, shape, oversamp=1.25, width=4.0))
    np.savez_compressed(os.path.join(out_dir, "nufft.npz"), **out)


TOEPLITZ_SPECS = {
    # name: (grid_size, points, batch of the image, density weights)
    "2d": ((16, 16), 60, (), False),
    "2d_batch_dcf": ((12, 16), 45, (3,), True),
    # 14 pads to 17, and the 2x grid's 28 to 35, not 2 * 17: the reference
    # rescales the points to 34 cells on a 35-cell grid (its PSF is then off)
    "2d_odd_pad": ((12, 14), 45, (2,), False),
    "3d": ((8, 8, 8), 40, (), False),
}


def make_toeplitz(L, out_dir):
    """The NUFFT's Toeplitz normal (linops/nufft.py:226-239, 395-494): the
    PSF kernel (the Dense weight, centred k-space on the 2x grid) and the
    normal operator applied to a seeded image, with and without a diagonal
    weighting of the points (``inner``)."""
    from torchlinops.linops.nufft import toeplitz_psf

    out = {}
    for name, (shape, npts, batch, dcf) in TOEPLITZ_SPECS.items():
        gen = torch.Generator().manual_seed(7 + len(shape) + npts)
        locs = (torch.rand(npts, len(shape), generator=gen) - 0.5) * torch.tensor(shape, dtype=torch.float32)
        x = _rand(tuple(batch) + tuple(shape), True, gen)
        A = L.NUFFT(locs, shape, output_shape=("K",), toeplitz=True)
        inner = None
        if dcf:
            w = torch.rand(npts, generator=gen) + 0.5
            inner = L.Diagonal(w, ioshape=("...", "K"))
            out[f"{name}_dcf"] = _np(w)
        T = A.normal(inner)
        kern = toeplitz_psf(A, inner)
        out[f"{name}_locs"] = _np(locs)
        out[f"{name}_x"] = _np(x)
        out[f"{name}_kernel"] = _np(kern.weight.reshape(kern.weight.shape[-len(shape):]))
        out[f"{name}_normal"] = _np(T(x).reshape(x.shape))
    np.savez_compressed(os.path.join(out_dir, "toeplitz.npz"), **out)


def make_kernels(K, out_dir):
    x = torch.linspace(-1.2, 1.2, 241)
    out = {"x": _np(x)}
    for beta in (1.0, 2.0, NUFFT_BETA, 12.0):
        out[f"kb_{beta:.5f}"] = _np(K.kaiser_bessel_torch(x, beta=beta))
    out["spline"] = _np(K.spline_torch(x))
    np.savez_compressed(os.path.join(out_dir, "kernels.npz"), **out)


BLOCK_SPECS = {
    # reference fixtures of _unfold/tests/conftest.py (+ the 3D mask cross)
    "small1d": ((1,), (15,), (3,), (1,), [0, 1, 0]),
    "medium1d": ((2, 2), (33,), (7,), (2,), None),
    "tiny2d": ((1,), (4, 4), (2, 2), (1, 1), None),
    "small2d": ((1,), (15, 15), (3, 3), (1, 1), [[0, 1, 0], [1, 1, 1], [0, 1, 0]]),
    "medium2d": ((2, 2), (33, 43), (7, 7), (2, 2), None),
    "tiny3d": ((1,), (4, 4, 4), (2, 2, 2), (1, 1, 1), None),
    "small3d": (
        (1,),
        (15, 15, 15),
        (3, 3, 3),
        (1, 1, 1),
        [[[0, 0, 0], [0, 1, 0], [0, 0, 0]], [[0, 1, 0], [1, 1, 1], [0, 1, 0]], [[0, 0, 0], [0, 1, 0], [0, 0, 0]]],
    ),
    "medium3d": ((2,), (17, 21, 13), (7, 7, 5), (2, 2, 2), None),
    "overlap3d": ((2,), (16, 16, 16), (8, 8, 8), (4, 4, 4), None),
}


def make_blocks(F, out_dir):
    cases = {}
    seed = 1000
    for name, (N, shape, blk, st, mask) in BLOCK_SPECS.items():
        dts = (torch.float32, torch.float64, torch.complex64)
        if name.startswith(("medium", "overlap")):
            dts = (torch.float32, torch.complex64)
        for dt in dts:
            seed += 1
            gen = torch.Generator().manual_seed(seed)
            nb = F.get_nblocks(shape, blk, st)
            cplx = dt.is_complex
            x = _rand((*N, *shape), cplx, gen)
            y = _rand((*N, *nb, *blk), cplx, gen)
            if not cplx:
                x, y = x.to(dt), y.to(dt)
            ux = F.array_to_blocks(x, blk, st)
            fy = F.blocks_to_array(y, shape, blk, st)
            rec = dict(x=_np(x), y=_np(y), unfold=_np(ux), fold=_np(fy))
            if mask is not None:
                m = torch.tensor(mask, dtype=torch.bool)
                ym = y[..., m].contiguous()
                rec["mask"] = m.numpy()
                rec["unfold_masked"] = _np(F.array_to_blocks(x, blk, st, m))
                rec["ym"] = _np(ym)
                rec["fold_masked"] = _np(F.blocks_to_array(ym, shape, blk, st, m))
            meta = dict(spec=name, N=list(N), shape=list(shape), block=list(blk), stride=list(st), dtype=str(dt), nblocks=list(nb))
            rec["meta"] = json.dumps(meta)
            cases[f"{name}-{str(dt).split('.')[-1]}"] = rec
    np.savez_compressed(os.path.join(out_dir, "blocks_cases.npz"), **_flatten(cases))
    return len(cases)


def make_index(F, out_dir):
    """Sampling ops: the reference's known answer (_index/tests/test_index.py:26-34),
    collisions in 1D/2D/3D with negative indices, real, complex and integer
    values, a broadcast index and a sliced index for the gather."""
    cases = {}
    gen = torch.Generator().manual_seed(2024)

    def rnd_idx(shape, size):
        return torch.randint(-size, size, shape, generator=gen)

    def add(name, vals, idx, grid, fwd_vals=None):
        rec = dict(vals=_np(vals), out=_np(F.index_adjoint(vals, idx, grid)))
        for d, i in enumerate(idx):
            rec[f"idx{d}"] = i.numpy()
        if fwd_vals is not None:
            rec["grid_vals"] = _np(fwd_vals)
            rec["fwd"] = _np(F.index(fwd_vals, idx))
        rec["meta"] = json.dumps(dict(grid=list(grid), ndim=len(idx), dtype=str(vals.dtype)))
        cases[name] = rec

    add("known1d", torch.tensor([[5.0, 4.0, -1.0], [5.0, 4.0, -1.0]]), (torch.tensor([1, 3, 2]),), (4,))
    i1 = (rnd_idx((2000,), 37),)
    add("collide1d_f32", torch.randn(3, 2000, generator=gen), i1, (37,), torch.randn(3, 37, generator=gen))
    add("collide1d_i64", torch.randint(-50, 50, (2, 2000), generator=gen), i1, (37,))
    i2 = (rnd_idx((50, 40), 23), rnd_idx((50, 40), 31))
    v2 = torch.complex(torch.randn(2, 4, 50, 40, generator=gen), torch.randn(2, 4, 50, 40, generator=gen))
    g2 = torch.complex(torch.randn(2, 4, 23, 31, generator=gen), torch.randn(2, 4, 23, 31, generator=gen))
    add("collide2d_c64", v2, i2, (23, 31), g2)
    i3 = (rnd_idx((5000,), 9), rnd_idx((5000,), 11), rnd_idx((5000,), 13))
    add("collide3d_f64", torch.randn(2, 5000, generator=gen, dtype=torch.float64), i3, (9, 11, 13),
        torch.randn(2, 9, 11, 13, generator=gen, dtype=torch.float64))
    # gathers only: a broadcast index and a sliced one
    gv = torch.randn(3, 7, 5, generator=gen)
    ib = (torch.tensor([1, 0, 6, -2])[:, None], torch.tensor([4, 2, 0])[None, :])
    cases["bcast_fwd"] = dict(grid_vals=_np(gv), idx0=ib[0].numpy(), idx1=ib[1].numpy(), fwd=_np(F.index(gv, ib)),
                              meta=json.dumps(dict(grid=[7, 5], ndim=2, dtype="torch.float32")))
    gs = torch.arange(8).reshape(2, 4)
    cases["slice_fwd"] = dict(grid_vals=gs.numpy(), fwd=F.index(gs, (slice(None), slice(1, 4))).numpy(),
                              meta=json.dumps(dict(grid=[2, 4], ndim=2, dtype="torch.int64", slices=[[None, None], [1, 4]])))
    np.savez_compressed(os.path.join(out_dir, "index_cases.npz"), **_flatten(cases))
    return len(cases)


def make_circpad(L, out_dir):
    """Circular padding (functional/_interp/_circ_pad.py) and the Convolution
    linop in circular mode (linops/convolution.py): the reference's own test
    shapes (_interp/tests/test_circular_pad.py), asymmetric and zero pads,
    batches, and a convolution forward / adjoint in 1D, 2D and 3D."""
    from torchlinops.functional._interp._circ_pad import circular_pad, circular_pad_adjoint

    cases = {}
    gen = torch.Generator().manual_seed(77)
    specs = {
        "ref2d": ((15, 20), [4, 4, 2, 2], False),
        "refnd": ((5, 15, 20, 19, 18), [1, 1, 2, 2, 3, 3, 5, 5], False),
        "ref1d_c": ((3,), [1, 1], True),
        "ref2d_c": ((3, 3), [2, 2, 1, 1], True),
        "asym3d_c": ((2, 3, 9, 10, 11), [3, 2, 0, 4, 1, 1], True),
        "full1d": ((4, 6), [6, 6], False),
    }
    for name, (shape, padding, cplx) in specs.items():
        x = _rand(shape, cplx, gen)
        y = circular_pad(x, padding)
        z = _rand(tuple(y.shape), cplx, gen)
        adj = circular_pad_adjoint(z, padding)
        meta = dict(padding=padding, complex=cplx)
        cases[name] = dict(x=_np(x), pad=_np(y), z=_np(z), adj=_np(adj.detach()), meta=json.dumps(meta))
    conv_specs = {
        "conv1d": ((3, 40), (5,)),
        "conv2d_even": ((2, 3, 21, 18), (4, 3)),
        "conv3d_c": ((2, 12, 13, 11), (3, 4, 3)),
    }
    for name, (xshape, kshape) in conv_specs.items():
        cplx = name.endswith("_c")
        kern = _rand(kshape, cplx, gen)
        x = _rand(xshape, cplx, gen)
        A = L.Convolution(kern, padding_mode="circular")
        y = A(x)
        z = _rand(tuple(y.shape), cplx, gen)
        yh = A.H(z)
        meta = dict(complex=cplx)
        cases[name] = dict(kernel=_np(kern), x=_np(x), fwd=_np(y), z=_np(z), adj=_np(yh), meta=json.dumps(meta))
    np.savez_compressed(os.path.join(out_dir, "circpad_cases.npz"), **_flatten(cases))
    return len(cases)


def make_nufft_sampling(L, out_dir):
    """The NUFFT in its "sampling" mode (linops/nufft.py:185-200): pad, centred
    FFT, then Sampling at rounded, wrapped k-space indices; forward and
    adjoint in 2D and 3D, complex64, with repeated indices."""
    out = {}
    gen = torch.Generator().manual_seed(31)
    for name, shape, npts in (("2d", (16, 20), 700), ("3d", (8, 10, 6), 900)):
        locs = (torch.rand(npts, len(shape), generator=gen) - 0.5) * torch.tensor(shape, dtype=torch.float32)
        x = _rand((2, *shape), True, gen)
        A = L.NUFFT(locs, shape, output_shape=("K",), mode="sampling")
        y = A(x)
        z = _rand(tuple(y.shape), True, gen)
        out[f"{name}_locs"] = locs.numpy()
        out[f"{name}_x"] = _np(x)
        out[f"{name}_fwd"] = _np(y)
        out[f"{name}_z"] = _np(z)
        out[f"{name}_adj"] = _np(A.H(z))
    np.savez_compressed(os.path.join(out_dir, "nufft_sampling.npz"), **out)
    return len(out) // 5


def _flatten(cases):
    flat = {}
    for k, rec in cases.items():
        for f, v in rec.items():
            flat[f"{k}|{f}"] = np.asarray(v)
    return flat


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("TORCHLINOPS_SRC"),
                    help="the reference's src/ directory (default: $TORCHLINOPS_SRC)")
    ap.add_argument("--out", default=HERE)
    ap.add_argument("--only", choices=["toeplitz", "index", "circpad", "nufft_sampling"], default=None, help="write only this fixture")
    args = ap.parse_args()
    if not args.ref:
        ap.error("give the reference's src/ directory with --ref or TORCHLINOPS_SRC")
    sys.path.insert(0, os.path.join(HERE, "_stubs"))
    sys.path.insert(0, args.ref)
    torch.set_num_threads(os.cpu_count() or 1)
    import torchlinops.functional as F
    import torchlinops.linops as L
    from torchlinops.functional._interp import kernels as K

    t0 = time.time()
    if args.only == "toeplitz":
        make_toeplitz(L, args.out)
        print(f"wrote toeplitz.npz in {time.time() - t0:.1f}s")
        return
    if args.only == "nufft_sampling":
        n = make_nufft_sampling(L, args.out)
        print(f"wrote {n} sampling-mode NUFFT cases in {time.time() - t0:.1f}s")
        return
    if args.only == "circpad":
        n = make_circpad(L, args.out)
        print(f"wrote {n} circular pad cases in {time.time() - t0:.1f}s")
        return
    if args.only == "index":
        n = make_index(F, args.out)
        print(f"wrote {n} index cases in {time.time() - t0:.1f}s")
        return
    make_kernels(K, args.out)
    make_edgecases(F, args.out)
    make_config1(F, args.out)
    make_nufft(F, args.out)
    make_toeplitz(L, args.out)
    n_i = make_interp(F, args.out)
    n_b = make_blocks(F, args.out)
    n_x = make_index(F, args.out)
    n_c = make_circpad(L, args.out)
    make_nufft_sampling(L, args.out)
    print(f"wrote {n_i} interp cases, {n_b} block cases, {n_x} index cases, {n_c} circular pad cases in "
          f"{time.time() - t0:.1f}s")


if __name__ == "__main__":
    main()
