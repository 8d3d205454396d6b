"""Checks that need no GPU: the C-ABI library loads, exports every symbol
that include/tlgb.h declares with the declared parameters, and validates
descriptors and launch sizes and sizes the gridding scratch on the host; the
Python layer's host-side logic
(location rescaling with the reference's rounding, batch ranges, the
Toeplitz normal's inner operators) runs as the reference's does."""

import ctypes
import os
import re

import pytest
import torch

from conftest import ROOT
from torchlinops_gb300 import _ext


def _header_symbols():
    txt = open(os.path.join(ROOT, "include", "tlgb.h")).read()
    return sorted(set(re.findall(r"\b(tlgb_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    L = _ext.lib()
    declared = _header_symbols()
    assert declared, "no declarations parsed"
    for name in declared:
        assert hasattr(L, name), f"{name} declared in include/tlgb.h but not exported"
    assert set(declared) == set(_ext.exported_symbols())
    assert L.tlgb_version() >= 100


def _desc(**kw):
    d = _ext.InterpDesc()
    d.ndim = kw.get("ndim", 3)
    d.kernel = kw.get("kernel", 0)
    d.norm = kw.get("norm", 1)
    d.pad_mode = kw.get("pad", 0)
    for i in range(3):
        d.grid_size[i] = kw.get("n", 64)
        d.width[i] = kw.get("width", 4.0)
    d.beta = 1.0
    d.npts = kw.get("npts", 1000)
    d.nbatch = kw.get("nbatch", 1)
    return d


def _size(d):
    pb, tb = ctypes.c_size_t(), ctypes.c_size_t()
    st = _ext.lib().tlgb_interp_plan_size(ctypes.byref(d), ctypes.byref(pb), ctypes.byref(tb))
    return st, pb.value, tb.value


def test_plan_size_and_host_validation():
    st, pb, tb = _size(_desc())
    assert st == 0 and pb > 1000 * 8 * 4 and tb > 0
    assert _size(_desc(ndim=4))[0] == _ext.TLGB_ERR_INVALID
    assert _size(_desc(kernel=7))[0] == _ext.TLGB_ERR_INVALID
    assert _size(_desc(norm=3))[0] == _ext.TLGB_ERR_INVALID
    assert _size(_desc(width=-1.0))[0] == _ext.TLGB_ERR_INVALID
    st = _size(_desc(width=9.0))[0]  # 3D width above the supported maximum
    assert st == _ext.TLGB_ERR_UNSUPPORTED
    assert b"width" in _ext.lib().tlgb_last_error()
    assert _size(_desc(ndim=2, width=9.0))[0] == 0


def test_blocks_host_validation():
    d = _ext.BlocksDesc()
    d.ndim = 3
    d.dtype = 2
    d.nbatch = 1
    for i in range(3):
        d.im_size[i] = 4
        d.block[i] = 8  # block larger than the array
        d.stride[i] = 1
    d.nnz = 512
    st = _ext.lib().tlgb_unfold(ctypes.byref(d), ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    assert st == _ext.TLGB_ERR_INVALID
    d.dtype = 9
    assert _ext.lib().tlgb_fold(ctypes.byref(d), ctypes.c_void_p(16), ctypes.c_void_p(16), None) != 0


def test_product_path_has_no_cpu_fallback():
    import torchlinops_gb300 as T

    x = torch.randn(8, 8, dtype=torch.complex64)
    locs = torch.rand(10, 2) * 8
    with pytest.raises(RuntimeError, match="CUDA"):
        T.interpolate(x, locs, 4.0)
    with pytest.raises(RuntimeError, match="CUDA"):
        T.unfold(x, (2, 2), (1, 1))
    with pytest.raises(ValueError):
        T.interpolate(x, locs, 4.0, kernel="gaussian")


@pytest.mark.parametrize("gs,ps", [((256, 256), (320, 320)), ((205, 205, 205), (256, 256, 256)),
                                   ((24, 20), (30, 25)), ((33,), (41,))])
@pytest.mark.parametrize("pad_mode", ["circular", "zero"])
def test_prep_locs_keeps_the_reference_rounding(gs, ps, pad_mode):
    """The NUFFT's location rescaling (host-side torch ops) gives the
    reference's float32 coordinates bit for bit: per dimension, multiply by
    Np/N, add Np//2, clamp or wrap (linops/nufft.py:242-334), whether it runs
    on all dimensions at once or one dimension at a time."""
    from torchlinops_gb300 import linops

    g = torch.Generator().manual_seed(len(gs) + ps[-1])
    locs = (torch.rand(50000, len(gs), generator=g) - 0.5) * torch.tensor(gs, dtype=torch.float32) * 1.02
    ref = locs.clone()
    for i in range(-len(gs), 0):
        ref[..., i] *= ps[i] / gs[i]
        ref[..., i] += ps[i] // 2
        if pad_mode == "zero":
            ref[..., i] = torch.clamp(ref[..., i], 0, ps[i] - 1)
        else:
            ref[..., i] = torch.remainder(ref[..., i], torch.tensor(ps[i]))
    assert torch.equal(linops.prep_locs(locs, gs, ps, pad_mode), ref)


def _header_prototypes():
    """{name: [parameter type, ...]} of the functions declared in tlgb.h."""
    txt = open(os.path.join(ROOT, "include", "tlgb.h")).read()
    txt = re.sub(r"/\*.*?\*/", " ", txt, flags=re.S)
    protos = {}
    for m in re.finditer(r"\b(?:int|size_t|const char\s*\*)\s+(tlgb_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", txt):
        params = " ".join(m.group(2).split())
        if params in ("", "void"):
            protos[m.group(1)] = []
            continue
        types = []
        for p in params.split(","):
            p = p.strip()
            # drop the parameter name
            p = re.sub(r"\b[a-z_][a-z0-9_]*$", "", p).strip() if not p.endswith("*") else p
            types.append(p)
        protos[m.group(1)] = types
    return protos


def _ctype_matches(c_type: str, ct) -> bool:
    if "*" in c_type or c_type == "tlgb_stream_t":
        return ct in (ctypes.c_void_p, ctypes.c_char_p) or getattr(ct, "__name__", "").startswith("LP_")
    table = {"int64_t": ctypes.c_int64, "int32_t": ctypes.c_int32, "size_t": ctypes.c_size_t, "float": ctypes.c_float,
             "double": ctypes.c_double, "int": ctypes.c_int}
    want = table.get(c_type.replace("const ", "").strip())
    return want is not None and ctypes.sizeof(want) == ctypes.sizeof(ct) and (want is ct or want == ct)


def test_ctypes_signatures_match_the_header():
    """Every binding in _ext has the declared number of parameters, each of a
    matching kind and width (pointer, 32/64-bit integer, size_t, float)."""
    protos = _header_prototypes()
    assert protos
    assert set(protos) == set(_ext._SIGNATURES), set(protos) ^ set(_ext._SIGNATURES)
    for name, ctypes_args in ((n, s[0]) for n, s in _ext._SIGNATURES.items()):
        c_args = protos[name]
        assert len(c_args) == len(ctypes_args), f"{name}: header {len(c_args)} params, ctypes {len(ctypes_args)}"
        for i, (c, ct) in enumerate(zip(c_args, ctypes_args)):
            assert _ctype_matches(c, ct), f"{name} parameter {i}: header {c!r}, ctypes {ct}"


def test_launch_limits_are_host_errors():
    """Sizes whose launch grid would overflow are rejected on the host before
    any launch, with TLGB_ERR_UNSUPPORTED: an interpolation batch above
    TLGB_INTERP_MAX_BATCH (the Python layer splits such batches), a block op
    with 2^31 rows of blocks or array planes, a pad/crop volume of 2^38
    voxels."""
    from torchlinops_gb300 import interp as I

    L = _ext.lib()
    txt = open(os.path.join(ROOT, "include", "tlgb.h")).read()
    assert I.MAX_BATCH == int(re.search(r"#define TLGB_INTERP_MAX_BATCH (\d+)", txt).group(1)) == 8 * 65535
    assert _size(_desc(nbatch=I.MAX_BATCH))[0] == 0
    assert _size(_desc(nbatch=I.MAX_BATCH + 1))[0] == _ext.TLGB_ERR_UNSUPPORTED
    assert b"batch" in L.tlgb_last_error()

    d = _ext.BlocksDesc()
    d.ndim, d.dtype, d.nbatch = 1, 0, 1 << 31
    d.im_size[0], d.block[0], d.stride[0] = 8, 4, 4
    d.nnz = 4
    p = ctypes.c_void_p(16)
    assert L.tlgb_unfold(ctypes.byref(d), p, p, None) == _ext.TLGB_ERR_UNSUPPORTED
    assert L.tlgb_fold(ctypes.byref(d), p, p, None) == _ext.TLGB_ERR_UNSUPPORTED
    assert b"batch" in L.tlgb_last_error()

    big = (ctypes.c_int64 * 3)(1 << 29, 1 << 29, 1 << 29)
    zero = (ctypes.c_int64 * 3)(0, 0, 0)
    st = L.tlgb_pad_shift_c64(p, 1, 3, big, big, zero, zero, 0, None, None, 0, p, None)
    assert st == _ext.TLGB_ERR_UNSUPPORTED
    st = L.tlgb_crop_shift_c64(p, 1, 3, big, big, zero, zero, 0, None, None, 0, 1.0, None, 0.0, p, None)
    assert st == _ext.TLGB_ERR_UNSUPPORTED


def test_batch_ranges():
    from torchlinops_gb300 import interp as I

    M = I.MAX_BATCH
    assert I._batch_chunks(0) == [(0, 0)]
    assert I._batch_chunks(5) == [(0, 5)]
    assert I._batch_chunks(M) == [(0, M)]
    assert I._batch_chunks(2 * M + 3) == [(0, M), (M, 2 * M), (2 * M, 2 * M + 3)]


@pytest.mark.parametrize("gs", [(16, 16), (12, 14), (205, 205, 205), (33,)])
def test_toeplitz_rescaling_keeps_the_reference_rounding(gs):
    """The Toeplitz kernel's point rescaling (host-side torch ops): from the
    padded grid Np to int(2 Np) cells, (loc - Np//2) * 2Np / Np + 2Np//2 per
    coordinate in float32 (linops/nufft.py:538-568), and the 2x sizes
    (scale_int, nufft.py:497-498)."""
    from torchlinops_gb300 import linops

    ps = tuple(int(1.25 * s) for s in gs)
    g = torch.Generator().manual_seed(sum(gs))
    locs = torch.rand(20000, len(gs), generator=g) * torch.tensor(ps, dtype=torch.float32)
    nw = linops.scale_int(ps, 2.0)
    assert nw == tuple(int(2.0 * p) for p in ps)
    ref = torch.stack([(locs[:, d] - ps[d] // 2) * nw[d] / ps[d] + nw[d] // 2 for d in range(len(gs))], dim=-1)
    got = linops.rescale_locs(locs, tuple(p // 2 for p in ps), ps, tuple(w // 2 for w in nw), nw)
    assert got.dtype == torch.float32 and torch.equal(got, ref)


def test_toeplitz_inner_operators():
    """NUFFT.normal(inner) embeds for no inner or a diagonal weighting of the
    points (a weight that broadcasts to the points' shape); other inner
    operators take the explicit chain."""
    from torchlinops_gb300 import linops

    pts = (40, 3)
    assert linops._point_weight(None, pts) is None
    w = torch.rand(40, 3)
    assert linops._point_weight(linops.Diagonal(w), pts) is not False
    assert linops._point_weight(linops.Diagonal(torch.rand(3)), pts) is not False
    assert linops._point_weight(linops.Scalar(2.0), pts) is not False
    assert linops._point_weight(linops.Diagonal(torch.rand(8, 40, 3)), pts) is False  # per-coil weights
    assert linops._point_weight(linops.Diagonal(torch.rand(7)), pts) is False
    assert linops._point_weight(linops.Pad((8, 8), (4, 4)), pts) is False


def test_cached_entries_go_with_their_locations():
    """Plan and prepared-location caches drop an entry when its locations
    tensor is freed (plans hold device memory), keep a newer entry under the
    same key, and evict the oldest beyond their size."""
    import gc
    from collections import OrderedDict

    from torchlinops_gb300 import interp as I

    cache = OrderedDict()
    a, b = torch.zeros(3), torch.zeros(4)
    I.remember(cache, ("a",), a, "plan a", 2)
    I.remember(cache, ("b",), b, "plan b", 2)
    assert list(cache) == [("a",), ("b",)]
    del a
    gc.collect()
    assert list(cache) == [("b",)]
    c = torch.zeros(5)
    I.remember(cache, ("b",), c, "plan c", 2)
    del b
    gc.collect()
    assert cache[("b",)][2] == "plan c"
    d, e = torch.zeros(1), torch.zeros(1)
    I.remember(cache, ("d",), d, "plan d", 2)
    I.remember(cache, ("e",), e, "plan e", 2)
    assert list(cache) == [("d",), ("e",)]
    assert cache[("e",)][0]() is e and cache[("e",)][1] == e._version


def test_cached_plans_order_other_streams_after_their_build(monkeypatch):
    """A cached plan used from another stream makes that stream wait for the
    build's event and records the stream on the plan's buffer; the build
    stream itself and captured streams add nothing."""
    from torchlinops_gb300 import interp as I

    calls = []

    class Stream:
        def __init__(self, handle):
            self.cuda_stream = handle

        def wait_event(self, event):
            calls.append(("wait", self.cuda_stream, event))

    class Buffer:
        def record_stream(self, stream):
            calls.append(("keep", stream.cuda_stream))

    plan = I.InterpolatePlan.__new__(I.InterpolatePlan)
    plan.device, plan.stream, plan.ready, plan.buffer = "cuda:0", Stream(1), "built", Buffer()
    cur, capturing = [Stream(1)], [False]
    monkeypatch.setattr(torch.cuda, "current_stream", lambda device=None: cur[0])
    monkeypatch.setattr(torch.cuda, "is_current_stream_capturing", lambda: capturing[0])
    plan.use_on_current_stream()
    assert calls == []
    cur[0] = Stream(2)
    plan.use_on_current_stream()
    assert calls == [("wait", 2, "built"), ("keep", 2)]
    capturing[0] = True
    plan.use_on_current_stream()
    assert len(calls) == 2
    # the torch calls the method makes
    assert all(hasattr(torch.cuda.Stream, m) for m in ("wait_event", "cuda_stream"))
    assert hasattr(torch.Tensor, "record_stream") and hasattr(torch.cuda.Event, "record")


@pytest.mark.parametrize("ndim,nbatch,entries,ncg,values_copy", [
    (3, 8, 8, 1, True), (3, 11, 8, 2, True), (3, 1, 1, 1, False), (3, 2, 2, 1, False), (3, 3, 4, 1, False),
    (3, 4, 4, 1, False), (3, 5, 8, 1, True), (2, 1, 8, 1, True), (2, 8, 8, 1, True)])
def test_adjoint_scratch_layout_of_the_block_path(ndim, nbatch, entries, ncg, values_copy):
    """Gridding scratch on the block-list path (host arithmetic only): the
    split blocks' parts (64 cells x E complex entries each, E = 1, 2 or 4 for
    3D batches of at most 4 entries, else 8 per group), one work counter per
    group of 8 entries, and the point-major value copy (64 bytes per point and
    group) only for the 8-entry kernels."""
    def up(x):
        return (x + 255) // 256 * 256

    npts, parts = 1000, 10
    d = _desc(ndim=ndim, nbatch=nbatch, npts=npts)
    d.is_complex = 1
    info = _ext.PlanInfo()
    info.n_blk_items, info.n_blk_partials, info.off_records = 50, parts, 4096
    sb = ctypes.c_size_t(0)
    assert _ext.lib().tlgb_interp_adjoint_scratch_size(ctypes.byref(d), ctypes.byref(info), ctypes.byref(sb)) == 0
    want = up(parts * ncg * 64 * 2 * entries * 4) + up(ncg * 4) + (ncg * npts * 64 if values_copy else 0)
    assert sb.value == want


def test_cg_info_record_is_valid_json():
    """The per-solve record: plain numbers and flags, non-finite residuals as
    null, the history only on request."""
    import json

    from torchlinops_gb300.alg import CGInfo

    info = CGInfo(iters=5, converged=True, rel_residual=1e-5, true_rel_residual=float("nan"), seconds=0.25,
                  restarts=1, history=[1.0, 0.1, float("inf")])
    rec = info.record(history=True)
    assert json.loads(json.dumps(rec, allow_nan=False)) == rec
    assert rec["true_rel_residual"] is None and rec["history"] == [1.0, 0.1, None]
    assert rec["iters"] == 5 and rec["restarts"] == 1 and "history" not in info.record()
