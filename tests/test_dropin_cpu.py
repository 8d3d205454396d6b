"""The drop-in patch (torchlinops_gb300.dropin) on the CPU.

* On a stand-in package that binds the hot-path functions by name the way
  torchlinops does (re-exports in its functional package, by-name imports in
  the NUFFT and autograd modules, run-time ``F.<name>`` lookups in its linops),
  every binding is rebound and ``unpatch`` restores them.
* With the reference itself importable (``TORCHLINOPS_SRC`` pointing at its
  ``src/`` directory; skipped otherwise): after the patch every by-name site
  of the real package points here, and the reference's own ``NUFFT``,
  ``Interpolate``, ``ArrayToBlocks``, ``Sampling`` and functional ``nufft``
  reach this package's functions -- which, given CPU tensors, raise this
  package's "CUDA tensors only" error instead of running the reference's torch
  path.
"""

import os
import sys
import textwrap

import pytest
import torch

from conftest import ROOT
from torchlinops_gb300 import dropin

FAKE = {
    "__init__.py": "from . import functional, linops\n",
    "functional/__init__.py": textwrap.dedent("""
        from ._interp.interp import *
        from ._interp.grid import *
        from ._interp.ungrid import *
        from ._index.index import *
        from ._nufft import *
        from ._unfold.array_to_blocks import *
        from ._unfold.fold import *
        from ._unfold.unfold import *
    """),
    "functional/_interp/__init__.py": "",
    "functional/_interp/grid.py": "__all__ = ['grid']\ndef grid(*a, **k): return 'ref-grid'\n",
    "functional/_interp/ungrid.py": "__all__ = ['ungrid']\ndef ungrid(*a, **k): return 'ref-ungrid'\n",
    "functional/_interp/interp.py": textwrap.dedent("""
        from .grid import grid
        from .ungrid import ungrid
        __all__ = ['interpolate', 'interpolate_adjoint']
        def interpolate(*a, **k): return ungrid(*a, **k)
        def interpolate_adjoint(*a, **k): return grid(*a, **k)
    """),
    "functional/_interp/_circ_pad.py": textwrap.dedent("""
        def circular_pad(t, padding): return 'ref-pad'
        def circular_pad_adjoint(t, padding): return 'ref-pad-adjoint'
    """),
    "functional/_index/__init__.py": "",
    "functional/_index/index.py": textwrap.dedent("""
        __all__ = ['index', 'index_adjoint']
        def index(*a, **k): return 'ref-index'
        def index_adjoint(*a, **k): return 'ref-index-adjoint'
    """),
    "functional/_nufft.py": textwrap.dedent("""
        from ._interp.interp import interpolate, interpolate_adjoint
        __all__ = ['nufft']
        def nufft(x, locs): return interpolate(x, locs, 4.0)
    """),
    "functional/_unfold/__init__.py": "",
    "functional/_unfold/unfold.py": "__all__ = ['unfold']\ndef unfold(*a, **k): return 'ref-unfold'\n",
    "functional/_unfold/fold.py": "__all__ = ['fold']\ndef fold(*a, **k): return 'ref-fold'\n",
    "functional/_unfold/array_to_blocks.py": textwrap.dedent("""
        from .fold import fold
        from .unfold import unfold
        __all__ = ['array_to_blocks', 'blocks_to_array', 'get_norm_weights']
        def array_to_blocks(*a, **k): return unfold(*a, **k)
        def blocks_to_array(*a, **k): return fold(*a, **k)
        def get_norm_weights(*a, **k): return 'ref-weights'
    """),
    "linops/__init__.py": textwrap.dedent("""
        import fakelinops.functional as F
        from ..functional._interp._circ_pad import circular_pad
        def interp_fn(x, locs): return F.interpolate(x, locs, 4.0)
    """),
}


@pytest.fixture
def fake_pkg(tmp_path):
    root = tmp_path / "fakelinops"
    for rel, src in FAKE.items():
        p = root / rel
        p.parent.mkdir(parents=True, exist_ok=True)
        p.write_text(src)
    sys.path.insert(0, str(tmp_path))
    import fakelinops  # noqa: F401

    yield "fakelinops"
    dropin.unpatch("fakelinops")
    for name in [m for m in sys.modules if m == "fakelinops" or m.startswith("fakelinops.")]:
        del sys.modules[name]
    sys.path.remove(str(tmp_path))


def test_patch_rebinds_every_by_name_site(fake_pkg):
    import fakelinops
    import fakelinops.functional._nufft as N
    import torchlinops_gb300 as T

    before = N.interpolate
    sites = dropin.patch(fake_pkg)
    # the by-name copies that rebinding only `functional.<name>` would miss
    assert ("fakelinops.functional._nufft", "interpolate") in sites
    assert ("fakelinops.functional._nufft", "interpolate_adjoint") in sites
    assert ("fakelinops.functional._interp.interp", "grid") in sites
    assert ("fakelinops.functional._interp.interp", "ungrid") in sites
    assert ("fakelinops.functional._unfold.array_to_blocks", "fold") in sites
    assert ("fakelinops.functional", "index_adjoint") in sites
    assert ("fakelinops.linops", "circular_pad") in sites
    assert N.interpolate is T.interpolate and fakelinops.functional.unfold is T.unfold
    # run-time lookups from the linops and the functional NUFFT reach this package
    with pytest.raises(RuntimeError, match="CUDA tensors only"):
        fakelinops.linops.interp_fn(torch.ones(4, 4), torch.zeros(3, 2))
    with pytest.raises(RuntimeError, match="CUDA tensors only"):
        N.nufft(torch.ones(4, 4), torch.zeros(3, 2))
    assert dropin.patch(fake_pkg) == sites  # idempotent
    dropin.unpatch(fake_pkg)
    assert N.interpolate is before and dropin.patched_sites(fake_pkg) == []
    assert fakelinops.functional.unfold() == "ref-unfold"


REF = os.environ.get("TORCHLINOPS_SRC")


@pytest.mark.skipif(not REF, reason="set TORCHLINOPS_SRC to the reference's src/ directory")
def test_patch_reroutes_the_reference_itself():
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden", "_stubs"))
    sys.path.insert(0, REF)
    try:
        import torchlinops
        import torchlinops.functional as F
        import torchlinops.functional._nufft as N
        import torchlinops.linops as L
        import torchlinops_gb300 as T

        sites = dict.fromkeys(dropin.patch("torchlinops"))
        try:
            for s in [("torchlinops.functional._nufft", "interpolate"),
                      ("torchlinops.functional._nufft", "interpolate_adjoint"),
                      ("torchlinops.functional._interp.interp", "grid"),
                      ("torchlinops.functional._interp.interp", "ungrid"),
                      ("torchlinops.functional._unfold.array_to_blocks", "fold"),
                      ("torchlinops.functional._unfold.array_to_blocks", "unfold"),
                      ("torchlinops.functional", "interpolate"),
                      ("torchlinops.functional", "array_to_blocks"),
                      ("torchlinops.functional", "index_adjoint"),
                      ("torchlinops.linops.convolution", "circular_pad")]:
                assert s in sites, s
            assert N.interpolate is T.interpolate
            locs = torch.rand(50, 2) * 10 - 5
            x = torch.randn(16, 16, dtype=torch.complex64)
            cuda_only = pytest.raises(RuntimeError, match="CUDA tensors only")
            with cuda_only:
                L.NUFFT(locs, (16, 16), output_shape=("K",))(x)  # the reference's NUFFT linop (linops/nufft.py:184)
            with cuda_only:
                N.nufft(x, locs)  # the functional NUFFT (functional/_nufft.py:54)
            with cuda_only:
                L.Interpolate(locs + 8, (16, 16))(x)  # linops/interp.py:97-104
            with cuda_only:
                L.ArrayToBlocks((16, 16), (4, 4), (2, 2))(x)  # linops/array_to_blocks.py:68
            with cuda_only:
                L.Sampling((torch.tensor([1, 2]), torch.tensor([3, 4])), (16, 16)).H(torch.ones(2))
            with cuda_only:
                L.Convolution(torch.ones(3, 3), padding_mode="circular")(x)  # linops/convolution.py:126
        finally:
            dropin.unpatch("torchlinops")
        assert F.interpolate is not T.interpolate
    finally:
        sys.path.remove(REF)
        sys.path.remove(os.path.join(ROOT, "tests", "golden", "_stubs"))
