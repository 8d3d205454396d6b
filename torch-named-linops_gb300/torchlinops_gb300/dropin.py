"""Re-point an imported torchlinops at this package's CUDA kernels.

torchlinops reaches its hot path through functions that several of its
modules bind by name at import time:

* ``functional/__init__.py:1-10`` re-exports them (``from ._interp.interp import *``, ...);
* ``functional/_nufft.py:11`` imports ``interpolate`` and ``interpolate_adjoint``
  (the functional ``nufft`` / ``nufft_adjoint`` call them at ``:54,101``);
* ``functional/_interp/interp.py:7-8`` imports ``grid`` and ``ungrid`` (its
  autograd functions call them);
* ``functional/_unfold/array_to_blocks.py:10-11`` imports ``fold`` and ``unfold``;
* ``linops/convolution.py:9`` imports ``circular_pad`` (its circular mode,
  ``:120-130,148-150``).

The linops (``linops/interp.py:97-104``, ``linops/array_to_blocks.py:68-90,163-180``,
``linops/sampling.py:95-101``) call ``torchlinops.functional.<name>`` at run
time. Rebinding only the names of ``torchlinops.functional`` would leave the
by-name copies above on the reference's own path, so ``patch`` walks every
loaded module of the package and replaces each attribute that *is* one of the
reference's hot-path functions with this package's function of the same name.
After it, ``NUFFT``, ``Interpolate``, ``.H``, ``.N``, ``Chain``, ``toeplitz_psf``,
``ArrayToBlocks``, ``Sampling``, ``Convolution`` (circular padding) and
``conjugate_gradients`` run on these
kernels unchanged. ``unpatch`` restores every rebound attribute.

One behaviour differs by design: CPU tensors raise instead of running a torch
fallback (there is none in this package).
"""

from __future__ import annotations

import importlib
import sys
from types import ModuleType

from . import blocks as _blocks
from . import circpad as _circpad
from . import interp as _interp
from .index import index as _index_fwd
from .index import index_adjoint as _index_adj

__all__ = ["HOT_PATH", "patch", "unpatch", "patched_sites"]

# (defining module under the package, function name) -> replacement
HOT_PATH = {
    ("functional._interp.interp", "interpolate"): _interp.interpolate,
    ("functional._interp.interp", "interpolate_adjoint"): _interp.interpolate_adjoint,
    ("functional._interp.ungrid", "ungrid"): _interp.ungrid,
    ("functional._interp.grid", "grid"): _interp.grid,
    ("functional._unfold.array_to_blocks", "array_to_blocks"): _blocks.array_to_blocks,
    ("functional._unfold.array_to_blocks", "blocks_to_array"): _blocks.blocks_to_array,
    ("functional._unfold.array_to_blocks", "get_norm_weights"): _blocks.get_norm_weights,
    ("functional._unfold.unfold", "unfold"): _blocks.unfold,
    ("functional._unfold.fold", "fold"): _blocks.fold,
    ("functional._index.index", "index"): _index_fwd,
    ("functional._index.index", "index_adjoint"): _index_adj,
    ("functional._interp._circ_pad", "circular_pad"): _circpad.circular_pad,
    ("functional._interp._circ_pad", "circular_pad_adjoint"): _circpad.circular_pad_adjoint,
}

# package name -> list of (module, attribute, original object)
_PATCHED: dict[str, list[tuple[ModuleType, str, object]]] = {}


def _package_modules(pkg: str):
    for name, mod in list(sys.modules.items()):
        if mod is not None and (name == pkg or name.startswith(pkg + ".")):
            yield mod


def patch(package: str = "torchlinops") -> list[tuple[str, str]]:
    """Rebind the hot-path functions of an imported ``package`` (torchlinops)
    in every one of its loaded modules. Returns the (module, attribute) sites
    that now point at this package. Calling it again is harmless."""
    importlib.import_module(package)
    originals = {}
    for (modname, name), new in HOT_PATH.items():
        orig = getattr(importlib.import_module(f"{package}.{modname}"), name)
        if orig is not new:
            originals[id(orig)] = (orig, new)
    done = _PATCHED.setdefault(package, [])
    for mod in _package_modules(package):
        for attr, val in list(vars(mod).items()):
            hit = originals.get(id(val))
            if hit is not None and hit[0] is val:
                setattr(mod, attr, hit[1])
                done.append((mod, attr, val))
    return patched_sites(package)


def patched_sites(package: str = "torchlinops") -> list[tuple[str, str]]:
    """(module, attribute) pairs currently pointing at this package's functions."""
    news = {id(f) for f in HOT_PATH.values()}
    return sorted(
        (mod.__name__, attr)
        for mod in _package_modules(package)
        for attr, val in vars(mod).items()
        if id(val) in news
    )


def unpatch(package: str = "torchlinops") -> None:
    """Undo ``patch``: every rebound attribute gets the reference's function back."""
    for mod, attr, orig in reversed(_PATCHED.pop(package, [])):
        setattr(mod, attr, orig)
