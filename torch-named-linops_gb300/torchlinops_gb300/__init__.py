"""GB300-native (sm_103a) interpolation and block kernels for torchlinops.

A drop-in for the data-parallel hot path of torch-named-linops 0.7.4: the
Interpolate linop's Kaiser-Bessel / spline ungridding and gridding in 1D-3D,
the ArrayToBlocks / BlocksToArray pair, and the Sampling linop's integer
index / index_adjoint, with the reference's functional signatures. All
compute runs in the hand-written CUDA library ``libtlgb.so`` (C ABI in
``include/tlgb.h``); there is no CPU fallback.
"""

from .blocks import (
    array_to_blocks,
    blocks_to_array,
    fold,
    get_nblocks,
    get_norm_weights,
    unfold,
)
from .circpad import circular_pad, circular_pad_adjoint
from .index import index, index_adjoint
from .interp import (
    clear_plan_cache,
    get_plan,
    grid,
    interpolate,
    interpolate_adjoint,
    kaiser_bessel_beta,
    ungrid,
)

__version__ = "0.1.0"


def build(verbose: bool = False) -> str:
    """Compile libtlgb.so for sm_103a (in-tree) and return its path."""
    from ._build import build as _b

    return _b(verbose=verbose)
