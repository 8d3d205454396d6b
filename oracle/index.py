"""CPU restatement of the reference sampling path (TEST INFRASTRUCTURE ONLY).

* ``ravel``          <- ``functional/_index/index.py:187-201``: per indexed
  dimension ``out += idx % size; out *= next size`` with Python's
  non-negative modulo.
* ``index``          <- ``index`` (index.py:17-49) with ``multi_index``
  (:52-72): ``index_select`` of the raveled cells over the flattened grid.
* ``index_adjoint``  <- ``index_adjoint`` + ``multi_grid`` (index.py:75-100,
  141-184): bounds check (``IndexError`` for an index >= size or < -size),
  then ``index_add_`` of the samples into a zero grid. On the CPU that sum runs
  in ascending sample order per cell, which the GPU adjoint reproduces bit for
  bit.
"""

from __future__ import annotations

from math import prod

import torch

__all__ = ["ravel", "index", "index_adjoint"]


def ravel(idx: tuple[torch.Tensor, ...], grid_size) -> torch.Tensor:
    out = torch.zeros_like(idx[0], dtype=torch.int64)
    nxt = tuple(grid_size[1:]) + (1,)
    for i, s, sn in zip(idx, grid_size, nxt):
        out = (out + torch.remainder(i.to(torch.int64), s)) * sn
    return out


def index(vals: torch.Tensor, idx: tuple[torch.Tensor, ...]) -> torch.Tensor:
    nd = len(idx)
    grid_size = tuple(vals.shape[-nd:])
    idx = torch.broadcast_tensors(*idx)
    cells = ravel(idx, grid_size)
    flat = vals.reshape(*vals.shape[: vals.ndim - nd], prod(grid_size))
    out = torch.index_select(flat, -1, cells.reshape(-1))
    return out.reshape(*vals.shape[: vals.ndim - nd], *cells.shape)


def index_adjoint(vals: torch.Tensor, idx: tuple[torch.Tensor, ...], grid_size) -> torch.Tensor:
    grid_size = tuple(int(s) for s in grid_size)
    for d, (i, s) in enumerate(zip(idx, grid_size)):
        if (i >= s).any() or (i < -s).any():
            raise IndexError(f"Out-of-bounds index for grid of shape {grid_size}: idx[{d}]")
    cells = ravel(tuple(idx), grid_size)
    ns = cells.ndim
    batch = vals.shape[: vals.ndim - ns]
    x = vals.reshape(*batch, -1)
    y = torch.zeros(*batch, prod(grid_size), dtype=vals.dtype)
    y.index_add_(-1, cells.reshape(-1), x)
    return y.reshape(*batch, *grid_size)
