"""Cartesian points onto the grid: ``cart2grid`` (kwave/utils/conversion.py:164-325).

Used to turn a Cartesian sensor (e.g. a circle of points) into the binary mask
that ``TimeReversal`` needs.  Host-side index arithmetic on the point list, as
in the reference; the same return values ``(grid_data, order_index,
reorder_index)``, the same index conventions (including the reference's
0-based point index in 2-D and 1-based in 1-D / 3-D) and the same errors.
When several points fall on one grid point the last one wins, as in the
reference's sequential loop.
"""
from __future__ import annotations

import logging
import warnings

import numpy as np

_DEFAULT = object()


def _last_wins(flat_index, values, size, fill):
    """Array of ``size`` with values[j] at flat_index[j], later j overwriting earlier."""
    out = np.full(size, fill, dtype=np.int64)
    rev = flat_index[::-1]
    _, first = np.unique(rev, return_index=True)        # first in reversed order = last in original
    keep = len(flat_index) - 1 - first
    out[flat_index[keep]] = values[keep]
    return out


def _grid_geometry(kgrid):
    """(shape, spacing) of a kWaveGrid-like object (N/spacing or Nx/dx...)."""
    n, d = getattr(kgrid, "N", None), getattr(kgrid, "spacing", None)
    if n is not None and d is not None:
        return tuple(int(v) for v in np.atleast_1d(n)), tuple(float(v) for v in np.atleast_1d(d))
    shape, spacing = [], []
    for ax in "xyz":
        n, d = getattr(kgrid, f"N{ax}", None), getattr(kgrid, f"d{ax}", None)
        if n is None or d is None:
            break
        shape.append(int(n))
        spacing.append(float(d))
    return tuple(shape), tuple(spacing)


def cart2grid(kgrid, cart_data, axisymmetric=False, *, order=_DEFAULT):
    """Nearest-grid-point mapping of Cartesian points (metres, grid centred at
    the origin) onto a binary mask of the grid's shape.

    Returns ``(grid_data, order_index, reorder_index)``: the int mask, for each
    grid point of the mask (in ``order``, "C" or "F") the 1-based index of its
    Cartesian point, and the inverse permutation.  ``order`` defaults to "F"
    with a FutureWarning, as in the reference.
    """
    if order is _DEFAULT:
        warnings.warn("cart2grid default order='F' will change to order='C' in a future release. "
                      "Pass order='C' explicitly.", FutureWarning, stacklevel=2)
        order = "F"
    shape, spacing = _grid_geometry(kgrid)
    dim = len(shape)
    if axisymmetric and dim != 2:
        raise AssertionError("Axisymmetric flag only supported in 2D.")
    cart = np.asarray(cart_data, dtype=float)
    if cart.ndim != 2 or cart.shape[0] != dim:
        raise ValueError("Input cart_data must be a 1, 2, or 3 dimensional matrix.")
    idx = [np.round(cart[a] / spacing[a]).astype(int) for a in range(dim)]
    for a in range(dim):
        if not (axisymmetric and a == 1):
            idx[a] = idx[a] + shape[a] // 2
    npts = cart.shape[1]
    if dim == 1:
        if idx[0].max() > shape[0] or idx[0].min() < 1:
            raise AssertionError("Cartesian points must lie within the grid defined by kgrid.")
        grid = _last_wins(idx[0], np.arange(1, npts + 1), shape[0], 0).reshape(shape[0], 1).astype(float)
        reorder = grid[grid != 0].reshape(-1, 1)
    else:
        if any(idx[a].min() < 0 or idx[a].max() >= shape[a] for a in range(dim)):
            raise AssertionError("Cartesian points must lie within the grid defined by kgrid.")
        flat = np.ravel_multi_index(tuple(idx), shape)
        # the reference stores the 0-based point index in 2-D and the 1-based one in 3-D
        vals = np.arange(npts) if dim == 2 else np.arange(1, npts + 1)
        grid = _last_wins(flat, vals, int(np.prod(shape)), -1).reshape(shape)
        if dim == 2:
            grid = grid.astype(float)  # the reference's 2-D grid (and reorder index) is float
        f = grid.ravel(order=order)
        reorder = f[f != -1]
        reorder = reorder[:, None] + 1 if dim == 2 else reorder[:, None, None]
    order_index = np.ones((reorder.size, 2), dtype=int)
    order_index[:, 0] = np.squeeze(reorder)
    order_index[:, 1] = np.arange(1, reorder.size + 1)
    order_index = order_index[order_index[:, 0].argsort()][:, 1][:, None]
    if dim == 1:
        grid[grid != 0] = 1
    else:
        grid[grid != -1] = 1
        grid[grid == -1] = 0
    discarded = npts - np.sum(grid)
    if discarded != 0:
        logging.log(logging.INFO, f"  cart2grid: {discarded} Cartesian points mapped to overlapping grid points")
    return grid.astype(int), order_index, reorder
