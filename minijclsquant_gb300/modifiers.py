"""Operator modifiers on the KPM path (host, FP64), drop-in for the four
jclsquant/modifiers.py functions that feed the recursions.

Each returns a new ``data`` array; ``ell_matrix.modifier`` wraps it into a new
matrix.  The arithmetic is the reference's: a complex scalar times each
entry, so the rescaled values are bit-identical to jclsquant's.
"""
from __future__ import annotations

import numpy as np


def _diagonal_add(A, diagonal_array):
    """data with diagonal_array[row] added to every valid (row, row) slot
    (jclsquant/cython_modules/Extra_funs.pyx:352-362, diagonal_modifier)."""
    data_new = np.array(A.data, dtype=np.complex128, copy=True)
    n = int(A.shape[0])
    L = int(A.len_row)
    rows = np.repeat(np.arange(n), L)
    mask = (np.asarray(A.indices) == rows) & (np.asarray(A.valid_row_values) == 1)
    data_new[mask] = np.asarray(diagonal_array, dtype=np.complex128)[rows[mask]] + data_new[mask]
    return data_new


def modifier_bounds(A):
    """H~ = (H - c) / a with a = (b1 - b0)/2, c = (b1 + b0)/2 (jclsquant/modifiers.py:14-36).

    Symmetric bounds: every entry times (1/a + 0j).  Otherwise the diagonal is
    shifted by -c first, then scaled.
    """
    b0, b1 = float(A.bounds[0]), float(A.bounds[1])
    if np.abs(b1) == np.abs(b0):
        s = 1 / ((b1 - b0) / 2) + 0j
        return np.asarray(A.data, dtype=np.complex128) * s
    diag = (-0.5 * (b1 + b0)) * np.ones(int(A.shape[0]), dtype=np.complex128)
    data_new = _diagonal_add(A, diag)
    return data_new * (1 / (0.5 * (b1 - b0)) + 0j)


def modifier_bounds_inverse(A):
    """Undo the symmetric rescaling (jclsquant/modifiers.py:39-51)."""
    return np.asarray(A.data, dtype=np.complex128) * (((A.bounds[1] - A.bounds[0]) / 2) + 0j)


def _direction_vec(A, direction):
    if direction == 0 or direction == "x":
        return A.dx_vec
    if direction == 1 or direction == "y":
        return A.dy_vec
    if direction == 2 or direction == "z":
        return A.dz_vec
    return None


def modifier_velocity(A, direction=None):
    """V = -i H o d  (d = dx_vec or dy_vec; jclsquant/modifiers.py:56-79)."""
    d = _direction_vec(A, direction)
    if d is None:
        print(" You must introduce a valid direction: 0,1,2 or x,y,z ")
        return None
    return (-1j) * np.asarray(d, dtype=np.complex128) * np.asarray(A.data, dtype=np.complex128)


def modifier_velocity_bounds(A, direction=None):
    """H o d / a  (jclsquant/modifiers.py:82-105)."""
    d = _direction_vec(A, direction)
    if d is None:
        print(" You must introduce a valid direction: 0,1,2 or x,y,z ")
        return None
    s = 1 / ((A.bounds[1] - A.bounds[0]) / 2) + 0j
    return s * np.asarray(d, dtype=np.complex128) * np.asarray(A.data, dtype=np.complex128)


def modifier_diagonal_anderson(A, W=None, seed=None):
    """Add Anderson disorder W*(2U - 1) on the diagonal, U from default_rng(seed)
    (jclsquant/modifiers.py:287-309)."""
    if W is None:
        print("You must introduce a disorder strength to modify the system. ")
        return None
    rng = np.random.default_rng(seed)
    diag = W * (2 * rng.random(int(A.shape[0])) - 1)
    return _diagonal_add(A, diag)
