"""Operator modifiers on the KPM path (host, FP64), drop-in for the four
jclsquant/modifiers.py functions that feed the recursions.

Each returns a new ``data`` array; ``ell_matrix.modifier`` wraps it into a new
matrix.  The arithmetic is the reference's: a complex scalar times each
entry, so the rescaled values are bit-identical to jclsquant's.
"""
from __future__ import annotations

import numpy as np

from . import errors


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
        return errors.missing(" You must introduce a valid direction: 0,1,2 or x,y,z ")
    return (-1j) * np.asarray(d, dtype=np.complex128) * np.asarray(A.data, dtype=np.complex128)


def modifier_velocity_bounds(A, direction=None):
    """H o d / a  (jclsquant/modifiers.py:82-105)."""
    d = _direction_vec(A, direction)
    if d is None:
        return errors.missing(" You must introduce a valid direction: 0,1,2 or x,y,z ")
    s = 1 / ((A.bounds[1] - A.bounds[0]) / 2) + 0j
    return s * np.asarray(d, dtype=np.complex128) * np.asarray(A.data, dtype=np.complex128)


def modifier_diagonal_anderson(A, W=None, seed=None):
    """Add Anderson disorder W*(2U - 1) on the diagonal, U from default_rng(seed)
    (jclsquant/modifiers.py:287-309)."""
    if W is None:
        return errors.missing("You must introduce a disorder strength to modify the system. ")
    rng = np.random.default_rng(seed)
    diag = W * (2 * rng.random(int(A.shape[0])) - 1)
    return _diagonal_add(A, diag)


# ---- time-dependent operators of driven systems (computed on the GPU) -------------
def _light_params(modifier_id, modifier_params, t):
    """(a, A0, t, w, Tp, eta) of the light forms (jclsquant/modifiers.py:133-182, 369-413),
    or None after the reference's message."""
    if modifier_id is None or modifier_params is None:
        return errors.missing(' You must introduce a valid id : light, circle,light_packed or circle packed with irs valid parameters .')
    pol_eta = {"r": 1.0, "l": -1.0}
    if modifier_id == "linear":
        A0, w = modifier_params
        return (1.0, A0, t, w, 0.0, 0.0)
    if modifier_id == "circle":
        A0, w, pol = modifier_params
        if pol not in pol_eta:
            return errors.missing('You must introduce a valid polarization')
        return (1.0, A0, t, w, 0.0, pol_eta[pol])
    if modifier_id == "linear_packed":
        A0, w, Tp = modifier_params
        return (1.0, A0, t, w, Tp, 0.0)
    if modifier_id == "circle_packed":
        A0, w, pol, Tp = modifier_params
        if pol not in pol_eta:
            return errors.missing('You must introduce a valid polarization')
        return (1.0, A0, t, w, Tp, pol_eta[pol])
    return errors.missing(' You must introduce a valid id : light, circle,light_packed or circle packed with irs valid parameters .')


def _complex_params(values):
    return np.ascontiguousarray(np.array([complex(x) for x in values], dtype=np.complex128).view(np.float64))


def _dev(x):
    import torch

    if isinstance(x, torch.Tensor):
        return x.to(device="cuda", dtype=torch.complex128).contiguous()
    return torch.from_numpy(np.ascontiguousarray(np.asarray(x, dtype=np.complex128))).cuda()


def light_modifier_device(data, dx, dy, modifier_id, modifier_params, t):
    """H(t) = H o exp(i A0 (...)) on the GPU (kpm_light_modifier) for device or host arrays;
    returns a CUDA tensor (None after the reference's message for invalid ids)."""
    import torch

    from . import _capi, device

    prm = _light_params(modifier_id, modifier_params, t)
    if prm is None:
        return None
    d, x, y = _dev(data), _dev(dx), _dev(dy)
    out = torch.empty_like(d)
    p = _complex_params(prm)
    st = _capi.lib().kpm_light_modifier(d.numel(), p.ctypes.data, d.data_ptr(), x.data_ptr(), y.data_ptr(),
                                        out.data_ptr(), device._stream_ptr())
    _capi.check(st, "kpm_light_modifier")
    return out


def modifier_light(A, data_new, modifier_id=None, modifier_params=None, t=None):
    """Peierls substitution of a light pulse into data_new (jclsquant/modifiers.py:133-182),
    computed on the GPU; data_new is filled in place and returned."""
    out = light_modifier_device(A.data, A.dx_vec, A.dy_vec, modifier_id, modifier_params, t)
    if out is None:
        return None
    data_new[...] = out.cpu().numpy().reshape(np.shape(data_new))
    return data_new


def _phonon_polarisation(pol, n, a0):
    """e_pol [n, 2] and q of modifier_hoppings_c_r's phonon polarisations (jclsquant/modifiers.py:414-432)."""
    e_pol = np.zeros((n, 2), dtype=complex, order="C")
    if pol == "chiral_+":
        q = np.array([4 * np.pi / (3 * np.sqrt(3) * a0), 0], dtype=complex)
        e_pol[:, 0] = np.array([1 / np.sqrt(2), 1 / np.sqrt(2)] * (n // 2))
        e_pol[:, 1] = np.array([1j / np.sqrt(2), -1j / np.sqrt(2)] * (n // 2))
    elif pol == "chiral_-":
        q = np.array([-4 * np.pi / (3 * np.sqrt(3) * a0), 0], dtype=complex)
        e_pol[:, 0] = np.array([1 / np.sqrt(2), 1 / np.sqrt(2)] * (n // 2))
        e_pol[:, 1] = np.array([-1j / np.sqrt(2), 1j / np.sqrt(2)] * (n // 2))
    elif pol == "optical":
        q = np.array([0, 0], dtype=complex)
        e_pol[:, 0] = np.array([0, 0] * (n // 2))
        e_pol[:, 1] = np.array([1, -1] * (n // 2))
    else:
        return None, None
    return e_pol, q


def phonon_modifier_device(data, indices, dx, dy, len_row, a0, b, Aq, wq, t, q, e_pol_x, e_pol_y, Sx, Sy,
                           data_new=None, dx_new=None, dy_new=None):
    """hopping_pos_phonons_modifier on the GPU (kpm_phonon_modifier).  The outputs start as
    data_new / dx_new / dy_new (default: copies of the inputs); slots on the diagonal keep
    those values.  Returns three CUDA tensors."""
    import torch

    from . import _capi, device

    d, x, y = _dev(data), _dev(dx), _dev(dy)
    idx = torch.as_tensor(np.ascontiguousarray(np.asarray(indices, dtype=np.int32))).cuda() if not isinstance(
        indices, torch.Tensor) else indices.to(device="cuda", dtype=torch.int32).contiguous()
    dn = _dev(data_new) if data_new is not None else d.clone()
    xn = _dev(dx_new) if dx_new is not None else x.clone()
    yn = _dev(dy_new) if dy_new is not None else y.clone()
    ex, ey, sx, sy = _dev(e_pol_x), _dev(e_pol_y), _dev(Sx), _dev(Sy)
    n = d.numel() // int(len_row)
    p = _complex_params([a0, b, Aq, wq, t, q[0], q[1]])
    st = _capi.lib().kpm_phonon_modifier(n, int(len_row), p.ctypes.data, d.data_ptr(), idx.data_ptr(), x.data_ptr(),
                                         y.data_ptr(), ex.data_ptr(), ey.data_ptr(), sx.data_ptr(), sy.data_ptr(),
                                         dn.data_ptr(), xn.data_ptr(), yn.data_ptr(), device._stream_ptr())
    _capi.check(st, "kpm_phonon_modifier")
    return dn, xn, yn


def modifier_hoppings_c(A, data_new, dx_vec_new, dy_vec_new, modifier_id=None, modifier_params=None, t=None):
    """jclsquant/modifiers.py:362-366: real-space operators go to modifier_hoppings_c_r; the
    k-space form is outside this library (k-space loops are not on its path)."""
    if getattr(A, "space", "r") == "r":
        return modifier_hoppings_c_r(A, data_new, dx_vec_new, dy_vec_new, modifier_id, modifier_params, t)
    raise NotImplementedError("k-space operators are not supported")


def modifier_hoppings_c_r(A, data_new, dx_vec_new, dy_vec_new, modifier_id=None, modifier_params=None, t=None):
    """Peierls light forms and the packed phonon modifier on the GPU, filling the caller's
    arrays as the reference's Cython route does (jclsquant/modifiers.py:369-445)."""
    if modifier_id == "phonons_packed":
        a0, b, Aq, wq, pol, S = modifier_params
        e_pol, q = _phonon_polarisation(pol, int(A.shape[0]), a0)
        if e_pol is None:
            return errors.missing('You must introduce a valid polarization')
        S = np.asarray(S)
        dn, xn, yn = phonon_modifier_device(A.data, A.indices, A.dx_vec, A.dy_vec, A.len_row, a0, b, Aq, wq, t, q,
                                            e_pol[:, 0], e_pol[:, 1], S[:, 0], S[:, 1], data_new, dx_vec_new,
                                            dy_vec_new)
        data_new[...] = dn.cpu().numpy()
        dx_vec_new[...] = xn.cpu().numpy()
        dy_vec_new[...] = yn.cpu().numpy()
        return data_new, dx_vec_new, dy_vec_new
    out = light_modifier_device(A.data, A.dx_vec, A.dy_vec, modifier_id, modifier_params, t)
    if out is None:
        return None
    data_new[...] = out.cpu().numpy()
    return data_new
