"""numpy-facing wrapper of the C oracle -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py``
use this module, as the oracle (and the CPU baseline "port"); the product
library never imports it.  Each function follows the reference routine named
in its docstring (the C file gives file:line for each).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        c = ctypes.CDLL(path)
        P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        c.oracle_aAxby.argtypes = [D, D, D, D, P, P, P, P, I, I, I]
        c.oracle_aAxby.restype = None
        c.oracle_vdot.argtypes = [D, D, P, P, I, I, P]
        c.oracle_vdot.restype = None
        c.oracle_dot.argtypes = [D, D, P, P, I, I, P]
        c.oracle_dot.restype = None
        c.oracle_rec_A_tab.argtypes = [I, P, P, I, I, P, P, I]
        c.oracle_rec_A_tab2v.argtypes = [I, P, P, I, I, P, P, P, I]
        c.oracle_rec_A_tab2v_2.argtypes = [I, P, P, I, I, P, P, P, P, I]
        c.oracle_rec_A_vec.argtypes = [I, P, P, I, I, P, P, P, I]
        c.oracle_rec_com_A_vec.argtypes = [I, P, P, P, I, I, P, P, P, I]
        c.oracle_rec_com_A_vec_tab.argtypes = [I, P, P, P, I, I, P, P, P, I]
        c.oracle_for_time_sigma.argtypes = [P, P, P, P, I, I, P, P, I, P, P, I, I, I]
        c.oracle_max_threads.restype = I
        c.oracle_adjoint_grad.argtypes = [I, P, P, I, I, P, P, P]
        _lib = c
    return _lib


def default_threads() -> int:
    env = os.environ.get("OMP_NUM_THREADS")
    return int(env) if env else (os.cpu_count() or 1)


def _c(a, dtype):
    return np.ascontiguousarray(np.asarray(a, dtype=dtype))


def _check(rc, what):
    if rc != 0:
        raise RuntimeError("oracle %s failed (%d)" % (what, rc))


def aAxby(a, b, x, y, data, indices, len_row, threads=None):
    """y <- b*y + a*A x in place (blas_funs.pyx:64-71)."""
    x = _c(x, np.complex128)
    assert y.dtype == np.complex128 and y.flags.c_contiguous
    data, indices = _c(data, np.complex128), _c(indices, np.int32)
    a, b = complex(a), complex(b)
    lib().oracle_aAxby(a.real, a.imag, b.real, b.imag, x.ctypes.data, y.ctypes.data, data.ctypes.data,
                       indices.ctypes.data, int(len_row), y.size, threads or default_threads())
    return y


def vdot(x, y, threads=None):
    """sum y * conj(x) (blas_funs.pyx:83-88)."""
    x, y = _c(x, np.complex128), _c(y, np.complex128)
    out = np.zeros(2)
    lib().oracle_vdot(1.0, 0.0, x.ctypes.data, y.ctypes.data, x.size, threads or default_threads(), out.ctypes.data)
    return out[0] + 1j * out[1]


def rec_A_tab(M, data, indices, len_row, v, threads=None):
    """<v|T_m v>, m < M (recurrence_functions.py:9-40)."""
    data, indices, v = _c(data, np.complex128), _c(indices, np.int32), _c(v, np.complex128)
    mu = np.zeros(M, dtype=np.complex128)
    _check(lib().oracle_rec_A_tab(int(M), data.ctypes.data, indices.ctypes.data, int(len_row), v.size, v.ctypes.data,
                                  mu.ctypes.data, threads or default_threads()), "rec_A_tab")
    return mu


def rec_A_tab2v(M, data, indices, len_row, v_l, v_r, threads=None):
    """<v_l|T_m v_r> (recurrence_functions.py:44-74)."""
    data, indices = _c(data, np.complex128), _c(indices, np.int32)
    v_l, v_r = _c(v_l, np.complex128), _c(v_r, np.complex128)
    mu = np.zeros(M, dtype=np.complex128)
    _check(lib().oracle_rec_A_tab2v(int(M), data.ctypes.data, indices.ctypes.data, int(len_row), v_r.size,
                                    v_l.ctypes.data, v_r.ctypes.data, mu.ctypes.data, threads or default_threads()),
           "rec_A_tab2v")
    return mu


def rec_A_tab2v_2(M, data, indices, len_row, v_l, v_r, threads=None):
    """(<v_l|T_m v_r>, <v_r|T_m v_r>) (recurrence_functions.py:76-111)."""
    data, indices = _c(data, np.complex128), _c(indices, np.int32)
    v_l, v_r = _c(v_l, np.complex128), _c(v_r, np.complex128)
    m1 = np.zeros(M, dtype=np.complex128)
    m2 = np.zeros(M, dtype=np.complex128)
    _check(lib().oracle_rec_A_tab2v_2(int(M), data.ctypes.data, indices.ctypes.data, int(len_row), v_r.size,
                                      v_l.ctypes.data, v_r.ctypes.data, m1.ctypes.data, m2.ctypes.data,
                                      threads or default_threads()), "rec_A_tab2v_2")
    return m1, m2


def rec_A_vec(M, data, indices, len_row, c, v, threads=None):
    """sum_m c_m T_m v (recurrence_functions.py:114-143)."""
    data, indices = _c(data, np.complex128), _c(indices, np.int32)
    c, v = _c(c, np.complex128), _c(v, np.complex128)
    out = np.zeros_like(v)
    _check(lib().oracle_rec_A_vec(int(M), data.ctypes.data, indices.ctypes.data, int(len_row), v.size, c.ctypes.data,
                                  v.ctypes.data, out.ctypes.data, threads or default_threads()), "rec_A_vec")
    return out


def for_time(data, indices, len_row, c, len_t, U, U_c, M, threads=None):
    """(U, U_c) after len_t applications of sum_m c_m T_m to each (obv.cu:93-122: the
    loop over len_t calling the device rec_A, recursions.cu:267-317, on U and on U_c)."""
    U, U_c = _c(U, np.complex128).copy(), _c(U_c, np.complex128).copy()
    for _ in range(int(len_t)):
        U = rec_A_vec(M, data, indices, len_row, c, U, threads)
        U_c = rec_A_vec(M, data, indices, len_row, c, U_c, threads)
    return U, U_c


def rec_com_A_vec(M, data_a, data_v, indices, len_row, c, v, threads=None):
    """Commutator series (recurrence_functions.py:146-196); A and V share `indices`."""
    data_a, data_v = _c(data_a, np.complex128), _c(data_v, np.complex128)
    indices, c, v = _c(indices, np.int32), _c(c, np.complex128), _c(v, np.complex128)
    out = np.zeros_like(v)
    _check(lib().oracle_rec_com_A_vec(int(M), data_a.ctypes.data, data_v.ctypes.data, indices.ctypes.data,
                                      int(len_row), v.size, c.ctypes.data, v.ctypes.data, out.ctypes.data,
                                      threads or default_threads()), "rec_com_A_vec")
    return out


def rec_com_A_vec_tab(M, data_a, data_v, indices, len_row, c, v, threads=None):
    """Commutator table C_tab[m] = c_m C_m, [M, n] (recurrence_functions.py:202-250)."""
    data_a, data_v = _c(data_a, np.complex128), _c(data_v, np.complex128)
    indices, c, v = _c(indices, np.int32), _c(c, np.complex128), _c(v, np.complex128)
    tab = np.zeros((int(M), v.size), dtype=np.complex128)
    _check(lib().oracle_rec_com_A_vec_tab(int(M), data_a.ctypes.data, data_v.ctypes.data, indices.ctypes.data,
                                          int(len_row), v.size, c.ctypes.data, v.ctypes.data, tab.ctypes.data,
                                          threads or default_threads()), "rec_com_A_vec_tab")
    return tab


def for_time_sigma(data_h, data_v1, data_v2, indices, len_row, c_u, c_fd, len_t, v, M, M2, threads=None):
    """<U_c(t_j)|V1 U(t_j)> (obv.cu:124-176)."""
    arrs = [_c(a, np.complex128) for a in (data_h, data_v1, data_v2, c_u, c_fd, v)]
    indices = _c(indices, np.int32)
    sig = np.zeros(int(len_t), dtype=np.complex128)
    _check(lib().oracle_for_time_sigma(arrs[0].ctypes.data, arrs[1].ctypes.data, arrs[2].ctypes.data,
                                       indices.ctypes.data, int(len_row), arrs[5].size, arrs[3].ctypes.data,
                                       arrs[4].ctypes.data, int(len_t), sig.ctypes.data, arrs[5].ctypes.data, int(M),
                                       int(M2), threads or default_threads()), "for_time_sigma")
    return sig


def moment_tolerance_ok(mu, ref, rel=1e-10, floor_frac=1e-6):
    """Per-order check |mu_m - ref_m| <= rel * max(|ref_m|, floor_frac * |ref_0|)."""
    mu, ref = np.asarray(mu), np.asarray(ref)
    scale = np.maximum(np.abs(ref), floor_frac * np.abs(ref[..., :1]))
    err = np.abs(mu - ref) / scale
    return bool(np.all(err <= rel)), float(np.max(err))


def adjoint_grad(M, data, indices, len_row, v, c):
    """d/dH(slot) of sum_m c_m Re <v|T_m v> for real symmetric H (all t_m stored)."""
    data, indices, v = _c(data, np.complex128), _c(indices, np.int32), _c(v, np.complex128)
    c = _c(c, np.float64)
    grad = np.zeros(data.size, dtype=np.float64)
    _check(lib().oracle_adjoint_grad(int(M), data.ctypes.data, indices.ctypes.data, int(len_row), v.size,
                                     v.ctypes.data, c.ctypes.data, grad.ctypes.data), "adjoint_grad")
    return grad


def light_modifier(a, A0, t, w, Tp, eta, data, dx, dy):
    """The Peierls substitution of light_modifier_cython (jclsquant/cython_modules/
    Extra_funs.pyx:319-342, the forms at :236-317), in numpy complex arithmetic."""
    data, dx, dy = (np.asarray(x, dtype=np.complex128) for x in (data, dx, dy))
    a, A0, t, w, Tp, eta = (complex(x) for x in (a, A0, t, w, Tp, eta))
    if eta == 0:
        arg = 1j * A0 * (np.sin(w * t) * dy)  # linear forms (:257-299)
    else:
        arg = 1j * A0 * (np.cos(w * t) * dx + eta * np.sin(w * t) * dy)  # circular forms (:236-255, :301-317)
    if Tp != 0:
        arg = arg / np.cosh((t - 2 * Tp) / (0.5673 * Tp))
    return a * data * np.exp(arg)


def phonon_modifier(a0, b, Aq, wq, t, q, data, indices, dx, dy, e_pol_x, e_pol_y, Sx, Sy, len_row):
    """hopping_pos_phonons_modifier (jclsquant/cython_modules/Extra_funs.pyx:540-560):
    (data_new, dx_new, dy_new); slots on the diagonal keep their values."""
    data, dx, dy = (np.asarray(x, dtype=np.complex128) for x in (data, dx, dy))
    indices = np.asarray(indices)
    Tp = 2 * np.pi / wq
    ch = np.cosh((t - 2 * Tp) / (0.5673 * Tp))
    rows = np.arange(data.size) // int(len_row)
    m = rows != indices
    r, c = rows[m], indices[m]
    dn, dxn, dyn = data.copy(), dx.copy(), dy.copy()
    dxn[m] = dx[m] + Aq * (e_pol_x[r] * np.cos(wq * t - q[0] * Sx[r]) - e_pol_x[c] * np.cos(wq * t - q[0] * Sx[c])) / ch
    dyn[m] = dy[m] + Aq * (e_pol_y[r] * np.cos(wq * t - q[1] * Sy[r]) - e_pol_y[c] * np.cos(wq * t - q[1] * Sy[c])) / ch
    dn[m] = data[m] * np.exp(-b * (np.sqrt(np.abs(dxn[m]) ** 2 + np.abs(dyn[m]) ** 2 + 0j) / a0 - 1))
    return dn, dxn, dyn
