"""Compatibility shim with the names of jclsquant's GPU bridge
(jclsquant/cuda_cython/obv.pyx:23-75).

Each function takes host numpy arrays, calls the reference-compatible
host-pointer entry point of libkpm (upload, run, download, synchronous, as the
reference does) and writes the result into the caller's output array.
"""
from __future__ import annotations

import numpy as np

from . import _capi


def _c128(x, name):
    if not (isinstance(x, np.ndarray) and x.dtype == np.complex128 and x.flags.c_contiguous):
        raise TypeError("%s must be a C-contiguous complex128 numpy array" % name)
    return x


def _i32(x, name):
    if not (isinstance(x, np.ndarray) and x.dtype == np.int32 and x.flags.c_contiguous):
        raise TypeError("%s must be a C-contiguous int32 numpy array" % name)
    return x


def _status(what):
    _capi.check(_capi.lib().kpm_last_status(), what)


def rec_A_tab_gpu(data, indices, len_row, v, A_vec, M):
    """A_vec[m] = <v|T_m v> (obv.pyx:23-35 -> recursions.cu:17-98)."""
    _c128(data, "data"), _i32(indices, "indices"), _c128(v, "v"), _c128(A_vec, "A_vec")
    if A_vec.size < M:
        raise ValueError("A_vec is shorter than M")
    _capi.lib().rec_A_tab(data.ctypes.data, indices.ctypes.data, int(len_row), int(v.shape[0]),
                          A_vec.ctypes.data, v.ctypes.data, int(M))
    _status("rec_A_tab")


def rec_A_tab_2_gpu(data, indices, len_row, v_l, v_r, A_vec, M):
    """A_vec[m] = <v_l|T_m v_r> (obv.pyx:37-49 -> recursions.cu:180-263)."""
    _c128(data, "data"), _i32(indices, "indices"), _c128(v_l, "v_l"), _c128(v_r, "v_r"), _c128(A_vec, "A_vec")
    if A_vec.size < M:
        raise ValueError("A_vec is shorter than M")
    _capi.lib().rec_A_tab_2(data.ctypes.data, indices.ctypes.data, int(len_row), int(v_r.shape[0]),
                            A_vec.ctypes.data, v_l.ctypes.data, v_r.ctypes.data, int(M))
    _status("rec_A_tab_2")


def for_time_gpu(data, indices, len_row, moments_kernel, len_t, U, U_c, M):
    """U, U_c <- (sum_m c_m T_m)^len_t applied to each, in place (obv.pyx:52-62 -> obv.cu:93-122)."""
    _c128(data, "data"), _i32(indices, "indices"), _c128(moments_kernel, "moments_kernel")
    _c128(U, "U"), _c128(U_c, "U_c")
    if U_c.shape[0] != U.shape[0]:
        raise ValueError("U and U_c differ in length")
    if moments_kernel.size < M:
        raise ValueError("moments_kernel is shorter than M")
    _capi.lib().for_time(data.ctypes.data, indices.ctypes.data, int(len_row), int(U.shape[0]),
                         moments_kernel.ctypes.data, int(len_t), U.ctypes.data, U_c.ctypes.data, int(M))
    _status("for_time")


def for_time_sigma_gpu(data, data2, data3, indices, len_row, moments_kernel_U, moments_kernel_FD, len_t, sigma_vec,
                       v, M, M2):
    """sigma_vec[j] = <U_c(t_j)|V1 U(t_j)> (obv.pyx:66-75 -> obv.cu:124-176)."""
    for a, n in ((data, "data"), (data2, "data2"), (data3, "data3"), (moments_kernel_U, "moments_kernel_U"),
                 (moments_kernel_FD, "moments_kernel_FD"), (sigma_vec, "sigma_vec"), (v, "v")):
        _c128(a, n)
    _i32(indices, "indices")
    _capi.lib().for_time_sigma(data.ctypes.data, data2.ctypes.data, data3.ctypes.data, indices.ctypes.data,
                               int(len_row), int(v.shape[0]), moments_kernel_U.ctypes.data,
                               moments_kernel_FD.ctypes.data, int(len_t), sigma_vec.ctypes.data, v.ctypes.data,
                               int(M), int(M2))
    _status("for_time_sigma")
