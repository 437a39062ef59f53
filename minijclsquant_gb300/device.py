"""Device-side operators and recursion calls (thin layer over the C ABI).

``DeviceELL`` owns a libkpm operator handle.  The call wrappers accept numpy
arrays (copied to the GPU per call, results copied back) or CUDA torch tensors
(zero copy, results stay on the GPU), and always launch on torch's current
CUDA stream.  PyTorch is used only for device memory and streams.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _capi


def _require_cuda() -> None:
    if not torch.cuda.is_available():
        raise RuntimeError("minijclsquant_gb300 needs a CUDA GPU; none is visible")


def _stream_ptr(stream=None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


def _as_device_c128(x, n: int | None = None) -> torch.Tensor:
    """Return a contiguous complex128 CUDA tensor view/copy of x."""
    if isinstance(x, torch.Tensor):
        t = x
        if t.dtype != torch.complex128:
            t = t.to(torch.complex128)
        if not t.is_cuda:
            t = t.cuda()
        return t.contiguous()
    a = np.ascontiguousarray(np.asarray(x, dtype=np.complex128))
    return torch.from_numpy(a).cuda()


class DeviceELL:
    """A libkpm operator: SoA ELL on the GPU (values doubled, rows padded)."""

    def __init__(self, data, indices, len_row: int, n_rows: int | None = None, *, doubling: bool = False,
                 complex_values: bool = False):
        """doubling=True: DOS moments of a Hermitian operator use the doubling
        identity (ceil(M/2) - 1 recursion steps instead of M - 2).  complex_values=True
        stores complex values even when every imaginary part is zero (an operator whose
        values light_update will make complex)."""
        _require_cuda()
        lib = _capi.lib()
        data_is_dev = isinstance(data, torch.Tensor) and data.is_cuda
        if data_is_dev:
            d = data.to(torch.complex128).contiguous()
            ix = indices.to(device=d.device, dtype=torch.int32).contiguous()
            self._keep = (d, ix)
            dptr, iptr = d.data_ptr(), ix.data_ptr()
            flags = _capi.KPM_FLAG_DEVICE_PTRS
            count = d.numel()
        else:
            d = np.ascontiguousarray(np.asarray(data, dtype=np.complex128))
            ix = np.ascontiguousarray(np.asarray(indices, dtype=np.int32))
            self._keep = None
            dptr, iptr = d.ctypes.data, ix.ctypes.data
            flags = 0
            count = d.size
        len_row = int(len_row)
        if len_row < 1 or count % len_row != 0:
            raise ValueError("ELL arrays of %d entries do not split into rows of %d" % (count, len_row))
        n = count // len_row if n_rows is None else int(n_rows)
        if n * len_row != count:
            raise ValueError("ELL arrays hold %d entries, expected %d x %d" % (count, n, len_row))
        if (not data_is_dev) and ix.size != count:
            raise ValueError("data and indices differ in length")
        if doubling:
            flags |= _capi.KPM_FLAG_DOUBLING
        if complex_values:
            flags |= _capi.KPM_FLAG_COMPLEX
        handle = ctypes.c_void_p()
        torch.cuda.synchronize()
        st = lib.kpm_ell_create(ctypes.byref(handle), n, len_row, dptr, iptr, flags, _stream_ptr())
        _capi.check(st, "kpm_ell_create")
        self._h = handle
        self.n = n
        self.len_row = len_row
        info_n = ctypes.c_int64()
        is_real = ctypes.c_int()
        lib.kpm_ell_info(self._h, ctypes.byref(info_n), None, ctypes.byref(is_real), None)
        self.is_real = bool(is_real.value)

    @property
    def hermitian(self) -> bool:
        """H == H^dagger exactly (checked on the device at creation)."""
        h = ctypes.c_int()
        _capi.check(_capi.lib().kpm_ell_props(self._h, ctypes.byref(h), None), "kpm_ell_props")
        return bool(h.value)

    @property
    def doubling(self) -> bool:
        """Whether DOS moment calls use the doubling identity."""
        d = ctypes.c_int()
        _capi.check(_capi.lib().kpm_ell_props(self._h, None, ctypes.byref(d)), "kpm_ell_props")
        return bool(d.value)

    def light_update(self, data0, dx, dy, modifier_id, modifier_params, t, stream=None):
        """Replace the values by H(t) = H0 o exp(i A0 (...)) of a light pulse, computed on
        the device from H0 = data0 and its bond vectors (kpm_ell_light_update; the forms of
        jclsquant/modifiers.py:133-182).  The operator must hold complex values."""
        from .modifiers import _complex_params, _dev, _light_params

        prm = _light_params(modifier_id, modifier_params, t)
        if prm is None:
            return None
        d, x, y = _dev(data0), _dev(dx), _dev(dy)
        if d.numel() != self.n * self.len_row:
            raise ValueError("H0 arrays must hold %d entries" % (self.n * self.len_row))
        p = _complex_params(prm)
        st = _capi.lib().kpm_ell_light_update(self._h, p.ctypes.data, d.data_ptr(), x.data_ptr(), y.data_ptr(),
                                              _stream_ptr(stream))
        _capi.check(st, "kpm_ell_light_update")
        return self

    def set_doubling(self, on: bool):
        _capi.check(_capi.lib().kpm_ell_set_doubling(self._h, int(bool(on))), "kpm_ell_set_doubling")

    @property
    def handle(self):
        return self._h

    def device_bytes(self) -> int:
        b = ctypes.c_int64()
        _capi.check(_capi.lib().kpm_ell_info(self._h, None, None, None, ctypes.byref(b)), "kpm_ell_info")
        return int(b.value)

    def reserve(self, dtype="c128", R: int = 1, M: int = 2) -> None:
        _capi.check(_capi.lib().kpm_ell_reserve(self._h, _capi.dtype_code(dtype), int(R), int(M)), "kpm_ell_reserve")

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _capi.lib().kpm_ell_destroy(h)
            except Exception:
                pass
        self._h = None

    def __del__(self):
        self.close()


def _vectors(v, n: int):
    """(tensor [R, n] complex128 on GPU, R, squeeze-flag, was-numpy)."""
    was_np = not isinstance(v, torch.Tensor)
    t = _as_device_c128(v)
    squeeze = t.dim() == 1
    if squeeze:
        t = t.reshape(1, -1)
    if t.dim() != 2 or t.shape[1] != n:
        raise ValueError("vectors must have shape [n] or [R, n] with n = %d, got %s" % (n, tuple(t.shape)))
    return t.contiguous(), t.shape[0], squeeze, was_np


def _finish(out: torch.Tensor, squeeze: bool, was_np: bool):
    if squeeze:
        out = out[0]
    if was_np:
        return out.cpu().numpy()
    return out


def cheb_moments(op: DeviceELL, M: int, v_r, v_l=None, dtype="c128", both: bool = False, stream=None):
    """mu[r, m] = <v_l[r] | T_m(H) v_r[r]>; with both=True also <v_r|T_m v_r>."""
    M = int(M)
    if M < 1:
        raise ValueError("M must be >= 1")
    tr, R, squeeze, was_np = _vectors(v_r, op.n)
    tl = None
    if v_l is not None:
        tl, Rl, _, _ = _vectors(v_l, op.n)
        if Rl != R:
            raise ValueError("left and right vector sets differ in count")
    mu = torch.empty((R, M), dtype=torch.complex128, device=tr.device)
    mu2 = torch.empty((R, M), dtype=torch.complex128, device=tr.device) if both else None
    st = _capi.lib().kpm_cheb_moments(op.handle, _capi.dtype_code(dtype), R, M, tr.data_ptr(),
                                      tl.data_ptr() if tl is not None else None, mu.data_ptr(),
                                      mu2.data_ptr() if mu2 is not None else None, _stream_ptr(stream))
    _capi.check(st, "kpm_cheb_moments")
    if both:
        return _finish(mu, squeeze, was_np), _finish(mu2, squeeze, was_np)
    return _finish(mu, squeeze, was_np)


def _coef(c, M: int, device) -> torch.Tensor:
    a = np.ascontiguousarray(np.asarray(c, dtype=np.complex128).reshape(-1)) if not isinstance(c, torch.Tensor) else c
    t = _as_device_c128(a).reshape(-1)
    if t.numel() < M:
        raise ValueError("need at least %d coefficients, got %d" % (M, t.numel()))
    return t[:M].contiguous()


def cheb_series(op: DeviceELL, M: int, c, v, dtype="c128", stream=None):
    """out = sum_{m<M} c[m] T_m(H) v  (rec_A_vec)."""
    M = int(M)
    if M < 2:
        raise ValueError("M must be >= 2")
    tv, R, squeeze, was_np = _vectors(v, op.n)
    tc = _coef(c, M, tv.device)
    out = torch.empty_like(tv)
    st = _capi.lib().kpm_cheb_series(op.handle, _capi.dtype_code(dtype), R, M, tc.data_ptr(), tv.data_ptr(),
                                     out.data_ptr(), _stream_ptr(stream))
    _capi.check(st, "kpm_cheb_series")
    return _finish(out, squeeze, was_np)


def time_evolve(op: DeviceELL, M: int, c, steps: int, v, dtype="c128", stream=None):
    """P(H)^steps v with P(H) = sum_{m<M} c[m] T_m(H) (for_time, obv.cu:93-122); all
    vectors of v advance together."""
    M, steps = int(M), int(steps)
    if M < 2:
        raise ValueError("M must be >= 2")
    if steps < 0:
        raise ValueError("steps must be >= 0")
    tv, R, squeeze, was_np = _vectors(v, op.n)
    tc = _coef(c, M, tv.device)
    out = torch.empty_like(tv)
    st = _capi.lib().kpm_time_evolve(op.handle, _capi.dtype_code(dtype), R, M, tc.data_ptr(), steps, tv.data_ptr(),
                                     out.data_ptr(), _stream_ptr(stream))
    _capi.check(st, "kpm_time_evolve")
    return _finish(out, squeeze, was_np)


def cheb_commutator_series(op: DeviceELL, vop: DeviceELL, M: int, c, v, dtype="c128", stream=None):
    """out = sum_m c[m] C_m with the commutator recursion (rec_com_A_vec); dtype c128 or c128f."""
    M = int(M)
    if M < 2:
        raise ValueError("M must be >= 2")
    tv, R, squeeze, was_np = _vectors(v, op.n)
    tc = _coef(c, M, tv.device)
    out = torch.empty_like(tv)
    st = _capi.lib().kpm_cheb_commutator_series(op.handle, vop.handle, _capi.dtype_code(dtype), R, M, tc.data_ptr(),
                                                tv.data_ptr(), out.data_ptr(), _stream_ptr(stream))
    _capi.check(st, "kpm_cheb_commutator_series")
    return _finish(out, squeeze, was_np)


def cheb_commutator_table(op: DeviceELL, vop: DeviceELL, M: int, c, v, dtype="c128", stream=None):
    """tab[m] = c[m] C_m, m < M, of the commutator recursion (rec_com_A_vec_tab): [M, n] for
    one vector, [R, M, n] for R vectors."""
    M = int(M)
    if M < 2:
        raise ValueError("M must be >= 2")
    tv, R, squeeze, was_np = _vectors(v, op.n)
    tc = _coef(c, M, tv.device)
    tab = torch.empty((R, M, op.n), dtype=torch.complex128, device=tv.device)
    st = _capi.lib().kpm_cheb_commutator_table(op.handle, vop.handle, _capi.dtype_code(dtype), R, M, tc.data_ptr(),
                                               tv.data_ptr(), tab.data_ptr(), _stream_ptr(stream))
    _capi.check(st, "kpm_cheb_commutator_table")
    return _finish(tab, squeeze, was_np)


def ell_dot(op: DeviceELL, a, b, x, y, stream=None):
    """y <- b*y + a*H x on the GPU; y is updated in place (numpy or CUDA tensor)."""
    tx, R, squeeze, _ = _vectors(x, op.n)
    y_is_np = not isinstance(y, torch.Tensor)
    ty = _as_device_c128(y)
    if ty.dim() == 1:
        ty = ty.reshape(1, -1)
    a = complex(a)
    b = complex(b)
    st = _capi.lib().kpm_ell_dot(op.handle, a.real, a.imag, b.real, b.imag, tx.data_ptr(), ty.data_ptr(), R,
                                 _stream_ptr(stream))
    _capi.check(st, "kpm_ell_dot")
    if y_is_np:
        y[...] = ty.reshape(np.shape(y)).cpu().numpy()
    elif ty.data_ptr() != y.data_ptr():
        y.copy_(ty.reshape(y.shape))
    return y


def time_sigma(op: DeviceELL, v1: DeviceELL, v2: DeviceELL, c_u, M2: int, c_fd, M: int, len_t: int, v,
               dtype="c128", stream=None):
    """sigma[r, j] = <U_c(t_j) | V1 U(t_j)> (for_time_sigma, without the -i); dtype c128 or c128f."""
    tv, R, squeeze, was_np = _vectors(v, op.n)
    tcu = _coef(c_u, int(M2), tv.device)
    tcf = _coef(c_fd, int(M), tv.device)
    sig = torch.empty((R, int(len_t)), dtype=torch.complex128, device=tv.device)
    st = _capi.lib().kpm_time_sigma(op.handle, v1.handle, v2.handle, _capi.dtype_code(dtype), R, tcu.data_ptr(), int(M2),
                                    tcf.data_ptr(), int(M), int(len_t), tv.data_ptr(), sig.data_ptr(),
                                    _stream_ptr(stream))
    _capi.check(st, "kpm_time_sigma")
    return _finish(sig, squeeze, was_np)
