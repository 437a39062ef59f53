"""The ELL operator object, drop-in for jclsquant/ell_matrix.py.

``ell_matrix`` keeps the reference's host-side attributes (``data``,
``indices``, ``len_row``, ``shape``, ``bounds``, ``valid_row_values``,
``dx_vec``, ``dy_vec``, ``conjugates``, ``n_threads``) in the reference's
padded row-major layout, so code that reads or edits them keeps working.
Every product with the operator (``dot``, the recursions) runs on the GPU on
a cached device copy (:class:`minijclsquant_gb300.device.DeviceELL`), built on
first use and rebuilt when ``data`` or ``indices`` is reassigned.  Code that
edits ``data`` in place must call :meth:`ell_matrix.invalidate_device`.
"""
from __future__ import annotations

import copy
import os

import numpy as np
import scipy.sparse as sp


def csr_to_ell_arrays(A, extra=()):
    """Padded row-major ELL from a CSR matrix.

    Mirrors csr_to_ell + data_indices_c (jclsquant/ell_matrix.py:187-200,
    jclsquant/cython_modules/Extra_funs.pyx:81-137): len_row = max row length;
    row i holds its CSR entries in stored order in slots 0..nnz_i-1; padding
    slots get value 0, valid 0 and the last real column of the row.  A row
    without entries (undefined in the reference) is padded with its own index.
    ``extra`` is a sequence of CSR matrices with A's sparsity pattern (DX, DY,
    CJ) laid out the same way.  Returns (len_row, data, indices, valid, [extras]).
    """
    A = A.tocsr()
    n = A.shape[0]
    indptr = np.asarray(A.indptr, dtype=np.int64)
    nnz = np.diff(indptr)
    L = int(nnz.max()) if n else 0
    rows = np.repeat(np.arange(n, dtype=np.int64), nnz)
    k = np.arange(indptr[-1], dtype=np.int64) - np.repeat(indptr[:-1], nnz)
    pos = rows * L + k
    cols = np.asarray(A.indices, dtype=np.int32)
    last = np.where(nnz > 0, cols[np.maximum(indptr[1:] - 1, 0)] if cols.size else 0,
                    np.arange(n, dtype=np.int32)).astype(np.int32)
    indices = np.repeat(last, L)
    indices[pos] = cols
    data = np.zeros(n * L, dtype=np.complex128)
    data[pos] = np.asarray(A.data, dtype=np.complex128)
    valid = np.zeros(n * L, dtype=np.int32)
    valid[pos] = 1
    outs = []
    for E in extra:
        e = np.zeros(n * L, dtype=np.complex128)
        E = E.tocsr()
        if E.nnz != A.nnz:
            raise ValueError("companion matrix has %d entries, operator has %d" % (E.nnz, A.nnz))
        e[pos] = np.asarray(E.data, dtype=np.complex128)
        outs.append(e)
    return L, data, indices, valid, outs


def csr_to_ell_device(A, extra=(), conjugates=None, stream=None):
    """csr_to_ell_arrays on the GPU (kpm_csr_row_max + kpm_csr_to_ell): the same
    padded row-major arrays, bit for bit, as CUDA tensors.  ``A`` is a scipy CSR
    matrix (uploaded) or a tuple (indptr, indices, data) of CUDA tensors.  ``extra``
    holds companion matrices with A's sparsity (DX, DY); ``conjugates`` an int32
    array of the entries' conjugate slots (the reference's CJ data).  Returns
    (len_row, data, indices, valid, [extras], conj or None)."""
    import ctypes

    import torch

    from . import _capi, device

    dev = torch.device("cuda")
    if isinstance(A, tuple):
        indptr, cols, vals = A
        indptr = indptr.to(device=dev, dtype=torch.int64).contiguous()
        cols = cols.to(device=dev, dtype=torch.int32).contiguous()
        vals = vals.to(device=dev, dtype=torch.complex128).contiguous()
        extras = [e.to(device=dev, dtype=torch.complex128).contiguous() for e in extra]
    else:
        A = A.tocsr()
        indptr = torch.from_numpy(np.asarray(A.indptr, dtype=np.int64)).to(dev)
        cols = torch.from_numpy(np.asarray(A.indices, dtype=np.int32)).to(dev)
        vals = torch.from_numpy(np.asarray(A.data, dtype=np.complex128)).to(dev)
        extras = []
        for E in extra:
            E = E.tocsr()
            if E.nnz != A.nnz:
                raise ValueError("companion matrix has %d entries, operator has %d" % (E.nnz, A.nnz))
            extras.append(torch.from_numpy(np.asarray(E.data, dtype=np.complex128)).to(dev))
    if len(extras) > 2:
        raise ValueError("at most two companion matrices (DX, DY)")
    cj = None
    if conjugates is not None:
        cj = torch.as_tensor(np.asarray(conjugates, dtype=np.int32) if not isinstance(conjugates, torch.Tensor)
                             else conjugates).to(device=dev, dtype=torch.int32).contiguous()
    n = int(indptr.numel() - 1)
    lib = _capi.lib()
    sp = device._stream_ptr(stream)
    L = ctypes.c_int()
    _capi.check(lib.kpm_csr_row_max(n, indptr.data_ptr(), ctypes.byref(L), sp), "kpm_csr_row_max")
    L = int(L.value)
    if L < 1:
        raise ValueError("matrix without entries")
    data = torch.empty(n * L, dtype=torch.complex128, device=dev)
    idx = torch.empty(n * L, dtype=torch.int32, device=dev)
    valid = torch.empty(n * L, dtype=torch.int32, device=dev)
    outs = [torch.empty(n * L, dtype=torch.complex128, device=dev) for _ in extras]
    cj_out = torch.empty(n * L, dtype=torch.int32, device=dev) if cj is not None else None
    ptr = lambda t: t.data_ptr() if t is not None else None  # noqa: E731
    src = extras + [None] * (2 - len(extras))
    dst = outs + [None] * (2 - len(outs))
    st = lib.kpm_csr_to_ell(n, L, indptr.data_ptr(), cols.data_ptr(), vals.data_ptr(), ptr(src[0]), ptr(src[1]),
                            ptr(cj), data.data_ptr(), idx.data_ptr(), ptr(dst[0]), ptr(dst[1]), ptr(cj_out),
                            valid.data_ptr(), sp)
    _capi.check(st, "kpm_csr_to_ell")
    return L, data, idx, valid, outs, cj_out


def ell_to_csr(A):
    """ELL object -> scipy CSR (jclsquant/ell_matrix.py:15-31), vectorised."""
    n = int(A.shape[0])
    L = int(A.len_row)
    rows = np.repeat(np.arange(n), L)
    return sp.csr_matrix((np.asarray(A.data), (rows, np.asarray(A.indices))), shape=(n, n))


def Gershgorin(H):
    """Gershgorin interval from column sums of |H| (jclsquant/ell_matrix.py:83-93)."""
    centers = H.diagonal()
    radii = np.asarray(np.abs(H).sum(axis=0)).ravel() - np.abs(centers)
    return np.array([np.amin(centers - radii), np.amax(centers + radii)])


def bounds(H):
    """Symmetric spectral bounds with a 2.5 % margin (jclsquant/ell_matrix.py:96-114)."""
    if not sp.isspmatrix_csr(H):
        H = ell_to_csr(H)
    g = Gershgorin(H).real
    extra = (g[1] - g[0]) * 0.025
    b = np.array([g[0] - extra, g[1] + extra])
    m = np.max(np.abs(b))
    return np.array([-m, m])


def gershgorin_bounds_ell(data, indices, n, factor=1.01):
    """Symmetric Gershgorin bound from ELL arrays, scaled by ``factor``.

    Centre = diagonal entry, radius = column sum of |H| minus |centre|, the same
    quantities as :func:`Gershgorin`; used by the lattice builder for its
    configurations (bound times 1.01 instead of the reference's 2.5 % margin).
    """
    data = np.asarray(data)
    indices = np.asarray(indices, dtype=np.int64)
    L = data.size // n
    rows = np.repeat(np.arange(n), L)
    absd = np.abs(data)
    colsum = np.bincount(indices, weights=absd, minlength=n)
    diag = np.zeros(n, dtype=np.complex128)
    dmask = indices == rows
    np.add.at(diag, rows[dmask], data[dmask])
    c = diag.real
    r = colsum - np.abs(diag)
    b = max(abs(np.min(c - r)), abs(np.max(c + r))) * factor
    return np.array([-b, b])


class ell_matrix:
    """ELL sparse operator with GPU products (drop-in for jclsquant's ell_matrix,
    jclsquant/ell_matrix.py:119-258)."""

    def __init__(self, A, DX=None, DY=None, CJ=None, velocities="False", space="r"):
        self.A = A
        self.type = None
        self.len_row = None
        self.len_col = None
        self.shape = None
        self.n_threads = None
        self.DX, self.DY, self.CJ = DX, DY, CJ
        self.dx_vec = self.dy_vec = self.dz_vec = None
        self.Omega = None
        self.conjugates = None
        self.valid_row_values = None
        self._data = None
        self._indices = None
        self._dev = None
        self.set_n_threads()
        if A is not None:
            self.check_format()
            self.bounds = bounds(self.A)
        else:
            self.bounds = None
        self.space = space
        self.velocities = velocities

    # -- construction -------------------------------------------------------
    @classmethod
    def from_ell(cls, data, indices, len_row, bounds=None, valid_row_values=None, dx_vec=None, dy_vec=None,
                 conjugates=None):
        """Wrap ready-made padded row-major ELL arrays (no CSR detour)."""
        self = cls(None)
        data = np.ascontiguousarray(np.asarray(data, dtype=np.complex128))
        indices = np.ascontiguousarray(np.asarray(indices, dtype=np.int32))
        self.len_row = int(len_row)
        n = data.size // self.len_row
        if n * self.len_row != data.size or indices.size != data.size:
            raise ValueError("ELL arrays do not match len_row")
        self.shape = np.array([n, n], dtype=np.int32)
        self.len_col = n
        self._data = data
        self._indices = indices
        self.valid_row_values = (np.ascontiguousarray(valid_row_values, dtype=np.int32) if valid_row_values is not None
                                 else (data != 0).astype(np.int32))
        self.dx_vec = dx_vec
        self.dy_vec = dy_vec
        self.conjugates = conjugates
        self.type = "ELLPACK(ELL) sparse matrix format"
        self.bounds = np.asarray(bounds, dtype=np.float64) if bounds is not None else \
            gershgorin_bounds_ell(data, indices, n, factor=1.0)
        return self

    def check_format(self):
        if sp.isspmatrix_csr(self.A):
            self.csr_to_ell()
            self.type = "ELLPACK(ELL) sparse matrix format"
        else:
            raise TypeError("ell_matrix expects a scipy CSR matrix")

    def set_n_threads(self):
        if self.n_threads is None:
            env = os.getenv("OMP_NUM_THREADS")
            self.n_threads = 8 if env is None else int(env)

    def csr_to_ell(self):
        extra = []
        if self.DX is not None and self.DY is not None:
            extra = [self.DX, self.DY, self.CJ if self.CJ is not None else self.DX]
        L, data, indices, valid, outs = csr_to_ell_arrays(self.A, extra)
        self.len_row = L
        self.shape = np.array([self.A.shape[0], self.A.shape[0]], dtype=np.int32)
        self.len_col = self.shape[0]
        self._data = data
        self._indices = indices
        self.valid_row_values = valid
        if outs:
            self.dx_vec, self.dy_vec = outs[0], outs[1]
            self.conjugates = np.real(outs[2]).astype(np.int32)

    # -- attributes that invalidate the device copy ---------------------------
    @property
    def data(self):
        return self._data

    @data.setter
    def data(self, value):
        self._data = value
        self._dev = None

    @property
    def indices(self):
        return self._indices

    @indices.setter
    def indices(self, value):
        self._indices = value
        self._dev = None

    def invalidate_device(self):
        self._dev = None

    def device(self):
        """The cached GPU operator holding exactly ``self.data`` / ``self.indices``."""
        if self._dev is None:
            from .device import DeviceELL

            self._dev = DeviceELL(self._data, self._indices, self.len_row, int(self.shape[0]))
        return self._dev

    # -- reference API --------------------------------------------------------
    def save(self, path=None):
        import joblib

        joblib.dump(self, path or "./H.json")

    def dot(self, a, b, x, y):
        """y <- b*y + a*A x, in place (jclsquant/ell_matrix.py:209-211), on the GPU."""
        from .device import ell_dot

        ell_dot(self.device(), a, b, x, y)

    def deep_copy(self):
        return copy.deepcopy(self)

    def modifier(self, func, *args, **kwargs):
        """New matrix whose data is func(self, ...) (jclsquant/ell_matrix.py:218-223)."""
        new_data = func(self, *args, **kwargs)
        new = self.deep_copy()
        new.data = new_data
        return new

    def modifier_nocop(self, other, func, *args, **kwargs):
        """Replace data (and optionally dx/dy) by func(other, copies...) (jclsquant/ell_matrix.py:225-246)."""
        data_new = np.ascontiguousarray(np.copy(self.data))
        dx_new = np.ascontiguousarray(np.copy(self.dx_vec))
        dy_new = np.ascontiguousarray(np.copy(self.dy_vec))
        result = func(other, data_new, dx_new, dy_new, *args, **kwargs)
        if isinstance(result, tuple):
            self.data, self.dx_vec, self.dy_vec = result[0], result[1], result[2]
        else:
            self.data = result

    def __deepcopy__(self, memo):
        new = self.__class__.__new__(self.__class__)
        memo[id(self)] = new
        for k, v in self.__dict__.items():
            if k == "_dev":
                new._dev = None
            elif k in ("A", "DX", "DY", "CJ"):
                setattr(new, k, v)  # scipy matrices are never modified in place here
            else:
                setattr(new, k, copy.deepcopy(v, memo))
        return new

    def __getstate__(self):
        st = dict(self.__dict__)
        st["_dev"] = None
        return st
