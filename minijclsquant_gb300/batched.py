"""Batched KPM: many independent Hamiltonians of uneven size in one recursion.

``BatchedELL`` stacks already-rescaled ELL operators (equal ``len_row``)
block-diagonally on the GPU (``kpm_batch_create``).  ``moments`` advances R
random vectors of every instance together, one launch per Chebyshev step over
all instances, the recursion replayed as one CUDA graph
(``kpm_batch_moments``).  The reference computes the same moments with one
``rec_A_tab`` call per instance and vector (jclsquant/recurrence_functions.py:9-40).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _capi, lattice
from .ell_matrix import gershgorin_bounds_ell
from .observables import dos_from_moments, random_vector_generator


class BatchedELL:
    def __init__(self, datas, indices, len_row):
        """datas/indices: per-instance rescaled reference-layout AoS ELL arrays."""
        if not torch.cuda.is_available():
            raise RuntimeError("BatchedELL needs a CUDA GPU")
        lib = _capi.lib()
        L = int(len_row)
        rows = np.array([np.asarray(d).size // L for d in datas], dtype=np.int64)
        for d, ix, n in zip(datas, indices, rows):
            if np.asarray(d).size != n * L or np.asarray(ix).size != n * L:
                raise ValueError("instance arrays do not match len_row")
        data = np.ascontiguousarray(np.concatenate([np.asarray(d, dtype=np.complex128) for d in datas]))
        idx = np.ascontiguousarray(np.concatenate([np.asarray(i, dtype=np.int32) for i in indices]))
        h = ctypes.c_void_p()
        torch.cuda.synchronize()
        st = lib.kpm_batch_create(ctypes.byref(h), len(rows), rows.ctypes.data, L, data.ctypes.data, idx.ctypes.data,
                                  int(torch.cuda.current_stream().cuda_stream))
        _capi.check(st, "kpm_batch_create")
        self._h = h
        self.rows = rows
        self.offsets = np.concatenate([[0], np.cumsum(rows)[:-1]]).astype(np.int64)
        self.n_total = int(rows.sum())
        self.len_row = L
        n_inst, tot, pad, real = ctypes.c_int(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int()
        lib.kpm_batch_info(h, ctypes.byref(n_inst), ctypes.byref(tot), ctypes.byref(pad), ctypes.byref(real))
        self.rows_padded = int(pad.value)
        self.is_real = bool(real.value)

    @property
    def n_inst(self):
        return len(self.rows)

    def moments(self, M, v, dtype="c64", stream=None):
        """mu[k, r, m] = <v_r^(k)|T_m(H_k) v_r^(k)>.  v: [R, n_total] (numpy or CUDA tensor)."""
        was_np = not isinstance(v, torch.Tensor)
        t = torch.from_numpy(np.ascontiguousarray(np.asarray(v, dtype=np.complex128))).cuda() if was_np else \
            v.to(torch.complex128).contiguous()
        if t.dim() != 2 or t.shape[1] != self.n_total:
            raise ValueError("v must be [R, %d]" % self.n_total)
        R = int(t.shape[0])
        mu = torch.empty((self.n_inst, R, int(M)), dtype=torch.complex128, device=t.device)
        s = stream if stream is not None else torch.cuda.current_stream()
        st = _capi.lib().kpm_batch_moments(self._h, _capi.dtype_code(dtype), R, int(M), t.data_ptr(), mu.data_ptr(),
                                           int(s.cuda_stream))
        _capi.check(st, "kpm_batch_moments")
        if was_np:
            out = mu.cpu().numpy()
            _capi.check(_capi.lib().kpm_batch_check(self._h, int(s.cuda_stream)), "kpm_batch_check")
            return out
        return mu

    _KINDS = {0: "grid-stride", 1: "staged", 2: "staged+producer-warp"}

    @property
    def hermitian(self) -> bool:
        """Every instance is Hermitian (checked on the device at creation)."""
        h = ctypes.c_int()
        _capi.check(_capi.lib().kpm_batch_props(self._h, ctypes.byref(h), None), "kpm_batch_props")
        return bool(h.value)

    @property
    def doubling(self) -> bool:
        """Whether moments use the doubling identity (ceil(M/2) - 1 steps for M moments)."""
        d = ctypes.c_int()
        _capi.check(_capi.lib().kpm_batch_props(self._h, None, ctypes.byref(d)), "kpm_batch_props")
        return bool(d.value)

    def set_doubling(self, on: bool):
        _capi.check(_capi.lib().kpm_batch_set_doubling(self._h, int(bool(on))), "kpm_batch_set_doubling")

    def step_config(self, dtype="c64", R=2, stream=None):
        """The recursion-step kernel the batched autotuner chose for (dtype, R):
        dict(kind, kernel, rows_per_thread, grid, step_us); tunes it first if needed."""
        kind, U, grid, us = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
        s = stream if stream is not None else torch.cuda.current_stream()
        _capi.check(_capi.lib().kpm_batch_step_config(self._h, _capi.dtype_code(dtype), int(R), ctypes.byref(kind),
                                                      ctypes.byref(U), ctypes.byref(grid), ctypes.byref(us),
                                                      int(s.cuda_stream)), "kpm_batch_step_config")
        return {"kind": kind.value, "kernel": self._KINDS.get(kind.value, "?"), "rows_per_thread": U.value,
                "grid": grid.value, "step_us": float(us.value)}

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _capi.lib().kpm_batch_destroy(h)
            except Exception:
                pass
        self._h = None

    def __del__(self):
        self.close()


def honeycomb_ensemble(n_inst=256, side_range=(32, 512), W_range=(0.0, 2.0), seed=42, t=-2.7, bounds_factor=1.01):
    """The uneven-lattice ensemble of the batched configuration.

    Side L_k ~ uniform integer in side_range (L_k x L_k primitive cells, 2 L_k^2
    sites), W_k ~ U[W_range], disorder seed derived per instance, all from
    default_rng(seed).  Each instance is rescaled by its own Gershgorin bound
    times bounds_factor.  Returns (datas, indices, len_row, bounds list, params).
    """
    rng = np.random.default_rng(seed)
    sides = rng.integers(side_range[0], side_range[1] + 1, size=n_inst)
    Ws = rng.uniform(W_range[0], W_range[1], size=n_inst)
    seeds = rng.integers(0, 2 ** 31 - 1, size=n_inst)
    datas, idxs, bnds = [], [], []
    L = None
    for k in range(n_inst):
        arr = lattice.honeycomb_arrays(int(sides[k]), int(sides[k]), t=t, W=float(Ws[k]), seed=int(seeds[k]),
                                       with_geometry=False)
        if L is None:
            L = arr["len_row"]
        if arr["len_row"] != L:
            raise ValueError("instances differ in ELL width")
        b = gershgorin_bounds_ell(arr["data"], arr["indices"], arr["n"], factor=bounds_factor)
        datas.append(arr["data"] * (1 / ((b[1] - b[0]) / 2) + 0j))
        idxs.append(arr["indices"])
        bnds.append(b)
    return datas, idxs, L, bnds, dict(sides=sides, W=Ws, seeds=seeds)


def ensemble_vectors(rows, R, seed0=1000):
    """R random-phase vectors per instance, instance k seeded seed0 + k*R + r, stacked [R, n_total]."""
    out = np.empty((R, int(np.sum(rows))), dtype=np.complex128)
    off = 0
    for k, n in enumerate(rows):
        for r in range(R):
            out[r, off:off + n] = random_vector_generator(int(n), seed0 + k * R + r)
        off += int(n)
    return out


def batched_dos(mu, bounds, M, n_energies=None):
    """Per-instance DOS (averaged over the R vectors) from mu [K, R, M]."""
    mu = np.asarray(mu)
    return [dos_from_moments(mu[k], bounds[k], M, n_energies) for k in range(mu.shape[0])]
