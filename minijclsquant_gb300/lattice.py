"""Honeycomb (graphene) lattice builder that emits ELL arrays directly.

Vectorised numpy, O(N): it replaces the reference's lattice_hexagonal +
H_graphene route (jclsquant/lattice.py:6-47, jclsquant/hams.py:63-168), whose
periodic-border pairing is an O(B^2) Python loop, for the lattice sizes of the
benchmark configurations (up to 2048 x 2048 cells, 8.4M sites).

Geometry: primitive 2-site cells (A, B) on a1 = a(1, 0), a2 = a(1/2, sqrt3/2),
a = sqrt3 * a_cc; site index 2*(iy*nx + ix) + s.  Each A site bonds to the B
sites of cells (ix, iy), (ix-1, iy), (ix, iy-1); each B site to the A sites of
(ix, iy), (ix+1, iy), (ix, iy+1) (periodic wrap, or padding at open edges).
Row layout: slot 0 = on-site (if any on-site term is present), then the three
bonds.  Bond displacements follow the reference convention
dx_vec(i, j) = x_j - x_i (jclsquant/hams.py:96-100).  On-site disorder is
W*(2U - 1), U ~ default_rng(seed).random(N) (the convention of
modifier_diagonal_anderson, jclsquant/modifiers.py:306); mass is +m on A, -m on B.
The matrix is Hermitian (real symmetric) by construction.
"""
from __future__ import annotations

import numpy as np

from .ell_matrix import ell_matrix, gershgorin_bounds_ell

A_CC = 0.14199929870718847  # nm, carbon-carbon distance


def honeycomb_arrays(nx, ny, t=-2.7, W=0.0, seed=None, periodic=True, mass=0.0, onsite=None, a_cc=A_CC,
                     with_geometry=True):
    """ELL arrays of nearest-neighbour graphene on nx x ny primitive cells.

    Returns dict(data, indices, valid, len_row, n, dx, dy, partner, onsite).
    ``partner[i*L + s]`` is the slot index (row-major) of the reverse bond
    (j, i) for bond slots, -1 for on-site and padding slots.
    """
    nx, ny = int(nx), int(ny)
    if nx < 2 or ny < 2:
        raise ValueError("need at least 2 x 2 cells")
    n = 2 * nx * ny
    eps, has_diag = _onsite_energies(n, W, seed, mass, onsite)
    L = 4 if has_diag else 3
    first = 1 if has_diag else 0

    cell = np.arange(nx * ny, dtype=np.int64)
    ix = cell % nx
    iy = cell // nx
    A = 2 * cell
    B = 2 * cell + 1

    def cid(x, y):
        return (y % ny) * nx + (x % nx)

    # neighbours: A -> B(ix,iy), B(ix-1,iy), B(ix,iy-1);  B -> A(ix,iy), A(ix+1,iy), A(ix,iy+1)
    nbA = np.stack([2 * cid(ix, iy) + 1, 2 * cid(ix - 1, iy) + 1, 2 * cid(ix, iy - 1) + 1], axis=1)
    nbB = np.stack([2 * cid(ix, iy), 2 * cid(ix + 1, iy), 2 * cid(ix, iy + 1)], axis=1)
    okA = np.ones((nx * ny, 3), dtype=bool)
    okB = np.ones((nx * ny, 3), dtype=bool)
    if not periodic:
        okA[:, 1] = ix - 1 >= 0
        okA[:, 2] = iy - 1 >= 0
        okB[:, 1] = ix + 1 < nx
        okB[:, 2] = iy + 1 < ny
    # bond displacement x_j - x_i for each of the three bond types
    dA = _bond_displacements(a_cc)                                  # A -> B
    dB = -dA                                                        # B -> A (reverse bonds)

    data = np.zeros((n, L), dtype=np.complex128)
    indices = np.zeros((n, L), dtype=np.int32)
    valid = np.zeros((n, L), dtype=np.int32)
    dx = np.zeros((n, L))
    dy = np.zeros((n, L))
    partner = np.full((n, L), -1, dtype=np.int64)
    if has_diag:
        data[:, 0] = eps
        indices[:, 0] = np.arange(n)
        valid[:, 0] = 1
    for rows, nb, ok, d in ((A, nbA, okA, dA), (B, nbB, okB, dB)):
        for k in range(3):
            s = first + k
            m = ok[:, k]
            data[rows[m], s] = t
            indices[rows[m], s] = nb[m, k]
            valid[rows[m], s] = 1
            dx[rows[m], s] = d[k, 0]
            dy[rows[m], s] = d[k, 1]
            # reverse bond of A-slot k is B-slot k at the neighbour, and vice versa
            partner[rows[m], s] = nb[m, k] * L + s
            # padding (open edges): value 0, index = last real column of the row
            pad = ~m
            if np.any(pad):
                prev = indices[rows[pad], s - 1] if s > 0 else rows[pad]
                indices[rows[pad], s] = prev
    out = dict(data=data.reshape(-1), indices=indices.reshape(-1), valid=valid.reshape(-1), len_row=L, n=n,
               partner=partner.reshape(-1), onsite=eps)
    if with_geometry:
        out["dx"] = dx.reshape(-1).astype(np.complex128)
        out["dy"] = dy.reshape(-1).astype(np.complex128)
    return out


def honeycomb(nx, ny, t=-2.7, W=0.0, seed=None, periodic=True, mass=0.0, onsite=None, bounds_factor=1.01,
              bounds=None):
    """An ell_matrix for nearest-neighbour graphene (see module docstring).

    ``bounds`` defaults to the symmetric Gershgorin bound times ``bounds_factor``.
    """
    arr = honeycomb_arrays(nx, ny, t=t, W=W, seed=seed, periodic=periodic, mass=mass, onsite=onsite)
    if bounds is None:
        bounds = gershgorin_bounds_ell(arr["data"], arr["indices"], arr["n"], factor=bounds_factor)
    H = ell_matrix.from_ell(arr["data"], arr["indices"], arr["len_row"], bounds=bounds,
                            valid_row_values=arr["valid"], dx_vec=arr["dx"], dy_vec=arr["dy"])
    H.partner = arr["partner"]
    H.onsite = arr["onsite"]
    a = np.sqrt(3.0) * A_CC
    H.Omega = nx * ny * a * a * np.sqrt(3.0) / 2
    return H


def _onsite_energies(n, W, seed, mass, onsite):
    """On-site terms of honeycomb_arrays: onsite + mass (+m on A, -m on B) + W(2U - 1)."""
    eps = np.zeros(n)
    if onsite is not None:
        eps = np.asarray(onsite, dtype=np.float64).copy()
        if eps.shape != (n,):
            raise ValueError("onsite must have %d entries" % n)
    if mass:
        eps[0::2] += mass
        eps[1::2] -= mass
    if W:
        rng = np.random.default_rng(seed)
        eps += W * (2 * rng.random(n) - 1)
    has_diag = bool(np.any(eps != 0)) or onsite is not None
    return eps, has_diag


def _bond_displacements(a_cc):
    """x_j - x_i of the three A -> B bonds, as honeycomb_arrays computes them: [3, 2]."""
    a = np.sqrt(3.0) * a_cc
    a1 = np.array([a, 0.0])
    a2 = np.array([a / 2, a * np.sqrt(3.0) / 2])
    delta_ab = (a1 + a2) / 3.0
    return np.stack([delta_ab, delta_ab - a1, delta_ab - a2])


class DeviceLattice:
    """Graphene ELL arrays built on the GPU (see :func:`honeycomb_device`).

    Attributes: ``n``, ``len_row``, ``bounds`` (numpy [-b, b]); torch CUDA tensors
    ``data`` (H, complex128 [n * L]), ``indices`` (int32), ``valid`` (int32),
    ``partner`` (int64), ``dx`` / ``dy`` (complex128, when geometry was asked for),
    ``data_kpm`` (H~ = H / b); ``op`` (a :class:`device.DeviceELL` of H~).
    """


def honeycomb_device(nx, ny, t=-2.7, W=0.0, seed=None, periodic=True, mass=0.0, onsite=None, a_cc=A_CC,
                     bounds_factor=1.01, bounds=None, geometry=False, doubling=False, stream=None):
    """honeycomb() with the operator built on the GPU: the ELL arrays, the Gershgorin
    bound and the rescaled values H~ are made by kernels (kpm_honeycomb_ell,
    kpm_ell_gershgorin_partner, kpm_ell_scale_values) and stay in device memory; the
    host computes only the on-site energies (numpy's generator, as honeycomb_arrays
    does) and uploads them.  Arrays, bound and H~ are bit-identical to
    honeycomb_arrays + gershgorin_bounds_ell + modifier_bounds.  Replaces the setup
    route of the reference's configurations (jclsquant/lattice.py:6-47,
    jclsquant/hams.py:63-168, jclsquant/ell_matrix.py:187-200) for graphene."""
    import ctypes

    import torch

    from . import _capi, device

    if isinstance(t, complex) or np.iscomplexobj(t):
        if np.imag(t) != 0:
            raise ValueError("the device builder takes a real hopping")
        t = float(np.real(t))
    nx, ny = int(nx), int(ny)
    if nx < 2 or ny < 2:
        raise ValueError("need at least 2 x 2 cells")
    n = 2 * nx * ny
    eps, has_diag = _onsite_energies(n, W, seed, mass, onsite)
    L = 4 if has_diag else 3
    lib = _capi.lib()
    dev = torch.device("cuda")
    sp = device._stream_ptr(stream)
    out = DeviceLattice()
    out.n, out.len_row = n, L
    out.data = torch.empty(n * L, dtype=torch.complex128, device=dev)
    out.indices = torch.empty(n * L, dtype=torch.int32, device=dev)
    out.valid = torch.empty(n * L, dtype=torch.int32, device=dev)
    out.partner = torch.empty(n * L, dtype=torch.int64, device=dev)
    out.dx = torch.empty(n * L, dtype=torch.complex128, device=dev) if geometry else None
    out.dy = torch.empty(n * L, dtype=torch.complex128, device=dev) if geometry else None
    eps_d = torch.from_numpy(eps).to(dev) if has_diag else None
    disp = np.ascontiguousarray(_bond_displacements(a_cc).reshape(-1))
    st = lib.kpm_honeycomb_ell(nx, ny, int(bool(periodic)), float(t),
                               eps_d.data_ptr() if eps_d is not None else None, L, disp.ctypes.data,
                               out.data.data_ptr(), out.indices.data_ptr(), out.valid.data_ptr(),
                               out.dx.data_ptr() if geometry else None, out.dy.data_ptr() if geometry else None,
                               out.partner.data_ptr(), sp)
    _capi.check(st, "kpm_honeycomb_ell")
    if bounds is None:
        b = ctypes.c_double()
        st = lib.kpm_ell_gershgorin_partner(n, L, out.data.data_ptr(), out.indices.data_ptr(),
                                            out.partner.data_ptr(), float(bounds_factor), ctypes.byref(b), sp)
        _capi.check(st, "kpm_ell_gershgorin_partner")
        bounds = np.array([-b.value, b.value])
    out.bounds = np.asarray(bounds, dtype=np.float64)
    b0, b1 = float(out.bounds[0]), float(out.bounds[1])
    if abs(b1) != abs(b0):
        raise ValueError("the device builder rescales with symmetric bounds only")
    out.data_kpm = out.data.clone()
    st = lib.kpm_ell_scale_values(n * L, 1 / ((b1 - b0) / 2), out.data_kpm.data_ptr(), sp)
    _capi.check(st, "kpm_ell_scale_values")
    out.op = device.DeviceELL(out.data_kpm, out.indices, L, doubling=doubling)
    a = np.sqrt(3.0) * a_cc
    out.Omega = nx * ny * a * a * np.sqrt(3.0) / 2
    return out


def to_csr(arr):
    """scipy CSR of builder arrays (valid slots only), e.g. to feed jclsquant's ell_matrix."""
    import scipy.sparse as sp

    n, L = arr["n"], arr["len_row"]
    rows = np.repeat(np.arange(n), L)
    m = arr["valid"] == 1
    return sp.csr_matrix((arr["data"][m], (rows[m], arr["indices"][m])), shape=(n, n))
