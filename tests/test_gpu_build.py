"""Operator construction on the device (kpm_build.cu), bit for bit against the host:

* kpm_csr_to_ell against the reference's own data_indices_c output (the padded ELL
  arrays stored in the golden fixtures, made by jclsquant's ell_matrix) and against
  csr_to_ell_arrays;
* kpm_honeycomb_ell + kpm_ell_gershgorin_partner + kpm_ell_scale_values against
  honeycomb_arrays + gershgorin_bounds_ell + modifier_bounds, at small sizes and on the
  1024 x 1024 lattice; the moments of the two operators are then the same numbers.
Index work is compared exactly (np.array_equal / torch.equal), values bitwise."""
import ctypes

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def _csr_from_ell(data, indices, valid, L, *companions):
    """The CSR a padded ELL was made from: the valid slots of each row in slot order."""
    import torch

    n = data.size // L
    v = valid.reshape(n, L) == 1
    indptr = np.concatenate([[0], np.cumsum(v.sum(axis=1))]).astype(np.int64)
    m = valid == 1
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    return (t(indptr), t(indices[m].astype(np.int32)), t(data[m])), [t(c[m]) for c in companions]


@pytest.mark.parametrize("case", ["honeycomb_8x8", "ref_graphene_256", "complex_open_6x5", "irregular_300",
                                  "tiny_2x2"])
def test_csr_to_ell_reproduces_reference_arrays(cuda_lib, case):
    from minijclsquant_gb300.ell_matrix import csr_to_ell_device

    z = golden(case)
    L = int(z["len_row"])
    csr, _ = _csr_from_ell(z["data"], z["indices"], z["valid"], L)
    L2, data, idx, valid, _, _ = csr_to_ell_device(csr)
    assert L2 == L
    assert np.array_equal(data.cpu().numpy(), z["data"])
    assert np.array_equal(idx.cpu().numpy(), z["indices"])
    assert np.array_equal(valid.cpu().numpy(), z["valid"])


def test_csr_to_ell_companions_match_reference(cuda_lib):
    from minijclsquant_gb300.ell_matrix import csr_to_ell_device

    z = golden("honeycomb_8x8")
    x = golden("honeycomb_8x8_more")
    L = int(z["len_row"])
    csr, comp = _csr_from_ell(z["data"], z["indices"], z["valid"], L, x["dx_vec"], x["dy_vec"])
    _, data, idx, valid, outs, _ = csr_to_ell_device(csr, extra=comp)
    assert np.array_equal(outs[0].cpu().numpy(), x["dx_vec"])
    assert np.array_equal(outs[1].cpu().numpy(), x["dy_vec"])


def test_csr_to_ell_matches_host_conversion_on_irregular_rows(cuda_lib):
    import scipy.sparse as sp

    from minijclsquant_gb300.ell_matrix import csr_to_ell_arrays, csr_to_ell_device

    rng = np.random.default_rng(11)
    n = 5000
    nnz_row = rng.integers(0, 9, size=n)
    nnz_row[17] = 0  # rows without entries: padded with their own index
    nnz_row[4000] = 0
    rows = np.repeat(np.arange(n), nnz_row)
    cols = np.concatenate([rng.choice(n, size=k, replace=False) for k in nnz_row])
    vals = rng.normal(size=rows.size) + 1j * rng.normal(size=rows.size)
    A = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    DX = A.copy()
    DX.data = rng.normal(size=A.nnz) + 0j
    conj = rng.integers(0, A.nnz, size=A.nnz).astype(np.int32)
    L, data, idx, valid, (dx,) = csr_to_ell_arrays(A, extra=(DX,))
    L2, d_data, d_idx, d_valid, (d_dx,), d_conj = csr_to_ell_device(A, extra=(DX,), conjugates=conj)
    assert L2 == L
    assert np.array_equal(d_data.cpu().numpy(), data)
    assert np.array_equal(d_idx.cpu().numpy(), idx)
    assert np.array_equal(d_valid.cpu().numpy(), valid)
    assert np.array_equal(d_dx.cpu().numpy(), dx)
    # conjugate companions: stored order, zero padding
    cj = np.zeros(n * L, dtype=np.int32)
    cj[valid == 1] = conj
    assert np.array_equal(d_conj.cpu().numpy(), cj)


def test_csr_to_ell_errors(cuda_lib):
    import torch

    from minijclsquant_gb300 import _capi

    lib = _capi.lib()
    indptr = torch.tensor([0, 2, 1, 3], dtype=torch.int64, device="cuda")  # decreasing
    L = ctypes.c_int()
    assert lib.kpm_csr_row_max(3, indptr.data_ptr(), ctypes.byref(L), None) == _capi.KPM_ERR_SHAPE
    assert lib.kpm_csr_row_max(0, indptr.data_ptr(), ctypes.byref(L), None) == _capi.KPM_ERR_INVALID_ARG
    ip = torch.tensor([0, 3, 4], dtype=torch.int64, device="cuda")
    cols = torch.tensor([0, 1, 1, 0], dtype=torch.int32, device="cuda")
    vals = torch.ones(4, dtype=torch.complex128, device="cuda")
    d = torch.empty(4, dtype=torch.complex128, device="cuda")
    i = torch.empty(4, dtype=torch.int32, device="cuda")
    # row 0 holds 3 entries: len_row 2 is too short
    st = lib.kpm_csr_to_ell(2, 2, ip.data_ptr(), cols.data_ptr(), vals.data_ptr(), None, None, None, d.data_ptr(),
                            i.data_ptr(), None, None, None, None, None)
    assert st == _capi.KPM_ERR_SHAPE
    st = lib.kpm_csr_to_ell(2, 2, ip.data_ptr(), None, vals.data_ptr(), None, None, None, d.data_ptr(),
                            i.data_ptr(), None, None, None, None, None)
    assert st == _capi.KPM_ERR_INVALID_ARG
    # a companion output without its input
    st = lib.kpm_csr_to_ell(2, 3, ip.data_ptr(), cols.data_ptr(), vals.data_ptr(), None, None, None, d.data_ptr(),
                            i.data_ptr(), d.data_ptr(), None, None, None, None)
    assert st == _capi.KPM_ERR_INVALID_ARG


HONEY = [
    dict(nx=8, ny=8, W=0.5, seed=1234),
    dict(nx=2, ny=2, W=0.2, seed=1),
    dict(nx=5, ny=3, periodic=False),
    dict(nx=6, ny=4, mass=0.3, W=0.2, seed=3, periodic=False),
    dict(nx=40, ny=36, t=-2.7, W=0.7, seed=5),
    dict(nx=33, ny=17, t=-1.0, W=2.0, seed=9, periodic=False),
    dict(nx=200, ny=150, W=1.0, seed=2),  # several hundred CTAs in the bound's reduction
]


@pytest.mark.parametrize("kw", HONEY)
def test_honeycomb_device_is_bit_identical_to_host_builder(cuda_lib, kw):
    from minijclsquant_gb300 import lattice
    from minijclsquant_gb300.ell_matrix import gershgorin_bounds_ell
    from minijclsquant_gb300.modifiers import modifier_bounds

    arr = lattice.honeycomb_arrays(**kw)
    g = lattice.honeycomb_device(geometry=True, **kw)
    assert g.len_row == arr["len_row"] and g.n == arr["n"]
    for key in ("data", "indices", "valid", "partner", "dx", "dy"):
        assert np.array_equal(getattr(g, key).cpu().numpy(), arr[key]), key
    b = gershgorin_bounds_ell(arr["data"], arr["indices"], arr["n"], factor=1.01)
    assert np.array_equal(g.bounds, b)
    H = lattice.honeycomb(**kw)
    assert np.array_equal(g.data_kpm.cpu().numpy(), modifier_bounds(H))


def test_honeycomb_device_explicit_onsite_and_complex_dtype_hopping(cuda_lib):
    from minijclsquant_gb300 import lattice

    n = 2 * 7 * 5
    onsite = np.linspace(-1.0, 1.0, n)
    arr = lattice.honeycomb_arrays(7, 5, t=-2.7 + 0j, onsite=onsite, periodic=False)
    g = lattice.honeycomb_device(7, 5, t=-2.7 + 0j, onsite=onsite, periodic=False)
    assert np.array_equal(g.data.cpu().numpy(), arr["data"])
    with pytest.raises(ValueError):
        lattice.honeycomb_device(7, 5, t=-2.7 + 0.1j)
    with pytest.raises(ValueError):
        lattice.honeycomb_device(1, 5)


def test_honeycomb_device_full_size_and_moments(cuda_lib, monkeypatch):
    import torch

    from minijclsquant_gb300 import device, lattice
    from minijclsquant_gb300.ell_matrix import gershgorin_bounds_ell
    from minijclsquant_gb300.modifiers import modifier_bounds
    from minijclsquant_gb300.observables import random_vector_generator

    kw = dict(nx=1024, ny=1024, t=-2.7, W=1.0, seed=1234)
    arr = lattice.honeycomb_arrays(with_geometry=False, **kw)
    monkeypatch.setenv("KPM_STEP_KERNEL", "ws1")
    g = lattice.honeycomb_device(**kw)
    assert torch.equal(g.data, torch.from_numpy(arr["data"]).cuda())
    assert torch.equal(g.indices, torch.from_numpy(arr["indices"]).cuda())
    assert torch.equal(g.partner, torch.from_numpy(arr["partner"]).cuda())
    b = gershgorin_bounds_ell(arr["data"], arr["indices"], arr["n"], factor=1.01)
    assert np.array_equal(g.bounds, b)

    class _H:
        pass

    H = _H()
    H.data, H.bounds, H.shape = arr["data"], b, (arr["n"], arr["n"])
    data_kpm = modifier_bounds(H)
    assert torch.equal(g.data_kpm, torch.from_numpy(data_kpm).cuda())
    # one step kernel for both handles, so the reduction order is the same
    monkeypatch.setenv("KPM_STEP_KERNEL", "ws1")
    host_op = device.DeviceELL(data_kpm, arr["indices"], arr["len_row"])
    v = np.stack([random_vector_generator(arr["n"], 40 + r) for r in range(2)])
    assert np.array_equal(device.cheb_moments(g.op, 64, v), device.cheb_moments(host_op, 64, v))


def test_honeycomb_ell_invalid_arguments(cuda_lib):
    import torch

    from minijclsquant_gb300 import _capi

    lib = _capi.lib()
    disp = np.zeros(6)
    d = torch.empty(64, dtype=torch.complex128, device="cuda")
    i = torch.empty(64, dtype=torch.int32, device="cuda")
    args = (disp.ctypes.data, d.data_ptr(), i.data_ptr(), None, None, None, None, None)
    assert lib.kpm_honeycomb_ell(1, 4, 1, -1.0, None, 3, *args) == _capi.KPM_ERR_INVALID_ARG
    assert lib.kpm_honeycomb_ell(4, 4, 1, -1.0, None, 4, *args) == _capi.KPM_ERR_INVALID_ARG  # no on-site array
    assert lib.kpm_honeycomb_ell(4, 4, 1, -1.0, None, 5, *args) == _capi.KPM_ERR_INVALID_ARG
    b = ctypes.c_double()
    assert lib.kpm_ell_gershgorin_partner(8, 17, d.data_ptr(), i.data_ptr(), i.data_ptr(), 1.0, ctypes.byref(b),
                                          None) == _capi.KPM_ERR_INVALID_ARG
    assert lib.kpm_ell_scale_values(0, 2.0, d.data_ptr(), None) == _capi.KPM_ERR_INVALID_ARG
