"""GPU parity: libkpm (through its C ABI and through the drop-in Python API)
against the reference's golden vectors and against the oracle.

Tolerance for complex128 moments (the drop-in form), per order m:
    |mu_m - ref_m| <= 1e-10 * max(|ref_m|, 1e-6 * |ref_0|)
and for vectors (series, commutator, sigma): max|diff| <= 1e-10 * max|ref|.
"""
import ctypes

import numpy as np
import pytest

from conftest import golden
from oracle import oracle

pytestmark = pytest.mark.gpu

CASES = ["honeycomb_8x8", "ref_graphene_256", "complex_open_6x5", "irregular_300"]
REL = 1e-10


def _torch():
    import torch

    return torch


def _dev(a):
    torch = _torch()
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _create(lib, data, indices, L):
    from minijclsquant_gb300 import _capi

    d = np.ascontiguousarray(data, dtype=np.complex128)
    ix = np.ascontiguousarray(indices, dtype=np.int32)
    h = ctypes.c_void_p()
    st = lib.kpm_ell_create(ctypes.byref(h), d.size // L, L, d.ctypes.data, ix.ctypes.data, 0, None)
    assert st == _capi.KPM_OK, lib.kpm_strerror(st)
    return h


@pytest.mark.parametrize("case", CASES)
def test_cabi_moments_match_reference(cuda_lib, case):
    torch = _torch()
    z = golden(case)
    L, M = int(z["len_row"]), int(z["M"])
    h = _create(cuda_lib, z["data_kpm"], z["indices"], L)
    try:
        v = _dev(z["v"])
        R = v.shape[0]
        mu = torch.empty((R, M), dtype=torch.complex128, device="cuda")
        st = cuda_lib.kpm_cheb_moments(h, 0, R, M, v.data_ptr(), None, mu.data_ptr(), None, None)
        assert st == 0
        torch.cuda.synchronize()
        ok, err = oracle.moment_tolerance_ok(mu.cpu().numpy(), z["mu"], REL)
        assert ok, err
    finally:
        cuda_lib.kpm_ell_destroy(h)


@pytest.mark.parametrize("case", CASES)
def test_dropin_rec_A_tab_matches_reference(cuda_lib, case):
    from minijclsquant_gb300.ell_matrix import ell_matrix
    from minijclsquant_gb300.recurrence_functions import rec_A_tab

    z = golden(case)
    Hk = ell_matrix.from_ell(z["data_kpm"], z["indices"], int(z["len_row"]), bounds=z["bounds"])
    for r in range(z["v"].shape[0]):
        mu = rec_A_tab(int(z["M"]), Hk, z["v"][r])
        assert isinstance(mu, np.ndarray) and mu.dtype == np.complex128 and mu.shape == (int(z["M"]),)
        ok, err = oracle.moment_tolerance_ok(mu, z["mu"][r], REL)
        assert ok, (r, err)


def test_dropin_full_pipeline_from_csr(cuda_lib):
    """ell_matrix from CSR -> bounds -> modifier_bounds -> kpm_dos_gpu, as a user of the reference would."""
    from minijclsquant_gb300 import lattice
    from minijclsquant_gb300.ell_matrix import ell_matrix
    from minijclsquant_gb300.observables_gpu import kpm_dos_gpu

    z = golden("honeycomb_64x64")
    arr = lattice.honeycomb_arrays(64, 64, t=-2.7, W=0.5, seed=1234)
    H = ell_matrix(lattice.to_csr(arr))
    from minijclsquant_gb300.observables import random_vector_generator

    v = random_vector_generator(8192, 1000)
    dos = kpm_dos_gpu(H, 512, v)
    assert np.array_equal(dos[:, 0], z["dos"][:, 0])
    assert np.max(np.abs(dos[:, 1] - z["dos"][:, 1])) <= 1e-10 * np.max(np.abs(z["dos"][:, 1]))


def test_cpu_dos_configuration_four_vectors(cuda_lib):
    """64 x 64 cells, M = 512, R = 4 random vectors in one call."""
    from minijclsquant_gb300 import device, lattice
    from minijclsquant_gb300.ell_matrix import ell_matrix
    from minijclsquant_gb300.modifiers import modifier_bounds
    from minijclsquant_gb300.observables import random_vector_generator

    z = golden("honeycomb_64x64")
    H = ell_matrix(lattice.to_csr(lattice.honeycomb_arrays(64, 64, t=-2.7, W=0.5, seed=1234)))
    Hk = H.modifier(modifier_bounds)
    vs = np.stack([random_vector_generator(8192, int(s)) for s in z["seeds"]])
    mu = device.cheb_moments(Hk.device(), 512, vs)
    ok, err = oracle.moment_tolerance_ok(mu, z["mu"], REL)
    assert ok, err


@pytest.mark.parametrize("R", [1, 2, 3, 5, 8, 11])
def test_vector_batches_equal_single_vectors(cuda_lib, R):
    from minijclsquant_gb300 import device

    z = golden("irregular_300")
    op = device.DeviceELL(z["data_kpm"], z["indices"], int(z["len_row"]))
    rng = np.random.default_rng(R)
    vs = np.exp(1j * rng.uniform(0, 2 * np.pi, (R, op.n)))
    mu = device.cheb_moments(op, 37, vs)
    for r in range(R):
        ref = oracle.rec_A_tab(37, z["data_kpm"], z["indices"], int(z["len_row"]), vs[r])
        ok, err = oracle.moment_tolerance_ok(mu[r], ref, REL)
        assert ok, (r, err)


def test_two_vector_moments(cuda_lib):
    from minijclsquant_gb300.ell_matrix import ell_matrix
    from minijclsquant_gb300.recurrence_functions import rec_A_tab2v, rec_A_tab2v_2

    z = golden("honeycomb_8x8")
    x = golden("honeycomb_8x8_more")
    Hk = ell_matrix.from_ell(z["data_kpm"], z["indices"], int(z["len_row"]), bounds=z["bounds"])
    M = int(z["M"])
    assert oracle.moment_tolerance_ok(rec_A_tab2v(M, Hk, x["v_l"], z["v"][0]), x["mu_lr"], REL)[0]
    a, b = rec_A_tab2v_2(M, Hk, x["v_l"], z["v"][0])
    assert oracle.moment_tolerance_ok(a, x["mu2_a"], REL)[0]
    assert oracle.moment_tolerance_ok(b, x["mu2_b"], REL)[0]


def test_series_commutator_and_time_sigma(cuda_lib):
    from minijclsquant_gb300.ell_matrix import ell_matrix
    from minijclsquant_gb300.recurrence_functions import rec_A_vec, rec_com_A_vec
    from minijclsquant_gb300 import device

    z = golden("honeycomb_8x8")
    x = golden("honeycomb_8x8_more")
    L = int(z["len_row"])
    Hk = ell_matrix.from_ell(z["data_kpm"], z["indices"], L, bounds=z["bounds"])
    V2 = ell_matrix.from_ell(x["v2_data"], z["indices"], L, bounds=z["bounds"])
    V1 = ell_matrix.from_ell(x["v1_data"], z["indices"], L, bounds=z["bounds"])
    Ms = len(x["coef"])
    v = z["v"][0]
    s = rec_A_vec(Ms, Hk, x["coef"], v)
    assert np.max(np.abs(s - x["series"])) <= REL * np.max(np.abs(x["series"]))
    c = rec_com_A_vec(Ms, Hk, V2, x["coef"], v)
    assert np.max(np.abs(c - x["comm"])) <= REL * np.max(np.abs(x["comm"]))
    sig = device.time_sigma(Hk.device(), V1.device(), V2.device(), x["cu"], int(x["M2"]), x["coef"], Ms,
                            int(x["len_t"]), v)
    assert np.max(np.abs(sig - x["sigma"])) <= REL * np.max(np.abs(x["sigma"]))


def test_reference_compatible_host_entry_points(cuda_lib):
    from minijclsquant_gb300 import obv_gpu

    z = golden("ref_graphene_256")
    x = golden("honeycomb_8x8_more")
    h8 = golden("honeycomb_8x8")
    M = int(z["M"])
    out = np.zeros(M, dtype=np.complex128)
    obv_gpu.rec_A_tab_gpu(z["data_kpm"], z["indices"], int(z["len_row"]), np.ascontiguousarray(z["v"][0]), out, M)
    assert oracle.moment_tolerance_ok(out, z["mu"][0], REL)[0]
    out2 = np.zeros(int(h8["M"]), dtype=np.complex128)
    obv_gpu.rec_A_tab_2_gpu(h8["data_kpm"], h8["indices"], int(h8["len_row"]), x["v_l"],
                            np.ascontiguousarray(h8["v"][0]), out2, int(h8["M"]))
    assert oracle.moment_tolerance_ok(out2, x["mu_lr"], REL)[0]
    sig = np.zeros(int(x["len_t"]), dtype=np.complex128)
    obv_gpu.for_time_sigma_gpu(h8["data_kpm"], x["v1_data"], x["v2_data"], h8["indices"], int(h8["len_row"]),
                               x["cu"], x["coef"], int(x["len_t"]), sig, np.ascontiguousarray(h8["v"][0]),
                               len(x["coef"]), int(x["M2"]))
    assert np.max(np.abs(sig - x["sigma"])) <= REL * np.max(np.abs(x["sigma"]))


def test_host_entry_point_reuses_its_operator_across_calls(cuda_lib):
    """rec_A_tab keeps one operator's device arrays between calls of the same shape and reloads
    the values every call: consecutive calls with different operators of one shape (real, then
    complex hoppings, then real again, then the same values twice), a call of another shape, and
    a call after kpm_host_cache_release each match the oracle; rec_A_tab_2 shares the cache."""
    from minijclsquant_gb300 import lattice, obv_gpu
    from minijclsquant_gb300.modifiers import modifier_bounds
    from minijclsquant_gb300.observables import random_vector_generator

    def op(nx, ny, seed, phase):
        arr = lattice.honeycomb_arrays(nx, ny, t=-2.7, W=0.7, seed=seed)
        if phase:
            ph = np.exp(1j * phase * np.real(arr["dx"]) / 0.142)
            arr = dict(arr, data=np.where(np.real(arr["dx"]) != 0, arr["data"] * ph, arr["data"]))
        from minijclsquant_gb300.ell_matrix import ell_matrix

        return ell_matrix(lattice.to_csr(arr)).modifier(modifier_bounds)

    M = 80
    cases = [op(24, 20, 1, 0.0), op(24, 20, 2, 0.3), op(24, 20, 3, 0.0), op(24, 20, 3, 0.0), op(30, 18, 4, 0.2)]
    for k, Hk in enumerate(cases + cases[:2]):
        if k == len(cases):
            assert cuda_lib.kpm_host_cache_release() == 0
        n = Hk.data.size // Hk.len_row
        v = random_vector_generator(n, 600 + k)
        out = np.zeros(M, dtype=np.complex128)
        data = np.ascontiguousarray(Hk.data, dtype=np.complex128)
        idx = np.ascontiguousarray(Hk.indices, dtype=np.int32)
        obv_gpu.rec_A_tab_gpu(data, idx, Hk.len_row, v, out, M)
        ref = oracle.rec_A_tab(M, Hk.data, Hk.indices, Hk.len_row, v)
        assert oracle.moment_tolerance_ok(out, ref, REL)[0], k
        vl = random_vector_generator(n, 700 + k)
        out2 = np.zeros(M, dtype=np.complex128)
        obv_gpu.rec_A_tab_2_gpu(data, idx, Hk.len_row, vl, v, out2, M)
        ref2 = oracle.rec_A_tab2v(M, Hk.data, Hk.indices, Hk.len_row, vl, v)
        assert oracle.moment_tolerance_ok(out2, ref2, REL)[0], k
    assert cuda_lib.kpm_host_cache_release() == 0


def test_ell_dot_matches_oracle(cuda_lib):
    from minijclsquant_gb300.ell_matrix import ell_matrix

    z = golden("complex_open_6x5")
    L = int(z["len_row"])
    H = ell_matrix.from_ell(z["data"], z["indices"], L, bounds=z["bounds"])
    rng = np.random.default_rng(1)
    n = int(z["n"])
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    y0 = rng.normal(size=n) + 1j * rng.normal(size=n)
    for a, b in [(1, 0), (2, -1), (0.3 - 1.2j, 0.5 + 0.25j)]:
        y = y0.copy()
        H.dot(a, b, x, y)
        yr = y0.copy()
        oracle.aAxby(a, b, x, yr, z["data"], z["indices"], L)
        assert np.max(np.abs(y - yr)) <= 1e-13 * np.max(np.abs(yr))


def test_tiny_and_short(cuda_lib):
    from minijclsquant_gb300.ell_matrix import ell_matrix
    from minijclsquant_gb300.recurrence_functions import rec_A_tab

    z = golden("tiny_2x2")
    Hk = ell_matrix.from_ell(z["data_kpm"], z["indices"], int(z["len_row"]), bounds=z["bounds"])
    assert np.allclose(rec_A_tab(2, Hk, z["v"]), z["mu2"], rtol=1e-12, atol=1e-13)
    assert np.allclose(rec_A_tab(3, Hk, z["v"]), z["mu3"], rtol=1e-12, atol=1e-13)
    with pytest.raises(IndexError):
        rec_A_tab(1, Hk, z["v"])


def test_long_recursion_crosses_moment_chunks(cuda_lib):
    """M well above the 128-step partial-sum chunk, against the oracle."""
    from minijclsquant_gb300 import device

    z = golden("ref_graphene_256")
    op = device.DeviceELL(z["data_kpm"], z["indices"], int(z["len_row"]))
    for M in (128, 129, 130, 300):
        mu = device.cheb_moments(op, M, z["v"][0])
        ref = oracle.rec_A_tab(M, z["data_kpm"], z["indices"], int(z["len_row"]), z["v"][0])
        assert oracle.moment_tolerance_ok(mu, ref, REL)[0], M


@pytest.mark.parametrize("doubled", [False, True])
@pytest.mark.parametrize("kernel", ["simple", "staged1", "staged2", "ws1", "ws2", "ws1s2"])
@pytest.mark.parametrize("dtype,R", [("c128", 8), ("c128", 1), ("c128", 4), ("c64", 2), ("c64", 8), ("c64", 1)])
def test_every_step_kernel_variant(cuda_lib, monkeypatch, kernel, dtype, R, doubled):
    """Each recursion-step kernel the autotuner can pick, forced, against the oracle
    (complex128 at 1e-10; complex64 at its own precision), for the direct recursion
    and for doubled moments (which the staged kernels do not serve)."""
    if doubled and kernel.startswith("staged"):
        pytest.skip("doubled moments run on the grid-stride and producer-warp kernels")
    if kernel == "ws1s2" and dtype == "c64":
        pytest.skip("two sub-tiles per stage is a complex128 form")
    from minijclsquant_gb300 import _capi, device, lattice
    from minijclsquant_gb300.modifiers import modifier_bounds
    from minijclsquant_gb300.observables import random_vector_generator

    monkeypatch.setenv("KPM_STEP_KERNEL", kernel)
    H = lattice.honeycomb(40, 36, t=-2.7, W=0.7, seed=5)  # 2880 sites: several tiles, ragged last CTA
    Hk = H.modifier(modifier_bounds)
    op = device.DeviceELL(Hk.data, Hk.indices, Hk.len_row, doubling=doubled)
    assert op.doubling == doubled
    n = op.n
    vs = np.stack([random_vector_generator(n, 40 + r) for r in range(R)])
    mu = device.cheb_moments(op, 150, vs, dtype=dtype)
    kind, U = ctypes.c_int(), ctypes.c_int()
    code = _capi.KPM_C128 if dtype == "c128" else _capi.KPM_C64
    assert cuda_lib.kpm_ell_step_config(op.handle, code, R, ctypes.byref(kind), ctypes.byref(U), None, None) == 0
    assert (kind.value, U.value) == {"simple": (0, 1), "staged1": (1, 1), "staged2": (1, 2), "ws1": (2, 1),
                                     "ws2": (2, 2), "ws1s2": (3, 1)}[kernel]
    assert cuda_lib.kpm_ell_check(op.handle, None) == 0
    for r in range(R):
        ref = oracle.rec_A_tab(150, Hk.data, Hk.indices, Hk.len_row, vs[r])
        if dtype == "c128":
            ok, err = oracle.moment_tolerance_ok(mu[r], ref, REL)
            assert ok, (kernel, r, err)
        else:
            assert np.max(np.abs(mu[r] - ref)) / n < 2e-6, (kernel, r)


def test_larger_lattice_against_oracle(cuda_lib):
    """256 x 256 cells (131k sites), M = 160, R = 2: GPU vs oracle; properties at this size."""
    from minijclsquant_gb300 import device, lattice
    from minijclsquant_gb300.modifiers import modifier_bounds
    from minijclsquant_gb300.observables import random_vector_generator

    H = lattice.honeycomb(256, 256, t=-2.7, W=1.0, seed=7)
    Hk = H.modifier(modifier_bounds)
    n = H.shape[0]
    vs = np.stack([random_vector_generator(n, 100 + r) for r in range(2)])
    mu = device.cheb_moments(Hk.device(), 160, vs)
    for r in range(2):
        ref = oracle.rec_A_tab(160, Hk.data, Hk.indices, Hk.len_row, vs[r])
        ok, err = oracle.moment_tolerance_ok(mu[r], ref, REL)
        assert ok, err
    # mu_0 = N for unit-modulus vectors; Hermitian H gives real moments
    assert np.allclose(mu[:, 0], n, rtol=1e-13)
    assert np.max(np.abs(mu.imag)) <= 1e-9 * n


def test_linearity_in_the_left_vector(cuda_lib):
    from minijclsquant_gb300 import device

    z = golden("irregular_300")
    op = device.DeviceELL(z["data_kpm"], z["indices"], int(z["len_row"]))
    v = z["v"][0]
    a = 0.7 - 0.4j
    m1 = device.cheb_moments(op, 50, v, v_l=v)
    m2 = device.cheb_moments(op, 50, v, v_l=a * v)
    assert np.max(np.abs(m2 - np.conj(a) * m1)) <= 1e-12 * np.max(np.abs(m1))


@pytest.mark.parametrize("case", ["honeycomb_64x64"])
def test_complex64_error_against_complex128(cuda_lib, case):
    """Mixed precision: complex64 recursion, FP64 accumulation.  Per-order moment error
    (relative to mu_0) and the DOS error against the complex128 reference."""
    from minijclsquant_gb300 import device, lattice
    from minijclsquant_gb300.ell_matrix import ell_matrix
    from minijclsquant_gb300.modifiers import modifier_bounds
    from minijclsquant_gb300.observables import dos_from_moments, random_vector_generator

    z = golden(case)
    H = ell_matrix(lattice.to_csr(lattice.honeycomb_arrays(64, 64, t=-2.7, W=0.5, seed=1234)))
    Hk = H.modifier(modifier_bounds)
    vs = np.stack([random_vector_generator(8192, int(s)) for s in z["seeds"]])
    mu64 = device.cheb_moments(Hk.device(), 512, vs, dtype="c64")
    err_mom = np.max(np.abs(mu64 - z["mu"])) / 8192
    d64 = dos_from_moments(mu64, z["bounds"], 512)
    d128 = dos_from_moments(z["mu"], z["bounds"], 512)
    err_dos = np.max(np.abs(d64[:, 1] - d128[:, 1])) / np.max(np.abs(d128[:, 1]))
    print("c64 max|dmu|/mu0 = %.3e  DOS error = %.3e" % (err_mom, err_dos))
    assert err_mom < 1e-6
    assert err_dos < 1e-6


def test_bad_column_index_is_rejected(cuda_lib):
    from minijclsquant_gb300 import _capi, device

    z = golden("tiny_2x2")
    bad = z["indices"].copy()
    bad[3] = 8  # == n: out of range
    with pytest.raises(_capi.KPMError) as e:
        device.DeviceELL(z["data_kpm"], bad, int(z["len_row"]))
    assert e.value.status == _capi.KPM_ERR_INDEX
    bad[3] = -1
    with pytest.raises(_capi.KPMError) as e:
        device.DeviceELL(z["data_kpm"], bad, int(z["len_row"]))
    assert e.value.status == _capi.KPM_ERR_INDEX


def test_invalid_arguments_return_status(cuda_lib):
    from minijclsquant_gb300 import _capi

    z = golden("tiny_2x2")
    h = _create(cuda_lib, z["data_kpm"], z["indices"], int(z["len_row"]))
    try:
        assert cuda_lib.kpm_cheb_moments(h, 0, 1, 4, None, None, None, None, None) == _capi.KPM_ERR_INVALID_ARG
        assert cuda_lib.kpm_cheb_moments(h, 7, 1, 4, 1, None, 1, None, None) == _capi.KPM_ERR_DTYPE
        assert cuda_lib.kpm_cheb_moments(h, 0, 0, 4, 1, None, 1, None, None) == _capi.KPM_ERR_INVALID_ARG
        assert cuda_lib.kpm_cheb_series(h, 0, 1, 1, 1, 1, 1, None) == _capi.KPM_ERR_INVALID_ARG
    finally:
        cuda_lib.kpm_ell_destroy(h)
    hh = ctypes.c_void_p()
    assert cuda_lib.kpm_ell_create(ctypes.byref(hh), 0, 4, 1, 1, 0, None) == _capi.KPM_ERR_INVALID_ARG
    assert cuda_lib.kpm_ell_create(ctypes.byref(hh), 8, 4, 1, 1, 999, None) == _capi.KPM_ERR_INVALID_ARG


def test_device_tensors_zero_copy(cuda_lib):
    torch = _torch()
    from minijclsquant_gb300 import device

    z = golden("honeycomb_8x8")
    op = device.DeviceELL(_dev(z["data_kpm"]), _dev(z["indices"]), int(z["len_row"]))
    v = _dev(z["v"])
    mu = device.cheb_moments(op, int(z["M"]), v)
    assert isinstance(mu, torch.Tensor) and mu.is_cuda
    assert oracle.moment_tolerance_ok(mu.cpu().numpy(), z["mu"], REL)[0]
