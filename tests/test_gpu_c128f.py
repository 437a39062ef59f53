"""KPM_C128F: complex128 moments in float-float arithmetic (FP32 pipe), held to the
drop-in tolerance against the reference's golden vectors and the oracle, per order m:
    |mu_m - ref_m| <= 1e-10 * max(|ref_m|, 1e-6 * |ref_0|)."""
import numpy as np
import pytest

from conftest import golden
from oracle import oracle

pytestmark = pytest.mark.gpu

REL = 1e-10
CASES = ["honeycomb_8x8", "ref_graphene_256", "complex_open_6x5", "irregular_300"]


@pytest.mark.parametrize("case", CASES)
def test_c128f_matches_reference_golden(cuda_lib, case):
    from minijclsquant_gb300 import device

    z = golden(case)
    op = device.DeviceELL(z["data_kpm"], z["indices"], int(z["len_row"]))
    mu = device.cheb_moments(op, int(z["M"]), z["v"], dtype="c128f")
    ok, err = oracle.moment_tolerance_ok(mu, z["mu"], REL)
    assert ok, err


@pytest.mark.parametrize("R", [1, 2, 3, 4, 8])
@pytest.mark.parametrize("M", [1, 2, 3, 150, 300])
def test_c128f_vector_groups_and_lengths(cuda_lib, R, M):
    from minijclsquant_gb300 import device, lattice
    from minijclsquant_gb300.modifiers import modifier_bounds
    from minijclsquant_gb300.observables import random_vector_generator

    H = lattice.honeycomb(40, 36, t=-2.7, W=0.7, seed=5)
    Hk = H.modifier(modifier_bounds)
    op = device.DeviceELL(Hk.data, Hk.indices, Hk.len_row)
    vs = np.stack([random_vector_generator(op.n, 40 + r) for r in range(R)])
    mu = device.cheb_moments(op, M, vs, dtype="c128f")
    assert mu.shape == (R, M)
    for r in range(R):
        ref = oracle.rec_A_tab(max(M, 2), Hk.data, Hk.indices, Hk.len_row, vs[r])[:M]
        ok, err = oracle.moment_tolerance_ok(mu[r], ref, REL)
        assert ok, (R, M, r, err)


def test_c128f_two_vector_moments(cuda_lib):
    from minijclsquant_gb300 import device

    z = golden("complex_open_6x5")
    data, idx, L = z["data_kpm"], z["indices"], int(z["len_row"])
    n = data.size // L
    rng = np.random.default_rng(3)
    vl = np.exp(2j * np.pi * rng.random((2, n)))
    vr = np.exp(2j * np.pi * rng.random((2, n)))
    op = device.DeviceELL(data, idx, L)
    mu = device.cheb_moments(op, 200, vr, vl, dtype="c128f")
    for r in range(2):
        ref = oracle.rec_A_tab2v(200, data, idx, L, vl[r], vr[r])
        ok, err = oracle.moment_tolerance_ok(mu[r], ref, REL)
        assert ok, (r, err)


def test_c128f_larger_lattice_and_agreement_with_c128(cuda_lib):
    from minijclsquant_gb300 import device, lattice
    from minijclsquant_gb300.modifiers import modifier_bounds
    from minijclsquant_gb300.observables import random_vector_generator

    H = lattice.honeycomb(256, 256, t=-2.7, W=1.0, seed=7)
    Hk = H.modifier(modifier_bounds)
    op = device.DeviceELL(Hk.data, Hk.indices, Hk.len_row)
    vs = np.stack([random_vector_generator(op.n, 900 + r) for r in range(2)])
    M = 400
    mf = device.cheb_moments(op, M, vs, dtype="c128f")
    md = device.cheb_moments(op, M, vs, dtype="c128")
    ref = oracle.rec_A_tab(M, Hk.data, Hk.indices, Hk.len_row, vs[0])
    ok, err = oracle.moment_tolerance_ok(mf[0], ref, REL)
    assert ok, err
    assert np.max(np.abs(mf - md)) <= 1e-12 * np.max(np.abs(md[:, 0]))


def test_c128f_rejects_second_moment_set(cuda_lib):
    import ctypes

    import torch

    from minijclsquant_gb300 import _capi, device

    z = golden("honeycomb_8x8")
    op = device.DeviceELL(z["data_kpm"], z["indices"], int(z["len_row"]))
    v = torch.from_numpy(np.ascontiguousarray(z["v"])).cuda()
    R, M = v.shape[0], 16
    mu = torch.empty((R, M), dtype=torch.complex128, device="cuda")
    mu2 = torch.empty((R, M), dtype=torch.complex128, device="cuda")
    st = cuda_lib.kpm_cheb_moments(op.handle, _capi.KPM_C128F, R, M, v.data_ptr(), None, mu.data_ptr(),
                                   mu2.data_ptr(), None)
    assert st == _capi.KPM_ERR_UNSUPPORTED
    assert isinstance(ctypes.c_int(st).value, int)
