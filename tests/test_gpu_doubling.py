"""Doubled DOS moments (opt-in, Hermitian operators): mu_{2k} = 2 sum (|t_k|^2 - |v|^2/2),
mu_{2k+1} = 2 <t_{k+1}|t_k> - mu_1, ceil(M/2) - 1 recursion steps.

Checked against the oracle (the reference's recursion, M - 2 steps) at the
drop-in tolerance, per order m:  |mu_m - ref_m| <= 1e-10 * max(|ref_m|, 1e-6 |ref_0|),
and against the direct recursion on the same handle.  The reference's own
H_graphene is not Hermitian (a 1e-6 asymmetric term) and must keep the direct
recursion."""
import numpy as np
import pytest

from conftest import golden
from oracle import oracle

pytestmark = pytest.mark.gpu

REL = 1e-10


def _vectors(n, R, seed0):
    from minijclsquant_gb300.observables import random_vector_generator

    return np.stack([random_vector_generator(n, seed0 + r) for r in range(R)])


@pytest.mark.parametrize("case,hermitian", [("honeycomb_8x8", True), ("ref_graphene_256", False),
                                            ("complex_open_6x5", True), ("irregular_300", True)])
def test_hermitian_detection(cuda_lib, case, hermitian):
    from minijclsquant_gb300 import device

    z = golden(case)
    op = device.DeviceELL(z["data_kpm"], z["indices"], int(z["len_row"]), doubling=True)
    assert op.hermitian == hermitian
    assert op.doubling == hermitian
    plain = device.DeviceELL(z["data_kpm"], z["indices"], int(z["len_row"]))
    assert plain.hermitian == hermitian and not plain.doubling  # opt-in


def test_one_asymmetric_entry_disables_doubling(cuda_lib):
    from minijclsquant_gb300 import device

    z = golden("honeycomb_8x8")
    data = np.array(z["data_kpm"], copy=True)
    L = int(z["len_row"])
    rows = np.arange(data.size) // L
    off_diag = np.flatnonzero((data != 0) & (np.asarray(z["indices"]) != rows))
    k = int(off_diag[5])
    data[k] = data[k] * (1 + 2.0 ** -40)  # one hopping off by a few ulp; its transpose unchanged
    op = device.DeviceELL(data, z["indices"], int(z["len_row"]), doubling=True)
    assert not op.hermitian and not op.doubling


@pytest.mark.parametrize("M", [4, 5, 6, 7, 64, 129, 300])
@pytest.mark.parametrize("case", ["honeycomb_8x8", "complex_open_6x5", "irregular_300"])
def test_doubled_moments_match_oracle_and_direct(cuda_lib, case, M):
    from minijclsquant_gb300 import device

    z = golden(case)
    data, idx, L = z["data_kpm"], z["indices"], int(z["len_row"])
    n = data.size // L
    vs = _vectors(n, 3, 70)
    op = device.DeviceELL(data, idx, L, doubling=True)
    assert op.doubling
    mu = device.cheb_moments(op, M, vs)
    for r in range(3):
        ref = oracle.rec_A_tab(M, data, idx, L, vs[r], threads=1)
        ok, err = oracle.moment_tolerance_ok(mu[r], ref, REL)
        assert ok, (case, M, r, err)
    op.set_doubling(False)
    mu_d = device.cheb_moments(op, M, vs)
    assert np.max(np.abs(mu - mu_d)) <= 1e-12 * np.max(np.abs(mu_d[:, 0]))


def test_non_hermitian_reference_graphene_keeps_direct_parity(cuda_lib):
    from minijclsquant_gb300 import device

    z = golden("ref_graphene_256")
    op = device.DeviceELL(z["data_kpm"], z["indices"], int(z["len_row"]), doubling=True)
    assert not op.doubling  # requested, but H is not Hermitian
    M = int(z["M"])
    mu = device.cheb_moments(op, M, z["v"][0])
    ok, err = oracle.moment_tolerance_ok(mu, z["mu"][0], REL)
    assert ok, err


def test_doubled_complex64_against_oracle(cuda_lib):
    from minijclsquant_gb300 import device, lattice
    from minijclsquant_gb300.modifiers import modifier_bounds

    H = lattice.honeycomb(40, 36, t=-2.7, W=0.7, seed=5)
    Hk = H.modifier(modifier_bounds)
    op = device.DeviceELL(Hk.data, Hk.indices, Hk.len_row, doubling=True)
    assert op.doubling
    n = op.n
    vs = _vectors(n, 2, 90)
    for M in (150, 151):
        mu = device.cheb_moments(op, M, vs, dtype="c64")
        for r in range(2):
            ref = oracle.rec_A_tab(M, Hk.data, Hk.indices, Hk.len_row, vs[r])
            assert np.max(np.abs(mu[r] - ref)) / n < 2e-6, (M, r)


def test_doubled_dos_equals_direct_dos(cuda_lib):
    """The reconstructed DOS of the drop-in API is the same with and without doubling."""
    from minijclsquant_gb300 import device, lattice
    from minijclsquant_gb300.modifiers import modifier_bounds
    from minijclsquant_gb300.observables import dos_from_moments

    H = lattice.honeycomb(48, 48, t=-2.7, W=1.0, seed=8)
    Hk = H.modifier(modifier_bounds)
    vs = _vectors(H.shape[0], 4, 300)
    a = device.DeviceELL(Hk.data, Hk.indices, Hk.len_row, doubling=True)
    b = device.DeviceELL(Hk.data, Hk.indices, Hk.len_row)
    M = 512
    da = dos_from_moments(device.cheb_moments(a, M, vs), H.bounds, M)
    db = dos_from_moments(device.cheb_moments(b, M, vs), H.bounds, M)
    assert np.max(np.abs(da[:, 1] - db[:, 1])) <= 1e-10 * np.max(np.abs(db[:, 1]))


def test_batched_doubling_flag_and_parity(cuda_lib):
    from minijclsquant_gb300 import batched

    datas, idxs, L, _, _ = batched.honeycomb_ensemble(5, side_range=(3, 40), W_range=(0.0, 2.0), seed=21)
    B = batched.BatchedELL(datas, idxs, L)
    assert B.hermitian and not B.doubling  # opt-in
    B.set_doubling(True)
    assert B.doubling
    v = batched.ensemble_vectors(B.rows, 2)
    for M in (6, 7, 120):
        mu = B.moments(M, v, dtype="c128")
        for k in range(5):
            o, n = int(B.offsets[k]), int(B.rows[k])
            for r in range(2):
                ref = oracle.rec_A_tab(M, datas[k], idxs[k], L, v[r, o:o + n])
                ok, err = oracle.moment_tolerance_ok(mu[k, r], ref, REL)
                assert ok, (M, k, r, err)
    B.set_doubling(False)
    assert not B.doubling
    mu_d = B.moments(120, v, dtype="c128")
    B.set_doubling(True)
    mu2 = B.moments(120, v, dtype="c128")
    assert np.max(np.abs(mu2 - mu_d)) <= 1e-12 * np.max(np.abs(mu_d[:, :, 0]))
