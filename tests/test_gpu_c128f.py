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


def test_c128f_commutator_and_time_sigma_match_reference_golden(cuda_lib):
    """The commutator series and the time-domain Kubo correlator in float-float arithmetic
    against the reference's own outputs (rec_com_A_vec and the kpm_sigma_time loop)."""
    from minijclsquant_gb300 import device

    z = golden("honeycomb_8x8")
    x = golden("honeycomb_8x8_more")
    L = int(z["len_row"])
    H = device.DeviceELL(z["data_kpm"], z["indices"], L)
    V2 = device.DeviceELL(x["v2_data"], z["indices"], L)
    V1 = device.DeviceELL(x["v1_data"], z["indices"], L)
    Ms = len(x["coef"])
    v = z["v"][0]
    c = device.cheb_commutator_series(H, V2, Ms, x["coef"], v, dtype="c128f")
    assert np.max(np.abs(c - x["comm"])) <= REL * np.max(np.abs(x["comm"]))
    sig = device.time_sigma(H, V1, V2, x["cu"], int(x["M2"]), x["coef"], Ms, int(x["len_t"]), v, dtype="c128f")
    assert np.max(np.abs(sig - x["sigma"])) <= REL * np.max(np.abs(x["sigma"]))


@pytest.mark.parametrize("R", [1, 2, 3, 5])
def test_c128f_time_sigma_groups_against_oracle_and_c128(cuda_lib, R):
    from minijclsquant_gb300 import device, lattice
    from minijclsquant_gb300.kernel_and_moments import JacksonKernel, moments_FD_T0, moments_U
    from minijclsquant_gb300.modifiers import modifier_bounds, modifier_velocity, modifier_velocity_bounds
    from minijclsquant_gb300.observables import random_vector_generator

    H = lattice.honeycomb(20, 16, t=-2.7, W=0.8, seed=R)
    Hk = H.modifier(modifier_bounds)
    v1 = modifier_velocity(H, "y")
    v2 = modifier_velocity_bounds(H, "x")
    L = Hk.len_row
    ops = [device.DeviceELL(d, Hk.indices, L) for d in (Hk.data, v1, v2)]
    M, M2, len_t = 64, 12, 5
    cu = moments_U(1.1, M2).astype(np.complex128)
    cfd = (moments_FD_T0(0.05, M) * JacksonKernel(M)).astype(np.complex128)
    vs = np.stack([random_vector_generator(ops[0].n, 60 + r) for r in range(R)])
    f = np.asarray(device.time_sigma(*ops, cu, M2, cfd, M, len_t, vs, dtype="c128f")).reshape(R, len_t)
    d = np.asarray(device.time_sigma(*ops, cu, M2, cfd, M, len_t, vs)).reshape(R, len_t)
    for r in range(R):
        ref = oracle.for_time_sigma(Hk.data, v1, v2, Hk.indices, L, cu, cfd, len_t, vs[r], M, M2)
        assert np.max(np.abs(f[r] - ref)) <= REL * np.max(np.abs(ref)), r
    assert np.max(np.abs(f - d)) <= 1e-12 * np.max(np.abs(d))


def test_c128f_commutator_complex_hoppings_larger(cuda_lib):
    from minijclsquant_gb300 import device, lattice
    from minijclsquant_gb300.ell_matrix import ell_matrix
    from minijclsquant_gb300.kernel_and_moments import JacksonKernel, moments_FD_T0
    from minijclsquant_gb300.modifiers import modifier_bounds, modifier_velocity_bounds
    from minijclsquant_gb300.observables import random_vector_generator

    arr = lattice.honeycomb_arrays(64, 48, t=-2.7, W=0.6, seed=12)
    phase = np.exp(1j * 0.3 * np.real(arr["dx"]) / 0.142)
    arr = dict(arr, data=np.where(np.real(arr["dx"]) != 0, arr["data"] * phase, arr["data"]))
    dx = lattice.to_csr(dict(arr, data=arr["dx"]))
    dy = lattice.to_csr(dict(arr, data=arr["dy"]))
    H = ell_matrix(lattice.to_csr(arr), dx, dy)
    Hk = H.modifier(modifier_bounds)
    V = modifier_velocity_bounds(H, "x")
    L = Hk.len_row
    hop = device.DeviceELL(Hk.data, Hk.indices, L)
    vop = device.DeviceELL(V, Hk.indices, L)
    M = 200
    c = (moments_FD_T0(-0.2, M) * JacksonKernel(M)).astype(np.complex128)
    vs = np.stack([random_vector_generator(hop.n, 7 + r) for r in range(4)])
    out = np.asarray(device.cheb_commutator_series(hop, vop, M, c, vs, dtype="c128f"))
    for r in range(4):
        ref = oracle.rec_com_A_vec(M, Hk.data, V, Hk.indices, L, c, vs[r])
        assert np.max(np.abs(out[r] - ref)) <= REL * np.max(np.abs(ref)), r


def test_c128f_commutator_and_time_sigma_on_reused_handles(cuda_lib):
    """Workspace reuse: the commutator recursion reads C_0 = 0 from a scratch buffer that an
    earlier call (of either precision) left filled; repeated calls on the same handles and a
    float-float call after an FP64 one return the oracle's values."""
    from minijclsquant_gb300 import device, lattice
    from minijclsquant_gb300.kernel_and_moments import JacksonKernel, moments_FD_T0, moments_U
    from minijclsquant_gb300.modifiers import modifier_bounds, modifier_velocity, modifier_velocity_bounds
    from minijclsquant_gb300.observables import random_vector_generator

    H = lattice.honeycomb(20, 16, t=-2.7, W=0.8, seed=3)
    Hk = H.modifier(modifier_bounds)
    v1, v2 = modifier_velocity(H, "y"), modifier_velocity_bounds(H, "x")
    L = Hk.len_row
    ops = [device.DeviceELL(d, Hk.indices, L) for d in (Hk.data, v1, v2)]
    M, M2, len_t = 64, 12, 4
    cu = moments_U(1.1, M2).astype(np.complex128)
    cfd = (moments_FD_T0(0.05, M) * JacksonKernel(M)).astype(np.complex128)
    vs = np.stack([random_vector_generator(ops[0].n, 60 + r) for r in range(3)])
    sig_ref = [oracle.for_time_sigma(Hk.data, v1, v2, Hk.indices, L, cu, cfd, len_t, vs[r], M, M2) for r in range(3)]
    com_ref = [oracle.rec_com_A_vec(M, Hk.data, v2, Hk.indices, L, cfd, vs[r]) for r in range(3)]
    for dtypes in (("c128", "c128f"), ("c128f", "c128f")):
        for dt in dtypes:
            s = np.asarray(device.time_sigma(*ops, cu, M2, cfd, M, len_t, vs, dtype=dt)).reshape(3, len_t)
            c = np.asarray(device.cheb_commutator_series(ops[0], ops[2], M, cfd, vs, dtype=dt))
            for r in range(3):
                assert np.max(np.abs(s[r] - sig_ref[r])) <= REL * np.max(np.abs(sig_ref[r])), (dt, r)
                assert np.max(np.abs(c[r] - com_ref[r])) <= REL * np.max(np.abs(com_ref[r])), (dt, r)


def test_kpm_sigma_time_gpu_both_precisions(cuda_lib):
    """The observable drop-in (kpm_sigma_time_gpu of jclsquant's observables_gpu): its c128
    result equals -i times the oracle's for_time_sigma on the moments it builds, and the
    float-float run agrees with it."""
    from minijclsquant_gb300 import lattice
    from minijclsquant_gb300.constants import hbar_fs
    from minijclsquant_gb300.kernel_and_moments import JacksonKernel, moments_FD_T0, moments_U
    from minijclsquant_gb300.modifiers import modifier_bounds, modifier_velocity, modifier_velocity_bounds
    from minijclsquant_gb300.observables import random_vector_generator
    from minijclsquant_gb300.observables_gpu import kpm_sigma_time_gpu

    H = lattice.honeycomb(14, 12, t=-2.7, W=0.6, seed=4)
    n = H.shape[0]
    v = random_vector_generator(n, 21)
    M, Ef = 96, 0.3
    t_vec = np.linspace(0, 4.0, 7)
    sig = kpm_sigma_time_gpu(H, "x", "y", t_vec=t_vec, Ef=Ef, M=M, random_vector=v)
    sig_f = kpm_sigma_time_gpu(H, "x", "y", t_vec=t_vec, Ef=Ef, M=M, random_vector=v, dtype="c128f")
    dt = t_vec[1] * H.bounds[1] / hbar_fs
    mu_u = moments_U(dt, M)
    M2 = 0
    while np.abs(mu_u[M2]) > 1e-15 and M2 < M - 1:
        M2 += 1
    cu = moments_U(dt, M2).astype(np.complex128)
    cfd = (moments_FD_T0(Ef / H.bounds[1], M) * JacksonKernel(M)).astype(np.complex128)
    Hk = H.modifier(modifier_bounds)
    ref = -1j * oracle.for_time_sigma(Hk.data, H.modifier(modifier_velocity, "x").data,
                                      H.modifier(modifier_velocity_bounds, "y").data, Hk.indices, Hk.len_row, cu, cfd,
                                      len(t_vec), v, M, M2)
    assert np.max(np.abs(sig - ref)) <= REL * np.max(np.abs(ref))
    assert np.max(np.abs(sig_f - sig)) <= REL * np.max(np.abs(sig))
