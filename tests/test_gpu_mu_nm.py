"""Kubo-Greenwood moment matrix on the tensor cores.

The reference has no mu_nm (parity unpinned); the checks are an FP64
restatement: mu_nm = (1/R) sum_r <v_r| V T_n(H) V T_m(H) |v_r> from the oracle's
own complex128 SpMV (oracle.aAxby), and an FP64 numpy product for the
contraction alone.

Tolerances: the contraction (3xTF32, FP32 accumulation) within 2e-5 of max|mu|;
the full mu_nm (complex64 recursions + contraction) within 1e-4 of max|mu|.
"""
import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu


def _contract(cuda_lib, L, Rm, Nm, scale=1.0, acc=0, mu0=None):
    import torch

    from minijclsquant_gb300 import _capi

    tl = torch.from_numpy(np.ascontiguousarray(L)).cuda()
    tr = torch.from_numpy(np.ascontiguousarray(Rm)).cuda()
    mu = torch.zeros((Nm, Nm), dtype=torch.complex128, device="cuda") if mu0 is None else mu0
    st = cuda_lib.kpm_mu_contract(tl.data_ptr(), tr.data_ptr(), L.shape[1], L.shape[1], Nm, scale, acc,
                                  mu.data_ptr(), None)
    assert st == 0, _capi.lib().kpm_strerror(st)
    return mu


@pytest.mark.parametrize("nvec,Nm", [(8, 256), (4096, 256), (70000, 200)])
def test_tensor_core_contraction_matches_fp64(cuda_lib, nvec, Nm):
    rng = np.random.default_rng(nvec)
    L = rng.normal(size=(256, 2 * nvec)).astype(np.float32)
    Rm = rng.normal(size=(256, 2 * nvec)).astype(np.float32)
    mu = _contract(cuda_lib, L, Rm, Nm).cpu().numpy()
    Lc = L[:Nm, 0::2].astype(np.float64) + 1j * L[:Nm, 1::2]
    Rc = Rm[:Nm, 0::2].astype(np.float64) + 1j * Rm[:Nm, 1::2]
    ref = np.conj(Lc) @ Rc.T
    err = np.max(np.abs(mu - ref)) / np.max(np.abs(ref))
    assert err < 2e-5, err


def test_contraction_accumulates_and_scales(cuda_lib):
    rng = np.random.default_rng(1)
    L = rng.normal(size=(256, 64)).astype(np.float32)
    Rm = rng.normal(size=(256, 64)).astype(np.float32)
    a = _contract(cuda_lib, L, Rm, 256, scale=0.5)
    b = _contract(cuda_lib, L, Rm, 256, scale=0.25, acc=1, mu0=a.clone())
    assert np.allclose(b.cpu().numpy(), 0.75 / 0.5 * a.cpu().numpy(), rtol=1e-12, atol=1e-12)


def _oracle_mu_nm(Hd, Vd, idx, L, vs, Nm):
    """FP64: L_n = T_n(H) V v, R_m = V T_m(H) v, mu = (1/R) sum_r L^H R."""
    n = vs.shape[1]
    mu = np.zeros((Nm, Nm), dtype=np.complex128)
    for v in vs:
        w = np.zeros(n, np.complex128)
        oracle.aAxby(1, 0, v, w, Vd, idx, L)
        Ls = [w.copy()]
        t = np.zeros(n, np.complex128)
        oracle.aAxby(1, 0, w, t, Hd, idx, L)
        Ls.append(t.copy())
        while len(Ls) < Nm:
            nxt = Ls[-2].copy()
            oracle.aAxby(2, -1, Ls[-1], nxt, Hd, idx, L)
            Ls.append(nxt)
        Ts = [v.copy()]
        t = np.zeros(n, np.complex128)
        oracle.aAxby(1, 0, v, t, Hd, idx, L)
        Ts.append(t)
        while len(Ts) < Nm:
            nxt = Ts[-2].copy()
            oracle.aAxby(2, -1, Ts[-1], nxt, Hd, idx, L)
            Ts.append(nxt)
        Rs = []
        for t in Ts:
            r = np.zeros(n, np.complex128)
            oracle.aAxby(1, 0, t, r, Vd, idx, L)
            Rs.append(r)
        mu += np.conj(np.array(Ls[:Nm])) @ np.array(Rs).T
    return mu / len(vs)


@pytest.mark.parametrize("Nm,R", [(64, 2), (256, 1)])
def test_mu_nm_matches_fp64_restatement(cuda_lib, Nm, R):
    import torch

    from minijclsquant_gb300 import device, lattice
    from minijclsquant_gb300.modifiers import modifier_bounds, modifier_velocity
    from minijclsquant_gb300.observables import random_vector_generator

    H = lattice.honeycomb(20, 18, t=-2.7, W=1.0, seed=4)
    Hk = H.modifier(modifier_bounds)
    Vx = H.modifier(modifier_velocity, "x")
    Vk = Vx.data / H.bounds[1]  # rescaled velocity, Hermitian
    n = H.shape[0]
    vs = np.stack([random_vector_generator(n, 50 + r) for r in range(R)])
    hop = device.DeviceELL(Hk.data, Hk.indices, Hk.len_row)
    vop = device.DeviceELL(Vk, Hk.indices, Hk.len_row)
    tv = torch.from_numpy(vs).cuda()
    mu = torch.empty((Nm, Nm), dtype=torch.complex128, device="cuda")
    from minijclsquant_gb300 import _capi

    st = cuda_lib.kpm_mu_nm(hop.handle, vop.handle, R, Nm, tv.data_ptr(), mu.data_ptr(), None)
    assert st == 0, _capi.lib().kpm_strerror(st)
    assert cuda_lib.kpm_ell_check(hop.handle, None) == 0
    ref = _oracle_mu_nm(Hk.data, Vk, Hk.indices, Hk.len_row, vs, Nm)
    err = np.max(np.abs(mu.cpu().numpy() - ref)) / np.max(np.abs(ref))
    assert err < 1e-4, err


@pytest.mark.parametrize("R", [1, 2, 4, 5])
def test_fused_velocity_step_matches_separate_products(cuda_lib, monkeypatch, R):
    """V T_m computed inside the H step (V with H's columns) against the separate V product,
    for every vector-group width; and a V with other columns takes the separate path."""
    import torch

    from minijclsquant_gb300 import _capi, device, lattice
    from minijclsquant_gb300.modifiers import modifier_bounds, modifier_velocity
    from minijclsquant_gb300.observables import random_vector_generator

    H = lattice.honeycomb(40, 30, t=-2.7, W=1.0, seed=8)
    Hk = H.modifier(modifier_bounds)
    Vk = H.modifier(modifier_velocity, "y").data / H.bounds[1]
    n = H.shape[0]
    Nm = 96
    vs = torch.from_numpy(np.stack([random_vector_generator(n, 70 + r) for r in range(R)])).cuda()

    def run(unfused):
        if unfused:
            monkeypatch.setenv("KPM_MU_NM_UNFUSED", "1")
        else:
            monkeypatch.delenv("KPM_MU_NM_UNFUSED", raising=False)
        hop = device.DeviceELL(Hk.data, Hk.indices, Hk.len_row)
        vop = device.DeviceELL(Vk, Hk.indices, Hk.len_row)
        mu = torch.empty((Nm, Nm), dtype=torch.complex128, device="cuda")
        st = cuda_lib.kpm_mu_nm(hop.handle, vop.handle, R, Nm, vs.data_ptr(), mu.data_ptr(), None)
        assert st == 0, _capi.lib().kpm_strerror(st)
        assert cuda_lib.kpm_ell_check(hop.handle, None) == 0
        return mu.cpu().numpy()

    fused, separate = run(False), run(True)
    assert np.max(np.abs(fused - separate)) <= 1e-6 * np.max(np.abs(separate))
    # a velocity operator with its own (permuted) column order: same matrix, separate products
    L = Hk.len_row
    perm = np.arange(L)[::-1]
    Vp = Vk.reshape(n, L)[:, perm].reshape(-1)
    Ip = Hk.indices.reshape(n, L)[:, perm].reshape(-1)
    hop = device.DeviceELL(Hk.data, Hk.indices, L)
    vop = device.DeviceELL(Vp, Ip, L)
    mu = torch.empty((Nm, Nm), dtype=torch.complex128, device="cuda")
    monkeypatch.delenv("KPM_MU_NM_UNFUSED", raising=False)
    assert cuda_lib.kpm_mu_nm(hop.handle, vop.handle, R, Nm, vs.data_ptr(), mu.data_ptr(), None) == 0
    assert np.max(np.abs(mu.cpu().numpy() - separate)) <= 1e-5 * np.max(np.abs(separate))


VARIANTS = {"legacy": 2, "tma": 3, "legacy_plain": 0, "tma_plain": 1}  # kpm_mu_gemm_path: TMA bit, swizzle bit


@pytest.mark.parametrize("nvec,Nm", [(8, 256), (4096, 64), (70000, 200), (300000, 256)])
def test_contraction_variants_agree_bit_for_bit(cuda_lib, monkeypatch, nvec, Nm):
    """The four forms of the contraction kernel -- operand tiles loaded by the threads or by the
    TMA engine, in the 64-byte-swizzled or the no-swizzle layout -- run the same MMAs on the
    same values in the same order, so their moment matrices agree bit for bit; the default is
    the TMA engine's loads into the no-swizzle layout.  Each matches an FP64 product at 2e-5."""
    rng = np.random.default_rng(nvec + Nm)
    L = rng.normal(size=(256, 2 * nvec)).astype(np.float32)
    Rm = rng.normal(size=(256, 2 * nvec)).astype(np.float32)
    mu_default = _contract(cuda_lib, L, Rm, Nm).cpu().numpy()
    assert cuda_lib.kpm_mu_gemm_path() == VARIANTS["tma_plain"]
    for name, path in VARIANTS.items():
        monkeypatch.setenv("KPM_MU_GEMM", name)
        mu = _contract(cuda_lib, L, Rm, Nm).cpu().numpy()
        assert cuda_lib.kpm_mu_gemm_path() == path, name
        assert np.array_equal(mu, mu_default), name
    monkeypatch.delenv("KPM_MU_GEMM")
    Lc = L[:Nm, 0::2].astype(np.float64) + 1j * L[:Nm, 1::2]
    Rc = Rm[:Nm, 0::2].astype(np.float64) + 1j * Rm[:Nm, 1::2]
    ref = np.conj(Lc) @ Rc.T
    assert np.max(np.abs(mu_default - ref)) / np.max(np.abs(ref)) < 2e-5
