"""The vector-table entry points through the C ABI (kpm_cheb_table, kpm_cheb_clenshaw_table,
kpm_ell_slot_sum) against CPU restatements built on the oracle's SpMV (oracle.aAxby, the
reference's aAxby restated, jclsquant/cython_modules/blas_funs.pyx:64-71).  Complex128 at 1e-12
of the largest entry; overlapping buffers are refused."""
import ctypes

import numpy as np
import pytest

from conftest import golden
from oracle import oracle

pytestmark = pytest.mark.gpu


def _op(lib, data, idx, L):
    d = np.ascontiguousarray(data, dtype=np.complex128)
    ix = np.ascontiguousarray(idx, dtype=np.int32)
    h = ctypes.c_void_p()
    assert lib.kpm_ell_create(ctypes.byref(h), d.size // L, L, d.ctypes.data, ix.ctypes.data, 0, None) == 0
    return h


def _mv(data, idx, L, x):
    y = np.zeros_like(x)
    oracle.aAxby(1.0, 0.0, x, y, data, idx, L)
    return y


def test_tables_match_cpu_restatement(cuda_lib):
    import torch

    from minijclsquant_gb300 import _capi

    z = golden("honeycomb_8x8")
    x = golden("honeycomb_8x8_more")
    L, n = int(z["len_row"]), int(z["n"])
    Hd, Vd, idx = z["data_kpm"], x["v2_data"], z["indices"]
    h, s = _op(cuda_lib, Hd, idx, L), _op(cuda_lib, Vd, idx, L)
    try:
        M = 23
        v = z["v"][0]
        T = [v.copy(), _mv(Hd, idx, L, v)]
        while len(T) < M:
            T.append(2 * _mv(Hd, idx, L, T[-1]) - T[-2])
        T = np.stack(T)
        ST = np.stack([_mv(Vd, idx, L, t) for t in T])
        tv = torch.from_numpy(v).cuda()
        tab = torch.empty((M, n), dtype=torch.complex128, device="cuda")
        stab = torch.empty_like(tab)
        assert cuda_lib.kpm_cheb_table(h, s, M, tv.data_ptr(), tab.data_ptr(), stab.data_ptr(), None) == 0
        g, gs = tab.cpu().numpy(), stab.cpu().numpy()
        assert np.max(np.abs(g - T)) <= 1e-12 * np.max(np.abs(T))
        assert np.max(np.abs(gs - ST)) <= 1e-12 * np.max(np.abs(ST))
        # v may be row 0 of the table; tab and stab may not overlap
        tab2 = torch.zeros_like(tab)
        tab2[0] = tv
        assert cuda_lib.kpm_cheb_table(h, None, M, tab2.data_ptr(), tab2.data_ptr(), None, None) == 0
        assert torch.equal(tab2, tab)
        assert cuda_lib.kpm_cheb_table(h, s, M, tv.data_ptr(), tab.data_ptr(), tab[1:].data_ptr(), None) == \
            _capi.KPM_ERR_INVALID_ARG
        # Clenshaw: lam_k = S z_k + 2H lam_{k+1} - lam_{k+2}, lam_0 = S z_0 + H lam_1 - lam_2
        rng = np.random.default_rng(3)
        Z = rng.normal(size=(M, n)) + 1j * rng.normal(size=(M, n))
        lam = [None] * M + [np.zeros(n, complex)] * 2
        for k in range(M - 1, -1, -1):
            lam[k] = _mv(Vd, idx, L, Z[k]) + (1.0 if k == 0 else 2.0) * _mv(Hd, idx, L, lam[k + 1]) - lam[k + 2]
        lam = np.stack(lam[:M])
        tz = torch.from_numpy(Z).cuda()
        tl = torch.empty_like(tz)
        assert cuda_lib.kpm_cheb_clenshaw_table(h, s, M, tz.data_ptr(), tl.data_ptr(), None) == 0
        assert np.max(np.abs(tl.cpu().numpy() - lam)) <= 1e-12 * np.max(np.abs(lam))
        # lam_0 is the series sum_k T_k(H) S z_k
        acc = np.zeros(n, complex)
        for k in range(M):
            w = _mv(Vd, idx, L, Z[k])
            P = [w, _mv(Hd, idx, L, w)]
            while len(P) <= k:
                P.append(2 * _mv(Hd, idx, L, P[-1]) - P[-2])
            acc += P[k]
        assert np.max(np.abs(tl[0].cpu().numpy() - acc)) <= 1e-11 * np.max(np.abs(acc))
        assert cuda_lib.kpm_cheb_clenshaw_table(h, s, M, tz.data_ptr(), tz[2:].data_ptr(), None) == \
            _capi.KPM_ERR_INVALID_ARG
        # slot sums: out[i, s] = sum_k c_k conj(A_k[i]) B_k[col(i, s)]
        K = 9
        A = rng.normal(size=(K, n)) + 1j * rng.normal(size=(K, n))
        B = rng.normal(size=(K, n)) + 1j * rng.normal(size=(K, n))
        c = rng.uniform(0.5, 2.0, K)
        ref = np.zeros((n, L), complex)
        col = idx.reshape(n, L)
        for k in range(K):
            ref += c[k] * np.conj(A[k])[:, None] * B[k][col]
        out = torch.full((n * L,), 1.0 + 1.0j, dtype=torch.complex128, device="cuda")
        ta, tb, tc = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda(), torch.from_numpy(c).cuda()
        assert cuda_lib.kpm_ell_slot_sum(h, K, tc.data_ptr(), ta.data_ptr(), n, tb.data_ptr(), n, 0, out.data_ptr(),
                                         None) == 0
        assert np.max(np.abs(out.cpu().numpy().reshape(n, L) - ref)) <= 1e-12 * np.max(np.abs(ref))
        assert cuda_lib.kpm_ell_slot_sum(h, K, tc.data_ptr(), ta.data_ptr(), n, tb.data_ptr(), n, 1, out.data_ptr(),
                                         None) == 0
        assert np.max(np.abs(out.cpu().numpy().reshape(n, L) - 2 * ref)) <= 1e-12 * np.max(np.abs(ref))
    finally:
        cuda_lib.kpm_ell_destroy(h)
        cuda_lib.kpm_ell_destroy(s)
