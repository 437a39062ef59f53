"""GPU parity of the drop-in entry points that build on the recursion, against the
reference's own outputs (golden fixtures made by tests/golden/make_golden.py):

* rec_com_A_vec_tab (jclsquant/recurrence_functions.py:202-250), the [M, N] table of
  the commutator series, through the drop-in and through the C ABI;
* kpm_n_dos_n (jclsquant/observables.py:59-120) and kpm_dos_2_gpu
  (jclsquant/observables_gpu.py:46-93) with and without a projector on the bra vector,
  and with bounds=False (an operator rescaled by the caller).

Tolerance (complex128): max|diff| <= 1e-10 * max|ref| for tables and DOS curves; the
energy columns are bit-identical.
"""
import ctypes

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu
REL = 1e-10


def _ops(z):
    from minijclsquant_gb300.ell_matrix import ell_matrix

    L = int(z["len_row"])
    Hk = ell_matrix.from_ell(z["data_kpm"], z["indices"], L)
    V = ell_matrix.from_ell(z["v_data"], z["indices"], L)
    return Hk, V


def test_commutator_table_dropin_matches_reference(cuda_lib):
    from minijclsquant_gb300.recurrence_functions import rec_com_A_vec, rec_com_A_vec_tab

    z = golden("commutator_table_5x4")
    Hk, V = _ops(z)
    M = int(z["M"])
    tab = rec_com_A_vec_tab(M, Hk, V, z["coef"], z["v"])
    assert isinstance(tab, np.ndarray) and tab.shape == z["tab"].shape and tab.dtype == np.complex128
    assert np.all(tab[0] == 0)
    assert np.max(np.abs(tab - z["tab"])) <= REL * np.max(np.abs(z["tab"]))
    # the rows of the table sum to the series
    assert np.max(np.abs(tab.sum(axis=0) - z["series"])) <= REL * np.max(np.abs(z["series"]))
    ser = rec_com_A_vec(M, Hk, V, z["coef"], z["v"])
    assert np.max(np.abs(ser - z["series"])) <= REL * np.max(np.abs(z["series"]))


@pytest.mark.parametrize("R", [1, 3, 8])
def test_commutator_table_cabi_vector_sets(cuda_lib, R):
    """R vectors in one call: each [M, n] block equals the table of that vector alone
    (computed by the oracle's restatement of the reference recursion)."""
    import torch

    from minijclsquant_gb300 import _capi
    from oracle import oracle

    z = golden("commutator_table_5x4")
    L, n, M = int(z["len_row"]), int(z["n"]), int(z["M"])
    rng = np.random.default_rng(40 + R)
    vs = np.exp(1j * rng.uniform(0, 2 * np.pi, (R, n)))
    vs[0] = z["v"]
    hs = []
    for data in (z["data_kpm"], z["v_data"]):
        d = np.ascontiguousarray(data)
        ix = np.ascontiguousarray(z["indices"], dtype=np.int32)
        h = ctypes.c_void_p()
        assert cuda_lib.kpm_ell_create(ctypes.byref(h), n, L, d.ctypes.data, ix.ctypes.data, 0, None) == 0
        hs.append(h)
    try:
        tv = torch.from_numpy(vs).cuda()
        tc = torch.from_numpy(z["coef"]).cuda()
        tab = torch.full((R, M, n), complex(7.0, 7.0), dtype=torch.complex128, device="cuda")
        st = cuda_lib.kpm_cheb_commutator_table(hs[0], hs[1], _capi.KPM_C128, R, M, tc.data_ptr(), tv.data_ptr(),
                                                tab.data_ptr(), None)
        assert st == 0
        got = tab.cpu().numpy()
        assert np.max(np.abs(got[0] - z["tab"])) <= REL * np.max(np.abs(z["tab"]))
        for r in range(R):
            ref = oracle.rec_com_A_vec_tab(M, z["data_kpm"], z["v_data"], z["indices"], L, z["coef"], vs[r])
            assert np.max(np.abs(got[r] - ref)) <= REL * np.max(np.abs(ref)), r
        # unsupported precision and bad sizes are refused
        assert cuda_lib.kpm_cheb_commutator_table(hs[0], hs[1], _capi.KPM_C64, R, M, tc.data_ptr(), tv.data_ptr(),
                                                  tab.data_ptr(), None) == _capi.KPM_ERR_UNSUPPORTED
        assert cuda_lib.kpm_cheb_commutator_table(hs[0], hs[1], _capi.KPM_C128, R, 1, tc.data_ptr(), tv.data_ptr(),
                                                  tab.data_ptr(), None) == _capi.KPM_ERR_INVALID_ARG
    finally:
        for h in hs:
            cuda_lib.kpm_ell_destroy(h)


def test_commutator_table_missing_arguments(cuda_lib, capsys):
    from minijclsquant_gb300.recurrence_functions import rec_com_A_vec_tab

    z = golden("commutator_table_5x4")
    Hk, V = _ops(z)
    assert rec_com_A_vec_tab(8, Hk, None, z["coef"], z["v"]) is None
    assert rec_com_A_vec_tab(8, Hk, V, z["coef"], None) is None
    assert "velocity" in capsys.readouterr().out
    with pytest.raises(TypeError):
        rec_com_A_vec_tab(8, Hk, V, None, z["v"])
    with pytest.raises(IndexError):
        rec_com_A_vec_tab(1, Hk, V, z["coef"], z["v"])


def _two_vector_inputs():
    from minijclsquant_gb300.ell_matrix import ell_matrix

    z = golden("two_vector_dos_8x8")
    L = int(z["len_row"])
    H = ell_matrix.from_ell(z["data"], z["indices"], L, bounds=z["bounds"], valid_row_values=z["valid"])
    P = ell_matrix.from_ell(z["proj_data"], z["proj_indices"], int(z["proj_len_row"]))
    return z, H, P


def _same_dos(got, ref):
    assert got.shape == ref.shape
    assert np.array_equal(got[:, 0], ref[:, 0])
    assert np.max(np.abs(got[:, 1] - ref[:, 1])) <= REL * np.max(np.abs(ref[:, 1]))


@pytest.mark.parametrize("fn_name", ["kpm_n_dos_n", "kpm_dos_2_gpu"])
def test_two_vector_dos_matches_reference(cuda_lib, fn_name):
    from minijclsquant_gb300 import observables, observables_gpu
    from minijclsquant_gb300.modifiers import modifier_bounds

    fn = getattr(observables if fn_name == "kpm_n_dos_n" else observables_gpu, fn_name)
    z, H, P = _two_vector_inputs()
    M = int(z["M"])
    _same_dos(fn(H, M, z["v_l"], z["v_r"]), z["dos"])
    _same_dos(fn(H, M, z["v_l"], z["v_r"], True, P), z["dos_proj"])
    Hk = H.modifier(modifier_bounds)
    Hk.bounds = H.bounds
    _same_dos(fn(Hk, M, z["v_l"], z["v_r"], False), z["dos_nobounds"])
    # the projector changes the curve (it is applied, not ignored)
    assert np.max(np.abs(z["dos_proj"][:, 1] - z["dos"][:, 1])) > 1e-3 * np.max(np.abs(z["dos"][:, 1]))
