"""Host-side logic of the drop-in modules against the reference's own outputs
(golden fixtures): ELL construction, bounds, rescaling, kernels, DOS
reconstruction, the lattice builder.  CPU only, no GPU calls."""
import numpy as np
import pytest

from conftest import golden
from minijclsquant_gb300 import kernel_and_moments as km
from minijclsquant_gb300 import lattice
from minijclsquant_gb300.ell_matrix import bounds, csr_to_ell_arrays, ell_matrix
from minijclsquant_gb300.modifiers import modifier_bounds, modifier_velocity, modifier_velocity_bounds
from minijclsquant_gb300.observables import dos_from_moments, random_vector_generator


def _h8():
    arr = lattice.honeycomb_arrays(8, 8, t=-2.7, W=0.5, seed=1234)
    dx = lattice.to_csr(dict(arr, data=arr["dx"]))
    dy = lattice.to_csr(dict(arr, data=arr["dy"]))
    return ell_matrix(lattice.to_csr(arr), dx, dy, None)


def test_csr_to_ell_matches_reference_layout():
    z = golden("honeycomb_8x8")
    H = _h8()
    assert H.len_row == int(z["len_row"])
    assert np.array_equal(H.data, z["data"])
    assert np.array_equal(H.indices, z["indices"])
    assert np.array_equal(H.valid_row_values, z["valid"])


def test_csr_to_ell_irregular_padding():
    z = golden("irregular_300")
    # rebuild the CSR from the reference's ELL (valid slots) and convert back
    import scipy.sparse as sp

    n, L = int(z["n"]), int(z["len_row"])
    rows = np.repeat(np.arange(n), L)
    m = z["valid"] == 1
    csr = sp.csr_matrix((z["data"][m], (rows[m], z["indices"][m])), shape=(n, n))
    Lr, data, idx, valid, _ = csr_to_ell_arrays(csr)
    assert Lr == L
    assert np.array_equal(data, z["data"])
    assert np.array_equal(idx, z["indices"])
    assert np.array_equal(valid, z["valid"])


def test_bounds_and_rescaling_bit_identical():
    z = golden("honeycomb_8x8")
    H = _h8()
    assert np.array_equal(H.bounds, z["bounds"])
    Hk = H.modifier(modifier_bounds)
    assert np.array_equal(Hk.data, z["data_kpm"])
    x = golden("honeycomb_8x8_more")
    assert np.array_equal(H.modifier(modifier_velocity_bounds, "x").data, x["v2_data"])
    assert np.array_equal(H.modifier(modifier_velocity, "y").data, x["v1_data"])
    assert np.array_equal(H.dx_vec, x["dx_vec"])


def test_modifier_returns_independent_copy():
    H = _h8()
    Hk = H.modifier(modifier_bounds)
    Hk.indices[0] = 5
    assert H.indices[0] != 5 or golden("honeycomb_8x8")["indices"][0] == 5


def test_kernels_match_reference():
    z = golden("kernels")
    assert np.allclose(km.JacksonKernel(64), z["jackson_64"], rtol=0, atol=1e-15)
    assert np.allclose(km.JacksonKernel(512), z["jackson_512"], rtol=0, atol=1e-15)
    for i, e in enumerate(z["E"]):
        assert np.allclose(km.moments_delta(e, 32), z["delta"][i], rtol=1e-15, atol=1e-15)
        assert np.allclose(km.moments_FD_T0(e, 32), z["fd_t0"][i], rtol=1e-15, atol=1e-15)
        assert np.allclose(km.moments_Gmas(e, 16), z["gmas"][i], rtol=1e-15, atol=1e-15)
    assert np.allclose(km.moments_U(1.3, 40), z["mu_U"], rtol=1e-14, atol=1e-16)
    tab = km.moments_delta_table(z["E"], 32)
    assert np.allclose(tab, z["delta"], rtol=1e-14, atol=1e-14)


def test_broadened_and_tabulated_moments_match_reference():
    """moments_Gmas_2, moments_delta_2 and moments_FD (jclsquant/kernel_and_moments.py:33-44,
    107-115) against the reference's own outputs."""
    z = golden("kernels_more")
    for i, e in enumerate(z["E"]):
        for j, b in enumerate(z["eta"]):
            g = km.moments_Gmas_2(e, b, 48)
            assert g.dtype == np.complex128 and g.shape == (48,)
            assert np.allclose(g, z["gmas2"][i, j], rtol=1e-13, atol=1e-13 * np.max(np.abs(z["gmas2"][i, j])))
            assert np.allclose(km.moments_delta_2(e, b, 48), z["delta2"][i, j], rtol=1e-13,
                               atol=1e-13 * np.max(np.abs(z["delta2"][i, j])))
    for k, f in enumerate(z["fd_tab"]):
        assert np.allclose(km.moments_FD(64, f), z["moments_fd"][k], rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("case", ["honeycomb_8x8", "ref_graphene_256", "irregular_300", "honeycomb_64x64"])
def test_dos_reconstruction_matches_reference(case):
    z = golden(case)
    M = int(z["M"])
    dos = dos_from_moments(z["mu"][0], z["bounds"], M)
    ref = z["dos"]
    assert np.array_equal(dos[:, 0], ref[:, 0])
    assert np.max(np.abs(dos[:, 1] - ref[:, 1])) <= 1e-12 * np.max(np.abs(ref[:, 1]))


def test_random_vector_generator_matches_reference():
    z = golden("honeycomb_8x8")
    for r, s in enumerate(z["seeds"]):
        assert np.array_equal(random_vector_generator(int(z["n"]), int(s)), z["v"][r])


def test_lattice_is_hermitian_with_partner_map():
    arr = lattice.honeycomb_arrays(6, 4, t=-2.7, W=1.0, seed=3)
    csr = lattice.to_csr(arr)
    assert abs(csr - csr.getH()).max() == 0
    n, L = arr["n"], arr["len_row"]
    rows = np.repeat(np.arange(n), L)
    p = arr["partner"]
    bond = p >= 0
    # partner of (i -> j) sits in row j and points back to i
    assert np.array_equal(p[bond] // L, arr["indices"][bond])
    assert np.array_equal(arr["indices"][p[bond]], rows[bond])
    assert np.array_equal(p[p[bond]], np.nonzero(bond)[0])
    # every bond is a nearest neighbour
    d = np.hypot(np.real(arr["dx"][bond]), np.real(arr["dy"][bond]))
    assert np.allclose(d, lattice.A_CC)
    # x_j - x_i antisymmetry
    assert np.allclose(arr["dx"][p[bond]], -arr["dx"][bond])


def test_lattice_open_boundary_padding():
    arr = lattice.honeycomb_arrays(3, 3, t=-1.0, periodic=False)
    n, L = arr["n"], arr["len_row"]
    assert L == 3
    assert np.sum(arr["valid"]) == 2 * (3 * 3 * 3 - 3 - 3)  # directed bonds of a 3x3 open flake
    assert np.all(arr["data"][arr["valid"] == 0] == 0)
    assert np.all((arr["indices"] >= 0) & (arr["indices"] < n))


def test_honeycomb_ensemble_is_seeded_and_rescaled():
    from minijclsquant_gb300 import batched

    d1, i1, L, b1, p1 = batched.honeycomb_ensemble(5, side_range=(4, 9), seed=7)
    d2, i2, _, b2, p2 = batched.honeycomb_ensemble(5, side_range=(4, 9), seed=7)
    assert all(np.array_equal(x, y) for x, y in zip(d1, d2))
    assert np.array_equal(p1["sides"], p2["sides"]) and np.all((p1["sides"] >= 4) & (p1["sides"] <= 9))
    for d, b, s in zip(d1, b1, p1["sides"]):
        assert d.size == 2 * s * s * L
        # rescaled by the instance's own bound: every Gershgorin disc inside [-1/1.01, 1/1.01]
        rows = np.abs(d.reshape(-1, L)).sum(axis=1)
        assert rows.max() <= 1 / 1.01 + 1e-12
    v = batched.ensemble_vectors([8, 18], 2, seed0=3)
    assert v.shape == (2, 26) and np.allclose(np.abs(v), 1.0)


def test_strict_error_mode(capsys):
    """Default: the reference's message and None.  Strict mode: ValueError with that message."""
    from minijclsquant_gb300 import errors
    from minijclsquant_gb300 import recurrence_functions as rf

    H = _h8()
    assert rf.rec_A_tab(8, H, None) is None
    assert modifier_velocity(H, "w") is None
    assert "You must introduce a vector." in capsys.readouterr().out
    with errors.strict():
        with pytest.raises(ValueError, match="introduce a vector"):
            rf.rec_A_tab(8, H, None)
        with pytest.raises(ValueError, match="valid direction"):
            modifier_velocity(H, "w")
        with pytest.raises(ValueError, match="velocity"):
            rf.rec_com_A_vec(8, H, None, np.ones(8), np.ones(H.shape[0]))
    assert not errors.is_strict()
    errors.set_strict(True)
    try:
        with pytest.raises(ValueError):
            rf.rec_A_vec(8, H, None, np.ones(H.shape[0]))
    finally:
        errors.set_strict(False)
