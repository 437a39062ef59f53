"""The oracle (C restatement of jclsquant's CPU path) pinned against the
golden vectors produced by the reference itself (tests/golden/make_golden.py).
CPU only."""
import numpy as np
import pytest

from conftest import golden
from oracle import oracle, reference_import

CASES = ["honeycomb_8x8", "ref_graphene_256", "complex_open_6x5", "irregular_300"]


@pytest.mark.parametrize("case", CASES)
def test_oracle_moments_match_reference(case):
    z = golden(case)
    L = int(z["len_row"])
    for r in range(z["v"].shape[0]):
        mu = oracle.rec_A_tab(int(z["M"]), z["data_kpm"], z["indices"], L, z["v"][r])
        ok, err = oracle.moment_tolerance_ok(mu, z["mu"][r], rel=1e-12)
        assert ok, (case, r, err)


def test_oracle_moments_thread_count_independent():
    z = golden("irregular_300")
    L = int(z["len_row"])
    a = oracle.rec_A_tab(int(z["M"]), z["data_kpm"], z["indices"], L, z["v"][0], threads=1)
    b = oracle.rec_A_tab(int(z["M"]), z["data_kpm"], z["indices"], L, z["v"][0], threads=4)
    assert oracle.moment_tolerance_ok(a, b, rel=1e-12)[0]


def test_oracle_other_recursions_match_reference():
    z = golden("honeycomb_8x8")
    x = golden("honeycomb_8x8_more")
    L = int(z["len_row"])
    d, ix, v = z["data_kpm"], z["indices"], z["v"][0]
    M = int(z["M"])
    assert oracle.moment_tolerance_ok(oracle.rec_A_tab2v(M, d, ix, L, x["v_l"], v), x["mu_lr"], 1e-12)[0]
    a, b = oracle.rec_A_tab2v_2(M, d, ix, L, x["v_l"], v)
    assert oracle.moment_tolerance_ok(a, x["mu2_a"], 1e-12)[0]
    assert oracle.moment_tolerance_ok(b, x["mu2_b"], 1e-12)[0]
    Ms = len(x["coef"])
    s = oracle.rec_A_vec(Ms, d, ix, L, x["coef"], v)
    assert np.max(np.abs(s - x["series"])) <= 1e-12 * np.max(np.abs(x["series"]))
    c = oracle.rec_com_A_vec(Ms, d, x["v2_data"], ix, L, x["coef"], v)
    assert np.max(np.abs(c - x["comm"])) <= 1e-12 * np.max(np.abs(x["comm"]))
    sig = oracle.for_time_sigma(d, x["v1_data"], x["v2_data"], ix, L, x["cu"], x["coef"], int(x["len_t"]), v, Ms,
                                int(x["M2"]))
    assert np.max(np.abs(sig - x["sigma"])) <= 1e-11 * np.max(np.abs(x["sigma"]))


def test_oracle_commutator_table_matches_reference():
    z = golden("commutator_table_5x4")
    tab = oracle.rec_com_A_vec_tab(int(z["M"]), z["data_kpm"], z["v_data"], z["indices"], int(z["len_row"]),
                                   z["coef"], z["v"])
    assert np.max(np.abs(tab - z["tab"])) <= 1e-13 * np.max(np.abs(z["tab"]))
    ser = oracle.rec_com_A_vec(int(z["M"]), z["data_kpm"], z["v_data"], z["indices"], int(z["len_row"]), z["coef"],
                               z["v"])
    assert np.max(np.abs(ser - z["series"])) <= 1e-13 * np.max(np.abs(z["series"]))


def test_oracle_two_vector_dos_matches_reference():
    """The two-vector DOS fixture (kpm_n_dos_n with and without a projector) rebuilt from the
    oracle's rec_A_tab2v and the host reconstruction."""
    from minijclsquant_gb300.ell_matrix import ell_matrix
    from minijclsquant_gb300.modifiers import modifier_bounds
    from minijclsquant_gb300.observables import dos_from_moments

    z = golden("two_vector_dos_8x8")
    L, M = int(z["len_row"]), int(z["M"])
    H = ell_matrix.from_ell(z["data"], z["indices"], L, bounds=z["bounds"], valid_row_values=z["valid"])
    dk = H.modifier(modifier_bounds).data
    mu = oracle.rec_A_tab2v(M, dk, z["indices"], L, z["v_l"], z["v_r"])
    got = dos_from_moments(mu, z["bounds"], M)
    assert np.max(np.abs(got[:, 1] - z["dos"][:, 1])) <= 1e-12 * np.max(np.abs(z["dos"][:, 1]))
    pl = np.zeros_like(z["v_l"])
    oracle.aAxby(1.0, 0.0, z["v_l"], pl, z["proj_data"], z["proj_indices"], int(z["proj_len_row"]))
    mu_p = oracle.rec_A_tab2v(M, dk, z["indices"], L, pl, z["v_r"])
    got_p = dos_from_moments(mu_p, z["bounds"], M)
    assert np.max(np.abs(got_p[:, 1] - z["dos_proj"][:, 1])) <= 1e-12 * np.max(np.abs(z["dos_proj"][:, 1]))


def test_oracle_time_evolution_matches_reference():
    z = golden("time_evolution_6x5")
    U, Uc = oracle.for_time(z["data_kpm"], z["indices"], int(z["len_row"]), z["c"], int(z["len_t"]), z["U0"],
                            z["Uc0"], int(z["M"]))
    assert np.max(np.abs(U - z["U"])) <= 1e-13 * np.max(np.abs(z["U"]))
    assert np.max(np.abs(Uc - z["Uc"])) <= 1e-13 * np.max(np.abs(z["Uc"]))
    # exp(-i H dt) is unitary and the moments are converged: norms are kept
    assert abs(np.linalg.norm(z["U"]) - np.linalg.norm(z["U0"])) <= 1e-10 * np.linalg.norm(z["U0"])


def test_oracle_tiny_and_short_recursions():
    z = golden("tiny_2x2")
    L = int(z["len_row"])
    assert np.allclose(oracle.rec_A_tab(2, z["data_kpm"], z["indices"], L, z["v"]), z["mu2"], rtol=1e-14, atol=1e-14)
    assert np.allclose(oracle.rec_A_tab(3, z["data_kpm"], z["indices"], L, z["v"]), z["mu3"], rtol=1e-14, atol=1e-14)
    # the reference rejects M = 1 with an IndexError
    assert str(z["m1_error"]) == "IndexError"


def test_oracle_cpu_dos_configuration():
    """64 x 64 cells (8192 sites), M = 512, 4 vectors: inputs rebuilt by the lattice builder,
    checked by digest against what the reference was fed, then the oracle against its moments."""
    from minijclsquant_gb300 import lattice
    from minijclsquant_gb300.modifiers import modifier_bounds
    from tests.golden.make_golden import digest

    z = golden("honeycomb_64x64")
    arr = lattice.honeycomb_arrays(64, 64, t=-2.7, W=0.5, seed=1234)
    from minijclsquant_gb300.ell_matrix import ell_matrix

    H = ell_matrix(lattice.to_csr(arr))
    assert digest(H.data, H.indices) == str(z["input_digest"])
    assert np.array_equal(H.bounds, z["bounds"])
    Hk = H.modifier(modifier_bounds)
    assert digest(Hk.data) == str(z["kpm_digest"])
    from minijclsquant_gb300.observables import random_vector_generator

    for r, seed in enumerate(z["seeds"]):
        v = random_vector_generator(8192, int(seed))
        mu = oracle.rec_A_tab(int(z["M"]), Hk.data, Hk.indices, int(z["len_row"]), v)
        # OpenMP combines per-thread partial sums in completion order, so two runs of
        # the same code differ by up to ~1e-12 per order at M = 512: pin at 1e-11.
        ok, err = oracle.moment_tolerance_ok(mu, z["mu"][r], rel=1e-11)
        assert ok, err


def test_oracle_adjoint_gradient_against_finite_differences():
    """The FP64 adjoint oracle (the reference gradient for the GPU adjoint) is pinned by
    central differences of the oracle's own moments, h = 1e-6."""
    from minijclsquant_gb300 import lattice

    arr = lattice.honeycomb_arrays(4, 3, t=-1.0, W=0.8, seed=2, with_geometry=False)
    n, L = arr["n"], arr["len_row"]
    d = arr["data"] / 4.0
    v = np.exp(1j * np.random.default_rng(1).uniform(0, 2 * np.pi, n))
    M = 20
    c = np.random.default_rng(2).normal(size=M)

    def loss(dd):
        return float(np.sum(c * oracle.rec_A_tab(M, dd, arr["indices"], L, v, threads=1).real))

    g = oracle.adjoint_grad(M, d, arr["indices"], L, v, c)
    h = 1e-6
    for q in range(0, n * L, 7):
        dp, dm = d.copy(), d.copy()
        dp[q] += h
        dm[q] -= h
        fd = (loss(dp) - loss(dm)) / (2 * h)
        assert abs(g[q] - fd) <= 1e-7 * max(1.0, abs(fd)), (q, g[q], fd)


@pytest.mark.skipif(not reference_import.available(), reason="reference tree not present")
def test_oracle_against_live_reference():
    """Fresh seeded case, run through the live reference (built from its .pyx) and the oracle."""
    ref = reference_import.load()
    from minijclsquant_gb300 import lattice

    arr = lattice.honeycomb_arrays(5, 7, t=-2.1, W=0.8, seed=4321, periodic=False)
    H = ref.ell_matrix.ell_matrix(lattice.to_csr(arr))
    Hk = H.modifier(ref.modifiers.modifier_bounds)
    v = ref.observables.random_vector_generator(H.shape[0], 99)
    mu_ref = ref.recurrence_functions.rec_A_tab(40, Hk, v)
    mu = oracle.rec_A_tab(40, Hk.data, Hk.indices, H.len_row, v)
    assert oracle.moment_tolerance_ok(mu, mu_ref, 1e-12)[0]
    y_ref = np.zeros_like(v)
    y = np.zeros_like(v)
    ref.blas_funs.aAxby(2 + 0j, -1 + 0j, v, y_ref, Hk.data, Hk.indices, H.len_row, H.shape[0], 2)
    oracle.aAxby(2, -1, v, y, Hk.data, Hk.indices, H.len_row)
    assert np.max(np.abs(y - y_ref)) <= 1e-14 * np.max(np.abs(y_ref))


def test_oracle_known_answers():
    """The oracle on operators with closed-form moments: diag(e) gives
    sum_i |v_i|^2 cos(m arccos e_i); the periodic chain (S + S^dagger)/2 gives
    (1/2) sum_i conj(v_i)(v_{i+m} + v_{i-m})."""
    rng = np.random.default_rng(5)
    n, M = 2000, 200
    e = rng.uniform(-0.99, 0.99, n)
    v = np.exp(2j * np.pi * rng.random(n))
    mu = oracle.rec_A_tab(M, e.astype(np.complex128), np.arange(n, dtype=np.int32), 1, v)
    ref = np.array([np.sum(np.abs(v) ** 2 * np.cos(m * np.arccos(e))) for m in range(M)])
    assert oracle.moment_tolerance_ok(mu, ref, 1e-10)[0]
    i = np.arange(n)
    idx = np.stack([(i + 1) % n, (i - 1) % n], axis=1).astype(np.int32).reshape(-1)
    mu = oracle.rec_A_tab(M, np.full(2 * n, 0.5, dtype=np.complex128), idx, 2, v)
    ref = np.array([0.5 * np.vdot(v, np.roll(v, -m) + np.roll(v, m)) for m in range(M)])
    assert oracle.moment_tolerance_ok(mu, ref, 1e-10)[0]
    assert abs(mu[0] - n) <= 1e-12 * n


def test_oracle_modifiers_match_reference():
    """The light and phonon modifiers against the reference's own Cython outputs."""
    z = golden("modifiers_6x5")
    for prm, want in zip(z["light_params"], z["light_out"]):
        got = oracle.light_modifier(*prm, z["data"], z["dx"], z["dy"])
        assert np.max(np.abs(got - want)) <= 1e-14 * np.max(np.abs(want)), prm
    a0, b, Aq, wq, t, q0, q1 = z["phonon_params"]
    dn, dxn, dyn = oracle.phonon_modifier(a0, b, Aq, wq, t, np.array([q0, q1]), z["data"], z["indices"], z["dx"],
                                          z["dy"], z["e_pol_x"], z["e_pol_y"], z["Sx"], z["Sy"], int(z["len_row"]))
    assert np.max(np.abs(dn - z["phonon_data"])) <= 1e-14 * np.max(np.abs(z["phonon_data"]))
    assert np.max(np.abs(dxn - z["phonon_dx"])) <= 1e-14 * np.max(np.abs(z["phonon_dx"]))
    assert np.max(np.abs(dyn - z["phonon_dy"])) <= 1e-14 * np.max(np.abs(z["phonon_dy"]))
