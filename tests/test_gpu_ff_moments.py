"""The FP64 recursion with float-float moment products (the default for one-set complex128
moments on the producer-warp step kernel): against the oracle at 1e-10 per order, against
the all-FP64 products (KPM_MOMENTS_FP64=1) at 2e-11 (the float pairs carry 2^-49 per
product; on 2880 sites that reaches ~1e-12 of the per-order scale), and on vectors whose elements leave the
float-pair range (tiny, huge, exactly zero, localized), which take the FP64 product."""
import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu

REL = 1e-10


def _op(complex_hops, seed=5):
    from minijclsquant_gb300 import lattice
    from minijclsquant_gb300.ell_matrix import ell_matrix
    from minijclsquant_gb300.modifiers import modifier_bounds

    if not complex_hops:
        return lattice.honeycomb(40, 36, t=-2.7, W=0.7, seed=seed).modifier(modifier_bounds)
    arr = lattice.honeycomb_arrays(40, 36, t=-2.7, W=0.7, seed=seed)
    phase = np.exp(1j * 0.4 * np.real(arr["dx"]) / 0.142)
    arr = dict(arr, data=np.where(np.real(arr["dx"]) != 0, arr["data"] * phase, arr["data"]))
    dx = lattice.to_csr(dict(arr, data=arr["dx"]))
    dy = lattice.to_csr(dict(arr, data=arr["dy"]))
    return ell_matrix(lattice.to_csr(arr), dx, dy).modifier(modifier_bounds)


def _moments(monkeypatch, Hk, vs, M, kernel, fp64, v_l=None):
    from minijclsquant_gb300 import device

    monkeypatch.setenv("KPM_STEP_KERNEL", kernel)
    if fp64:
        monkeypatch.setenv("KPM_MOMENTS_FP64", "1")
    else:
        monkeypatch.delenv("KPM_MOMENTS_FP64", raising=False)
    op = device.DeviceELL(Hk.data, Hk.indices, Hk.len_row)
    return np.asarray(device.cheb_moments(op, M, vs, v_l=v_l))


@pytest.mark.parametrize("kernel", ["ws1", "ws2", "ws1s2"])
@pytest.mark.parametrize("complex_hops", [False, True])
@pytest.mark.parametrize("R", [1, 3, 8])
def test_ff_products_against_oracle_and_fp64(cuda_lib, monkeypatch, kernel, complex_hops, R):
    from minijclsquant_gb300.observables import random_vector_generator

    Hk = _op(complex_hops)
    vs = np.stack([random_vector_generator(Hk.data.size // Hk.len_row, 70 + r) for r in range(R)])
    M = 200
    mu = _moments(monkeypatch, Hk, vs, M, kernel, fp64=False)
    mu64 = _moments(monkeypatch, Hk, vs, M, kernel, fp64=True)
    for r in range(R):
        ref = oracle.rec_A_tab(M, Hk.data, Hk.indices, Hk.len_row, vs[r])
        ok, err = oracle.moment_tolerance_ok(mu[r], ref, REL)
        assert ok, (r, err)
        ok, err = oracle.moment_tolerance_ok(mu[r], mu64[r], 2e-11)
        assert ok, ("vs FP64 products", r, err)


def test_ff_products_two_vector_moments(cuda_lib, monkeypatch):
    """<v_l|T_m v_r>: the left vector is the one packed as float pairs."""
    from minijclsquant_gb300.observables import random_vector_generator

    Hk = _op(True)
    n = Hk.data.size // Hk.len_row
    v_r = np.stack([random_vector_generator(n, 3 + r) for r in range(2)])
    v_l = np.stack([random_vector_generator(n, 13 + r) for r in range(2)])
    mu = _moments(monkeypatch, Hk, v_r, 120, "ws1", fp64=False, v_l=v_l)
    for r in range(2):
        ref = oracle.rec_A_tab2v(120, Hk.data, Hk.indices, Hk.len_row, v_l[r], v_r[r])
        ok, err = oracle.moment_tolerance_ok(mu[r], ref, REL)
        assert ok, (r, err)


@pytest.mark.parametrize("case", ["tiny", "huge", "mixed", "localized", "zeros"])
def test_ff_products_out_of_range_elements(cuda_lib, monkeypatch, case):
    from minijclsquant_gb300.observables import random_vector_generator

    Hk = _op(False)
    n = Hk.data.size // Hk.len_row
    rng = np.random.default_rng(11)
    v = random_vector_generator(n, 8)
    if case == "tiny":
        v = v * 1e-20
    elif case == "huge":
        v = v * 1e25
    elif case == "mixed":  # magnitudes from 1e-30 to 1e30 across the elements
        v = v * 10.0 ** rng.uniform(-30, 30, n)
    elif case == "localized":  # T_m v decays away from the seed: tiny elements at every step
        v = np.zeros(n, dtype=np.complex128)
        v[n // 2] = 1.0
    else:  # half the elements exactly zero
        v = np.where(rng.random(n) < 0.5, 0, v)
    M = 150
    mu = _moments(monkeypatch, Hk, v[None, :], M, "ws1", fp64=False)[0]
    ref = oracle.rec_A_tab(M, Hk.data, Hk.indices, Hk.len_row, v)
    ok, err = oracle.moment_tolerance_ok(mu, ref, REL)
    assert ok, (case, err)


@pytest.mark.parametrize("kernel", ["simple", "staged1", "ws1", "ws2", "ws1s2"])
@pytest.mark.parametrize("fp64", [False, True])
def test_step_forms_are_deterministic(cuda_lib, monkeypatch, kernel, fp64):
    """Each step form the autotuner can pick gives bit-identical moments when called twice on the same
    inputs (every partial sum has a fixed place and order), at a size with several hundred tiles per
    launch, so rounding differences between runs can only come from a change of form, never from
    the run itself."""
    from minijclsquant_gb300 import lattice
    from minijclsquant_gb300.modifiers import modifier_bounds
    from minijclsquant_gb300.observables import random_vector_generator

    Hk = lattice.honeycomb(192, 160, t=-2.7, W=0.7, seed=9).modifier(modifier_bounds)
    n = Hk.data.size // Hk.len_row
    vs = np.stack([random_vector_generator(n, 90 + r) for r in range(8)])
    a = _moments(monkeypatch, Hk, vs, 96, kernel, fp64)
    b = _moments(monkeypatch, Hk, vs, 96, kernel, fp64)
    assert np.array_equal(a, b), kernel
    ref = oracle.rec_A_tab(96, Hk.data, Hk.indices, Hk.len_row, vs[0])
    assert oracle.moment_tolerance_ok(a[0], ref, REL)[0]
