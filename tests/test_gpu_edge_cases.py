"""Edge cases of the moment and series calls against the oracle, for every precision:
tiny operators (1 row; a prime number of rows far below the 512-row padding), wide rows
(33 slots, more than one staged slot group), vector counts that are not powers of two,
and the shortest recursions (M = 1, 2, 3)."""
import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu

REL = 1e-10
TOL = {"c128": REL, "c128f": REL}


def _check(mu, ref, dtype, n):
    if dtype == "c64":
        assert np.max(np.abs(mu - ref)) <= 2e-6 * max(n, 1) ** 0.5 * max(1.0, np.abs(ref[0])), (dtype,)
    else:
        ok, err = oracle.moment_tolerance_ok(mu, ref, TOL[dtype])
        assert ok, (dtype, err)


def _random_hermitian_ell(n, L, seed, complex_values=True):
    """Random Hermitian ELL with exactly L slots per row (padding on the row's last column)."""
    rng = np.random.default_rng(seed)
    import scipy.sparse as sp

    rows, cols, vals = [], [], []
    for i in range(n):
        for j in rng.choice(n, size=min(n, max(1, L // 2)), replace=False):
            w = rng.normal() + (1j * rng.normal() if complex_values else 0)
            if j == i:
                w = w.real
            rows += [i, j]
            cols += [j, i]
            vals += [w, np.conj(w)]
    A = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    A.sum_duplicates()
    from minijclsquant_gb300.ell_matrix import csr_to_ell_arrays

    L2, data, idx, valid, _ = csr_to_ell_arrays(A)
    scale = 1.05 * np.max(np.abs(A).sum(axis=1))
    return L2, data / scale, idx


@pytest.mark.parametrize("dtype", ["c128", "c64", "c128f"])
def test_one_row_operator(cuda_lib, dtype):
    from minijclsquant_gb300 import device

    op = device.DeviceELL(np.array([0.5 + 0j]), np.array([0], dtype=np.int32), 1)
    v = np.array([np.exp(0.3j)])
    for M in (1, 2, 3, 40):
        mu = np.asarray(device.cheb_moments(op, M, v, dtype=dtype))
        ref = np.cos(np.arange(M) * np.arccos(0.5))  # T_m(1/2) |v|^2
        _check(mu, ref.astype(np.complex128), dtype, 1)


@pytest.mark.parametrize("dtype", ["c128", "c64", "c128f"])
@pytest.mark.parametrize("n,L", [(7, 3), (13, 33), (1000, 33)])
def test_small_and_wide_operators(cuda_lib, dtype, n, L):
    from minijclsquant_gb300 import device
    from minijclsquant_gb300.observables import random_vector_generator

    L2, data, idx = _random_hermitian_ell(n, L, seed=n + L)
    op = device.DeviceELL(data, idx, L2)
    vs = np.stack([random_vector_generator(n, 5 + r) for r in range(3)])
    M = 64
    mu = np.asarray(device.cheb_moments(op, M, vs, dtype=dtype))
    for r in range(3):
        _check(mu[r], oracle.rec_A_tab(M, data, idx, L2, vs[r]), dtype, n)
    if dtype != "c64":
        c = (np.arange(1, 33) ** -2.0).astype(np.complex128)
        s = np.asarray(device.cheb_series(op, 32, c, vs, dtype=dtype))
        for r in range(3):
            ref = oracle.rec_A_vec(32, data, idx, L2, c, vs[r])
            assert np.max(np.abs(s[r] - ref)) <= REL * np.max(np.abs(ref))


@pytest.mark.parametrize("dtype", ["c128", "c64", "c128f"])
@pytest.mark.parametrize("R", [3, 5, 6, 7, 9, 13])
def test_vector_counts_not_powers_of_two(cuda_lib, dtype, R):
    from minijclsquant_gb300 import device, lattice
    from minijclsquant_gb300.modifiers import modifier_bounds
    from minijclsquant_gb300.observables import random_vector_generator

    Hk = lattice.honeycomb(17, 13, t=-2.7, W=0.9, seed=R).modifier(modifier_bounds)
    op = device.DeviceELL(Hk.data, Hk.indices, Hk.len_row)
    vs = np.stack([random_vector_generator(op.n, 100 + r) for r in range(R)])
    mu = np.asarray(device.cheb_moments(op, 50, vs, dtype=dtype))
    assert mu.shape == (R, 50)
    for r in range(R):
        _check(mu[r], oracle.rec_A_tab(50, Hk.data, Hk.indices, Hk.len_row, vs[r]), dtype, op.n)


@pytest.mark.parametrize("dtype", ["c128", "c64", "c128f"])
def test_shortest_recursions(cuda_lib, dtype):
    from minijclsquant_gb300 import device, lattice
    from minijclsquant_gb300.modifiers import modifier_bounds
    from minijclsquant_gb300.observables import random_vector_generator

    Hk = lattice.honeycomb(9, 11, t=-2.7, W=0.4, seed=2).modifier(modifier_bounds)
    op = device.DeviceELL(Hk.data, Hk.indices, Hk.len_row)
    v = random_vector_generator(op.n, 1)
    for M in (1, 2, 3):
        mu = np.atleast_1d(np.asarray(device.cheb_moments(op, M, v, dtype=dtype)))
        assert mu.shape == (M,)
        _check(mu, oracle.rec_A_tab(max(M, 2), Hk.data, Hk.indices, Hk.len_row, v)[:M], dtype, op.n)
