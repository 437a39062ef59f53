"""Known answers that need no reference run:

* diagonal H~ = diag(e), |e_i| < 1: T_m(H~) = diag(T_m(e_i)), so
  mu_m = sum_i |v_i|^2 cos(m arccos e_i);
* the periodic chain H~ = (S + S^dagger)/2 (S the cyclic shift): T_m(H~) = (S^m + S^-m)/2
  exactly, so mu_m = (1/2) sum_i conj(v_i) (v_{i+m} + v_{i-m}), indices mod N;
* mu_0 = N for unit-modulus vectors;
* the invariant the reference's own smoke script checks (dos_test_only_cpu.py:33-40):
  for graphene with mass 0.5, M = sqrt(N), the DOS divided by N b1 integrates to ~1.

Every moment form is held to these: complex128 and float-float complex128 at 1e-10 per
order, doubled moments at 1e-10 per order, complex64 at 1e-5 of mu_0, and the batched
ensemble per instance."""
import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu

REL = 1e-10


def _diag_case(n, seed):
    rng = np.random.default_rng(seed)
    e = rng.uniform(-0.99, 0.99, n)
    data = e.astype(np.complex128)  # ELL width 1: the diagonal; the step kernels use 2H~
    idx = np.arange(n, dtype=np.int32)
    return data, idx, 1, e


def _diag_mu(e, v, M):
    w = np.abs(v) ** 2
    th = np.arccos(e)
    return np.array([np.sum(w * np.cos(m * th)) for m in range(M)], dtype=np.complex128)


def _chain_case(n):
    i = np.arange(n)
    idx = np.stack([(i + 1) % n, (i - 1) % n], axis=1).astype(np.int32).reshape(-1)
    data = np.full(2 * n, 0.5, dtype=np.complex128)
    return data, idx, 2


def _chain_mu(v, M):
    return np.array([0.5 * np.vdot(v, np.roll(v, -m) + np.roll(v, m)) for m in range(M)], dtype=np.complex128)


def _vectors(n, R, seed0):
    from minijclsquant_gb300.observables import random_vector_generator

    return np.stack([random_vector_generator(n, seed0 + r) for r in range(R)])


@pytest.mark.parametrize("dtype", ["c128", "c128f", "c64"])
@pytest.mark.parametrize("R", [1, 4])
def test_diagonal_operator_moments(cuda_lib, dtype, R):
    from minijclsquant_gb300 import device

    n, M = 5000, 300
    data, idx, L, e = _diag_case(n, 3)
    op = device.DeviceELL(data, idx, L)
    vs = _vectors(n, R, 10)
    mu = np.asarray(device.cheb_moments(op, M, vs, dtype=dtype)).reshape(R, M)
    for r in range(R):
        ref = _diag_mu(e, vs[r], M)
        if dtype == "c64":
            assert np.max(np.abs(mu[r] - ref)) <= 1e-5 * abs(ref[0])
        else:
            ok, err = oracle.moment_tolerance_ok(mu[r], ref, REL)
            assert ok, (dtype, r, err)
        # unit-modulus vector: mu_0 = N (complex64 rounds the vector, ~1e-8 relative)
        assert abs(mu[r][0] - n) <= (1e-7 if dtype == "c64" else 1e-12) * n


@pytest.mark.parametrize("dtype", ["c128", "c128f", "c64"])
def test_periodic_chain_moments(cuda_lib, dtype):
    from minijclsquant_gb300 import device

    n, M = 4099, 600  # odd length: no symmetry hides an index error
    data, idx, L = _chain_case(n)
    op = device.DeviceELL(data, idx, L)
    vs = _vectors(n, 2, 20)
    mu = np.asarray(device.cheb_moments(op, M, vs, dtype=dtype)).reshape(2, M)
    for r in range(2):
        ref = _chain_mu(vs[r], M)
        if dtype == "c64":
            assert np.max(np.abs(mu[r] - ref)) <= 1e-5 * n
        else:
            ok, err = oracle.moment_tolerance_ok(mu[r], ref, REL)
            assert ok, (dtype, r, err)


def test_doubled_moments_known_answers(cuda_lib):
    from minijclsquant_gb300 import device

    n, M = 5000, 301
    data, idx, L, e = _diag_case(n, 4)
    op = device.DeviceELL(data, idx, L, doubling=True)
    assert op.doubling
    v = _vectors(n, 2, 30)
    mu = np.asarray(device.cheb_moments(op, M, v))
    for r in range(2):
        ok, err = oracle.moment_tolerance_ok(mu[r], _diag_mu(e, v[r], M), REL)
        assert ok, err
    cdata, cidx, cL = _chain_case(1031)
    cop = device.DeviceELL(cdata, cidx, cL, doubling=True)
    assert cop.doubling
    cv = _vectors(1031, 2, 40)
    cmu = np.asarray(device.cheb_moments(cop, 500, cv))
    for r in range(2):
        ok, err = oracle.moment_tolerance_ok(cmu[r], _chain_mu(cv[r], 500), REL)
        assert ok, err


@pytest.mark.parametrize("dtype", ["c128", "c64"])
def test_batched_known_answers(cuda_lib, dtype):
    """Diagonal and chain instances of uneven size in one batched recursion."""
    from minijclsquant_gb300.batched import BatchedELL

    M = 200
    datas, idxs, refs_of = [], [], []
    for k, n in enumerate([700, 1300, 257, 2049]):
        if k % 2 == 0:
            d, ix, _, e = _diag_case(n, 50 + k)
            # width 2: pad the diagonal with a zero slot on the row's own column
            d2 = np.stack([d, np.zeros(n, np.complex128)], axis=1).reshape(-1)
            ix2 = np.stack([ix, ix], axis=1).reshape(-1).astype(np.int32)
            datas.append(d2)
            idxs.append(ix2)
            refs_of.append(lambda v, e=e: _diag_mu(e, v, M))
        else:
            d, ix, _ = _chain_case(n)
            datas.append(d)
            idxs.append(ix)
            refs_of.append(lambda v: _chain_mu(v, M))
    b = BatchedELL(datas, idxs, 2)
    v = _vectors(b.n_total, 2, 60)
    mu = b.moments(M, v, dtype=dtype)
    for k in range(b.n_inst):
        o, n = int(b.offsets[k]), int(b.rows[k])
        for r in range(2):
            ref = refs_of[k](v[r, o:o + n])
            if dtype == "c64":
                assert np.max(np.abs(mu[k, r] - ref)) <= 1e-5 * n, (k, r)
            else:
                ok, err = oracle.moment_tolerance_ok(mu[k, r], ref, REL)
                assert ok, (k, r, err)


def test_reference_dos_integral_invariant(cuda_lib):
    """The check of the reference's smoke script, on its lattice size (262,144 sites) and
    mass (0.5), without disorder: DOS / (N b1) integrates to 1 within the KPM truncation."""
    from scipy.integrate import simpson

    from minijclsquant_gb300 import lattice
    from minijclsquant_gb300.observables import random_vector_generator
    from minijclsquant_gb300.observables_gpu import kpm_dos_gpu

    H = lattice.honeycomb(362, 362, t=-2.7, mass=0.5, periodic=True)
    N = H.shape[0]
    dos = kpm_dos_gpu(H, int(np.sqrt(N)), random_vector_generator(N, 1))
    dos[:, 1] = dos[:, 1] / (N * H.bounds[1])
    integral = simpson(dos[:, 1], x=dos[:, 0])
    assert abs(integral - 1.0) < 1e-2, integral
    # Jackson-damped DOS stays non-negative up to the noise of one random vector
    assert np.min(dos[:, 1]) > -1e-2 * np.max(dos[:, 1])
