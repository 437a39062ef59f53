"""Kubo-Greenwood sigma(E) from the moment matrix (kubo.sigma_from_mu) against an FP64
restatement by exact diagonalisation.

In the eigenbasis of H~ = H / a (eigenvalues w_a) the double Chebyshev sum is

    sigma(E) = 2 / (Omega a^2 (1 - e^2)) sum_{a,b} |V_ab|^2 K_a(e) K_b(e),
    K_a(e) = sum_n h_n T_n(e) T_n(w_a),  h_n = (2 - delta_n0) g_n (Jackson),  e = E / a,

since Tr[V T_n(H~) V T_m(H~)] = sum_ab |V_ab|^2 T_n(w_b) T_m(w_a).  That is the KPM
Kubo-Greenwood conductivity (pi hbar e^2 / Omega) Tr[v delta(E - H) v delta(E - H)] in
units of e^2/h with Jackson-broadened deltas (A. Weisse et al., Rev. Mod. Phys. 78, 275
(2006)).  The restatement shares no code with kubo.py: eigenvectors instead of
Chebyshev vectors, a per-eigenpair sum instead of the moment matrix.

CPU: sigma_from_mu on the exact FP64 trace mu_nm (dense Chebyshev matrices) agrees to
1e-11 of max sigma.  GPU: kpm_mu_nm (complex64 recursions, 3xTF32 tensor-core
contraction) over all N basis vectors gives the exact trace times 1/N; sigma(E) from it
agrees with the restatement to 2e-4 of max sigma.
"""
import numpy as np
import pytest

from minijclsquant_gb300 import lattice
from minijclsquant_gb300.kernel_and_moments import JacksonKernel
from minijclsquant_gb300.kubo import sigma_from_mu

OMEGA = 3.7


def _problem(cells=6, W=1.2, seed=3):
    from minijclsquant_gb300.ell_matrix import ell_matrix
    from minijclsquant_gb300.modifiers import modifier_bounds, modifier_velocity

    arr = lattice.honeycomb_arrays(cells, cells, t=-2.7, W=W, seed=seed)
    dx = lattice.to_csr(dict(arr, data=arr["dx"]))
    dy = lattice.to_csr(dict(arr, data=arr["dy"]))
    H = ell_matrix(lattice.to_csr(arr), dx, dy, None)
    Hk = H.modifier(modifier_bounds)
    V = H.modifier(modifier_velocity, "x")
    return H, Hk, V


def _dense(op):
    n = op.shape[0]
    L = op.len_row
    D = np.zeros((n, n), dtype=np.complex128)
    rows = np.repeat(np.arange(n), L)
    np.add.at(D, (rows, op.indices), op.data)
    return D


def _sigma_ed(Hk_d, V_d, bounds, energies, Nm, omega):
    a = 0.5 * (bounds[1] - bounds[0])
    w, U = np.linalg.eigh(Hk_d)
    Vab2 = np.abs(U.conj().T @ V_d @ U) ** 2
    h = JacksonKernel(Nm) * np.where(np.arange(Nm) == 0, 1.0, 2.0)
    e = np.asarray(energies) / a
    Tn_e = np.cos(np.arange(Nm)[None, :] * np.arccos(e)[:, None])        # [E, Nm]
    Tn_w = np.cos(np.arange(Nm)[:, None] * np.arccos(np.clip(w, -1, 1))[None, :])  # [Nm, N]
    K = (Tn_e * h[None, :]) @ Tn_w                                          # [E, N]
    core = np.einsum("ea,ab,eb->e", K, Vab2, K)
    return 2.0 * core / (omega * a * a * (1.0 - e * e))


def _mu_exact(Hk_d, V_d, Nm):
    n = Hk_d.shape[0]
    T = [np.eye(n, dtype=np.complex128), Hk_d.copy()]
    for m in range(2, Nm):
        T.append(2 * Hk_d @ T[-1] - T[-2])
    VT = np.stack([V_d @ t for t in T])                                     # [Nm, n, n]
    # mu_nm = Tr[V T_n V T_m] = sum_ij (V T_n)_ij (V T_m)_ji
    return np.einsum("nij,mji->nm", VT, VT)


def test_sigma_from_mu_matches_eigenbasis_restatement():
    H, Hk, V = _problem()
    Nm = 96
    Hd, Vd = _dense(Hk), _dense(V)
    assert np.allclose(Hd, Hd.conj().T, atol=1e-14) and np.allclose(Vd, Vd.conj().T, atol=1e-14)
    mu = _mu_exact(Hd, Vd, Nm)
    out = sigma_from_mu(mu, H.bounds, OMEGA, n_energies=301)
    ref = _sigma_ed(Hd, Vd, H.bounds, out[:, 0], Nm, OMEGA)
    assert np.array_equal(out[:, 0], np.linspace(H.bounds[0] + 1e-3, H.bounds[1] - 1e-3, 301))
    assert np.max(np.abs(out[:, 1] - ref)) <= 1e-11 * np.max(np.abs(ref))
    assert np.max(ref) > 0 and np.min(ref) > -1e-12 * np.max(ref)  # a conductivity is non-negative
    # explicit energies, and the symmetry of mu_nm the formula relies on
    E = np.array([-3.1, -0.4, 0.0, 1.7])
    assert np.allclose(sigma_from_mu(mu, H.bounds, OMEGA, energies=E)[:, 1], _sigma_ed(Hd, Vd, H.bounds, E, Nm, OMEGA),
                       rtol=1e-10, atol=1e-12 * np.max(ref))
    assert np.max(np.abs(mu - mu.T)) <= 1e-10 * np.max(np.abs(mu))


@pytest.mark.gpu
def test_kubo_greenwood_gpu_matches_eigenbasis_restatement(cuda_lib):
    from minijclsquant_gb300 import kubo

    H, Hk, V = _problem()
    n = Hk.shape[0]
    Nm = 256
    basis = np.eye(n, dtype=np.complex128)
    mu = kubo.mu_nm(Hk.device(), V.device(), Nm, basis) * n  # (1/R) sum_r over all basis vectors = Tr / n
    out = sigma_from_mu(mu, H.bounds, OMEGA, n_energies=401)
    ref = _sigma_ed(_dense(Hk), _dense(V), H.bounds, out[:, 0], Nm, OMEGA)
    assert np.max(np.abs(out[:, 1] - ref)) <= 2e-4 * np.max(np.abs(ref)), np.max(np.abs(out[:, 1] - ref)) / np.max(ref)
