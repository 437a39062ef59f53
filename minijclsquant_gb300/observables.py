"""KPM observables, drop-in for jclsquant/observables.py (DOS entry points).

``kpm_dos`` and ``kpm_n_dos_n`` keep the reference's signatures and return
value (an array [n_E, 2]: unnormalised energies and DOS); the recursion runs on
the GPU, the Jackson/DOS reconstruction is an FP64 matrix-vector product on
the host (the reference loops over energies in Python).  Keyword-only extras:
``dtype`` ('c128' | 'c64') and ``n_energies`` (default 2M+1, the reference's
grid).  With R random vectors ([R, N]) the DOS is the average over vectors.
"""
from __future__ import annotations

import functools

import numpy as np

from . import recurrence_functions as rf
from .kernel_and_moments import JacksonKernel, moments_delta_table
from .modifiers import modifier_bounds


def random_vector_generator(shape_H, seed=None):
    """Random-phase vector exp(i U[0, 2pi)) from default_rng(seed) (jclsquant/observables.py:19-21)."""
    rng = np.random.default_rng(seed)
    return np.exp(1j * rng.uniform(0, 2 * np.pi, shape_H))


def energy_grid(bounds, M, n_energies=None):
    """The reference's energy grid linspace(b0 + 1e-3, b1 - 1e-3, 2M + 1) (jclsquant/observables.py:39)."""
    n_e = 2 * M + 1 if n_energies is None else int(n_energies)
    return np.linspace(bounds[0] + 1e-3, bounds[1] - 1e-3, n_e)


def rescaled_energies(Ef_vec, bounds):
    """E~ = E/a - c/a with a = (b1-b0)/2, c = (b1+b0)/2 (jclsquant/observables.py:52)."""
    a = 0.5 * (bounds[1] - bounds[0])
    return Ef_vec / a - (0.5 * (bounds[1] + bounds[0])) / a


@functools.lru_cache(maxsize=16)
def _dos_table(b0, b1, M, n_energies):
    """(energies, the Jackson-damped delta moments [n_E, M]) of a grid, kept for reuse: the
    table depends only on the bounds, M and the grid, not on the moments."""
    bounds = (b0, b1)
    Ef_vec = energy_grid(bounds, M, n_energies)
    table = moments_delta_table(rescaled_energies(Ef_vec, bounds), M) * JacksonKernel(M)[None, :]
    Ef_vec.setflags(write=False)
    table.setflags(write=False)
    return Ef_vec, table


def dos_from_moments(mu, bounds, M, n_energies=None):
    """[E, rho(E)] with rho = Re sum_m delta_m(E~) g_m mu_m (jclsquant/observables.py:49-52).

    ``mu`` is [M] or [R, M]; several moment sets are averaged first (the DOS is
    linear in the moments).
    """
    mu = np.asarray(mu)
    if mu.ndim == 2:
        mu = mu.mean(axis=0)
    Ef_vec, table = _dos_table(float(bounds[0]), float(bounds[1]), int(M),
                               None if n_energies is None else int(n_energies))
    out = np.zeros((len(Ef_vec), 2))
    out[:, 0] = Ef_vec
    # Re(table . mu) with a real table: two real products, no complex copy of the table
    mu = mu.astype(np.complex128)
    out[:, 1] = table @ mu.real
    return out


def kpm_dos(H, M=None, random_vector=None, *, dtype="c128", n_energies=None):
    """Density of states by KPM (jclsquant/observables.py:26-54)."""
    if M is None:
        M = int(np.sqrt(H.shape[0]))
    if random_vector is None:
        random_vector = random_vector_generator(H.shape[0])
    H_kpm = H.modifier(modifier_bounds)
    mu = rf.rec_A_tab(M, H_kpm, random_vector, dtype=dtype)
    return dos_from_moments(_host(mu), H.bounds, M, n_energies)


def kpm_n_dos_n(H, M=None, random_vector_l=None, random_vector_r=None, bounds=True, proyector=None, *,
                dtype="c128", n_energies=None):
    """DOS with different bra and ket vectors, optional projector on the bra
    (jclsquant/observables.py:59-120)."""
    if M is None:
        M = int(np.sqrt(H.shape[0]))
    if random_vector_l is None and random_vector_r is None:
        random_vector_r = random_vector_generator(H.shape[0])
        random_vector_l = np.copy(random_vector_r)
    if proyector is not None:
        projected = np.zeros(np.shape(random_vector_l), dtype=np.complex128)
        proyector.dot(1.0 + 0j, 0 + 0j, random_vector_l, projected)
        random_vector_l = projected
    op = H.modifier(modifier_bounds) if bounds is True else H
    mu = rf.rec_A_tab2v(M, op, random_vector_l, random_vector_r, dtype=dtype)
    return dos_from_moments(_host(mu), H.bounds, M, n_energies)


def _host(x):
    try:
        import torch

        if isinstance(x, torch.Tensor):
            return x.detach().cpu().numpy()
    except ImportError:  # pragma: no cover
        pass
    return np.asarray(x)
