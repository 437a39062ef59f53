"""KPM kernels and analytic Chebyshev moments (FP64, host).

Same names, arguments and formulas as jclsquant/kernel_and_moments.py; the
functions are vectorised over energies where the reference loops.  These are
O(M) (or O(E*M)) host computations that feed the GPU recursions; they are not
on the hot path.
"""
from __future__ import annotations

from math import pi

import numpy as np


def JacksonKernel(N):
    """Jackson damping g_n, n = 0..N-1 (jclsquant/kernel_and_moments.py:19-24)."""
    n = np.arange(0, N)
    g = (N - n + 1) * np.cos(np.pi * n / (N + 1)) + np.sin(np.pi * n / (N + 1)) * (1 / np.tan(np.pi / (N + 1)))
    return g / (N + 1)


def moments_delta(Ef, N):
    """Chebyshev moments of delta(E - Ef) on the rescaled axis
    (jclsquant/kernel_and_moments.py:72-78): [1, 2cos(n acos Ef)] / (pi sqrt(1 - Ef^2))."""
    n = np.arange(1, N)
    body = 2 * np.cos(n * np.arccos(Ef))
    return np.concatenate((np.array([1.0]), body)) / (pi * np.sqrt(1 - Ef ** 2))


def moments_delta_table(Ef_tilde, N):
    """moments_delta for a vector of energies at once: array [len(Ef), N]."""
    e = np.asarray(Ef_tilde, dtype=np.float64).reshape(-1, 1)
    n = np.arange(N).reshape(1, -1)
    tab = 2 * np.cos(n * np.arccos(e))
    tab[:, 0] = 1.0
    return tab / (pi * np.sqrt(1 - e ** 2))


def moments_FD_T0(Ef, N):
    """Zero-temperature Fermi-Dirac step moments (jclsquant/kernel_and_moments.py:27-31)."""
    n = np.arange(1, N)
    body = -2 * np.sin(n * np.arccos(Ef)) / (n * pi)
    return np.concatenate((np.array([1 - np.arccos(Ef) / pi]), body))


def moments_FD_T(Ef, T_mod, N):
    """Finite-temperature Fermi-Dirac moments by Simpson quadrature on 2N points
    (jclsquant/kernel_and_moments.py:87-103)."""
    import warnings

    from scipy.integrate import simpson

    E = np.linspace(-1 + 1e-3, 1 - 1e-3, 2 * N)
    mu = np.zeros(N)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)
        fd = 1 / (1 + np.exp((E - Ef) / T_mod))
        w = 1 / (pi * np.sqrt(1 - E ** 2))
        for m in range(N):
            f = fd * np.cos(m * np.arccos(E)) * w
            val = simpson(f, x=E, dx=np.abs(E[1] - E[0]))
            mu[m] = val if m == 0 else 2 * val
    return mu


def moments_FD(N, FD):
    """Chebyshev moments of a tabulated occupation FD(E) on linspace(-1 + 1e-3, 1 - 1e-3, len(FD))
    by Simpson quadrature, the n = 0 weight halved (jclsquant/kernel_and_moments.py:107-115)."""
    from scipy.integrate import simpson

    FD = np.asarray(FD)
    E = np.linspace(-1 + 1e-3, 1 - 1e-3, len(FD))
    w = FD / (pi * np.sqrt(1 - E ** 2))
    theta = np.arccos(E)
    mu = np.zeros(N)
    for m in range(N):
        mu[m] = 2 * simpson(w * np.cos(m * theta), x=E, dx=np.abs(E[1] - E[0]))
    mu[0] = mu[0] / 2
    return mu


def moments_Gmas(Ef, N):
    """Retarded Green's function moments (jclsquant/kernel_and_moments.py:47-54)."""
    n = np.arange(1, N)
    s = np.sqrt(1 - Ef ** 2)
    body = -2j * np.exp(-1j * n * np.arccos(Ef)) / s
    return np.concatenate((np.array([-1j / s]), body))


def moments_Gmas_2(Ef, broadening, N):
    """Retarded Green's function moments at the complex energy z = Ef + i*broadening
    (jclsquant/kernel_and_moments.py:33-41): [-i/s, 2 (z - i s)^n / (i s)] with s = sqrt(1 - z^2)."""
    z = Ef + 1j * broadening
    s = np.sqrt(1 - z ** 2)
    n = np.arange(1, N)
    body = 2 * (z - 1j * s) ** n / (1j * s)
    return np.concatenate((np.array([-1j / s]), body))


def moments_delta_2(Ef, broadening, M):
    """Lorentzian-broadened delta moments, -Im G+ / pi (jclsquant/kernel_and_moments.py:43-44)."""
    return -np.imag(moments_Gmas_2(Ef, broadening, M)) / np.pi


def moments_Gmin(Ef, N):
    """Advanced Green's function moments (jclsquant/kernel_and_moments.py:56-62)."""
    n = np.arange(1, N)
    s = np.sqrt(1 - Ef ** 2)
    body = 2j * np.exp(1j * n * np.arccos(Ef)) / s
    return np.concatenate((np.array([1j / s]), body))


def moments_Gsum(Ef, N):
    """G+ + G- moments (jclsquant/kernel_and_moments.py:64-69)."""
    n = np.arange(1, N)
    body = -4 * np.sin(n * np.arccos(Ef)) / np.sqrt(1 - Ef ** 2)
    return np.concatenate((np.array([0.0]), body))


def moments_U(t, N):
    """Time-evolution moments of exp(-i H t): [J_0(t), 2(-i)^n J_n(t)]
    (jclsquant/kernel_and_moments.py:82-85)."""
    from scipy.special import jv

    n = np.arange(1, N)
    body = 2 * (-1j) ** n * jv(n, t)
    return np.concatenate((np.array([jv(0, t)]), body))


def moments_by_matrix(moments_vec, matrix):
    """sum_i moments_vec[i] * matrix[i, :] (jclsquant/kernel_and_moments.py:11-15)."""
    return np.asarray(moments_vec) @ np.asarray(matrix)
