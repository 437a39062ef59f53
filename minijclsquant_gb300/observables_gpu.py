"""GPU observables, drop-in for the KPM-path functions of jclsquant/observables_gpu.py.

``kpm_dos_gpu`` / ``kpm_dos_2_gpu`` keep the reference signatures and outputs;
``kpm_sigma_time_gpu`` is the reference's time-domain Kubo correlator
(historical jclsquant observables_gpu, sigma via for_time_sigma).  All
recursions run in libkpm; the operator is uploaded once and cached on the
rescaled matrix object.
"""
from __future__ import annotations

import copy

import numpy as np

from . import device
from .constants import hbar_fs, kb
from .kernel_and_moments import JacksonKernel, moments_FD_T, moments_FD_T0, moments_U
from .modifiers import modifier_bounds, modifier_velocity, modifier_velocity_bounds
from .observables import dos_from_moments, kpm_dos, kpm_n_dos_n, random_vector_generator  # noqa: F401


def kpm_dos_gpu(H, M=None, random_vector=None, *, dtype="c128", n_energies=None):
    """DOS on the GPU (jclsquant/observables_gpu.py:12-42)."""
    return kpm_dos(H, M, random_vector, dtype=dtype, n_energies=n_energies)


def kpm_dos_2_gpu(H, M=None, random_vector_l=None, random_vector_r=None, bounds=True, proyector=None, *,
                  dtype="c128", n_energies=None):
    """DOS with separate bra/ket vectors on the GPU (jclsquant/observables_gpu.py:46-93)."""
    return kpm_n_dos_n(H, M, random_vector_l, random_vector_r, bounds, proyector, dtype=dtype,
                       n_energies=n_energies)


def kpm_sigma_time_gpu(H, direction_1=None, direction_2=None, t_vec=None, Ef=None, Temp=None, M=None,
                       random_vector=None, velocities=None, *, dtype="c128"):
    """Time-dependent Kubo conductivity correlator -i <U_c(t)|V1 U(t)>.

    Follows kpm_sigma_time_gpu of jclsquant's observables_gpu (historical
    version, .history/jclsquant/observables_gpu_20260306165252.py:103-175):
    Bessel moments truncated where |c_m| <= 1e-15, Fermi-Dirac moments times
    Jackson, V2 = H o d / a (rescaled), V1 = -i H o d, and the GPU
    for_time_sigma recursion.  ``dtype="c128f"`` runs the recursion in float-float
    arithmetic (about 48-bit mantissas) on the FP32 pipe.
    """
    if M is None:
        M = int(np.sqrt(H.shape[0]))
    if Ef is None:
        Ef = 0
    if random_vector is None:
        random_vector = random_vector_generator(H.shape[0])
    if t_vec is None:
        t_vec = np.linspace(0, 5 * hbar_fs * M / (np.pi * (0.5 * (H.bounds[1] - H.bounds[0]))), 500)
    delta_t_kpm = t_vec[1] * H.bounds[1] / hbar_fs
    mu_u = moments_U(delta_t_kpm, M)
    m = 0
    while np.abs(mu_u[m]) > 1e-15 and m < M - 1:
        m += 1
    M2 = m
    mu_u = moments_U(delta_t_kpm, M2)
    H_kpm = H.modifier(modifier_bounds)
    if Temp is None or Temp == 0:
        mk_fd = moments_FD_T0(Ef / H.bounds[1], M) * JacksonKernel(M)
    else:
        mk_fd = moments_FD_T(Ef / H.bounds[1], Temp * kb / H.bounds[1], M) * JacksonKernel(M)
    mk_fd = mk_fd.astype(np.complex128)
    if velocities is None:
        V2_kpm = H.modifier(modifier_velocity_bounds, direction_2)
        V1 = H.modifier(modifier_velocity, direction_1)
    else:
        V2_kpm = copy.deepcopy(H)
        V1 = copy.deepcopy(H)
        d1 = V1.dx_vec if direction_1 == "x" else V1.dy_vec
        d2 = V2_kpm.dx_vec if direction_2 == "x" else V2_kpm.dy_vec
        V1.data = np.copy(d1)
        V2_kpm.data = (1j / ((H.bounds[1] - H.bounds[0]) / 2)) * d2 + 0 * V2_kpm.data
    sigma = device.time_sigma(H_kpm.device(), V1.device(), V2_kpm.device(), mu_u.astype(np.complex128), M2, mk_fd, M,
                              len(t_vec), np.asarray(random_vector, dtype=np.complex128), dtype=dtype)
    return -1j * sigma
