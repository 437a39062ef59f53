"""Kubo-Greenwood DC conductivity from the KPM double expansion.

    sigma_xx(E) = (pi hbar e^2 / Omega) Tr[ v_x delta(E - H) v_x delta(E - H) ]

with v_x = -V/hbar, V = -i H o dx (jclsquant's modifier_velocity convention,
jclsquant/modifiers.py:56-79) and
delta(E - H) = (1/a) sum_n h_n T_n(E~) T_n(H~) / (pi sqrt(1 - E~^2)),
h_n = (2 - delta_{n0}) g_n (Jackson), gives, in units of e^2/h,

    sigma(E) = 2 / (Omega a^2 (1 - E~^2)) * sum_{n,m} h_n h_m T_n(E~) T_m(E~) Re mu_nm,

mu_nm = Tr[V T_n(H~) V T_m(H~)] estimated with random-phase vectors on the GPU
(``kpm_mu_nm``: complex64 recursions, 3xTF32 tensor-core contraction).  This
is the standard double-Chebyshev form (A. Weisse et al., Rev. Mod. Phys. 78,
275 (2006); Garcia, Covaci, Rappoport, PRL 114, 116602 (2015)).  The reference
has no such observable (its conductivity is the time-domain correlator, see
observables_gpu.kpm_sigma_time_gpu), so there is no parity pin for it.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _capi
from .device import DeviceELL
from .kernel_and_moments import JacksonKernel
from .modifiers import modifier_bounds, modifier_velocity
from .observables import random_vector_generator


def mu_nm(h_op: DeviceELL, v_op: DeviceELL, Nm, vectors, stream=None):
    """mu[n][m] = (1/R) sum_r <v_r| V T_n(H) V T_m(H) |v_r>, n, m < Nm (<= 256)."""
    Nm = int(Nm)
    was_np = not isinstance(vectors, torch.Tensor)
    tv = torch.from_numpy(np.ascontiguousarray(np.atleast_2d(vectors), dtype=np.complex128)).cuda() if was_np \
        else vectors.to(torch.complex128).contiguous()
    if tv.dim() == 1:
        tv = tv.reshape(1, -1)
    R = int(tv.shape[0])
    mu = torch.empty((Nm, Nm), dtype=torch.complex128, device=tv.device)
    s = stream if stream is not None else torch.cuda.current_stream()
    _capi.check(_capi.lib().kpm_mu_nm(h_op.handle, v_op.handle, R, Nm, tv.data_ptr(), mu.data_ptr(),
                                      int(s.cuda_stream)), "kpm_mu_nm")
    return mu.cpu().numpy() if was_np else mu


def sigma_from_mu(mu, bounds, omega, energies=None, n_energies=None):
    """sigma(E) in e^2/h (array [n_E, 2]: E, sigma) from mu_nm of the physical velocity V."""
    mu = np.asarray(mu)
    Nm = mu.shape[0]
    a = 0.5 * (bounds[1] - bounds[0])
    if energies is None:
        n_e = 2 * Nm + 1 if n_energies is None else int(n_energies)
        energies = np.linspace(bounds[0] + 1e-3, bounds[1] - 1e-3, n_e)
    e = np.asarray(energies, dtype=np.float64) / a
    h = JacksonKernel(Nm) * np.where(np.arange(Nm) == 0, 1.0, 2.0)
    Tn = np.cos(np.arange(Nm)[None, :] * np.arccos(e)[:, None]) * h[None, :]  # [E, Nm]
    core = np.einsum("en,nm,em->e", Tn, np.real(mu), Tn)
    out = np.zeros((len(e), 2))
    out[:, 0] = energies
    out[:, 1] = 2.0 * core / (omega * a * a * (1.0 - e * e))
    return out


def kpm_sigma_kubo_greenwood_gpu(H, direction="x", Nm=256, R=4, seed=1000, n_energies=None):
    """Kubo-Greenwood sigma_xx(E) [e^2/h] of an ell_matrix with dx_vec/dy_vec and Omega set."""
    H_kpm = H.modifier(modifier_bounds)
    V = H.modifier(modifier_velocity, direction)
    hop = H_kpm.device()
    vop = V.device()
    n = int(H.shape[0])
    vs = np.stack([random_vector_generator(n, seed + r) for r in range(R)])
    mu = mu_nm(hop, vop, Nm, vs)
    return sigma_from_mu(mu, H.bounds, H.Omega, n_energies=n_energies)
