"""Differentiable KPM DOS: gradients with respect to on-site potentials and
per-bond hoppings through a hand-written adjoint Chebyshev recursion.

``DosPlan`` fixes everything except the parameters: the honeycomb ELL
pattern, the map from ELL slots to parameters (on-site slot -> site, bond slot
-> undirected bond, both directions of a bond sharing one hopping, so the
operator stays real symmetric), the spectral bound a (held constant: the
Gershgorin bound of the initial parameters times 1.01), the random vectors,
M, the energy grid and the checkpoint interval.

``kpm_dos(onsite, hopping, plan)`` is a ``torch.autograd.Function``: forward
builds H/a on the GPU from the parameters, runs the complex128 recursion
(``kpm_adjoint_forward``, checkpoints every ``ckpt`` orders) and returns the
Jackson-damped DOS averaged over the vectors,

    rho(E) = (1/R) sum_r Re sum_m delta_m(E/a) g_m mu_m^(r)        (FP64);

backward maps dL/drho to c_m, runs the adjoint recursion (``kpm_adjoint_backward_ex``,
float-float arithmetic by default) and folds the per-slot derivatives into on-site
and bond gradients (divided by a).

The reference has no derivatives; the forward quantity is its kpm_dos
(jclsquant/observables.py:26-54) on these parameters.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _capi, lattice
from .device import DeviceELL
from .ell_matrix import gershgorin_bounds_ell
from .kernel_and_moments import JacksonKernel, moments_delta_table
from .observables import random_vector_generator


class DosPlan:
    def __init__(self, nx, ny, M, R=4, n_energies=512, ckpt=32, onsite0=None, hopping0=None, t=-2.7,
                 vector_seed=1000, bounds_factor=1.01, energy_margin=1e-3, backward="c128f"):
        """backward: arithmetic of the adjoint pass, "c128" (FP64) or "c128f" (float-float on
        the FP32 pipe, ~1e-14 of the FP64 gradient); the forward is always FP64."""
        self.backward_dtype = _capi.dtype_code(backward)
        arr = lattice.honeycomb_arrays(nx, ny, t=t, W=0.0, onsite=np.zeros(2 * nx * ny), with_geometry=False)
        self.n = arr["n"]
        self.L = arr["len_row"]
        self.M = int(M)
        self.R = int(R)
        self.ckpt = int(ckpt)
        n, L = self.n, self.L
        idx = arr["indices"]
        partner = arr["partner"]
        rows = np.repeat(np.arange(n), L)
        diag = (idx == rows) & (partner < 0)
        bond = partner >= 0
        # one id per undirected bond: the smaller of the two slot indices
        slot = np.arange(n * L)
        owner = np.where(bond, np.minimum(slot, partner), -1)
        uniq = np.unique(owner[bond])
        bond_id = np.full(n * L, -1, dtype=np.int64)
        bond_id[bond] = np.searchsorted(uniq, owner[bond])
        self.n_bonds = len(uniq)
        self.indices = idx
        self.diag_slot = np.nonzero(diag)[0]             # slot of site i's on-site term, ordered by site
        self.diag_site = rows[self.diag_slot]
        self.bond_slot = np.nonzero(bond)[0]
        self.bond_of_slot = bond_id[self.bond_slot]
        if onsite0 is None:
            onsite0 = np.zeros(n)
        if hopping0 is None:
            hopping0 = np.full(self.n_bonds, t)
        data0 = self.values(np.asarray(onsite0, dtype=np.float64), np.asarray(hopping0, dtype=np.float64))
        self.bounds = gershgorin_bounds_ell(data0, idx, n, factor=bounds_factor)
        self.a = 0.5 * (self.bounds[1] - self.bounds[0])
        self.op = DeviceELL(data0 / self.a, idx, L)
        if not self.op.is_real:
            raise ValueError("the learnable Hamiltonian must be real")
        dev = torch.device("cuda")
        self.d_diag_slot = torch.from_numpy(self.diag_slot).to(dev)
        self.d_diag_site = torch.from_numpy(self.diag_site).to(dev)
        self.d_bond_slot = torch.from_numpy(self.bond_slot).to(dev)
        self.d_bond_of_slot = torch.from_numpy(self.bond_of_slot).to(dev)
        self.v = torch.from_numpy(np.stack([random_vector_generator(n, vector_seed + r) for r in range(self.R)])).to(dev)
        E = np.linspace(self.bounds[0] + energy_margin, self.bounds[1] - energy_margin, int(n_energies))
        self.energies = E
        table = moments_delta_table(E / self.a, self.M) * JacksonKernel(self.M)[None, :]
        self.table = torch.from_numpy(np.ascontiguousarray(table)).to(dev)  # [E, M] float64

    def values(self, onsite, hopping):
        """Reference-layout ELL values (complex128, unscaled) of the parameters (numpy)."""
        data = np.zeros(self.n * self.L, dtype=np.complex128)
        data[self.diag_slot] = onsite[self.diag_site]
        data[self.bond_slot] = hopping[self.bond_of_slot]
        return data

    def device_values(self, onsite, hopping):
        """Rescaled values H/a on the GPU from parameter tensors (float64, CUDA)."""
        data = torch.zeros(self.n * self.L, dtype=torch.float64, device=onsite.device)
        data[self.d_diag_slot] = onsite[self.d_diag_site]
        data[self.d_bond_slot] = hopping[self.d_bond_of_slot]
        data = data / self.a
        return torch.complex(data, torch.zeros_like(data))


class _KPMDos(torch.autograd.Function):
    @staticmethod
    def forward(ctx, onsite, hopping, plan):
        lib = _capi.lib()
        stream = int(torch.cuda.current_stream().cuda_stream)
        vals = plan.device_values(onsite.detach(), hopping.detach()).contiguous()
        _capi.check(lib.kpm_ell_set_values(plan.op.handle, vals.data_ptr(), _capi.KPM_FLAG_DEVICE_PTRS, stream),
                    "kpm_ell_set_values")
        mu = torch.empty((plan.R, plan.M), dtype=torch.complex128, device=onsite.device)
        _capi.check(lib.kpm_adjoint_forward(plan.op.handle, plan.R, plan.M, plan.ckpt, plan.v.data_ptr(),
                                            mu.data_ptr(), stream), "kpm_adjoint_forward")
        ctx.plan = plan
        mu_mean = mu.real.mean(dim=0)
        return plan.table @ mu_mean

    @staticmethod
    def backward(ctx, grad_rho):
        plan = ctx.plan
        lib = _capi.lib()
        stream = int(torch.cuda.current_stream().cuda_stream)
        c = (plan.table.t() @ grad_rho.to(torch.float64)) / plan.R
        c = c.contiguous()
        g = torch.empty(plan.n * plan.L, dtype=torch.float64, device=grad_rho.device)
        _capi.check(lib.kpm_adjoint_backward_ex(plan.op.handle, c.data_ptr(), g.data_ptr(), plan.backward_dtype,
                                                stream), "kpm_adjoint_backward_ex")
        g = g / plan.a
        g_onsite = torch.zeros(plan.n, dtype=torch.float64, device=g.device)
        g_onsite.index_add_(0, plan.d_diag_site, g[plan.d_diag_slot])
        g_hop = torch.zeros(plan.n_bonds, dtype=torch.float64, device=g.device)
        g_hop.index_add_(0, plan.d_bond_of_slot, g[plan.d_bond_slot])
        return g_onsite, g_hop, None


def kpm_dos(onsite, hopping, plan):
    """Differentiable DOS rho(E) on plan.energies (unnormalised, as jclsquant's kpm_dos)."""
    return _KPMDos.apply(onsite, hopping, plan)


def dos_l2_loss(onsite, hopping, plan, target):
    """sum_E (rho(E) - target(E))^2."""
    rho = kpm_dos(onsite, hopping, plan)
    return torch.sum((rho - target) ** 2)
