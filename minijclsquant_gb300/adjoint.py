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

``KuboPlan`` / ``kpm_sigma(onsite, hopping, plan)`` do the same for the Kubo-Greenwood
conductivity sigma(E) of kubo.py: the velocity V = -i H o dx (jclsquant/modifiers.py:56-79)
depends on the hoppings too, so the gradient flows through both operators.  With
C_nm = sum_E dL/dsigma(E) P(E) w_n(E) w_m(E) (w_n = h_n T_n(E/a), P = 2 / (Omega a^2 (1 - e^2))),
the loss depends on the parameters through

    F = (1/R) sum_r Re sum_nm C_nm <v| V T_n(H~) V T_m(H~) |v>,

whose derivative needs, per vector, the tables T_m(H~) v and T_n(H~) V v (all orders: C
couples every n with every m), Q = C T(v) and P = C T(Vv) (two plain GEMMs), and two
reverse (Clenshaw) recursions with per-order sources V Q_k and V P_k:

    dF/dH~_ij = sum_k c_k [conj(lamA_{k+1,i}) (T_k Vv)_j + conj(lamB_{k+1,i}) (T_k v)_j],
    dF/dV_ij  = conj(v_i) lamA_{0,j} + sum_m conj(P_{m,i}) (T_m v)_j,

c_0 = 1, c_k = 2 (libkpm: kpm_cheb_table, kpm_cheb_clenshaw_table, kpm_ell_slot_sum).  A real
parameter entering H_ij by dH and V_ij = -i dx_ij H_ij contributes Re(dF/dH~_ij) / a +
dx_ij Im(dF/dV_ij) per unit change.  Everything is complex128; the moment-matrix GEMMs run in
cuBLAS FP64 (plain library GEMMs).
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


class _HoneycombParams:
    """The honeycomb ELL pattern and the map from its slots to learnable parameters: the
    on-site slot of site i -> onsite[i], both slots of an undirected bond -> one hopping (so
    the operator stays real symmetric), numbered by the smaller of the two slot indices."""

    def _init_params(self, nx, ny, t, with_geometry):
        arr = lattice.honeycomb_arrays(nx, ny, t=t, W=0.0, onsite=np.zeros(2 * nx * ny), with_geometry=with_geometry)
        self.n = arr["n"]
        self.L = arr["len_row"]
        n, L = self.n, self.L
        idx = arr["indices"]
        partner = arr["partner"]
        rows = np.repeat(np.arange(n), L)
        diag = (idx == rows) & (partner < 0)
        bond = partner >= 0
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
        dev = torch.device("cuda")
        self.d_diag_slot = torch.from_numpy(self.diag_slot).to(dev)
        self.d_diag_site = torch.from_numpy(self.diag_site).to(dev)
        self.d_bond_slot = torch.from_numpy(self.bond_slot).to(dev)
        self.d_bond_of_slot = torch.from_numpy(self.bond_of_slot).to(dev)
        return arr

    def values(self, onsite, hopping):
        """Reference-layout ELL values (complex128, unscaled) of the parameters (numpy)."""
        data = np.zeros(self.n * self.L, dtype=np.complex128)
        data[self.diag_slot] = onsite[self.diag_site]
        data[self.bond_slot] = hopping[self.bond_of_slot]
        return data

    def real_values(self, onsite, hopping):
        """Unscaled real ELL values on the GPU from parameter tensors (float64, CUDA)."""
        data = torch.zeros(self.n * self.L, dtype=torch.float64, device=onsite.device)
        data[self.d_diag_slot] = onsite[self.d_diag_site]
        data[self.d_bond_slot] = hopping[self.d_bond_of_slot]
        return data

    def fold(self, g_slot):
        """Per-slot derivatives (float64, AoS) summed into (d/d onsite, d/d hopping)."""
        g_onsite = torch.zeros(self.n, dtype=torch.float64, device=g_slot.device)
        g_onsite.index_add_(0, self.d_diag_site, g_slot[self.d_diag_slot])
        g_hop = torch.zeros(self.n_bonds, dtype=torch.float64, device=g_slot.device)
        g_hop.index_add_(0, self.d_bond_of_slot, g_slot[self.d_bond_slot])
        return g_onsite, g_hop


class DosPlan(_HoneycombParams):
    def __init__(self, nx, ny, M, R=4, n_energies=512, ckpt=32, onsite0=None, hopping0=None, t=-2.7,
                 vector_seed=1000, bounds_factor=1.01, energy_margin=1e-3, backward="c128f"):
        """backward: arithmetic of the adjoint pass, "c128" (FP64) or "c128f" (float-float on
        the FP32 pipe, ~1e-14 of the FP64 gradient); the forward is always FP64."""
        self.backward_dtype = _capi.dtype_code(backward)
        self._init_params(nx, ny, t, with_geometry=False)
        self.M = int(M)
        self.R = int(R)
        self.ckpt = int(ckpt)
        n, L = self.n, self.L
        if onsite0 is None:
            onsite0 = np.zeros(n)
        if hopping0 is None:
            hopping0 = np.full(self.n_bonds, t)
        data0 = self.values(np.asarray(onsite0, dtype=np.float64), np.asarray(hopping0, dtype=np.float64))
        self.bounds = gershgorin_bounds_ell(data0, self.indices, n, factor=bounds_factor)
        self.a = 0.5 * (self.bounds[1] - self.bounds[0])
        self.op = DeviceELL(data0 / self.a, self.indices, L)
        if not self.op.is_real:
            raise ValueError("the learnable Hamiltonian must be real")
        dev = torch.device("cuda")
        self.v = torch.from_numpy(np.stack([random_vector_generator(n, vector_seed + r) for r in range(self.R)])).to(dev)
        E = np.linspace(self.bounds[0] + energy_margin, self.bounds[1] - energy_margin, int(n_energies))
        self.energies = E
        table = moments_delta_table(E / self.a, self.M) * JacksonKernel(self.M)[None, :]
        self.table = torch.from_numpy(np.ascontiguousarray(table)).to(dev)  # [E, M] float64

    def device_values(self, onsite, hopping):
        """Rescaled values H/a on the GPU from parameter tensors (float64, CUDA)."""
        data = self.real_values(onsite, hopping) / self.a
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
        g_onsite, g_hop = plan.fold(g / plan.a)
        return g_onsite, g_hop, None


def kpm_dos(onsite, hopping, plan):
    """Differentiable DOS rho(E) on plan.energies (unnormalised, as jclsquant's kpm_dos)."""
    return _KPMDos.apply(onsite, hopping, plan)


def dos_l2_loss(onsite, hopping, plan, target):
    """sum_E (rho(E) - target(E))^2."""
    rho = kpm_dos(onsite, hopping, plan)
    return torch.sum((rho - target) ** 2)


class KuboPlan(_HoneycombParams):
    """Everything of the differentiable Kubo-Greenwood conductivity except the parameters:
    the honeycomb pattern and parameter map, the bond displacements along `direction`, the
    spectral bound a (Gershgorin bound of the initial parameters x bounds_factor, then held
    constant), Nm, the R random-phase vectors, the energies, Omega."""

    def __init__(self, nx, ny, Nm, R=4, n_energies=64, energies=None, onsite0=None, hopping0=None, t=-2.7,
                 vector_seed=2000, bounds_factor=1.01, direction="x", omega=None, energy_fraction=0.9):
        arr = self._init_params(nx, ny, t, with_geometry=True)
        self.Nm = int(Nm)
        self.R = int(R)
        n, L = self.n, self.L
        d = arr["dx"] if direction in ("x", 0) else arr["dy"]
        self.disp = torch.from_numpy(np.ascontiguousarray(np.real(d))).cuda()  # x_j - x_i per slot (AoS)
        if onsite0 is None:
            onsite0 = np.zeros(n)
        if hopping0 is None:
            hopping0 = np.full(self.n_bonds, t)
        data0 = self.values(np.asarray(onsite0, dtype=np.float64), np.asarray(hopping0, dtype=np.float64))
        self.bounds = gershgorin_bounds_ell(data0, self.indices, n, factor=bounds_factor)
        self.a = 0.5 * (self.bounds[1] - self.bounds[0])
        self.omega = float(omega) if omega is not None else nx * ny * (np.sqrt(3.0) * lattice.A_CC) ** 2 * np.sqrt(3.0) / 2
        self.op_h = DeviceELL(data0 / self.a, self.indices, L)
        self.op_v = DeviceELL(-1j * np.real(d) * data0, self.indices, L, complex_values=True)
        dev = torch.device("cuda")
        self.v = torch.from_numpy(np.stack([random_vector_generator(n, vector_seed + r) for r in range(self.R)])).to(dev)
        if energies is None:
            energies = np.linspace(-energy_fraction * self.a, energy_fraction * self.a, int(n_energies))
        self.energies = np.asarray(energies, dtype=np.float64)
        e = self.energies / self.a
        h = JacksonKernel(self.Nm) * np.where(np.arange(self.Nm) == 0, 1.0, 2.0)
        w = np.cos(np.arange(self.Nm)[None, :] * np.arccos(e)[:, None]) * h[None, :]
        self.w = torch.from_numpy(np.ascontiguousarray(w)).to(dev)                       # [E, Nm]
        self.pref = torch.from_numpy(2.0 / (self.omega * self.a * self.a * (1.0 - e * e))).to(dev)  # [E]
        cp = np.full(self.Nm - 1, 2.0)
        cp[0] = 1.0
        self.c_adj = torch.from_numpy(cp).to(dev)  # c_k of the adjoint sums, k = 0 .. Nm-2

    def set_operators(self, onsite, hopping):
        """H~ = H / a and V = -i H o d on the device from parameter tensors."""
        lib = _capi.lib()
        stream = int(torch.cuda.current_stream().cuda_stream)
        d = self.real_values(onsite, hopping)
        hv = torch.complex(d / self.a, torch.zeros_like(d)).contiguous()
        vv = torch.complex(torch.zeros_like(d), -self.disp * d).contiguous()
        _capi.check(lib.kpm_ell_set_values(self.op_h.handle, hv.data_ptr(), _capi.KPM_FLAG_DEVICE_PTRS, stream),
                    "kpm_ell_set_values")
        _capi.check(lib.kpm_ell_set_values(self.op_v.handle, vv.data_ptr(), _capi.KPM_FLAG_DEVICE_PTRS, stream),
                    "kpm_ell_set_values")

    # -- libkpm calls on one vector -------------------------------------------------
    def _table(self, x, with_v=False):
        lib = _capi.lib()
        stream = int(torch.cuda.current_stream().cuda_stream)
        tab = torch.empty((self.Nm, self.n), dtype=torch.complex128, device=x.device)
        vtab = torch.empty_like(tab) if with_v else None
        _capi.check(lib.kpm_cheb_table(self.op_h.handle, self.op_v.handle if with_v else None, self.Nm, x.data_ptr(),
                                       tab.data_ptr(), vtab.data_ptr() if with_v else None, stream), "kpm_cheb_table")
        return tab, vtab

    def _apply_v(self, x):
        lib = _capi.lib()
        y = torch.empty_like(x)
        _capi.check(lib.kpm_ell_dot(self.op_v.handle, 1.0, 0.0, 0.0, 0.0, x.data_ptr(), y.data_ptr(), 1,
                                    int(torch.cuda.current_stream().cuda_stream)), "kpm_ell_dot")
        return y

    def _clenshaw(self, z):
        lib = _capi.lib()
        lam = torch.empty_like(z)
        _capi.check(lib.kpm_cheb_clenshaw_table(self.op_h.handle, self.op_v.handle, self.Nm, z.data_ptr(),
                                                lam.data_ptr(), int(torch.cuda.current_stream().cuda_stream)),
                    "kpm_cheb_clenshaw_table")
        return lam

    def _slot_sum(self, K, coef, A, B, out, accumulate=True):
        lib = _capi.lib()
        _capi.check(lib.kpm_ell_slot_sum(self.op_h.handle, int(K), coef.data_ptr() if coef is not None else None,
                                         A.data_ptr(), self.n, B.data_ptr(), self.n, int(accumulate), out.data_ptr(),
                                         int(torch.cuda.current_stream().cuda_stream)), "kpm_ell_slot_sum")

    def mu_nm(self):
        """mu[n][m] = (1/R) sum_r <v_r| V T_n(H~) V T_m(H~) |v_r> (complex128) for the operators
        last set: tables of T_n(H~) V v and V T_m(H~) v per vector, one FP64 GEMM."""
        mu = torch.zeros((self.Nm, self.Nm), dtype=torch.complex128, device=self.v.device)
        for r in range(self.R):
            v = self.v[r].contiguous()
            _, vtv = self._table(v, with_v=True)
            tu, _ = self._table(self._apply_v(v))
            mu += tu.conj() @ vtv.transpose(0, 1)
            del tu, vtv
        return mu / self.R

    def sigma_from_mu(self, mu):
        """sigma(E) [e^2/h] on self.energies (kubo.sigma_from_mu on the device)."""
        return self.pref * torch.einsum("en,nm,em->e", self.w, mu.real, self.w)

    def slot_gradient(self, C):
        """d/d(slot value) of F = (1/R) sum_r Re sum_nm C_nm <v_r|V T_n V T_m|v_r> for every ELL
        slot (float64, AoS): Re(dF/dH~) / a + d Im(dF/dV)."""
        gH = torch.zeros(self.n * self.L, dtype=torch.complex128, device=C.device)
        gV = torch.zeros_like(gH)
        Cr = C.to(torch.float64).contiguous()
        for r in range(self.R):
            v = self.v[r].contiguous()
            u = self._apply_v(v)
            tv, _ = self._table(v)
            tu, _ = self._table(u)
            # Q = C T(v), P = C T(Vv): real C on the (re, im) pairs of every entry
            Q = torch.view_as_complex((Cr @ torch.view_as_real(tv).reshape(self.Nm, -1)).reshape(self.Nm, self.n, 2))
            P = torch.view_as_complex((Cr @ torch.view_as_real(tu).reshape(self.Nm, -1)).reshape(self.Nm, self.n, 2))
            lam_a = self._clenshaw(Q.contiguous())
            del Q
            self._slot_sum(self.Nm - 1, self.c_adj, lam_a[1:], tu, gH)
            self._slot_sum(1, None, v, lam_a, gV)
            del lam_a, tu
            self._slot_sum(self.Nm, None, P, tv, gV)
            lam_b = self._clenshaw(P.contiguous())
            del P
            self._slot_sum(self.Nm - 1, self.c_adj, lam_b[1:], tv, gH)
            del lam_b, tv
        return (gH.real / self.a + self.disp * gV.imag) / self.R


class _KPMSigma(torch.autograd.Function):
    @staticmethod
    def forward(ctx, onsite, hopping, plan):
        plan.set_operators(onsite.detach(), hopping.detach())
        mu = plan.mu_nm()
        ctx.plan = plan
        return plan.sigma_from_mu(mu)

    @staticmethod
    def backward(ctx, grad_sigma):
        plan = ctx.plan
        gw = (grad_sigma.to(torch.float64) * plan.pref)[:, None] * plan.w  # [E, Nm]
        C = plan.w.t() @ gw                                                  # [Nm, Nm], symmetric
        g_onsite, g_hop = plan.fold(plan.slot_gradient(C))
        return g_onsite, g_hop, None


def kpm_sigma(onsite, hopping, plan):
    """Differentiable Kubo-Greenwood sigma_xx(E) [e^2/h] on plan.energies."""
    return _KPMSigma.apply(onsite, hopping, plan)


def sigma_l2_loss(onsite, hopping, plan, target):
    """sum_E (sigma(E) - target(E))^2."""
    sig = kpm_sigma(onsite, hopping, plan)
    return torch.sum((sig - target) ** 2)
