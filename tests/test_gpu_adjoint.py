"""Reverse-mode KPM: libkpm's adjoint recursion against the FP64 oracle
gradient (which is itself checked against finite differences on the CPU), and
the autograd DOS loss against central finite differences of the GPU forward.

Tolerances: per-slot gradient vs oracle <= 1e-10 * max|grad|; autograd vs
central differences (h = 1e-6) <= 1e-6 * max(|grad|) + 1e-8.  Both backward
arithmetics are held to them: FP64 and float-float (KPM_C128F).
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu


def _problem(nx=6, ny=5, W=0.8, seed=3):
    from minijclsquant_gb300 import lattice

    arr = lattice.honeycomb_arrays(nx, ny, t=-2.7, W=W, seed=seed, with_geometry=False)
    from minijclsquant_gb300.ell_matrix import gershgorin_bounds_ell

    b = gershgorin_bounds_ell(arr["data"], arr["indices"], arr["n"], 1.01)
    return arr, arr["data"] / b[1]


@pytest.mark.parametrize("backward", ["c128", "c128f"])
@pytest.mark.parametrize("M,ckpt,R", [(2, 2, 1), (3, 2, 2), (50, 7, 4), (64, 32, 4), (40, 64, 8), (97, 3, 2)])
def test_adjoint_gradient_matches_oracle(cuda_lib, M, ckpt, R, backward):
    from minijclsquant_gb300 import _capi

    import torch

    arr, d = _problem()
    n, L = arr["n"], arr["len_row"]
    from minijclsquant_gb300 import device
    from minijclsquant_gb300.observables import random_vector_generator

    op = device.DeviceELL(d, arr["indices"], L)
    vs = np.stack([random_vector_generator(n, 70 + r) for r in range(R)])
    c = np.random.default_rng(M).normal(size=M)
    tv = torch.from_numpy(vs).cuda()
    mu = torch.empty((R, M), dtype=torch.complex128, device="cuda")
    assert cuda_lib.kpm_adjoint_forward(op.handle, R, M, ckpt, tv.data_ptr(), mu.data_ptr(), None) == 0
    tc = torch.from_numpy(c).cuda()
    g = torch.empty(n * L, dtype=torch.float64, device="cuda")
    assert cuda_lib.kpm_adjoint_backward_ex(op.handle, tc.data_ptr(), g.data_ptr(), _capi.dtype_code(backward),
                                            None) == 0
    assert cuda_lib.kpm_ell_check(op.handle, None) == 0
    g = g.cpu().numpy()
    ref = sum(oracle.adjoint_grad(M, d, arr["indices"], L, vs[r], c) for r in range(R))
    assert np.max(np.abs(g - ref)) <= 1e-10 * np.max(np.abs(ref))
    for r in range(R):  # the forward moments are the plain ones
        assert oracle.moment_tolerance_ok(mu[r].cpu().numpy(),
                                          oracle.rec_A_tab(M, d, arr["indices"], L, vs[r]), 1e-10)[0]


@pytest.mark.parametrize("backward", ["c128", "c128f"])
def test_autograd_dos_loss_matches_finite_differences(cuda_lib, backward):
    import torch

    from minijclsquant_gb300 import adjoint

    rng = np.random.default_rng(0)
    nx, ny = 8, 7
    n = 2 * nx * ny
    plan0 = adjoint.DosPlan(nx, ny, M=96, R=2, n_energies=64, ckpt=8,
                            onsite0=rng.uniform(-0.5, 0.5, n), hopping0=-2.7 + rng.uniform(-0.1, 0.1, 3 * nx * ny),
                            backward=backward)
    onsite = torch.tensor(rng.uniform(-0.5, 0.5, n), dtype=torch.float64, device="cuda", requires_grad=True)
    hop = torch.tensor(-2.7 + rng.uniform(-0.1, 0.1, plan0.n_bonds), dtype=torch.float64, device="cuda",
                       requires_grad=True)
    target = adjoint.kpm_dos(onsite.detach() * 0.7, hop.detach() * 1.02, plan0).detach()
    loss = adjoint.dos_l2_loss(onsite, hop, plan0, target)
    loss.backward()
    go, gh = onsite.grad.cpu().numpy(), hop.grad.cpu().numpy()
    h = 1e-6
    scale = max(np.max(np.abs(go)), np.max(np.abs(gh)))
    with torch.no_grad():
        for which, idx in [("o", 0), ("o", 17), ("o", n - 1), ("h", 0), ("h", 5), ("h", plan0.n_bonds - 1)]:
            p = onsite if which == "o" else hop
            old = p[idx].item()
            p[idx] = old + h
            lp = adjoint.dos_l2_loss(onsite, hop, plan0, target).item()
            p[idx] = old - h
            lm = adjoint.dos_l2_loss(onsite, hop, plan0, target).item()
            p[idx] = old
            fd = (lp - lm) / (2 * h)
            an = (go if which == "o" else gh)[idx]
            assert abs(an - fd) <= 1e-6 * scale + 1e-8, (which, idx, an, fd)


def test_set_values_rejects_imaginary_part_on_real_operator(cuda_lib):
    import torch

    from minijclsquant_gb300 import _capi, device

    arr, d = _problem(3, 3)
    op = device.DeviceELL(d, arr["indices"], arr["len_row"])
    bad = torch.from_numpy(d + 0.25j).cuda()
    assert cuda_lib.kpm_ell_set_values(op.handle, bad.data_ptr(), _capi.KPM_FLAG_DEVICE_PTRS, None) == 0
    assert cuda_lib.kpm_ell_check(op.handle, None) == _capi.KPM_ERR_DTYPE
    assert cuda_lib.kpm_ell_check(op.handle, None) == 0
