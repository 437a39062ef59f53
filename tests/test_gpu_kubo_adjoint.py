"""Gradients of a Kubo-Greenwood conductivity loss (adjoint.KuboPlan, kpm_sigma) with respect
to on-site potentials and per-bond hoppings, through H~ = H / a and V = -i H o dx
(jclsquant/modifiers.py:56-79).

Checked against
* an FP64 restatement: the same loss written densely in torch (T_n(H~) as dense matrices,
  mu_nm = (1/R) sum_r v^H V T_n V T_m v, sigma(E), L2 loss) and differentiated by torch's
  autograd on the CPU, a route that shares nothing with the libkpm adjoint;
* central finite differences of the FP64 loss at h = 1e-6 on 64 seeded parameters, within
  1e-6 of the largest gradient entry.
The reference has no derivatives (parity unpinned); the forward quantity is kubo.py's
sigma(E), whose moment matrix is also checked against the dense restatement.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _plan(cells=6, Nm=40, R=2, E=23, seed=4):
    from minijclsquant_gb300 import adjoint

    rng = np.random.default_rng(seed)
    n = 2 * cells * cells
    on0 = rng.uniform(-0.5, 0.5, n)
    n_bonds = 3 * cells * cells  # three bonds per primitive cell (periodic honeycomb)
    hop0 = -2.7 + rng.uniform(-0.1, 0.1, n_bonds)
    plan = adjoint.KuboPlan(cells, cells, Nm, R=R, n_energies=E, onsite0=on0, hopping0=hop0,
                            vector_seed=300 + seed)
    assert plan.n_bonds == n_bonds
    return plan, on0, hop0, rng


def _dense_loss(plan, onsite, hopping, target):
    """The loss restated densely in torch (float64 / complex128), differentiable by autograd."""
    import torch

    n, L = plan.n, plan.L
    rows = torch.from_numpy(np.repeat(np.arange(n), L))
    cols = torch.from_numpy(plan.indices.astype(np.int64))
    d = torch.zeros(n * L, dtype=torch.float64)
    d = d.index_put((torch.from_numpy(plan.diag_slot),), onsite[torch.from_numpy(plan.diag_site)])
    d = d.index_put((torch.from_numpy(plan.bond_slot),), hopping[torch.from_numpy(plan.bond_of_slot)])
    disp = plan.disp.cpu()
    H = torch.zeros((n, n), dtype=torch.complex128).index_put((rows, cols), (d / plan.a).to(torch.complex128),
                                                              accumulate=True)
    V = torch.zeros((n, n), dtype=torch.complex128).index_put((rows, cols), torch.complex(0 * d, -disp * d),
                                                              accumulate=True)
    T = [torch.eye(n, dtype=torch.complex128), H]
    for m in range(2, plan.Nm):
        T.append(2 * H @ T[-1] - T[-2])
    T = torch.stack(T[: plan.Nm])
    mu = torch.zeros((plan.Nm, plan.Nm), dtype=torch.complex128)
    for v in plan.v.cpu():
        R_m = V @ (T @ v).T            # columns V T_m v
        L_n = T @ (V @ v)              # rows T_n V v
        mu = mu + L_n.conj() @ R_m
    mu = mu / plan.R
    w, pref = plan.w.cpu(), plan.pref.cpu()
    sig = pref * torch.einsum("en,nm,em->e", w, mu.real, w)
    return torch.sum((sig - target) ** 2), mu, sig


def test_kubo_sigma_gradient_matches_dense_autograd(cuda_lib):
    import torch

    from minijclsquant_gb300 import adjoint

    plan, on0, hop0, rng = _plan()
    with torch.no_grad():
        sig0 = adjoint.kpm_sigma(torch.tensor(on0, device="cuda"), torch.tensor(hop0, device="cuda"), plan)
    target = (0.8 * sig0).cpu()  # a target the loss is not flat at
    onsite = torch.tensor(on0, device="cuda", requires_grad=True)
    hop = torch.tensor(hop0, device="cuda", requires_grad=True)
    loss = adjoint.sigma_l2_loss(onsite, hop, plan, target.cuda())
    loss.backward()
    te = torch.tensor(on0, requires_grad=True)
    th = torch.tensor(hop0, requires_grad=True)
    dloss, dmu, dsig = _dense_loss(plan, te, th, target)
    dloss.backward()
    assert abs(loss.item() - dloss.item()) <= 1e-11 * abs(dloss.item())
    mu = plan.mu_nm().cpu()
    assert torch.max(torch.abs(mu - dmu)) <= 1e-12 * torch.max(torch.abs(dmu))
    scale = max(torch.max(torch.abs(te.grad)).item(), torch.max(torch.abs(th.grad)).item())
    assert scale > 0
    err = max(torch.max(torch.abs(onsite.grad.cpu() - te.grad)).item(),
              torch.max(torch.abs(hop.grad.cpu() - th.grad)).item()) / scale
    assert err <= 1e-10, err
    # both parameter kinds carry gradient
    assert torch.max(torch.abs(th.grad)).item() > 1e-3 * scale and torch.max(torch.abs(te.grad)).item() > 1e-3 * scale


def test_kubo_sigma_gradient_matches_central_differences(cuda_lib):
    import torch

    from minijclsquant_gb300 import adjoint

    plan, on0, hop0, rng = _plan(cells=8, Nm=48, R=2, E=31, seed=9)
    with torch.no_grad():
        target = 0.7 * adjoint.kpm_sigma(torch.tensor(on0, device="cuda"), torch.tensor(hop0, device="cuda"), plan)
    onsite = torch.tensor(on0, device="cuda", requires_grad=True)
    hop = torch.tensor(hop0, device="cuda", requires_grad=True)
    loss = adjoint.sigma_l2_loss(onsite, hop, plan, target)
    loss.backward()
    go, gh = onsite.grad.cpu().numpy(), hop.grad.cpu().numpy()
    scale = max(np.max(np.abs(go)), np.max(np.abs(gh)))
    pick = np.random.default_rng(17)
    params = [("onsite", int(i)) for i in pick.choice(plan.n, 32, replace=False)] + \
             [("hopping", int(i)) for i in pick.choice(plan.n_bonds, 32, replace=False)]
    h = 1e-6
    worst = 0.0
    with torch.no_grad():
        for which, i in params:
            p = onsite if which == "onsite" else hop
            old = p[i].item()
            p[i] = old + h
            lp = adjoint.sigma_l2_loss(onsite, hop, plan, target).item()
            p[i] = old - h
            lm = adjoint.sigma_l2_loss(onsite, hop, plan, target).item()
            p[i] = old
            fd = (lp - lm) / (2 * h)
            an = (go if which == "onsite" else gh)[i]
            worst = max(worst, abs(an - fd) / scale)
    assert worst <= 1e-6, worst


def test_kubo_sigma_forward_is_deterministic(cuda_lib):
    import torch

    from minijclsquant_gb300 import adjoint

    plan, on0, hop0, _ = _plan(cells=6, Nm=32, R=2, E=17, seed=2)
    a = adjoint.kpm_sigma(torch.tensor(on0, device="cuda"), torch.tensor(hop0, device="cuda"), plan)
    b = adjoint.kpm_sigma(torch.tensor(on0, device="cuda"), torch.tensor(hop0, device="cuda"), plan)
    assert torch.equal(a, b)
    assert torch.all(torch.isfinite(a))
