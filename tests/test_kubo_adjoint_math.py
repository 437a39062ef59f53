"""The reverse-mode formulas of the Kubo-Greenwood conductivity loss, restated in numpy on
ELL arrays (tables of T_m v and T_n V v, Q = C T(v), P = C T(Vv), two reverse Clenshaw
recursions with sources V Q_k and V P_k, per-slot sums), against torch autograd through the
dense forward.  CPU only: this pins the derivation the libkpm kernels implement
(kpm_cheb_table, kpm_cheb_clenshaw_table, kpm_ell_slot_sum) independently of the GPU."""
import numpy as np
import pytest

from minijclsquant_gb300 import lattice
from minijclsquant_gb300.kernel_and_moments import JacksonKernel

torch = pytest.importorskip("torch")


def _setup(cells=4, Nm=24, R=2, E=17, seed=1):
    arr = lattice.honeycomb_arrays(cells, cells, t=-2.7, W=0.0, onsite=np.zeros(2 * cells * cells),
                                   with_geometry=True)
    n, L = arr["n"], arr["len_row"]
    idx, partner = arr["indices"], arr["partner"]
    rows = np.repeat(np.arange(n), L)
    diag = (idx == rows) & (partner < 0)
    bond = partner >= 0
    slot = np.arange(n * L)
    owner = np.where(bond, np.minimum(slot, partner), -1)
    uniq = np.unique(owner[bond])
    bond_id = np.full(n * L, -1)
    bond_id[bond] = np.searchsorted(uniq, owner[bond])
    rng = np.random.default_rng(seed)
    p = dict(n=n, L=L, idx=idx, rows=rows, diag=diag, bond=bond, bond_id=bond_id, nb=len(uniq),
             dx=np.real(arr["dx"]), a=9.0, Nm=Nm, R=R)
    p["eps"] = rng.uniform(-0.5, 0.5, n)
    p["hop"] = -2.7 + rng.uniform(-0.1, 0.1, len(uniq))
    p["vs"] = np.exp(1j * rng.uniform(0, 2 * np.pi, (R, n)))
    e = np.linspace(-7, 7, E) / p["a"]
    h = JacksonKernel(Nm) * np.where(np.arange(Nm) == 0, 1.0, 2.0)
    p["W"] = np.cos(np.arange(Nm)[None, :] * np.arccos(e)[:, None]) * h[None, :]
    p["P"] = 2.0 / (3.3 * p["a"] ** 2 * (1 - e * e))
    p["target"] = rng.uniform(0, 1, E)
    return p


def _values(p, eps, hop):
    d = np.zeros(p["n"] * p["L"])
    d[p["diag"]] = eps[p["rows"][p["diag"]]]
    d[p["bond"]] = hop[p["bond_id"][p["bond"]]]
    return d


def _mv(p, data, x):
    n, L = p["n"], p["L"]
    return (data.reshape(n, L) * x[p["idx"].reshape(n, L)]).sum(1)


def _table(p, data, x):
    T = [x.copy(), _mv(p, data, x)]
    for _ in range(2, p["Nm"]):
        T.append(2 * _mv(p, data, T[-1]) - T[-2])
    return np.stack(T[: p["Nm"]])


def _clenshaw(p, dh, ds, z):
    M = len(z)
    lam = [None] * M + [np.zeros(p["n"], complex)] * 2
    for k in range(M - 1, -1, -1):
        lam[k] = _mv(p, ds, z[k]) + (1.0 if k == 0 else 2.0) * _mv(p, dh, lam[k + 1]) - lam[k + 2]
    return np.stack(lam[:M])


def _slot_sum(p, coef, A, B):
    ix = p["idx"].reshape(p["n"], p["L"])
    out = np.zeros((p["n"], p["L"]), complex)
    for k in range(len(A)):
        out += coef[k] * np.conj(A[k])[:, None] * B[k][ix]
    return out.reshape(-1)


def _forward(p, eps, hop):
    d = _values(p, eps, hop)
    dh, dv = d / p["a"], -1j * p["dx"] * d
    mu = np.zeros((p["Nm"], p["Nm"]), complex)
    for v in p["vs"]:
        tu = _table(p, dh, _mv(p, dv, v))
        vtv = np.stack([_mv(p, dv, t) for t in _table(p, dh, v)])
        mu += tu.conj() @ vtv.T / p["R"]
    sig = p["P"] * np.einsum("en,nm,em->e", p["W"], mu.real, p["W"])
    return np.sum((sig - p["target"]) ** 2), sig


def _adjoint(p, eps, hop):
    _, sig = _forward(p, eps, hop)
    C = p["W"].T @ np.diag(2 * (sig - p["target"]) * p["P"]) @ p["W"]
    d = _values(p, eps, hop)
    dh, dv = d / p["a"], -1j * p["dx"] * d
    gH = np.zeros(p["n"] * p["L"], complex)
    gV = np.zeros_like(gH)
    cp = np.full(p["Nm"] - 1, 2.0)
    cp[0] = 1.0
    for v in p["vs"]:
        tv, tu = _table(p, dh, v), _table(p, dh, _mv(p, dv, v))
        Q, P = C @ tv, C @ tu
        la, lb = _clenshaw(p, dh, dv, Q), _clenshaw(p, dh, dv, P)
        gH += _slot_sum(p, cp, la[1:], tu[:-1]) + _slot_sum(p, cp, lb[1:], tv[:-1])
        gV += _slot_sum(p, [1.0], v[None], la[:1]) + _slot_sum(p, np.ones(p["Nm"]), P, tv)
    g = (gH.real / p["a"] + p["dx"] * gV.imag) / p["R"]
    ge, gh = np.zeros(p["n"]), np.zeros(p["nb"])
    np.add.at(ge, p["rows"][p["diag"]], g[p["diag"]])
    np.add.at(gh, p["bond_id"][p["bond"]], g[p["bond"]])
    return ge, gh


def _autograd(p, eps, hop):
    n, L = p["n"], p["L"]
    te, th = torch.tensor(eps, requires_grad=True), torch.tensor(hop, requires_grad=True)
    d = torch.zeros(n * L, dtype=torch.float64)
    d = d.index_put((torch.from_numpy(np.nonzero(p["diag"])[0]),), te[torch.from_numpy(p["rows"][p["diag"]])])
    d = d.index_put((torch.from_numpy(np.nonzero(p["bond"])[0]),), th[torch.from_numpy(p["bond_id"][p["bond"]])])
    ri, ci = torch.from_numpy(p["rows"]), torch.from_numpy(p["idx"].astype(np.int64))
    H = torch.zeros((n, n), dtype=torch.complex128).index_put((ri, ci), (d / p["a"]).to(torch.complex128), True)
    V = torch.zeros((n, n), dtype=torch.complex128).index_put((ri, ci), torch.complex(0 * d, -torch.from_numpy(p["dx"]) * d),
                                                              True)
    T = [torch.eye(n, dtype=torch.complex128), H]
    for _ in range(2, p["Nm"]):
        T.append(2 * H @ T[-1] - T[-2])
    mu = 0
    for v in p["vs"]:
        vt = torch.from_numpy(v)
        mu = mu + torch.stack([t @ (V @ vt) for t in T]).conj() @ torch.stack([V @ (t @ vt) for t in T]).T / p["R"]
    sig = torch.from_numpy(p["P"]) * torch.einsum("en,nm,em->e", torch.from_numpy(p["W"]), mu.real,
                                                  torch.from_numpy(p["W"]))
    torch.sum((sig - torch.from_numpy(p["target"])) ** 2).backward()
    return te.grad.numpy(), th.grad.numpy()


def test_adjoint_formulas_match_autograd():
    p = _setup()
    ge, gh = _adjoint(p, p["eps"], p["hop"])
    te, th = _autograd(p, p["eps"], p["hop"])
    scale = max(np.abs(te).max(), np.abs(th).max())
    assert np.abs(ge - te).max() <= 1e-12 * scale
    assert np.abs(gh - th).max() <= 1e-12 * scale
    # and against central differences on a few parameters
    h = 1e-6
    for which, i in (("e", 3), ("h", 5), ("h", 11)):
        e2, h2 = p["eps"].copy(), p["hop"].copy()
        (e2 if which == "e" else h2)[i] += h
        lp = _forward(p, e2, h2)[0]
        (e2 if which == "e" else h2)[i] -= 2 * h
        lm = _forward(p, e2, h2)[0]
        assert abs((lp - lm) / (2 * h) - (ge if which == "e" else gh)[i]) <= 1e-6 * scale
