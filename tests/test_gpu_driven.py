"""Time-dependent operators of driven systems on the GPU, against the reference's own
Cython outputs (tests/golden/modifiers_6x5.npz: light_modifier_cython and
hopping_pos_phonons_modifier, jclsquant/cython_modules/Extra_funs.pyx:236-342, 540-560)
and the oracle's numpy restatement.  Elementwise complex arithmetic: relative 1e-13."""
import ctypes

import numpy as np
import pytest

from conftest import golden
from oracle import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-13


def _rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b)))


def _params(values):
    return np.ascontiguousarray(np.array(values, dtype=np.complex128).view(np.float64))


def test_light_modifier_matches_reference(cuda_lib):
    import torch

    from minijclsquant_gb300 import _capi

    z = golden("modifiers_6x5")
    d = torch.from_numpy(z["data"]).cuda()
    x = torch.from_numpy(z["dx"]).cuda()
    y = torch.from_numpy(z["dy"]).cuda()
    for prm, want in zip(z["light_params"], z["light_out"]):
        out = torch.empty_like(d)
        p = _params(prm)
        st = _capi.lib().kpm_light_modifier(d.numel(), p.ctypes.data, d.data_ptr(), x.data_ptr(), y.data_ptr(),
                                            out.data_ptr(), None)
        assert st == 0
        assert _rel(out.cpu().numpy(), want) <= TOL, prm
    # in place (data_new aliasing data)
    prm = z["light_params"][3]
    dd = d.clone()
    assert _capi.lib().kpm_light_modifier(dd.numel(), _params(prm).ctypes.data, dd.data_ptr(), x.data_ptr(),
                                          y.data_ptr(), dd.data_ptr(), None) == 0
    assert _rel(dd.cpu().numpy(), z["light_out"][3]) <= TOL


def test_phonon_modifier_matches_reference(cuda_lib):
    from minijclsquant_gb300.modifiers import phonon_modifier_device

    z = golden("modifiers_6x5")
    a0, b, Aq, wq, t, q0, q1 = z["phonon_params"]
    dn, xn, yn = phonon_modifier_device(z["data"], z["indices"], z["dx"], z["dy"], int(z["len_row"]), a0, b, Aq, wq,
                                        t, (q0, q1), z["e_pol_x"], z["e_pol_y"], z["Sx"], z["Sy"])
    assert _rel(dn.cpu().numpy(), z["phonon_data"]) <= TOL
    assert _rel(xn.cpu().numpy(), z["phonon_dx"]) <= TOL
    assert _rel(yn.cpu().numpy(), z["phonon_dy"]) <= TOL


class _Ell:
    """The attributes of jclsquant's ell_matrix that the modifiers read."""

    def __init__(self, z):
        self.data, self.indices, self.len_row = z["data"], z["indices"], int(z["len_row"])
        self.dx_vec, self.dy_vec = z["dx"], z["dy"]
        self.shape = (self.data.size // self.len_row,) * 2
        self.space = "r"


@pytest.mark.parametrize("mode,params,t,row", [
    ("linear", (2.1, 1.9), 0.37, 0), ("circle", (2.1, 1.9, "r"), 0.37, 1),
    ("linear_packed", (1.4, 2.3, 0.6), 0.9, 2), ("circle_packed", (1.4, 2.3, "l", 0.6), 0.9, 3)])
def test_modifier_drop_ins(cuda_lib, mode, params, t, row):
    """modifier_light (jclsquant/modifiers.py:133-182) and modifier_hoppings_c (:362-445)
    with the reference's ids and parameter tuples, filling the caller's array."""
    from minijclsquant_gb300 import modifiers

    z = golden("modifiers_6x5")
    A = _Ell(z)
    out = np.zeros_like(z["data"])
    assert modifiers.modifier_light(A, out, mode, params, t) is out
    assert _rel(out, z["light_out"][row]) <= TOL
    out2 = np.zeros_like(z["data"])
    modifiers.modifier_hoppings_c(A, out2, None, None, mode, params, t)
    assert _rel(out2, z["light_out"][row]) <= TOL


def test_modifier_hoppings_phonons_drop_in(cuda_lib):
    from minijclsquant_gb300 import modifiers

    z = golden("modifiers_6x5")
    A = _Ell(z)
    a0, b, Aq, wq, t, _, _ = z["phonon_params"]
    S = np.stack([z["Sx"], z["Sy"]], axis=1)
    dn, xn, yn = z["data"].copy(), z["dx"].copy(), z["dy"].copy()
    r = modifiers.modifier_hoppings_c(A, dn, xn, yn, "phonons_packed", (a0, b, Aq, wq, "chiral_+", S), t)
    assert r is not None
    assert _rel(dn, z["phonon_data"]) <= TOL
    assert _rel(xn, z["phonon_dx"]) <= TOL
    assert _rel(yn, z["phonon_dy"]) <= TOL


def test_modifier_messages_and_invalid_ids(cuda_lib, capsys):
    from minijclsquant_gb300 import modifiers

    z = golden("modifiers_6x5")
    A = _Ell(z)
    out = np.zeros_like(z["data"])
    assert modifiers.modifier_light(A, out, "sideways", (1.0, 1.0), 0.1) is None
    assert modifiers.modifier_light(A, out, "circle", (1.0, 1.0, "x"), 0.1) is None
    assert modifiers.modifier_light(A, out) is None
    assert "valid" in capsys.readouterr().out
    A.space = "k"
    with pytest.raises(NotImplementedError):
        modifiers.modifier_hoppings_c(A, out, None, None, "linear", (1.0, 1.0), 0.1)


def test_light_update_in_place_drives_the_recursion(cuda_lib):
    """H(t) written into the operator's values: moments equal those of the modified
    arrays (oracle), Hermiticity is kept (bond vectors are antisymmetric), and a
    real-stored operator is refused."""
    from minijclsquant_gb300 import _capi, device, lattice
    from minijclsquant_gb300.modifiers import modifier_bounds
    from minijclsquant_gb300.observables import random_vector_generator

    H = lattice.honeycomb(24, 20, t=-2.7, W=0.5, seed=3)
    Hk = H.modifier(modifier_bounds)
    op = device.DeviceELL(Hk.data, Hk.indices, Hk.len_row, complex_values=True)
    assert not op.is_real
    v = random_vector_generator(op.n, 9)
    for mode, prm, t in [("circle_packed", (2.0, 1.7, "r", 0.8), 1.1), ("linear", (1.2, 0.9), 0.4)]:
        op.light_update(Hk.data, H.dx_vec, H.dy_vec, mode, prm, t)
        assert cuda_lib.kpm_ell_check(op.handle, None) == 0
        assert op.hermitian
        Ht = oracle.light_modifier(*_light_tuple(mode, prm, t), Hk.data, H.dx_vec, H.dy_vec)
        mu = device.cheb_moments(op, 120, v)
        ok, err = oracle.moment_tolerance_ok(mu, oracle.rec_A_tab(120, Ht, Hk.indices, Hk.len_row, v), 1e-10)
        assert ok, (mode, err)
    real_op = device.DeviceELL(Hk.data, Hk.indices, Hk.len_row)
    assert real_op.is_real
    p = _params(_light_tuple("linear", (1.2, 0.9), 0.4))
    import torch

    d = torch.from_numpy(Hk.data).cuda()
    x = torch.from_numpy(np.ascontiguousarray(H.dx_vec)).cuda()
    st = cuda_lib.kpm_ell_light_update(real_op.handle, p.ctypes.data, d.data_ptr(), x.data_ptr(), x.data_ptr(),
                                       None)
    assert st == _capi.KPM_ERR_DTYPE


def _light_tuple(mode, prm, t):
    eta = {"r": 1.0, "l": -1.0}
    if mode == "linear":
        return (1, prm[0], t, prm[1], 0, 0)
    if mode == "circle_packed":
        return (1, prm[0], t, prm[1], prm[3], eta[prm[2]])
    raise ValueError(mode)


def test_phonon_modifier_rejects_columns_outside_the_operator(cuda_lib):
    import torch

    from minijclsquant_gb300 import _capi

    z = golden("modifiers_6x5")
    idx = z["indices"].copy()
    idx[7] = 10_000  # outside [0, n)
    if idx[7] == 7 // int(z["len_row"]):
        idx[7] = 10_001
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    d, x, y = t(z["data"]), t(z["dx"]), t(z["dy"])
    ex, ey, sx, sy = t(z["e_pol_x"]), t(z["e_pol_y"]), t(z["Sx"]), t(z["Sy"])
    ti = t(idx.astype(np.int32))
    dn, xn, yn = d.clone(), x.clone(), y.clone()
    n = z["data"].size // int(z["len_row"])
    p = _params(list(z["phonon_params"]))
    st = _capi.lib().kpm_phonon_modifier(n, int(z["len_row"]), p.ctypes.data, d.data_ptr(), ti.data_ptr(),
                                         x.data_ptr(), y.data_ptr(), ex.data_ptr(), ey.data_ptr(), sx.data_ptr(),
                                         sy.data_ptr(), dn.data_ptr(), xn.data_ptr(), yn.data_ptr(), None)
    assert st == _capi.KPM_ERR_INDEX
    assert _capi.lib().kpm_light_modifier(0, p.ctypes.data, d.data_ptr(), x.data_ptr(), y.data_ptr(), dn.data_ptr(),
                                          None) == _capi.KPM_ERR_INVALID_ARG
    assert isinstance(ctypes.c_int(st).value, int)


def test_light_phase_table_accuracy(cuda_lib):
    """The light kernels' table-driven sin and cos (256-entry table, Cody-Waite reduction,
    Taylor polynomials): exp(i x) for data = 1 and the circular form at t = 0 (arg = i A0 dx),
    within 4e-16 absolute of numpy's cos and sin, on small, O(1), near-multiple-of-pi/2 and
    large arguments, and above 2e4 where the kernels fall back to sincos()."""
    import torch

    rng = np.random.default_rng(3)
    k = rng.integers(-5000, 5000, 20000)
    x = np.concatenate([rng.uniform(-4, 4, 200000), rng.uniform(-2e4, 2e4, 200000),
                        np.ldexp(rng.uniform(-1, 1, 20000), -rng.integers(1, 60, 20000)),
                        k * (np.pi / 2) + rng.uniform(-1e-9, 1e-9, k.size), rng.uniform(2e4, 1e6, 5000),
                        [0.0, -0.0, 2e4, -2e4, np.pi, -np.pi]])
    n = x.size
    d = torch.ones(n, dtype=torch.complex128, device="cuda")
    dx = torch.from_numpy(x.astype(np.complex128)).cuda()
    dy = torch.zeros(n, dtype=torch.complex128, device="cuda")
    out = torch.empty_like(d)
    p = _params([1, 1, 0, 1, 0, 1])  # a, A0, t, w, Tp, eta
    assert cuda_lib.kpm_light_modifier(n, p.ctypes.data, d.data_ptr(), dx.data_ptr(), dy.data_ptr(), out.data_ptr(),
                                       None) == 0
    o = out.cpu().numpy()
    assert np.max(np.abs(o.real - np.cos(x))) <= 4e-16
    assert np.max(np.abs(o.imag - np.sin(x))) <= 4e-16


def test_light_phase_relative_accuracy_near_zeros(cuda_lib):
    """Where sin or cos is nearly zero the table method keeps a small RELATIVE error too: the
    reduction x = k 2pi/256 + r is accurate to a few ulps of r itself, and the table holds
    exact zeros at multiples of pi/2.  Phases within 1e-9 of k pi (sin) and of (k + 1/2) pi
    (cos), |k| < 6000, against numpy's sin and cos at 1e-13 relative."""
    import torch

    rng = np.random.default_rng(8)
    k = rng.integers(-6000, 6000, 40000).astype(np.float64)
    k[k == 0] = 1.0
    d = rng.uniform(-1e-9, 1e-9, k.size)
    d[:100] = np.ldexp(1.0, -rng.integers(35, 60, 100)) * np.sign(rng.uniform(-1, 1, 100))
    for x, pick in ((k * np.pi + d, "sin"), ((k + 0.5) * np.pi + d, "cos")):
        n = x.size
        ones = torch.ones(n, dtype=torch.complex128, device="cuda")
        dx = torch.from_numpy(x.astype(np.complex128)).cuda()
        dy = torch.zeros(n, dtype=torch.complex128, device="cuda")
        out = torch.empty_like(ones)
        p = _params([1, 1, 0, 1, 0, 1])
        assert cuda_lib.kpm_light_modifier(n, p.ctypes.data, ones.data_ptr(), dx.data_ptr(), dy.data_ptr(),
                                           out.data_ptr(), None) == 0
        o = out.cpu().numpy()
        got, ref = (o.imag, np.sin(x)) if pick == "sin" else (o.real, np.cos(x))
        assert np.min(np.abs(ref)) > 0
        rel = np.max(np.abs(got - ref) / np.abs(ref))
        assert rel <= 1e-13, (pick, rel)
