"""Time evolution (for_time, jclsquant/cuda_cython/cuda/obv.cu:93-122): U and U_c advanced
len_t times by the series sum_m c_m T_m(H) with the moments of exp(-i H dt).

Parity against the golden vectors made by the reference's own rec_A_vec and against the
oracle: max|diff| <= 1e-10 * max|ref| (complex128), 2e-5 for complex64.  At full size the
size-independent properties are checked: composition (a steps then b steps is the same
kernel sequence as a + b steps, so the results are bitwise equal) and unitarity (norms are
kept to the truncation error of the series)."""
import numpy as np
import pytest

from conftest import golden
from oracle import oracle

pytestmark = pytest.mark.gpu

REL = 1e-10


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_time_evolve_matches_reference_golden(cuda_lib):
    from minijclsquant_gb300 import device

    z = golden("time_evolution_6x5")
    op = device.DeviceELL(z["data_kpm"], z["indices"], int(z["len_row"]))
    out = device.time_evolve(op, int(z["M"]), z["c"], int(z["len_t"]), np.stack([z["U0"], z["Uc0"]]))
    assert _rel(out[0], z["U"]) <= REL
    assert _rel(out[1], z["Uc"]) <= REL


def test_for_time_host_entry_point_matches_reference_golden(cuda_lib):
    from minijclsquant_gb300 import obv_gpu

    z = golden("time_evolution_6x5")
    U, Uc = z["U0"].copy(), z["Uc0"].copy()
    obv_gpu.for_time_gpu(z["data_kpm"], z["indices"], int(z["len_row"]), z["c"], int(z["len_t"]), U, Uc,
                         int(z["M"]))
    assert _rel(U, z["U"]) <= REL
    assert _rel(Uc, z["Uc"]) <= REL
    # len_t = 0: the reference's loop runs no step
    U2, Uc2 = z["U0"].copy(), z["Uc0"].copy()
    obv_gpu.for_time_gpu(z["data_kpm"], z["indices"], int(z["len_row"]), z["c"], 0, U2, Uc2, int(z["M"]))
    assert np.array_equal(U2, z["U0"]) and np.array_equal(Uc2, z["Uc0"])


@pytest.mark.parametrize("R", [1, 2, 3, 8])
def test_time_evolve_vector_groups_against_oracle(cuda_lib, R):
    from minijclsquant_gb300 import device, lattice
    from minijclsquant_gb300.kernel_and_moments import moments_U
    from minijclsquant_gb300.modifiers import modifier_bounds
    from minijclsquant_gb300.observables import random_vector_generator

    H = lattice.honeycomb(24, 20, t=-2.7, W=0.8, seed=12)
    Hk = H.modifier(modifier_bounds)
    op = device.DeviceELL(Hk.data, Hk.indices, Hk.len_row)
    M, steps = 40, 3
    c = moments_U(2.0, M).astype(np.complex128)
    vs = np.stack([random_vector_generator(op.n, 70 + r) for r in range(R)])
    out = device.time_evolve(op, M, c, steps, vs)
    for r in range(R):
        ref = vs[r]
        for _ in range(steps):
            ref = oracle.rec_A_vec(M, Hk.data, Hk.indices, Hk.len_row, c, ref)
        assert _rel(out[r], ref) <= REL, (R, r)


def test_time_evolve_zero_steps_and_aliasing(cuda_lib):
    import torch

    from minijclsquant_gb300 import device

    z = golden("time_evolution_6x5")
    op = device.DeviceELL(z["data_kpm"], z["indices"], int(z["len_row"]))
    v = np.stack([z["U0"], z["Uc0"]])
    assert np.array_equal(device.time_evolve(op, int(z["M"]), z["c"], 0, v), v)
    # in place through the C ABI: out == v
    from minijclsquant_gb300 import _capi

    tv = torch.from_numpy(v.copy()).cuda()
    tc = torch.from_numpy(np.ascontiguousarray(z["c"])).cuda()
    st = _capi.lib().kpm_time_evolve(op.handle, _capi.KPM_C128, 2, int(z["M"]), tc.data_ptr(), int(z["len_t"]),
                                     tv.data_ptr(), tv.data_ptr(), None)
    assert st == _capi.KPM_OK
    got = tv.cpu().numpy()
    assert _rel(got[0], z["U"]) <= REL and _rel(got[1], z["Uc"]) <= REL


def test_time_evolve_invalid_arguments(cuda_lib):
    import torch

    from minijclsquant_gb300 import _capi, device

    z = golden("time_evolution_6x5")
    op = device.DeviceELL(z["data_kpm"], z["indices"], int(z["len_row"]))
    tv = torch.from_numpy(np.stack([z["U0"], z["Uc0"]])).cuda()
    tc = torch.from_numpy(np.ascontiguousarray(z["c"])).cuda()
    lib = _capi.lib()
    M = int(z["M"])
    assert lib.kpm_time_evolve(None, 0, 2, M, tc.data_ptr(), 1, tv.data_ptr(), tv.data_ptr(), None) == \
        _capi.KPM_ERR_INVALID_ARG
    assert lib.kpm_time_evolve(op.handle, 0, 2, 1, tc.data_ptr(), 1, tv.data_ptr(), tv.data_ptr(), None) == \
        _capi.KPM_ERR_INVALID_ARG
    assert lib.kpm_time_evolve(op.handle, 0, 2, M, tc.data_ptr(), -1, tv.data_ptr(), tv.data_ptr(), None) == \
        _capi.KPM_ERR_INVALID_ARG
    assert lib.kpm_time_evolve(op.handle, 0, 0, M, tc.data_ptr(), 1, tv.data_ptr(), tv.data_ptr(), None) == \
        _capi.KPM_ERR_INVALID_ARG
    assert lib.kpm_time_evolve(op.handle, 9, 2, M, tc.data_ptr(), 1, tv.data_ptr(), tv.data_ptr(), None) == \
        _capi.KPM_ERR_DTYPE
    with pytest.raises(ValueError):
        device.time_evolve(op, M, z["c"], -1, z["U0"])
    # the host-pointer symbol reports through kpm_last_status
    U, Uc = z["U0"].copy(), z["Uc0"].copy()
    lib.for_time(z["data_kpm"].ctypes.data, z["indices"].ctypes.data, int(z["len_row"]), U.shape[0],
                 z["c"].ctypes.data, 2, U.ctypes.data, Uc.ctypes.data, 1)
    assert lib.kpm_last_status() == _capi.KPM_ERR_INVALID_ARG
    assert np.array_equal(U, z["U0"])


def test_time_evolve_complex64(cuda_lib):
    from minijclsquant_gb300 import device

    z = golden("time_evolution_6x5")
    op = device.DeviceELL(z["data_kpm"], z["indices"], int(z["len_row"]))
    out = device.time_evolve(op, int(z["M"]), z["c"], int(z["len_t"]), np.stack([z["U0"], z["Uc0"]]),
                             dtype="c64")
    assert _rel(out[0], z["U"]) <= 2e-5
    assert _rel(out[1], z["Uc"]) <= 2e-5


def test_time_evolve_full_size_composition_and_unitarity(cuda_lib):
    import torch

    from minijclsquant_gb300 import device, lattice
    from minijclsquant_gb300.kernel_and_moments import moments_U
    from minijclsquant_gb300.modifiers import modifier_bounds
    from minijclsquant_gb300.observables import random_vector_generator

    H = lattice.honeycomb(512, 512, t=-2.7, W=1.0, seed=3)
    Hk = H.modifier(modifier_bounds)
    op = device.DeviceELL(Hk.data, Hk.indices, Hk.len_row)
    M = 64
    c = moments_U(3.0, M).astype(np.complex128)
    v = torch.from_numpy(np.stack([random_vector_generator(op.n, 5 + r) for r in range(2)])).cuda()
    a = device.time_evolve(op, M, c, 3, v)
    ab = device.time_evolve(op, M, c, 2, a)
    direct = device.time_evolve(op, M, c, 5, v)
    assert torch.equal(ab, direct)
    n0 = torch.linalg.vector_norm(v, dim=1)
    n5 = torch.linalg.vector_norm(direct, dim=1)
    assert float(torch.max(torch.abs(n5 - n0) / n0)) <= 1e-10


def _complex_lattice(nx, ny, seed):
    """Honeycomb with a Peierls-like phase on every bond (complex hoppings), scaled into [-1, 1]."""
    from minijclsquant_gb300 import lattice
    from minijclsquant_gb300.ell_matrix import ell_matrix
    from minijclsquant_gb300.modifiers import modifier_bounds

    arr = lattice.honeycomb_arrays(nx, ny, t=-2.7, W=0.6, seed=seed)
    phase = np.exp(1j * 0.4 * np.real(arr["dx"]) / 0.142)
    arr = dict(arr, data=np.where(np.real(arr["dx"]) != 0, arr["data"] * phase, arr["data"]))
    return ell_matrix(lattice.to_csr(arr)).modifier(modifier_bounds)


@pytest.mark.parametrize("complex_op", [False, True])
@pytest.mark.parametrize("kernel", ["simple", "ws1", "ws2", "ws1s2"])
@pytest.mark.parametrize("dtype,R", [("c128", 1), ("c128", 2), ("c128", 8), ("c64", 2), ("c64", 8)])
def test_series_every_step_kernel_variant(cuda_lib, monkeypatch, kernel, dtype, R, complex_op):
    """The series step (rec_A_vec; the time-evolution and time-domain Kubo inner loop) on
    each kernel the autotuner can pick for it, forced, against the oracle."""
    from minijclsquant_gb300 import device, lattice
    from minijclsquant_gb300.kernel_and_moments import moments_U
    from minijclsquant_gb300.modifiers import modifier_bounds
    from minijclsquant_gb300.observables import random_vector_generator

    if kernel == "ws1s2" and dtype == "c64":
        pytest.skip("two sub-tiles per stage is a complex128 form")
    monkeypatch.setenv("KPM_STEP_KERNEL", kernel)
    if complex_op:
        Hk = _complex_lattice(40, 36, 8)
    else:
        Hk = lattice.honeycomb(40, 36, t=-2.7, W=0.7, seed=5).modifier(modifier_bounds)
    op = device.DeviceELL(Hk.data, Hk.indices, Hk.len_row)
    assert op.is_real != complex_op
    M = 60
    c = moments_U(4.0, M).astype(np.complex128)
    vs = np.stack([random_vector_generator(op.n, 300 + r) for r in range(R)])
    s = device.cheb_series(op, M, c, vs, dtype=dtype)
    e = device.time_evolve(op, M, c, 2, vs, dtype=dtype)
    assert cuda_lib.kpm_ell_check(op.handle, None) == 0
    import ctypes

    from minijclsquant_gb300 import _capi

    kind, U = ctypes.c_int(), ctypes.c_int()
    assert cuda_lib.kpm_ell_series_config(op.handle, _capi.dtype_code(dtype), R, ctypes.byref(kind),
                                          ctypes.byref(U), None, None) == 0
    want = {"simple": (0, 1), "ws1": (2, 1), "ws2": (2, 2), "ws1s2": (3, 1)}[kernel]
    threads_per_row = R // (2 if dtype == "c64" and R >= 2 else 1)
    if kernel == "ws2" and complex_op and threads_per_row == 1:
        # 4 stages of 512-row complex tiles (56 KB each) exceed the shared-memory cap:
        # no producer-warp candidate, the forced choice falls back to the grid-stride kernel
        want = (0, 1)
    assert (kind.value, U.value) == want
    tol = REL if dtype == "c128" else 2e-5
    for r in range(R):
        ref = oracle.rec_A_vec(M, Hk.data, Hk.indices, Hk.len_row, c, vs[r])
        assert _rel(s[r], ref) <= tol, (kernel, r, _rel(s[r], ref))
        ref2 = oracle.rec_A_vec(M, Hk.data, Hk.indices, Hk.len_row, c, ref)
        assert _rel(e[r], ref2) <= tol, (kernel, r, _rel(e[r], ref2))


@pytest.mark.parametrize("complex_op", [False, True])
@pytest.mark.parametrize("kernel", ["simple", "ws1", "ws2"])
@pytest.mark.parametrize("R", [1, 2, 8])
def test_series_float_float_every_kernel(cuda_lib, monkeypatch, kernel, R, complex_op):
    """KPM_C128F series and time evolution (float-float arithmetic on the FP32 pipe) on each
    float-float step kernel, forced, against the oracle at the complex128 tolerance."""
    from minijclsquant_gb300 import device, lattice
    from minijclsquant_gb300.kernel_and_moments import moments_U
    from minijclsquant_gb300.modifiers import modifier_bounds
    from minijclsquant_gb300.observables import random_vector_generator

    monkeypatch.setenv("KPM_STEP_KERNEL", kernel)
    if complex_op:
        Hk = _complex_lattice(40, 36, 8)
    else:
        Hk = lattice.honeycomb(40, 36, t=-2.7, W=0.7, seed=5).modifier(modifier_bounds)
    op = device.DeviceELL(Hk.data, Hk.indices, Hk.len_row)
    M = 60
    c = moments_U(4.0, M).astype(np.complex128)
    vs = np.stack([random_vector_generator(op.n, 500 + r) for r in range(R)])
    s = device.cheb_series(op, M, c, vs, dtype="c128f")
    e = device.time_evolve(op, M, c, 3, vs, dtype="c128f")
    assert cuda_lib.kpm_ell_check(op.handle, None) == 0
    for r in range(R):
        ref = oracle.rec_A_vec(M, Hk.data, Hk.indices, Hk.len_row, c, vs[r])
        assert _rel(s[r], ref) <= REL, (kernel, r, _rel(s[r], ref))
        for _ in range(2):
            ref = oracle.rec_A_vec(M, Hk.data, Hk.indices, Hk.len_row, c, ref)
        assert _rel(e[r], ref) <= REL, (kernel, r, _rel(e[r], ref))


def test_time_evolve_float_float_matches_reference_golden(cuda_lib):
    from minijclsquant_gb300 import device

    z = golden("time_evolution_6x5")
    op = device.DeviceELL(z["data_kpm"], z["indices"], int(z["len_row"]))
    out = device.time_evolve(op, int(z["M"]), z["c"], int(z["len_t"]), np.stack([z["U0"], z["Uc0"]]),
                             dtype="c128f")
    assert _rel(out[0], z["U"]) <= REL
    assert _rel(out[1], z["Uc"]) <= REL
    x = golden("honeycomb_8x8_more")
    h8 = golden("honeycomb_8x8")
    op8 = device.DeviceELL(h8["data_kpm"], h8["indices"], int(h8["len_row"]))
    s = device.cheb_series(op8, len(x["coef"]), x["coef"], h8["v"][0], dtype="c128f")
    assert _rel(s, x["series"]) <= REL


def test_time_evolve_float_float_full_size_against_complex128(cuda_lib):
    import torch

    from minijclsquant_gb300 import device, lattice
    from minijclsquant_gb300.kernel_and_moments import moments_U
    from minijclsquant_gb300.modifiers import modifier_bounds
    from minijclsquant_gb300.observables import random_vector_generator

    H = lattice.honeycomb(512, 512, t=-2.7, W=1.0, seed=3)
    Hk = H.modifier(modifier_bounds)
    op = device.DeviceELL(Hk.data, Hk.indices, Hk.len_row)
    M = 64
    c = moments_U(3.0, M).astype(np.complex128)
    v = torch.from_numpy(np.stack([random_vector_generator(op.n, 5 + r) for r in range(2)])).cuda()
    f = device.time_evolve(op, M, c, 5, v, dtype="c128f")
    d = device.time_evolve(op, M, c, 5, v)
    assert float(torch.max(torch.abs(f - d)) / torch.max(torch.abs(d))) <= 1e-12
    n0 = torch.linalg.vector_norm(v, dim=1)
    assert float(torch.max(torch.abs(torch.linalg.vector_norm(f, dim=1) - n0) / n0)) <= 1e-10
