"""Small (L2-resident) operators replay each moment recursion as one CUDA graph launch
(kpm_cheb_moments).  The replay must give bit for bit the moments of the same kernels
launched one by one (KPM_NO_GRAPH=1), for new input and output buffers on every call, for
vector counts split into several groups, with a left vector set and with both moment sets,
in complex128 and complex64, and after the operator's values change."""
import os

import numpy as np
import pytest

from conftest import golden
from oracle import oracle

pytestmark = pytest.mark.gpu


def _moments(op, M, v, **kw):
    from minijclsquant_gb300 import device

    return device.cheb_moments(op, M, v, **kw)


def _direct(fn):
    os.environ["KPM_NO_GRAPH"] = "1"
    try:
        return fn()
    finally:
        del os.environ["KPM_NO_GRAPH"]


@pytest.mark.parametrize("dtype", ["c128", "c64"])
@pytest.mark.parametrize("R", [1, 4, 11])
def test_graph_replay_equals_direct_launches(cuda_lib, dtype, R):
    import torch

    from minijclsquant_gb300 import device

    z = golden("irregular_300")
    op = device.DeviceELL(z["data_kpm"], z["indices"], int(z["len_row"]))
    rng = np.random.default_rng(R)
    M = 97
    for rep in range(3):  # fresh tensors every call: the staging copies keep the graph valid
        vs = torch.from_numpy(np.exp(1j * rng.uniform(0, 2 * np.pi, (R, op.n)))).cuda()
        vl = torch.from_numpy(np.exp(1j * rng.uniform(0, 2 * np.pi, (R, op.n)))).cuda()
        g = _moments(op, M, vs, dtype=dtype)
        d = _direct(lambda: _moments(op, M, vs, dtype=dtype))
        assert torch.equal(g, d), rep
        g2 = _moments(op, M, vs, v_l=vl, dtype=dtype, both=True)
        d2 = _direct(lambda: _moments(op, M, vs, v_l=vl, dtype=dtype, both=True))
        assert torch.equal(g2[0], d2[0]) and torch.equal(g2[1], d2[1]), rep
    if dtype == "c128":
        v = vs.cpu().numpy()
        for r in range(R):
            ref = oracle.rec_A_tab(M, z["data_kpm"], z["indices"], int(z["len_row"]), v[r])
            ok, err = oracle.moment_tolerance_ok(g[r].cpu().numpy(), ref, 1e-10)
            assert ok, (r, err)


def test_graph_replay_after_new_values(cuda_lib):
    """kpm_ell_set_values (and the complex64 copy it drops and rebuilds) between calls."""
    import ctypes

    import torch

    from minijclsquant_gb300 import _capi, device

    z = golden("honeycomb_8x8")
    L = int(z["len_row"])
    op = device.DeviceELL(z["data_kpm"], z["indices"], L)
    v = torch.from_numpy(np.ascontiguousarray(z["v"])).cuda()
    M = int(z["M"])
    for dtype in ("c128", "c64"):
        a = _moments(op, M, v, dtype=dtype)
    scaled = np.ascontiguousarray(z["data_kpm"] * 0.5)
    assert cuda_lib.kpm_ell_set_values(op.handle, scaled.ctypes.data, 0, None) == 0
    for dtype in ("c128", "c64"):
        g = _moments(op, M, v, dtype=dtype)
        d = _direct(lambda: _moments(op, M, v, dtype=dtype))
        assert torch.equal(g, d), dtype
    ref = oracle.rec_A_tab(M, scaled, z["indices"], L, z["v"][0])
    ok, err = oracle.moment_tolerance_ok(_moments(op, M, v)[0].cpu().numpy(), ref, 1e-10)
    assert ok, err
    assert isinstance(ctypes.c_int(_capi.KPM_OK).value, int)
