"""The timeout path of the bounded device waits, exercised without any fault.

kpm_ell_test_timeout runs one producer-warp step in which the producer arms the first
stage barrier of every CTA for its transaction bytes but never issues the copies.  No
copy is outstanding for that stage, so nothing can land late: the waits on it simply run
out after the short budget given here (2e7 SM cycles, ~10 ms), the kernel records
KPM_ERR_TIMEOUT in the operator's status word, waits (bounded) for the copies it did
issue, and returns.  The test checks the status, that it is cleared once read, that the
call ends promptly, and that the same operator then gives correct moments (the context
is intact).
"""
import ctypes
import time

import numpy as np
import pytest

from conftest import golden
from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["honeycomb_8x8", "complex_open_6x5", "ref_graphene_256", "irregular_300"])
def test_withheld_stage_times_out_and_reports(cuda_lib, case):
    import torch

    from minijclsquant_gb300 import _capi

    z = golden(case)
    L, M = int(z["len_row"]), int(z["M"])
    d = np.ascontiguousarray(z["data_kpm"])
    ix = np.ascontiguousarray(z["indices"], dtype=np.int32)
    h = ctypes.c_void_p()
    assert cuda_lib.kpm_ell_create(ctypes.byref(h), d.size // L, L, d.ctypes.data, ix.ctypes.data, 0, None) == 0
    try:
        assert cuda_lib.kpm_ell_test_timeout(h, 10, None) == _capi.KPM_ERR_INVALID_ARG
        t0 = time.perf_counter()
        st = cuda_lib.kpm_ell_test_timeout(h, 20_000_000, None)
        dt = time.perf_counter() - t0
        if case == "irregular_300":
            # 9 complex slots per row: four shared-memory stages exceed the producer-warp
            # kernel's limit, so the hook launches nothing and says so
            assert st == _capi.KPM_ERR_UNSUPPORTED
        else:
            assert st == _capi.KPM_ERR_TIMEOUT, cuda_lib.kpm_strerror(st)
        assert dt < 5.0
        assert cuda_lib.kpm_ell_check(h, None) == _capi.KPM_OK  # read once, then cleared
        # the operator and the context are intact: moments as before
        v = torch.from_numpy(np.ascontiguousarray(z["v"])).cuda()
        R = v.shape[0]
        mu = torch.empty((R, M), dtype=torch.complex128, device="cuda")
        assert cuda_lib.kpm_cheb_moments(h, 0, R, M, v.data_ptr(), None, mu.data_ptr(), None, None) == 0
        assert cuda_lib.kpm_ell_check(h, None) == _capi.KPM_OK
        torch.cuda.synchronize()
        ok, err = oracle.moment_tolerance_ok(mu.cpu().numpy(), z["mu"], 1e-10)
        assert ok, err
    finally:
        cuda_lib.kpm_ell_destroy(h)
