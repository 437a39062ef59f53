"""The no-allocation moment entry point, kpm_cheb_moments_noalloc, through the C ABI.

It serves callers that may not allocate device memory (a plugin inside a host
application that owns the device budget, or code that must not trigger the
device synchronisation cudaMalloc / cudaFree can cause): it takes the operator
straight from the caller's device arrays and keeps its scratch in one fixed
device array inside the library.

Checked against the handle-based kpm_cheb_moments on the same inputs, on two
calls in a row with different operators and sizes (the second call must not
see anything the first left in the shared scratch), at the complex128 parity
tolerance used everywhere: per order |d mu_m| <= 1e-10 * max(|mu_m|, 1e-6 |mu_0|).
This file is collected last so a stop at its first failure has already run
every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(nx, ny, W, seed, M):
    import torch

    from minijclsquant_gb300 import lattice
    from minijclsquant_gb300.modifiers import modifier_bounds
    from minijclsquant_gb300.observables import random_vector_generator

    H = lattice.honeycomb(nx, ny, t=-2.7, W=W, seed=seed)
    data = np.ascontiguousarray(modifier_bounds(H))
    idx = np.ascontiguousarray(H.indices)
    v = random_vector_generator(H.shape[0], seed + 1)
    return dict(data=data, idx=idx, L=int(H.len_row), n=int(H.shape[0]), v=v, M=M,
                d_data=torch.from_numpy(data).cuda(), d_idx=torch.from_numpy(idx).cuda(),
                d_v=torch.from_numpy(v).cuda())


def _with_handle(lib, c):
    import torch

    h = ctypes.c_void_p()
    assert lib.kpm_ell_create(ctypes.byref(h), c["n"], c["L"], c["data"].ctypes.data, c["idx"].ctypes.data, 0,
                              None) == 0
    try:
        mu = torch.empty(c["M"], dtype=torch.complex128, device="cuda")
        assert lib.kpm_cheb_moments(h, 0, 1, c["M"], c["d_v"].data_ptr(), None, mu.data_ptr(), None, None) == 0
        torch.cuda.synchronize()
        return mu.cpu().numpy()
    finally:
        lib.kpm_ell_destroy(h)


def _noalloc(lib, c):
    import torch

    mu = torch.full((c["M"],), complex(np.nan, np.nan), dtype=torch.complex128, device="cuda")
    st = lib.kpm_cheb_moments_noalloc(c["d_data"].data_ptr(), c["d_idx"].data_ptr(), c["L"], c["n"],
                                      c["d_v"].data_ptr(), c["M"], mu.data_ptr(), None)
    assert st == 0, lib.kpm_strerror(st)
    return mu.cpu().numpy()


def _close(mu, ref):
    scale = np.maximum(np.abs(ref), 1e-6 * np.abs(ref[0]))
    return float(np.max(np.abs(mu - ref) / scale))


def test_noalloc_matches_handle_path_on_two_calls_in_a_row(cuda_lib):
    first = _case(96, 80, W=1.0, seed=11, M=300)   # 15,360 sites, crosses the 64-step partial chunk
    second = _case(40, 52, W=0.4, seed=3, M=130)   # smaller: a stale first-call vector would show
    for c in (first, second):
        ref = _with_handle(cuda_lib, c)
        got = _noalloc(cuda_lib, c)
        assert _close(got, ref) <= 1e-10


def test_noalloc_rejects_sizes_beyond_its_scratch(cuda_lib):
    from minijclsquant_gb300 import _capi

    st = cuda_lib.kpm_cheb_moments_noalloc(1, 1, 4, (1 << 20) + 1, 1, 8, 1, None)
    assert st == _capi.KPM_ERR_TOO_LARGE
    assert b"fixed scratch" in cuda_lib.kpm_strerror(st)
