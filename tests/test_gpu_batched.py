"""Batched operators (uneven instances in one recursion) against the oracle,
one instance at a time.  Complex128 tolerance as the plain path (1e-10 per
order); complex64 against its own error budget."""
import ctypes

import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu

REL = 1e-10


def _ensemble(n_inst, side_range, seed):
    from minijclsquant_gb300 import batched

    return batched.honeycomb_ensemble(n_inst, side_range=side_range, W_range=(0.0, 2.0), seed=seed)


@pytest.mark.parametrize("R", [1, 2, 4, 8])
def test_batched_c128_matches_oracle_per_instance(cuda_lib, R):
    from minijclsquant_gb300 import batched

    datas, idxs, L, bnds, _ = _ensemble(7, (2, 23), seed=3 + R)  # 8 .. 1058 sites, some under one tile
    B = batched.BatchedELL(datas, idxs, L)
    v = batched.ensemble_vectors(B.rows, R, seed0=500)
    M = 140
    mu = B.moments(M, v, dtype="c128")
    assert mu.shape == (7, R, M)
    for k in range(7):
        o, n = int(B.offsets[k]), int(B.rows[k])
        for r in range(R):
            ref = oracle.rec_A_tab(M, datas[k], idxs[k], L, v[r, o:o + n])
            ok, err = oracle.moment_tolerance_ok(mu[k, r], ref, REL)
            assert ok, (k, r, err)


def test_batched_graph_replay_is_deterministic(cuda_lib):
    from minijclsquant_gb300 import batched

    datas, idxs, L, _, _ = _ensemble(5, (10, 40), seed=11)
    B = batched.BatchedELL(datas, idxs, L)
    v = batched.ensemble_vectors(B.rows, 2)
    a = B.moments(200, v, dtype="c64")
    b = B.moments(200, v, dtype="c64")
    c = B.moments(200, v, dtype="c128")
    d = B.moments(200, v, dtype="c128")
    assert np.array_equal(a, b) and np.array_equal(c, d)
    # complex64 recursion against complex128, per moment order, relative to mu_0
    err = np.max(np.abs(a - c) / np.abs(c[:, :, :1]))
    assert err < 5e-6


KINDS = {"simple": (0, 1), "staged1": (1, 1), "staged2": (1, 2), "ws1": (2, 1), "ws2": (2, 2)}


@pytest.mark.parametrize("doubled", [False, True])
@pytest.mark.parametrize("kernel", list(KINDS))
@pytest.mark.parametrize("dtype,R", [("c128", 4), ("c64", 2), ("c64", 8)])
def test_batched_kernel_variants_agree(cuda_lib, monkeypatch, kernel, dtype, R, doubled):
    """Every kernel the batched autotuner can pick, forced, against the oracle per
    instance (complex128 at 1e-10 per order; complex64 at its own precision), for the
    direct recursion and for doubled moments."""
    from minijclsquant_gb300 import batched

    if doubled and kernel.startswith("staged"):
        pytest.skip("doubled moments run on the grid-stride and producer-warp kernels")
    monkeypatch.setenv("KPM_STEP_KERNEL", kernel)
    datas, idxs, L, _, _ = _ensemble(6, (3, 70), seed=5)  # 18 .. 9800 sites: tiny and multi-tile instances
    B = batched.BatchedELL(datas, idxs, L)
    B.set_doubling(doubled)
    assert B.doubling == doubled
    v = batched.ensemble_vectors(B.rows, R)
    mu = B.moments(90, v, dtype=dtype)
    cfg = B.step_config(dtype, R)
    assert (cfg["kind"], cfg["rows_per_thread"]) == KINDS[kernel], cfg
    for k in range(6):
        o, n = int(B.offsets[k]), int(B.rows[k])
        for r in range(R):
            ref = oracle.rec_A_tab(90, datas[k], idxs[k], L, v[r, o:o + n])
            if dtype == "c128":
                assert oracle.moment_tolerance_ok(mu[k, r], ref, REL)[0], (k, r)
            else:
                assert np.max(np.abs(mu[k, r] - ref)) / n < 2e-6, (k, r)


def test_batched_autotuner_reports_its_choice(cuda_lib):
    from minijclsquant_gb300 import batched

    datas, idxs, L, _, _ = _ensemble(5, (20, 60), seed=9)
    B = batched.BatchedELL(datas, idxs, L)
    cfg = B.step_config("c64", 2)
    assert cfg["kind"] in (0, 1, 2) and cfg["grid"] >= 1 and cfg["step_us"] > 0
    v = batched.ensemble_vectors(B.rows, 2)
    a = B.moments(64, v, dtype="c64")
    assert B.step_config("c64", 2) == cfg  # the plan is kept
    b = B.moments(64, v, dtype="c64")
    assert np.array_equal(a, b)


def test_batched_rejects_column_outside_its_instance(cuda_lib):
    from minijclsquant_gb300 import _capi, batched

    datas, idxs, L, _, _ = _ensemble(3, (4, 6), seed=1)
    bad = [i.copy() for i in idxs]
    bad[1][0] = datas[1].size // L  # one past the instance's last row (a valid row of the stack)
    with pytest.raises(_capi.KPMError) as e:
        batched.BatchedELL(datas, bad, L)
    assert e.value.status == _capi.KPM_ERR_INDEX


def test_batched_dos_per_instance(cuda_lib):
    """DOS of each instance from the batched moments equals the plain drop-in path."""
    from minijclsquant_gb300 import batched, device

    datas, idxs, L, bnds, _ = _ensemble(3, (12, 20), seed=8)
    B = batched.BatchedELL(datas, idxs, L)
    v = batched.ensemble_vectors(B.rows, 2)
    mu = B.moments(64, v, dtype="c128")
    dos = batched.batched_dos(mu, bnds, 64)
    for k in range(3):
        o, n = int(B.offsets[k]), int(B.rows[k])
        op = device.DeviceELL(datas[k], idxs[k], L)
        mk = device.cheb_moments(op, 64, v[:, o:o + n])
        from minijclsquant_gb300.observables import dos_from_moments

        ref = dos_from_moments(mk, bnds[k], 64)
        assert np.max(np.abs(dos[k][:, 1] - ref[:, 1])) <= 1e-10 * np.max(np.abs(ref[:, 1]))
