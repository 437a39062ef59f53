"""The complex64 form's accuracy bar: DOS error <= 1e-6 against complex128.

An ensemble shaped like the batched configuration (square honeycomb instances with
sides drawn from 32..96 cells, W ~ U[0, 2] eV, own disorder seed each, R = 2 random
vectors, M = 1024, Jackson kernel), smaller so the oracle finishes in seconds.  The
complex64 moments come from the batched recursion and from the plain per-operator
call; the reference moments from the oracle's complex128 restatement of rec_A_tab
(jclsquant/recurrence_functions.py:9-40), which the golden vectors pin.

DOS error of an instance = max_E |rho64(E) - rho128(E)| / max_E |rho128(E)| on the
reference's energy grid (2M + 1 points, jclsquant/observables.py:39); the bar is 1e-6
for the worst instance.  Per-order moment error (relative to mu_0) is held under 1e-7.
"""
import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu

DOS_BAR = 1e-6
M = 1024
R = 2


def _dos_err(d, ref):
    return float(np.max(np.abs(d[:, 1] - ref[:, 1])) / np.max(np.abs(ref[:, 1])))


@pytest.fixture(scope="module")
def ensemble():
    from minijclsquant_gb300 import batched

    datas, idxs, L, bnds, prm = batched.honeycomb_ensemble(10, side_range=(32, 96), W_range=(0.0, 2.0), seed=42)
    rows = np.array([d.size // L for d in datas])
    v = batched.ensemble_vectors(rows, R, seed0=1000)
    offs = np.concatenate([[0], np.cumsum(rows)[:-1]])
    ref = np.stack([np.stack([oracle.rec_A_tab(M, datas[k], idxs[k], L, v[r, offs[k]:offs[k] + rows[k]])
                              for r in range(R)]) for k in range(len(datas))])
    return dict(datas=datas, idxs=idxs, L=L, bnds=bnds, rows=rows, offs=offs, v=v, ref=ref, W=prm["W"])


def test_batched_c64_dos_error_under_bar(cuda_lib, ensemble):
    from minijclsquant_gb300 import batched

    e = ensemble
    B = batched.BatchedELL(e["datas"], e["idxs"], e["L"])
    mu64 = B.moments(M, e["v"], dtype="c64")
    d64 = batched.batched_dos(mu64, e["bnds"], M)
    d128 = batched.batched_dos(e["ref"], e["bnds"], M)
    errs = [_dos_err(a, b) for a, b in zip(d64, d128)]
    assert max(errs) <= DOS_BAR, errs
    per_order = np.max(np.abs(mu64 - e["ref"]) / np.abs(e["ref"][:, :, :1]), axis=(0, 1))
    assert per_order.max() < 1e-7, per_order.max()
    # the complex128 batched recursion meets the drop-in tolerance on the same ensemble
    mu128 = B.moments(M, e["v"], dtype="c128")
    for k in range(len(e["datas"])):
        for r in range(R):
            ok, err = oracle.moment_tolerance_ok(mu128[k, r], e["ref"][k, r], 1e-10)
            assert ok, (k, r, err)


def test_plain_c64_dos_error_under_bar(cuda_lib, ensemble):
    """The same bar through the per-operator call (device.cheb_moments, dtype c64)."""
    from minijclsquant_gb300 import device
    from minijclsquant_gb300.observables import dos_from_moments

    e = ensemble
    for k in (int(np.argmax(e["rows"])), int(np.argmax(e["W"]))):
        op = device.DeviceELL(e["datas"][k], e["idxs"][k], e["L"])
        o, n = int(e["offs"][k]), int(e["rows"][k])
        mu = device.cheb_moments(op, M, e["v"][:, o:o + n], dtype="c64")
        err = _dos_err(dos_from_moments(mu, e["bnds"][k], M), dos_from_moments(e["ref"][k], e["bnds"][k], M))
        assert err <= DOS_BAR, (k, err)
