"""The tf32 rounding of the tensor-core contraction's operand split (to_tf32_int in
minijclsquant_gb300/csrc/kpm_tc.cuh): add half of the dropped unit (bit 12) to the FP32 bits and
clear the 13 low bits.  Restated here on uint32 arrays and checked against an independent
round-to-nearest, ties-away-from-zero to 10 explicit mantissa bits computed in float64, over
random values, exact ties, carries into the exponent, subnormals and the top of the range.  On the
GPU the contraction that rounds this way agrees bit for bit with the one using cvt.rna.tf32.f32
(tests/test_gpu_mu_nm.py)."""
import numpy as np


def tf32_int(x):
    b = np.asarray(x, dtype=np.float32).view(np.uint32)
    return ((b + np.uint32(0x1000)) & np.uint32(0xFFFFE000)).view(np.float32)


def tf32_rna_reference(x):
    """Nearest value with 10 explicit mantissa bits (11 significant), ties away from zero; the
    exponent range of FP32 (subnormals keep the same absolute quantum, 2^-136)."""
    x = np.asarray(x, dtype=np.float32).astype(np.float64)
    out = np.zeros_like(x)
    nz = x != 0
    a = np.abs(x[nz])
    e = np.floor(np.log2(a))
    e = np.where(np.ldexp(1.0, e.astype(np.int64)) > a, e - 1, e)  # exact floor(log2) for powers of two
    e = np.maximum(e, -126.0)  # subnormals: the quantum of the smallest normal binade
    q = np.ldexp(1.0, (e - 10).astype(np.int64))
    k = np.floor(a / q + 0.5)  # half away from zero for the magnitude
    r = k * q
    out[nz] = np.sign(x[nz]) * r
    with np.errstate(over="ignore"):
        return out.astype(np.float32)


def test_random_values_match():
    rng = np.random.default_rng(11)
    bits = rng.integers(0, 0x7F800000, 2_000_000, dtype=np.uint64).astype(np.uint32)  # finite, >= 0
    x = bits.view(np.float32)
    x = np.concatenate([x, -x])
    assert np.array_equal(tf32_int(x).view(np.uint32), tf32_rna_reference(x).view(np.uint32))


def test_ties_carries_and_edges():
    base = np.array([1.0, 1.5, 3.0, 1e-3, 6.0e4, 2.0 ** -126, 2.0 ** -130, 1.7e38], dtype=np.float32)
    b = base.view(np.uint32)
    cases = []
    for low in (0x0FFF, 0x1000, 0x1001, 0x1FFF, 0x0001):  # below, at and above the tie; largest; smallest
        cases.append((b & np.uint32(0xFFFFE000)) | np.uint32(low))
    cases.append(np.uint32(0x3FFFF000) + np.zeros(1, np.uint32))  # mantissa all ones at a tie: carries to 2.0
    cases.append(np.uint32(0x007FF000) + np.zeros(1, np.uint32))  # largest subnormal tie: carries to 2^-126
    cases.append(np.uint32(0x7F7FF000) + np.zeros(1, np.uint32))  # FLT_MAX's tie: rounds up to infinity
    x = np.concatenate(cases).view(np.float32)
    x = np.concatenate([x, -x, np.zeros(1, np.float32)])
    got = tf32_int(x)
    ref = tf32_rna_reference(x)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    assert got[0].view(np.uint32) & np.uint32(0x1FFF) == 0
    assert np.isinf(tf32_int(np.array([np.float32(3.4028235e38)]))[0]) == np.isinf(
        tf32_rna_reference(np.array([np.float32(3.4028235e38)]))[0])
