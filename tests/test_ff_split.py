"""The integer split of an FP64 value into a float pair used by the FP64 recursion's
float-float moment products (ff_split_f64 in minijclsquant_gb300/csrc/kpm_ff.cuh), restated
step for step in numpy integer arithmetic: hi + lo = x to 2^-49 relative, |lo| <= 2^-24 |hi|,
zero and FP64 subnormals split to (0, 0), and values outside [2^-50, 2^59) report False."""
import numpy as np


def _split(x):
    x = np.asarray(x, dtype=np.float64)
    b = x.view(np.uint64)
    r = b + np.uint64(1 << 28)
    hb = (b >> np.uint64(32)).astype(np.uint32)
    lb = (b & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    rh = (r >> np.uint64(32)).astype(np.uint32)
    rlw = (r & np.uint64(0xFFFFFFFF)).astype(np.uint32) & np.uint32(0xE0000000)
    sgn = hb & np.uint32(0x80000000)
    e = (hb >> np.uint32(20)) & np.uint32(0x7FF)
    er = (rh >> np.uint32(20)) & np.uint32(0x7FF)
    normal = e >= 973
    with np.errstate(over="ignore"):
        hbits = sgn | ((er - np.uint32(896)) << np.uint32(23)) | ((rh & np.uint32(0xFFFFF)) << np.uint32(3)) | (
            rlw >> np.uint32(29))
        hi = np.where(normal, hbits, np.uint32(0)).view(np.float32)
        d = (lb - rlw).view(np.int32)
        ch = np.where(normal, ((e - np.uint32(911)) << np.uint32(23)) | np.uint32(0x400000), np.uint32(0))
        cl = np.where(normal, ((e - np.uint32(925)) << np.uint32(23)) | np.uint32(0x400000), np.uint32(0))
        fh = (ch + (d >> 14).view(np.uint32)).view(np.float32) - ch.view(np.float32)
        fl = (cl + (d & 0x3FFF).view(np.uint32)).view(np.float32) - cl.view(np.float32)
        s = (fh + fl).astype(np.float32)
    lo = np.where(normal, (s.view(np.uint32) ^ sgn).view(np.float32), np.float32(0))
    ok = (e == 0) | (normal & (e <= 1081))
    return hi, lo, ok


def test_split_error_bound_and_range():
    rng = np.random.default_rng(7)
    n = 2_000_000
    x = rng.uniform(1, 2, n) * np.exp2(rng.integers(-50, 59, n).astype(np.float64))  # [2^-50, 2^59)
    k = rng.integers(-49, 60, n // 4)
    x[: n // 4] = np.ldexp(1.0 - np.ldexp(1.0, -30), k)  # just below a power of two: the rounding carries
    x[n // 2:] *= -1
    hi, lo, ok = _split(x)
    assert ok.all()
    rel = np.abs((hi.astype(np.float64) + lo.astype(np.float64)) - x) / np.abs(x)
    assert rel.max() <= 2.0 ** -49
    assert np.all(np.abs(lo) <= np.ldexp(np.abs(hi).astype(np.float64), -24))


def test_split_edges():
    vals = np.array([0.0, -0.0, 5e-324, -2.2e-308, 1e-20, 2.0 ** -51, 2.0 ** -50, 2.0 ** 59 - 2.0 ** 28, 2.0 ** 59,
                     1e25, np.inf, -np.inf, np.nan])
    hi, lo, ok = _split(vals)
    assert ok.tolist() == [True, True, True, True, False, False, True, True, False, False, False, False, False]
    assert np.all(hi[:4] == 0) and np.all(lo[:4] == 0)
    assert hi[6] == np.float32(2.0 ** -50) and lo[6] == 0


def test_fold_interval_keeps_float_pair_sums_finite():
    """The float-pair moment sums of the complex128 step are folded into FP64 every kFfFoldRows rows;
    each component adds two products per row, each below (2^upper)^2 for split inputs below 2^upper.
    The constants are read from the kernel header, so a longer fold interval without a tighter range
    (or the reverse) fails here before any float-pair sum can overflow."""
    import os
    import re

    src = open(os.path.join(os.path.dirname(__file__), "..", "minijclsquant_gb300", "csrc", "kpm_ff.cuh")).read()
    rows = int(re.search(r"constexpr int kFfFoldRows = (\d+);", src).group(1))
    e_max = int(re.search(r"normal && e <= (\d+)u", src).group(1))  # FP64 exponent field of the largest split
    ef_max = int(re.search(r"ef >= 77u && ef <= (\d+)u", src).group(1))  # float exponent field, left vector
    upper = e_max - 1023 + 1  # split values are below 2^upper
    assert ef_max - 127 + 1 == upper  # the left vector's guard matches the split's
    assert 2 * rows * 2.0 ** (2 * upper) < 2.0 ** 128  # below FLT_MAX's binade
