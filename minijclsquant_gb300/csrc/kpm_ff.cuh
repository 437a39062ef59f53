// kpm_ff.cuh -- float-float arithmetic for complex128-accurate work on the FP32 pipe.
//
// A real number is an unevaluated pair hi + lo of floats (~48 significant bits).
// Products are split exactly (TwoProduct through FMA) and sums are exact (TwoSum),
// so a sum of products rounds only at the 2^-48 level.  A complex number is a
// float4 {re_hi, im_hi, re_lo, im_lo}, 16 bytes like a complex128; a real
// operator value is the float2 {hi, lo} of 2H.  (Float-float arithmetic:
// T. J. Dekker, Numer. Math. 18 (1971) 224; D. E. Knuth, TAOCP vol. 2, 4.2.2.)
#pragma once

#include "kpm_cheb.cuh"

namespace kpm {

constexpr int kFfFlush = 8;

struct FF {  // complex value (rh + rl) + i (ih + il)
  float rh, ih, rl, il;
};

__device__ __forceinline__ FF ff_of(const float4& q) { return FF{q.x, q.y, q.z, q.w}; }
__device__ __forceinline__ float4 ff_raw(const FF& a) { return make_float4(a.rh, a.ih, a.rl, a.il); }

// (hi, lo) += (ah + al)(bh + bl); the al*bl term (below 2^-48 relative) is dropped
__device__ __forceinline__ void ff_madd(float& hi, float& lo, float ah, float al, float bh, float bl) {
  two_prod_add(hi, lo, ah, bh);
  lo = __fmaf_rn(ah, bl, lo);
  lo = __fmaf_rn(al, bh, lo);
}

// (hi, lo) -> (s, e), s = fl(hi + lo), e the exact remainder
__device__ __forceinline__ void ff_norm(float& hi, float& lo) {
  const float s = __fadd_rn(hi, lo);
  const float bp = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(lo, bp));
  hi = s;
  lo = e;
}

// (hi, lo) += (hi2, lo2), exact in the hi parts (TwoSum)
__device__ __forceinline__ void ff_add(float& hi, float& lo, float hi2, float lo2) {
  const float s = __fadd_rn(hi, hi2);
  const float bp = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(hi2, bp));
  hi = s;
  lo = __fadd_rn(__fadd_rn(lo, lo2), e);
}

// acc += h x, h real (float2 {hi, lo}) or complex (float4 {re_hi, im_hi, re_lo, im_lo})
__device__ __forceinline__ void ff_mac(FF& a, float2 h, const FF& x) {
  ff_madd(a.rh, a.rl, h.x, h.y, x.rh, x.rl);
  ff_madd(a.ih, a.il, h.x, h.y, x.ih, x.il);
}
__device__ __forceinline__ void ff_mac(FF& a, float4 h, const FF& x) {
  ff_madd(a.rh, a.rl, h.x, h.z, x.rh, x.rl);
  ff_madd(a.rh, a.rl, -h.y, -h.w, x.ih, x.il);
  ff_madd(a.ih, a.il, h.x, h.z, x.ih, x.il);
  ff_madd(a.ih, a.il, h.y, h.w, x.rh, x.rl);
}

// moment accumulator: (re, im) as float pairs, += conj(l) t
struct FFMom {
  float rh, rl, ih, il;
};
__device__ __forceinline__ void ff_cdot(FFMom& m, const FF& l, const FF& t) {
  ff_madd(m.rh, m.rl, l.rh, l.rl, t.rh, t.rl);
  ff_madd(m.rh, m.rl, l.ih, l.il, t.ih, t.il);
  ff_madd(m.ih, m.il, l.rh, l.rl, t.ih, t.il);
  ff_madd(m.ih, m.il, -l.ih, -l.il, t.rh, t.rl);
}
__device__ __forceinline__ void ff_fold(double& re, double& im, FFMom& m) {
  re += (double)m.rh + (double)m.rl;
  im += (double)m.ih + (double)m.il;
  m = FFMom{0.f, 0.f, 0.f, 0.f};
}

// ---- FP64 recursion with float-float moment products -------------------------------
// The FP64 vector T_{m+1} is split into float pairs with integer operations only (the FP64
// pipe, the bound of the FP64 recursion, does no extra work): hi is x rounded to 24
// significant bits (an integer add of half the dropped unit carries into the exponent
// when it must), lo = x - hi exactly as a signed 29-bit count of x's last-place units,
// rounded to a float, so hi + lo = x to 2^-49 relative.  The left vector is packed once
// per call (pack_left_ff).  Products run through ff_cdot, and the float-pair sums are
// folded into FP64 every kFfFoldRows rows.  A value outside [2^-50, 2^59) that is not zero
// (nor an FP64 subnormal, taken as zero) reports false, and the caller forms that row's
// product in FP64 instead: every float-pair product and its rounding error then stay
// normal floats, and a component's sum of 2 kFfFoldRows products stays below 2^126, so the
// folds (DADDs and conversions on the FP64 pipe, the bound of this step) come every 128 rows.
constexpr int kFfFoldRows = 128;

__device__ __forceinline__ bool ff_split_f64(double x, float& hi, float& lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned long long r = b + (1ull << 28);  // round the 29 dropped bits to nearest
  const unsigned hb = (unsigned)(b >> 32), lb = (unsigned)b;
  const unsigned rh = (unsigned)(r >> 32), rlw = (unsigned)r & 0xe0000000u;
  const unsigned sgn = hb & 0x80000000u;
  const unsigned e = (hb >> 20) & 0x7ffu;
  const unsigned er = (rh >> 20) & 0x7ffu;  // e or e + 1
  const bool normal = e >= 973u;
  // float exponent field er - 896 (= er - 1023 + 127); 20 + 3 mantissa bits
  hi = __uint_as_float(normal ? (sgn | ((er - 896u) << 23) | ((rh & 0xfffffu) << 3) | (rlw >> 29)) : 0u);
  // |x| - |hi| = d 2^(e - 1075): d the low words' difference, within [-2^28, 2^28].  d is
  // converted without a conversion instruction (those issue on the FP64 pipe): for |k| < 2^22,
  // bits(1.5 2^(23+s)) + k read as a float is 1.5 2^(23+s) + k 2^s exactly, so subtracting
  // the constant leaves k 2^s.  d = dh 2^14 + dl with dh (signed) and dl in [0, 2^14).
  const int d = (int)(lb - rlw);
  const unsigned ch = normal ? (((e - 911u) << 23) | 0x400000u) : 0u;  // 1.5 2^(23 + e - 1061)
  const unsigned cl = normal ? (((e - 925u) << 23) | 0x400000u) : 0u;  // 1.5 2^(23 + e - 1075)
  const float fh = __fsub_rn(__uint_as_float(ch + (unsigned)(d >> 14)), __uint_as_float(ch));
  const float fl = __fsub_rn(__uint_as_float(cl + (unsigned)(d & 0x3fff)), __uint_as_float(cl));
  lo = normal ? __uint_as_float(__float_as_uint(__fadd_rn(fh, fl)) ^ sgn) : 0.f;
  return e == 0u || (normal && e <= 1081u);
}

// a packed left-vector high part: zero, or a normal float in [2^-50, 2^59) (NaN marks an
// element that pack_left_ff could not carry)
__device__ __forceinline__ bool ff_left_ok(float h) {
  const unsigned u = __float_as_uint(h) & 0x7fffffffu;
  const unsigned ef = u >> 23;
  return u == 0u || (ef >= 77u && ef <= 185u);
}

// the float pairs of a packed left-vector entry carried in a double2 slot
__device__ __forceinline__ FF ff_from_slot(double re, double im) {
  const unsigned long long a = (unsigned long long)__double_as_longlong(re);
  const unsigned long long b = (unsigned long long)__double_as_longlong(im);
  return FF{__uint_as_float((unsigned)a), __uint_as_float((unsigned)(a >> 32)), __uint_as_float((unsigned)b),
            __uint_as_float((unsigned)(b >> 32))};
}

template <bool REAL>
struct FFVal { using type = float2; };
template <>
struct FFVal<false> { using type = float4; };

}  // namespace kpm
