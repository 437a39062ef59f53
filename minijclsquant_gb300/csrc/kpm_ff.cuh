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

template <bool REAL>
struct FFVal { using type = float2; };
template <>
struct FFVal<false> { using type = float4; };

}  // namespace kpm
