// kpm_cheb.cuh -- the fused Chebyshev step kernel (SpMV + recursion + epilogues).
//
// One launch advances R vectors by one Chebyshev order over the whole operator:
//
//   MODE_FIRST : T_1 = H T_0                      (values are 2H, result * 0.5)
//   MODE_NEXT  : T_{m+1} = 2H T_m - T_{m-1}        (in place over T_{m-1})
//   MODE_APPLY : y = (a/2)(2H) x + b y             (ell_matrix.dot)
//
// and, in the same pass over the rows, optionally
//   EPI_MOM1/2 : per-CTA partial sums of <v_l | T_new> (conjugate on v_l),
//                accumulated in FP64, deterministic order (no atomics);
//   EPI_SERIES : acc += c_m T_new (rec_A_vec), acc = c_0 T_0 + c_1 T_1 at m = 1.
//
// Reference semantics: aAxby_c (jclsquant/cython_modules/blas_funs.pyx:64-71),
// vdot_c (blas_funs.pyx:83-88), the loop of rec_A_tab
// (jclsquant/recurrence_functions.py:18-38) and of rec_A_vec
// (recurrence_functions.py:121-141).
//
// Thread mapping: TPR threads serve one row; each holds VPT complex values of
// the R = TPR*VPT vectors as one 16-byte (or 8-byte) vector load.  The CTA
// grid-strides over rows so per-thread moment partials are reduced once per
// launch.  Matrix slots are streamed with evict-first loads (read once per
// step), gathered vector entries go through the read-only L1 path.
#pragma once

#include <type_traits>

#include "kpm_async.cuh"
#include "kpm_internal.cuh"

namespace kpm {

template <typename T, int VPT>
struct RawT;
template <>
struct RawT<double, 1> { using type = double2; };
template <>
struct RawT<float, 1> { using type = float2; };
template <>
struct RawT<float, 2> { using type = float4; };

template <typename T, int VPT>
struct Cx {
  T re[VPT];
  T im[VPT];
};

__device__ __forceinline__ void unpack(const double2& r, Cx<double, 1>& c) { c.re[0] = r.x; c.im[0] = r.y; }
__device__ __forceinline__ void unpack(const float2& r, Cx<float, 1>& c) { c.re[0] = r.x; c.im[0] = r.y; }
__device__ __forceinline__ void unpack(const float4& r, Cx<float, 2>& c) {
  c.re[0] = r.x; c.im[0] = r.y; c.re[1] = r.z; c.im[1] = r.w;
}
__device__ __forceinline__ double2 pack(const Cx<double, 1>& c) { return make_double2(c.re[0], c.im[0]); }
__device__ __forceinline__ float2 pack(const Cx<float, 1>& c) { return make_float2(c.re[0], c.im[0]); }
__device__ __forceinline__ float4 pack(const Cx<float, 2>& c) {
  return make_float4(c.re[0], c.im[0], c.re[1], c.im[1]);
}

// Operator value types.  complex128 path: double (real) or double2 (complex).
// complex64 path: every value is carried as an exact two-float split of the FP64
// value 2H = hi + lo (hi = fl32(2H), lo = fl32(2H - hi)): float2 {hi, lo} for a
// real operator, float4 {re_hi, im_hi, re_lo, im_lo} for a complex one.  The
// vectors and all arithmetic stay in FP32; the split only keeps the operator
// itself from being perturbed by float rounding, which would shift the whole
// spectrum (a systematic DOS error that no averaging removes).
template <typename T, bool REAL>
struct MatV { using type = T; };
template <>
struct MatV<double, false> { using type = double2; };
template <>
struct MatV<float, true> { using type = float2; };
template <>
struct MatV<float, false> { using type = float4; };

// acc += h * x
template <int VPT>
__device__ __forceinline__ void madd(Cx<double, VPT>& acc, double h, const Cx<double, VPT>& x) {
#pragma unroll
  for (int k = 0; k < VPT; ++k) {
    acc.re[k] = fma(h, x.re[k], acc.re[k]);
    acc.im[k] = fma(h, x.im[k], acc.im[k]);
  }
}
template <int VPT>
__device__ __forceinline__ void madd(Cx<double, VPT>& acc, double2 h, const Cx<double, VPT>& x) {
#pragma unroll
  for (int k = 0; k < VPT; ++k) {
    acc.re[k] = fma(h.x, x.re[k], acc.re[k]);
    acc.re[k] = fma(-h.y, x.im[k], acc.re[k]);
    acc.im[k] = fma(h.x, x.im[k], acc.im[k]);
    acc.im[k] = fma(h.y, x.re[k], acc.im[k]);
  }
}
// Complex64 accumulation without intermediate rounding: every product h*x is
// split exactly (TwoProduct via FMA) and added with an exact TwoSum into a
// (hi, lo) pair, so a recursion row T_{m+1} = 2H T_m - T_{m-1} is rounded to
// float once, when it is stored.  The _rn intrinsics keep the compiler from
// contracting these steps.  (Error-free transformations: T. J. Dekker,
// Numer. Math. 18 (1971) 224; D. E. Knuth, TAOCP vol. 2, 4.2.2.)
template <int VPT>
struct CxC {
  Cx<float, VPT> hi, lo;
};

__device__ __forceinline__ void two_prod_add(float& hi, float& lo, float a, float b) {
  const float p = __fmul_rn(a, b);
  const float e = __fmaf_rn(a, b, -p);
  const float s = __fadd_rn(hi, p);
  const float bp = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(p, bp));
  hi = s;
  lo = __fadd_rn(lo, __fadd_rn(err, e));
}

// acc += (h.x + h.y) * x, h a real value split into float hi / lo
template <int VPT>
__device__ __forceinline__ void madd(CxC<VPT>& acc, float2 h, const Cx<float, VPT>& x) {
#pragma unroll
  for (int k = 0; k < VPT; ++k) {
    two_prod_add(acc.hi.re[k], acc.lo.re[k], h.x, x.re[k]);
    two_prod_add(acc.hi.im[k], acc.lo.im[k], h.x, x.im[k]);
    acc.lo.re[k] = __fmaf_rn(h.y, x.re[k], acc.lo.re[k]);
    acc.lo.im[k] = __fmaf_rn(h.y, x.im[k], acc.lo.im[k]);
  }
}
// acc += h * x, h a complex value split as {re_hi, im_hi, re_lo, im_lo}
template <int VPT>
__device__ __forceinline__ void madd(CxC<VPT>& acc, float4 h, const Cx<float, VPT>& x) {
#pragma unroll
  for (int k = 0; k < VPT; ++k) {
    two_prod_add(acc.hi.re[k], acc.lo.re[k], h.x, x.re[k]);
    two_prod_add(acc.hi.re[k], acc.lo.re[k], -h.y, x.im[k]);
    two_prod_add(acc.hi.im[k], acc.lo.im[k], h.x, x.im[k]);
    two_prod_add(acc.hi.im[k], acc.lo.im[k], h.y, x.re[k]);
    acc.lo.re[k] = __fmaf_rn(h.z, x.re[k], __fmaf_rn(-h.w, x.im[k], acc.lo.re[k]));
    acc.lo.im[k] = __fmaf_rn(h.z, x.im[k], __fmaf_rn(h.w, x.re[k], acc.lo.im[k]));
  }
}
template <int VPT, typename HS>
__device__ __forceinline__ void madd_first_neg(CxC<VPT>& acc, HS h, const Cx<float, VPT>& x,
                                               const Cx<float, VPT>& old) {
#pragma unroll
  for (int k = 0; k < VPT; ++k) {
    acc.hi.re[k] = -old.re[k];
    acc.hi.im[k] = -old.im[k];
    acc.lo.re[k] = acc.lo.im[k] = 0.f;
  }
  madd(acc, h, x);
}
template <int VPT, typename HS>
__device__ __forceinline__ void mul_first(CxC<VPT>& acc, HS h, const Cx<float, VPT>& x) {
#pragma unroll
  for (int k = 0; k < VPT; ++k) acc.hi.re[k] = acc.hi.im[k] = acc.lo.re[k] = acc.lo.im[k] = 0.f;
  madd(acc, h, x);
}
// The stored (rounded once) value of an accumulator.
template <int VPT>
__device__ __forceinline__ Cx<float, VPT> finish(const CxC<VPT>& a) {
  Cx<float, VPT> r;
#pragma unroll
  for (int k = 0; k < VPT; ++k) {
    r.re[k] = __fadd_rn(a.hi.re[k], a.lo.re[k]);
    r.im[k] = __fadd_rn(a.hi.im[k], a.lo.im[k]);
  }
  return r;
}
template <typename T, int VPT>
__device__ __forceinline__ Cx<T, VPT> finish(const Cx<T, VPT>& a) {
  return a;
}
// Accumulator type: plain for complex128, compensated for complex64.
template <typename T, int VPT>
struct AccOf { using type = Cx<T, VPT>; };
template <int VPT>
struct AccOf<float, VPT> { using type = CxC<VPT>; };

// acc = h * x - old: the first slot of a recursion row, with -T_{m-1} folded
// into the addend of the multiply-add (no separate negation).
template <int VPT>
__device__ __forceinline__ void madd_first_neg(Cx<double, VPT>& acc, double h, const Cx<double, VPT>& x,
                                               const Cx<double, VPT>& old) {
#pragma unroll
  for (int k = 0; k < VPT; ++k) {
    acc.re[k] = fma(h, x.re[k], -old.re[k]);
    acc.im[k] = fma(h, x.im[k], -old.im[k]);
  }
}
template <int VPT>
__device__ __forceinline__ void madd_first_neg(Cx<double, VPT>& acc, double2 h, const Cx<double, VPT>& x,
                                               const Cx<double, VPT>& old) {
#pragma unroll
  for (int k = 0; k < VPT; ++k) {
    acc.re[k] = fma(h.x, x.re[k], -old.re[k]);
    acc.re[k] = fma(-h.y, x.im[k], acc.re[k]);
    acc.im[k] = fma(h.x, x.im[k], -old.im[k]);
    acc.im[k] = fma(h.y, x.re[k], acc.im[k]);
  }
}
// acc = h * x (first slot without a previous vector).
template <int VPT>
__device__ __forceinline__ void mul_first(Cx<double, VPT>& acc, double h, const Cx<double, VPT>& x) {
#pragma unroll
  for (int k = 0; k < VPT; ++k) {
    acc.re[k] = h * x.re[k];
    acc.im[k] = h * x.im[k];
  }
}
template <int VPT>
__device__ __forceinline__ void mul_first(Cx<double, VPT>& acc, double2 h, const Cx<double, VPT>& x) {
#pragma unroll
  for (int k = 0; k < VPT; ++k) {
    acc.re[k] = fma(-h.y, x.im[k], h.x * x.re[k]);
    acc.im[k] = fma(h.y, x.re[k], h.x * x.im[k]);
  }
}
// conj(l) * t, accumulated into (re, im).
template <typename A, typename T>
__device__ __forceinline__ void cdot_acc(A& re, A& im, T lr, T li, T tr, T ti) {
  re = fma((A)lr, (A)tr, re);
  re = fma((A)li, (A)ti, re);
  im = fma((A)lr, (A)ti, im);
  im = fma(-(A)li, (A)tr, im);
}

// Reduce VPT complex FP64 values over the lanes that serve the same vectors,
// then over the warps of the CTA, and store the R totals at out[0..R).
template <int TPR, int VPT>
__device__ __forceinline__ void block_reduce_store(double (&re)[VPT], double (&im)[VPT], double2* out,
                                                   double2* smem, bool named = false) {
  constexpr int R = TPR * VPT;
#pragma unroll
  for (int off = TPR; off < 32; off <<= 1) {
#pragma unroll
    for (int k = 0; k < VPT; ++k) {
      re[k] += __shfl_xor_sync(0xffffffffu, re[k], off);
      im[k] += __shfl_xor_sync(0xffffffffu, im[k], off);
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane < TPR) {
#pragma unroll
    for (int k = 0; k < VPT; ++k) smem[warp * R + lane * VPT + k] = make_double2(re[k], im[k]);
  }
  // `named`: only the kBlock compute threads take part (a warp-specialised CTA)
  if (named) named_sync(kBlock); else __syncthreads();
  if (threadIdx.x < R) {
    double2 s = make_double2(0.0, 0.0);
#pragma unroll 1
    for (int w = 0; w < kBlock / 32; ++w) {
      s.x += smem[w * R + threadIdx.x].x;
      s.y += smem[w * R + threadIdx.x].y;
    }
    out[threadIdx.x] = s;
  }
  if (named) named_sync(kBlock); else __syncthreads();
}

template <typename T, bool REAL, int TPR, int VPT, int MODE, int EPI>
__global__ void __launch_bounds__(kBlock) cheb_step_kernel(const StepParams p) {
  using Raw = typename RawT<T, VPT>::type;
  using MV = typename MatV<T, REAL>::type;
  constexpr int R = TPR * VPT;
  constexpr int RPB = kBlock / TPR;
  constexpr bool MOM = (EPI & EPI_MOM1) != 0;
  constexpr bool SERIES = (EPI & EPI_SERIES) != 0;
  constexpr bool STORE = (EPI & EPI_STORE) != 0;
  constexpr bool F32 = std::is_same<T, float>::value;
  // complex64 products are summed in float over at most kFlush rows per thread,
  // then folded into the FP64 accumulators.
  constexpr int kFlush = 8;

  __shared__ double2 smem[(kBlock / 32) * R];

  const int sub = threadIdx.x % TPR;
  const int rl = threadIdx.x / TPR;
  const MV* __restrict__ val = static_cast<const MV*>(p.val);
  const int32_t* __restrict__ col = p.col;
  const Raw* __restrict__ tcur = static_cast<const Raw*>(p.tcur);
  Raw* tout = static_cast<Raw*>(p.tout);
  const Raw* __restrict__ vl = static_cast<const Raw*>(p.vl);
  const Raw* __restrict__ vl2 = static_cast<const Raw*>(p.vl2);
  const bool mom2 = MOM && (vl2 != nullptr);
  // doubling: set 0 <T_{m}|T_{m-1}> (own row of tcur), set 1 sum (|T_{m-1}|^2 - hv)
  const bool dbl = MOM && MODE == MODE_NEXT && p.dbl != 0;
  const int L = p.L;
  const int64_t ld = p.ld;

  double m1r[VPT], m1i[VPT], m2r[VPT], m2i[VPT];     // moment of the new vector
  double z1r[VPT], z1i[VPT], z2r[VPT], z2i[VPT];     // FIRST: moment of T_0
  T f1r[VPT], f1i[VPT], f2r[VPT], f2i[VPT], g1r[VPT], g1i[VPT], g2r[VPT], g2i[VPT];
#pragma unroll
  for (int k = 0; k < VPT; ++k) {
    m1r[k] = m1i[k] = m2r[k] = m2i[k] = 0.0;
    z1r[k] = z1i[k] = z2r[k] = z2i[k] = 0.0;
    f1r[k] = f1i[k] = f2r[k] = f2i[k] = g1r[k] = g1i[k] = g2r[k] = g2i[k] = T(0);
  }
  int pending = 0;

  double2 c_lo = make_double2(0.0, 0.0), c_hi = make_double2(0.0, 0.0);
  if (SERIES) {
    if (MODE == MODE_FIRST) {
      c_lo = p.coef[0];
      c_hi = p.coef[1];
    } else {
      c_hi = p.coef[p.m];
    }
  }

  const int64_t stride = (int64_t)gridDim.x * RPB;
  for (int64_t row = (int64_t)blockIdx.x * RPB + rl; row < p.n_pad; row += stride) {
    const int64_t vi = row * TPR + sub;
    typename AccOf<T, VPT>::type accum;
    Cx<T, VPT> old;
    if (MODE == MODE_NEXT && p.tprev != nullptr) {
      unpack(static_cast<const Raw*>(p.tprev)[vi], old);
    } else if (MODE == MODE_NEXT || (MODE == MODE_APPLY && p.b.x != 0.0) || (MODE == MODE_APPLY && p.b.y != 0.0)) {
      unpack(tout[vi], old);
    } else {
#pragma unroll
      for (int k = 0; k < VPT; ++k) old.re[k] = old.im[k] = T(0);
    }
    // slots in groups of four: all loads of a group are issued before its FMAs;
    // the first slot folds -T_{m-1} into its multiply-add.
    for (int s = 0; s < L; s += 4) {
      int c[4];
      MV h[4];
      Cx<T, VPT> x[4];
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (s + u < L) {
          c[u] = __ldcs(col + (int64_t)(s + u) * ld + row);
          h[u] = __ldcs(val + (int64_t)(s + u) * ld + row);
        }
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (s + u < L) unpack(__ldg(tcur + (int64_t)c[u] * TPR + sub), x[u]);
      if (s == 0) {
        if (MODE == MODE_NEXT)
          madd_first_neg(accum, h[0], x[0], old);
        else
          mul_first(accum, h[0], x[0]);
      } else {
        madd(accum, h[0], x[0]);
      }
#pragma unroll
      for (int u = 1; u < 4; ++u)
        if (s + u < L) madd(accum, h[u], x[u]);
    }
    Cx<T, VPT> acc = finish(accum);
    if (MODE == MODE_FIRST) {
#pragma unroll
      for (int k = 0; k < VPT; ++k) {
        acc.re[k] *= T(0.5);
        acc.im[k] *= T(0.5);
      }
    }
    if (MODE == MODE_APPLY) {
      const T ar = (T)p.a_half.x, ai = (T)p.a_half.y, br = (T)p.b.x, bi = (T)p.b.y;
#pragma unroll
      for (int k = 0; k < VPT; ++k) {
        const T xr = acc.re[k], xi = acc.im[k];
        acc.re[k] = ar * xr - ai * xi + (br * old.re[k] - bi * old.im[k]);
        acc.im[k] = ar * xi + ai * xr + (br * old.im[k] + bi * old.re[k]);
      }
    }
    if (STORE) tout[vi] = pack(acc);

    if (MOM && dbl) {
      Cx<T, VPT> own;
      unpack(__ldg(tcur + vi), own);
      const T* hv = static_cast<const T*>(p.hv) + vi * VPT;
#pragma unroll
      for (int k = 0; k < VPT; ++k) {
        const T hk = __ldg(hv + k);
        if (F32) {
          cdot_acc(f1r[k], f1i[k], acc.re[k], acc.im[k], own.re[k], own.im[k]);
          f2r[k] += fmaf(own.re[k], own.re[k], fmaf(own.im[k], own.im[k], -hk));
        } else {
          cdot_acc(m1r[k], m1i[k], acc.re[k], acc.im[k], own.re[k], own.im[k]);
          m2r[k] += fma(own.re[k], own.re[k], fma(own.im[k], own.im[k], -hk));
        }
      }
      if (F32 && ++pending == kFlush) {
        pending = 0;
#pragma unroll
        for (int k = 0; k < VPT; ++k) {
          m1r[k] += (double)f1r[k]; m1i[k] += (double)f1i[k]; f1r[k] = f1i[k] = T(0);
          m2r[k] += (double)f2r[k]; f2r[k] = T(0);
        }
      }
    } else if (MOM) {
      Cx<T, VPT> l;
      unpack(__ldg(vl + vi), l);
      Cx<T, VPT> l2;
      if (mom2) unpack(__ldg(vl2 + vi), l2);
      Cx<T, VPT> t0;
      if (MODE == MODE_FIRST) unpack(__ldg(tcur + vi), t0);
#pragma unroll
      for (int k = 0; k < VPT; ++k) {
        if (F32) {
          cdot_acc(f1r[k], f1i[k], l.re[k], l.im[k], acc.re[k], acc.im[k]);
          if (mom2) cdot_acc(f2r[k], f2i[k], l2.re[k], l2.im[k], acc.re[k], acc.im[k]);
          if (MODE == MODE_FIRST) {
            cdot_acc(g1r[k], g1i[k], l.re[k], l.im[k], t0.re[k], t0.im[k]);
            if (mom2) cdot_acc(g2r[k], g2i[k], l2.re[k], l2.im[k], t0.re[k], t0.im[k]);
          }
        } else {
          cdot_acc(m1r[k], m1i[k], l.re[k], l.im[k], acc.re[k], acc.im[k]);
          if (mom2) cdot_acc(m2r[k], m2i[k], l2.re[k], l2.im[k], acc.re[k], acc.im[k]);
          if (MODE == MODE_FIRST) {
            cdot_acc(z1r[k], z1i[k], l.re[k], l.im[k], t0.re[k], t0.im[k]);
            if (mom2) cdot_acc(z2r[k], z2i[k], l2.re[k], l2.im[k], t0.re[k], t0.im[k]);
          }
        }
      }
      if (F32 && ++pending == kFlush) {
        pending = 0;
#pragma unroll
        for (int k = 0; k < VPT; ++k) {
          m1r[k] += (double)f1r[k]; m1i[k] += (double)f1i[k]; f1r[k] = f1i[k] = T(0);
          m2r[k] += (double)f2r[k]; m2i[k] += (double)f2i[k]; f2r[k] = f2i[k] = T(0);
          z1r[k] += (double)g1r[k]; z1i[k] += (double)g1i[k]; g1r[k] = g1i[k] = T(0);
          z2r[k] += (double)g2r[k]; z2i[k] += (double)g2i[k]; g2r[k] = g2i[k] = T(0);
        }
      }
    }

    if (SERIES) {
      Raw* ser = static_cast<Raw*>(p.series);
      Cx<T, VPT> o;
      if (MODE == MODE_FIRST) {
        Cx<T, VPT> t0;
        unpack(__ldg(tcur + vi), t0);
#pragma unroll
        for (int k = 0; k < VPT; ++k) {
          // c0*T0 + c1*T1 (rec_A_vec: A_kpm = c0*v; A_kpm += c1*T1)
          const T r0 = (T)c_lo.x * t0.re[k] - (T)c_lo.y * t0.im[k];
          const T i0 = (T)c_lo.x * t0.im[k] + (T)c_lo.y * t0.re[k];
          o.re[k] = r0 + ((T)c_hi.x * acc.re[k] - (T)c_hi.y * acc.im[k]);
          o.im[k] = i0 + ((T)c_hi.x * acc.im[k] + (T)c_hi.y * acc.re[k]);
        }
      } else {
        unpack(ser[vi], o);
#pragma unroll
        for (int k = 0; k < VPT; ++k) {
          // axpy2(c_m, 1, T1, A_kpm): y = c_m*x + 1*y as two nested FMAs per component (the
          // producer-warp series step uses the same expression)
          o.re[k] = fma((T)c_hi.x, acc.re[k], fma(-(T)c_hi.y, acc.im[k], o.re[k]));
          o.im[k] = fma((T)c_hi.x, acc.im[k], fma((T)c_hi.y, acc.re[k], o.im[k]));
        }
      }
      ser[vi] = pack(o);
    }
  }

  if (MOM) {
    if (F32) {
#pragma unroll
      for (int k = 0; k < VPT; ++k) {
        m1r[k] += (double)f1r[k]; m1i[k] += (double)f1i[k];
        m2r[k] += (double)f2r[k]; m2i[k] += (double)f2i[k];
        z1r[k] += (double)g1r[k]; z1i[k] += (double)g1i[k];
        z2r[k] += (double)g2r[k]; z2i[k] += (double)g2i[k];
      }
    }
    const int64_t set_stride = (int64_t)gridDim.x * R;
    const int sets = (mom2 || dbl) ? 2 : 1;
    // partial layout for one step: [sets][grid][R]
    if (MODE == MODE_FIRST) {
      double2* p0 = p.part;                       // step m = 0
      double2* p1 = p.part + p.part_step_stride;  // step m = 1
      block_reduce_store<TPR, VPT>(z1r, z1i, p0 + (int64_t)blockIdx.x * R, smem);
      block_reduce_store<TPR, VPT>(m1r, m1i, p1 + (int64_t)blockIdx.x * R, smem);
      if (sets == 2) {
        block_reduce_store<TPR, VPT>(z2r, z2i, p0 + set_stride + (int64_t)blockIdx.x * R, smem);
        block_reduce_store<TPR, VPT>(m2r, m2i, p1 + set_stride + (int64_t)blockIdx.x * R, smem);
      }
    } else {
      block_reduce_store<TPR, VPT>(m1r, m1i, p.part + (int64_t)blockIdx.x * R, smem);
      if (sets == 2) block_reduce_store<TPR, VPT>(m2r, m2i, p.part + set_stride + (int64_t)blockIdx.x * R, smem);
    }
  }
}

// Dispatch over (real, R, mode, epi) for one precision.
template <typename T, bool REAL, int TPR, int VPT>
int launch_mode_epi(int mode, int epi, const StepParams& p, int grid, cudaStream_t s) {
#define KPM_L(MODE_, EPI_) cheb_step_kernel<T, REAL, TPR, VPT, MODE_, EPI_><<<grid, kBlock, 0, s>>>(p)
  const int key = mode * 64 + epi;
  switch (key) {
    case MODE_FIRST * 64 + (EPI_STORE | EPI_MOM1): KPM_L(MODE_FIRST, EPI_STORE | EPI_MOM1); break;
    case MODE_FIRST * 64 + (EPI_STORE | EPI_SERIES): KPM_L(MODE_FIRST, EPI_STORE | EPI_SERIES); break;
    case MODE_FIRST * 64 + EPI_STORE: KPM_L(MODE_FIRST, EPI_STORE); break;
    case MODE_NEXT * 64 + (EPI_STORE | EPI_MOM1): KPM_L(MODE_NEXT, EPI_STORE | EPI_MOM1); break;
    case MODE_NEXT * 64 + (EPI_STORE | EPI_SERIES): KPM_L(MODE_NEXT, EPI_STORE | EPI_SERIES); break;
    case MODE_NEXT * 64 + EPI_STORE: KPM_L(MODE_NEXT, EPI_STORE); break;
    case MODE_APPLY * 64 + EPI_STORE: KPM_L(MODE_APPLY, EPI_STORE); break;
    case MODE_APPLY * 64 + EPI_MOM1: KPM_L(MODE_APPLY, EPI_MOM1); break;
    default: return KPM_ERR_UNSUPPORTED;
  }
#undef KPM_L
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_cuda_error(e);
    return KPM_ERR_CUDA;
  }
  return KPM_OK;
}

}  // namespace kpm
