// kpm_adjoint.cu -- reverse-mode (adjoint) Chebyshev recursion.
//
// For L = sum_m c_m Re <v | T_m(H) v> with H real symmetric (rescaled), the
// adjoint vectors obey the backward three-term recursion
//
//     lambda_M = lambda_{M+1} = 0,
//     lambda_m = c_m conj(v) + 2 H lambda_{m+1} - lambda_{m+2},   m = M-1 .. 1,
//
// and the derivative with respect to the operator entry in row i, column j is
//
//     dL/dH_ij = Re[ lambda_1[i] t_0[j] + 2 sum_{m>=2} lambda_m[i] t_{m-1}[j] ],
//
// t_m = T_m(H) v.  The forward pass keeps (t_k, t_{k+1}) every `ckpt` steps;
// the backward pass walks the segments from last to first, recomputes the
// segment's t_m from its checkpoint, and runs the adjoint steps through it.
// Gradients are accumulated per ELL slot in FP64 (one read-modify-write per
// slot and step), summed over the R vectors inside one thread.
//
// This has no counterpart in the reference, which has no derivatives; the
// forward recursion it differentiates is rec_A_tab
// (jclsquant/recurrence_functions.py:9-40).
#include <algorithm>
#include <cstring>

#include "kpm_cheb.cuh"
#include "kpm_ff.cuh"

namespace kpm {

struct AdjParams {
  const double* val;     // 2H, real, [L][ld]
  const int32_t* col;
  int64_t ld;
  int L;
  int64_t n_pad;
  const double2* lam1;   // lambda_{m+1}, gathered        [n_pad][R]
  double2* lam2;         // lambda_{m+2} in, lambda_m out  [n_pad][R]
  const double2* u;      // v (conjugated on use)          [n_pad][R]
  const double2* tprev;  // t_{m-1}, gathered              [n_pad][R]
  double* grad;          // dL/dH per slot, [L][ld], accumulated
  double c;              // c_m
  double w;              // 1 for m = 1, else 2
  // optional forward step of the segment recomputed next, out of place:
  // rout = 2H rcur - rprev ([n_pad][R]); skipped when rout is null
  const double2* rcur;
  const double2* rprev;
  double2* rout;
};

// One adjoint order for every row, and (RC) one forward recompute step of the
// next segment in the same pass over the operator: the two are independent, so
// each row's entries are read once and the FP64 pipe gets two FMA streams.  The
// recompute keeps the forward kernel's order (first product folded with
// -t_{j-2}, then the slots in order), so it reproduces the forward pass exactly.
template <int R, bool RC>
__global__ void __launch_bounds__(kBlock) adj_step_kernel(const AdjParams p) {
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < p.n_pad;
       row += (int64_t)gridDim.x * blockDim.x) {
    double ar[R], ai[R], fr[R], fi[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const double2 o = p.lam2[row * R + r];
      const double2 v = __ldg(p.u + row * R + r);
      ar[r] = fma(p.c, v.x, -o.x);   // c * conj(v) - lambda_{m+2}
      ai[r] = fma(-p.c, v.y, -o.y);
      if (RC) {
        const double2 q = p.rprev[row * R + r];
        fr[r] = -q.x;
        fi[r] = -q.y;
      }
    }
    for (int s = 0; s < p.L; ++s) {
      const int j = __ldcs(p.col + (int64_t)s * p.ld + row);
      const double h = __ldcs(p.val + (int64_t)s * p.ld + row);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const double2 x = __ldg(p.lam1 + (int64_t)j * R + r);
        ar[r] = fma(h, x.x, ar[r]);
        ai[r] = fma(h, x.y, ai[r]);
        if (RC) {
          const double2 y = __ldg(p.rcur + (int64_t)j * R + r);
          fr[r] = fma(h, y.x, fr[r]);
          fi[r] = fma(h, y.y, fi[r]);
        }
      }
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
      p.lam2[row * R + r] = make_double2(ar[r], ai[r]);
      if (RC) p.rout[row * R + r] = make_double2(fr[r], fi[r]);
    }
    for (int s = 0; s < p.L; ++s) {
      const int j = __ldcs(p.col + (int64_t)s * p.ld + row);
      double g = 0.0;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const double2 t = __ldg(p.tprev + (int64_t)j * R + r);
        g = fma(ar[r], t.x, g);
        g = fma(-ai[r], t.y, g);
      }
      double* gp = p.grad + (int64_t)s * p.ld + row;
      *gp = fma(p.w, g, *gp);
    }
  }
}

template <int R>
static int launch_adj_r(const AdjParams& p, int grid, cudaStream_t s) {
  if (p.rout)
    adj_step_kernel<R, true><<<grid, kBlock, 0, s>>>(p);
  else
    adj_step_kernel<R, false><<<grid, kBlock, 0, s>>>(p);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_cuda_error(e);
    return KPM_ERR_CUDA;
  }
  return KPM_OK;
}

static int launch_adj(int R, const AdjParams& p, int grid, cudaStream_t s) {
  switch (R) {
    case 1: return launch_adj_r<1>(p, grid, s);
    case 2: return launch_adj_r<2>(p, grid, s);
    case 4: return launch_adj_r<4>(p, grid, s);
    case 8: return launch_adj_r<8>(p, grid, s);
    default: return KPM_ERR_UNSUPPORTED;
  }
}

// [L][ld] -> [n][L]
__global__ void slots_to_rows_kernel(const double* __restrict__ src, int64_t ld, int L, int64_t n, double* dst) {
  const int64_t total = n * L;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = t / L;
    const int s = (int)(t % L);
    dst[t] = src[(int64_t)s * ld + row];
  }
}

// New values (AoS c128, device) into an existing operator, doubled; a non-zero
// imaginary part on a real-stored operator is reported through err.
__global__ void set_values_kernel(const double2* __restrict__ data, int64_t n, int64_t n_pad, int L, bool real,
                                  void* val, int* err) {
  const int64_t total = (int64_t)L * n_pad;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int s = (int)(t / n_pad);
    const int64_t row = t % n_pad;
    double2 v = make_double2(0.0, 0.0);
    if (row < n) v = data[row * L + s];
    if (real) {
      static_cast<double*>(val)[t] = 2.0 * v.x;
      if (v.y != 0.0) atomicExch(err, KPM_ERR_DTYPE);
    } else {
      static_cast<double2*>(val)[t] = make_double2(2.0 * v.x, 2.0 * v.y);
    }
  }
}

// ---- the backward pass in float-float arithmetic (KPM_C128F) -----------------
// The same adjoint order and fused recompute as adj_step_kernel, with every real
// number a float pair (kpm_ff.cuh): the FP32 pipe instead of GB300's 1/64-rate
// FP64 pipe.  lam*, u, segment vectors: float4 per complex; grad: float2 {hi, lo}
// per ELL slot; values: the float pairs of 2H.
struct AdjFFParams {
  const float2* val;  // 2H, [L][ld]
  const int32_t* col;
  int64_t ld;
  int L;
  int64_t n_pad;
  const float4* lam1;  // lambda_{m+1}, gathered
  float4* lam2;        // lambda_{m+2} in, lambda_m out
  const float4* u;     // v
  const float4* tprev; // t_{m-1}, gathered
  float2* grad;        // per slot, accumulated
  float c_hi, c_lo;    // c_m
  float w;             // 1 for m = 1, else 2 (exact)
  const float4* rcur;  // optional recompute step: rout = 2H rcur - rprev
  const float4* rprev;
  float4* rout;
};

template <int R, bool RC>
__global__ void __launch_bounds__(kBlock) adj_ff_kernel(const AdjFFParams p) {
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < p.n_pad;
       row += (int64_t)gridDim.x * blockDim.x) {
    FF a[R], f[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const FF o = ff_of(p.lam2[row * R + r]);
      const FF v = ff_of(__ldg(p.u + row * R + r));
      a[r] = FF{-o.rh, -o.ih, -o.rl, -o.il};
      ff_madd(a[r].rh, a[r].rl, p.c_hi, p.c_lo, v.rh, v.rl);   // + c Re v
      ff_madd(a[r].ih, a[r].il, -p.c_hi, -p.c_lo, v.ih, v.il); // - c Im v (conj)
      if (RC) {
        const FF q = ff_of(p.rprev[row * R + r]);
        f[r] = FF{-q.rh, -q.ih, -q.rl, -q.il};
      }
    }
    for (int s = 0; s < p.L; ++s) {
      const int64_t j = __ldcs(p.col + (int64_t)s * p.ld + row);
      const float2 h = __ldcs(p.val + (int64_t)s * p.ld + row);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        ff_mac(a[r], h, ff_of(__ldg(p.lam1 + j * R + r)));
        if (RC) ff_mac(f[r], h, ff_of(__ldg(p.rcur + j * R + r)));
      }
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
      ff_norm(a[r].rh, a[r].rl);
      ff_norm(a[r].ih, a[r].il);
      p.lam2[row * R + r] = ff_raw(a[r]);
      if (RC) {
        ff_norm(f[r].rh, f[r].rl);
        ff_norm(f[r].ih, f[r].il);
        p.rout[row * R + r] = ff_raw(f[r]);
      }
    }
    for (int s = 0; s < p.L; ++s) {
      const int64_t j = __ldcs(p.col + (int64_t)s * p.ld + row);
      float gh = 0.f, gl = 0.f;  // sum_r Re(lambda_m[i] t_{m-1}[j])
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const FF t = ff_of(__ldg(p.tprev + j * R + r));
        ff_madd(gh, gl, a[r].rh, a[r].rl, t.rh, t.rl);
        ff_madd(gh, gl, -a[r].ih, -a[r].il, t.ih, t.il);
      }
      float2* gp = p.grad + (int64_t)s * p.ld + row;
      float2 gv = *gp;
      ff_add(gv.x, gv.y, p.w * gh, p.w * gl);
      *gp = gv;
    }
  }
}

// t_j = 2H t_{j-1} - t_{j-2} out of place (the segment recompute without an adjoint order)
template <int R>
__global__ void __launch_bounds__(kBlock) ff_recompute_kernel(const float2* __restrict__ val,
                                                               const int32_t* __restrict__ col, int64_t ld, int L,
                                                               int64_t n_pad, const float4* __restrict__ tcur,
                                                               const float4* __restrict__ tprev, float4* tout) {
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < n_pad;
       row += (int64_t)gridDim.x * blockDim.x) {
    FF f[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const FF q = ff_of(tprev[row * R + r]);
      f[r] = FF{-q.rh, -q.ih, -q.rl, -q.il};
    }
    for (int s = 0; s < L; ++s) {
      const int64_t j = __ldcs(col + (int64_t)s * ld + row);
      const float2 h = __ldcs(val + (int64_t)s * ld + row);
#pragma unroll
      for (int r = 0; r < R; ++r) ff_mac(f[r], h, ff_of(__ldg(tcur + j * R + r)));
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
      ff_norm(f[r].rh, f[r].rl);
      ff_norm(f[r].ih, f[r].il);
      tout[row * R + r] = ff_raw(f[r]);
    }
  }
}

// complex128 -> float pairs, elementwise
__global__ void c128_to_ff_kernel(const double2* __restrict__ src, int64_t count, float4* __restrict__ dst) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < count; t += (int64_t)gridDim.x * blockDim.x) {
    const double2 z = src[t];
    const float xh = (float)z.x, yh = (float)z.y;
    dst[t] = make_float4(xh, yh, (float)(z.x - (double)xh), (float)(z.y - (double)yh));
  }
}

// float-pair gradient [L][ld] -> FP64 [n][L]
__global__ void ff_slots_to_rows_kernel(const float2* __restrict__ src, int64_t ld, int L, int64_t n, double* dst) {
  const int64_t total = n * L;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = t / L;
    const int s = (int)(t % L);
    const float2 g = src[(int64_t)s * ld + row];
    dst[t] = (double)g.x + (double)g.y;
  }
}

template <int R>
static int launch_adj_ff_r(const AdjFFParams& p, int grid, cudaStream_t s) {
  if (p.rout)
    adj_ff_kernel<R, true><<<grid, kBlock, 0, s>>>(p);
  else
    adj_ff_kernel<R, false><<<grid, kBlock, 0, s>>>(p);
  return check_cuda(cudaGetLastError());
}

static int launch_adj_ff(int R, const AdjFFParams& p, int grid, cudaStream_t s) {
  switch (R) {
    case 1: return launch_adj_ff_r<1>(p, grid, s);
    case 2: return launch_adj_ff_r<2>(p, grid, s);
    case 4: return launch_adj_ff_r<4>(p, grid, s);
    case 8: return launch_adj_ff_r<8>(p, grid, s);
    default: return KPM_ERR_UNSUPPORTED;
  }
}

static int launch_ff_recompute(int R, const kpm_ell_s* h, const void* tcur, const void* tprev, void* tout, int grid,
                               cudaStream_t s) {
  const float2* val = static_cast<const float2*>(h->val32);
#define KPM_RC(RR)                                                                                          \
  ff_recompute_kernel<RR><<<grid, kBlock, 0, s>>>(val, h->col, h->n_pad, h->L, h->n_pad,                    \
                                                  static_cast<const float4*>(tcur),                         \
                                                  static_cast<const float4*>(tprev), static_cast<float4*>(tout)); \
  break
  switch (R) {
    case 1: KPM_RC(1);
    case 2: KPM_RC(2);
    case 4: KPM_RC(4);
    case 8: KPM_RC(8);
    default: return KPM_ERR_UNSUPPORTED;
  }
#undef KPM_RC
  return check_cuda(cudaGetLastError());
}

static int grid_rows(const kpm_ell_s* h) {
  const int64_t g = (h->n_pad + kBlock - 1) / kBlock;
  return (int)std::max<int64_t>(1, std::min<int64_t>(g, (int64_t)h->sm_count * 8));
}

}  // namespace kpm

using namespace kpm;

namespace kpm {

static int backward_fp64(kpm_ell_s* h, const double* c, double* grad, cudaStream_t s) {
  const int R = h->adj_R, M = h->adj_M, ckpt = h->adj_ckpt;
  Workspace& ws = h->ws;
  const size_t vb = (size_t)h->n_pad * R * sizeof(double2);
  const int nseg = (M - 1 + ckpt - 1) / ckpt;
  KPM_TRY(ensure(ws.seg, (size_t)2 * ckpt * vb));  // two segment buffers: consumed, recomputed
  KPM_TRY(ensure(ws.acc, vb));
  KPM_TRY(ensure(ws.acc2, vb));
  KPM_TRY(ensure(ws.grad, (size_t)h->L * h->n_pad * sizeof(double)));
  std::vector<double> ch(M);
  KPM_CUDA_TRY(cudaMemcpyAsync(ch.data(), c, M * sizeof(double), cudaMemcpyDeviceToHost, s));
  KPM_CUDA_TRY(cudaStreamSynchronize(s));
  double2* la = static_cast<double2*>(ws.acc.p);   // lambda_{m+1}
  double2* lb = static_cast<double2*>(ws.acc2.p);  // lambda_{m+2} -> lambda_m
  KPM_CUDA_TRY(cudaMemsetAsync(la, 0, vb, s));
  KPM_CUDA_TRY(cudaMemsetAsync(lb, 0, vb, s));
  KPM_CUDA_TRY(cudaMemsetAsync(ws.grad.p, 0, (size_t)h->L * h->n_pad * sizeof(double), s));
  char* ck = static_cast<char*>(ws.ckpt.p);
  char* segs[2] = {static_cast<char*>(ws.seg.p), static_cast<char*>(ws.seg.p) + (size_t)ckpt * vb};
  const int grid = grid_rows(h);
  StepParams p = base_params(h, false);
  // segment q holds t_{k0} .. t_{k0 + count - 1}, k0 = q * ckpt; the adjoint orders
  // m = k0 + count .. k0 + 1 use t_{m-1}
  auto seg_count = [&](int q) { return std::min(q * ckpt + ckpt, M - 1) - q * ckpt; };
  auto load_ckpt = [&](int q, char* dst) -> int {
    KPM_CUDA_TRY(cudaMemcpyAsync(dst, ck + (size_t)q * 2 * vb, (seg_count(q) > 1 ? 2 : 1) * vb,
                                 cudaMemcpyDeviceToDevice, s));
    return KPM_OK;
  };
  auto recompute_step = [&](char* sg, int j) -> int {  // t_j of a segment from t_{j-1}, t_{j-2}
    p.tcur = sg + (size_t)(j - 1) * vb;
    p.tprev = sg + (size_t)(j - 2) * vb;
    p.tout = sg + (size_t)j * vb;
    return launch_step(false, true, R, MODE_NEXT, EPI_STORE, p, grid, s);
  };
  // the last segment is recomputed alone; every earlier one during the adjoint
  // orders of the segment after it
  int cur = 0;
  KPM_TRY(load_ckpt(nseg - 1, segs[cur]));
  for (int j = 2; j < seg_count(nseg - 1); ++j) KPM_TRY(recompute_step(segs[cur], j));
  for (int q = nseg - 1; q >= 0; --q) {
    const int k0 = q * ckpt;
    const int count = seg_count(q);
    const int nxt = cur ^ 1;
    const int rc_steps = q > 0 ? std::max(0, seg_count(q - 1) - 2) : 0;
    if (q > 0) KPM_TRY(load_ckpt(q - 1, segs[nxt]));
    int i = 0;
    for (int m = k0 + count; m >= k0 + 1; --m) {
      AdjParams a;
      a.val = static_cast<const double*>(h->val64);
      a.col = h->col;
      a.ld = h->n_pad;
      a.L = h->L;
      a.n_pad = h->n_pad;
      a.lam1 = la;
      a.lam2 = lb;
      a.u = static_cast<const double2*>(ws.vl.p);
      a.tprev = reinterpret_cast<const double2*>(segs[cur] + (size_t)(m - 1 - k0) * vb);
      a.grad = static_cast<double*>(ws.grad.p);
      a.c = ch[m];
      a.w = m == 1 ? 1.0 : 2.0;
      a.rcur = a.rprev = nullptr;
      a.rout = nullptr;
      if (i < rc_steps) {  // fused: t_{i+2} of segment q - 1
        a.rprev = reinterpret_cast<const double2*>(segs[nxt] + (size_t)i * vb);
        a.rcur = reinterpret_cast<const double2*>(segs[nxt] + (size_t)(i + 1) * vb);
        a.rout = reinterpret_cast<double2*>(segs[nxt] + (size_t)(i + 2) * vb);
        ++i;
      }
      KPM_TRY(launch_adj(R, a, grid, s));
      std::swap(la, lb);  // lambda_m becomes lambda_{m'+1} of the next (lower) order
    }
    for (; i < rc_steps; ++i) KPM_TRY(recompute_step(segs[nxt], i + 2));
    cur = nxt;
  }
  const int64_t total = h->n * (int64_t)h->L;
  slots_to_rows_kernel<<<(int)std::min<int64_t>((total + 255) / 256, 65536), 256, 0, s>>>(
      static_cast<const double*>(ws.grad.p), h->n_pad, h->L, h->n, grad);
  KPM_CUDA_TRY(cudaGetLastError());
  return KPM_OK;
}


static int backward_ff(kpm_ell_s* h, const double* c, double* grad, cudaStream_t s) {
  const int R = h->adj_R, M = h->adj_M, ckpt = h->adj_ckpt;
  KPM_TRY(ensure_f32_values(h, s));
  Workspace& ws = h->ws;
  const int64_t count = h->n_pad * R;                      // complex entries of one vector set
  const size_t vb = (size_t)count * sizeof(float4);       // float pairs: the size of complex128
  const int nseg = (M - 1 + ckpt - 1) / ckpt;
  KPM_TRY(ensure(ws.seg, (size_t)2 * ckpt * vb));
  KPM_TRY(ensure(ws.acc, vb));
  KPM_TRY(ensure(ws.acc2, vb));
  KPM_TRY(ensure(ws.td, vb));
  KPM_TRY(ensure(ws.grad, (size_t)h->L * h->n_pad * sizeof(float2)));
  std::vector<double> ch(M);
  KPM_CUDA_TRY(cudaMemcpyAsync(ch.data(), c, M * sizeof(double), cudaMemcpyDeviceToHost, s));
  KPM_CUDA_TRY(cudaStreamSynchronize(s));
  float4* la = static_cast<float4*>(ws.acc.p);   // lambda_{m+1}
  float4* lb = static_cast<float4*>(ws.acc2.p);  // lambda_{m+2} -> lambda_m
  KPM_CUDA_TRY(cudaMemsetAsync(la, 0, vb, s));
  KPM_CUDA_TRY(cudaMemsetAsync(lb, 0, vb, s));
  KPM_CUDA_TRY(cudaMemsetAsync(ws.grad.p, 0, (size_t)h->L * h->n_pad * sizeof(float2), s));
  const int cg = (int)std::min<int64_t>((2 * count + 255) / 256, 65536);
  float4* u = static_cast<float4*>(ws.td.p);
  c128_to_ff_kernel<<<cg, 256, 0, s>>>(static_cast<const double2*>(ws.vl.p), count, u);
  KPM_CUDA_TRY(cudaGetLastError());
  const char* ck = static_cast<const char*>(ws.ckpt.p);  // complex128 checkpoint pairs
  const size_t ckb = (size_t)count * sizeof(double2);
  char* segs[2] = {static_cast<char*>(ws.seg.p), static_cast<char*>(ws.seg.p) + (size_t)ckpt * vb};
  const int grid = grid_rows(h);
  auto seg_count = [&](int q) { return std::min(q * ckpt + ckpt, M - 1) - q * ckpt; };
  auto load_ckpt = [&](int q, char* dst) -> int {
    c128_to_ff_kernel<<<cg, 256, 0, s>>>(reinterpret_cast<const double2*>(ck + (size_t)q * 2 * ckb),
                                         (seg_count(q) > 1 ? 2 : 1) * count, reinterpret_cast<float4*>(dst));
    return check_cuda(cudaGetLastError());
  };
  auto recompute_step = [&](char* sg, int j) -> int {
    return launch_ff_recompute(R, h, sg + (size_t)(j - 1) * vb, sg + (size_t)(j - 2) * vb, sg + (size_t)j * vb, grid,
                               s);
  };
  int cur = 0;
  KPM_TRY(load_ckpt(nseg - 1, segs[cur]));
  for (int j = 2; j < seg_count(nseg - 1); ++j) KPM_TRY(recompute_step(segs[cur], j));
  for (int q = nseg - 1; q >= 0; --q) {
    const int k0 = q * ckpt;
    const int cnt = seg_count(q);
    const int nxt = cur ^ 1;
    const int rc_steps = q > 0 ? std::max(0, seg_count(q - 1) - 2) : 0;
    if (q > 0) KPM_TRY(load_ckpt(q - 1, segs[nxt]));
    int i = 0;
    for (int m = k0 + cnt; m >= k0 + 1; --m) {
      AdjFFParams a;
      a.val = static_cast<const float2*>(h->val32);
      a.col = h->col;
      a.ld = h->n_pad;
      a.L = h->L;
      a.n_pad = h->n_pad;
      a.lam1 = la;
      a.lam2 = lb;
      a.u = u;
      a.tprev = reinterpret_cast<const float4*>(segs[cur] + (size_t)(m - 1 - k0) * vb);
      a.grad = static_cast<float2*>(ws.grad.p);
      a.c_hi = (float)ch[m];
      a.c_lo = (float)(ch[m] - (double)a.c_hi);
      a.w = m == 1 ? 1.f : 2.f;
      a.rcur = a.rprev = nullptr;
      a.rout = nullptr;
      if (i < rc_steps) {  // fused: t_{i+2} of segment q - 1
        a.rprev = reinterpret_cast<const float4*>(segs[nxt] + (size_t)i * vb);
        a.rcur = reinterpret_cast<const float4*>(segs[nxt] + (size_t)(i + 1) * vb);
        a.rout = reinterpret_cast<float4*>(segs[nxt] + (size_t)(i + 2) * vb);
        ++i;
      }
      KPM_TRY(launch_adj_ff(R, a, grid, s));
      std::swap(la, lb);
    }
    for (; i < rc_steps; ++i) KPM_TRY(recompute_step(segs[nxt], i + 2));
    cur = nxt;
  }
  const int64_t total = h->n * (int64_t)h->L;
  ff_slots_to_rows_kernel<<<(int)std::min<int64_t>((total + 255) / 256, 65536), 256, 0, s>>>(
      static_cast<const float2*>(ws.grad.p), h->n_pad, h->L, h->n, grad);
  KPM_CUDA_TRY(cudaGetLastError());
  return KPM_OK;
}

}  // namespace kpm

using namespace kpm;

extern "C" {

int kpm_ell_set_values(kpm_ell* h, const double* data, unsigned flags, void* stream) {
  if (!h || !data) return KPM_ERR_INVALID_ARG;
  if (flags & ~(unsigned)KPM_FLAG_DEVICE_PTRS) return KPM_ERR_INVALID_ARG;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int64_t count = h->n * (int64_t)h->L;
  const double2* src = reinterpret_cast<const double2*>(data);
  DevBuf stage;
  if (!(flags & KPM_FLAG_DEVICE_PTRS)) {
    KPM_TRY(ensure(stage, count * sizeof(double2)));
    KPM_CUDA_TRY(cudaMemcpyAsync(stage.p, data, count * sizeof(double2), cudaMemcpyHostToDevice, s));
    src = static_cast<const double2*>(stage.p);
  }
  const int64_t slots = (int64_t)h->L * h->n_pad;
  set_values_kernel<<<(int)std::min<int64_t>((slots + 255) / 256, 65536), 256, 0, s>>>(src, h->n, h->n_pad, h->L,
                                                                                       h->is_real != 0, h->val64,
                                                                                       h->err_flag);
  KPM_CUDA_TRY(cudaGetLastError());
  if (stage.p) {
    KPM_CUDA_TRY(cudaStreamSynchronize(s));
    release(stage);
  }
  return values_changed(h, s);
}

int kpm_adjoint_forward(kpm_ell* h, int R, int M, int ckpt, const double* v, double* mu, void* stream) {
  if (!h || !v || !mu || M < 2 || ckpt < 2) return KPM_ERR_INVALID_ARG;
  if (R != 1 && R != 2 && R != 4 && R != 8) return KPM_ERR_UNSUPPORTED;
  if (!h->is_real) return KPM_ERR_UNSUPPORTED;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  Workspace& ws = h->ws;
  const size_t vb = (size_t)h->n_pad * R * sizeof(double2);
  const int nseg = (M - 1 + ckpt - 1) / ckpt;
  StepConfig cfg;
  KPM_TRY(step_config(h, false, R, kSetsFp64Products, s, &cfg));  // FP64 moments: the checkpointed forward
  KPM_TRY(ensure(ws.ta, vb));
  KPM_TRY(ensure(ws.tb, vb));
  KPM_TRY(ensure(ws.vl, vb));
  KPM_TRY(ensure(ws.ckpt, (size_t)nseg * 2 * vb));
  const int64_t step_stride = (int64_t)cfg.grid * R;
  KPM_TRY(ensure(ws.part, (size_t)kChunk * step_stride * sizeof(double2)));
  KPM_TRY(pack_vectors(v, h->n, h->n_pad, R, 0, R, false, ws.ta.p, s));
  KPM_CUDA_TRY(cudaMemcpyAsync(ws.vl.p, ws.ta.p, vb, cudaMemcpyDeviceToDevice, s));
  char* ck = static_cast<char*>(ws.ckpt.p);
  double2* part = static_cast<double2*>(ws.part.p);
  double* outs[2] = {mu, mu};
  StepParams p = base_params(h, false);
  p.vl = ws.vl.p;
  p.part_step_stride = step_stride;
  p.tcur = ws.ta.p;
  p.tout = ws.tb.p;
  p.part = part;
  KPM_TRY(launch_step(false, true, R, MODE_FIRST, EPI_STORE | EPI_MOM1, p, cfg.grid, s));
  KPM_CUDA_TRY(cudaMemcpyAsync(ck, ws.ta.p, vb, cudaMemcpyDeviceToDevice, s));
  KPM_CUDA_TRY(cudaMemcpyAsync(ck + vb, ws.tb.p, vb, cudaMemcpyDeviceToDevice, s));
  void* tprev = ws.ta.p;
  void* tcur = ws.tb.p;
  int m0 = 0;
  for (int m = 2; m < M; ++m) {
    if (m - m0 == kChunk) {
      KPM_TRY(reduce_partials(part, kChunk, 1, cfg.grid, R, outs, R, 0, M, m0, s));
      m0 = m;
    }
    p.tcur = tcur;
    p.tout = tprev;
    p.part = part + (int64_t)(m - m0) * step_stride;
    KPM_TRY(launch_next(false, true, R, cfg, p, s));
    if (m % ckpt == 0 && m / ckpt < nseg)
      KPM_CUDA_TRY(cudaMemcpyAsync(ck + (size_t)(m / ckpt) * 2 * vb, tprev, vb, cudaMemcpyDeviceToDevice, s));
    if (m % ckpt == 1 && m / ckpt < nseg)
      KPM_CUDA_TRY(cudaMemcpyAsync(ck + (size_t)(m / ckpt) * 2 * vb + vb, tprev, vb, cudaMemcpyDeviceToDevice, s));
    std::swap(tprev, tcur);
  }
  KPM_TRY(reduce_partials(part, M - m0, 1, cfg.grid, R, outs, R, 0, M, m0, s));
  h->adj_R = R;
  h->adj_M = M;
  h->adj_ckpt = ckpt;
  return KPM_OK;
}

int kpm_adjoint_backward(kpm_ell* h, const double* c, double* grad, void* stream) {
  return kpm_adjoint_backward_ex(h, c, grad, KPM_C128, stream);
}

int kpm_adjoint_backward_ex(kpm_ell* h, const double* c, double* grad, int dtype, void* stream) {
  if (!h || !c || !grad) return KPM_ERR_INVALID_ARG;
  if (h->adj_M < 2) return KPM_ERR_INVALID_ARG;  // no forward pass recorded
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (dtype == KPM_C128) return backward_fp64(h, c, grad, s);
  if (dtype == KPM_C128F) return backward_ff(h, c, grad, s);
  return KPM_ERR_DTYPE;
}

}  // extern "C"
