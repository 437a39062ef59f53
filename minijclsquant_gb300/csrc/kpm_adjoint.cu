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

static int grid_rows(const kpm_ell_s* h) {
  const int64_t g = (h->n_pad + kBlock - 1) / kBlock;
  return (int)std::max<int64_t>(1, std::min<int64_t>(g, (int64_t)h->sm_count * 8));
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
  if (h->val32) {  // the complex64 copy is rebuilt on its next use
    KPM_CUDA_TRY(cudaStreamSynchronize(s));
    cudaFree(h->val32);
    h->val32 = nullptr;
  }
  if (stage.p) {
    KPM_CUDA_TRY(cudaStreamSynchronize(s));
    release(stage);
  }
  return KPM_OK;
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
  KPM_TRY(step_config(h, false, R, 1, s, &cfg));
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
  if (!h || !c || !grad) return KPM_ERR_INVALID_ARG;
  if (h->adj_M < 2) return KPM_ERR_INVALID_ARG;  // no forward pass recorded
  const int R = h->adj_R, M = h->adj_M, ckpt = h->adj_ckpt;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
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

}  // extern "C"
