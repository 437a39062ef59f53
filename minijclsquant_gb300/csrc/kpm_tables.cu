// kpm_tables.cu -- Chebyshev vector tables, Clenshaw tables and per-slot sums (complex128).
//
// These are the pieces of reverse-mode differentiation of the Kubo-Greenwood
// conductivity (minijclsquant_gb300/adjoint.py, KuboPlan): its moment matrix
//   mu_nm = <v| V T_n(H) V T_m(H) |v>
// couples every order n with every order m, so the backward pass needs every
// T_m(H) v and T_n(H) V v at once (as tables of one vector each), two reverse
// recursions with a different source vector per order, and per-slot sums over
// the orders that turn them into d/dH and d/dV of every stored matrix entry.
//
// Layout: a table is M rows of n complex128 (row m of vector v at tab + m n), the
// caller's unpadded layout; operators are the handles' SoA doubled values 2H
// (double when real, double2 otherwise) with int32 columns, [slot][n_pad].
// Every kernel is deterministic (no atomics): one thread owns one row.
#include <algorithm>

#include "kpm_internal.cuh"

namespace kpm {
namespace {

__device__ __forceinline__ void cfma(double2& acc, double h, double2 x) {
  acc.x = fma(h, x.x, acc.x);
  acc.y = fma(h, x.y, acc.y);
}
__device__ __forceinline__ void cfma(double2& acc, double2 h, double2 x) {
  acc.x = fma(h.x, x.x, fma(-h.y, x.y, acc.x));
  acc.y = fma(h.x, x.y, fma(h.y, x.x, acc.y));
}

template <bool REAL>
struct Val {
  using T = double2;
};
template <>
struct Val<true> {
  using T = double;
};

// Operator term sum_s 2M[s][i] x[col(s, i)] of one row.
template <bool REAL>
__device__ __forceinline__ double2 row_product(const void* val, const int32_t* __restrict__ col, int L, int64_t ld,
                                               int64_t i, const double2* __restrict__ x) {
  using V = typename Val<REAL>::T;
  const V* __restrict__ v = static_cast<const V*>(val);
  double2 acc = make_double2(0.0, 0.0);
  for (int s = 0; s < L; ++s) {
    const int j = col[(int64_t)s * ld + i];
    cfma(acc, v[(int64_t)s * ld + i], __ldg(x + j));
  }
  return acc;
}

// One row block of a table step:
//   dst[i]  = fh * (2H x)[i] + fs * (2S z)[i] + bp * prev[i] + add[i]
//   dst2[i] = fs2 * (2S x)[i]                                     (dst2 != null)
// Terms whose pointer is null are left out.  fh, fs, fs2 carry the 1/2 or 1 that turns
// the stored doubled values into H, 2H, S.
struct TableStep {
  const void* vh;
  const int32_t* ch;
  int Lh;
  const void* vs;
  const int32_t* cs;
  int Ls;
  int64_t ld, n;
  double fh, fs, fs2, bp;
  const double2* x;
  const double2* z;
  const double2* prev;
  const double2* add;
  double2* dst;
  double2* dst2;
};

template <bool RH, bool RS>
__global__ void __launch_bounds__(256) table_step_kernel(const TableStep p) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < p.n; i += (int64_t)gridDim.x * blockDim.x) {
    double2 out = make_double2(0.0, 0.0);
    if (p.x && p.vh) {
      const double2 a = row_product<RH>(p.vh, p.ch, p.Lh, p.ld, i, p.x);
      out.x = p.fh * a.x;
      out.y = p.fh * a.y;
    }
    if (p.z && p.vs) {
      const double2 a = row_product<RS>(p.vs, p.cs, p.Ls, p.ld, i, p.z);
      out.x = fma(p.fs, a.x, out.x);
      out.y = fma(p.fs, a.y, out.y);
    }
    if (p.prev) {
      const double2 q = p.prev[i];
      out.x = fma(p.bp, q.x, out.x);
      out.y = fma(p.bp, q.y, out.y);
    }
    if (p.add) {
      const double2 q = p.add[i];
      out.x += q.x;
      out.y += q.y;
    }
    if (p.dst) p.dst[i] = out;
    if (p.dst2) {
      const double2 a = row_product<RS>(p.vs, p.cs, p.Ls, p.ld, i, p.x);
      p.dst2[i] = make_double2(p.fs2 * a.x, p.fs2 * a.y);
    }
  }
}

// Whether two device ranges of `bytes` bytes each share memory.
bool overlap(const void* a, const void* b, size_t bytes) {
  const uintptr_t x = reinterpret_cast<uintptr_t>(a), y = reinterpret_cast<uintptr_t>(b);
  return x < y + bytes && y < x + bytes;
}

int grid_rows(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 8192)); }

int launch_table_step(bool rh, bool rs, const TableStep& p, cudaStream_t s) {
  const int g = grid_rows(p.n);
  if (rh && rs)
    table_step_kernel<true, true><<<g, 256, 0, s>>>(p);
  else if (rh)
    table_step_kernel<true, false><<<g, 256, 0, s>>>(p);
  else if (rs)
    table_step_kernel<false, true><<<g, 256, 0, s>>>(p);
  else
    table_step_kernel<false, false><<<g, 256, 0, s>>>(p);
  return check_cuda(cudaGetLastError());
}

// out[i L + s] (+)= sum_{k<K} coef[k] conj(A[k lda + i]) B[k ldb + col(s, i)]   (coef null: 1)
template <int LMAX>
__global__ void __launch_bounds__(256) slot_sum_kernel(const int32_t* __restrict__ col, int L, int64_t ld, int64_t n,
                                                       int K, const double* __restrict__ coef,
                                                       const double2* __restrict__ A, int64_t lda,
                                                       const double2* __restrict__ B, int64_t ldb, int accumulate,
                                                       double2* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int c[LMAX];
    double2 acc[LMAX];
#pragma unroll
    for (int s = 0; s < LMAX; ++s) {
      if (s < L) {
        c[s] = col[(int64_t)s * ld + i];
        acc[s] = accumulate ? out[i * L + s] : make_double2(0.0, 0.0);
      }
    }
    for (int k = 0; k < K; ++k) {
      double2 a = A[(int64_t)k * lda + i];
      const double w = coef ? coef[k] : 1.0;
      a.x *= w;
      a.y *= -w;  // conj(A) scaled
      const double2* __restrict__ b = B + (int64_t)k * ldb;
#pragma unroll
      for (int s = 0; s < LMAX; ++s)
        if (s < L) cfma(acc[s], a, __ldg(b + c[s]));
    }
#pragma unroll
    for (int s = 0; s < LMAX; ++s)
      if (s < L) out[i * L + s] = acc[s];
  }
}

}  // namespace
}  // namespace kpm

using namespace kpm;

extern "C" {

int kpm_cheb_table(kpm_ell* h, kpm_ell* s_op, int M, const double* v, double* tab, double* stab, void* stream) {
  if (!h || !v || !tab || M < 1 || (s_op && !stab) || (!s_op && stab)) return KPM_ERR_INVALID_ARG;
  if (s_op && (s_op->n != h->n || s_op->n_pad != h->n_pad)) return KPM_ERR_SHAPE;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int64_t n = h->n;
  double2* T = reinterpret_cast<double2*>(tab);
  double2* ST = reinterpret_cast<double2*>(stab);
  if (s_op && overlap(tab, stab, (size_t)M * n * sizeof(double2))) return KPM_ERR_INVALID_ARG;
  if (v != tab) {  // v may be row 0 of the table itself
    if (overlap(v, tab, (size_t)n * sizeof(double2))) return KPM_ERR_INVALID_ARG;
    KPM_CUDA_TRY(cudaMemcpyAsync(T, v, (size_t)n * sizeof(double2), cudaMemcpyDeviceToDevice, s));
  }
  TableStep p{};
  p.vh = h->val64;
  p.ch = h->col;
  p.Lh = h->L;
  p.vs = s_op ? s_op->val64 : nullptr;
  p.cs = s_op ? s_op->col : nullptr;
  p.Ls = s_op ? s_op->L : 0;
  p.ld = h->n_pad;
  p.n = n;
  p.fs2 = 0.5;  // S from the stored 2S
  const bool rs = s_op ? s_op->is_real != 0 : true;
  for (int m = 1; m < M; ++m) {
    // T_m = H T_0 (m = 1) or 2H T_{m-1} - T_{m-2}; with S, also S T_{m-1}
    p.x = T + (int64_t)(m - 1) * n;
    p.fh = m == 1 ? 0.5 : 1.0;
    p.prev = m == 1 ? nullptr : T + (int64_t)(m - 2) * n;
    p.bp = -1.0;
    p.dst = T + (int64_t)m * n;
    p.dst2 = s_op ? ST + (int64_t)(m - 1) * n : nullptr;
    KPM_TRY(launch_table_step(h->is_real != 0, rs, p, s));
  }
  if (s_op) {  // S T_{M-1}
    TableStep q = p;
    q.x = T + (int64_t)(M - 1) * n;
    q.vh = nullptr;
    q.prev = nullptr;
    q.dst = nullptr;
    q.dst2 = ST + (int64_t)(M - 1) * n;
    KPM_TRY(launch_table_step(h->is_real != 0, rs, q, s));
  }
  return KPM_OK;
}

int kpm_cheb_clenshaw_table(kpm_ell* h, kpm_ell* s_op, int M, const double* z, double* lam, void* stream) {
  if (!h || !z || !lam || M < 1) return KPM_ERR_INVALID_ARG;
  if (s_op && (s_op->n != h->n || s_op->n_pad != h->n_pad)) return KPM_ERR_SHAPE;
  // every row of z is gathered while rows of lam are written: the two may not share memory
  if (overlap(z, lam, (size_t)M * h->n * sizeof(double2))) return KPM_ERR_INVALID_ARG;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int64_t n = h->n;
  const double2* Z = reinterpret_cast<const double2*>(z);
  double2* Lm = reinterpret_cast<double2*>(lam);
  TableStep p{};
  p.vh = h->val64;
  p.ch = h->col;
  p.Lh = h->L;
  p.vs = s_op ? s_op->val64 : nullptr;
  p.cs = s_op ? s_op->col : nullptr;
  p.Ls = s_op ? s_op->L : 0;
  p.ld = h->n_pad;
  p.n = n;
  p.fs = 0.5;  // S from the stored 2S
  p.bp = -1.0;
  const bool rs = s_op ? s_op->is_real != 0 : true;
  for (int k = M - 1; k >= 0; --k) {
    // lam_k = S z_k + f H lam_{k+1} - lam_{k+2},  f = 2 (k >= 1) or 1 (k = 0)
    p.x = k + 1 < M ? Lm + (int64_t)(k + 1) * n : nullptr;
    p.fh = k == 0 ? 0.5 : 1.0;
    p.prev = k + 2 < M ? Lm + (int64_t)(k + 2) * n : nullptr;
    p.z = s_op ? Z + (int64_t)k * n : nullptr;
    p.add = s_op ? nullptr : Z + (int64_t)k * n;
    p.dst = Lm + (int64_t)k * n;
    KPM_TRY(launch_table_step(h->is_real != 0, rs, p, s));
  }
  return KPM_OK;
}

int kpm_ell_slot_sum(kpm_ell* h, int K, const double* coef, const double* A, int64_t lda, const double* B,
                     int64_t ldb, int accumulate, double* out, void* stream) {
  if (!h || !A || !B || !out || K < 1 || lda < h->n || ldb < h->n) return KPM_ERR_INVALID_ARG;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int g = grid_rows(h->n);
  const double2* a = reinterpret_cast<const double2*>(A);
  const double2* b = reinterpret_cast<const double2*>(B);
  double2* o = reinterpret_cast<double2*>(out);
  const int acc = accumulate ? 1 : 0;
  if (h->L <= 4)
    slot_sum_kernel<4><<<g, 256, 0, s>>>(h->col, h->L, h->n_pad, h->n, K, coef, a, lda, b, ldb, acc, o);
  else if (h->L <= 8)
    slot_sum_kernel<8><<<g, 256, 0, s>>>(h->col, h->L, h->n_pad, h->n, K, coef, a, lda, b, ldb, acc, o);
  else if (h->L <= 16)
    slot_sum_kernel<16><<<g, 256, 0, s>>>(h->col, h->L, h->n_pad, h->n, K, coef, a, lda, b, ldb, acc, o);
  else
    return KPM_ERR_UNSUPPORTED;
  return check_cuda(cudaGetLastError());
}

}  // extern "C"
