/*
 * kpm_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C (C99 + OpenMP) restatement of jclsquant's CPU hot path: the
 * oracle the tests hold the CUDA kernels to, and the CPU baseline ("port") in
 * the benchmark.  Nothing in the product library links or calls this file.
 *
 * Every function follows one reference routine; the citation is given on
 * each.  The loop structure (per-row accumulation order inside the SpMV,
 * static OpenMP schedule, conjugation on the LEFT vector of every dot
 * product) mirrors the reference exactly; only the order in which OpenMP
 * combines per-thread partial sums differs, which moves results at the
 * 1e-16 relative level.
 *
 * Complex numbers cross the ctypes boundary as interleaved (re, im) doubles;
 * scalars are passed as separate re / im arguments.
 */
#include <complex.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex zc;

static int clamp_threads(int t) { return t < 1 ? 1 : t; }

/* y <- b*y + a * A x, A in padded row-major (AoS) ELL.
 * Follows jclsquant/cython_modules/blas_funs.pyx:64-71 (aAxby_c): per row,
 * y[i] *= b first, then y[i] += a*data[idx]*x[indices[idx]] for j = 0..len_row-1. */
void oracle_aAxby(double a_re, double a_im, double b_re, double b_im,
                  const zc* x, zc* y, const zc* data, const int32_t* indices,
                  int len_row, int n, int threads) {
  const zc a = a_re + a_im * I, b = b_re + b_im * I;
  int i;
#pragma omp parallel for schedule(static) num_threads(clamp_threads(threads))
  for (i = 0; i < n; ++i) {
    zc acc = y[i] * b;
    for (int j = 0; j < len_row; ++j) {
      const int64_t idx = (int64_t)i * len_row + j;
      acc += a * data[idx] * x[indices[idx]];
    }
    y[i] = acc;
  }
}

/* sum_i y[i] * a * conj(x[i]).  Follows blas_funs.pyx:83-88 (vdot_c). */
void oracle_vdot(double a_re, double a_im, const zc* x, const zc* y, int n,
                 int threads, double* out) {
  const zc a = a_re + a_im * I;
  double sr = 0.0, si = 0.0;
  int i;
#pragma omp parallel for schedule(static) reduction(+ : sr, si) num_threads(clamp_threads(threads))
  for (i = 0; i < n; ++i) {
    const zc t = y[i] * a * conj(x[i]);
    sr += creal(t);
    si += cimag(t);
  }
  out[0] = sr;
  out[1] = si;
}

/* sum_i y[i] * a * x[i] (no conjugation).  Follows blas_funs.pyx:97-102 (dot_c). */
void oracle_dot(double a_re, double a_im, const zc* x, const zc* y, int n,
                int threads, double* out) {
  const zc a = a_re + a_im * I;
  double sr = 0.0, si = 0.0;
  int i;
#pragma omp parallel for schedule(static) reduction(+ : sr, si) num_threads(clamp_threads(threads))
  for (i = 0; i < n; ++i) {
    const zc t = y[i] * a * x[i];
    sr += creal(t);
    si += cimag(t);
  }
  out[0] = sr;
  out[1] = si;
}

/* y <- a*x + b*y.  Follows blas_funs.pyx:48-52 (axpy2_c). */
void oracle_axpy2(double a_re, double a_im, double b_re, double b_im,
                  const zc* x, zc* y, int n, int threads) {
  const zc a = a_re + a_im * I, b = b_re + b_im * I;
  int i;
#pragma omp parallel for schedule(static) num_threads(clamp_threads(threads))
  for (i = 0; i < n; ++i) y[i] = a * x[i] + b * y[i];
}

static zc vdot1(const zc* x, const zc* y, int n, int threads) {
  double o[2];
  oracle_vdot(1.0, 0.0, x, y, n, threads, o);
  return o[0] + o[1] * I;
}

/* Chebyshev moments mu_m = <v_l | T_m(A) | v_r>, m = 0..M-1.
 * Follows jclsquant/recurrence_functions.py:44-74 (rec_A_tab2v); with
 * v_l == v_r it is rec_A_tab (recurrence_functions.py:9-40):
 *   T0 = v_r, T1 = A v_r, mu0 = <v_l|v_r>, mu1 = <v_l|T1>,
 *   for m >= 2: T0 <- 2 A T1 - T0 (in place), swap(T0, T1), mu_m = <v_l|T1>.
 * Returns 0, or -1 on bad arguments / allocation failure. */
int oracle_rec_A_tab2v(int M, const zc* data, const int32_t* indices, int len_row,
                       int n, const zc* v_l, const zc* v_r, zc* mu, int threads) {
  if (M < 1 || n < 1 || len_row < 1) return -1;
  zc* T0 = (zc*)malloc(sizeof(zc) * (size_t)n);
  zc* T1 = (zc*)calloc((size_t)n, sizeof(zc));
  if (!T0 || !T1) { free(T0); free(T1); return -1; }
  memcpy(T0, v_r, sizeof(zc) * (size_t)n);
  oracle_aAxby(1.0, 0.0, 0.0, 0.0, v_r, T1, data, indices, len_row, n, threads);
  mu[0] = vdot1(v_l, v_r, n, threads);
  if (M > 1) mu[1] = vdot1(v_l, T1, n, threads);
  for (int m = 2; m < M; ++m) {
    oracle_aAxby(2.0, 0.0, -1.0, 0.0, T1, T0, data, indices, len_row, n, threads);
    zc* t = T0; T0 = T1; T1 = t;
    mu[m] = vdot1(v_l, T1, n, threads);
  }
  free(T0);
  free(T1);
  return 0;
}

int oracle_rec_A_tab(int M, const zc* data, const int32_t* indices, int len_row,
                     int n, const zc* v, zc* mu, int threads) {
  return oracle_rec_A_tab2v(M, data, indices, len_row, n, v, v, mu, threads);
}

/* Two moment sets from one recursion: mu1_m = <v_l|T_m v_r>, mu2_m = <v_r|T_m v_r>.
 * Follows recurrence_functions.py:76-111 (rec_A_tab2v_2). */
int oracle_rec_A_tab2v_2(int M, const zc* data, const int32_t* indices, int len_row,
                         int n, const zc* v_l, const zc* v_r, zc* mu1, zc* mu2,
                         int threads) {
  if (M < 1 || n < 1 || len_row < 1) return -1;
  zc* T0 = (zc*)malloc(sizeof(zc) * (size_t)n);
  zc* T1 = (zc*)calloc((size_t)n, sizeof(zc));
  if (!T0 || !T1) { free(T0); free(T1); return -1; }
  memcpy(T0, v_r, sizeof(zc) * (size_t)n);
  oracle_aAxby(1.0, 0.0, 0.0, 0.0, v_r, T1, data, indices, len_row, n, threads);
  mu1[0] = vdot1(v_l, v_r, n, threads);
  mu2[0] = vdot1(v_r, v_r, n, threads);
  if (M > 1) {
    mu1[1] = vdot1(v_l, T1, n, threads);
    mu2[1] = vdot1(v_r, T1, n, threads);
  }
  for (int m = 2; m < M; ++m) {
    oracle_aAxby(2.0, 0.0, -1.0, 0.0, T1, T0, data, indices, len_row, n, threads);
    zc* t = T0; T0 = T1; T1 = t;
    mu1[m] = vdot1(v_l, T1, n, threads);
    mu2[m] = vdot1(v_r, T1, n, threads);
  }
  free(T0);
  free(T1);
  return 0;
}

/* Chebyshev series applied to a vector: out = sum_m c_m T_m(A) v.
 * Follows recurrence_functions.py:114-143 (rec_A_vec): out = c0 v + c1 T1,
 * then out <- c_m T1 + out after each in-place step (axpy2 with b = 1). */
int oracle_rec_A_vec(int M, const zc* data, const int32_t* indices, int len_row, int n,
                     const zc* c, const zc* v, zc* out, int threads) {
  if (M < 2 || n < 1 || len_row < 1) return -1;
  zc* T0 = (zc*)malloc(sizeof(zc) * (size_t)n);
  zc* T1 = (zc*)calloc((size_t)n, sizeof(zc));
  if (!T0 || !T1) { free(T0); free(T1); return -1; }
  memcpy(T0, v, sizeof(zc) * (size_t)n);
  oracle_aAxby(1.0, 0.0, 0.0, 0.0, v, T1, data, indices, len_row, n, threads);
  for (int i = 0; i < n; ++i) out[i] = c[0] * v[i];
  for (int i = 0; i < n; ++i) out[i] += c[1] * T1[i];
  for (int m = 2; m < M; ++m) {
    oracle_aAxby(2.0, 0.0, -1.0, 0.0, T1, T0, data, indices, len_row, n, threads);
    zc* t = T0; T0 = T1; T1 = t;
    oracle_axpy2(creal(c[m]), cimag(c[m]), 1.0, 0.0, T1, out, n, threads);
  }
  free(T0);
  free(T1);
  return 0;
}

/* Commutator series out = sum_m c_m C_m with C_0 = 0, C_1 = V v,
 * C_m = 2 A C_{m-1} - C_{m-2} + 2 V T_{m-1}; A and V share one ELL pattern.
 * Follows recurrence_functions.py:146-196 (rec_com_A_vec), including its
 * update order: C0 <- 2 A C1 - C0; C0 <- 2 V T1 + C0; swap; then the T step. */
/* out != NULL: the series; tab != NULL: the table tab[m*n + i] = c_m C_m,i of
 * rec_com_A_vec_tab (recurrence_functions.py:202-250), row 0 = c_0 C_0 = 0. */
static int com_recursion(int M, const zc* data_a, const zc* data_v, const int32_t* indices,
                         int len_row, int n, const zc* c, const zc* v, zc* out, zc* tab,
                         int threads) {
  if (M < 2 || n < 1 || len_row < 1) return -1;
  zc* T0 = (zc*)malloc(sizeof(zc) * (size_t)n);
  zc* T1 = (zc*)calloc((size_t)n, sizeof(zc));
  zc* C0 = (zc*)calloc((size_t)n, sizeof(zc));
  zc* C1 = (zc*)calloc((size_t)n, sizeof(zc));
  if (!T0 || !T1 || !C0 || !C1) { free(T0); free(T1); free(C0); free(C1); return -1; }
  memcpy(T0, v, sizeof(zc) * (size_t)n);
  oracle_aAxby(1.0, 0.0, 0.0, 0.0, v, T1, data_a, indices, len_row, n, threads);
  oracle_aAxby(1.0, 0.0, 0.0, 0.0, v, C1, data_v, indices, len_row, n, threads);
  if (out)
    for (int i = 0; i < n; ++i) out[i] = c[1] * C1[i];
  if (tab)
    for (int i = 0; i < n; ++i) {
      tab[i] = c[0] * C0[i];
      tab[(size_t)n + i] = c[1] * C1[i];
    }
  for (int m = 2; m < M; ++m) {
    oracle_aAxby(2.0, 0.0, -1.0, 0.0, C1, C0, data_a, indices, len_row, n, threads);
    oracle_aAxby(2.0, 0.0, 1.0, 0.0, T1, C0, data_v, indices, len_row, n, threads);
    zc* t = C0; C0 = C1; C1 = t;
    oracle_aAxby(2.0, 0.0, -1.0, 0.0, T1, T0, data_a, indices, len_row, n, threads);
    t = T0; T0 = T1; T1 = t;
    if (out) oracle_axpy2(creal(c[m]), cimag(c[m]), 1.0, 0.0, C1, out, n, threads);
    if (tab)
      for (int i = 0; i < n; ++i) tab[(size_t)m * n + i] = c[m] * C1[i];
  }
  free(T0); free(T1); free(C0); free(C1);
  return 0;
}

int oracle_rec_com_A_vec(int M, const zc* data_a, const zc* data_v,
                         const int32_t* indices, int len_row, int n, const zc* c,
                         const zc* v, zc* out, int threads) {
  return com_recursion(M, data_a, data_v, indices, len_row, n, c, v, out, NULL, threads);
}

/* rec_com_A_vec_tab (recurrence_functions.py:202-250): tab is [M][n]. */
int oracle_rec_com_A_vec_tab(int M, const zc* data_a, const zc* data_v,
                             const int32_t* indices, int len_row, int n, const zc* c,
                             const zc* v, zc* tab, int threads) {
  return com_recursion(M, data_a, data_v, indices, len_row, n, c, v, NULL, tab, threads);
}

/* Time-domain Kubo sigma(t_j) = <U_c(t_j) | V1 U(t_j)> (without the final
 * -i factor, which the Python caller applies).  Follows
 * jclsquant/cuda_cython/cuda/obv.cu:124-176 (for_time_sigma): U = v,
 * U_c = rec_com_A_vec(M, H, V2, c_FD, v); sigma_0 = <U_c|V1 U>; then for each
 * later time both U and U_c advance by rec_A_vec(M2, H, c_U, .). */
int oracle_for_time_sigma(const zc* data_h, const zc* data_v1, const zc* data_v2,
                          const int32_t* indices, int len_row, int n, const zc* c_u,
                          const zc* c_fd, int len_t, zc* sigma, const zc* v, int M,
                          int M2, int threads) {
  if (len_t < 1) return -1;
  zc* U = (zc*)malloc(sizeof(zc) * (size_t)n);
  zc* Uc = (zc*)malloc(sizeof(zc) * (size_t)n);
  zc* tmp = (zc*)malloc(sizeof(zc) * (size_t)n);
  zc* aux = (zc*)malloc(sizeof(zc) * (size_t)n);
  if (!U || !Uc || !tmp || !aux) { free(U); free(Uc); free(tmp); free(aux); return -1; }
  memcpy(U, v, sizeof(zc) * (size_t)n);
  int rc = oracle_rec_com_A_vec(M, data_h, data_v2, indices, len_row, n, c_fd, v, Uc, threads);
  for (int j = 0; rc == 0 && j < len_t; ++j) {
    if (j > 0) {
      rc |= oracle_rec_A_vec(M2, data_h, indices, len_row, n, c_u, U, tmp, threads);
      memcpy(U, tmp, sizeof(zc) * (size_t)n);
      rc |= oracle_rec_A_vec(M2, data_h, indices, len_row, n, c_u, Uc, tmp, threads);
      memcpy(Uc, tmp, sizeof(zc) * (size_t)n);
    }
    memset(aux, 0, sizeof(zc) * (size_t)n);
    oracle_aAxby(1.0, 0.0, 0.0, 0.0, U, aux, data_v1, indices, len_row, n, threads);
    sigma[j] = vdot1(Uc, aux, n, threads);
  }
  free(U); free(Uc); free(tmp); free(aux);
  return rc;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* Gradient of L = sum_m c_m Re <v|T_m(A) v> with respect to every ELL slot
 * value of a real symmetric A (no reference counterpart: the reference has no
 * derivatives).  Stores every t_m = T_m(A) v, then runs the adjoint recursion
 *   lambda_m = c_m conj(v) + 2 A lambda_{m+1} - lambda_{m+2},  m = M-1 .. 1,
 * and accumulates grad[i*L + s] = Re[w_m lambda_m[i] t_{m-1}[col(i,s)]] with
 * w_1 = 1, w_m = 2 otherwise.  The forward recursion is the oracle's own
 * (rec_A_tab, recurrence_functions.py:9-40); `data` is complex128 with zero
 * imaginary parts.  Returns 0, or -1 on bad arguments / allocation failure. */
int oracle_adjoint_grad(int M, const zc* data, const int32_t* indices, int len_row, int n, const zc* v,
                        const double* c, double* grad) {
  if (M < 2 || n < 1 || len_row < 1) return -1;
  zc* t = (zc*)calloc((size_t)M * (size_t)n, sizeof(zc));
  zc* la = (zc*)calloc((size_t)n, sizeof(zc));
  zc* lb = (zc*)calloc((size_t)n, sizeof(zc));
  zc* ln = (zc*)calloc((size_t)n, sizeof(zc));
  if (!t || !la || !lb || !ln) { free(t); free(la); free(lb); free(ln); return -1; }
  memcpy(t, v, sizeof(zc) * (size_t)n);
  if (M > 1) oracle_aAxby(1.0, 0.0, 0.0, 0.0, t, t + n, data, indices, len_row, n, 1);
  for (int m = 2; m < M; ++m) {
    zc* out = t + (size_t)m * n;
    memcpy(out, t + (size_t)(m - 2) * n, sizeof(zc) * (size_t)n);
    oracle_aAxby(2.0, 0.0, -1.0, 0.0, t + (size_t)(m - 1) * n, out, data, indices, len_row, n, 1);
  }
  memset(grad, 0, sizeof(double) * (size_t)n * len_row);
  /* la = lambda_{m+1}, lb = lambda_{m+2} */
  for (int m = M - 1; m >= 1; --m) {
    for (int i = 0; i < n; ++i) ln[i] = c[m] * conj(v[i]) - lb[i];
    oracle_aAxby(2.0, 0.0, 1.0, 0.0, la, ln, data, indices, len_row, n, 1);
    const double w = m == 1 ? 1.0 : 2.0;
    const zc* tp = t + (size_t)(m - 1) * n;
    for (int i = 0; i < n; ++i)
      for (int s = 0; s < len_row; ++s) {
        const int64_t q = (int64_t)i * len_row + s;
        grad[q] += w * creal(ln[i] * tp[indices[q]]);
      }
    zc* tmp = lb; lb = la; la = ln; ln = tmp;
  }
  free(t); free(la); free(lb); free(ln);
  return 0;
}
