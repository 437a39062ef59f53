/*
 * kpm.h -- C ABI of libkpm, the sm_103a Kernel Polynomial Method hot path.
 *
 * The library holds an ELL Hamiltonian on one GPU and runs the fused
 * "ELL SpMV + three-term Chebyshev recursion + moment reduction" on it:
 *
 *     T_0 = v,  T_1 = H v,  T_{m+1} = 2 H T_m - T_{m-1},
 *     mu_m = <v_l | T_m>   (conjugate on the left vector)
 *
 * where H is the already-rescaled operator (spectrum inside [-1, 1]).
 *
 * Conventions
 *  - Every entry point returns an int status (KPM_OK == 0); kpm_strerror()
 *    names it.  The reference-compatible entry points at the end return void,
 *    exactly like the functions they replace; their status is read with
 *    kpm_last_status().
 *  - Complex numbers are interleaved (re, im) doubles: a "c128 array of n"
 *    is 2n doubles.  Sets of R vectors are passed vector-major: [R][n].
 *  - Pointers marked "device" must be CUDA device (or managed) memory; the
 *    caller owns every buffer it passes.  Operators (kpm_ell) own their
 *    device storage and a reusable workspace.
 *  - `stream` is a cudaStream_t (NULL = legacy default stream).  Calls are
 *    stream-ordered; they return once the work is enqueued unless stated.
 *  - One handle may be used by one host thread at a time; distinct handles
 *    are independent.
 */
#ifndef KPM_GB300_H
#define KPM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define KPM_OK 0
#define KPM_ERR_INVALID_ARG 1   /* null pointer, non-positive size, bad flag  */
#define KPM_ERR_SHAPE 2         /* sizes that do not match the operator       */
#define KPM_ERR_DTYPE 3         /* unknown precision selector                 */
#define KPM_ERR_OOM 4           /* device allocation failed                   */
#define KPM_ERR_CUDA 5          /* a CUDA runtime call or launch failed       */
#define KPM_ERR_TIMEOUT 6       /* a bounded device-side wait gave up         */
#define KPM_ERR_INDEX 7         /* an ELL column index is outside [0, n)      */
#define KPM_ERR_UNSUPPORTED 8   /* valid request the library does not serve   */
#define KPM_ERR_NONFINITE 9     /* a moment came out NaN or Inf               */
#define KPM_ERR_TOO_LARGE 10    /* beyond the fixed scratch of kpm_cheb_moments_noalloc */

/* ---- precision selectors ----------------------------------------------- */
#define KPM_C128 0   /* complex128 recursion, FP64 moments (the drop-in form;
                        see kpm_cheb_moments for the arithmetic of the products) */
#define KPM_C64 1    /* complex64 recursion and values, FP64 moment accumulation */
#define KPM_C128F 2  /* complex128 accuracy in float-float arithmetic on the FP32 pipe
                        (kpm_cheb_moments without mu_rr, kpm_cheb_series,
                        kpm_time_evolve, kpm_cheb_commutator_series,
                        kpm_time_sigma, kpm_adjoint_backward_ex; see kpm_cheb_moments) */

/* ---- operator creation flags ------------------------------------------- */
#define KPM_FLAG_DEVICE_PTRS 1u   /* data/indices are device pointers        */
#define KPM_FLAG_SPLIT_DIAG 2u    /* accepted; the diagonal stays an ELL slot  */
#define KPM_FLAG_DOUBLING 4u      /* DOS moments by the doubling identity      */
#define KPM_FLAG_COMPLEX 8u       /* store complex values even when every imaginary
                                     part is zero (an operator whose values will be
                                     made complex later, e.g. kpm_ell_light_update) */

typedef struct kpm_ell_s kpm_ell;

const char* kpm_strerror(int status);
/* Library version as major*10000 + minor*100 + patch. */
int kpm_version(void);

/*
 * Create a device-resident operator from the reference's padded row-major
 * (AoS) ELL arrays: data[i*len_row + j] (c128) and indices[i*len_row + j]
 * (int32), the layout built by jclsquant's data_indices_c
 * (jclsquant/cython_modules/Extra_funs.pyx:81-137) and consumed by
 * aAxby_c (jclsquant/cython_modules/blas_funs.pyx:64-71).  Padding slots
 * (value 0) are kept; column indices are validated (KPM_ERR_INDEX).
 * The values are stored as given (no rescaling): pass H~ = H / a, as the
 * reference passes H_kpm.data to rec_A_tab_gpu (jclsquant/observables_gpu.py:37).
 * When every value has a zero imaginary part the operator stores real values
 * (half the bytes, half the FP64 work); results are unchanged.
 * Replaces the per-call uploads of jclsquant/cuda_cython/cuda/recursions.cu:24-28.
 */
int kpm_ell_create(kpm_ell** out, int64_t n_rows, int len_row, const double* data,
                   const int32_t* indices, unsigned flags, void* stream);
int kpm_ell_destroy(kpm_ell* h);
/* Query: n_rows, len_row, 1 if values are stored real, device bytes held. */
int kpm_ell_info(const kpm_ell* h, int64_t* n_rows, int* len_row, int* is_real,
                 int64_t* device_bytes);
/* Pre-size the workspace for (dtype, R) so later calls allocate nothing, and
 * pick the recursion-step kernel for it (the first moment call would otherwise
 * do this, synchronously). */
int kpm_ell_reserve(kpm_ell* h, int dtype, int R, int M);
/* Synchronise `stream` and return the status a kernel of h recorded on the
 * device (KPM_ERR_TIMEOUT if a bounded wait ran out), then clear it. */
int kpm_ell_check(kpm_ell* h, void* stream);
/* The recursion-step kernel chosen for (dtype, R): kind 0 = grid-stride,
 * 1 = bulk-copy staged, 2 = bulk-copy staged with a producer warp, 3 = the
 * producer-warp kernel with two sub-tiles per shared-memory stage (complex128);
 * rows per thread per tile; CTAs; measured us per step.  A choice is timed once per
 * operator shape and column structure in a process and shared by later handles
 * (KPM_STEP_KERNEL=simple|staged1|staged2|ws1|ws2|ws1s2 forces one and bypasses that).
 * Operators of at most 2^20 / R padded rows (L2-resident recursions, where launch
 * latency sets the pace) replay each recursion of kpm_cheb_moments as one CUDA graph
 * launch, recorded on first use per shape (KPM_NO_GRAPH=1 launches step by step). */
int kpm_ell_step_config(kpm_ell* h, int dtype, int R, int* kind, int* rows_per_thread, int* grid,
                        float* step_us);
/* The same for the series step (kpm_cheb_series, kpm_time_evolve, kpm_time_sigma):
 * kind 0 = grid-stride, 2 = producer warp or 3 = producer warp with two sub-tiles per
 * stage (complex128), timed on the operator at first use. */
int kpm_ell_series_config(kpm_ell* h, int dtype, int R, int* kind, int* rows_per_thread, int* grid,
                          float* step_us);
/* Doubling (opt-in: KPM_FLAG_DOUBLING at creation or kpm_ell_set_doubling).
 * Whether H == H^dagger exactly (entry by entry, duplicate slots summed) is checked on
 * the device: at creation when KPM_FLAG_DOUBLING is given, else when doubling is
 * switched on or kpm_ell_props is first called (and again after new values).  For such an operator with doubling on, moment
 * calls with v_l == NULL and mu_rr == NULL (DOS moments, M >= 4) use
 *   mu_{2k} = 2 sum_i (|t_k,i|^2 - |v_i|^2/2),  mu_{2k+1} = 2 <t_{k+1}|t_k> - mu_1,
 * t_k = T_k(H) v: ceil(M/2) - 1 recursion steps instead of M - 2.  complex128
 * results agree with the direct recursion to ~1e-16 mu_0.  In complex64 every
 * step's FP32 rounding enters all later doubled moments alike (an error coherent
 * across orders, ~1e-8 mu_0), so complex64 DOS work should stay direct.  The
 * reference always runs the M - 2 steps (jclsquant/recurrence_functions.py:18-38).
 * kpm_ell_props reports whether H is Hermitian and whether DOS calls double. */
int kpm_ell_props(const kpm_ell* h, int* hermitian, int* doubling);
int kpm_ell_set_doubling(kpm_ell* h, int on);

/*
 * y <- b*y + a*H x on R vectors ([R][n] c128, device).
 * Replaces ell_matrix.dot (jclsquant/ell_matrix.py:209-211) ->
 * aAxby (jclsquant/cython_modules/blas_funs.pyx:64-71).
 */
int kpm_ell_dot(kpm_ell* h, double a_re, double a_im, double b_re, double b_im,
                const double* x, double* y, int R, void* stream);

/*
 * Chebyshev moments for R vector pairs, m = 0..M-1:
 *   mu[r][m]    = <v_l[r] | T_m(H) v_r[r]>        (v_l == NULL: v_l = v_r)
 *   mu_rr[r][m] = <v_r[r] | T_m(H) v_r[r]>        (optional, may be NULL)
 * v_r, v_l: device [R][n] c128.  mu, mu_rr: device [R][M] c128.
 * dtype KPM_C128 is the drop-in form; KPM_C64 runs the recursion in
 * complex64 and accumulates moments in FP64.
 * Replaces rec_A_tab (jclsquant/recurrence_functions.py:9-40;
 * jclsquant/cuda_cython/cuda/recursions.cu:17-98), rec_A_tab2v
 * (recurrence_functions.py:44-74; recursions.cu:180-263) and
 * rec_A_tab2v_2 (recurrence_functions.py:76-111), for R vectors per call.
 */
int kpm_cheb_moments(kpm_ell* h, int dtype, int R, int M, const double* v_r,
                     const double* v_l, double* mu, double* mu_rr, void* stream);
/* dtype KPM_C128 arithmetic: the recursion is FP64 throughout.  With one moment set
 * (mu_rr NULL, no doubling) on the producer-warp step kernel, the products
 * conj(v_l) T_m are formed in float-float arithmetic: each FP64 element is split exactly
 * into a float pair to 2^-49, products use TwoProduct, and the float-pair sums are
 * folded into FP64 every 128 rows.  That frees the FP64 pipe, the bound of this step
 * on GB300.  An element that is neither zero nor in [2^-50, 2^59) takes the FP64
 * product.  Per order the moments are within about 6e-11 of all-FP64 products,
 * relative to max(|mu_m|, 1e-6 |mu_0|) (measured over 2,048 orders).  Setting
 * KPM_MOMENTS_FP64=1 in the environment keeps every product in FP64. */
/* dtype KPM_C128F: the same moments with every real number carried as a pair of
 * floats (~48 significant bits; exact products and sums), so the recursion runs on
 * the FP32 pipe -- GB300's FP64 rate is 1/64 of its FP32 rate -- with the memory
 * streams of complex128 (16 bytes per complex).  Within 1e-10 per order of the
 * complex128 form.  No counterpart in the reference.  mu_rr must be NULL. */

/*
 * out[r] = sum_{m<M} c[m] T_m(H) v[r]   (c: device [M] c128; v, out: device [R][n] c128;
 * out may alias v).  dtype KPM_C128, KPM_C64 or KPM_C128F (float-float arithmetic,
 * within 1e-12 of KPM_C128).  Replaces rec_A_vec (jclsquant/recurrence_functions.py:114-143)
 * and the device rec_A (jclsquant/cuda_cython/cuda/recursions.cu:267-317).
 */
int kpm_cheb_series(kpm_ell* h, int dtype, int R, int M, const double* c, const double* v,
                    double* out, void* stream);

/*
 * Time evolution by a repeated series: out[r] = P(H)^steps v[r] with
 * P(H) = sum_{m<M} c[m] T_m(H) (c: the time-step moments of exp(-i H dt)),
 * steps >= 0 (0 copies v).  c: device [M] c128; v, out: device [R][n] c128; out
 * may alias v.  The R vectors advance together, one pass over H per order.
 * dtype KPM_C64 carries the vectors in complex64 between steps, KPM_C128F in float
 * pairs (~48 significant bits; the result is within 1e-12 of KPM_C128).
 * Replaces for_time (jclsquant/cuda_cython/cuda/obv.cu:93-122), which advances
 * U and U_c (R = 2) by len_t calls of the device rec_A each.
 */
int kpm_time_evolve(kpm_ell* h, int dtype, int R, int M, const double* c, int steps,
                    const double* v, double* out, void* stream);

/*
 * Commutator series out[r] = sum_m c[m] C_m with C_0 = 0, C_1 = V v,
 * C_m = 2 H C_{m-1} - C_{m-2} + 2 V T_{m-1}.  H and V are separate operators
 * of equal size.  Replaces rec_com_A_vec (jclsquant/recurrence_functions.py:146-196;
 * jclsquant/cuda_cython/cuda/recursions.cu:319-388).
 * dtype KPM_C128 or KPM_C128F (the recursion and the series in float pairs,
 * H and V read as float pairs; the result unpacked to complex128).
 */
int kpm_cheb_commutator_series(kpm_ell* h, kpm_ell* v_op, int dtype, int R, int M,
                               const double* c, const double* v, double* out, void* stream);

/*
 * Table of the commutator series: tab[r][m] = c[m] C_m (C_m of kpm_cheb_commutator_series
 * for vector r; row m = 0 is c[0] C_0 = 0), m < M.  tab: device [R][M][n] c128 (each
 * vector's table is the reference's [M, N] array).  dtype KPM_C128.
 * Replaces rec_com_A_vec_tab (jclsquant/recurrence_functions.py:202-250).
 */
int kpm_cheb_commutator_table(kpm_ell* h, kpm_ell* v_op, int dtype, int R, int M, const double* c,
                              const double* v, double* tab, void* stream);

/*
 * Time-domain Kubo correlator sigma[r][j] = <U_c(t_j) | V1 U(t_j)>, j < len_t,
 * with U(t_0) = v, U_c(t_0) = sum_m c_fd[m] C_m (commutator series with V2),
 * and both advanced per time step by the series with c_u (M2 terms).
 * The caller multiplies by -i as jclsquant/observables_gpu.py does.
 * c_u: device [M2] c128; c_fd: device [M] c128; v: device [R][n]; sigma: device [R][len_t].
 * Replaces for_time_sigma (jclsquant/cuda_cython/cuda/obv.cu:124-176).
 * dtype KPM_C128, or KPM_C128F: U and U_c stay in float pairs on the device for
 * all len_t steps (commutator series, series steps and the V1 products in float
 * pairs); each sigma[r][j] is reduced in FP64.
 */
int kpm_time_sigma(kpm_ell* h, kpm_ell* v1, kpm_ell* v2, int dtype, int R, const double* c_u,
                   int M2, const double* c_fd, int M, int len_t, const double* v,
                   double* sigma, void* stream);

/* ---- values update and reverse mode --------------------------------------
 * No counterpart in the reference (it has no derivatives); they differentiate
 * rec_A_tab (jclsquant/recurrence_functions.py:9-40).
 * kpm_ell_set_values: replace the operator values (same reference AoS layout
 *   and sparsity as at creation; host or device pointer per flags).  A value
 *   with an imaginary part on a real-stored operator is reported by
 *   kpm_ell_check as KPM_ERR_DTYPE.
 * kpm_adjoint_forward: complex128 moments mu[r][m] = <v_r|T_m(H) v_r> (as
 *   kpm_cheb_moments) of a real symmetric H, keeping (t_k, t_{k+1}) every
 *   `ckpt` orders for the backward pass.  R in {1, 2, 4, 8}.
 * kpm_adjoint_backward: for L = sum_r sum_m c[m] Re mu[r][m] (c: device [M]
 *   doubles) writes grad[i*len_row + s] = dL/dH(i, col(i, s)) (device doubles,
 *   reference AoS layout), H the rescaled operator; recomputes each checkpoint
 *   segment and runs the adjoint recursion through it. */
int kpm_ell_set_values(kpm_ell* h, const double* data, unsigned flags, void* stream);
int kpm_adjoint_forward(kpm_ell* h, int R, int M, int ckpt, const double* v, double* mu, void* stream);
int kpm_adjoint_backward(kpm_ell* h, const double* c, double* grad, void* stream);
/* kpm_adjoint_backward with the arithmetic chosen: KPM_C128 (FP64, as above) or
 * KPM_C128F (the adjoint recursion, segment recompute and gradient in float-float
 * arithmetic on the FP32 pipe; checkpoints and the result stay FP64; ~1e-14
 * relative to the FP64 gradient). */
int kpm_adjoint_backward_ex(kpm_ell* h, const double* c, double* grad, int dtype, void* stream);

/* ---- vector tables (reverse mode of the Kubo-Greenwood conductivity) -------
 * No counterpart in the reference.  A table is M rows of n c128 values (row m at
 * tab + 2 m n doubles), one vector, device memory; h is the rescaled H, s_op a second
 * operator of the same size (e.g. the velocity V = -i H o dx of modifier_velocity,
 * jclsquant/modifiers.py:56-79).  Stream-ordered; nothing is allocated.
 * kpm_cheb_table: tab[m] = T_m(H) v, m < M (the recursion of rec_A_tab,
 *   jclsquant/recurrence_functions.py:9-40, with every vector kept); with s_op also
 *   stab[m] = S T_m(H) v from the same gathers (stab must then be given, else NULL).
 *   v may be row 0 of tab; tab and stab may not overlap (KPM_ERR_INVALID_ARG).
 * kpm_cheb_clenshaw_table: the reverse recursion lam_k = S z_k + 2 H lam_{k+1} - lam_{k+2}
 *   (k = M-1 .. 1), lam_0 = S z_0 + H lam_1 - lam_2, lam_M = lam_{M+1} = 0, all rows kept
 *   (S = identity when s_op is NULL; z and lam may not overlap).  lam_0 = sum_k T_k(H) S z_k
 *   (Clenshaw), and for a
 *   functional Re sum_k (S z_k)^H T_k(H) w the rows are its adjoint vectors: the derivative
 *   by the entry (i, j) of H is sum_{k <= M-2} c_k conj(lam_{k+1}[i]) (T_k(H) w)[j], c_0 = 1,
 *   c_k = 2 (kpm_ell_slot_sum).
 * kpm_ell_slot_sum: per stored entry of h (reference AoS layout [n][len_row], c128),
 *   out[i][s] (+)= sum_{k<K} coef[k] conj(A[k][i]) B[k][col(i, s)], rows of A and B lda, ldb
 *   complex numbers apart (>= n); coef device [K] doubles or NULL (all 1); accumulate != 0
 *   adds to out.  len_row <= 16. */
int kpm_cheb_table(kpm_ell* h, kpm_ell* s_op, int M, const double* v, double* tab, double* stab, void* stream);
int kpm_cheb_clenshaw_table(kpm_ell* h, kpm_ell* s_op, int M, const double* z, double* lam, void* stream);
int kpm_ell_slot_sum(kpm_ell* h, int K, const double* coef, const double* A, int64_t lda, const double* B,
                     int64_t ldb, int accumulate, double* out, void* stream);

/* ---- Kubo-Greenwood moment matrix on the tensor cores ---------------------
 * No counterpart in the reference (its conductivity is the time-domain
 * correlator of for_time_sigma); velocity conventions are those of
 * modifier_velocity (jclsquant/modifiers.py:56-79).
 * kpm_mu_nm: mu[n][m] = (1/R) sum_r <v_r | V T_n(H) V T_m(H) | v_r>, n, m < Nm
 *   (Nm <= 256), H and V Hermitian operators of equal size (V a second
 *   operator, e.g. -i H o dx).  Complex64 recursions over groups of up to 4
 *   vectors (the workspace holds 2 x 256 rows of 2 x group x n floats: 34 GB
 *   at n = 2.1M, group 4); the contraction runs on tcgen05 tensor cores (kind::tf32, 3xTF32 split, FP32 accumulation, split-K
 *   reduced in FP64).  v: device [R][n] c128; mu: device [Nm][Nm] c128.
 *   When V holds complex values on H's ELL columns (checked on the device once per
 *   pair of handles), V T_m is formed inside the H recursion step from the same
 *   gathers of T_m (KPM_MU_NM_UNFUSED=1 in the environment keeps them separate).
 * kpm_mu_contract: the contraction alone, mu (+)= scale * sum_k conj(L_n) R_m
 *   for row blocks L, R of 256 complex64 vectors ([256][ld] floats, interleaved
 *   re/im, rows >= Nm ignored), k_floats = 2 * vector length (multiple of 16),
 *   16-byte aligned device pointers; accumulate != 0 adds into mu. */
int kpm_mu_nm(kpm_ell* h, kpm_ell* v_op, int R, int Nm, const double* v, double* mu, void* stream);
int kpm_mu_contract(const float* L, const float* R, int64_t k_floats, int64_t ld, int Nm, double scale,
                    int accumulate, double* mu, void* stream);

/* ---- batched operators ---------------------------------------------------
 * n_inst independent operators of one ELL width, stacked block-diagonally and
 * advanced by one recursion (one launch per step over all instances, the
 * whole recursion replayed as one CUDA graph).  The reference runs one
 * rec_A_tab per instance and vector (jclsquant/recurrence_functions.py:9-40);
 * this batches that loop.
 * kpm_batch_create: data/indices are the instances' reference-layout AoS ELL
 *   arrays concatenated (instance k's rows after instance k-1's), columns local
 *   to each instance; inst_rows[k] rows each; host pointers.  Values as given
 *   (pass each instance already rescaled).
 * kpm_batch_moments: v is device [R][sum_k inst_rows[k]] c128 (instance k at
 *   its row offset in every vector); mu is device [n_inst][R][M] c128 with
 *   mu[k][r][m] = <v_r^(k) | T_m(H_k) v_r^(k)>.  R in {1, 2, 4, 8}.
 *   The first call per (dtype, R, M) records the graph (synchronously).
 */
typedef struct kpm_batch_s kpm_batch;
int kpm_batch_create(kpm_batch** out, int n_inst, const int64_t* inst_rows, int len_row,
                     const double* data, const int32_t* indices, void* stream);
int kpm_batch_destroy(kpm_batch* b);
int kpm_batch_info(const kpm_batch* b, int* n_inst, int64_t* rows_total, int64_t* rows_padded,
                   int* is_real);
int kpm_batch_moments(kpm_batch* b, int dtype, int R, int M, const double* v, double* mu,
                      void* stream);
/* The recursion-step kernel the batched autotuner chose for (dtype, R) (kind
 * as for kpm_ell_step_config), tuning it on `stream` first if no call has yet;
 * rows per thread, CTAs and the measured us of one step over all instances.
 * No counterpart in the reference. */
int kpm_batch_step_config(kpm_batch* b, int dtype, int R, int* kind, int* rows_per_thread, int* grid,
                          float* step_us, void* stream);
/* Doubling for batched operators, as kpm_ell_props / kpm_ell_set_doubling: the
 * stacked operator is Hermitian when every instance is. */
int kpm_batch_props(const kpm_batch* b, int* hermitian, int* doubling);
int kpm_batch_set_doubling(kpm_batch* b, int on);
int kpm_batch_check(kpm_batch* b, void* stream);

/* ---- moments without any device allocation --------------------------------
 * No counterpart in the reference.  For callers that may not allocate device
 * memory: a plugin inside a host application that owns the whole device
 * budget, or code between latency-critical launches where cudaMalloc /
 * cudaFree (which can synchronise the device) are not allowed.  Such callers
 * cannot create a kpm_ell handle, which allocates.
 * mu[m] = <v | T_m(H) v>, m < M, for ONE vector, with H given directly as the
 * caller's device arrays in jclsquant's padded row-major ELL layout
 * (data: n*len_row c128, indices: n*len_row int32, already rescaled).
 * v: device [n] c128; mu: device [M] c128.  Nothing is allocated: the working
 * vectors and moment partials live in one fixed file-scope device array
 * (about 33 MiB), so n <= 1,048,576 sites; larger n returns KPM_ERR_TOO_LARGE.
 * Under lazy module loading (the CUDA default) that array is reserved in a
 * CUDA context when the library's device code is first used there, which for
 * a caller of this entry point alone is its first call: make that call at
 * set-up time (while the device has room for the array) and outside any
 * stream capture, or set CUDA_MODULE_LOADING=EAGER.  The context then holds
 * the array until it is destroyed.  Each call finds the array's address in
 * the context current on the calling thread, so call with the context that
 * should run the work current.  All calls in a context share the array:
 * calls that overlap on the GPU race; serialise them.  The call waits for its
 * stream to finish so it can return KPM_ERR_INDEX when a column index is
 * outside [0, n) (such entries are skipped).
 */
int kpm_cheb_moments_noalloc(const double* data, const int32_t* indices, int len_row, int64_t n,
                             const double* v, int M, double* mu, void* stream);

/* ---- operator construction on the device ---------------------------------
 * kpm_csr_row_max: len_row = max_i (indptr[i+1] - indptr[i]) of a device CSR
 *   (KPM_ERR_SHAPE when indptr decreases).
 * kpm_csr_to_ell: data_indices_c (jclsquant/cython_modules/Extra_funs.pyx:81-137,
 *   called from jclsquant/ell_matrix.py:187-200) on the GPU.  Padded row-major ELL
 *   arrays from device CSR arrays (indptr int64 [n+1], indices int32, data c128):
 *   row i holds its entries in stored order in slots 0..nnz_i-1; padding slots get
 *   value 0, valid 0 and the row's last stored column (its own index for a row
 *   without entries, where the reference reads out of bounds).  dx, dy (c128) and
 *   conj (int32) are companions with the same sparsity, laid out alike; each output
 *   may be NULL.  KPM_ERR_SHAPE if a row is longer than len_row.  Synchronous.
 * kpm_honeycomb_ell: nearest-neighbour graphene on nx x ny primitive cells, the
 *   arrays of the O(N) host builder (site 2 (iy nx + ix) + s; A bonds to B(ix, iy),
 *   B(ix-1, iy), B(ix, iy-1), B to A(ix, iy), A(ix+1, iy), A(ix, iy+1); periodic or
 *   open).  len_row 4: slot 0 = on-site energy onsite[i] (device [n] doubles), then
 *   the bonds; len_row 3: bonds only (onsite unused).  disp: host [3][2], x_j - x_i
 *   of the three A->B bonds.  Outputs (device, [n][len_row]): data c128 (t on bonds),
 *   indices, and optional valid, dx, dy (c128), partner (int64: flat slot of the
 *   reverse bond, -1 for on-site and padding).  Replaces the reference's setup route
 *   lattice_hexagonal + H_graphene (jclsquant/lattice.py:6-47, jclsquant/hams.py:63-168)
 *   for its graphene configurations.
 * kpm_ell_gershgorin_partner: the symmetric Gershgorin bound b (host out) of such
 *   arrays: c_j = diagonal, r_j = sum_i |H_ij| - |c_j| (column sums, each in flat slot
 *   order through partner), b = max(|min(c - r)|, |max(c + r)|) * factor.
 *   Bit-identical to the host builder's bound for real values.  Synchronous.
 * kpm_ell_scale_values: data[k] *= scale (both components), modifier_bounds for
 *   symmetric bounds (jclsquant/modifiers.py:14-36) with scale = 1 / b.
 */
int kpm_csr_row_max(int64_t n, const int64_t* indptr, int* len_row, void* stream);
int kpm_csr_to_ell(int64_t n, int len_row, const int64_t* indptr, const int32_t* indices,
                   const double* data, const double* dx, const double* dy, const int32_t* conj,
                   double* ell_data, int32_t* ell_indices, double* ell_dx, double* ell_dy,
                   int32_t* ell_conj, int32_t* valid, void* stream);
int kpm_honeycomb_ell(int nx, int ny, int periodic, double t, const double* onsite, int len_row,
                      const double* disp, double* data, int32_t* indices, int32_t* valid,
                      double* dx, double* dy, int64_t* partner, void* stream);
int kpm_ell_gershgorin_partner(int64_t n, int len_row, const double* data, const int32_t* indices,
                               const int64_t* partner, double factor, double* bound, void* stream);
int kpm_ell_scale_values(int64_t count, double scale, double* data, void* stream);

/* ---- time-dependent operators of driven systems ---------------------------
 * Complex scalars are passed as host arrays of (re, im) pairs; arrays are device
 * c128 in the reference's padded row-major ELL layout.
 * kpm_light_modifier: the Peierls substitution of light_modifier_cython
 *   (jclsquant/cython_modules/Extra_funs.pyx:236-342):
 *     data_new[i] = a data[i] exp(i A0 (cx dx[i] + cy dy[i]) / ch),
 *   (cx, cy) = (0, sin wt) if eta == 0 (linear) else (cos wt, eta sin wt) (circular),
 *   ch = cosh((t - 2 Tp) / (0.5673 Tp)) if Tp != 0 (pulse), else 1.
 *   params: [6] complex a, A0, t, w, Tp, eta.  data_new may alias data.
 * kpm_ell_light_update: the same H(t) from H0 = data0 written straight into h's stored
 *   values (one pass, no array in between; kpm_ell_set_values semantics afterwards).
 *   h must store complex values: create it with KPM_FLAG_COMPLEX (KPM_ERR_DTYPE otherwise).
 * kpm_phonon_modifier: hopping_pos_phonons_modifier (Extra_funs.pyx:540-560): for every
 *   slot whose column is not its row, dx_new = dx + Aq (ex[row] cos(wq t - q0 Sx[row])
 *   - ex[col] cos(wq t - q0 Sx[col])) / ch, dy_new likewise (ey, q1, Sy), data_new =
 *   data exp(-b (sqrt(|dx_new|^2 + |dy_new|^2) / a0 - 1)), ch = cosh((t - 2 Tp) /
 *   (0.5673 Tp)), Tp = 2 pi / wq; the other slots of the outputs are left as they are.
 *   params: [7] complex a0, b, Aq, wq, t, q0, q1.  e_pol_x, e_pol_y, Sx, Sy: device [n]
 *   c128.  KPM_ERR_INDEX for a column outside [0, n) (that slot is skipped).  Synchronous.
 */
int kpm_light_modifier(int64_t count, const double* params, const double* data, const double* dx,
                       const double* dy, double* data_new, void* stream);
int kpm_ell_light_update(kpm_ell* h, const double* params, const double* data0, const double* dx,
                         const double* dy, void* stream);
int kpm_phonon_modifier(int64_t n, int len_row, const double* params, const double* data,
                        const int32_t* indices, const double* dx, const double* dy,
                        const double* e_pol_x, const double* e_pol_y, const double* Sx,
                        const double* Sy, double* data_new, double* dx_new, double* dy_new,
                        void* stream);

/* ---- reference-compatible host-pointer entry points ---------------------
 * Same names and argument lists as jclsquant/cuda_cython/cuda/obv.h:21-23,27,30,
 * where std::complex<double>* is passed as double* (identical layout).
 * Host buffers in and out; synchronous; the operator is uploaded per call,
 * as in the reference.  Status: kpm_last_status() (per host thread).
 * rec_A_tab and rec_A_tab_2 keep one operator's device arrays and buffers
 * allocated between calls of the same shape on the same device (the values are
 * still uploaded, validated and repacked every call), so a loop over vectors
 * allocates device memory once; a call made while another thread is in one
 * uses buffers of its own.
 * for_time updates U and U_c in place (len_t <= 0 leaves them unchanged, as the
 * reference's loop does).
 */
void rec_A_tab(double* data, int* indices, int len_row, int N, double* A_vec, double* v, int M);
void rec_A_tab_2(double* data, int* indices, int len_row, int N, double* A_vec, double* v_l,
                 double* v_r, int M);
void for_time(double* data, int* indices, int len_row, int N, double* moments_kernel, int len_t,
              double* U, double* U_c, int M);
void for_time_sigma(double* data, double* data2, double* data3, int* indices, int len_row, int N,
                    double* moments_kernel_U, double* moments_kernel_FD, int len_t,
                    double* sigma_vec, double* v, int M, int M2);
int kpm_last_status(void);
/* Frees the device memory rec_A_tab / rec_A_tab_2 keep between calls (no
 * counterpart in the reference, whose wrappers allocate per call). */
int kpm_host_cache_release(void);

/* ---- measurement hooks (no counterpart in the reference) ----------------
 * kpm_ell_profile(h, 1) starts recording CUDA events around every recursion
 * step loop run on h (on the call's stream); kpm_ell_profile_read()
 * synchronises on them and returns the summed loop time, the number of step
 * launches timed and the rows each launch covers.  kpm_ell_profile(h, 0)
 * stops recording and drops what was recorded.
 * kpm_measure_fp64_fma_rate() times a kernel of independent FP64 FMA chains
 * on every SM and returns FMA/s (the FP64 ceiling of the complex128 path). */
/* kpm_ell_test_timeout: a test hook of the bounded device waits (no counterpart in the
 * reference).  Runs one producer-warp recursion step on h (one vector, zeroed workspace
 * vectors) in which the producer arms the first shared-memory stage of every CTA for its
 * bytes but issues none of its copies, with every wait bounded by budget_cycles SM clock
 * cycles (1000 .. 2e9).  No copy is ever in flight for that stage, so the waits on it run
 * out and the kernel takes its timeout path: it records KPM_ERR_TIMEOUT, waits (bounded)
 * for the copies it did issue, and returns.  The call synchronises `stream` and returns
 * what kpm_ell_check reads (KPM_ERR_TIMEOUT, then cleared); h stays usable. */
int kpm_ell_test_timeout(kpm_ell* h, int64_t budget_cycles, void* stream);
int kpm_ell_profile(kpm_ell* h, int enable);
int kpm_ell_profile_read(kpm_ell* h, double* loop_ms, int64_t* step_launches, int64_t* rows_per_launch);
int kpm_measure_fp64_fma_rate(double* fma_per_second, void* stream);
/* kpm_mu_gemm_path: which kernel the last tensor-core contraction (kpm_mu_nm,
 * kpm_mu_contract) ran: bit 0 = operand tiles brought in by the TMA engine
 * (mu_gemm_tma_kernel) rather than loaded by the threads (mu_gemm_kernel); bit 1 = the
 * 64-byte-swizzled shared-memory operand layout rather than the no-swizzle one; -1 =
 * none yet.  KPM_MU_GEMM=legacy|tma|legacy_plain|tma_plain picks one (default: tma_plain,
 * the TMA engine into the no-swizzle layout; the threads' loads when the driver offers no
 * tensor-map encoder).  All four give bit-identical results. */
int kpm_mu_gemm_path(void);

#ifdef __cplusplus
}
#endif

#endif /* KPM_GB300_H */
