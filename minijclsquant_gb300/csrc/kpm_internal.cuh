// kpm_internal.cuh -- shared definitions of libkpm (not part of the public ABI).
//
// Device layout of an operator (struct kpm_ell_s):
//   val64 : 2*H values, SoA [slot][n_pad]; double when every value is real,
//           double2 (re, im) otherwise.  Doubling is exact in binary floating
//           point, so T_{m+1} = (2H) T_m - T_{m-1} needs no extra multiply.
//   val32 : the same values as exact float pairs (hi, lo): float2 per real value,
//           float4 per complex value (built on first KPM_C64 use)
//   col   : int32 column indices, SoA [slot][n_pad]
// Rows are padded to a multiple of kRowAlign with value 0 and column 0, so
// every kernel runs without a bounds check in its inner loop.
//
// Vectors inside the library are "site-major": R vectors of one site are
// adjacent ([n_pad][R] complex), so the R threads (or R/2 for complex64) that
// serve one row read one contiguous 16-byte-aligned segment per gathered site.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstddef>
#include <utility>
#include <vector>

#include "../../include/kpm.h"

namespace kpm {

constexpr int kBlock = 256;       // threads per CTA of every streaming kernel
constexpr int kRowAlign = 512;    // n_pad is a multiple of this (and of every staged tile)
constexpr int kMaxGroupR = 8;     // vectors advanced together by one launch
constexpr int kChunk = 128;       // recursion steps whose moment partials are buffered
// Budget of every bounded mbarrier wait: ~1 s at 2 GHz, far beyond any legitimate wait for a
// few kilobytes.
constexpr long long kWaitBudgetCycles = 2000000000LL;

void set_last_cuda_error(cudaError_t e);

// Status of a CUDA runtime result (records it and clears the sticky error state).
inline int check_cuda(cudaError_t e) {
  if (e == cudaSuccess) return KPM_OK;
  set_last_cuda_error(e);
  (void)cudaGetLastError();
  return e == cudaErrorMemoryAllocation ? KPM_ERR_OOM : KPM_ERR_CUDA;
}

#define KPM_CUDA_TRY(expr)                                  \
  do {                                                      \
    cudaError_t kpm_e_ = (expr);                            \
    if (kpm_e_ != cudaSuccess) {                            \
      ::kpm::set_last_cuda_error(kpm_e_);                   \
      return kpm_e_ == cudaErrorMemoryAllocation ? KPM_ERR_OOM : KPM_ERR_CUDA; \
    }                                                       \
  } while (0)

#define KPM_TRY(expr)            \
  do {                           \
    int kpm_s_ = (expr);         \
    if (kpm_s_ != KPM_OK) return kpm_s_; \
  } while (0)

// Grow-only device buffer.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};
int ensure(DevBuf& b, size_t bytes);
void release(DevBuf& b);

struct Workspace {
  DevBuf ta, tb, tc, td;   // recursion vectors
  DevBuf vl, vr;           // packed left vectors for the moments
  DevBuf acc, acc2;        // series accumulators
  DevBuf part;             // per-CTA moment partials [kChunk][sets][grid][R] double2
  DevBuf coef;             // small device staging (coefficients)
  DevBuf ckpt, seg, grad;  // adjoint: checkpoint pairs, recomputed segment, per-slot gradient
  DevBuf red;              // doubling: reduced sets [2][R][K + 1], then the per-vector corrections
  DevBuf vf;               // float-pair left vectors of the FP64 recursion's moment products
  DevBuf gin, gin2, gout;  // graph replays of small recursions: staged inputs and moments
};

// A recorded moment recursion of one vector group (L2-resident operators replay it as one
// CUDA graph launch): its shape and every device pointer it was recorded with.
struct MomentGraph {
  int f32 = 0, Rg = 0, M = 0, sets = 0, has_vl = 0, ffm = 0, kind = 0, U = 0, grid = 0;
  const void* bufs[10] = {};
  cudaGraphExec_t exec = nullptr;
};

// Kernel choice for the recursion step of one (precision, R group, moment sets).
struct StepConfig {
  int kind = 0;  // 0: grid-stride kernel, 1: bulk-copy staged kernel, 2: staged with a producer warp
  int U = 1;     // rows per thread per tile (staged)
  int sb = 1;    // sub-tiles of TILE rows per shared-memory stage (producer-warp kernel, complex128)
  int grid = 0;  // CTAs
  float us = 0;  // measured time of one step launch when tuned
};

}  // namespace kpm

struct kpm_ell_s {
  int64_t n = 0;       // rows (= columns)
  int64_t n_pad = 0;   // padded rows
  int L = 0;           // ELL slots per row
  int is_real = 0;     // values stored real
  int device = 0;
  void* val64 = nullptr;
  void* val32 = nullptr;
  int32_t* col = nullptr;
  int sm_count = 0;
  kpm::Workspace ws;
  // measurement hook state (kpm_ell_profile)
  int prof = 0;
  int64_t prof_launches = 0;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> prof_events;
  // device status word written by kernels whose bounded waits ran out
  int* err_flag = nullptr;
  // tuned step kernels, key = f32 * 1000 + R * 10 + sets
  std::vector<std::pair<int, kpm::StepConfig>> tuned;
  // the forward pass the next kpm_adjoint_backward differentiates
  int adj_R = 0, adj_M = 0, adj_ckpt = 0;
  // H == H^dagger, checked on the device at creation; doubling allowed for DOS moments
  int hermitian = 0;
  int herm_stale = 0;  // values changed since the last check (checked when doubling or a query needs it)
  int doubling = 0;  // requested (KPM_FLAG_DOUBLING / kpm_ell_set_doubling)
  // process-unique id of this handle, and the id of an operator whose ELL column arrays
  // were found equal to this one's (kpm_mu_nm fuses V T_m into the H step then)
  uint64_t id = 0;
  uint64_t same_cols_id = 0;
  // fingerprint of the column structure (sum of (column - row) * (2 slot + 1))
  uint64_t structure = 0;
  // recorded recursions of small operators (kpm_cheb_moments)
  std::vector<kpm::MomentGraph> graphs;
};

namespace kpm {

// Kernel parameter block of the fused step kernel (kpm_cheb.cuh).
struct StepParams {
  const void* val;        // 2H values [L][ld] (T or complex T)
  const int32_t* col;     // [L][ld]
  int64_t ld;             // SoA row stride (= n_pad)
  int L;
  int64_t n_pad;          // rows to process
  const void* tcur;       // gathered vector set      [n_pad][R]
  void* tout;             // NEXT: T_{m-1} in, T_{m+1} out (in place); FIRST/APPLY: output
  const void* t0;         // FIRST: own-row T_0 for mu_0 (== tcur)
  const void* vl;         // left vectors for moment set 1 [n_pad][R]
  const void* vl2;        // left vectors for moment set 2 (or null)
  double2* part;          // partials for this launch: [sets][grid][R] (FIRST: [2 steps][sets][grid][R])
  int64_t part_step_stride;  // elements between consecutive steps' partial blocks
  void* series;           // series accumulator [n_pad][R]
  const double2* coef;    // series coefficients (device)
  int m;                  // recursion index of the vector being produced
  double2 a_half;         // APPLY: a/2 (values are 2H)
  double2 b;              // APPLY: b
  int* err;               // device status word (KPM_ERR_TIMEOUT from a bounded wait)
  int per_tile;           // staged kernel, batched operators: contiguous tile range per CTA, partials per
                          // (CTA, instance) run at part + (seg_base[cta] + run) * R
  const void* tprev;      // grid-stride MODE_NEXT: read T_{m-1} here instead of tout (out of place)
  const int* tile_inst;   // per_tile: instance of every tile
  const int* seg_base;    // per_tile: first partial slot of every CTA
  // Doubling (Hermitian H, DOS moments): the step producing t_{k+1} = T_{k+1} v
  // accumulates two sets instead of <v_l|T_{m+1}>: set 0 <t_{k+1}|t_k> and set 1
  // sum_i (|t_k,i|^2 - hv_i) with hv = |v|^2 / 2, so that mu_{2k+1} = 2 set0 - mu_1
  // and mu_{2k} = 2 set1.  t_k is the own row of tcur.
  int dbl;
  const void* hv;         // dbl: |v|^2 / 2, real, [n_pad][R] (working precision)
  int64_t part_set_stride;  // per_tile with two sets: elements between the sets' slot blocks
  // FP64 recursion with float-float moment products (producer-warp kernel, one moment
  // set): vl holds the float pairs of pack_left_ff, vl64 the same vectors in FP64
  int vl_ff;
  const void* vl64;
  // Budget of the producer-warp kernel's mbarrier waits in SM clock cycles (base_params sets
  // kWaitBudgetCycles, about 1 s).  withhold_first (test hook kpm_ell_test_timeout only): the
  // producer arms the first stage's barrier for its bytes but issues no copy, so the waits on
  // it run out and the kernel takes its timeout path.
  long long wait_budget;
  int withhold_first;
};

// Launch helpers implemented per precision (kpm_cheb_c128.cu, kpm_cheb_c64.cu).
enum Mode { MODE_FIRST = 0, MODE_NEXT = 1, MODE_APPLY = 2 };
enum Epi { EPI_STORE = 1, EPI_MOM1 = 2, EPI_MOM2 = 4, EPI_SERIES = 8, EPI_APPLY_B = 16 };

int launch_step_f64(bool real, int R, int mode, int epi, const StepParams& p, int grid, cudaStream_t s);
int launch_step_f32(bool real, int R, int mode, int epi, const StepParams& p, int grid, cudaStream_t s);
// Bulk-copy staged MODE_NEXT step (kpm_staged.cuh), and how many of its CTAs fit one SM.
int launch_staged_f64(bool real, int R, int U, const StepParams& p, int grid, cudaStream_t s);
int launch_staged_f32(bool real, int R, int U, const StepParams& p, int grid, cudaStream_t s);
int staged_ctas_f64(bool real, int R, int U, int L, int nvec);
int staged_ctas_f32(bool real, int R, int U, int L, int nvec);
// The same step with a producer warp and full/empty stage barriers (kpm_ws.cuh).
int launch_ws_f64(bool real, int R, int U, const StepParams& p, int grid, cudaStream_t s, int sb = 1);
int launch_ws_f32(bool real, int R, int U, const StepParams& p, int grid, cudaStream_t s);
// ff: CTAs of the float-float-products variant (one moment set, FP64 recursion)
int ws_ctas_f64(bool real, int R, int U, int L, int nvec, bool ff = false, int sb = 1);
int ws_ctas_f32(bool real, int R, int U, int L, int nvec);
// Driver helpers (kpm_capi.cu).
int pow2_group(int remaining);
int vpt_for(bool f32, int Rg);
StepParams base_params(kpm_ell_s* h, bool f32);
int launch_step(bool f32, bool real, int R, int mode, int epi, const StepParams& p, int grid, cudaStream_t s);
int launch_next(bool f32, bool real, int R, const StepConfig& cfg, const StepParams& p, cudaStream_t s,
                bool series = false);
int step_config(kpm_ell_s* h, bool f32, int Rg, int sets, cudaStream_t s, StepConfig* out);
// Doubling: whether a DOS moment call on h uses it; |v|^2 / 2 of a packed set; the
// Hermitian check run at creation; the assembly of mu from the reduced sets.
bool use_doubling(const kpm_ell_s* h, int M);
int half_norms(const void* packed, bool f32, int64_t n_pad, int Rg, void* hv, cudaStream_t s);
int check_hermitian(kpm_ell_s* h, cudaStream_t s);
// After new values: drop the complex64 copy (rebuilt on its next use); H == H^dagger
// is checked again now when doubling is on, else on the next query (kpm_capi.cu).
int values_changed(kpm_ell_s* h, cudaStream_t s);
int doubling_corr(const void* packed, const void* hv, bool f32, int64_t n_pad, int Rg, const int64_t* seg_begin,
                  int nseg, double* corr, cudaStream_t s);
int mu1_exact(const kpm_ell_s* h, const void* packed_f32, int Rg, const int64_t* seg_begin, int nseg, double2* out,
              int64_t stride, int64_t row0, DevBuf& scratch, cudaStream_t s);
int assemble_doubled(const double2* red_b, const double2* red_d, const double* corr, int rows, int K, int M,
                     double2* mu, int64_t mu_row_stride, int64_t mu_row0, cudaStream_t s);
int check_dtype(int dtype);
// KPM_C128F: moments of one vector group in float-float arithmetic (kpm_ff.cu).
int moments_group_ff(kpm_ell_s* h, int R, int r0, int Rg, int M, const double* v_r, const double* v_l, double* mu,
                     cudaStream_t s);
// Kubo right rows: T_{m+1} = 2H T_m - T_{m-1} and B_m = V T_m in one pass when V has H's
// columns (kpm_kubo_step.cu); complex64, complex V values (float4 splits), R in {1, 2, 4}.
// launch == false only checks that the form fits (KPM_ERR_UNSUPPORTED otherwise).
int kubo_step(bool real_h, int R, const StepParams& p, const void* vval, void* bout, int sm_count, cudaStream_t s,
              bool launch);
// KPM_C128F: the commutator series and the time-domain Kubo correlator of one vector
// group (kpm_ff.cu); time_sigma_group_ff needs Rg <= 4.
int comm_series_group_ff(kpm_ell_s* h, kpm_ell_s* v, int R, int r0, int Rg, int M, const double* c, const double* x,
                         double* out, cudaStream_t s);
int time_sigma_group_ff(kpm_ell_s* h, kpm_ell_s* v1, kpm_ell_s* v2, int R, int r0, int Rg, const double* c_u, int M2,
                        const double* c_fd, int M, int len_t, const double* v, double* sigma, cudaStream_t s);
// KPM_C128F: out = (sum_{m<M} c_m T_m)^steps v for one vector group (kpm_ff.cu).
int series_group_ff(kpm_ell_s* h, int R, int r0, int Rg, int M, const double* c, int steps, const double* v,
                    double* out, cudaStream_t s);

// Rows per tile of the staged kernel (complex64 packs two vectors per thread).
inline int staged_tile_rows(bool f32, int R, int U) {
  const int vpt = (f32 && R >= 2) ? 2 : 1;
  return (kBlock / (R / vpt)) * U;
}
int grid_for(const kpm_ell_s* h, int R, int vpt);

// Layout helpers (kpm_util.cu).
int pack_vectors(const double* src, int64_t n, int64_t n_pad, int R, int r0, int Rg, bool to_f32,
                 void* dst, cudaStream_t s);
int unpack_vectors(const void* src, bool from_f32, int64_t n, int64_t n_pad, int R, int r0, int Rg,
                   double* dst, cudaStream_t s);
int reduce_partials(const double2* part, int steps, int sets, int grid, int Rg, double* const* outs,
                    int R, int r0, int M, int m0, cudaStream_t s);
// Two [n_pad][Rg] sets of 16-byte entries joined into / split from one [n_pad][2 Rg] set
// (slots 0..Rg-1 from a, Rg..2Rg-1 from b) (kpm_capi.cu).
int join_split(double2* a, double2* b, double2* both, int64_t n_pad, int Rg, bool join, cudaStream_t s);
// Float pairs of the left vectors r0 .. r0 + Rg for the FP64 recursion's float-float moment
// products ([n_pad][Rg] float4; kpm_ff.cu).
int pack_left_ff(const double* v, int64_t n, int64_t n_pad, int R, int r0, int Rg, void* dst, cudaStream_t s);
// FP64 one-set moments form their products in float-float arithmetic (producer-warp
// kernel) unless KPM_MOMENTS_FP64 is set to a nonzero value.
bool ff_moment_products(bool f32, int sets);
// step_config moment-set codes: 1 one set, 2 two sets, 3 doubled, 4 series, and
// kSetsFp64Products: one set whose products stay FP64 (callers that launch the FP64
// moment variant themselves)
constexpr int kSetsFp64Products = 5;
int ensure_f32_values(kpm_ell_s* h, cudaStream_t s);
// Profiling helpers: bracket a step loop with events when h->prof is set.
int prof_begin(kpm_ell_s* h, cudaStream_t s, cudaEvent_t* ev);
int prof_end(kpm_ell_s* h, cudaStream_t s, cudaEvent_t ev, int64_t launches);

}  // namespace kpm
