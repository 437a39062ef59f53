// kpm_mu_nm.cu -- the Kubo-Greenwood moment matrix on the tensor cores.
//
//   mu_nm = (1/R) sum_r <v_r | V T_n(H) V T_m(H) | v_r>,   n, m < Nm <= 256,
//
// computed as mu_nm = (1/R) sum_r L_n^H R_m with L_n = T_n(H) (V v) and
// R_m = V T_m(H) v (H and V Hermitian).  The recursions run in complex64 with the
// step kernels of this library and store every L_n and R_m as a row of a
// [256][2 n_pad] float matrix (interleaved re, im).  The contraction is one real
// GEMM per half of the n range,
//
//   Re mu[n][m] = sum_k A[n][k] B[m][k],   Im mu[n][m] = sum_k A'[n][k] B[m][k],
//
// with A = L rows, B = R rows and A' the pairwise (-im, re) swap of A, done by
// tcgen05.mma kind::tf32 (M = 128, N = 256, K = 8) with the 3xTF32 split
// x = hi + lo (D += Ahi Bhi + Ahi Blo + Alo Bhi), FP32 accumulation in TMEM
// (Re in columns 0..255, Im in 256..511), split-K over CTAs and an FP64
// reduction of the per-CTA partials.
//
// The reference has no such contraction (its conductivity is the time-domain
// correlator of kpm_time_sigma); the operator conventions are those of
// modifier_velocity (jclsquant/modifiers.py:56-79).
#include <algorithm>
#include <cstring>

#include "kpm_async.cuh"
#include "kpm_internal.cuh"
#include "kpm_tc.cuh"

namespace kpm {

constexpr int kTM = 128;                      // A rows (n) per CTA
constexpr int kTN = 256;                      // B rows (m) = MMA N
constexpr int kKt = 16;                       // tf32 K elements per stage
constexpr int kGemmThreads = 256;
constexpr uint32_t kLBO = 128;                // bytes between K-adjacent core matrices
constexpr uint32_t kSBO = (kKt / 4) * 128;    // bytes between 8-row groups (512)
constexpr uint32_t kTileA = kTM * kKt * 4;    // 8 KB
constexpr uint32_t kTileB = kTN * kKt * 4;    // 16 KB
constexpr uint32_t kStageBytes = 4 * kTileA + 2 * kTileB;  // Ahi Alo A'hi A'lo Bhi Blo = 64 KB
constexpr int kGemmStages = 2;
constexpr uint32_t kGemmSmem = kGemmStages * kStageBytes;  // 128 KB
constexpr uint32_t kTmemCols = 512;

struct GemmParams {
  const float* A;   // [256][lda]
  const float* B;   // [256][lda]
  int64_t lda;      // floats per row
  int64_t K;        // floats of K to contract (multiple of kKt)
  int64_t k_per_cta;
  float* part;      // [KS][256][512]
  int* err;
};

// Byte offset of the 16-byte chunk (row r, k-chunk kc) in a canonical no-swizzle K-major tile.
__device__ __forceinline__ uint32_t chunk_off(int r, int kc) {
  return (uint32_t)(r >> 3) * kSBO + (uint32_t)kc * kLBO + (uint32_t)(r & 7) * 16;
}

__device__ __forceinline__ float4 tf32x4(float4 x) {
  return make_float4(to_tf32(x.x), to_tf32(x.y), to_tf32(x.z), to_tf32(x.w));
}

__global__ void __launch_bounds__(kGemmThreads, 1) mu_gemm_kernel(const GemmParams p) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t bars[kGemmStages];
  __shared__ uint32_t tmem_slot;

  const int n0 = blockIdx.x * kTM;
  const int64_t k_begin = (int64_t)blockIdx.y * p.k_per_cta;
  const int64_t k_end = min(p.K, k_begin + p.k_per_cta);
  const int k_tiles = k_end > k_begin ? (int)((k_end - k_begin) / kKt) : 0;
  float* out = p.part + ((int64_t)blockIdx.y * 256 + n0) * 512;
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;

  if (k_tiles == 0) {  // nothing to contract: a zero partial
    for (int i = tid; i < kTM * 512; i += kGemmThreads) out[(int64_t)(i / 512) * 512 + (i % 512)] = 0.f;
    return;
  }
  if (tid == 0) {
    for (int s = 0; s < kGemmStages; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
  }
  if (warp == 0) {
    tmem_alloc(&tmem_slot, kTmemCols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t smem_base = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
  const uint32_t idesc = idesc_tf32(kTM, kTN);

  // this thread's chunks of a tile: A 2 x 16 B, B 4 x 16 B
  float4 ra[2], rb[4];
  auto load_tile = [&](int t) {
    const int64_t k0 = k_begin + (int64_t)t * kKt;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int c = tid + kGemmThreads * i;
      ra[i] = __ldcs(reinterpret_cast<const float4*>(p.A + (int64_t)(n0 + (c >> 2)) * p.lda + k0) + (c & 3));
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int c = tid + kGemmThreads * i;
      rb[i] = __ldcs(reinterpret_cast<const float4*>(p.B + (int64_t)(c >> 2) * p.lda + k0) + (c & 3));
    }
  };
  load_tile(0);
  bool ok = true;
  for (int t = 0; t < k_tiles; ++t) {
    const int st = t % kGemmStages;
    if (t >= kGemmStages) ok = mbar_wait_bounded(&bars[st], (uint32_t)(((t - kGemmStages) / kGemmStages) & 1));
    if (__syncthreads_or(!ok)) break;
    unsigned char* stage = smem + (size_t)st * kStageBytes;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int c = tid + kGemmThreads * i;
      const uint32_t off = chunk_off(c >> 2, c & 3);
      const float4 x = ra[i];
      const float4 hi = tf32x4(x);
      const float4 lo = tf32x4(make_float4(x.x - hi.x, x.y - hi.y, x.z - hi.z, x.w - hi.w));
      *reinterpret_cast<float4*>(stage + 0 * kTileA + off) = hi;
      *reinterpret_cast<float4*>(stage + 1 * kTileA + off) = lo;
      *reinterpret_cast<float4*>(stage + 2 * kTileA + off) = make_float4(-hi.y, hi.x, -hi.w, hi.z);
      *reinterpret_cast<float4*>(stage + 3 * kTileA + off) = make_float4(-lo.y, lo.x, -lo.w, lo.z);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int c = tid + kGemmThreads * i;
      const uint32_t off = chunk_off(c >> 2, c & 3);
      const float4 x = rb[i];
      const float4 hi = tf32x4(x);
      const float4 lo = tf32x4(make_float4(x.x - hi.x, x.y - hi.y, x.z - hi.z, x.w - hi.w));
      *reinterpret_cast<float4*>(stage + 4 * kTileA + off) = hi;
      *reinterpret_cast<float4*>(stage + 4 * kTileA + kTileB + off) = lo;
    }
    if (t + 1 < k_tiles) load_tile(t + 1);
    fence_proxy_async_shared();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      const uint32_t s0 = smem_base + (uint32_t)st * kStageBytes;
#pragma unroll
      for (int j = 0; j < kKt / 8; ++j) {
        const uint32_t kofs = (uint32_t)j * 2 * kLBO;
        const uint64_t a_hi = smem_desc(s0 + 0 * kTileA + kofs, kLBO, kSBO);
        const uint64_t a_lo = smem_desc(s0 + 1 * kTileA + kofs, kLBO, kSBO);
        const uint64_t ap_hi = smem_desc(s0 + 2 * kTileA + kofs, kLBO, kSBO);
        const uint64_t ap_lo = smem_desc(s0 + 3 * kTileA + kofs, kLBO, kSBO);
        const uint64_t b_hi = smem_desc(s0 + 4 * kTileA + kofs, kLBO, kSBO);
        const uint64_t b_lo = smem_desc(s0 + 4 * kTileA + kTileB + kofs, kLBO, kSBO);
        const bool acc = (t > 0) || (j > 0);
        mma_tf32(tmem + 0, a_hi, b_hi, idesc, acc);
        mma_tf32(tmem + 0, a_hi, b_lo, idesc, true);
        mma_tf32(tmem + 0, a_lo, b_hi, idesc, true);
        mma_tf32(tmem + 256, ap_hi, b_hi, idesc, acc);
        mma_tf32(tmem + 256, ap_hi, b_lo, idesc, true);
        mma_tf32(tmem + 256, ap_lo, b_hi, idesc, true);
      }
      mma_commit(&bars[st]);
    }
  }
  // all MMAs issued so far are tracked by the last commit
  const int last = k_tiles - 1;
  if (ok) ok = mbar_wait_bounded(&bars[last % kGemmStages], (uint32_t)((last / kGemmStages) & 1));
  if (__syncthreads_or(!ok)) {
    if (tid == 0) {
      atomicExch(p.err, KPM_ERR_TIMEOUT);
      // wait (bounded) for the MMAs still in flight before the accumulator is released
      for (int q = max(0, last - kGemmStages + 1); q <= last; ++q)
        (void)mbar_wait_bounded(&bars[q % kGemmStages], (uint32_t)((q / kGemmStages) & 1));
    }
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, kTmemCols);
    return;
  }
  tc_fence_after();
  // epilogue: warp w reads TMEM lanes 32*(w%4).. and the Re (w < 4) or Im (w >= 4) columns
  {
    const int q = warp & 3, half = warp >> 2;
    const int row = 32 * q + lane;
    float* orow = out + (int64_t)row * 512 + half * 256;
    for (int c = 0; c < 256 / 16; ++c) {
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(half * 256 + c * 16), v);
#pragma unroll
      for (int i = 0; i < 16; i += 4)
        *reinterpret_cast<float4*>(orow + c * 16 + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, kTmemCols);
}

// mu[n][m] = (accumulate ? mu : 0) + scale * sum_ks (part re, part im), FP64.
__global__ void mu_reduce_kernel(const float* __restrict__ part, int KS, int Nm, double scale, int accumulate,
                                 double2* __restrict__ mu) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= Nm * Nm) return;
  const int n = idx / Nm, m = idx % Nm;
  double re = 0.0, im = 0.0;
  for (int ks = 0; ks < KS; ++ks) {
    const float* row = part + ((int64_t)ks * 256 + n) * 512;
    re += (double)row[m];
    im += (double)row[256 + m];
  }
  double2 o = make_double2(scale * re, scale * im);
  if (accumulate) {
    o.x += mu[idx].x;
    o.y += mu[idx].y;
  }
  mu[idx] = o;
}

int mu_contract(const float* A, const float* B, int64_t K, int64_t lda, int Nm, double scale, int accumulate,
                double2* mu, float* part, int KS, int* err, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    KPM_CUDA_TRY(cudaFuncSetAttribute(mu_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGemmSmem));
    attr = true;
  }
  GemmParams g;
  g.A = A;
  g.B = B;
  g.lda = lda;
  g.K = K;
  g.k_per_cta = ((K / KS + kKt - 1) / kKt) * kKt;
  if (g.k_per_cta < kKt) g.k_per_cta = kKt;
  g.part = part;
  g.err = err;
  mu_gemm_kernel<<<dim3(2, KS), kGemmThreads, kGemmSmem, s>>>(g);
  KPM_CUDA_TRY(cudaGetLastError());
  mu_reduce_kernel<<<(Nm * Nm + 255) / 256, 256, 0, s>>>(part, KS, Nm, scale, accumulate, mu);
  KPM_CUDA_TRY(cudaGetLastError());
  return KPM_OK;
}

int contract_splits(int64_t K, int sm_count) {
  int64_t ks = std::max<int64_t>(1, sm_count / 2);
  ks = std::min<int64_t>(ks, K / kKt);
  return (int)std::max<int64_t>(1, ks);
}

}  // namespace kpm

using namespace kpm;

extern "C" {

int kpm_mu_contract(const float* L, const float* R, int64_t k_floats, int64_t ld, int Nm, double scale,
                    int accumulate, double* mu, void* stream) {
  if (!L || !R || !mu || Nm < 1 || Nm > 256 || k_floats < kKt || ld < k_floats) return KPM_ERR_INVALID_ARG;
  if (k_floats % kKt != 0 || ld % 4 != 0) return KPM_ERR_SHAPE;
  if ((reinterpret_cast<uintptr_t>(L) | reinterpret_cast<uintptr_t>(R)) & 15) return KPM_ERR_INVALID_ARG;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int dev = 0, sms = 0;
  KPM_CUDA_TRY(cudaGetDevice(&dev));
  KPM_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int KS = contract_splits(k_floats, sms);
  float* part = nullptr;
  int* err = nullptr;
  KPM_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&part), (size_t)KS * 256 * 512 * sizeof(float), s));
  KPM_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&err), sizeof(int), s));
  KPM_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
  int rc = mu_contract(L, R, k_floats, ld, Nm, scale, accumulate, reinterpret_cast<double2*>(mu), part, KS, err, s);
  int herr = 0;
  if (rc == KPM_OK) {
    KPM_CUDA_TRY(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    KPM_CUDA_TRY(cudaStreamSynchronize(s));
  }
  cudaFreeAsync(part, s);
  cudaFreeAsync(err, s);
  return rc != KPM_OK ? rc : herr;
}

int kpm_mu_nm(kpm_ell* h, kpm_ell* v_op, int R, int Nm, const double* v, double* mu, void* stream) {
  if (!h || !v_op || !v || !mu || R < 1 || Nm < 2 || Nm > 256) return KPM_ERR_INVALID_ARG;
  if (v_op->n != h->n) return KPM_ERR_SHAPE;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  KPM_TRY(ensure_f32_values(h, s));
  KPM_TRY(ensure_f32_values(v_op, s));
  Workspace& ws = h->ws;
  const int64_t lda = 2 * h->n_pad;                        // floats per stored vector
  const size_t mat = (size_t)256 * lda * sizeof(float);    // 256 rows, unused rows zero
  const size_t vb = (size_t)h->n_pad * sizeof(float2);
  KPM_TRY(ensure(ws.ckpt, 2 * mat));                        // A = L rows, B = R rows
  KPM_TRY(ensure(ws.ta, vb));
  KPM_TRY(ensure(ws.tb, vb));
  const int KS = contract_splits(lda, h->sm_count);
  KPM_TRY(ensure(ws.part, (size_t)KS * 256 * 512 * sizeof(float)));
  float* A = static_cast<float*>(ws.ckpt.p);
  float* B = A + (size_t)256 * lda;
  if (Nm < 256) KPM_CUDA_TRY(cudaMemsetAsync(ws.ckpt.p, 0, 2 * mat, s));
  const int grid_h = grid_for(h, 1, 1);
  const int grid_v = grid_for(v_op, 1, 1);
  for (int r = 0; r < R; ++r) {
    KPM_TRY(pack_vectors(v, h->n, h->n_pad, R, r, 1, true, ws.ta.p, s));
    // A[0] = V v, A[1] = H A[0], A[m+1] = 2 H A[m] - A[m-1]  (out of place, every row kept)
    StepParams pv = base_params(v_op, true);
    pv.tcur = ws.ta.p;
    pv.tout = A;
    pv.a_half = make_double2(0.5, 0.0);
    KPM_TRY(launch_step(true, v_op->is_real, 1, MODE_APPLY, EPI_STORE, pv, grid_v, s));
    StepParams ph = base_params(h, true);
    ph.tcur = A;
    ph.tout = A + lda;
    KPM_TRY(launch_step(true, h->is_real, 1, MODE_FIRST, EPI_STORE, ph, grid_h, s));
    for (int m = 1; m + 1 < Nm; ++m) {
      ph.tcur = A + (size_t)m * lda;
      ph.tprev = A + (size_t)(m - 1) * lda;
      ph.tout = A + (size_t)(m + 1) * lda;
      KPM_TRY(launch_step(true, h->is_real, 1, MODE_NEXT, EPI_STORE, ph, grid_h, s));
    }
    // T recursion on v (in place), B[m] = V T_m
    void* t_prev = ws.ta.p;  // T_0
    void* t_cur = ws.tb.p;
    pv.tcur = t_prev;
    pv.tout = B;
    KPM_TRY(launch_step(true, v_op->is_real, 1, MODE_APPLY, EPI_STORE, pv, grid_v, s));
    StepParams pt = base_params(h, true);
    pt.tcur = t_prev;
    pt.tout = t_cur;
    KPM_TRY(launch_step(true, h->is_real, 1, MODE_FIRST, EPI_STORE, pt, grid_h, s));
    for (int m = 1; m < Nm; ++m) {
      pv.tcur = t_cur;
      pv.tout = B + (size_t)m * lda;
      KPM_TRY(launch_step(true, v_op->is_real, 1, MODE_APPLY, EPI_STORE, pv, grid_v, s));
      if (m + 1 < Nm) {
        pt.tcur = t_cur;
        pt.tout = t_prev;
        KPM_TRY(launch_step(true, h->is_real, 1, MODE_NEXT, EPI_STORE, pt, grid_h, s));
        std::swap(t_prev, t_cur);
      }
    }
    KPM_TRY(mu_contract(A, B, lda, lda, Nm, 1.0 / R, r > 0, reinterpret_cast<double2*>(mu),
                        static_cast<float*>(ws.part.p), KS, h->err_flag, s));
  }
  return KPM_OK;
}

}  // extern "C"
