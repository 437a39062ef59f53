// kpm_util.cu -- layout kernels (ELL repack, vector pack/unpack), the
// deterministic moment reduction and small device-memory helpers.
#include <cstring>

#include "kpm_internal.cuh"

namespace kpm {

static thread_local cudaError_t g_last_cuda = cudaSuccess;
void set_last_cuda_error(cudaError_t e) { g_last_cuda = e; }

int ensure(DevBuf& b, size_t bytes) {
  if (bytes <= b.bytes && b.p) return KPM_OK;
  if (b.p) {
    cudaError_t e = cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
    if (e != cudaSuccess) {
      set_last_cuda_error(e);
      return KPM_ERR_CUDA;
    }
  }
  if (bytes == 0) return KPM_OK;
  cudaError_t e = cudaMalloc(&b.p, bytes);
  if (e != cudaSuccess) {
    b.p = nullptr;
    set_last_cuda_error(e);
    (void)cudaGetLastError();
    return KPM_ERR_OOM;
  }
  b.bytes = bytes;
  return KPM_OK;
}

void release(DevBuf& b) {
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
}

// ---------------------------------------------------------------------------
// Vector packing: user layout [R][n] complex128 -> site-major [n_pad][Rg]
// (complex128 or complex64), rows >= n zero.  One thread per (row, vector).
__global__ void pack_vectors_kernel(const double2* __restrict__ src, int64_t n, int64_t n_pad, int r0,
                                    int Rg, bool to_f32, void* dst) {
  const int64_t total = n_pad * Rg;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = t / Rg;
    const int r = (int)(t % Rg);
    double2 z = make_double2(0.0, 0.0);
    if (row < n) z = src[(int64_t)(r0 + r) * n + row];
    if (to_f32)
      static_cast<float2*>(dst)[t] = make_float2((float)z.x, (float)z.y);
    else
      static_cast<double2*>(dst)[t] = z;
  }
}

__global__ void unpack_vectors_kernel(const void* src, bool from_f32, int64_t n, int r0, int Rg,
                                      double2* __restrict__ dst) {
  const int64_t total = n * Rg;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = t / Rg;
    const int r = (int)(t % Rg);
    double2 z;
    if (from_f32) {
      const float2 f = static_cast<const float2*>(src)[t];
      z = make_double2((double)f.x, (double)f.y);
    } else {
      z = static_cast<const double2*>(src)[t];
    }
    dst[(int64_t)(r0 + r) * n + row] = z;
  }
}

static int launch_grid_for(int64_t total) {
  int64_t g = (total + 255) / 256;
  if (g > 65536) g = 65536;
  if (g < 1) g = 1;
  return (int)g;
}

int pack_vectors(const double* src, int64_t n, int64_t n_pad, int R, int r0, int Rg, bool to_f32, void* dst,
                 cudaStream_t s) {
  (void)R;
  pack_vectors_kernel<<<launch_grid_for(n_pad * Rg), 256, 0, s>>>(reinterpret_cast<const double2*>(src), n,
                                                                  n_pad, r0, Rg, to_f32, dst);
  KPM_CUDA_TRY(cudaGetLastError());
  return KPM_OK;
}

int unpack_vectors(const void* src, bool from_f32, int64_t n, int64_t n_pad, int R, int r0, int Rg, double* dst,
                   cudaStream_t s) {
  (void)R;
  (void)n_pad;
  unpack_vectors_kernel<<<launch_grid_for(n * Rg), 256, 0, s>>>(src, from_f32, n, r0, Rg,
                                                               reinterpret_cast<double2*>(dst));
  KPM_CUDA_TRY(cudaGetLastError());
  return KPM_OK;
}

// ---------------------------------------------------------------------------
// Moment reduction: part[step][set][grid][Rg] -> out[set][(r0 + r) * M + m0 + step].
// One CTA per (r, set, step); fixed-order strided sums and a fixed tree, so the
// result does not depend on scheduling.
__global__ void reduce_partials_kernel(const double2* __restrict__ part, int sets, int grid, int Rg,
                                       double2* out0, double2* out1, int M, int m0, int r0) {
  const int r = blockIdx.x, set = blockIdx.y, step = blockIdx.z;
  const double2* base = part + (((int64_t)step * sets + set) * grid) * Rg + r;
  double sr = 0.0, si = 0.0;
  for (int b = threadIdx.x; b < grid; b += blockDim.x) {
    const double2 v = base[(int64_t)b * Rg];
    sr += v.x;
    si += v.y;
  }
  __shared__ double shr[128], shi[128];
  shr[threadIdx.x] = sr;
  shi[threadIdx.x] = si;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      shr[threadIdx.x] += shr[threadIdx.x + w];
      shi[threadIdx.x] += shi[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double2* out = set == 0 ? out0 : out1;
    out[(int64_t)(r0 + r) * M + m0 + step] = make_double2(shr[0], shi[0]);
  }
}

int reduce_partials(const double2* part, int steps, int sets, int grid, int Rg, double* const* outs, int R, int r0,
                    int M, int m0, cudaStream_t s) {
  (void)R;
  if (steps <= 0) return KPM_OK;
  dim3 g(Rg, sets, steps);
  reduce_partials_kernel<<<g, 128, 0, s>>>(part, sets, grid, Rg, reinterpret_cast<double2*>(outs[0]),
                                           reinterpret_cast<double2*>(sets > 1 ? outs[1] : outs[0]), M, m0, r0);
  KPM_CUDA_TRY(cudaGetLastError());
  return KPM_OK;
}

// ---------------------------------------------------------------------------
// Complex64 form of the operator values: each FP64 value 2H (doubling exact) as an
// exact pair of floats hi = fl32(2H), lo = fl32(2H - hi) -- float2 {hi, lo} per
// real value, float4 {re_hi, im_hi, re_lo, im_lo} per complex value.
__global__ void values_split_kernel(const double* __restrict__ src, int64_t count, bool cplx, void* dst) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < count;
       t += (int64_t)gridDim.x * blockDim.x) {
    if (cplx) {
      const double re = src[2 * t], im = src[2 * t + 1];
      const float rh = (float)re, ih = (float)im;
      static_cast<float4*>(dst)[t] = make_float4(rh, ih, (float)(re - (double)rh), (float)(im - (double)ih));
    } else {
      const double v = src[t];
      const float h = (float)v;
      static_cast<float2*>(dst)[t] = make_float2(h, (float)(v - (double)h));
    }
  }
}

int ensure_f32_values(kpm_ell_s* h, cudaStream_t s) {
  if (h->val32) return KPM_OK;
  const int64_t count = (int64_t)h->L * h->n_pad;  // values
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, count * (h->is_real ? sizeof(float2) : sizeof(float4)));
  if (e != cudaSuccess) {
    set_last_cuda_error(e);
    (void)cudaGetLastError();
    return KPM_ERR_OOM;
  }
  values_split_kernel<<<launch_grid_for(count), 256, 0, s>>>(static_cast<const double*>(h->val64), count,
                                                             h->is_real == 0, p);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    cudaFree(p);
    set_last_cuda_error(e);
    return KPM_ERR_CUDA;
  }
  h->val32 = p;
  return KPM_OK;
}

int grid_for(const kpm_ell_s* h, int R, int vpt) {
  const int tpr = R / vpt;
  const int rpb = kBlock / tpr;
  const int64_t tiles = (h->n_pad + rpb - 1) / rpb;
  const int64_t cap = (int64_t)h->sm_count * 6;
  int64_t g = tiles < cap ? tiles : cap;
  return (int)(g < 1 ? 1 : g);
}

}  // namespace kpm

// ---------------------------------------------------------------------------
// Measurement hooks.
namespace kpm {

int prof_begin(kpm_ell_s* h, cudaStream_t s, cudaEvent_t* ev) {
  *ev = nullptr;
  if (!h->prof) return KPM_OK;
  KPM_CUDA_TRY(cudaEventCreate(ev));
  KPM_CUDA_TRY(cudaEventRecord(*ev, s));
  return KPM_OK;
}

int prof_end(kpm_ell_s* h, cudaStream_t s, cudaEvent_t ev, int64_t launches) {
  if (!h->prof || !ev) return KPM_OK;
  cudaEvent_t e1;
  KPM_CUDA_TRY(cudaEventCreate(&e1));
  KPM_CUDA_TRY(cudaEventRecord(e1, s));
  h->prof_events.emplace_back(ev, e1);
  h->prof_launches += launches;
  return KPM_OK;
}

// Independent FMA chains: 8 per thread, every SM busy; the result is stored
// so nothing is optimised away.
__global__ void fp64_fma_rate_kernel(double* out, int iters, double a, double b) {
  double c0 = threadIdx.x, c1 = c0 + 1, c2 = c0 + 2, c3 = c0 + 3, c4 = c0 + 4, c5 = c0 + 5, c6 = c0 + 6, c7 = c0 + 7;
  for (int i = 0; i < iters; ++i) {
    c0 = fma(c0, a, b); c1 = fma(c1, a, b); c2 = fma(c2, a, b); c3 = fma(c3, a, b);
    c4 = fma(c4, a, b); c5 = fma(c5, a, b); c6 = fma(c6, a, b); c7 = fma(c7, a, b);
  }
  out[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = c0 + c1 + c2 + c3 + c4 + c5 + c6 + c7;
}

}  // namespace kpm

extern "C" int kpm_ell_profile(kpm_ell* h, int enable) {
  if (!h) return KPM_ERR_INVALID_ARG;
  for (auto& pr : h->prof_events) {
    cudaEventDestroy(pr.first);
    cudaEventDestroy(pr.second);
  }
  h->prof_events.clear();
  h->prof_launches = 0;
  h->prof = enable ? 1 : 0;
  return KPM_OK;
}

extern "C" int kpm_ell_profile_read(kpm_ell* h, double* loop_ms, int64_t* step_launches, int64_t* rows_per_launch) {
  if (!h) return KPM_ERR_INVALID_ARG;
  double total = 0.0;
  for (auto& pr : h->prof_events) {
    KPM_CUDA_TRY(cudaEventSynchronize(pr.second));
    float ms = 0.f;
    KPM_CUDA_TRY(cudaEventElapsedTime(&ms, pr.first, pr.second));
    total += ms;
  }
  if (loop_ms) *loop_ms = total;
  if (step_launches) *step_launches = h->prof_launches;
  if (rows_per_launch) *rows_per_launch = h->n;
  return KPM_OK;
}

extern "C" int kpm_measure_fp64_fma_rate(double* fma_per_second, void* stream) {
  if (!fma_per_second) return KPM_ERR_INVALID_ARG;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int dev = 0, sms = 0;
  KPM_CUDA_TRY(cudaGetDevice(&dev));
  KPM_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = sms * 8, threads = 256, iters = 2048;
  kpm::DevBuf out;
  KPM_TRY(kpm::ensure(out, (size_t)blocks * threads * sizeof(double)));
  cudaEvent_t e0, e1;
  KPM_CUDA_TRY(cudaEventCreate(&e0));
  KPM_CUDA_TRY(cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    KPM_CUDA_TRY(cudaEventRecord(e0, s));
    kpm::fp64_fma_rate_kernel<<<blocks, threads, 0, s>>>(static_cast<double*>(out.p), iters, 0.999, 0.001);
    KPM_CUDA_TRY(cudaGetLastError());
    KPM_CUDA_TRY(cudaEventRecord(e1, s));
    KPM_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    KPM_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  kpm::release(out);
  *fma_per_second = (double)blocks * threads * iters * 8.0 / (best * 1e-3);
  return KPM_OK;
}
