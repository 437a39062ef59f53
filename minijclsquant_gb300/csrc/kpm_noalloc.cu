// kpm_noalloc.cu -- Chebyshev moments for callers that cannot allocate device memory.
//
// Who needs this: code that runs where another component owns all device
// memory (a plugin inside a host application with a fixed memory budget), or
// between latency-critical launches where cudaMalloc / cudaFree may not be
// called because they can synchronise the whole device.  Such a caller cannot
// create a kpm_ell handle (that allocates the operator copy and a workspace).
//
// kpm_cheb_moments_noalloc reads the operator straight from the caller's
// device arrays in jclsquant's padded row-major ELL layout and keeps its own
// working vectors and moment partials in one file-scope device array of fixed
// size, g_noalloc_scratch (kNoAllocScratchBytes, about 33 MiB).  The call
// allocates nothing: no cudaMalloc, no cudaFree, no allocating library routine.
//
// When the array is reserved: with lazy module loading (CUDA_MODULE_LOADING=LAZY, the
// default since CUDA 12.2) the library's device code, this array included, is loaded
// into a CUDA context on the first use of the library in that context -- for a caller
// that uses only this entry point, its first call there.  That first call can therefore
// fail with KPM_ERR_CUDA when the context has no room left for the array, and it can
// synchronise the device.  Make it at set-up time, while memory is available and
// outside any stream capture, or set CUDA_MODULE_LOADING=EAGER so the array is reserved
// when the context loads the library.  From then on the context holds the array until
// it is destroyed or the process exits.
//
// Address: each call looks up the array's device address in the CUDA context that is
// current on the calling thread (cudaGetSymbolAddress, which after the module load only
// reads a table and allocates nothing).  A __device__ array has a different address in
// every context, so a host application that makes its own driver-API context must have
// that context current when it calls.
//
// Sharing: every call on a device uses the same array and leaves its contents
// behind.  Each call writes every scratch word it later reads (vectors,
// partials, the status word it clears first), so nothing carries over, but
// two calls whose work overlaps on the GPU (different streams, or different
// host threads on one stream order) race on the array and corrupt each other.
// Serialise them.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/kpm.h"

namespace {

constexpr int64_t kNoAllocMaxRows = 1 << 20;  // 1,048,576 sites
constexpr int kNoAllocMaxGrid = 1024;         // CTAs per step launch
constexpr int kNoAllocChunk = 64;             // steps whose partials are buffered
constexpr int kNoAllocBlock = 256;
constexpr size_t kVecBytes = (size_t)kNoAllocMaxRows * 16;
constexpr size_t kPartBytes = (size_t)kNoAllocChunk * kNoAllocMaxGrid * 16;
constexpr size_t kNoAllocScratchBytes = 2 * kVecBytes + kPartBytes + 256;

// Layout: [T_a : kNoAllocMaxRows double2][T_b : same][partials][status int]
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of the scratch array in the calling thread's current CUDA context.
int scratch_for_current_context(char** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p) {
    (void)cudaGetLastError();
    return KPM_ERR_CUDA;
  }
  *out = static_cast<char*>(p);
  return KPM_OK;
}

__global__ void noalloc_start_kernel(const double2* __restrict__ v, int64_t n, double2* t0, int* status) {
  if (blockIdx.x == 0 && threadIdx.x == 0) *status = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    t0[i] = v[i];
}

// One Chebyshev order on one vector: first = T_1 = H T_0 (written to tout);
// otherwise T_{m+1} = 2 H T_m - T_{m-1} in place over tout (= T_{m-1}).
// Partials of <v | T_new> (and of <v | T_0> when first) per CTA, FP64.
__global__ void __launch_bounds__(kNoAllocBlock) noalloc_step_kernel(
    const double2* __restrict__ data, const int32_t* __restrict__ idx, int L, int64_t n,
    const double2* __restrict__ v, const double2* __restrict__ tcur, double2* tout, bool first,
    double2* part_new, double2* part_t0, int* status) {
  double mr = 0.0, mi = 0.0, zr = 0.0, zi = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double sr = 0.0, si = 0.0;
    for (int s = 0; s < L; ++s) {
      const int64_t q = i * L + s;
      const int32_t c = idx[q];
      if (c < 0 || (int64_t)c >= n) {  // out-of-range column: skipped and reported
        atomicExch(status, KPM_ERR_INDEX);
        continue;
      }
      const double2 h = data[q];
      const double2 x = tcur[c];
      sr = fma(h.x, x.x, sr);
      sr = fma(-h.y, x.y, sr);
      si = fma(h.x, x.y, si);
      si = fma(h.y, x.x, si);
    }
    double2 out;
    if (first) {
      out = make_double2(sr, si);
    } else {
      const double2 old = tout[i];
      out = make_double2(fma(2.0, sr, -old.x), fma(2.0, si, -old.y));
    }
    tout[i] = out;
    const double2 l = v[i];
    mr = fma(l.x, out.x, mr);
    mr = fma(l.y, out.y, mr);
    mi = fma(l.x, out.y, mi);
    mi = fma(-l.y, out.x, mi);
    if (first) {
      const double2 t = tcur[i];
      zr = fma(l.x, t.x, zr);
      zr = fma(l.y, t.y, zr);
      zi = fma(l.x, t.y, zi);
      zi = fma(-l.y, t.x, zi);
    }
  }
  __shared__ double sh[4][kNoAllocBlock / 32];
  for (int off = 16; off > 0; off >>= 1) {
    mr += __shfl_xor_sync(0xffffffffu, mr, off);
    mi += __shfl_xor_sync(0xffffffffu, mi, off);
    zr += __shfl_xor_sync(0xffffffffu, zr, off);
    zi += __shfl_xor_sync(0xffffffffu, zi, off);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    sh[0][warp] = mr;
    sh[1][warp] = mi;
    sh[2][warp] = zr;
    sh[3][warp] = zi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0, c = 0.0, d = 0.0;
    for (int w = 0; w < kNoAllocBlock / 32; ++w) {
      a += sh[0][w];
      b += sh[1][w];
      c += sh[2][w];
      d += sh[3][w];
    }
    part_new[blockIdx.x] = make_double2(a, b);
    if (first) part_t0[blockIdx.x] = make_double2(c, d);
  }
}

// mu[m0 + k] = sum over CTAs of part[k][cta], fixed order.
__global__ void noalloc_reduce_kernel(const double2* __restrict__ part, int grid, double2* mu, int m0) {
  const int k = blockIdx.x;
  double sr = 0.0, si = 0.0;
  for (int b = threadIdx.x; b < grid; b += blockDim.x) {
    sr += part[(int64_t)k * grid + b].x;
    si += part[(int64_t)k * grid + b].y;
  }
  __shared__ double shr[128], shi[128];
  shr[threadIdx.x] = sr;
  shi[threadIdx.x] = si;
  __syncthreads();
  for (int w = 64; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      shr[threadIdx.x] += shr[threadIdx.x + w];
      shi[threadIdx.x] += shi[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) mu[m0 + k] = make_double2(shr[0], shi[0]);
}

int launched() {
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? KPM_OK : KPM_ERR_CUDA;
}

}  // namespace

extern "C" int kpm_cheb_moments_noalloc(const double* data, const int32_t* indices, int len_row, int64_t n,
                                        const double* v, int M, double* mu, void* stream) {
  if (!data || !indices || !v || !mu || len_row < 1 || n < 1 || M < 1) return KPM_ERR_INVALID_ARG;
  if (n > kNoAllocMaxRows) return KPM_ERR_TOO_LARGE;
  char* base = nullptr;
  int rc = scratch_for_current_context(&base);
  if (rc != KPM_OK) return rc;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  double2* ta = reinterpret_cast<double2*>(base);
  double2* tb = reinterpret_cast<double2*>(base + kVecBytes);
  double2* part = reinterpret_cast<double2*>(base + 2 * kVecBytes);
  int* status = reinterpret_cast<int*>(base + 2 * kVecBytes + kPartBytes);
  const double2* d2 = reinterpret_cast<const double2*>(data);
  const double2* v2 = reinterpret_cast<const double2*>(v);
  double2* mu2 = reinterpret_cast<double2*>(mu);
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    (void)cudaGetLastError();
    return KPM_ERR_CUDA;
  }
  int64_t g = (n + kNoAllocBlock - 1) / kNoAllocBlock;
  if (g > (int64_t)sms * 4) g = (int64_t)sms * 4;
  if (g > kNoAllocMaxGrid) g = kNoAllocMaxGrid;
  const int grid = g < 1 ? 1 : (int)g;
  noalloc_start_kernel<<<grid, kNoAllocBlock, 0, s>>>(v2, n, ta, status);
  if ((rc = launched()) != KPM_OK) return rc;
  // partial slots: step k of the current chunk at part + k * grid
  noalloc_step_kernel<<<grid, kNoAllocBlock, 0, s>>>(d2, indices, len_row, n, v2, ta, tb, true, part + grid, part,
                                                      status);
  if ((rc = launched()) != KPM_OK) return rc;
  double2* tprev = ta;  // T_{m-2}
  double2* tcur = tb;   // T_{m-1}
  int m0 = 0;
  for (int m = 2; m < M; ++m) {
    if (m - m0 == kNoAllocChunk) {
      noalloc_reduce_kernel<<<kNoAllocChunk, 128, 0, s>>>(part, grid, mu2, m0);
      if ((rc = launched()) != KPM_OK) return rc;
      m0 = m;
    }
    noalloc_step_kernel<<<grid, kNoAllocBlock, 0, s>>>(d2, indices, len_row, n, v2, tcur, tprev, false,
                                                        part + (int64_t)(m - m0) * grid, nullptr, status);
    if ((rc = launched()) != KPM_OK) return rc;
    double2* t = tprev;
    tprev = tcur;
    tcur = t;
  }
  noalloc_reduce_kernel<<<M - m0, 128, 0, s>>>(part, grid, mu2, m0);
  if ((rc = launched()) != KPM_OK) return rc;
  // report out-of-range columns: the call waits for its own stream
  int hstatus = 0;
  if (cudaMemcpyAsync(&hstatus, status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    (void)cudaGetLastError();
    return KPM_ERR_CUDA;
  }
  return hstatus;
}
