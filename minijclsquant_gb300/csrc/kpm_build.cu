// kpm_build.cu -- operator construction on the device.
//
//   kpm_csr_row_max / kpm_csr_to_ell : data_indices_c (jclsquant/cython_modules/
//       Extra_funs.pyx:81-137, called from jclsquant/ell_matrix.py:187-200): the
//       padded row-major ELL arrays from CSR, one thread per output slot.
//   kpm_honeycomb_ell : the nearest-neighbour graphene ELL arrays of the O(N)
//       lattice builder (minijclsquant_gb300/lattice.py, which replaces
//       jclsquant/lattice.py:6-47 + jclsquant/hams.py:63-168), one thread per slot.
//   kpm_ell_gershgorin_partner : that builder's column-sum Gershgorin bound, with
//       each column summed in the flat order numpy's bincount uses (bit-identical
//       for real values).
//   kpm_ell_scale_values : modifier_bounds for symmetric bounds (every entry times 1/a).
//
// All of these are HBM-bound streaming kernels (no reuse): grids of a few waves of
// 256-thread CTAs with grid-stride loops, 64-bit flat indices.
#include <algorithm>
#include <cmath>

#include "kpm_internal.cuh"

using namespace kpm;

namespace {

inline cudaStream_t stream_of(void* s) { return reinterpret_cast<cudaStream_t>(s); }

int stream_grid(int64_t work) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    (void)cudaGetLastError();
    sms = 152;
  }
  const int64_t want = (work + kBlock - 1) / kBlock;
  return (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sms * 8));
}

// Error bits of the build kernels.
constexpr unsigned kBadIndptr = 1u;   // indptr decreasing
constexpr unsigned kRowTooLong = 2u;  // a row longer than len_row

__global__ void csr_row_max_kernel(int64_t n, const int64_t* __restrict__ indptr, int* out, unsigned* flags) {
  int m = 0;
  unsigned f = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t len = indptr[i + 1] - indptr[i];
    if (len < 0) f |= kBadIndptr;
    else m = len > (int64_t)INT32_MAX ? INT32_MAX : max(m, (int)len);
  }
  for (int o = 16; o > 0; o >>= 1) {
    m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    f |= __shfl_xor_sync(0xffffffffu, f, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(out, m);
    if (f) atomicOr(flags, f);
  }
}

// One thread per output slot t = i * L + k: row i's k-th stored entry, or padding
// (value 0, valid 0, column = the row's last stored column; the row's own index
// for a row without entries).
__global__ void csr_to_ell_kernel(int64_t n, int L, const int64_t* __restrict__ indptr,
                                  const int32_t* __restrict__ indices, const double2* __restrict__ data,
                                  const double2* __restrict__ dx, const double2* __restrict__ dy,
                                  const int32_t* __restrict__ conj, double2* ell_data, int32_t* ell_indices,
                                  double2* ell_dx, double2* ell_dy, int32_t* ell_conj, int32_t* valid,
                                  unsigned* flags) {
  const int64_t total = n * (int64_t)L;
  const double2 zero = make_double2(0.0, 0.0);
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / L;
    const int k = (int)(t - i * L);
    const int64_t start = indptr[i];
    const int64_t len = indptr[i + 1] - start;
    if (k == 0 && len > L) atomicOr(flags, kRowTooLong);
    if (k < len) {
      const int64_t e = start + k;
      ell_indices[t] = indices[e];
      ell_data[t] = data[e];
      if (ell_dx) ell_dx[t] = dx[e];
      if (ell_dy) ell_dy[t] = dy[e];
      if (ell_conj) ell_conj[t] = conj[e];
      if (valid) valid[t] = 1;
    } else {
      ell_indices[t] = len > 0 ? indices[start + len - 1] : (int32_t)i;
      ell_data[t] = zero;
      if (ell_dx) ell_dx[t] = zero;
      if (ell_dy) ell_dy[t] = zero;
      if (ell_conj) ell_conj[t] = 0;
      if (valid) valid[t] = 0;
    }
  }
}

// Honeycomb: primitive 2-site cells (A, B); site 2 * (iy * nx + ix) + s.  A bonds to
// B(ix, iy), B(ix-1, iy), B(ix, iy-1); B to A(ix, iy), A(ix+1, iy), A(ix, iy+1).
// Row: slot 0 = on-site (when L == 4), then the three bonds in that order; an absent
// bond (open edge) is padding (value 0, column = the previous slot's column or the
// row itself).  disp: x_j - x_i of the three A->B bonds, (x, y) pairs; B rows use
// the negated table (passed as well, so the host's rounding is kept).
struct HoneyDisp {
  double ax[3], ay[3], bx[3], by[3];
};

// Neighbour k (0..2) of site i: its column, or -1 where an open edge has no bond.
// I is the index type: 32-bit arithmetic when every slot index fits (integer division
// by nx and L is the costliest part of this kernel), 64-bit otherwise.
template <typename I>
__device__ inline I honey_neighbour(I i, int k, int nx, int ny, int periodic) {
  const I cell = i >> 1;
  const int b = (int)(i & 1);
  const int iy = (int)(cell / (I)nx);
  const int ix = (int)(cell - (I)iy * nx);
  const int sgn = b ? 1 : -1;  // B: +1 neighbours, A: -1
  const int xk = k == 1 ? ix + sgn : ix;
  const int yk = k == 2 ? iy + sgn : iy;
  if (!periodic && (xk < 0 || xk >= nx || yk < 0 || yk >= ny)) return (I)-1;
  // a neighbour is at most one cell away: wrap by one period
  const int x = xk < 0 ? xk + nx : (xk >= nx ? xk - nx : xk);
  const int y = yk < 0 ? yk + ny : (yk >= ny ? yk - ny : yk);
  return 2 * ((I)y * nx + x) + (1 - b);
}

// One slot q = i * L + s: its value, column, valid flag, displacements and reverse-bond
// slot.  e is the site's on-site energy (read only for the on-site slot).
template <typename I, int L>
__device__ inline void honey_slot(I q, double e, int nx, int ny, int periodic, double t, const HoneyDisp& d,
                                  double2* data, int32_t* indices, int32_t* valid, double2* dxv, double2* dyv,
                                  int64_t* partner) {
  constexpr int first = L - 3;
  const double2 zero = make_double2(0.0, 0.0);
  const I i = q / (I)L;
  const int s = (int)(q - i * L);
  const int b = (int)(i & 1);
  if (s < first) {  // on-site slot
    data[q] = make_double2(e, 0.0);
    indices[q] = (int32_t)i;
    if (valid) valid[q] = 1;
    if (dxv) dxv[q] = zero;
    if (dyv) dyv[q] = zero;
    if (partner) partner[q] = -1;
    return;
  }
  const int k = s - first;
  const I j = honey_neighbour<I>(i, k, nx, ny, periodic);
  if (j >= 0) {
    data[q] = make_double2(t, 0.0);
    indices[q] = (int32_t)j;
    if (valid) valid[q] = 1;
    if (dxv) dxv[q] = make_double2(b ? d.bx[k] : d.ax[k], 0.0);
    if (dyv) dyv[q] = make_double2(b ? d.by[k] : d.ay[k], 0.0);
    if (partner) partner[q] = (int64_t)j * L + s;
  } else {
    // padding: the column of the last earlier bond of the row, else the row itself
    I prev = i;
    for (int kk = k - 1; kk >= 0; --kk) {
      const I jj = honey_neighbour<I>(i, kk, nx, ny, periodic);
      if (jj >= 0) {
        prev = jj;
        break;
      }
    }
    data[q] = zero;
    indices[q] = (int32_t)prev;
    if (valid) valid[q] = 0;
    if (dxv) dxv[q] = zero;
    if (dyv) dyv[q] = zero;
    if (partner) partner[q] = -1;
  }
}

// One thread per output slot, so consecutive threads write consecutive slots of every
// array.  Each thread takes kHoneyUnroll slots a grid stride apart and issues their
// on-site loads before any store, so the loads' latency overlaps.
constexpr int kHoneyUnroll = 4;

template <typename I, int L>
__global__ void honeycomb_kernel(int nx, int ny, int periodic, double t, const double* __restrict__ eps,
                                 HoneyDisp d, double2* data, int32_t* indices, int32_t* valid, double2* dxv,
                                 double2* dyv, int64_t* partner) {
  const I total = (I)2 * nx * ny * L;
  const I stride = (I)gridDim.x * blockDim.x;
  for (I q0 = (I)blockIdx.x * blockDim.x + threadIdx.x; q0 < total; q0 += kHoneyUnroll * stride) {
    double e[kHoneyUnroll];
#pragma unroll
    for (int u = 0; u < kHoneyUnroll; ++u) {
      const I q = q0 + u * stride;
      e[u] = (L == 4 && q < total) ? __ldg(eps + q / (I)L) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < kHoneyUnroll; ++u) {
      const I q = q0 + u * stride;
      if (q < total) honey_slot<I, L>(q, e[u], nx, ny, periodic, t, d, data, indices, valid, dxv, dyv, partner);
    }
  }
}

__device__ inline double abs_c(double2 z) { return z.y == 0.0 ? fabs(z.x) : hypot(z.x, z.y); }

// Per row j: c = the diagonal (slots whose column is j, in slot order), r = (column
// sum of |H| over column j) - |c|; per CTA min(c - r), max(c + r).  Column j's
// entries are the diagonal slot and the reverse bonds partner[j * L + s]; they are
// summed in increasing flat position (the order of numpy's bincount).  Padding
// entries carry 0 and change no sum.
__global__ void gershgorin_partner_kernel(int64_t n, int L, const double2* __restrict__ data,
                                          const int32_t* __restrict__ indices, const int64_t* __restrict__ partner,
                                          double2* block_out) {
  double lo = INFINITY, hi = -INFINITY;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    int64_t pos[16];
    int np_ = 0;
    double2 diag = make_double2(0.0, 0.0);
    for (int s = 0; s < L && s < 16; ++s) {
      const int64_t p = j * L + s;
      if (indices[p] == (int32_t)j) {
        const double2 v = data[p];
        diag.x += v.x;
        diag.y += v.y;
        if (partner[p] < 0 && (v.x != 0.0 || v.y != 0.0)) pos[np_++] = p;  // the on-site entry
      }
      if (partner[p] >= 0) pos[np_++] = partner[p];
    }
    // insertion sort of at most L positions
    for (int a = 1; a < np_; ++a) {
      const int64_t key = pos[a];
      int b = a - 1;
      while (b >= 0 && pos[b] > key) {
        pos[b + 1] = pos[b];
        --b;
      }
      pos[b + 1] = key;
    }
    double col = 0.0;
    for (int a = 0; a < np_; ++a) col += abs_c(data[pos[a]]);
    const double c = diag.x;
    const double r = col - abs_c(diag);
    lo = fmin(lo, c - r);
    hi = fmax(hi, c + r);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  __shared__ double2 w[kBlock / 32];
  if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = make_double2(lo, hi);
  __syncthreads();
  if (threadIdx.x == 0) {
    double2 acc = w[0];
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
      acc.x = fmin(acc.x, w[k].x);
      acc.y = fmax(acc.y, w[k].y);
    }
    block_out[blockIdx.x] = acc;
  }
}

// One warp: the per-CTA (min, max) pairs folded into one.
__global__ void minmax_finish_kernel(const double2* __restrict__ in, int count, double2* out) {
  double lo = INFINITY, hi = -INFINITY;
  for (int k = threadIdx.x; k < count; k += blockDim.x) {
    lo = fmin(lo, in[k].x);
    hi = fmax(hi, in[k].y);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if (threadIdx.x == 0) *out = make_double2(lo, hi);
}

__global__ void scale_values_kernel(int64_t count, double s, double2* data) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = data[k];
    data[k] = make_double2(v.x * s, v.y * s);
  }
}

int read_flags(DevBuf& fb, cudaStream_t s, unsigned* out) {
  KPM_CUDA_TRY(cudaMemcpyAsync(out, fb.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  KPM_CUDA_TRY(cudaStreamSynchronize(s));
  return KPM_OK;
}

}  // namespace

extern "C" {

int kpm_csr_row_max(int64_t n, const int64_t* indptr, int* len_row, void* stream) {
  if (n < 1 || !indptr || !len_row) return KPM_ERR_INVALID_ARG;
  cudaStream_t s = stream_of(stream);
  DevBuf b;
  KPM_TRY(ensure(b, 2 * sizeof(int)));
  int st = check_cuda(cudaMemsetAsync(b.p, 0, 2 * sizeof(int), s));
  int host[2] = {0, 0};
  if (st == KPM_OK) {
    int* out = static_cast<int*>(b.p);
    csr_row_max_kernel<<<stream_grid(n), kBlock, 0, s>>>(n, indptr, out, reinterpret_cast<unsigned*>(out + 1));
    st = check_cuda(cudaGetLastError());
  }
  if (st == KPM_OK) st = check_cuda(cudaMemcpyAsync(host, b.p, sizeof(host), cudaMemcpyDeviceToHost, s));
  if (st == KPM_OK) st = check_cuda(cudaStreamSynchronize(s));
  release(b);
  if (st != KPM_OK) return st;
  if (host[1] & kBadIndptr) return KPM_ERR_SHAPE;
  *len_row = host[0];
  return KPM_OK;
}

int kpm_csr_to_ell(int64_t n, int len_row, const int64_t* indptr, const int32_t* indices, const double* data,
                   const double* dx, const double* dy, const int32_t* conj, double* ell_data, int32_t* ell_indices,
                   double* ell_dx, double* ell_dy, int32_t* ell_conj, int32_t* valid, void* stream) {
  if (n < 1 || len_row < 1 || !indptr || !indices || !data || !ell_data || !ell_indices) return KPM_ERR_INVALID_ARG;
  if ((ell_dx && !dx) || (ell_dy && !dy) || (ell_conj && !conj)) return KPM_ERR_INVALID_ARG;
  cudaStream_t s = stream_of(stream);
  DevBuf fb;
  KPM_TRY(ensure(fb, sizeof(unsigned)));
  unsigned flags = 0;
  int st = check_cuda(cudaMemsetAsync(fb.p, 0, sizeof(unsigned), s));
  if (st == KPM_OK) {
    csr_to_ell_kernel<<<stream_grid(n * (int64_t)len_row), kBlock, 0, s>>>(
        n, len_row, indptr, indices, reinterpret_cast<const double2*>(data), reinterpret_cast<const double2*>(dx),
        reinterpret_cast<const double2*>(dy), conj, reinterpret_cast<double2*>(ell_data), ell_indices,
        reinterpret_cast<double2*>(ell_dx), reinterpret_cast<double2*>(ell_dy), ell_conj, valid,
        static_cast<unsigned*>(fb.p));
    st = check_cuda(cudaGetLastError());
  }
  if (st == KPM_OK) st = read_flags(fb, s, &flags);
  release(fb);
  if (st != KPM_OK) return st;
  return (flags & kRowTooLong) ? KPM_ERR_SHAPE : KPM_OK;
}

int kpm_honeycomb_ell(int nx, int ny, int periodic, double t, const double* onsite, int len_row,
                      const double* disp, double* data, int32_t* indices, int32_t* valid, double* dx, double* dy,
                      int64_t* partner, void* stream) {
  if (nx < 2 || ny < 2 || !disp || !data || !indices) return KPM_ERR_INVALID_ARG;
  if (len_row != 3 && len_row != 4) return KPM_ERR_INVALID_ARG;
  if (len_row == 4 && !onsite) return KPM_ERR_INVALID_ARG;
  if (2 * (int64_t)nx * ny > (int64_t)INT32_MAX) return KPM_ERR_SHAPE;
  HoneyDisp d;
  for (int k = 0; k < 3; ++k) {
    d.ax[k] = disp[2 * k];
    d.ay[k] = disp[2 * k + 1];
    d.bx[k] = -disp[2 * k];
    d.by[k] = -disp[2 * k + 1];
  }
  cudaStream_t s = stream_of(stream);
  const int64_t n = 2 * (int64_t)nx * ny;
  const int grid = stream_grid(n * len_row);
  // 32-bit slot indices when they cannot overflow (unrolled grid-stride increments included)
  const bool narrow = n * len_row + (int64_t)kHoneyUnroll * grid * kBlock < (int64_t)INT32_MAX;
  double2* dd = reinterpret_cast<double2*>(data);
  double2* dxx = reinterpret_cast<double2*>(dx);
  double2* dyy = reinterpret_cast<double2*>(dy);
  if (narrow && len_row == 4)
    honeycomb_kernel<int32_t, 4><<<grid, kBlock, 0, s>>>(nx, ny, periodic, t, onsite, d, dd, indices, valid, dxx,
                                                         dyy, partner);
  else if (narrow)
    honeycomb_kernel<int32_t, 3><<<grid, kBlock, 0, s>>>(nx, ny, periodic, t, onsite, d, dd, indices, valid, dxx,
                                                         dyy, partner);
  else if (len_row == 4)
    honeycomb_kernel<int64_t, 4><<<grid, kBlock, 0, s>>>(nx, ny, periodic, t, onsite, d, dd, indices, valid, dxx,
                                                         dyy, partner);
  else
    honeycomb_kernel<int64_t, 3><<<grid, kBlock, 0, s>>>(nx, ny, periodic, t, onsite, d, dd, indices, valid, dxx,
                                                         dyy, partner);
  return check_cuda(cudaGetLastError());
}

int kpm_ell_gershgorin_partner(int64_t n, int len_row, const double* data, const int32_t* indices,
                               const int64_t* partner, double factor, double* bound, void* stream) {
  if (n < 1 || len_row < 1 || len_row > 16 || !data || !indices || !partner || !bound) return KPM_ERR_INVALID_ARG;
  cudaStream_t s = stream_of(stream);
  const int grid = stream_grid(n);
  DevBuf b;
  KPM_TRY(ensure(b, (size_t)(grid + 1) * sizeof(double2)));
  double2* blocks = static_cast<double2*>(b.p);
  gershgorin_partner_kernel<<<grid, kBlock, 0, s>>>(n, len_row, reinterpret_cast<const double2*>(data), indices,
                                                     partner, blocks);
  int st = check_cuda(cudaGetLastError());
  double2 mm = make_double2(0.0, 0.0);
  if (st == KPM_OK) {
    minmax_finish_kernel<<<1, 32, 0, s>>>(blocks, grid, blocks + grid);
    st = check_cuda(cudaGetLastError());
  }
  if (st == KPM_OK) st = check_cuda(cudaMemcpyAsync(&mm, blocks + grid, sizeof(double2), cudaMemcpyDeviceToHost, s));
  if (st == KPM_OK) st = check_cuda(cudaStreamSynchronize(s));
  release(b);
  if (st != KPM_OK) return st;
  // b = max(|min(c - r)|, |max(c + r)|) * factor, as the host builder computes it
  *bound = std::max(std::fabs(mm.x), std::fabs(mm.y)) * factor;
  return KPM_OK;
}

int kpm_ell_scale_values(int64_t count, double scale, double* data, void* stream) {
  if (count < 1 || !data) return KPM_ERR_INVALID_ARG;
  cudaStream_t s = stream_of(stream);
  scale_values_kernel<<<stream_grid(count), kBlock, 0, s>>>(count, scale, reinterpret_cast<double2*>(data));
  return check_cuda(cudaGetLastError());
}

}  // extern "C"
