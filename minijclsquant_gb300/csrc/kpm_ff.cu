// kpm_ff.cu -- complex128 Chebyshev moments in float-float arithmetic (KPM_C128F).
//
// GB300 issues FP64 fused multiply-adds at 1/64 of its FP32 rate, so the
// complex128 recursion is bound by the FP64 pipe with HBM bandwidth to spare.
// This form keeps complex128 accuracy with FP32 instructions: every real number is
// an unevaluated pair hi + lo of floats (~48 significant bits), products are split
// exactly (TwoProduct through FMA) and sums are exact (TwoSum), so one step
//
//   T_{m+1} = 2H T_m - T_{m-1},   moments <v_l | T_{m+1}>
//
// rounds only at the 2^-48 level.  A complex number is a float4 {re_hi, im_hi,
// re_lo, im_lo}: 16 bytes, the size of a complex128, so the memory streams are
// those of the complex128 kernels.  The operator values are the exact float pairs
// of 2H that the complex64 path uses (hi = fl32(2h), lo = fl32(2h - hi)).
// Moment products are accumulated as float pairs over at most kFlush rows per
// thread and then in FP64.  (Float-float arithmetic: T. J. Dekker, Numer. Math. 18
// (1971) 224; D. E. Knuth, TAOCP vol. 2, 4.2.2.)
//
// Kernels: the first step (T_1 = H T_0, mu_0, mu_1) grid-stride, the later steps
// with the bulk-copy stages and producer warp of the staged step kernels.  Each
// thread serves one complex of one vector (R threads per row).
#include <cstdlib>
#include <string>

#include "kpm_ff.cuh"
#include "kpm_ws.cuh"

namespace kpm {

namespace {

// The series coefficient c_m as a complex float pair {re_hi, im_hi, re_lo, im_lo}.
__device__ __forceinline__ float4 ff_coef(const double2* coef, int m) {
  const double2 c = coef[m];
  const float rh = (float)c.x, ih = (float)c.y;
  return make_float4(rh, ih, (float)(c.x - (double)rh), (float)(c.y - (double)ih));
}

// series tile update o += c x (complex float pairs), normalised
__device__ __forceinline__ void ff_series_add(FF& o, float4 c, const FF& x) {
  ff_mac(o, c, x);
  ff_norm(o.rh, o.rl);
  ff_norm(o.ih, o.il);
}

// Grid-stride step.  FIRST: T_1 = (1/2)(2H) T_0 and the moments of T_0 and T_1,
// partials [2 steps][grid][R].  NEXT (operators too wide for the staged stages):
// T_{m+1} = 2H T_m - T_{m-1} in place and <v_l|T_{m+1}>, partials [grid][R].
// SER (the series of rec_A_vec): no moments; FIRST writes series = c_0 T_0 + c_1 T_1,
// NEXT adds c_m T_{m+1} to it.
template <bool REAL, int R, bool NEXT, bool SER>
__global__ void __launch_bounds__(kBlock) ff_step_kernel(const StepParams p) {
  using MV = typename FFVal<REAL>::type;
  constexpr int RPB = kBlock / R;
  __shared__ double2 red[(kBlock / 32) * R];
  const int sub = threadIdx.x % R, rl = threadIdx.x / R;
  const MV* __restrict__ val = static_cast<const MV*>(p.val);
  const float4* __restrict__ tcur = static_cast<const float4*>(p.tcur);
  const float4* __restrict__ vl = static_cast<const float4*>(p.vl);
  float4* tout = static_cast<float4*>(p.tout);
  float4* series = static_cast<float4*>(p.series);
  double zr[1] = {0.0}, zi[1] = {0.0}, mr[1] = {0.0}, mi[1] = {0.0};
  FFMom z{0.f, 0.f, 0.f, 0.f}, m{0.f, 0.f, 0.f, 0.f};
  int pending = 0;
  float4 c_lo = make_float4(0.f, 0.f, 0.f, 0.f), c_hi = c_lo;
  if (SER) {
    c_hi = ff_coef(p.coef, p.m);
    if (!NEXT) c_lo = ff_coef(p.coef, 0);
  }
  for (int64_t row = (int64_t)blockIdx.x * RPB + rl; row < p.n_pad; row += (int64_t)gridDim.x * RPB) {
    const int64_t vi = row * R + sub;
    FF acc{0.f, 0.f, 0.f, 0.f};
    if (NEXT) {
      const FF o = ff_of(tout[vi]);
      acc = FF{-o.rh, -o.ih, -o.rl, -o.il};
    }
    for (int s = 0; s < p.L; ++s) {
      const int32_t c = __ldcs(p.col + (int64_t)s * p.ld + row);
      const MV h = __ldcs(val + (int64_t)s * p.ld + row);
      ff_mac(acc, h, ff_of(__ldg(tcur + (int64_t)c * R + sub)));
    }
    ff_norm(acc.rh, acc.rl);
    ff_norm(acc.ih, acc.il);
    if (!NEXT) acc = FF{0.5f * acc.rh, 0.5f * acc.ih, 0.5f * acc.rl, 0.5f * acc.il};  // exact
    tout[vi] = ff_raw(acc);
    if (SER) {
      FF o{0.f, 0.f, 0.f, 0.f};
      if (NEXT) o = ff_of(series[vi]);
      else ff_series_add(o, c_lo, ff_of(__ldg(tcur + vi)));
      ff_series_add(o, c_hi, acc);
      series[vi] = ff_raw(o);
      continue;
    }
    const FF l = ff_of(__ldg(vl + vi));
    if (!NEXT) ff_cdot(z, l, ff_of(__ldg(tcur + vi)));
    ff_cdot(m, l, acc);
    if (++pending == kFfFlush) {
      pending = 0;
      ff_fold(zr[0], zi[0], z);
      ff_fold(mr[0], mi[0], m);
    }
  }
  if (SER) return;
  ff_fold(zr[0], zi[0], z);
  ff_fold(mr[0], mi[0], m);
  if (NEXT) {
    block_reduce_store<R, 1>(mr, mi, p.part + (int64_t)blockIdx.x * R, red);
  } else {
    block_reduce_store<R, 1>(zr, zi, p.part + (int64_t)blockIdx.x * R, red);
    block_reduce_store<R, 1>(mr, mi, p.part + p.part_step_stride + (int64_t)blockIdx.x * R, red);
  }
}

// T_{m+1} = 2H T_m - T_{m-1} (in place over T_{m-1}) and <v_l|T_{m+1}> per CTA, with
// the staged tiles, producer warp and full/empty barriers of cheb_next_ws_kernel.
// SER: no moments; the producer stages the series tile in the left-vector slot and the
// compute warps write series + c_m T_{m+1}.
template <bool REAL, int R, int U, bool SER>
__global__ void __launch_bounds__(kWsThreads, (U == 1 ? 3 : 1)) ff_next_kernel(const StepParams p) {
  using MV = typename FFVal<REAL>::type;
  constexpr int RPB = kBlock / R;
  constexpr int TILE = RPB * U;
  constexpr int kWarps = kBlock / 32;

  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[kWsStages];
  __shared__ __align__(8) uint64_t empty[kWsStages];
  __shared__ double2 red[kWarps * R];

  const int L = p.L;
  const uint32_t col_b = (uint32_t)align16((size_t)L * TILE * 4);
  const uint32_t val_b = (uint32_t)align16((size_t)L * TILE * sizeof(MV));
  const uint32_t vec_b = (uint32_t)(TILE * R * sizeof(float4));
  const uint32_t stage_b = col_b + val_b + 2 * vec_b;
  const int ntiles = (int)(p.n_pad / TILE);
  const int my_count = ((int)blockIdx.x < ntiles) ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  auto tile_of = [&](int k) -> int64_t { return (int64_t)blockIdx.x + (int64_t)k * gridDim.x; };

  if (threadIdx.x == 0) {
#pragma unroll
    for (int s = 0; s < kWsStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kWarps);
    }
    fence_mbar_init();
  }
  __syncthreads();

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == kWarps) {  // producer
    if (lane == 0 && my_count > 0) {
      TileCopy tc;
      const uint64_t pol = l2_evict_first_policy();
      tc.col = p.col;
      tc.val = static_cast<const unsigned char*>(p.val);
      tc.old = static_cast<const unsigned char*>(p.tout);
      tc.vl = static_cast<const unsigned char*>(SER ? p.series : p.vl);
      tc.vl2 = nullptr;
      tc.cur = nullptr;  // an L2 prefetch of T_m's rows measured slower here (1.07 -> 1.12 ms at 2048^2, R = 8)
      tc.ld = p.ld;
      tc.L = L;
      tc.col_slab = TILE * 4;
      tc.val_slab = (uint32_t)(TILE * sizeof(MV));
      tc.vec_slab = vec_b;
      tc.vl_slab = vec_b;
      tc.col_b = col_b;
      tc.val_b = val_b;
      tc.tx_bytes = (uint32_t)L * TILE * 4 + (uint32_t)L * TILE * (uint32_t)sizeof(MV) + 2 * vec_b;
      int issued = 0;
      for (int k = 0; k < my_count; ++k) {
        const int st = k % kWsStages;
        if (k >= kWsStages && !mbar_wait_bounded(&empty[st], (uint32_t)(((k / kWsStages) - 1) & 1))) {
          atomicExch(p.err, KPM_ERR_TIMEOUT);
          break;
        }
        fence_proxy_async_shared();
        issue_tile(tc, smem + st * stage_b, &full[st], tile_of(k) * TILE, R * (int)sizeof(float4), pol);
        issued = k + 1;
      }
      for (int q = issued > kWsStages ? issued - kWsStages : 0; q < issued; ++q)
        (void)mbar_wait_bounded(&full[q % kWsStages], (uint32_t)((q / kWsStages) & 1));
    }
    return;
  }

  const float4* __restrict__ tcur = static_cast<const float4*>(p.tcur);
  float4* tout = static_cast<float4*>(p.tout);
  float4* series = static_cast<float4*>(p.series);
  const float4 cm = SER ? ff_coef(p.coef, p.m) : make_float4(0.f, 0.f, 0.f, 0.f);
  const int sub = threadIdx.x % R, rl = threadIdx.x / R;
  double mr[1] = {0.0}, mi[1] = {0.0};
  FFMom mom{0.f, 0.f, 0.f, 0.f};
  int pending = 0;
  bool dead = false;
  for (int k = 0; k < my_count; ++k) {
    const int st = k % kWsStages;
    bool ok = !dead && mbar_wait_bounded(&full[st], (uint32_t)((k / kWsStages) & 1));
    ok = __all_sync(0xffffffffu, ok);
    if (!ok && !dead) {
      if (lane == 0) atomicExch(p.err, KPM_ERR_TIMEOUT);
      dead = true;
    }
    if (!ok) continue;
    const unsigned char* base = smem + st * stage_b;
    const int32_t* scol = reinterpret_cast<const int32_t*>(base);
    const MV* sval = reinterpret_cast<const MV*>(base + col_b);
    const float4* sold = reinterpret_cast<const float4*>(base + col_b + val_b);
    const float4* svl = reinterpret_cast<const float4*>(base + col_b + val_b + vec_b);
    const int64_t row0 = tile_of(k) * TILE;
    // even slots into acc, odd slots into acc2: two independent chains per component
    FF acc[U], acc2[U], l[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const FF o = ff_of(sold[(u * RPB + rl) * R + sub]);
      acc[u] = FF{-o.rh, -o.ih, -o.rl, -o.il};
      acc2[u] = FF{0.f, 0.f, 0.f, 0.f};
    }
    for (int s = 0; s < L; s += 4) {
      int c[U][4];
      MV h[U][4];
#pragma unroll
      for (int u = 0; u < U; ++u)
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (s + j < L) {
            c[u][j] = scol[(s + j) * TILE + u * RPB + rl];
            h[u][j] = sval[(s + j) * TILE + u * RPB + rl];
          }
      float4 x[U][4];
#pragma unroll
      for (int u = 0; u < U; ++u)
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (s + j < L) x[u][j] = __ldg(tcur + (int64_t)c[u][j] * R + sub);
#pragma unroll
      for (int u = 0; u < U; ++u)
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (s + j < L) ff_mac((j & 1) ? acc2[u] : acc[u], h[u][j], ff_of(x[u][j]));
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      ff_add(acc[u].rh, acc[u].rl, acc2[u].rh, acc2[u].rl);
      ff_add(acc[u].ih, acc[u].il, acc2[u].ih, acc2[u].il);
      ff_norm(acc[u].rh, acc[u].rl);
      ff_norm(acc[u].ih, acc[u].il);
      l[u] = ff_of(svl[(u * RPB + rl) * R + sub]);
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[st]);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      tout[(row0 + u * RPB + rl) * R + sub] = ff_raw(acc[u]);
      if (SER) {
        ff_series_add(l[u], cm, acc[u]);
        series[(row0 + u * RPB + rl) * R + sub] = ff_raw(l[u]);
        continue;
      }
      ff_cdot(mom, l[u], acc[u]);
      if (++pending == kFfFlush) {
        pending = 0;
        ff_fold(mr[0], mi[0], mom);
      }
    }
  }
  if (SER) return;
  ff_fold(mr[0], mi[0], mom);
  block_reduce_store<R, 1>(mr, mi, p.part + (int64_t)blockIdx.x * R, red, true);
}

// complex128 [R][n] (vector-major) -> float pairs [n_pad][Rg] for vectors r0 .. r0 + Rg
__global__ void ff_pack_kernel(const double2* __restrict__ src, int64_t n, int64_t n_pad, int R, int r0, int Rg,
                               float4* __restrict__ dst) {
  const int64_t total = n_pad * Rg;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = t / Rg;
    const int r = (int)(t % Rg);
    double2 z = make_double2(0.0, 0.0);
    if (row < n) z = src[(int64_t)(r0 + r) * n + row];
    const float xh = (float)z.x, yh = (float)z.y;
    dst[t] = make_float4(xh, yh, (float)(z.x - (double)xh), (float)(z.y - (double)yh));
  }
}

// float pairs [n_pad][Rg] -> complex128 [R][n] for vectors r0 .. r0 + Rg (hi + lo in FP64)
__global__ void ff_unpack_kernel(const float4* __restrict__ src, int64_t n, int Rg, int r0, double2* __restrict__ dst) {
  const int64_t total = n * Rg;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(t / n);
    const int64_t row = t - (int64_t)r * n;
    const float4 q = src[row * Rg + r];
    dst[(int64_t)(r0 + r) * n + row] = make_double2((double)q.x + (double)q.z, (double)q.y + (double)q.w);
  }
}

template <bool REAL, int R, int U, bool SER>
bool ff_smem_attr(size_t smem) {
  static size_t configured = 0;
  if (smem <= configured) return true;
  if (cudaFuncSetAttribute(ff_next_kernel<REAL, R, U, SER>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  configured = smem;
  return true;
}

template <bool REAL, int R, int U>
size_t ff_stage_bytes(int L) {
  constexpr int TILE = (kBlock / R) * U;
  return align16((size_t)L * TILE * 4) + align16((size_t)L * TILE * sizeof(typename FFVal<REAL>::type)) +
         2 * (size_t)TILE * R * sizeof(float4);
}

// One launch: kind -1 the first step, 0 a grid-stride later step, 1 / 2 a staged
// later step with U = kind rows per thread.  A series step (p.series set) runs the
// SER instantiations.
template <bool REAL, int R, int U, bool SER>
int ff_launch_staged(const StepParams& p, int grid, cudaStream_t s) {
  const size_t smem = kWsStages * ff_stage_bytes<REAL, R, U>(p.L);
  if (!ff_smem_attr<REAL, R, U, SER>(smem)) return KPM_ERR_UNSUPPORTED;
  ff_next_kernel<REAL, R, U, SER><<<grid, kWsThreads, smem, s>>>(p);
  return check_cuda(cudaGetLastError());
}

template <bool REAL, int R, bool SER>
int ff_launch_ser(int kind, const StepParams& p, int grid, cudaStream_t s) {
  if (kind < 0)
    ff_step_kernel<REAL, R, false, SER><<<grid, kBlock, 0, s>>>(p);
  else if (kind == 0)
    ff_step_kernel<REAL, R, true, SER><<<grid, kBlock, 0, s>>>(p);
  else
    return kind == 2 ? ff_launch_staged<REAL, R, 2, SER>(p, grid, s) : ff_launch_staged<REAL, R, 1, SER>(p, grid, s);
  return check_cuda(cudaGetLastError());
}

template <bool REAL, int R>
int ff_launch(int kind, const StepParams& p, int grid, cudaStream_t s) {
  return p.series ? ff_launch_ser<REAL, R, true>(kind, p, grid, s) : ff_launch_ser<REAL, R, false>(kind, p, grid, s);
}

template <bool REAL, int R, int U>
int ff_ctas(int L) {
  const size_t smem = kWsStages * ff_stage_bytes<REAL, R, U>(L);
  if (smem > 200 * 1024 || !ff_smem_attr<REAL, R, U, false>(smem)) return 0;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ff_next_kernel<REAL, R, U, false>, kWsThreads, smem) !=
      cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return n;
}

int ff_dispatch(bool real, int R, int kind, const StepParams& p, int grid, cudaStream_t s) {
#define KPM_FF(RR) \
  return real ? ff_launch<true, RR>(kind, p, grid, s) : ff_launch<false, RR>(kind, p, grid, s)
  switch (R) {
    case 1: KPM_FF(1);
    case 2: KPM_FF(2);
    case 4: KPM_FF(4);
    case 8: KPM_FF(8);
    default: return KPM_ERR_UNSUPPORTED;
  }
#undef KPM_FF
}

int ff_occupancy(bool real, int R, int U, int L) {
#define KPM_FO(RR) \
  return U == 2 ? (real ? ff_ctas<true, RR, 2>(L) : ff_ctas<false, RR, 2>(L)) \
                : (real ? ff_ctas<true, RR, 1>(L) : ff_ctas<false, RR, 1>(L))
  switch (R) {
    case 1: KPM_FO(1);
    case 2: KPM_FO(2);
    case 4: KPM_FO(4);
    case 8: KPM_FO(8);
    default: return 0;
  }
#undef KPM_FO
}

// The later-step kernel for (operator, R, series step or moment step): the grid-stride
// kernel or the staged kernel with 1 or 2 rows per thread, timed on the operator (a few
// launches on zeroed vectors) and kept in the handle's tuned list (key 2000 + 10 R, + 1
// for series steps).  KPM_STEP_KERNEL=simple|ws1|ws2 forces one.  Timing clears ws.ta,
// ws.tb and ws.vl: callers tune before they fill those.
int ff_config(kpm_ell_s* h, int Rg, bool series, cudaStream_t s, StepConfig* out) {
  const int key = 2000 + Rg * 10 + (series ? 1 : 0);
  for (auto& kv : h->tuned)
    if (kv.first == key) {
      *out = kv.second;
      return KPM_OK;
    }
  const char* force = getenv("KPM_STEP_KERNEL");
  const std::string f = force ? force : "";
  std::vector<StepConfig> cands;
  if (f.empty() || f == "simple") {
    StepConfig c0;
    c0.kind = 0;
    c0.grid = grid_for(h, Rg, 1);
    cands.push_back(c0);
  }
  for (int U = 1; U <= 2; ++U) {
    if (!f.empty() && f != std::string("ws") + (U == 1 ? "1" : "2")) continue;
    const int occ = ff_occupancy(h->is_real != 0, Rg, U, h->L);
    if (occ <= 0) continue;
    const int64_t ntiles = h->n_pad / ((kBlock / Rg) * U);
    StepConfig c;
    c.kind = 2;
    c.U = U;
    c.grid = (int)std::max<int64_t>(1, std::min<int64_t>(ntiles, (int64_t)occ * h->sm_count));
    cands.push_back(c);
  }
  if (cands.empty()) {  // a forced form that cannot serve this operator
    StepConfig c0;
    c0.kind = 0;
    c0.grid = grid_for(h, Rg, 1);
    cands.push_back(c0);
  }
  if (cands.size() > 1) {
    int max_grid = 0;
    for (auto& c : cands) max_grid = std::max(max_grid, c.grid);
    const size_t vb = (size_t)h->n_pad * Rg * sizeof(float4);
    Workspace& ws = h->ws;
    KPM_TRY(ensure(ws.ta, vb));
    KPM_TRY(ensure(ws.tb, vb));
    KPM_TRY(ensure(ws.vl, vb));
    KPM_TRY(ensure(ws.part, (size_t)max_grid * Rg * sizeof(double2)));
    KPM_CUDA_TRY(cudaMemsetAsync(ws.ta.p, 0, vb, s));
    KPM_CUDA_TRY(cudaMemsetAsync(ws.tb.p, 0, vb, s));
    KPM_CUDA_TRY(cudaMemsetAsync(ws.vl.p, 0, vb, s));
    KPM_CUDA_TRY(cudaMemsetAsync(ws.part.p, 0, sizeof(double2), s));
    StepParams p = base_params(h, true);
    p.tcur = ws.ta.p;
    p.tout = ws.tb.p;
    p.part = static_cast<double2*>(ws.part.p);
    if (series) {  // series into ws.vl with a zero coefficient
      p.series = ws.vl.p;
      p.coef = static_cast<const double2*>(ws.part.p);
      p.m = 0;
    } else {
      p.vl = ws.vl.p;
    }
    cudaEvent_t e0, e1;
    KPM_CUDA_TRY(cudaEventCreate(&e0));
    KPM_CUDA_TRY(cudaEventCreate(&e1));
    for (auto& c : cands) {
      const int kind = c.kind == 0 ? 0 : c.U;
      KPM_TRY(ff_dispatch(h->is_real != 0, Rg, kind, p, c.grid, s));
      KPM_CUDA_TRY(cudaEventRecord(e0, s));
      for (int r = 0; r < 3; ++r) KPM_TRY(ff_dispatch(h->is_real != 0, Rg, kind, p, c.grid, s));
      KPM_CUDA_TRY(cudaEventRecord(e1, s));
      KPM_CUDA_TRY(cudaEventSynchronize(e1));
      float ms = 0.f;
      KPM_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
      c.us = 1e3f * ms / 3;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  StepConfig best = cands[0];
  for (auto& c : cands)
    if (c.us < best.us) best = c;
  h->tuned.emplace_back(key, best);
  *out = best;
  return KPM_OK;
}

int ff_pack(const double* v, int64_t n, int64_t n_pad, int R, int r0, int Rg, void* dst, cudaStream_t s) {
  const int64_t total = n_pad * Rg;
  const int pg = (int)std::min<int64_t>((total + 255) / 256, 65536);
  ff_pack_kernel<<<pg, 256, 0, s>>>(reinterpret_cast<const double2*>(v), n, n_pad, R, r0, Rg,
                                    static_cast<float4*>(dst));
  return check_cuda(cudaGetLastError());
}

// sum_{m<M} c_m T_m x for one packed float-pair set x (ws.ta / ws.tb carry the recursion)
int ff_series_packed(kpm_ell_s* h, int Rg, int M, const StepConfig& cfg, const double2* coef, const void* x,
                     void* result, cudaStream_t s) {
  const size_t vb = (size_t)h->n_pad * Rg * sizeof(float4);
  Workspace& ws = h->ws;
  KPM_TRY(ensure(ws.ta, vb));
  KPM_TRY(ensure(ws.tb, vb));
  KPM_CUDA_TRY(cudaMemcpyAsync(ws.ta.p, x, vb, cudaMemcpyDeviceToDevice, s));
  StepParams p = base_params(h, true);
  p.series = result;
  p.coef = coef;
  p.tcur = ws.ta.p;
  p.tout = ws.tb.p;
  p.m = 1;
  KPM_TRY(ff_dispatch(h->is_real != 0, Rg, -1, p, grid_for(h, Rg, 1), s));
  void* tprev = ws.ta.p;
  void* tcur = ws.tb.p;
  cudaEvent_t ev = nullptr;
  if (M > 2) KPM_TRY(prof_begin(h, s, &ev));
  for (int m = 2; m < M; ++m) {
    p.tcur = tcur;
    p.tout = tprev;
    p.m = m;
    KPM_TRY(ff_dispatch(h->is_real != 0, Rg, cfg.kind == 0 ? 0 : cfg.U, p, cfg.grid, s));
    std::swap(tprev, tcur);
  }
  if (M > 2) KPM_TRY(prof_end(h, s, ev, M - 2));
  return KPM_OK;
}

// ---- commutator series and time-domain Kubo in float-float arithmetic ----------------
struct CommFFParams {
  const void* val_h;
  const int32_t* col_h;
  const void* val_v;
  const int32_t* col_v;
  int64_t ld;
  int Lh, Lv;
  int64_t n_pad;
  const float4* tcur;  // T_{m-1}            [n_pad][R]
  float4* tout;        // T_{m-2} -> T_m
  const float4* ccur;  // C_{m-1}
  float4* cout;        // C_{m-2} -> C_m (FIRST: C_1)
  float4* acc;         // series accumulator
  const double2* coef;
  int m;
};

// One order of rec_com_A_vec (jclsquant/recurrence_functions.py:146-196):
//   C_m = 2H C_{m-1} - C_{m-2} + 2V T_{m-1},  T_m = 2H T_{m-1} - T_{m-2},  acc += c_m C_m,
// at m = 1: T_1 = H v, C_1 = V v, acc = c_1 C_1 -- the step of kpm_comm.cu in float pairs
// (values: the exact float pairs of 2H and 2V).
template <bool RH, bool RV, int R, bool FIRST>
__global__ void __launch_bounds__(kBlock) ff_comm_kernel(const CommFFParams p) {
  using MVH = typename FFVal<RH>::type;
  using MVV = typename FFVal<RV>::type;
  constexpr int RPB = kBlock / R;
  const int sub = threadIdx.x % R, rl = threadIdx.x / R;
  const MVH* __restrict__ vh = static_cast<const MVH*>(p.val_h);
  const MVV* __restrict__ vv = static_cast<const MVV*>(p.val_v);
  const float4 cm = ff_coef(p.coef, p.m);
  for (int64_t row = (int64_t)blockIdx.x * RPB + rl; row < p.n_pad; row += (int64_t)gridDim.x * RPB) {
    const int64_t vi = row * R + sub;
    FF t{0.f, 0.f, 0.f, 0.f}, c{0.f, 0.f, 0.f, 0.f};
    if (!FIRST) {
      const FF to = ff_of(p.tout[vi]), co = ff_of(p.cout[vi]);
      t = FF{-to.rh, -to.ih, -to.rl, -to.il};
      c = FF{-co.rh, -co.ih, -co.rl, -co.il};
    }
    for (int s = 0; s < p.Lh; ++s) {
      const int32_t j = __ldcs(p.col_h + (int64_t)s * p.ld + row);
      const MVH hv = __ldcs(vh + (int64_t)s * p.ld + row);
      ff_mac(t, hv, ff_of(__ldg(p.tcur + (int64_t)j * R + sub)));
      if (!FIRST) ff_mac(c, hv, ff_of(__ldg(p.ccur + (int64_t)j * R + sub)));
    }
    for (int s = 0; s < p.Lv; ++s) {
      const int32_t j = __ldcs(p.col_v + (int64_t)s * p.ld + row);
      const MVV w = __ldcs(vv + (int64_t)s * p.ld + row);
      ff_mac(c, w, ff_of(__ldg(p.tcur + (int64_t)j * R + sub)));
    }
    ff_norm(t.rh, t.rl);
    ff_norm(t.ih, t.il);
    ff_norm(c.rh, c.rl);
    ff_norm(c.ih, c.il);
    if (FIRST) {  // the values are doubled: halve (exact)
      t = FF{0.5f * t.rh, 0.5f * t.ih, 0.5f * t.rl, 0.5f * t.il};
      c = FF{0.5f * c.rh, 0.5f * c.ih, 0.5f * c.rl, 0.5f * c.il};
    }
    p.tout[vi] = ff_raw(t);
    p.cout[vi] = ff_raw(c);
    FF a{0.f, 0.f, 0.f, 0.f};
    if (!FIRST) a = ff_of(p.acc[vi]);
    ff_series_add(a, cm, c);
    p.acc[vi] = ff_raw(a);
  }
}

template <bool RH, bool RV, int R>
int ff_comm_r(bool first, const CommFFParams& p, int grid, cudaStream_t s) {
  if (first)
    ff_comm_kernel<RH, RV, R, true><<<grid, kBlock, 0, s>>>(p);
  else
    ff_comm_kernel<RH, RV, R, false><<<grid, kBlock, 0, s>>>(p);
  return check_cuda(cudaGetLastError());
}

template <bool RH, bool RV>
int ff_comm_hv(int R, bool first, const CommFFParams& p, int grid, cudaStream_t s) {
  switch (R) {
    case 1: return ff_comm_r<RH, RV, 1>(first, p, grid, s);
    case 2: return ff_comm_r<RH, RV, 2>(first, p, grid, s);
    case 4: return ff_comm_r<RH, RV, 4>(first, p, grid, s);
    case 8: return ff_comm_r<RH, RV, 8>(first, p, grid, s);
    default: return KPM_ERR_UNSUPPORTED;
  }
}

int ff_comm_launch(bool rh, bool rv, int R, bool first, const CommFFParams& p, int grid, cudaStream_t s) {
  if (rh && rv) return ff_comm_hv<true, true>(R, first, p, grid, s);
  if (rh) return ff_comm_hv<true, false>(R, first, p, grid, s);
  if (rv) return ff_comm_hv<false, true>(R, first, p, grid, s);
  return ff_comm_hv<false, false>(R, first, p, grid, s);
}

// Commutator series of one packed float-pair set x into `result` (float pairs); the
// recursion uses ws.ta / ws.tc (T) and ws.td / ws.acc2 (C) of h.
int ff_comm_series_packed(kpm_ell_s* h, kpm_ell_s* v, int Rg, int M, const double2* coef, const float4* x,
                          float4* result, cudaStream_t s) {
  const size_t vb = (size_t)h->n_pad * Rg * sizeof(float4);
  Workspace& ws = h->ws;
  KPM_TRY(ensure(ws.ta, vb));
  KPM_TRY(ensure(ws.tc, vb));
  KPM_TRY(ensure(ws.td, vb));
  KPM_TRY(ensure(ws.acc2, vb));
  float4* t_a = static_cast<float4*>(ws.ta.p);
  float4* t_b = static_cast<float4*>(ws.tc.p);
  float4* c_a = static_cast<float4*>(ws.td.p);
  float4* c_b = static_cast<float4*>(ws.acc2.p);
  KPM_CUDA_TRY(cudaMemcpyAsync(t_a, x, vb, cudaMemcpyDeviceToDevice, s));
  KPM_CUDA_TRY(cudaMemsetAsync(c_a, 0, vb, s));  // C_0 = [V, T_0] = 0: read as C_{m-2} at m = 2
  const int grid = grid_for(h, Rg, 1);
  CommFFParams p;
  p.val_h = h->val32;
  p.col_h = h->col;
  p.val_v = v->val32;
  p.col_v = v->col;
  p.ld = h->n_pad;
  p.Lh = h->L;
  p.Lv = v->L;
  p.n_pad = h->n_pad;
  p.coef = coef;
  p.acc = result;
  p.tcur = t_a;  // m = 1: T_1 = H v, C_1 = V v, acc = c_1 C_1
  p.tout = t_b;
  p.ccur = nullptr;
  p.cout = c_b;
  p.m = 1;
  KPM_TRY(ff_comm_launch(h->is_real != 0, v->is_real != 0, Rg, true, p, grid, s));
  for (int m = 2; m < M; ++m) {  // T: t_b -> t_a (in place over T_{m-2}); C: c_b -> c_a
    p.tcur = t_b;
    p.tout = t_a;
    p.ccur = c_b;
    p.cout = c_a;
    p.m = m;
    KPM_TRY(ff_comm_launch(h->is_real != 0, v->is_real != 0, Rg, false, p, grid, s));
    std::swap(t_a, t_b);
    std::swap(c_a, c_b);
  }
  return KPM_OK;
}

// sigma partials: per CTA sum of conj(U_c) (V1 U) over its rows, in float pairs then FP64
// ([grid][R] double2); V1 values are the doubled float pairs (halved at the end, exact).
template <bool RV, int R>
__global__ void __launch_bounds__(kBlock) ff_corr_kernel(const void* val, const int32_t* __restrict__ col, int64_t ld,
                                                         int L, int64_t n_pad, const float4* __restrict__ u,
                                                         const float4* __restrict__ uc, double2* part) {
  using MV = typename FFVal<RV>::type;
  constexpr int RPB = kBlock / R;
  __shared__ double2 red[(kBlock / 32) * R];
  const int sub = threadIdx.x % R, rl = threadIdx.x / R;
  const MV* __restrict__ vv = static_cast<const MV*>(val);
  double mr[1] = {0.0}, mi[1] = {0.0};
  FFMom mom{0.f, 0.f, 0.f, 0.f};
  int pending = 0;
  for (int64_t row = (int64_t)blockIdx.x * RPB + rl; row < n_pad; row += (int64_t)gridDim.x * RPB) {
    FF y{0.f, 0.f, 0.f, 0.f};
    for (int s = 0; s < L; ++s) {
      const int32_t j = __ldcs(col + (int64_t)s * ld + row);
      ff_mac(y, __ldcs(vv + (int64_t)s * ld + row), ff_of(__ldg(u + (int64_t)j * R + sub)));
    }
    ff_norm(y.rh, y.rl);
    ff_norm(y.ih, y.il);
    y = FF{0.5f * y.rh, 0.5f * y.ih, 0.5f * y.rl, 0.5f * y.il};
    ff_cdot(mom, ff_of(__ldg(uc + row * R + sub)), y);
    if (++pending == kFfFlush) {
      pending = 0;
      ff_fold(mr[0], mi[0], mom);
    }
  }
  ff_fold(mr[0], mi[0], mom);
  block_reduce_store<R, 1>(mr, mi, part + (int64_t)blockIdx.x * R, red);
}

int ff_corr_launch(bool rv, int R, const kpm_ell_s* v1, const float4* u, const float4* uc, double2* part, int grid,
                   cudaStream_t s) {
#define KPM_FFC(RR)                                                                                             \
  if (rv)                                                                                                       \
    ff_corr_kernel<true, RR><<<grid, kBlock, 0, s>>>(v1->val32, v1->col, v1->n_pad, v1->L, v1->n_pad, u, uc,    \
                                                     part);                                                      \
  else                                                                                                          \
    ff_corr_kernel<false, RR><<<grid, kBlock, 0, s>>>(v1->val32, v1->col, v1->n_pad, v1->L, v1->n_pad, u, uc,   \
                                                      part);                                                     \
  return check_cuda(cudaGetLastError())
  switch (R) {
    case 1: KPM_FFC(1);
    case 2: KPM_FFC(2);
    case 4: KPM_FFC(4);
    case 8: KPM_FFC(8);
    default: return KPM_ERR_UNSUPPORTED;
  }
#undef KPM_FFC
}

}  // namespace

// Left vectors for float-float moment products of the FP64 recursion: complex128 [R][n] ->
// float pairs [n_pad][Rg] (hi = the nearest float, lo = the nearest float to the rest).  A
// component that is neither zero nor in [2^-50, 2^59) gets a NaN high part, which sends
// that element to the FP64 product (ff_left_ok).
__global__ void pack_left_ff_kernel(const double2* __restrict__ src, int64_t n, int64_t n_pad, int R, int r0, int Rg,
                                    float4* __restrict__ dst) {
  const int64_t total = n_pad * Rg;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = t / Rg;
    const int r = (int)(t % Rg);
    double2 z = make_double2(0.0, 0.0);
    if (row < n) z = src[(int64_t)(r0 + r) * n + row];
    float q[4];
    const double c[2] = {z.x, z.y};
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const double a = fabs(c[k]);
      if (c[k] == 0.0 || (a >= 0x1p-50 && a < 0x1p59)) {
        q[k] = (float)c[k];
        q[k + 2] = (float)(c[k] - (double)q[k]);
      } else {
        q[k] = __uint_as_float(0x7fffffffu);
        q[k + 2] = 0.f;
      }
    }
    dst[t] = make_float4(q[0], q[1], q[2], q[3]);
  }
}

int pack_left_ff(const double* v, int64_t n, int64_t n_pad, int R, int r0, int Rg, void* dst, cudaStream_t s) {
  const int64_t total = n_pad * Rg;
  const int pg = (int)std::min<int64_t>((total + 255) / 256, 65536);
  pack_left_ff_kernel<<<pg, 256, 0, s>>>(reinterpret_cast<const double2*>(v), n, n_pad, R, r0, Rg,
                                         static_cast<float4*>(dst));
  return check_cuda(cudaGetLastError());
}

// Commutator series (rec_com_A_vec) of vectors r0 .. r0 + Rg in float-float arithmetic.
int comm_series_group_ff(kpm_ell_s* h, kpm_ell_s* v, int R, int r0, int Rg, int M, const double* c, const double* x,
                         double* out, cudaStream_t s) {
  KPM_TRY(ensure_f32_values(h, s));
  KPM_TRY(ensure_f32_values(v, s));
  const size_t vb = (size_t)h->n_pad * Rg * sizeof(float4);
  Workspace& ws = h->ws;
  KPM_TRY(ensure(ws.vl, vb));
  KPM_TRY(ensure(ws.acc, vb));
  KPM_TRY(ff_pack(x, h->n, h->n_pad, R, r0, Rg, ws.vl.p, s));
  KPM_TRY(ff_comm_series_packed(h, v, Rg, M, reinterpret_cast<const double2*>(c), static_cast<const float4*>(ws.vl.p),
                                static_cast<float4*>(ws.acc.p), s));
  const int64_t total = h->n * Rg;
  const int g = (int)std::min<int64_t>((total + 255) / 256, 65536);
  ff_unpack_kernel<<<g, 256, 0, s>>>(static_cast<const float4*>(ws.acc.p), h->n, Rg, r0,
                                     reinterpret_cast<double2*>(out));
  return check_cuda(cudaGetLastError());
}

// Time-domain Kubo correlator of vectors r0 .. r0 + Rg (Rg <= 4) in float-float arithmetic:
// U_c(t_0) by the commutator series, U and U_c advanced as one set of 2 Rg vectors by the
// series with c_u, sigma[r][j] = <U_c(t_j)|V1 U(t_j)> reduced in FP64.
int time_sigma_group_ff(kpm_ell_s* h, kpm_ell_s* v1, kpm_ell_s* v2, int R, int r0, int Rg, const double* c_u, int M2,
                        const double* c_fd, int M, int len_t, const double* v, double* sigma, cudaStream_t s) {
  KPM_TRY(ensure_f32_values(h, s));
  KPM_TRY(ensure_f32_values(v1, s));
  KPM_TRY(ensure_f32_values(v2, s));
  const size_t vb = (size_t)h->n_pad * Rg * sizeof(float4);
  Workspace& ws = h->ws;
  StepConfig cfg;
  if (M2 > 2) KPM_TRY(ff_config(h, 2 * Rg, true, s, &cfg));  // before the buffers its timing clears are filled
  KPM_TRY(ensure(ws.vr, vb));        // U
  KPM_TRY(ensure(ws.acc, vb));       // U_c
  KPM_TRY(ensure(ws.td, 2 * vb));    // joined state (also commutator scratch)
  KPM_TRY(ensure(ws.acc2, 2 * vb));  // the next joined state (likewise)
  const int grid = grid_for(v1, Rg, 1);
  KPM_TRY(ensure(ws.part, (size_t)grid * Rg * sizeof(double2)));
  KPM_TRY(ff_pack(v, h->n, h->n_pad, R, r0, Rg, ws.vr.p, s));
  KPM_TRY(ff_comm_series_packed(h, v2, Rg, M, reinterpret_cast<const double2*>(c_fd),
                                static_cast<const float4*>(ws.vr.p), static_cast<float4*>(ws.acc.p), s));
  double* outs[2] = {sigma, sigma};
  double2* U = static_cast<double2*>(ws.vr.p);  // 16-byte entries: float pairs moved as double2
  double2* Uc = static_cast<double2*>(ws.acc.p);
  void* cur = ws.td.p;
  void* nxt = ws.acc2.p;
  for (int j = 0; j < len_t; ++j) {
    if (j > 0) {
      if (j == 1) KPM_TRY(join_split(U, Uc, static_cast<double2*>(cur), h->n_pad, Rg, true, s));
      KPM_TRY(ff_series_packed(h, 2 * Rg, M2, cfg, reinterpret_cast<const double2*>(c_u), cur, nxt, s));
      std::swap(cur, nxt);
      KPM_TRY(join_split(U, Uc, static_cast<double2*>(cur), h->n_pad, Rg, false, s));
    }
    KPM_TRY(ff_corr_launch(v1->is_real != 0, Rg, v1, reinterpret_cast<const float4*>(U),
                           reinterpret_cast<const float4*>(Uc), static_cast<double2*>(ws.part.p), grid, s));
    KPM_TRY(reduce_partials(static_cast<double2*>(ws.part.p), 1, 1, grid, Rg, outs, R, r0, len_t, j, s));
  }
  return KPM_OK;
}

// out[r] = P^steps v[r], P = sum_{m<M} c_m T_m(H), for vectors r0 .. r0 + Rg in float-float
// arithmetic (steps = 1: the series of rec_A_vec).  The state ping-pongs between ws.tc and
// ws.acc; the recursion uses ws.ta / ws.tb.
int series_group_ff(kpm_ell_s* h, int R, int r0, int Rg, int M, const double* c, int steps, const double* v,
                    double* out, cudaStream_t s) {
  KPM_TRY(ensure_f32_values(h, s));
  StepConfig cfg;
  if (M > 2) KPM_TRY(ff_config(h, Rg, true, s, &cfg));
  const size_t vb = (size_t)h->n_pad * Rg * sizeof(float4);
  Workspace& ws = h->ws;
  KPM_TRY(ensure(ws.tc, vb));
  KPM_TRY(ensure(ws.acc, vb));
  KPM_TRY(ff_pack(v, h->n, h->n_pad, R, r0, Rg, ws.tc.p, s));
  void* x = ws.tc.p;
  void* y = ws.acc.p;
  for (int j = 0; j < steps; ++j) {
    KPM_TRY(ff_series_packed(h, Rg, M, cfg, reinterpret_cast<const double2*>(c), x, y, s));
    std::swap(x, y);
  }
  const int64_t total = h->n * Rg;
  const int g = (int)std::min<int64_t>((total + 255) / 256, 65536);
  ff_unpack_kernel<<<g, 256, 0, s>>>(static_cast<const float4*>(x), h->n, Rg, r0, reinterpret_cast<double2*>(out));
  return check_cuda(cudaGetLastError());
}

// DOS / two-vector moments <v_l|T_m v_r> of one group of Rg vectors in float-float arithmetic.
int moments_group_ff(kpm_ell_s* h, int R, int r0, int Rg, int M, const double* v_r, const double* v_l, double* mu,
                     cudaStream_t s) {
  KPM_TRY(ensure_f32_values(h, s));
  const size_t vb = (size_t)h->n_pad * Rg * sizeof(float4);
  Workspace& ws = h->ws;
  KPM_TRY(ensure(ws.ta, vb));
  KPM_TRY(ensure(ws.tb, vb));
  KPM_TRY(ensure(ws.vl, vb));
  StepConfig cfg;
  KPM_TRY(ff_config(h, Rg, false, s, &cfg));
  const int grid_first = grid_for(h, Rg, 1);
  const int grid_next = cfg.grid;
  const int grid = std::max(grid_next, grid_first);
  const int64_t step_stride = (int64_t)grid * Rg;
  KPM_TRY(ensure(ws.part, (size_t)kChunk * step_stride * sizeof(double2)));
  const int64_t total = h->n_pad * Rg;
  const int pg = (int)std::min<int64_t>((total + 255) / 256, 65536);
  ff_pack_kernel<<<pg, 256, 0, s>>>(reinterpret_cast<const double2*>(v_r), h->n, h->n_pad, R, r0, Rg,
                                    static_cast<float4*>(ws.ta.p));
  ff_pack_kernel<<<pg, 256, 0, s>>>(reinterpret_cast<const double2*>(v_l ? v_l : v_r), h->n, h->n_pad, R, r0, Rg,
                                    static_cast<float4*>(ws.vl.p));
  KPM_CUDA_TRY(cudaGetLastError());
  double2* part = static_cast<double2*>(ws.part.p);
  double* outs[2] = {mu, mu};
  StepParams p = base_params(h, true);  // the float-pair values
  p.vl = ws.vl.p;
  p.part_step_stride = (int64_t)grid_first * Rg;
  p.tcur = ws.ta.p;
  p.tout = ws.tb.p;
  p.part = part;
  KPM_TRY(ff_dispatch(h->is_real != 0, Rg, -1, p, grid_first, s));
  KPM_TRY(reduce_partials(part, std::min(M, 2), 1, grid_first, Rg, outs, R, r0, M, 0, s));
  void* tprev = ws.ta.p;
  void* tcur = ws.tb.p;
  int m0 = 2;
  cudaEvent_t ev = nullptr;
  if (M > 2) KPM_TRY(prof_begin(h, s, &ev));
  for (int m = 2; m < M; ++m) {
    if (m - m0 == kChunk) {
      KPM_TRY(reduce_partials(part, kChunk, 1, grid_next, Rg, outs, R, r0, M, m0, s));
      m0 = m;
    }
    p.tcur = tcur;
    p.tout = tprev;
    p.part = part + (int64_t)(m - m0) * grid_next * Rg;
    KPM_TRY(ff_dispatch(h->is_real != 0, Rg, cfg.kind == 0 ? 0 : cfg.U, p, grid_next, s));
    std::swap(tprev, tcur);
  }
  if (M > 2) KPM_TRY(prof_end(h, s, ev, M - 2));
  if (M > m0) KPM_TRY(reduce_partials(part, M - m0, 1, grid_next, Rg, outs, R, r0, M, m0, s));
  return KPM_OK;
}

}  // namespace kpm
