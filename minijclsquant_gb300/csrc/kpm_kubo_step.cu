// kpm_kubo_step.cu -- one recursion step of the Kubo-Greenwood right rows with the
// velocity product fused in:
//
//   T_{m+1} = 2H T_m - T_{m-1}   (in place over T_{m-1})   and   B_m = V T_m,
//
// in complex64 with the split-float operator values and compensated accumulation of
// the step kernels.  V = H o d (modifier_velocity, jclsquant/modifiers.py:56-79) has
// H's sparsity, so when the two ELL column arrays are equal the gathers of T_m at
// the columns serve both products: one pass over the columns and over T_m instead
// of a recursion step plus a separate V T_m launch (the kpm_mu_nm right-row loop).
//
// Staging is that of cheb_next_ws_kernel: a producer warp issues 1-D bulk copies of
// the tile's column slabs, H value slabs, V value slabs and T_{m-1} into one of
// kWsStages shared-memory stages (full / empty mbarriers, every wait bounded); the
// compute warps gather T_m, accumulate both products and store T_{m+1} and B_m.
#include "kpm_ws.cuh"

namespace kpm {

namespace {

template <bool REAL, int TPR, int VPT>
__global__ void __launch_bounds__(kWsThreads, 2)
    kubo_step_kernel(const StepParams p, const float4* __restrict__ vval, void* bout) {
  using T = float;
  using Raw = typename RawT<T, VPT>::type;
  using MV = typename MatV<T, REAL>::type;
  constexpr int RPB = kBlock / TPR;
  constexpr int TILE = RPB;
  constexpr int kWarps = kBlock / 32;

  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[kWsStages];
  __shared__ __align__(8) uint64_t empty[kWsStages];

  const int L = p.L;
  const uint32_t col_b = (uint32_t)align16((size_t)L * TILE * 4);
  const uint32_t val_b = (uint32_t)align16((size_t)L * TILE * sizeof(MV));
  const uint32_t vv_b = (uint32_t)align16((size_t)L * TILE * sizeof(float4));
  const uint32_t vec_b = (uint32_t)(TILE * TPR * sizeof(Raw));
  const uint32_t stage_b = col_b + val_b + vv_b + vec_b;
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
      const uint64_t pol = l2_evict_first_policy();
      const unsigned char* hval = static_cast<const unsigned char*>(p.val);
      const unsigned char* old = static_cast<const unsigned char*>(p.tout);
      const uint32_t tx = (uint32_t)L * TILE * (4 + (uint32_t)sizeof(MV) + (uint32_t)sizeof(float4)) + vec_b;
      int issued = 0;
      for (int k = 0; k < my_count; ++k) {
        const int st = k % kWsStages;
        if (k >= kWsStages && !mbar_wait_bounded(&empty[st], (uint32_t)(((k / kWsStages) - 1) & 1))) {
          atomicExch(p.err, KPM_ERR_TIMEOUT);
          break;
        }
        fence_proxy_async_shared();
        unsigned char* stage = smem + (size_t)st * stage_b;
        const int64_t row0 = tile_of(k) * TILE;
        mbar_arrive_expect_tx(&full[st], tx);
        for (int s = 0; s < L; ++s)
          bulk_g2s(stage + (size_t)s * TILE * 4, p.col + (int64_t)s * p.ld + row0, TILE * 4, &full[st], pol);
        for (int s = 0; s < L; ++s)
          bulk_g2s(stage + col_b + (size_t)s * TILE * sizeof(MV), hval + ((int64_t)s * p.ld + row0) * sizeof(MV),
                   TILE * (uint32_t)sizeof(MV), &full[st], pol);
        for (int s = 0; s < L; ++s)
          bulk_g2s(stage + col_b + val_b + (size_t)s * TILE * sizeof(float4), vval + (int64_t)s * p.ld + row0,
                   TILE * (uint32_t)sizeof(float4), &full[st], pol);
        bulk_g2s(stage + col_b + val_b + vv_b, old + row0 * TPR * (int64_t)sizeof(Raw), vec_b, &full[st], pol);
        issued = k + 1;
      }
      // copies of the last stages may still be landing: wait for them before leaving
      for (int q = issued > kWsStages ? issued - kWsStages : 0; q < issued; ++q)
        (void)mbar_wait_bounded(&full[q % kWsStages], (uint32_t)((q / kWsStages) & 1));
    }
    return;
  }

  const Raw* __restrict__ tcur = static_cast<const Raw*>(p.tcur);
  Raw* tout = static_cast<Raw*>(p.tout);
  Raw* bo = static_cast<Raw*>(bout);
  const int sub = threadIdx.x % TPR;
  const int rl = threadIdx.x / TPR;
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
    const unsigned char* base = smem + (size_t)st * stage_b;
    const int32_t* scol = reinterpret_cast<const int32_t*>(base);
    const MV* sval = reinterpret_cast<const MV*>(base + col_b);
    const float4* svv = reinterpret_cast<const float4*>(base + col_b + val_b);
    const Raw* sold = reinterpret_cast<const Raw*>(base + col_b + val_b + vv_b);
    CxC<VPT> acc, vacc;
    for (int s = 0; s < L; s += 4) {
      int c[4];
      MV h[4];
      float4 w[4];
      Cx<T, VPT> x[4];
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (s + j < L) {
          c[j] = scol[(s + j) * TILE + rl];
          h[j] = sval[(s + j) * TILE + rl];
          w[j] = svv[(s + j) * TILE + rl];
        }
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (s + j < L) unpack(__ldg(tcur + (int64_t)c[j] * TPR + sub), x[j]);
      if (s == 0) {
        Cx<T, VPT> o;
        unpack(sold[rl * TPR + sub], o);
        madd_first_neg(acc, h[0], x[0], o);
        mul_first(vacc, w[0], x[0]);
      } else {
        madd(acc, h[0], x[0]);
        madd(vacc, w[0], x[0]);
      }
#pragma unroll
      for (int j = 1; j < 4; ++j)
        if (s + j < L) {
          madd(acc, h[j], x[j]);
          madd(vacc, w[j], x[j]);
        }
    }
    // the stage is no longer read: hand it back to the producer
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[st]);
    const int64_t vi = (tile_of(k) * TILE + rl) * TPR + sub;
    tout[vi] = pack(finish(acc));
    Cx<T, VPT> vb = finish(vacc);  // (2V) T_m: the stored values are doubled
#pragma unroll
    for (int q = 0; q < VPT; ++q) {
      vb.re[q] *= 0.5f;
      vb.im[q] *= 0.5f;
    }
    bo[vi] = pack(vb);
  }
}

template <bool REAL, int TPR, int VPT>
size_t kubo_stage_bytes(int L) {
  using MV = typename MatV<float, REAL>::type;
  constexpr int TILE = kBlock / TPR;
  return align16((size_t)L * TILE * 4) + align16((size_t)L * TILE * sizeof(MV)) +
         align16((size_t)L * TILE * sizeof(float4)) + (size_t)TILE * TPR * sizeof(typename RawT<float, VPT>::type);
}

template <bool REAL, int TPR, int VPT>
bool kubo_smem_attr(size_t smem) {
  static size_t configured = 0;
  if (smem <= configured) return true;
  if (cudaFuncSetAttribute(kubo_step_kernel<REAL, TPR, VPT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  configured = smem;
  return true;
}

template <bool REAL, int R>
int kubo_go(const StepParams& p, const void* vval, void* bout, int sm_count, cudaStream_t s, bool launch) {
  constexpr int VPT = R >= 2 ? 2 : 1;
  constexpr int TPR = R / VPT;
  const size_t smem = kWsStages * kubo_stage_bytes<REAL, TPR, VPT>(p.L);
  if (smem > 200 * 1024 || !kubo_smem_attr<REAL, TPR, VPT>(smem)) return KPM_ERR_UNSUPPORTED;
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kubo_step_kernel<REAL, TPR, VPT>, kWsThreads, smem) !=
          cudaSuccess ||
      occ < 1) {
    (void)cudaGetLastError();
    return KPM_ERR_UNSUPPORTED;
  }
  if (!launch) return KPM_OK;
  const int64_t ntiles = p.n_pad / (kBlock / TPR);
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ntiles, (int64_t)occ * sm_count));
  kubo_step_kernel<REAL, TPR, VPT><<<grid, kWsThreads, smem, s>>>(p, static_cast<const float4*>(vval), bout);
  return check_cuda(cudaGetLastError());
}

}  // namespace

// The fused step for R vectors (1, 2 or 4); launch == false only checks that it fits.
int kubo_step(bool real_h, int R, const StepParams& p, const void* vval, void* bout, int sm_count, cudaStream_t s,
              bool launch) {
  switch (R) {
    case 1: return real_h ? kubo_go<true, 1>(p, vval, bout, sm_count, s, launch)
                          : kubo_go<false, 1>(p, vval, bout, sm_count, s, launch);
    case 2: return real_h ? kubo_go<true, 2>(p, vval, bout, sm_count, s, launch)
                          : kubo_go<false, 2>(p, vval, bout, sm_count, s, launch);
    case 4: return real_h ? kubo_go<true, 4>(p, vval, bout, sm_count, s, launch)
                          : kubo_go<false, 4>(p, vval, bout, sm_count, s, launch);
    default: return KPM_ERR_UNSUPPORTED;
  }
}

}  // namespace kpm
