// kpm_staged.cuh -- the hot recursion step with bulk-copy staging.
//
//   T_{m+1} = 2H T_m - T_{m-1}  (in place over T_{m-1})  and  <v_l | T_{m+1}>
//
// Each CTA owns a strided set of row tiles.  For every tile, one thread issues
// 1-D cp.async.bulk copies (the TMA engine) of everything the tile streams:
// the L column slabs, the L value slabs, T_{m-1} and the left vector(s), into
// one of S shared-memory stages, counted on that stage's mbarrier.  While the
// CTA computes tile k, tiles k+1 .. k+S-1 are in flight.  Only the neighbour
// gathers T_m[col] remain on the load/store path, their addresses come from
// shared memory, and T_{m+1} is stored straight from registers.
//
// The first multiply-add of every row folds -T_{m-1} into its addend, so a
// real-valued operator costs exactly 2L + 4 FP64 FMAs per site-step.
//
// per_tile != 0 (batched operators): moment partials are stored per tile
// ([tile][R]) instead of per CTA, so tiles of different instances never mix.
#pragma once

#include "kpm_async.cuh"
#include "kpm_cheb.cuh"

namespace kpm {

__host__ __device__ constexpr size_t align16(size_t b) { return (b + 15) & ~size_t(15); }

// Shared-memory bytes of one stage.
template <typename T, bool REAL, int TPR, int VPT, int U>
__host__ __device__ constexpr size_t staged_stage_bytes(int L, int nvec) {
  using MVs = typename MatV<T, REAL>::type;
  constexpr int RPB = kBlock / TPR;
  constexpr int TILE = RPB * U;
  return align16((size_t)L * TILE * 4) + align16((size_t)L * TILE * sizeof(MVs)) +
         (size_t)nvec * TILE * TPR * sizeof(typename RawT<T, VPT>::type);
}

constexpr int kStages = 3;

// Issue the bulk copies of one tile into one stage (called by one thread).
// Kept out of line so its address arithmetic does not occupy registers of the
// compute loop.
struct TileCopy {
  const int32_t* col;
  const unsigned char* val;
  const unsigned char* old;
  const unsigned char* vl;
  const unsigned char* vl2;
  const unsigned char* cur;  // T_m: its rows of the tile are prefetched into L2 (null: none)
  int64_t ld;
  int L;
  uint32_t col_slab;   // bytes of one column slab (TILE * 4)
  uint32_t val_slab;   // bytes of one value slab
  uint32_t vec_slab;   // bytes of one vector tile
  uint32_t vl_slab;    // bytes of the left-vector (or half-norm) tile
  uint32_t col_b, val_b;  // stage offsets
  uint32_t tx_bytes;
};

static __device__ __noinline__ void issue_tile(const TileCopy& tc, unsigned char* stage, uint64_t* bar,
                                               int64_t row0, int vec_bytes_per_row, uint64_t pol) {
  mbar_arrive_expect_tx(bar, tc.tx_bytes);
  const int tile = (int)(tc.col_slab / 4);
  for (int s = 0; s < tc.L; ++s)
    bulk_g2s(stage + (size_t)s * tc.col_slab, tc.col + (int64_t)s * tc.ld + row0, tc.col_slab, bar, pol);
  const int64_t vbytes = tc.val_slab / tile;
  for (int s = 0; s < tc.L; ++s)
    bulk_g2s(stage + tc.col_b + (size_t)s * tc.val_slab, tc.val + ((int64_t)s * tc.ld + row0) * vbytes, tc.val_slab,
             bar, pol);
  const int64_t voff = row0 * vec_bytes_per_row;
  // the tile's own rows of T_m, which its neighbour gathers touch first, into L2 ahead of them
  if (tc.cur) bulk_prefetch_l2(tc.cur + voff, tc.vec_slab);
  bulk_g2s(stage + tc.col_b + tc.val_b, tc.old + voff, tc.vec_slab, bar, pol);
  if (tc.vl)
    bulk_g2s(stage + tc.col_b + tc.val_b + tc.vec_slab, tc.vl + row0 * (int64_t)(tc.vl_slab / tile), tc.vl_slab, bar,
             pol);
}

template <typename T, bool REAL, int TPR, int VPT, int U>
__global__ void __launch_bounds__(kBlock, (U == 1 ? 3 : 2)) cheb_next_staged_kernel(const StepParams p) {
  using Raw = typename RawT<T, VPT>::type;
  using MV = typename MatV<T, REAL>::type;
  constexpr int R = TPR * VPT;
  constexpr int RPB = kBlock / TPR;
  constexpr int TILE = RPB * U;
  constexpr bool F32 = std::is_same<T, float>::value;
  constexpr int kFlush = 8;

  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bars[kStages];
  __shared__ double2 red[(kBlock / 32) * R];

  const int L = p.L;
  const uint32_t col_b = (uint32_t)align16((size_t)L * TILE * 4);
  const uint32_t val_b = (uint32_t)align16((size_t)L * TILE * sizeof(MV));
  const uint32_t vec_b = (uint32_t)(TILE * TPR * sizeof(Raw));
  const uint32_t stage_b = col_b + val_b + 2 * vec_b;

  const int ntiles = (int)(p.n_pad / TILE);
  // tiles of this CTA: strided (plain operators) or one contiguous range (batched)
  const int seg_tb = (int)(((int64_t)blockIdx.x * ntiles) / gridDim.x);
  const int seg_te = (int)(((int64_t)(blockIdx.x + 1) * ntiles) / gridDim.x);
  // kernel-parameter fields read in the tile loop are copied to registers first (a
  // reference to p taken by a lambda would place p in local memory)
  const bool per_tile = p.per_tile != 0;
  const int my_count = per_tile ? seg_te - seg_tb
                                  : (((int)blockIdx.x < ntiles) ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0);
  auto tile_of = [per_tile, seg_tb](int k) -> int64_t {
    return per_tile ? (int64_t)seg_tb + k : (int64_t)blockIdx.x + (int64_t)k * gridDim.x;
  };

  if (threadIdx.x == 0) {
#pragma unroll
    for (int s = 0; s < kStages; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
  }
  __syncthreads();

  TileCopy tc;
  uint64_t pol = 0;
  if (threadIdx.x == 0) {
    pol = l2_evict_first_policy();
    tc.col = p.col;
    tc.val = static_cast<const unsigned char*>(p.val);
    tc.old = static_cast<const unsigned char*>(p.tout);
    tc.vl = static_cast<const unsigned char*>(p.vl);
    tc.vl2 = nullptr;
    tc.cur = nullptr;
    tc.ld = p.ld;
    tc.L = L;
    tc.col_slab = TILE * 4;
    tc.val_slab = (uint32_t)(TILE * sizeof(MV));
    tc.vec_slab = vec_b;
    tc.vl_slab = vec_b;
    tc.col_b = col_b;
    tc.val_b = val_b;
    tc.tx_bytes = (uint32_t)L * TILE * 4 + (uint32_t)L * TILE * (uint32_t)sizeof(MV) + 2 * vec_b;
    for (int k = 0; k < kStages - 1 && k < my_count; ++k)
      issue_tile(tc, smem + (k % kStages) * stage_b, &bars[k % kStages], tile_of(k) * TILE, TPR * (int)sizeof(Raw),
                 pol);
  }
  int seg = per_tile ? p.seg_base[blockIdx.x] : 0;
  int cur_inst = (per_tile && my_count > 0) ? p.tile_inst[seg_tb] : 0;

  const Raw* __restrict__ tcur = static_cast<const Raw*>(p.tcur);
  Raw* tout = static_cast<Raw*>(p.tout);
  const int sub = threadIdx.x % TPR;
  const int rl = threadIdx.x / TPR;
  double mr[VPT], mi[VPT];
  T fr[VPT], fi[VPT];
#pragma unroll
  for (int q = 0; q < VPT; ++q) {
    mr[q] = mi[q] = 0.0;
    fr[q] = fi[q] = T(0);
  }
  int pending = 0;

  for (int k = 0; k < my_count; ++k) {
    if (threadIdx.x == 0 && k + kStages - 1 < my_count) {
      fence_proxy_async_shared();
      const int kn = k + kStages - 1;
      issue_tile(tc, smem + (kn % kStages) * stage_b, &bars[kn % kStages], tile_of(kn) * TILE,
                 TPR * (int)sizeof(Raw), pol);
    }
    const int st = k % kStages;
    const bool ok = mbar_wait_bounded(&bars[st], (uint32_t)((k / kStages) & 1));
    if (ok) {
      const unsigned char* base = smem + st * stage_b;
      const int32_t* scol = reinterpret_cast<const int32_t*>(base);
      const MV* sval = reinterpret_cast<const MV*>(base + col_b);
      const Raw* sold = reinterpret_cast<const Raw*>(base + col_b + val_b);
      const Raw* svl = reinterpret_cast<const Raw*>(base + col_b + val_b + vec_b);
      const int64_t row0 = tile_of(k) * TILE;
      typename AccOf<T, VPT>::type accum[U];
      for (int s = 0; s < L; s += 4) {
        int c[U][4];
        MV h[U][4];
        Cx<T, VPT> x[U][4];
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
          for (int j = 0; j < 4; ++j)
            if (s + j < L) {
              c[u][j] = scol[(s + j) * TILE + u * RPB + rl];
              h[u][j] = sval[(s + j) * TILE + u * RPB + rl];
            }
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
          for (int j = 0; j < 4; ++j)
            if (s + j < L) unpack(__ldg(tcur + (int64_t)c[u][j] * TPR + sub), x[u][j]);
#pragma unroll
        for (int u = 0; u < U; ++u) {
          if (s == 0) {
            Cx<T, VPT> old;
            unpack(sold[(u * RPB + rl) * TPR + sub], old);
            madd_first_neg(accum[u], h[u][0], x[u][0], old);
          } else {
            madd(accum[u], h[u][0], x[u][0]);
          }
#pragma unroll
          for (int j = 1; j < 4; ++j)
            if (s + j < L) madd(accum[u], h[u][j], x[u][j]);
        }
      }
      Cx<T, VPT> acc[U];
#pragma unroll
      for (int u = 0; u < U; ++u) acc[u] = finish(accum[u]);
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int lr = u * RPB + rl;
        tout[(row0 + lr) * TPR + sub] = pack(acc[u]);
        Cx<T, VPT> l;
        unpack(svl[lr * TPR + sub], l);
#pragma unroll
        for (int q = 0; q < VPT; ++q) {
          if (F32)
            cdot_acc(fr[q], fi[q], l.re[q], l.im[q], acc[u].re[q], acc[u].im[q]);
          else
            cdot_acc(mr[q], mi[q], l.re[q], l.im[q], acc[u].re[q], acc[u].im[q]);
        }
        if (F32 && ++pending == kFlush) {
          pending = 0;
#pragma unroll
          for (int q = 0; q < VPT; ++q) {
            mr[q] += (double)fr[q];
            mi[q] += (double)fi[q];
            fr[q] = fi[q] = T(0);
          }
        }
      }
    }
    if (__syncthreads_or(!ok)) {
      // A bulk copy never arrived: record it, wait (bounded) for the copies this
      // CTA still has in flight so none lands after exit, and leave.
      if (threadIdx.x == 0) {
        atomicExch(p.err, KPM_ERR_TIMEOUT);
        for (int q = k; q < my_count && q < k + kStages; ++q)
          (void)mbar_wait_bounded(&bars[q % kStages], (uint32_t)((q / kStages) & 1));
      }
      return;
    }
    if (per_tile) {
      // flush the accumulators when the next tile belongs to another instance (or at the end)
      const int next_inst = (k + 1 < my_count) ? p.tile_inst[seg_tb + k + 1] : -1;
      if (next_inst != cur_inst) {
        if (F32) {
#pragma unroll
          for (int q = 0; q < VPT; ++q) {
            mr[q] += (double)fr[q];
            mi[q] += (double)fi[q];
            fr[q] = fi[q] = T(0);
          }
          pending = 0;
        }
        block_reduce_store<TPR, VPT>(mr, mi, p.part + (int64_t)seg * R, red);
#pragma unroll
        for (int q = 0; q < VPT; ++q) mr[q] = mi[q] = 0.0;
        ++seg;
        cur_inst = next_inst;
      }
    }
  }

  if (!per_tile) {
    if (F32) {
#pragma unroll
      for (int q = 0; q < VPT; ++q) {
        mr[q] += (double)fr[q];
        mi[q] += (double)fi[q];
      }
    }
    block_reduce_store<TPR, VPT>(mr, mi, p.part + (int64_t)blockIdx.x * R, red);
  }
}

// Raise the kernel's dynamic shared-memory limit to `smem` once (shared by the
// occupancy query, which runs before any graph capture, and the launch).
template <typename T, bool REAL, int TPR, int VPT, int U>
bool staged_smem_attr(size_t smem) {
  static size_t configured = 0;
  if (smem <= configured) return true;
  cudaError_t e = cudaFuncSetAttribute(cheb_next_staged_kernel<T, REAL, TPR, VPT, U>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) {
    set_last_cuda_error(e);
    (void)cudaGetLastError();
    return false;
  }
  configured = smem;
  return true;
}

// Launch with the dynamic shared memory one CTA needs (kStages stages).
template <typename T, bool REAL, int TPR, int VPT, int U>
int launch_staged(const StepParams& p, int grid, cudaStream_t s) {
  auto kern = cheb_next_staged_kernel<T, REAL, TPR, VPT, U>;
  const size_t smem = kStages * staged_stage_bytes<T, REAL, TPR, VPT, U>(p.L, 2);
  if (!staged_smem_attr<T, REAL, TPR, VPT, U>(smem)) return KPM_ERR_UNSUPPORTED;
  kern<<<grid, kBlock, smem, s>>>(p);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_cuda_error(e);
    return KPM_ERR_CUDA;
  }
  return KPM_OK;
}

// CTAs of the staged kernel that fit on one SM (0 if it cannot launch).
template <typename T, bool REAL, int TPR, int VPT, int U>
int staged_ctas_per_sm(int L, int nvec) {
  auto kern = cheb_next_staged_kernel<T, REAL, TPR, VPT, U>;
  const size_t smem = kStages * staged_stage_bytes<T, REAL, TPR, VPT, U>(L, nvec);
  if (smem > 200 * 1024) return 0;
  if (!staged_smem_attr<T, REAL, TPR, VPT, U>(smem)) return 0;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, kBlock, smem) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return n;
}

// Dispatch of the staged kernel over (real, R, U) for one precision T;
// VPT = 2 complex values per thread for float (R >= 2), else 1.
template <typename T>
struct Staged {
  template <bool REAL, int R, int U>
  static int go(const StepParams& p, int grid, cudaStream_t s) {
    constexpr int VPT = (std::is_same<T, float>::value && R >= 2) ? 2 : 1;
    return launch_staged<T, REAL, R / VPT, VPT, U>(p, grid, s);
  }
  template <bool REAL, int R, int U>
  static int occ(int L, int nvec) {
    constexpr int VPT = (std::is_same<T, float>::value && R >= 2) ? 2 : 1;
    return staged_ctas_per_sm<T, REAL, R / VPT, VPT, U>(L, nvec);
  }
  template <bool REAL, int R>
  static int go_u(int U, const StepParams& p, int grid, cudaStream_t s) {
    return U == 2 ? go<REAL, R, 2>(p, grid, s) : go<REAL, R, 1>(p, grid, s);
  }
  template <bool REAL, int R>
  static int occ_u(int U, int L, int nvec) {
    return U == 2 ? occ<REAL, R, 2>(L, nvec) : occ<REAL, R, 1>(L, nvec);
  }
  template <bool REAL>
  static int go_r(int R, int U, const StepParams& p, int grid, cudaStream_t s) {
    switch (R) {
      case 1: return go_u<REAL, 1>(U, p, grid, s);
      case 2: return go_u<REAL, 2>(U, p, grid, s);
      case 4: return go_u<REAL, 4>(U, p, grid, s);
      case 8: return go_u<REAL, 8>(U, p, grid, s);
      default: return KPM_ERR_UNSUPPORTED;
    }
  }
  template <bool REAL>
  static int occ_r(int R, int U, int L, int nvec) {
    switch (R) {
      case 1: return occ_u<REAL, 1>(U, L, nvec);
      case 2: return occ_u<REAL, 2>(U, L, nvec);
      case 4: return occ_u<REAL, 4>(U, L, nvec);
      case 8: return occ_u<REAL, 8>(U, L, nvec);
      default: return 0;
    }
  }
  static int launch(bool real, int R, int U, const StepParams& p, int grid, cudaStream_t s) {
    return real ? go_r<true>(R, U, p, grid, s) : go_r<false>(R, U, p, grid, s);
  }
  static int ctas_per_sm(bool real, int R, int U, int L, int nvec) {
    return real ? occ_r<true>(R, U, L, nvec) : occ_r<false>(R, U, L, nvec);
  }
};

}  // namespace kpm
