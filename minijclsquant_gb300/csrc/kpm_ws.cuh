// kpm_ws.cuh -- the staged recursion step with a producer warp.
//
//   T_{m+1} = 2H T_m - T_{m-1}  (in place over T_{m-1})  and  <v_l | T_{m+1}>
//
// Same tile layout and per-tile bulk copies as the staged kernel, but the CTA is
// split into kBlock compute threads and one producer warp.  Each of the NST
// shared-memory stages (ws_stages: four, or three for the one-vector float-float
// step) has a "full" mbarrier (the producer's expect_tx, completed by the copies)
// and an "empty" mbarrier (one arrival per compute warp once it has read the stage).  Compute warps never meet at a
// CTA-wide barrier inside the tile loop, so while one warp waits on its
// neighbour gathers T_m[col] the others compute, and the producer refills a
// stage as soon as the last warp has left it.  For complex128 the producer also
// prefetches the tile's own rows of T_m into L2 when it stages the tile, so the
// gathers, which touch those rows first, find them there.
//
// SB > 1 (complex128): a stage holds SB sub-tiles of TILE rows, taken by the compute
// warps one after the other (the stage's wait comes with the first, its release with
// the last), so each bulk copy brings SB times the rows at the registers of SB = 1.
//
// The series instantiation (K = kWsSeries) is a series step of rec_A_vec (p.series
// set, p.vl null, no doubling): the producer stages the series accumulator tile in
// the left-vector slot and the compute warps write back series + c_m T_{m+1}; no
// moments are formed.
//
// Moment partials follow the staged kernel: per CTA (strided tiles) or, for
// batched operators (per_tile), flushed per (CTA, instance) run with a block
// reduction over the compute warps alone (named barrier 1).  With p.vl null the
// step stores T_{m+1} only (no left vector is copied, no moments), and with
// p.tprev set T_{m-1} is read from there (out of place) instead of from tout.
// With p.dbl (doubling; K = kWsDbl) the producer stages |v|^2 / 2 in place of the
// left vector and the two moment sets <T_{m+1}|T_m>, sum (|T_m|^2 - |v|^2 / 2) are
// accumulated (T_m's own row read from tcur).
//
// With p.vl_ff (FP64 only, one moment set; K = kWsFF) the staged left vector holds float
// pairs and the moment products run in float-float arithmetic on the FP32 pipe
// (ff_split_f64 / ff_cdot, folded into FP64 every kFfFoldRows rows); an element outside the
// float-pair range takes the FP64 product with v_l read from p.vl64.  The recursion itself
// stays FP64.
//
// Every wait is bounded.  A compute warp whose wait runs out records
// KPM_ERR_TIMEOUT and stops computing but still takes part in the named
// barriers, so no warp waits on one that has left; the producer that times
// out stops issuing and waits (bounded) for its copies in flight before exit.
#pragma once

#include "kpm_ff.cuh"
#include "kpm_staged.cuh"

namespace kpm {

constexpr int kWsStages = 4;
constexpr int kWsThreads = kBlock + 32;  // compute warps + one producer warp

// Epilogue variants (template parameter K): each instantiation carries only its own code, so
// the registers of one do not limit the occupancy of another.
constexpr int kWsMom = 0;     // FP64 / complex64 moments (one set), or store only
constexpr int kWsSeries = 1;  // series step
constexpr int kWsFF = 2;      // FP64 recursion, one moment set with float-float products
constexpr int kWsDbl = 3;     // doubled moments (two sets per step)

// Shared-memory stages of one instantiation: three for the one-vector float-float step of a
// real operator (three of its 20 KB stages per CTA let three CTAs share an SM), four otherwise.
template <typename T, bool REAL, int TPR, int U, int K, int SB = 1>
__host__ __device__ constexpr int ws_stages() {
  // one-vector complex128 with two rows per thread: two 512-row stages, so two CTAs share an SM
  if (sizeof(T) == 8 && REAL && TPR == 1 && U == 2) return 2;
  return ((sizeof(T) == 8 && REAL && TPR == 1 && U == 1 && K == kWsFF) || SB > 1) ? 3 : kWsStages;
}

template <typename T, bool REAL, int TPR, int VPT, int U, int K, int SB = 1>
__global__ void __launch_bounds__(kWsThreads, (U == 1 ? ((sizeof(T) == 8 && REAL && (TPR >= 2 || K == kWsFF)) ? 3 : 2) : ((sizeof(T) == 8 && REAL) ? 2 : 1)))
    cheb_next_ws_kernel(const StepParams p) {
  using Raw = typename RawT<T, VPT>::type;
  using MV = typename MatV<T, REAL>::type;
  constexpr int R = TPR * VPT;
  constexpr int RPB = kBlock / TPR;
  constexpr int TILE = RPB * U;
  constexpr int STILE = TILE * SB;  // rows of one stage: SB sub-tiles of TILE rows
  constexpr bool F32 = std::is_same<T, float>::value;
  constexpr bool SER = K == kWsSeries;
  constexpr bool DBL = K == kWsDbl;
  constexpr int NST = ws_stages<T, REAL, TPR, U, K, SB>();
  constexpr int kFlush = 8;
  constexpr int kWarps = kBlock / 32;

  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[NST];
  __shared__ __align__(8) uint64_t empty[NST];
  __shared__ double2 red[kWarps * R];

  const int L = p.L;
  const uint32_t col_b = (uint32_t)align16((size_t)L * STILE * 4);
  const uint32_t val_b = (uint32_t)align16((size_t)L * STILE * sizeof(MV));
  const uint32_t vec_b = (uint32_t)(STILE * TPR * sizeof(Raw));
  const uint32_t stage_b = col_b + val_b + 2 * vec_b;

  const int ntiles = (int)(p.n_pad / STILE);
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
    for (int s = 0; s < NST; ++s) {
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
      tc.old = static_cast<const unsigned char*>(p.tprev ? p.tprev : p.tout);
      // a series step (no moments) stages the series accumulator in the left-vector slot
      tc.vl = static_cast<const unsigned char*>(SER ? p.series : p.vl);
      tc.vl2 = nullptr;
      // complex128: T_m's rows of each staged tile are prefetched into L2 (1.096 -> 1.063 ms per
      // default step at 2048^2, R = 8), where the tile's neighbour gathers find them; for the
      // complex64 steps no gain above the spread between GPUs was measured, so they go without
      tc.cur = sizeof(T) == 8 ? static_cast<const unsigned char*>(p.tcur) : nullptr;
      tc.ld = p.ld;
      tc.L = L;
      tc.col_slab = STILE * 4;
      tc.val_slab = (uint32_t)(STILE * sizeof(MV));
      tc.vec_slab = vec_b;
      tc.vl_slab = DBL ? (uint32_t)(STILE * R * sizeof(T)) : vec_b;
      if (DBL) tc.vl = static_cast<const unsigned char*>(p.hv);
      tc.col_b = col_b;
      tc.val_b = val_b;
      tc.tx_bytes = (uint32_t)L * STILE * 4 + (uint32_t)L * STILE * (uint32_t)sizeof(MV) + vec_b + (tc.vl ? tc.vl_slab : 0);
      int issued = 0;
      for (int k = 0; k < my_count; ++k) {
        const int st = k % NST;
        if (k >= NST && !mbar_wait_bounded(&empty[st], (uint32_t)(((k / NST) - 1) & 1), p.wait_budget)) {
          atomicExch(p.err, KPM_ERR_TIMEOUT);
          break;
        }
        fence_proxy_async_shared();
        if (k == 0 && p.withhold_first)  // test hook: the stage is armed, its copies never issued
          mbar_arrive_expect_tx(&full[st], tc.tx_bytes);
        else
          issue_tile(tc, smem + st * stage_b, &full[st], tile_of(k) * STILE, TPR * (int)sizeof(Raw), pol);
        issued = k + 1;
      }
      // copies of the last stages may still be landing: wait for them before leaving
      for (int q = issued > NST ? issued - NST : 0; q < issued; ++q)
        (void)mbar_wait_bounded(&full[q % NST], (uint32_t)((q / NST) & 1), p.wait_budget);
    }
    return;
  }

  int seg = per_tile ? p.seg_base[blockIdx.x] : 0;
  int cur_inst = (per_tile && my_count > 0) ? p.tile_inst[seg_tb] : 0;
  // float-float moment products (FP64 only, one moment set)
  constexpr bool FFM = K == kWsFF && !std::is_same<T, float>::value && VPT == 1;
  constexpr bool dbl = DBL;
  const bool mom = p.vl != nullptr || dbl;
  // series step: series += c_m T_{m+1} (rec_A_vec), the accumulator tile staged like v_l
  constexpr bool ser = SER;
  Raw* series = static_cast<Raw*>(p.series);
  const double2 cm = ser ? p.coef[p.m] : make_double2(0.0, 0.0);
  const int64_t set_stride = per_tile ? p.part_set_stride : (int64_t)gridDim.x * R;

  const Raw* __restrict__ tcur = static_cast<const Raw*>(p.tcur);
  Raw* tout = static_cast<Raw*>(p.tout);
  const int sub = threadIdx.x % TPR;
  const int rl = threadIdx.x / TPR;
  double mr[VPT], mi[VPT], mr2[VPT], mi2[VPT];
  T fr[VPT], fi[VPT], fr2[VPT];
#pragma unroll
  for (int q = 0; q < VPT; ++q) {
    mr[q] = mi[q] = mr2[q] = mi2[q] = 0.0;
    fr[q] = fi[q] = fr2[q] = T(0);
  }
  int pending = 0;
  bool dead = false;
  // FP64 recursion, float-float moment products
  const double2* __restrict__ vl64 = static_cast<const double2*>(p.vl64);
  FFMom fm{0.f, 0.f, 0.f, 0.f};
  int ffp = 0;
  auto fold = [&]() {
#pragma unroll
    for (int q = 0; q < VPT; ++q) {
      mr[q] += (double)fr[q];
      mi[q] += (double)fi[q];
      mr2[q] += (double)fr2[q];
      fr[q] = fi[q] = fr2[q] = T(0);
    }
  };
  auto flush_sets = [&](double2* dst) {
    if constexpr (FFM) {
      ff_fold(mr[0], mi[0], fm);
      ffp = 0;
    }
    block_reduce_store<TPR, VPT>(mr, mi, dst, red, true);
    if (dbl) block_reduce_store<TPR, VPT>(mr2, mi2, dst + set_stride, red, true);
#pragma unroll
    for (int q = 0; q < VPT; ++q) mr[q] = mi[q] = mr2[q] = 0.0;
  };

  // one iteration per sub-tile: stage k = it / SB, sub-tile sb = it % SB (the stage's wait
  // comes with its first sub-tile, its release with its last)
  for (int it = 0; it < my_count * SB; ++it) {
    const int k = it / SB, sb = it % SB;
    const int st = k % NST;
    bool ok = !dead;
    if (sb == 0) {
      ok = ok && mbar_wait_bounded(&full[st], (uint32_t)((k / NST) & 1), p.wait_budget);
      ok = __all_sync(0xffffffffu, ok);
      if (!ok && !dead) {
        if (lane == 0) atomicExch(p.err, KPM_ERR_TIMEOUT);
        dead = true;
      }
    }
    if (ok) {
      const unsigned char* base = smem + st * stage_b;
      const int32_t* scol = reinterpret_cast<const int32_t*>(base);
      const MV* sval = reinterpret_cast<const MV*>(base + col_b);
      const Raw* sold = reinterpret_cast<const Raw*>(base + col_b + val_b);
      const Raw* svl = reinterpret_cast<const Raw*>(base + col_b + val_b + vec_b);
      {
        const int rb = sb * TILE;  // this sub-tile's first row within the stage
        const int64_t row0 = tile_of(k) * STILE + rb;
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
                c[u][j] = scol[(s + j) * STILE + rb + u * RPB + rl];
                h[u][j] = sval[(s + j) * STILE + rb + u * RPB + rl];
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
              unpack(sold[(rb + u * RPB + rl) * TPR + sub], old);
              madd_first_neg(accum[u], h[u][0], x[u][0], old);
            } else {
              madd(accum[u], h[u][0], x[u][0]);
            }
#pragma unroll
            for (int j = 1; j < 4; ++j)
              if (s + j < L) madd(accum[u], h[u][j], x[u][j]);
          }
        }
        Cx<T, VPT> acc[U], l[U];
        T hvs[U][VPT];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          acc[u] = finish(accum[u]);
          if (dbl) {
            const T* shv = reinterpret_cast<const T*>(svl) + ((rb + u * RPB + rl) * TPR + sub) * VPT;
#pragma unroll
            for (int q = 0; q < VPT; ++q) hvs[u][q] = shv[q];
          } else if (mom || ser) {
            unpack(svl[(rb + u * RPB + rl) * TPR + sub], l[u]);
          }
        }
        // after its last sub-tile the stage is no longer read: hand it back to the producer
        if (sb == SB - 1) {
          __syncwarp();
          if (lane == 0) mbar_arrive(&empty[st]);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int64_t vi = (row0 + u * RPB + rl) * TPR + sub;
          tout[vi] = pack(acc[u]);
          if (ser) {
            Cx<T, VPT> o;
#pragma unroll
            for (int q = 0; q < VPT; ++q) {
              // y = c_m*x + 1*y, the expression of the grid-stride kernel (two nested FMAs)
              o.re[q] = fma((T)cm.x, acc[u].re[q], fma(-(T)cm.y, acc[u].im[q], l[u].re[q]));
              o.im[q] = fma((T)cm.x, acc[u].im[q], fma((T)cm.y, acc[u].re[q], l[u].im[q]));
            }
            series[vi] = pack(o);
            continue;
          }
          if (!mom) continue;
          if constexpr (FFM) {
            const FF lf = ff_from_slot(l[u].re[0], l[u].im[0]);
            FF tf;
            bool ok = ff_split_f64(acc[u].re[0], tf.rh, tf.rl);
            ok &= ff_split_f64(acc[u].im[0], tf.ih, tf.il);
            ok &= ff_left_ok(lf.rh) & ff_left_ok(lf.ih);
            if (ok) {
              ff_cdot(fm, lf, tf);
            } else {
              const double2 lv = __ldg(vl64 + vi);
              cdot_acc(mr[0], mi[0], lv.x, lv.y, acc[u].re[0], acc[u].im[0]);
            }
            if (++ffp == kFfFoldRows) {
              ffp = 0;
              ff_fold(mr[0], mi[0], fm);
            }
          } else if (dbl) {
            Cx<T, VPT> own;  // T_m at this row
            unpack(__ldg(tcur + vi), own);
#pragma unroll
            for (int q = 0; q < VPT; ++q) {
              if (F32) {
                cdot_acc(fr[q], fi[q], acc[u].re[q], acc[u].im[q], own.re[q], own.im[q]);
                fr2[q] += fmaf(own.re[q], own.re[q], fmaf(own.im[q], own.im[q], -hvs[u][q]));
              } else {
                cdot_acc(mr[q], mi[q], acc[u].re[q], acc[u].im[q], own.re[q], own.im[q]);
                mr2[q] += fma(own.re[q], own.re[q], fma(own.im[q], own.im[q], -hvs[u][q]));
              }
            }
          } else {
#pragma unroll
            for (int q = 0; q < VPT; ++q) {
              if (F32)
                cdot_acc(fr[q], fi[q], l[u].re[q], l[u].im[q], acc[u].re[q], acc[u].im[q]);
              else
                cdot_acc(mr[q], mi[q], l[u].re[q], l[u].im[q], acc[u].re[q], acc[u].im[q]);
            }
          }
          if (F32 && ++pending == kFlush) {
            pending = 0;
            fold();
          }
        }
      }
    }
    if (per_tile && mom && sb == SB - 1) {
      const int next_inst = (k + 1 < my_count) ? p.tile_inst[seg_tb + k + 1] : -1;
      if (next_inst != cur_inst) {
        if (F32) {
          fold();
          pending = 0;
        }
        flush_sets(p.part + (int64_t)seg * R);
        ++seg;
        cur_inst = next_inst;
      }
    }
  }

  if (!per_tile && mom) {
    if (F32) fold();
    flush_sets(p.part + (int64_t)blockIdx.x * R);
  }
}

template <typename T, bool REAL, int TPR, int VPT, int U, int K, int SB>
bool ws_smem_attr(size_t smem) {
  static size_t configured = 0;
  if (smem <= configured) return true;
  cudaError_t e = cudaFuncSetAttribute(cheb_next_ws_kernel<T, REAL, TPR, VPT, U, K, SB>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) {
    set_last_cuda_error(e);
    (void)cudaGetLastError();
    return false;
  }
  configured = smem;
  return true;
}

// Shared memory of one instantiation: its stage count times a stage of SB sub-tiles.
template <typename T, bool REAL, int TPR, int VPT, int U, int K, int SB>
size_t ws_smem_bytes(int L) {
  return ws_stages<T, REAL, TPR, U, K, SB>() * staged_stage_bytes<T, REAL, TPR, VPT, U * SB>(L, 2);
}

template <typename T, bool REAL, int TPR, int VPT, int U, int K, int SB>
bool ws_go(const StepParams& p, int grid, cudaStream_t s) {
  const size_t smem = ws_smem_bytes<T, REAL, TPR, VPT, U, K, SB>(p.L);
  if (!ws_smem_attr<T, REAL, TPR, VPT, U, K, SB>(smem)) return false;
  cheb_next_ws_kernel<T, REAL, TPR, VPT, U, K, SB><<<grid, kWsThreads, smem, s>>>(p);
  return true;
}

template <typename T, bool REAL, int TPR, int VPT, int U, int SB>
int launch_ws(const StepParams& p, int grid, cudaStream_t s) {
  bool ok;
  if (p.dbl) {
    ok = ws_go<T, REAL, TPR, VPT, U, kWsDbl, SB>(p, grid, s);
  } else if (p.series && !p.vl) {
    ok = ws_go<T, REAL, TPR, VPT, U, kWsSeries, SB>(p, grid, s);
  } else {
    bool ff = false;
    if constexpr (sizeof(T) == 8 && VPT == 1) ff = p.vl_ff && p.vl;
    if (ff) {
      if constexpr (sizeof(T) == 8 && VPT == 1) ok = ws_go<T, REAL, TPR, VPT, U, kWsFF, SB>(p, grid, s);
    } else {
      ok = ws_go<T, REAL, TPR, VPT, U, kWsMom, SB>(p, grid, s);
    }
  }
  if (!ok) return KPM_ERR_UNSUPPORTED;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_cuda_error(e);
    return KPM_ERR_CUDA;
  }
  return KPM_OK;
}

// CTAs of one SM for epilogue variant K
template <typename T, bool REAL, int TPR, int VPT, int U, int K, int SB>
int ws_ctas_per_sm_k(int L) {
  const size_t smem = ws_smem_bytes<T, REAL, TPR, VPT, U, K, SB>(L);
  if (smem > 200 * 1024) return 0;
  if (!ws_smem_attr<T, REAL, TPR, VPT, U, K, SB>(smem)) return 0;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, cheb_next_ws_kernel<T, REAL, TPR, VPT, U, K, SB>, kWsThreads,
                                                    smem) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return n;
}

// ff: the launches will be the float-float-products variant (its stage count and register
// bound can differ); otherwise the moment variant, whose bound the series and doubled
// variants share
template <typename T, bool REAL, int TPR, int VPT, int U, int SB>
int ws_ctas_per_sm(int L, bool ff) {
  if constexpr (sizeof(T) == 8 && VPT == 1) {
    if (ff) return ws_ctas_per_sm_k<T, REAL, TPR, VPT, U, kWsFF, SB>(L);
  }
  return ws_ctas_per_sm_k<T, REAL, TPR, VPT, U, kWsMom, SB>(L);
}

// Dispatch over (real, R, U, SB) for one precision (VPT as in the staged kernel).  SB = 2
// (two sub-tiles per stage) exists for complex128, U = 1 and plain operators (the batched
// per-tile tables count tiles of TILE rows).
template <typename T>
struct Ws {
  template <bool REAL, int R, int U, int SB>
  static int go(const StepParams& p, int grid, cudaStream_t s) {
    constexpr int VPT = (std::is_same<T, float>::value && R >= 2) ? 2 : 1;
    return launch_ws<T, REAL, R / VPT, VPT, U, SB>(p, grid, s);
  }
  template <bool REAL, int R, int U, int SB>
  static int occ(int L, bool ff) {
    constexpr int VPT = (std::is_same<T, float>::value && R >= 2) ? 2 : 1;
    return ws_ctas_per_sm<T, REAL, R / VPT, VPT, U, SB>(L, ff);
  }
  template <bool REAL, int R>
  static int go_u(int U, int SB, const StepParams& p, int grid, cudaStream_t s) {
    if constexpr (sizeof(T) == 8) {
      if (SB == 2 && U == 1) {
        if (p.per_tile) return KPM_ERR_UNSUPPORTED;
        return go<REAL, R, 1, 2>(p, grid, s);
      }
    }
    if (SB != 1) return KPM_ERR_UNSUPPORTED;
    return U == 2 ? go<REAL, R, 2, 1>(p, grid, s) : go<REAL, R, 1, 1>(p, grid, s);
  }
  template <bool REAL, int R>
  static int occ_u(int U, int SB, int L, bool ff) {
    if constexpr (sizeof(T) == 8) {
      if (SB == 2 && U == 1) return occ<REAL, R, 1, 2>(L, ff);
    }
    if (SB != 1) return 0;
    return U == 2 ? occ<REAL, R, 2, 1>(L, ff) : occ<REAL, R, 1, 1>(L, ff);
  }
  template <bool REAL>
  static int go_r(int R, int U, int SB, const StepParams& p, int grid, cudaStream_t s) {
    switch (R) {
      case 1: return go_u<REAL, 1>(U, SB, p, grid, s);
      case 2: return go_u<REAL, 2>(U, SB, p, grid, s);
      case 4: return go_u<REAL, 4>(U, SB, p, grid, s);
      case 8: return go_u<REAL, 8>(U, SB, p, grid, s);
      default: return KPM_ERR_UNSUPPORTED;
    }
  }
  template <bool REAL>
  static int occ_r(int R, int U, int SB, int L, bool ff) {
    switch (R) {
      case 1: return occ_u<REAL, 1>(U, SB, L, ff);
      case 2: return occ_u<REAL, 2>(U, SB, L, ff);
      case 4: return occ_u<REAL, 4>(U, SB, L, ff);
      case 8: return occ_u<REAL, 8>(U, SB, L, ff);
      default: return 0;
    }
  }
  static int launch(bool real, int R, int U, const StepParams& p, int grid, cudaStream_t s, int SB = 1) {
    return real ? go_r<true>(R, U, SB, p, grid, s) : go_r<false>(R, U, SB, p, grid, s);
  }
  static int ctas_per_sm(bool real, int R, int U, int L, bool ff = false, int SB = 1) {
    return real ? occ_r<true>(R, U, SB, L, ff) : occ_r<false>(R, U, SB, L, ff);
  }
};

}  // namespace kpm
