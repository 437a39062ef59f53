// kpm_mu_nm.cu -- the Kubo-Greenwood moment matrix on the tensor cores.
//
//   mu_nm = (1/R) sum_r <v_r | V T_n(H) V T_m(H) | v_r>,   n, m < Nm <= 256,
//
// computed as mu_nm = (1/R) sum_r L_n^H R_m with L_n = T_n(H) (V v) and
// R_m = V T_m(H) v (H and V Hermitian).  The recursions run in complex64 with the
// step kernels of this library, up to kMuGroup vectors at once, and store every
// L_n and R_m as a row of a [256][2 Rg n_pad] float matrix (the packed [n_pad][Rg]
// vector set, interleaved re, im): the contraction over a row sums over sites
// and the group's vectors alike.  It is one real GEMM per half of the n range,
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
#include <cuda.h>  // CUtensorMap and its enums; the encoder is looked up at run time (no libcuda link)

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>

#include "kpm_async.cuh"
#include "kpm_internal.cuh"
#include "kpm_tc.cuh"

namespace kpm {

constexpr int kTile = 128;                     // n rows and m rows of one output tile
constexpr int kKt = 16;                        // tf32 K elements per stage
constexpr int kGemmThreads = 512;                         // one A and one B chunk per thread per K tile
constexpr int kColsPerThread = 2 * kTile * kTile / kGemmThreads;  // 64 accumulator columns of one TMEM lane
constexpr uint32_t kLBO = 128;                 // bytes between K-adjacent core matrices
constexpr uint32_t kSBO = (kKt / 4) * 128;     // bytes between 8-row groups (512)
constexpr uint32_t kTileA = kTile * kKt * 4;   // 8 KB: 128 rows x 16 floats
constexpr uint32_t kTileBX = 2 * kTileA;       // 16 KB: 128 B rows, then the same rows swapped
constexpr uint32_t kStageBytes = 2 * kTileA + 2 * kTileBX;  // Ahi Alo BXhi BXlo = 48 KB
constexpr int kGemmStages = 3;
constexpr uint32_t kGemmSmem = kGemmStages * kStageBytes;  // 144 KB
constexpr uint32_t kTmemCols = 512;            // two accumulator buffers of 256 columns (Re | Im)
constexpr int kChainTiles = 2;                 // K tiles per TMEM accumulation chain (32 floats)
constexpr int kLevel1Chains = 64;              // chains summed in registers before a global flush
constexpr int kMuGroup = 4;                    // vectors per recursion group of kpm_mu_nm
constexpr int kTileElems = kTile * kTile;

struct GemmParams {
  const float* A;   // [256][lda]
  const float* B;   // [256][lda]
  int64_t lda;      // floats per row
  int64_t K;        // floats of K to contract (multiple of kKt)
  int64_t k_per_cta;
  int mt;           // m tiles (output tile index = n_tile * mt + m_tile)
  float* part_hi;   // [KS][tiles][Re, Im][128 m][128 n]: float-float partial sums
  float* part_lo;
  int* err;
};

// Byte offset of the 16-byte chunk (row r, k-chunk kc) in a canonical no-swizzle K-major tile.
__device__ __forceinline__ uint32_t chunk_off(int r, int kc) {
  return (uint32_t)(r >> 3) * kSBO + (uint32_t)kc * kLBO + (uint32_t)(r & 7) * 16;
}

// Operand layouts of a 16-float K tile.  SW = false: the canonical no-swizzle K-major layout
// above (core matrices of 8 rows x 16 B, LBO 128 B, SBO 512 B); the tensor core fetches the
// 8-row groups of one MMA at 512-byte strides, all on the same shared-memory banks.
// SW = true: the 64-byte-swizzled K-major layout: row r is 64 contiguous bytes at r * 64 with
// its 16-byte chunk kc stored at chunk kc ^ ((r >> 1) & 3) (address bits [4,6) XOR bits
// [7,9), the pattern repeating every 512 bytes = 8 rows), SBO 512 B; the chunks an MMA
// fetches then spread over all banks.  The K = 8 step j of an MMA starts 32 j bytes in.
template <bool SW>
__device__ __forceinline__ uint32_t tile_off(int r, int kc) {
  if constexpr (SW) return (uint32_t)r * 64u + ((uint32_t)(kc ^ ((r >> 1) & 3)) << 4);
  return chunk_off(r, kc);
}
template <bool SW>
__device__ __forceinline__ uint64_t operand_desc(uint32_t saddr) {
  if constexpr (SW) return smem_desc(saddr, 16, 512) | ((uint64_t)4 << 61);  // swizzle mode 4: 64 B
  return smem_desc(saddr, kLBO, kSBO);
}
template <bool SW>
__device__ __forceinline__ uint32_t kstep_off(int j) {
  return SW ? (uint32_t)j * 32u : (uint32_t)j * 2u * kLBO;
}

// The 16-byte chunk a thread moves: chunk c (0..511) of a 128-row x 16-float tile
// is row ((c >> 5) << 3 | (c & 7)), k-chunk ((c >> 3) & 3), so the eight threads of
// a shared-memory store phase write one 128-byte core-matrix column (no bank
// conflicts) and a warp still reads whole 32-byte sectors of 8 rows.
__device__ __forceinline__ int chunk_row(int c) { return ((c >> 5) << 3) | (c & 7); }
__device__ __forceinline__ int chunk_kc(int c) { return (c >> 3) & 3; }

__device__ __forceinline__ float4 tf32x4(float4 x) {
  return make_float4(to_tf32(x.x), to_tf32(x.y), to_tf32(x.z), to_tf32(x.w));
}
// The TMA-fed kernels round with integer operations (two per element instead of the
// compiler's sequence for cvt.rna.tf32); the thread-loaded kernel keeps cvt.rna, so the
// bit-for-bit agreement of the two forms also checks the rounding.
__device__ __forceinline__ float4 tf32x4_int(float4 x) {
  return make_float4(to_tf32_int(x.x), to_tf32_int(x.y), to_tf32_int(x.z), to_tf32_int(x.w));
}

// One thread's split of a raw A chunk and a raw B chunk of a K tile into the stage: hi and lo
// of A, and of B both as it is (rows 0..127 of BX) and pairwise swapped with the new
// imaginary part negated (rows 128..255).
__device__ __forceinline__ void split_chunks(const unsigned char* rw, unsigned char* stage, uint32_t off,
                                             uint32_t offs) {
  {
    const float4 x = *reinterpret_cast<const float4*>(rw + off);
    const float4 hi = tf32x4_int(x);
    const float4 lo = tf32x4_int(make_float4(x.x - hi.x, x.y - hi.y, x.z - hi.z, x.w - hi.w));
    *reinterpret_cast<float4*>(stage + off) = hi;
    *reinterpret_cast<float4*>(stage + kTileA + off) = lo;
  }
  {
    const float4 x = *reinterpret_cast<const float4*>(rw + kTileA + off);
    const float4 hi = tf32x4_int(x);
    const float4 lo = tf32x4_int(make_float4(x.x - hi.x, x.y - hi.y, x.z - hi.z, x.w - hi.w));
    unsigned char* bx = stage + 2 * kTileA;
    *reinterpret_cast<float4*>(bx + off) = hi;
    *reinterpret_cast<float4*>(bx + kTileBX + off) = lo;
    *reinterpret_cast<float4*>(bx + offs) = make_float4(hi.y, -hi.x, hi.w, -hi.z);
    *reinterpret_cast<float4*>(bx + kTileBX + offs) = make_float4(lo.y, -lo.x, lo.w, -lo.z);
  }
}

// Adds chain buffer columns [base, base + kColsPerThread) of this thread's TMEM lane into
// run[] with packed pairwise adds (one 16-column load per wait: a second one in flight
// would spill at this kernel's 128 registers).
__device__ __forceinline__ void fold_tmem(uint32_t base, float (&run)[kColsPerThread]) {
#pragma unroll
  for (int g = 0; g < kColsPerThread / 16; ++g) {
    uint32_t a[16];
    tmem_ld16_nowait(base + (uint32_t)(g * 16), a);
    tmem_wait_ld();
#pragma unroll
    for (int i = 0; i < 16; i += 2)
      add_f32x2(run[g * 16 + i], run[g * 16 + i + 1], __uint_as_float(a[i]), __uint_as_float(a[i + 1]));
  }
}

// Adds a thread's level-1 sums run[] (one TMEM lane, kColsPerThread columns; column c at
// ohi[c * kTile]) into its float-float partial (TwoSum into hi, the rounding error into lo)
// and restarts them.  The columns go in batches of kFlushBatch whose loads are all issued
// before any of the batch's stores: one store may alias a later column's load as far as the
// compiler knows, so column-by-column code waits a full global round trip per column
// (64 per flush, about a quarter of the contraction time at the Kubo size).
constexpr int kFlushBatch = 8;
__device__ __forceinline__ void flush_partials(float (&run)[kColsPerThread], float* ohi, float* olo, bool first) {
#pragma unroll
  for (int c0 = 0; c0 < kColsPerThread; c0 += kFlushBatch) {
    if (first) {
#pragma unroll
      for (int i = 0; i < kFlushBatch; ++i) {
        ohi[(c0 + i) * kTile] = run[c0 + i];
        olo[(c0 + i) * kTile] = 0.f;
      }
    } else {
      float a[kFlushBatch], l[kFlushBatch];
#pragma unroll
      for (int i = 0; i < kFlushBatch; ++i) {
        a[i] = ohi[(c0 + i) * kTile];
        l[i] = olo[(c0 + i) * kTile];
      }
#pragma unroll
      for (int i = 0; i < kFlushBatch; ++i) {
        const float b = run[c0 + i];
        const float s = __fadd_rn(a[i], b);
        const float bp = __fsub_rn(s, a[i]);
        const float e = __fadd_rn(__fsub_rn(a[i], __fsub_rn(s, bp)), __fsub_rn(b, bp));
        ohi[(c0 + i) * kTile] = s;
        olo[(c0 + i) * kTile] = __fadd_rn(l[i], e);
      }
    }
#pragma unroll
    for (int i = 0; i < kFlushBatch; ++i) run[c0 + i] = 0.f;
  }
}

// One CTA: output tile (n0.., m0..) of 128 x 128, Re and Im side by side as one
// M = 128, N = 256 MMA against BX = [B rows; B rows with (re, im) -> (im, -re)],
// over its K range.  The MMA accumulator is restarted every kChainTiles K tiles,
// alternating between two TMEM buffers: while one chain runs, the threads fold
// the previous one into FP32 register sums (every thread owns one TMEM lane and
// kColsPerThread columns), and every kLevel1Chains chains those sums go into a float-float
// (hi, lo) partial in global memory.  The tensor core's FP32 accumulation thus
// never runs longer than 3 * 2 * kChainTiles MMAs.
template <bool SW>
__global__ void __launch_bounds__(kGemmThreads, 1) mu_gemm_kernel(const GemmParams p) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t bars[kGemmStages];
  __shared__ __align__(8) uint64_t accbar[2];
  __shared__ uint32_t tmem_slot;

  const int tile = blockIdx.x;
  const int n0 = (tile / p.mt) * kTile, m0 = (tile % p.mt) * kTile;
  const int64_t k_begin = (int64_t)blockIdx.y * p.k_per_cta;
  const int64_t k_end = min(p.K, k_begin + p.k_per_cta);
  const int k_tiles = k_end > k_begin ? (int)((k_end - k_begin) / kKt) : 0;
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  // TMEM lane quarter (warp % 4) and this thread's block of accumulator columns:
  // buffer columns cb .. cb + kColsPerThread - 1 (Re: 0..127, Im: 128..255)
  const int q = warp & 3;
  const int cb = (warp >> 2) * kColsPerThread;
  const int half = cb / kTile;
  const int row = 32 * q + lane;
  const int64_t obase = (((int64_t)blockIdx.y * gridDim.x + tile) * 2 + half) * kTileElems +
                        (int64_t)(cb % kTile) * kTile + row;
  float* ohi = p.part_hi + obase;  // element (column cb + c) at ohi[c * kTile]
  float* olo = p.part_lo + obase;

  if (k_tiles == 0) {  // nothing to contract: a zero partial
    for (int c = 0; c < kColsPerThread; ++c) {
      ohi[c * kTile] = 0.f;
      olo[c * kTile] = 0.f;
    }
    return;
  }
  if (tid == 0) {
    for (int s = 0; s < kGemmStages; ++s) mbar_init(&bars[s], 1);
    mbar_init(&accbar[0], 1);
    mbar_init(&accbar[1], 1);
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
  const uint32_t idesc = idesc_tf32(kTile, 2 * kTile);

  float run[kColsPerThread];  // level-1 sums of this thread's lane and columns
#pragma unroll
  for (int i = 0; i < kColsPerThread; ++i) run[i] = 0.f;
  bool first_flush = true;
  int chains_in_l1 = 0;

  // fold chain c (TMEM buffer c & 1) into run[]; false if its commit never came
  auto fold_chain = [&](int c) -> bool {
    bool ok = mbar_wait_bounded(&accbar[c & 1], (uint32_t)((c >> 1) & 1));
    ok = __all_sync(0xffffffffu, ok);
    if (!ok) return false;
    tc_fence_after();
    const uint32_t base = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)((c & 1) * 256 + cb);
#pragma unroll
    for (int g = 0; g < kColsPerThread / 16; ++g) {
      float v[16];
      tmem_ld16(base + (uint32_t)(g * 16), v);
#pragma unroll
      for (int i = 0; i < 16; ++i) run[g * 16 + i] = __fadd_rn(run[g * 16 + i], v[i]);
    }
    return true;
  };
  // level-1 sums into the float-float partial (TwoSum), then restart them
  auto flush_l2 = [&]() {
    flush_partials(run, ohi, olo, first_flush);
    first_flush = false;
  };

  // this thread's 16-byte chunks of one K tile: chunk tid of the A rows and of the B rows
  struct RawTile {
    float4 a, b;
  };
  const int crow = chunk_row(tid), ckc = chunk_kc(tid);
  const uint32_t off = tile_off<SW>(crow, ckc);
  const uint32_t offs = tile_off<SW>(kTile + crow, ckc);
  const float* pa = p.A + (int64_t)(n0 + crow) * p.lda + k_begin + 4 * ckc;
  const float* pb = p.B + (int64_t)(m0 + crow) * p.lda + k_begin + 4 * ckc;
  auto load_tile = [&](int t, RawTile& r) {
    r.a = __ldcs(reinterpret_cast<const float4*>(pa + (int64_t)t * kKt));
    r.b = __ldcs(reinterpret_cast<const float4*>(pb + (int64_t)t * kKt));
  };
  int issued = 0;  // K tiles whose MMAs thread 0 has issued
  // one K tile: fold a finished chain when a new one starts, split r into the stage,
  // prefetch tile t + 2 into r, then thread 0 issues the tile's MMAs
  auto body = [&](int t, RawTile& r) -> bool {
    const int st = t % kGemmStages;
    const int c = t / kChainTiles;
    bool good = true;
    if (t % kChainTiles == 0 && c >= 2) {  // chain c - 2 used the buffer chain c starts
      good = fold_chain(c - 2);
      if (good && ++chains_in_l1 == kLevel1Chains) {
        flush_l2();
        chains_in_l1 = 0;
      }
    }
    if (good && t >= kGemmStages)
      good = mbar_wait_bounded(&bars[st], (uint32_t)(((t - kGemmStages) / kGemmStages) & 1));
    if (good) {
      unsigned char* stage = smem + (size_t)st * kStageBytes;
      {
        const float4 x = r.a;
        const float4 hi = tf32x4(x);
        const float4 lo = tf32x4(make_float4(x.x - hi.x, x.y - hi.y, x.z - hi.z, x.w - hi.w));
        *reinterpret_cast<float4*>(stage + off) = hi;
        *reinterpret_cast<float4*>(stage + kTileA + off) = lo;
      }
      {
        const float4 x = r.b;
        const float4 hi = tf32x4(x);
        const float4 lo = tf32x4(make_float4(x.x - hi.x, x.y - hi.y, x.z - hi.z, x.w - hi.w));
        unsigned char* bx = stage + 2 * kTileA;
        *reinterpret_cast<float4*>(bx + off) = hi;
        *reinterpret_cast<float4*>(bx + kTileBX + off) = lo;
        *reinterpret_cast<float4*>(bx + offs) = make_float4(hi.y, -hi.x, hi.w, -hi.z);
        *reinterpret_cast<float4*>(bx + kTileBX + offs) = make_float4(lo.y, -lo.x, lo.w, -lo.z);
      }
    }
    if (t + 2 < k_tiles) load_tile(t + 2, r);
    fence_proxy_async_shared();
    tc_fence_before();
    if (__syncthreads_or(!good)) return false;
    if (tid == 0) {
      tc_fence_after();
      const uint32_t s0 = smem_base + (uint32_t)st * kStageBytes;
      const uint32_t d = tmem + (uint32_t)((c & 1) * 256);
#pragma unroll
      for (int j = 0; j < kKt / 8; ++j) {
        const uint32_t kofs = kstep_off<SW>(j);
        const uint64_t a_hi = operand_desc<SW>(s0 + kofs);
        const uint64_t a_lo = operand_desc<SW>(s0 + kTileA + kofs);
        const uint64_t bx_hi = operand_desc<SW>(s0 + 2 * kTileA + kofs);
        const uint64_t bx_lo = operand_desc<SW>(s0 + 2 * kTileA + kTileBX + kofs);
        mma_tf32(d, a_hi, bx_hi, idesc, (t % kChainTiles) != 0 || j > 0);
        mma_tf32(d, a_hi, bx_lo, idesc, true);
        mma_tf32(d, a_lo, bx_hi, idesc, true);
      }
      mma_commit(&bars[st]);
      if ((t + 1) % kChainTiles == 0 || t + 1 == k_tiles) mma_commit(&accbar[c & 1]);
      issued = t + 1;
    }
    return true;
  };

  RawTile r0, r1;
  load_tile(0, r0);
  if (k_tiles > 1) load_tile(1, r1);
  bool ok = true;
  for (int t = 0; t < k_tiles && ok; t += 2) {
    ok = body(t, r0);
    if (ok && t + 1 < k_tiles) ok = body(t + 1, r1);
  }
  if (ok) {  // the last one or two chains
    const int nchains = (k_tiles + kChainTiles - 1) / kChainTiles;
    bool good = true;
    for (int c = max(0, nchains - 2); c < nchains && good; ++c) good = fold_chain(c);
    ok = !__syncthreads_or(!good);
  }
  if (!ok) {
    if (tid == 0) {
      atomicExch(p.err, KPM_ERR_TIMEOUT);
      // the last commit tracks every MMA issued: wait (bounded) before the accumulator is released
      if (issued > 0)
        (void)mbar_wait_bounded(&bars[(issued - 1) % kGemmStages], (uint32_t)(((issued - 1) / kGemmStages) & 1));
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, kTmemCols);
    return;
  }
  flush_l2();
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, kTmemCols);
}

// ---- the same contraction with its operand tiles brought in by the TMA engine -----------
// mu_gemm_kernel's threads load every K tile from global memory themselves (two tiles
// ahead in registers) and meet at a CTA barrier per tile, so the loop waits on those loads.
// Here one thread issues cp.async.bulk.tensor copies kRawStages tiles ahead into a ring of
// raw stages, and the threads only split a tile that has landed.  The 4-D tensor map
// (4 floats x 8 rows x K chunks of 16 bytes x 8-row groups; strides 4 B, one row, 16 B,
// 8 rows) makes each copy land in the MMA's canonical no-swizzle K-major layout (core
// matrices of 8 rows x 16 bytes, LBO 128 B, SBO 512 B), so a thread reads its raw chunk and
// writes its hi / lo / swapped chunks at the same offsets, free of bank conflicts.
// Accumulation, chains, folds and partials are those of mu_gemm_kernel.
constexpr int kRawStages = 4;
static_assert((kRawStages & (kRawStages - 1)) == 0, "the raw ring index wraps with a mask");
constexpr uint32_t kRawBytes = 2 * kTileA;                    // raw A and B tiles, 16 KB
constexpr uint32_t kTmaSmem = kRawStages * kRawBytes + kGemmStages * kStageBytes;  // 208 KB

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int c0, int c1, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
          "r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
      "%5}], [%6];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(bar))
      : "memory");
}

template <bool SW>
__global__ void __launch_bounds__(kGemmThreads, 1)
    mu_gemm_tma_kernel(const GemmParams p, const __grid_constant__ CUtensorMap map_a,
                       const __grid_constant__ CUtensorMap map_b) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t bars[kGemmStages];
  __shared__ __align__(8) uint64_t rawbar[kRawStages];
  __shared__ __align__(8) uint64_t accbar[2];
  __shared__ uint32_t tmem_slot;

  const int tile = blockIdx.x;
  const int n0 = (tile / p.mt) * kTile, m0 = (tile % p.mt) * kTile;
  const int64_t k_begin = (int64_t)blockIdx.y * p.k_per_cta;
  const int64_t k_end = min(p.K, k_begin + p.k_per_cta);
  const int k_tiles = k_end > k_begin ? (int)((k_end - k_begin) / kKt) : 0;
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int q = warp & 3;
  const int cb = (warp >> 2) * kColsPerThread;
  const int half = cb / kTile;
  const int row = 32 * q + lane;
  const int64_t obase = (((int64_t)blockIdx.y * gridDim.x + tile) * 2 + half) * kTileElems +
                        (int64_t)(cb % kTile) * kTile + row;
  float* ohi = p.part_hi + obase;
  float* olo = p.part_lo + obase;

  if (k_tiles == 0) {
    for (int c = 0; c < kColsPerThread; ++c) {
      ohi[c * kTile] = 0.f;
      olo[c * kTile] = 0.f;
    }
    return;
  }
  unsigned char* raw = smem;                                  // kRawStages x [A raw | B raw]
  unsigned char* split = smem + kRawStages * kRawBytes;       // kGemmStages x [Ahi Alo BXhi BXlo]
  if (tid == 0) {
    for (int s = 0; s < kGemmStages; ++s) mbar_init(&bars[s], 1);
    for (int s = 0; s < kRawStages; ++s) mbar_init(&rawbar[s], 1);
    mbar_init(&accbar[0], 1);
    mbar_init(&accbar[1], 1);
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
  const uint32_t split_base = static_cast<uint32_t>(__cvta_generic_to_shared(split));
  const uint32_t idesc = idesc_tf32(kTile, 2 * kTile);
  // raw tile t: A rows n0.., B rows m0.., K floats k_begin + 16 t ..
  const int kc0 = (int)(k_begin / 4);
  auto issue_raw = [&](int t) {
    const int rs = t % kRawStages;
    mbar_arrive_expect_tx(&rawbar[rs], kRawBytes);
    if constexpr (SW) {
      tma_load_2d(raw + (size_t)rs * kRawBytes, &map_a, 4 * kc0 + t * kKt, n0, &rawbar[rs]);
      tma_load_2d(raw + (size_t)rs * kRawBytes + kTileA, &map_b, 4 * kc0 + t * kKt, m0, &rawbar[rs]);
    } else {
      tma_load_4d(raw + (size_t)rs * kRawBytes, &map_a, 0, 0, kc0 + t * (kKt / 4), n0 / 8, &rawbar[rs]);
      tma_load_4d(raw + (size_t)rs * kRawBytes + kTileA, &map_b, 0, 0, kc0 + t * (kKt / 4), m0 / 8, &rawbar[rs]);
    }
  };
  int raw_issued = 0;  // thread 0: raw tiles whose copies were issued
  if (tid == 0) {
    for (; raw_issued < kRawStages && raw_issued < k_tiles; ++raw_issued) issue_raw(raw_issued);
  }

  float run[kColsPerThread];
#pragma unroll
  for (int i = 0; i < kColsPerThread; ++i) run[i] = 0.f;
  bool first_flush = true;
  int chains_in_l1 = 0;

  auto fold_chain = [&](int c) -> bool {
    bool ok = mbar_wait_bounded(&accbar[c & 1], (uint32_t)((c >> 1) & 1));
    ok = __all_sync(0xffffffffu, ok);
    if (!ok) return false;
    tc_fence_after();
    fold_tmem(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)((c & 1) * 256 + cb), run);
    return true;
  };
  auto flush_l2 = [&]() {
    flush_partials(run, ohi, olo, first_flush);
    first_flush = false;
  };

  const int crow = chunk_row(tid), ckc = chunk_kc(tid);
  const uint32_t off = tile_off<SW>(crow, ckc);
  const uint32_t offs = tile_off<SW>(kTile + crow, ckc);
  int issued = 0;  // K tiles whose MMAs thread 0 has issued
  int t = 0;
  bool ok = true;
  // the split stage of tile t and the parity of its next wait advance with t (no division by
  // three in the loop): bit s of sph is the parity of the next wait on split stage s; the raw
  // ring has a power-of-two length
  int st = 0;
  uint32_t sph = 0;
  for (; t < k_tiles && ok; ++t) {
    const int rs = t & (kRawStages - 1);
    const int c = t / kChainTiles;
    bool good = true;
    if (t % kChainTiles == 0 && c >= 2) {
      good = fold_chain(c - 2);
      if (good && ++chains_in_l1 == kLevel1Chains) {
        flush_l2();
        chains_in_l1 = 0;
      }
    }
    if (good && t >= kGemmStages) {
      good = mbar_wait_bounded(&bars[st], (sph >> st) & 1u);
      sph ^= 1u << st;
    }
    if (good) good = mbar_wait_bounded(&rawbar[rs], (uint32_t)(t / kRawStages) & 1u);
    if (good) split_chunks(raw + (size_t)rs * kRawBytes, split + (size_t)st * kStageBytes, off, offs);
    fence_proxy_async_shared();
    tc_fence_before();
    if (__syncthreads_or(!good)) {
      ok = false;
      break;
    }
    if (tid == 0) {
      tc_fence_after();
      const uint32_t s0 = split_base + (uint32_t)st * kStageBytes;
      const uint32_t d = tmem + (uint32_t)((c & 1) * 256);
#pragma unroll
      for (int j = 0; j < kKt / 8; ++j) {
        const uint32_t kofs = kstep_off<SW>(j);
        const uint64_t a_hi = operand_desc<SW>(s0 + kofs);
        const uint64_t a_lo = operand_desc<SW>(s0 + kTileA + kofs);
        const uint64_t bx_hi = operand_desc<SW>(s0 + 2 * kTileA + kofs);
        const uint64_t bx_lo = operand_desc<SW>(s0 + 2 * kTileA + kTileBX + kofs);
        mma_tf32(d, a_hi, bx_hi, idesc, (t % kChainTiles) != 0 || j > 0);
        mma_tf32(d, a_hi, bx_lo, idesc, true);
        mma_tf32(d, a_lo, bx_hi, idesc, true);
      }
      mma_commit(&bars[st]);
      if ((t + 1) % kChainTiles == 0 || t + 1 == k_tiles) mma_commit(&accbar[c & 1]);
      issued = t + 1;
      // every thread has read raw stage rs (the barrier above): refill it with tile t + kRawStages
      if (raw_issued < k_tiles) {
        fence_proxy_async_shared();
        issue_raw(raw_issued);
        ++raw_issued;
      }
    }
    st = st == kGemmStages - 1 ? 0 : st + 1;
  }
  if (ok) {
    const int nchains = (k_tiles + kChainTiles - 1) / kChainTiles;
    bool good = true;
    for (int c = max(0, nchains - 2); c < nchains && good; ++c) good = fold_chain(c);
    ok = !__syncthreads_or(!good);
  }
  if (!ok) {
    if (tid == 0) {
      atomicExch(p.err, KPM_ERR_TIMEOUT);
      if (issued > 0)
        (void)mbar_wait_bounded(&bars[(issued - 1) % kGemmStages], (uint32_t)(((issued - 1) / kGemmStages) & 1));
      // raw copies issued but not yet read: wait (bounded) for them to land before the CTA leaves
      for (int r = t; r < raw_issued; ++r) (void)mbar_wait_bounded(&rawbar[r % kRawStages], (uint32_t)((r / kRawStages) & 1));
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, kTmemCols);
    return;
  }
  flush_l2();
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, kTmemCols);
}

// cuTensorMapEncodeTiled from the driver, looked up once (nullptr if unavailable).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = []() -> EncodeTiledFn {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      (void)cudaGetLastError();
      return nullptr;
    }
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}

// The 64-byte-swizzled operand map of a [rows][lda] float matrix: dims (lda floats, rows), box
// (16 floats, 128 rows): one K tile lands as 128 rows of 64 bytes in the swizzled layout.
static bool operand_map_sw(CUtensorMap* m, const float* base, int64_t lda, int rows) {
  const EncodeTiledFn enc = encode_tiled();
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)lda, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)lda * 4};
  const cuuint32_t box[2] = {(cuuint32_t)kKt, (cuuint32_t)kTile};
  const cuuint32_t estr[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The operand map of a [rows][lda] float matrix (rows a multiple of 128): dims (4 floats, 8 rows,
// lda / 4 chunks, rows / 8 groups), box (4, 8, kKt / 4, 16) = one 128-row x 16-float tile in the
// canonical layout.
static bool operand_map(CUtensorMap* m, const float* base, int64_t lda, int rows) {
  const EncodeTiledFn enc = encode_tiled();
  if (!enc) return false;
  const cuuint64_t dims[4] = {4, 8, (cuuint64_t)(lda / 4), (cuuint64_t)(rows / 8)};
  const cuuint64_t strides[3] = {(cuuint64_t)lda * 4, 16, (cuuint64_t)lda * 4 * 8};
  const cuuint32_t box[4] = {4, 8, (cuuint32_t)(kKt / 4), (cuuint32_t)(kTile / 8)};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float*>(base), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// mu[n][m] = (accumulate ? mu : 0) + scale * sum_ks (hi + lo), Re and Im, in FP64.
__global__ void mu_reduce_kernel(const float* __restrict__ hi, const float* __restrict__ lo, int KS, int tiles,
                                 int mt, int Nm, double scale, int accumulate, double2* __restrict__ mu) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= Nm * Nm) return;
  const int n = idx / Nm, m = idx % Nm;
  const int tile = (n / kTile) * mt + (m / kTile);
  const int64_t off = (int64_t)(m % kTile) * kTile + (n % kTile);
  double re = 0.0, im = 0.0;
  for (int ks = 0; ks < KS; ++ks) {
    const int64_t b = ((int64_t)ks * tiles + tile) * 2 * kTileElems + off;
    re += (double)hi[b] + (double)lo[b];
    im += (double)hi[b + kTileElems] + (double)lo[b + kTileElems];
  }
  double2 o = make_double2(scale * re, scale * im);
  if (accumulate) {
    o.x += mu[idx].x;
    o.y += mu[idx].y;
  }
  mu[idx] = o;
}

int mu_tiles(int Nm) {
  const int t = (Nm + kTile - 1) / kTile;
  return t * t;
}

int contract_splits(int64_t K, int sm_count, int tiles) {
  int64_t ks = std::max<int64_t>(1, sm_count / tiles);
  ks = std::min<int64_t>(ks, K / kKt);
  return (int)std::max<int64_t>(1, ks);
}

// Floats of the partial buffer (hi and lo planes).
size_t contract_part_floats(int KS, int tiles) { return (size_t)2 * KS * tiles * 2 * kTileElems; }

// the last contraction's kernel (kpm_mu_gemm_path): bit 0 TMA loads, bit 1 swizzled layout
static int g_last_gemm_tma = -1;

int mu_contract(const float* A, const float* B, int64_t K, int64_t lda, int Nm, double scale, int accumulate,
                double2* mu, float* part, int KS, int* err, cudaStream_t s) {
  const int mt = (Nm + kTile - 1) / kTile;
  const int tiles = mt * mt;
  GemmParams g;
  g.A = A;
  g.B = B;
  g.lda = lda;
  g.K = K;
  g.k_per_cta = ((K / KS + kKt - 1) / kKt) * kKt;
  if (g.k_per_cta < kKt) g.k_per_cta = kKt;
  g.mt = mt;
  g.part_hi = part;
  g.part_lo = part + (size_t)KS * tiles * 2 * kTileElems;
  g.err = err;
  // kernel: operand tiles loaded by the threads ("legacy") or by the TMA engine ("tma"), in the
  // 64-byte-swizzled layout or the no-swizzle one ("_plain"); KPM_MU_GEMM picks one.  The
  // default is the TMA engine into the no-swizzle layout (the fastest measured; the threads'
  // loads take it when the tensor-map encoder is unavailable)
  const char* force = getenv("KPM_MU_GEMM");
  const std::string f = force ? force : "";
  const bool want_tma = !(f == "legacy" || f == "legacy_plain");
  const bool sw = f == "legacy" || f == "tma";
  CUtensorMap ma, mb;
  bool tma = false;
  if (want_tma)
    tma = sw ? (operand_map_sw(&ma, A, lda, mt * kTile) && operand_map_sw(&mb, B, lda, mt * kTile))
             : (operand_map(&ma, A, lda, mt * kTile) && operand_map(&mb, B, lda, mt * kTile));
  g_last_gemm_tma = (tma ? 1 : 0) + (sw ? 2 : 0);
  static bool attr[4] = {false, false, false, false};
  const int which = g_last_gemm_tma;
  if (!attr[which]) {
    const void* fn = tma ? (sw ? (const void*)mu_gemm_tma_kernel<true> : (const void*)mu_gemm_tma_kernel<false>)
                         : (sw ? (const void*)mu_gemm_kernel<true> : (const void*)mu_gemm_kernel<false>);
    KPM_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(tma ? kTmaSmem : kGemmSmem)));
    attr[which] = true;
  }
  if (tma && sw)
    mu_gemm_tma_kernel<true><<<dim3(tiles, KS), kGemmThreads, kTmaSmem, s>>>(g, ma, mb);
  else if (tma)
    mu_gemm_tma_kernel<false><<<dim3(tiles, KS), kGemmThreads, kTmaSmem, s>>>(g, ma, mb);
  else if (sw)
    mu_gemm_kernel<true><<<dim3(tiles, KS), kGemmThreads, kGemmSmem, s>>>(g);
  else
    mu_gemm_kernel<false><<<dim3(tiles, KS), kGemmThreads, kGemmSmem, s>>>(g);
  KPM_CUDA_TRY(cudaGetLastError());
  mu_reduce_kernel<<<(Nm * Nm + 255) / 256, 256, 0, s>>>(g.part_hi, g.part_lo, KS, tiles, mt, Nm, scale, accumulate,
                                                         mu);
  KPM_CUDA_TRY(cudaGetLastError());
  return KPM_OK;
}

}  // namespace kpm

using namespace kpm;

extern "C" {

int kpm_mu_gemm_path(void) { return g_last_gemm_tma; }

int kpm_mu_contract(const float* L, const float* R, int64_t k_floats, int64_t ld, int Nm, double scale,
                    int accumulate, double* mu, void* stream) {
  if (!L || !R || !mu || Nm < 1 || Nm > 256 || k_floats < kKt || ld < k_floats) return KPM_ERR_INVALID_ARG;
  if (k_floats % kKt != 0 || ld % 4 != 0) return KPM_ERR_SHAPE;
  if ((reinterpret_cast<uintptr_t>(L) | reinterpret_cast<uintptr_t>(R)) & 15) return KPM_ERR_INVALID_ARG;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int dev = 0, sms = 0;
  KPM_CUDA_TRY(cudaGetDevice(&dev));
  KPM_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int KS = contract_splits(k_floats, sms, mu_tiles(Nm));
  float* part = nullptr;
  int* err = nullptr;
  KPM_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&part), contract_part_floats(KS, mu_tiles(Nm)) * sizeof(float), s));
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

// Sets *flag when two [count] column arrays differ anywhere.
__global__ void cols_differ_kernel(const int32_t* __restrict__ a, const int32_t* __restrict__ b, int64_t count,
                                   unsigned* flag) {
  unsigned d = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
    d |= (a[i] != b[i]) ? 1u : 0u;
  if (__any_sync(0xffffffffu, d) && (threadIdx.x & 31) == 0) atomicOr(flag, 1u);
}

// Whether V's ELL column arrays equal H's (checked on the device once per pair of handles).
int same_columns(kpm_ell_s* h, kpm_ell_s* v, cudaStream_t s, bool* same) {
  *same = false;
  if (v->same_cols_id == h->id) {
    *same = true;
    return KPM_OK;
  }
  if (v->L != h->L || v->n_pad != h->n_pad) return KPM_OK;
  DevBuf f;
  KPM_TRY(ensure(f, sizeof(unsigned)));
  unsigned host = 1;
  const int64_t count = (int64_t)h->L * h->n_pad;
  int st = check_cuda(cudaMemsetAsync(f.p, 0, sizeof(unsigned), s));
  if (st == KPM_OK) {
    cols_differ_kernel<<<(int)std::min<int64_t>((count + 255) / 256, 4096), 256, 0, s>>>(h->col, v->col, count,
                                                                                        static_cast<unsigned*>(f.p));
    st = check_cuda(cudaGetLastError());
  }
  if (st == KPM_OK) st = check_cuda(cudaMemcpyAsync(&host, f.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  if (st == KPM_OK) st = check_cuda(cudaStreamSynchronize(s));
  release(f);
  if (st != KPM_OK) return st;
  if (host == 0) {
    v->same_cols_id = h->id;
    *same = true;
  }
  return KPM_OK;
}

int kpm_mu_nm(kpm_ell* h, kpm_ell* v_op, int R, int Nm, const double* v, double* mu, void* stream) {
  if (!h || !v_op || !v || !mu || R < 1 || Nm < 2 || Nm > 256) return KPM_ERR_INVALID_ARG;
  if (v_op->n != h->n) return KPM_ERR_SHAPE;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  KPM_TRY(ensure_f32_values(h, s));
  KPM_TRY(ensure_f32_values(v_op, s));
  Workspace& ws = h->ws;
  // up to kMuGroup vectors advance together; a stored row is one packed [n_pad][Rg] complex64 vector set
  const int G = pow2_group(std::min(R, kMuGroup));
  const int64_t lda = 2 * (int64_t)G * h->n_pad;            // floats per stored row
  const size_t mat = (size_t)256 * lda * sizeof(float);     // 256 rows; rows >= Nm stay zero
  const size_t vb = (size_t)h->n_pad * G * sizeof(float2);
  KPM_TRY(ensure(ws.ckpt, 2 * mat));                         // A = L rows, B = R rows
  KPM_TRY(ensure(ws.ta, vb));
  KPM_TRY(ensure(ws.tb, vb));
  const int KS = contract_splits(lda, h->sm_count, mu_tiles(Nm));
  KPM_TRY(ensure(ws.part, contract_part_floats(KS, mu_tiles(Nm)) * sizeof(float)));
  float* A = static_cast<float*>(ws.ckpt.p);
  float* B = A + (size_t)256 * lda;
  if (Nm < 256) {
    const size_t tail = (size_t)(256 - Nm) * lda * sizeof(float);
    KPM_CUDA_TRY(cudaMemsetAsync(A + (size_t)Nm * lda, 0, tail, s));
    KPM_CUDA_TRY(cudaMemsetAsync(B + (size_t)Nm * lda, 0, tail, s));
  }
  for (int r0 = 0; r0 < R;) {
    const int Rg = std::min(G, pow2_group(R - r0));
    const int64_t k = 2 * (int64_t)Rg * h->n_pad;  // floats of a row this group fills
    const int grid_h = grid_for(h, Rg, vpt_for(true, Rg));
    const int grid_v = grid_for(v_op, Rg, vpt_for(true, Rg));
    // recursion steps: the staged producer-warp kernel (no moments), else the grid-stride kernel
    const int occ = ws_ctas_f32(h->is_real, Rg, 1, h->L, 2);
    const int64_t ntiles = h->n_pad / staged_tile_rows(true, Rg, 1);
    const int grid_ws = occ > 0 ? (int)std::min<int64_t>(ntiles, (int64_t)occ * h->sm_count) : 0;
    auto next = [&](StepParams q) -> int {
      q.vl = nullptr;
      q.per_tile = 0;
      return grid_ws > 0 ? launch_ws_f32(h->is_real, Rg, 1, q, grid_ws, s)
                         : launch_step(true, h->is_real, Rg, MODE_NEXT, EPI_STORE, q, grid_h, s);
    };
    KPM_TRY(pack_vectors(v, h->n, h->n_pad, R, r0, Rg, true, ws.ta.p, s));
    // A[0] = V v, A[1] = H A[0], A[m+1] = 2 H A[m] - A[m-1]  (out of place, every row kept)
    StepParams pv = base_params(v_op, true);
    pv.tcur = ws.ta.p;
    pv.tout = A;
    pv.a_half = make_double2(0.5, 0.0);
    KPM_TRY(launch_step(true, v_op->is_real, Rg, MODE_APPLY, EPI_STORE, pv, grid_v, s));
    StepParams ph = base_params(h, true);
    ph.tcur = A;
    ph.tout = A + lda;
    KPM_TRY(launch_step(true, h->is_real, Rg, MODE_FIRST, EPI_STORE, ph, grid_h, s));
    for (int m = 1; m + 1 < Nm; ++m) {
      ph.tcur = A + (size_t)m * lda;
      ph.tprev = A + (size_t)(m - 1) * lda;
      ph.tout = A + (size_t)(m + 1) * lda;
      KPM_TRY(next(ph));
    }
    // T recursion on v (in place), B[m] = V T_m; when V has H's columns (and complex
    // values) the product rides in the H step: one gather of T_m for both operators
    void* t_prev = ws.ta.p;  // T_0
    void* t_cur = ws.tb.p;
    pv.tcur = t_prev;
    pv.tout = B;
    KPM_TRY(launch_step(true, v_op->is_real, Rg, MODE_APPLY, EPI_STORE, pv, grid_v, s));
    StepParams pt = base_params(h, true);
    pt.tcur = t_prev;
    pt.tout = t_cur;
    KPM_TRY(launch_step(true, h->is_real, Rg, MODE_FIRST, EPI_STORE, pt, grid_h, s));
    bool fuse = false;
    if (!v_op->is_real && !getenv("KPM_MU_NM_UNFUSED")) {
      KPM_TRY(same_columns(h, v_op, s, &fuse));
      if (fuse) fuse = kubo_step(h->is_real != 0, Rg, pt, v_op->val32, nullptr, h->sm_count, s, false) == KPM_OK;
    }
    for (int m = 1; m < Nm; ++m) {
      if (fuse && m + 1 < Nm) {
        pt.tcur = t_cur;
        pt.tout = t_prev;
        KPM_TRY(kubo_step(h->is_real != 0, Rg, pt, v_op->val32, B + (size_t)m * lda, h->sm_count, s, true));
        std::swap(t_prev, t_cur);
        continue;
      }
      pv.tcur = t_cur;
      pv.tout = B + (size_t)m * lda;
      KPM_TRY(launch_step(true, v_op->is_real, Rg, MODE_APPLY, EPI_STORE, pv, grid_v, s));
      if (m + 1 < Nm) {
        pt.tcur = t_cur;
        pt.tout = t_prev;
        KPM_TRY(next(pt));
        std::swap(t_prev, t_cur);
      }
    }
    // the group's rows contract over its k floats: sum over sites and the group's vectors
    KPM_TRY(mu_contract(A, B, k, lda, Nm, 1.0 / R, r0 > 0, reinterpret_cast<double2*>(mu),
                        static_cast<float*>(ws.part.p), KS, h->err_flag, s));
    r0 += Rg;
  }
  return KPM_OK;
}

}  // extern "C"
