// kpm_batch.cu -- many independent operators of uneven size advanced by one
// recursion: the instances are stacked block-diagonally into one operator whose
// rows are padded per instance to a multiple of kRowAlign, so a row tile never
// spans two instances.  Every step is one launch over all instances (load
// balance is by tile, not by instance); moment partials are kept per tile and
// summed per instance by a segmented, fixed-order reduction.  The whole
// recursion (first step, M-2 steps, reductions) is captured once into a CUDA
// graph per (precision, R, M) and replayed as a single graph launch.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "kpm_internal.cuh"

using namespace kpm;

struct kpm_batch_s {
  int n_inst = 0;
  int64_t n_total = 0;                 // unpadded rows of all instances
  std::vector<int64_t> rows;           // per instance
  std::vector<int64_t> off;            // unpadded row offset (user layout)
  std::vector<int64_t> poff;           // padded row offset (device layout)
  int64_t* d_off = nullptr;            // device copies
  int64_t* d_poff = nullptr;
  int64_t* d_rows = nullptr;
  kpm_ell_s* op = nullptr;             // the stacked operator
  // graph cache
  struct G {
    int f32, R, M, kind, dbl;
    const void* bufs[8];  // workspace pointers the graph was recorded with
    cudaGraphExec_t exec;
  };
  std::vector<G> graphs;
  DevBuf mu_int;                       // internal moments [n_inst][R][M]
  // partial-slot layout per (precision, R)
  struct Plan {
    int f32 = 0, R = 0;
    int tile_first = 0;                // grid-stride tile (first step)
    int64_t ntiles_first = 0;
    int64_t* d_ibeg_first = nullptr;   // [n_inst + 1] tile ranges of the first step
    int kind = 0, U = 1, grid = 0, tile = 0;
    int64_t nslots = 0;                // partial slots per later step
    int64_t* d_ibeg = nullptr;         // [n_inst + 1] slot ranges of later steps
    bool own_ibeg = false;
    int* d_tile_inst = nullptr;        // staged: instance of each tile
    int* d_seg_base = nullptr;         // staged: first slot of each CTA
    int chunk = 2;
    float step_us = 0.f;               // tuned time of one later step
    int dbl = 0;                       // doubled DOS moments: two partial sets per step
  };
  std::vector<Plan> plans;
};

namespace {

// padded row -> (instance, local row) by binary search on padded offsets
__device__ __forceinline__ int find_inst(const int64_t* poff, int n_inst, int64_t prow) {
  int lo = 0, hi = n_inst - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (poff[mid] <= prow)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__global__ void batch_validate_kernel(const double2* __restrict__ data, const int32_t* __restrict__ idx,
                                      const int64_t* __restrict__ off, const int64_t* __restrict__ rows, int n_inst,
                                      int L, int64_t n_total, unsigned* flags) {
  unsigned f = 0;
  const int64_t count = n_total * L;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < count; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = t / L;
    const int k = find_inst(off, n_inst, row);
    const int32_t c = idx[t];
    if (c < 0 || (int64_t)c >= rows[k]) f |= 1u;
    if (data[t].y != 0.0) f |= 2u;
    if (!isfinite(data[t].x) || !isfinite(data[t].y)) f |= 4u;
  }
  if (f) atomicOr(flags, f);
}

// user AoS (unpadded, local columns) -> padded SoA with global columns, values doubled
__global__ void batch_repack_kernel(const double2* __restrict__ data, const int32_t* __restrict__ idx,
                                    const int64_t* __restrict__ off, const int64_t* __restrict__ poff,
                                    const int64_t* __restrict__ rows, int n_inst, int L, int64_t n_pad, bool real,
                                    void* val, int32_t* col) {
  const int64_t total = (int64_t)L * n_pad;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int s = (int)(t / n_pad);
    const int64_t prow = t % n_pad;
    const int k = find_inst(poff, n_inst, prow);
    const int64_t lr = prow - poff[k];
    double2 v = make_double2(0.0, 0.0);
    int32_t c = (int32_t)prow;
    if (lr < rows[k]) {
      const int64_t src = (off[k] + lr) * L + s;
      v = data[src];
      c = (int32_t)(poff[k] + idx[src]);
    }
    col[t] = c;
    if (real)
      static_cast<double*>(val)[t] = 2.0 * v.x;
    else
      static_cast<double2*>(val)[t] = make_double2(2.0 * v.x, 2.0 * v.y);
  }
}

// user vectors [R][n_total] c128 -> padded site-major [n_pad][R]
__global__ void batch_pack_kernel(const double2* __restrict__ src, const int64_t* __restrict__ off,
                                  const int64_t* __restrict__ poff, const int64_t* __restrict__ rows, int n_inst,
                                  int64_t n_total, int64_t n_pad, int R, bool to_f32, void* dst) {
  const int64_t total = n_pad * R;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t prow = t / R;
    const int r = (int)(t % R);
    const int k = find_inst(poff, n_inst, prow);
    const int64_t lr = prow - poff[k];
    double2 z = make_double2(0.0, 0.0);
    if (lr < rows[k]) z = src[(int64_t)r * n_total + off[k] + lr];
    if (to_f32)
      static_cast<float2*>(dst)[t] = make_float2((float)z.x, (float)z.y);
    else
      static_cast<double2*>(dst)[t] = z;
  }
}

// part[step * step_stride + slot * R + r] -> mu[k][r][m0 + step]; instance k owns
// slots [ibeg[k], ibeg[k+1]).  One CTA per (r, instance, step); fixed-order
// strided sums and a fixed tree.
__global__ void batch_reduce_kernel(const double2* __restrict__ part, int64_t step_stride,
                                    const int64_t* __restrict__ ibeg, int R, double2* __restrict__ mu, int M,
                                    int m0) {
  const int r = blockIdx.x, k = blockIdx.y, step = blockIdx.z;
  const int64_t t0 = ibeg[k], t1 = ibeg[k + 1];
  const double2* base = part + (int64_t)step * step_stride;
  double sr = 0.0, si = 0.0;
  for (int64_t t = t0 + threadIdx.x; t < t1; t += blockDim.x) {
    const double2 v = base[t * R + r];
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
  if (threadIdx.x == 0) mu[((int64_t)k * R + r) * M + m0 + step] = make_double2(shr[0], shi[0]);
}

int grid1(int64_t total) { return (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 65536)); }

// Steps whose partials are buffered before a segmented reduction.
int batch_chunk(int64_t nslots, int R) {
  const int64_t per_step = nslots * R * (int64_t)sizeof(double2);
  int64_t c = ((int64_t)256 << 20) / std::max<int64_t>(1, per_step);
  return (int)std::max<int64_t>(2, std::min<int64_t>(c, kChunk));
}

int upload(void** dst, const void* src, size_t bytes) {
  int rc = check_cuda(cudaMalloc(dst, bytes));
  if (rc == KPM_OK) rc = check_cuda(cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice));
  return rc;
}

// Slot layout of a staged plan (contiguous tile ranges per CTA): the instance
// of every tile, the first partial slot of every CTA, and every instance's slot
// range (one slot per (CTA, instance) run).
int plan_layout(kpm_batch_s* b, kpm_batch_s::Plan& pl) {
  kpm_ell_s* h = b->op;
  const int64_t ntiles = h->n_pad / pl.tile;
  std::vector<int> tinst(ntiles);
  for (int k = 0; k < b->n_inst; ++k) {
    const int64_t t0 = b->poff[k] / pl.tile;
    const int64_t t1 = (k + 1 < b->n_inst ? b->poff[k + 1] : h->n_pad) / pl.tile;
    for (int64_t t = t0; t < t1; ++t) tinst[t] = k;
  }
  std::vector<int> seg_base(pl.grid);
  std::vector<int64_t> ibeg(b->n_inst + 1, -1);
  int64_t slot = 0;
  for (int g = 0; g < pl.grid; ++g) {
    const int64_t tb = ((int64_t)g * ntiles) / pl.grid, te = ((int64_t)(g + 1) * ntiles) / pl.grid;
    seg_base[g] = (int)slot;
    for (int64_t t = tb; t < te; ++t)
      if (t == tb || tinst[t] != tinst[t - 1]) {
        if (ibeg[tinst[t]] < 0) ibeg[tinst[t]] = slot;
        ++slot;
      }
  }
  ibeg[b->n_inst] = slot;
  pl.nslots = slot;
  KPM_TRY(upload(reinterpret_cast<void**>(&pl.d_tile_inst), tinst.data(), tinst.size() * sizeof(int)));
  KPM_TRY(upload(reinterpret_cast<void**>(&pl.d_seg_base), seg_base.data(), seg_base.size() * sizeof(int)));
  KPM_TRY(upload(reinterpret_cast<void**>(&pl.d_ibeg), ibeg.data(), ibeg.size() * sizeof(int64_t)));
  pl.own_ibeg = true;
  return KPM_OK;
}

void plan_free_layout(kpm_batch_s::Plan& pl) {
  if (pl.own_ibeg && pl.d_ibeg) cudaFree(pl.d_ibeg);
  if (pl.d_tile_inst) cudaFree(pl.d_tile_inst);
  if (pl.d_seg_base) cudaFree(pl.d_seg_base);
  pl.d_ibeg = nullptr;
  pl.d_tile_inst = nullptr;
  pl.d_seg_base = nullptr;
  pl.own_ibeg = false;
}

// One MODE_NEXT launch of a plan (moment partials into slot block `part`).
int plan_next(kpm_batch_s* b, bool f32, int R, const kpm_batch_s::Plan& pl, StepParams p, cudaStream_t s) {
  kpm_ell_s* h = b->op;
  p.tile_inst = pl.d_tile_inst;
  p.seg_base = pl.d_seg_base;
  p.part_set_stride = pl.nslots * R;
  if (pl.kind == 1) {
    p.per_tile = 1;
    return f32 ? launch_staged_f32(h->is_real, R, pl.U, p, pl.grid, s) : launch_staged_f64(h->is_real, R, pl.U, p, pl.grid, s);
  }
  if (pl.kind == 2) {
    p.per_tile = 1;
    return f32 ? launch_ws_f32(h->is_real, R, pl.U, p, pl.grid, s) : launch_ws_f64(h->is_real, R, pl.U, p, pl.grid, s);
  }
  p.per_tile = 0;
  return f32 ? launch_step_f32(h->is_real, R, MODE_NEXT, EPI_STORE | EPI_MOM1, p, pl.grid, s)
             : launch_step_f64(h->is_real, R, MODE_NEXT, EPI_STORE | EPI_MOM1, p, pl.grid, s);
}

StepParams batch_params(kpm_ell_s* h, bool f32) {
  StepParams p;
  std::memset(&p, 0, sizeof(p));
  p.val = f32 ? h->val32 : h->val64;
  p.col = h->col;
  p.ld = h->n_pad;
  p.L = h->L;
  p.n_pad = h->n_pad;
  p.a_half = make_double2(0.5, 0.0);
  p.err = h->err_flag;
  p.wait_budget = kWaitBudgetCycles;
  p.vl = h->ws.vl.p;
  return p;
}

// Build (or find) the plan of a batched recursion for (precision, R): the
// first step runs the grid-stride kernel with one CTA per tile (slots = tiles);
// later steps run the kernel the autotuner picks among the grid-stride kernel
// (one CTA per tile), the staged kernel and its producer-warp form (1 or 2 rows
// per thread, contiguous tile ranges per CTA, slots = (CTA, instance) runs).
// Each candidate is timed on the stacked operator itself (a few launches on
// zeroed vectors) and the fastest is kept.  KPM_STEP_KERNEL forces one
// (simple|staged1|staged2|ws1|ws2).
int batch_plan(kpm_batch_s* b, bool f32, int R, bool dbl, cudaStream_t s, const kpm_batch_s::Plan** out) {
  for (auto& pl : b->plans)
    if (pl.f32 == (int)f32 && pl.R == R && pl.dbl == (int)dbl) {
      *out = &pl;
      return KPM_OK;
    }
  kpm_ell_s* h = b->op;
  kpm_batch_s::Plan base;
  base.f32 = (int)f32;
  base.R = R;
  base.dbl = (int)dbl;
  base.tile_first = kBlock / (R / ((f32 && R >= 2) ? 2 : 1));
  base.ntiles_first = h->n_pad / base.tile_first;
  std::vector<int64_t> ib(b->n_inst + 1);
  for (int k = 0; k < b->n_inst; ++k) ib[k] = b->poff[k] / base.tile_first;
  ib[b->n_inst] = base.ntiles_first;
  KPM_TRY(upload(reinterpret_cast<void**>(&base.d_ibeg_first), ib.data(), ib.size() * sizeof(int64_t)));
  const char* force = getenv("KPM_STEP_KERNEL");
  const std::string f = force ? force : "";

  std::vector<kpm_batch_s::Plan> cands;
  if (f.empty() || f == "simple") {
    kpm_batch_s::Plan pl = base;
    pl.kind = 0;
    pl.tile = pl.tile_first;
    pl.grid = (int)pl.ntiles_first;
    pl.nslots = pl.ntiles_first;
    pl.d_ibeg = pl.d_ibeg_first;
    pl.own_ibeg = false;
    cands.push_back(pl);
  }
  int rc = KPM_OK;
  for (int kind = 1; kind <= 2 && rc == KPM_OK; ++kind)
    for (int U = 1; U <= 2 && rc == KPM_OK; ++U) {
      if (dbl && kind == 1) continue;  // doubling: grid-stride and producer-warp kernels
      if (!f.empty() && f != std::string(kind == 1 ? "staged" : "ws") + (U == 1 ? "1" : "2")) continue;
      const int occ = kind == 1 ? (f32 ? staged_ctas_f32(h->is_real, R, U, h->L, 2) : staged_ctas_f64(h->is_real, R, U, h->L, 2))
                                : (f32 ? ws_ctas_f32(h->is_real, R, U, h->L, 2) : ws_ctas_f64(h->is_real, R, U, h->L, 2));
      if (occ <= 0) continue;
      kpm_batch_s::Plan pl = base;
      pl.kind = kind;
      pl.U = U;
      pl.tile = staged_tile_rows(f32, R, U);
      const int64_t ntiles = h->n_pad / pl.tile;
      pl.grid = (int)std::max<int64_t>(1, std::min<int64_t>(ntiles, (int64_t)occ * h->sm_count));
      rc = plan_layout(b, pl);
      cands.push_back(pl);
    }
  if (cands.empty() && rc == KPM_OK) {  // a forced kernel that cannot run here: the grid-stride kernel
    kpm_batch_s::Plan pl = base;
    pl.kind = 0;
    pl.tile = pl.tile_first;
    pl.grid = (int)pl.ntiles_first;
    pl.nslots = pl.ntiles_first;
    pl.d_ibeg = pl.d_ibeg_first;
    cands.push_back(pl);
  }
  std::vector<float> us(cands.size(), 0.f);
  if (rc == KPM_OK && cands.size() > 1) {
    int64_t max_slots = 0;
    for (auto& c : cands) max_slots = std::max(max_slots, c.nslots);
    Workspace& ws = h->ws;
    const size_t vb = (size_t)h->n_pad * R * (f32 ? sizeof(float2) : sizeof(double2));
    rc = ensure(ws.part, (size_t)2 * max_slots * R * sizeof(double2));
    if (rc == KPM_OK) rc = ensure(ws.vr, vb);
    if (rc == KPM_OK) rc = check_cuda(cudaMemsetAsync(ws.ta.p, 0, vb, s));
    if (rc == KPM_OK) rc = check_cuda(cudaMemsetAsync(ws.tb.p, 0, vb, s));
    if (rc == KPM_OK) rc = check_cuda(cudaMemsetAsync(ws.vl.p, 0, vb, s));
    if (rc == KPM_OK) rc = check_cuda(cudaMemsetAsync(ws.vr.p, 0, vb, s));
    StepParams p = batch_params(h, f32);
    p.tcur = ws.ta.p;
    p.tout = ws.tb.p;
    p.part = static_cast<double2*>(ws.part.p);
    if (dbl) {
      p.vl = nullptr;
      p.dbl = 1;
      p.hv = ws.vr.p;
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (rc == KPM_OK) rc = check_cuda(cudaEventCreate(&e0));
    if (rc == KPM_OK) rc = check_cuda(cudaEventCreate(&e1));
    const int reps = 3;
    for (size_t i = 0; i < cands.size() && rc == KPM_OK; ++i) {
      rc = plan_next(b, f32, R, cands[i], p, s);
      if (rc == KPM_OK) rc = check_cuda(cudaEventRecord(e0, s));
      for (int r = 0; r < reps && rc == KPM_OK; ++r) rc = plan_next(b, f32, R, cands[i], p, s);
      if (rc == KPM_OK) rc = check_cuda(cudaEventRecord(e1, s));
      if (rc == KPM_OK) rc = check_cuda(cudaEventSynchronize(e1));
      float ms = 0.f;
      if (rc == KPM_OK) rc = check_cuda(cudaEventElapsedTime(&ms, e0, e1));
      us[i] = 1e3f * ms / reps;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
  }
  size_t best = 0;
  for (size_t i = 1; i < cands.size(); ++i)
    if (us[i] < us[best]) best = i;
  for (size_t i = 0; i < cands.size(); ++i)
    if (i != best || rc != KPM_OK) plan_free_layout(cands[i]);
  if (rc != KPM_OK) {
    cudaFree(base.d_ibeg_first);
    return rc;
  }
  kpm_batch_s::Plan pl = cands[best];
  pl.step_us = us[best];
  pl.chunk = batch_chunk((dbl ? 2 : 1) * pl.nslots, R);
  b->plans.push_back(pl);
  *out = &b->plans.back();
  return KPM_OK;
}

// Partial-buffer elements (double2) a plan needs: two first-step blocks, then chunk NEXT blocks.
int64_t plan_part_elems(const kpm_batch_s::Plan& pl, int R) {
  return 2 * pl.ntiles_first * R + (int64_t)pl.chunk * (pl.dbl ? 2 : 1) * pl.nslots * R;
}

bool batch_doubling(const kpm_batch_s* b, int M) { return use_doubling(b->op, M); }

// The launch sequence of one batched recursion on internal buffers:
// ta = T_0 (packed), tb = T_1, vl = left vectors, part = partials, mu_int = [n_inst][R][M].
int record_batched(kpm_batch_s* b, bool f32, int R, int M, const kpm_batch_s::Plan& pl, cudaStream_t s) {
  kpm_ell_s* h = b->op;
  Workspace& ws = h->ws;
  double2* part_first = static_cast<double2*>(ws.part.p);
  double2* part = part_first + 2 * pl.ntiles_first * R;
  double2* mu = static_cast<double2*>(b->mu_int.p);
  StepParams p = batch_params(h, f32);
  // m = 1 and mu_0: one grid-stride CTA per tile, so per-CTA partials are per-tile partials
  p.part_step_stride = pl.ntiles_first * R;
  p.tcur = ws.ta.p;
  p.tout = ws.tb.p;
  p.part = part_first;
  KPM_TRY(f32 ? launch_step_f32(h->is_real, R, MODE_FIRST, EPI_STORE | EPI_MOM1, p, (int)pl.ntiles_first, s)
              : launch_step_f64(h->is_real, R, MODE_FIRST, EPI_STORE | EPI_MOM1, p, (int)pl.ntiles_first, s));
  {
    dim3 g(R, b->n_inst, M >= 2 ? 2 : 1);
    batch_reduce_kernel<<<g, 128, 0, s>>>(part_first, pl.ntiles_first * R, pl.d_ibeg_first, R, mu, M, 0);
    KPM_CUDA_TRY(cudaGetLastError());
  }
  if (pl.dbl) {
    // doubled: steps m = 2 .. K = ceil(M/2), sets <t_m|t_{m-1}> and sum(|t_{m-1}|^2 - hv) per instance
    const int K = (M + 1) / 2;
    if (f32)  // mu_1 exactly for the float start vectors (enters every odd moment)
      KPM_TRY(mu1_exact(h, ws.vl.p, R, b->d_poff, b->n_inst, mu, M, 0, ws.tc, s));
    const int64_t sstride = 2 * pl.nslots * R;
    double2* rb = static_cast<double2*>(ws.red.p);
    double2* rd = rb + (size_t)b->n_inst * R * (K + 1);
    const double* corr = reinterpret_cast<const double*>(rd + (size_t)b->n_inst * R * (K + 1));
    p.vl = nullptr;
    p.dbl = 1;
    p.hv = ws.vr.p;
    auto reduce = [&](int m0, int steps) -> int {
      dim3 g(R, b->n_inst, steps);
      batch_reduce_kernel<<<g, 128, 0, s>>>(part, sstride, pl.d_ibeg, R, rb, K + 1, m0);
      batch_reduce_kernel<<<g, 128, 0, s>>>(part + pl.nslots * R, sstride, pl.d_ibeg, R, rd, K + 1, m0);
      KPM_CUDA_TRY(cudaGetLastError());
      return KPM_OK;
    };
    void* tprev = ws.ta.p;
    void* tcur = ws.tb.p;
    int m0 = 2;
    for (int m = 2; m <= K; ++m) {
      if (m - m0 == pl.chunk) {
        KPM_TRY(reduce(m0, pl.chunk));
        m0 = m;
      }
      p.tcur = tcur;
      p.tout = tprev;
      p.part = part + (int64_t)(m - m0) * sstride;
      KPM_TRY(plan_next(b, f32, R, pl, p, s));
      std::swap(tprev, tcur);
    }
    if (K + 1 > m0) KPM_TRY(reduce(m0, K + 1 - m0));
    return assemble_doubled(rb, rd, corr, b->n_inst * R, K, M, mu, M, 0, s);
  }
  void* tprev = ws.ta.p;
  void* tcur = ws.tb.p;
  int m0 = 2;
  for (int m = 2; m < M; ++m) {
    if (m - m0 == pl.chunk) {
      dim3 g(R, b->n_inst, pl.chunk);
      batch_reduce_kernel<<<g, 128, 0, s>>>(part, pl.nslots * R, pl.d_ibeg, R, mu, M, m0);
      KPM_CUDA_TRY(cudaGetLastError());
      m0 = m;
    }
    p.tcur = tcur;
    p.tout = tprev;
    p.part = part + (int64_t)(m - m0) * pl.nslots * R;
    KPM_TRY(plan_next(b, f32, R, pl, p, s));
    std::swap(tprev, tcur);
  }
  if (M > m0) {
    dim3 g(R, b->n_inst, M - m0);
    batch_reduce_kernel<<<g, 128, 0, s>>>(part, pl.nslots * R, pl.d_ibeg, R, mu, M, m0);
    KPM_CUDA_TRY(cudaGetLastError());
  }
  return KPM_OK;
}

}  // namespace

extern "C" {

int kpm_batch_create(kpm_batch** out, int n_inst, const int64_t* inst_rows, int len_row, const double* data,
                     const int32_t* indices, void* stream) {
  if (!out || n_inst < 1 || !inst_rows || len_row < 1 || !data || !indices) return KPM_ERR_INVALID_ARG;
  *out = nullptr;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  kpm_batch_s* b = new kpm_batch_s();
  b->n_inst = n_inst;
  b->rows.assign(inst_rows, inst_rows + n_inst);
  int64_t o = 0, po = 0;
  for (int k = 0; k < n_inst; ++k) {
    if (b->rows[k] < 1) {
      delete b;
      return KPM_ERR_INVALID_ARG;
    }
    b->off.push_back(o);
    b->poff.push_back(po);
    o += b->rows[k];
    po += ((b->rows[k] + kRowAlign - 1) / kRowAlign) * kRowAlign;
  }
  b->n_total = o;
  if (po > (int64_t)INT32_MAX) {
    delete b;
    return KPM_ERR_SHAPE;
  }
  kpm_ell_s* h = new kpm_ell_s();
  b->op = h;
  h->n = po;  // every padded row is a row of the stacked operator
  h->n_pad = po;
  h->L = len_row;
  int dev = 0;
  DevBuf st_data, st_idx, flag;
  auto fail = [&](int code) {
    release(st_data);
    release(st_idx);
    release(flag);
    kpm_batch_destroy(b);
    return code;
  };
  int rc = check_cuda(cudaGetDevice(&dev));
  if (rc == KPM_OK) rc = check_cuda(cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, dev));
  if (rc != KPM_OK) return fail(rc);
  h->device = dev;
  const int64_t count = b->n_total * len_row;
  if ((rc = ensure(st_data, count * sizeof(double2))) != KPM_OK) return fail(rc);
  if ((rc = ensure(st_idx, count * sizeof(int32_t))) != KPM_OK) return fail(rc);
  if ((rc = ensure(flag, sizeof(unsigned))) != KPM_OK) return fail(rc);
  rc = check_cuda(cudaMalloc(reinterpret_cast<void**>(&b->d_off), n_inst * sizeof(int64_t)));
  if (rc == KPM_OK) rc = check_cuda(cudaMalloc(reinterpret_cast<void**>(&b->d_poff), n_inst * sizeof(int64_t)));
  if (rc == KPM_OK) rc = check_cuda(cudaMalloc(reinterpret_cast<void**>(&b->d_rows), n_inst * sizeof(int64_t)));
  if (rc != KPM_OK) return fail(rc);
  rc = check_cuda(cudaMemcpyAsync(st_data.p, data, count * sizeof(double2), cudaMemcpyHostToDevice, s));
  if (rc == KPM_OK) rc = check_cuda(cudaMemcpyAsync(st_idx.p, indices, count * sizeof(int32_t), cudaMemcpyHostToDevice, s));
  if (rc == KPM_OK) rc = check_cuda(cudaMemcpyAsync(b->d_off, b->off.data(), n_inst * sizeof(int64_t), cudaMemcpyHostToDevice, s));
  if (rc == KPM_OK) rc = check_cuda(cudaMemcpyAsync(b->d_poff, b->poff.data(), n_inst * sizeof(int64_t), cudaMemcpyHostToDevice, s));
  if (rc == KPM_OK) rc = check_cuda(cudaMemcpyAsync(b->d_rows, b->rows.data(), n_inst * sizeof(int64_t), cudaMemcpyHostToDevice, s));
  if (rc == KPM_OK) rc = check_cuda(cudaMemsetAsync(flag.p, 0, sizeof(unsigned), s));
  if (rc != KPM_OK) return fail(rc);
  batch_validate_kernel<<<grid1(count), 256, 0, s>>>(static_cast<const double2*>(st_data.p),
                                                      static_cast<const int32_t*>(st_idx.p), b->d_off, b->d_rows,
                                                      n_inst, len_row, b->n_total, static_cast<unsigned*>(flag.p));
  unsigned hf = 0;
  rc = check_cuda(cudaGetLastError());
  if (rc == KPM_OK) rc = check_cuda(cudaMemcpyAsync(&hf, flag.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  if (rc == KPM_OK) rc = check_cuda(cudaStreamSynchronize(s));
  if (rc != KPM_OK) return fail(rc);
  if (hf & 1u) return fail(KPM_ERR_INDEX);
  if (hf & 4u) return fail(KPM_ERR_NONFINITE);
  h->is_real = (hf & 2u) ? 0 : 1;
  const int64_t slots = (int64_t)len_row * h->n_pad;
  rc = check_cuda(cudaMalloc(&h->val64, slots * (h->is_real ? sizeof(double) : sizeof(double2))));
  if (rc == KPM_OK) rc = check_cuda(cudaMalloc(reinterpret_cast<void**>(&h->col), slots * sizeof(int32_t)));
  if (rc == KPM_OK) rc = check_cuda(cudaMalloc(reinterpret_cast<void**>(&h->err_flag), sizeof(int)));
  if (rc == KPM_OK) rc = check_cuda(cudaMemsetAsync(h->err_flag, 0, sizeof(int), s));
  if (rc != KPM_OK) return fail(rc);
  batch_repack_kernel<<<grid1(slots), 256, 0, s>>>(static_cast<const double2*>(st_data.p),
                                                    static_cast<const int32_t*>(st_idx.p), b->d_off, b->d_poff,
                                                    b->d_rows, n_inst, len_row, h->n_pad, h->is_real != 0, h->val64,
                                                    h->col);
  rc = check_cuda(cudaGetLastError());
  if (rc == KPM_OK) rc = check_cuda(cudaStreamSynchronize(s));
  if (rc != KPM_OK) return fail(rc);
  release(st_data);
  release(st_idx);
  release(flag);
  h->doubling = 0;
  if ((rc = check_hermitian(h, s)) != KPM_OK) return fail(rc);
  *out = b;
  return KPM_OK;
}

int kpm_batch_destroy(kpm_batch* b) {
  if (!b) return KPM_ERR_INVALID_ARG;
  for (auto& g : b->graphs) cudaGraphExecDestroy(g.exec);
  for (auto& pl : b->plans) {
    if (pl.d_ibeg_first) cudaFree(pl.d_ibeg_first);
    if (pl.own_ibeg && pl.d_ibeg) cudaFree(pl.d_ibeg);
    if (pl.d_tile_inst) cudaFree(pl.d_tile_inst);
    if (pl.d_seg_base) cudaFree(pl.d_seg_base);
  }
  release(b->mu_int);
  if (b->d_off) cudaFree(b->d_off);
  if (b->d_poff) cudaFree(b->d_poff);
  if (b->d_rows) cudaFree(b->d_rows);
  if (b->op) kpm_ell_destroy(b->op);
  delete b;
  return KPM_OK;
}

int kpm_batch_info(const kpm_batch* b, int* n_inst, int64_t* rows_total, int64_t* rows_padded, int* is_real) {
  if (!b) return KPM_ERR_INVALID_ARG;
  if (n_inst) *n_inst = b->n_inst;
  if (rows_total) *rows_total = b->n_total;
  if (rows_padded) *rows_padded = b->op->n_pad;
  if (is_real) *is_real = b->op->is_real;
  return KPM_OK;
}

int kpm_batch_step_config(kpm_batch* b, int dtype, int R, int* kind, int* rows_per_thread, int* grid, float* step_us,
                          void* stream) {
  if (!b) return KPM_ERR_INVALID_ARG;
  if (dtype != KPM_C128 && dtype != KPM_C64) return KPM_ERR_DTYPE;
  if (R != 1 && R != 2 && R != 4 && R != 8) return KPM_ERR_UNSUPPORTED;
  const bool f32 = dtype == KPM_C64;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  kpm_ell_s* h = b->op;
  if (f32) KPM_TRY(ensure_f32_values(h, s));
  const size_t vb = (size_t)h->n_pad * R * (f32 ? sizeof(float2) : sizeof(double2));
  KPM_TRY(ensure(h->ws.ta, vb));
  KPM_TRY(ensure(h->ws.tb, vb));
  KPM_TRY(ensure(h->ws.vl, vb));
  const kpm_batch_s::Plan* plan = nullptr;
  KPM_TRY(batch_plan(b, f32, R, batch_doubling(b, 4), s, &plan));
  if (kind) *kind = plan->kind;
  if (rows_per_thread) *rows_per_thread = plan->kind == 0 ? 1 : plan->U;
  if (grid) *grid = plan->grid;
  if (step_us) *step_us = plan->step_us;
  return KPM_OK;
}

int kpm_batch_moments(kpm_batch* b, int dtype, int R, int M, const double* v, double* mu, void* stream) {
  if (!b || !v || !mu || M < 2) return KPM_ERR_INVALID_ARG;
  if (dtype != KPM_C128 && dtype != KPM_C64) return KPM_ERR_DTYPE;
  if (R != 1 && R != 2 && R != 4 && R != 8) return KPM_ERR_UNSUPPORTED;
  const bool f32 = dtype == KPM_C64;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  kpm_ell_s* h = b->op;
  if (f32) KPM_TRY(ensure_f32_values(h, s));
  const size_t vb = (size_t)h->n_pad * R * (f32 ? sizeof(float2) : sizeof(double2));
  Workspace& ws = h->ws;
  KPM_TRY(ensure(ws.ta, vb));
  KPM_TRY(ensure(ws.tb, vb));
  KPM_TRY(ensure(ws.vl, vb));
  KPM_TRY(ensure(b->mu_int, (size_t)b->n_inst * R * M * sizeof(double2)));
  // kernel choice and partial-slot layout (built once per precision, R and mode)
  const bool dbl = batch_doubling(b, M);
  const kpm_batch_s::Plan* plan = nullptr;
  KPM_TRY(batch_plan(b, f32, R, dbl, s, &plan));
  KPM_TRY(ensure(ws.part, (size_t)plan_part_elems(*plan, R) * sizeof(double2)));
  if (dbl) {
    KPM_TRY(ensure(ws.vr, vb));
    KPM_TRY(ensure(ws.red, (size_t)2 * b->n_inst * R * ((M + 1) / 2 + 1) * sizeof(double2) +
                               (size_t)b->n_inst * R * sizeof(double)));
    // scratch of the exact mu_1 (at most 64 partial blocks per instance and vector),
    // sized here because nothing may allocate while the graph is being recorded
    if (f32) KPM_TRY(ensure(ws.tc, (size_t)b->n_inst * 64 * R * sizeof(double2)));
  }
  // inputs into the internal buffers (outside the graph)
  batch_pack_kernel<<<grid1(h->n_pad * R), 256, 0, s>>>(reinterpret_cast<const double2*>(v), b->d_off, b->d_poff,
                                                         b->d_rows, b->n_inst, b->n_total, h->n_pad, R, f32, ws.ta.p);
  KPM_CUDA_TRY(cudaGetLastError());
  KPM_CUDA_TRY(cudaMemcpyAsync(ws.vl.p, ws.ta.p, vb, cudaMemcpyDeviceToDevice, s));
  if (dbl) {
    KPM_TRY(half_norms(ws.ta.p, f32, h->n_pad, R, ws.vr.p, s));
    // per (instance, vector) corrections, stored after the reduced sets: [n_inst][R]
    const int K = (M + 1) / 2;
    double* corr = reinterpret_cast<double*>(static_cast<double2*>(ws.red.p) + (size_t)2 * b->n_inst * R * (K + 1));
    KPM_TRY(doubling_corr(ws.ta.p, ws.vr.p, f32, h->n_pad, R, b->d_poff, b->n_inst, corr, s));
  }
  // the recursion: one graph launch (re-recorded if a workspace buffer moved)
  const void* bufs[8] = {ws.ta.p, ws.tb.p, ws.vl.p, ws.part.p, b->mu_int.p, dbl ? ws.vr.p : nullptr,
                         dbl ? ws.red.p : nullptr, (dbl && f32) ? ws.tc.p : nullptr};
  cudaGraphExec_t exec = nullptr;
  for (size_t i = 0; i < b->graphs.size(); ++i) {
    auto& g = b->graphs[i];
    if (g.f32 == (int)f32 && g.R == R && g.M == M && g.kind == plan->kind && g.dbl == (int)dbl) {
      if (std::equal(bufs, bufs + 8, g.bufs)) {
        exec = g.exec;
      } else {
        cudaGraphExecDestroy(g.exec);
        b->graphs.erase(b->graphs.begin() + i);
      }
      break;
    }
  }
  const bool use_graph = getenv("KPM_NO_GRAPH") == nullptr;
  if (!use_graph) {
    KPM_TRY(record_batched(b, f32, R, M, *plan, s));
  } else {
    if (!exec) {
      cudaStream_t cs;
      KPM_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
      cudaGraph_t graph;
      KPM_CUDA_TRY(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
      const int rc = record_batched(b, f32, R, M, *plan, cs);
      const cudaError_t ec = cudaStreamEndCapture(cs, &graph);
      cudaStreamDestroy(cs);
      if (rc != KPM_OK) return rc;
      KPM_CUDA_TRY(ec);
      const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      KPM_CUDA_TRY(ei);
      kpm_batch_s::G g;
      g.f32 = (int)f32;
      g.R = R;
      g.M = M;
      g.kind = plan->kind;
      g.dbl = (int)dbl;
      std::copy(bufs, bufs + 8, g.bufs);
      g.exec = exec;
      b->graphs.push_back(g);
    }
    KPM_CUDA_TRY(cudaGraphLaunch(exec, s));
  }
  KPM_CUDA_TRY(cudaMemcpyAsync(mu, b->mu_int.p, (size_t)b->n_inst * R * M * sizeof(double2), cudaMemcpyDeviceToDevice, s));
  return KPM_OK;
}

int kpm_batch_props(const kpm_batch* b, int* hermitian, int* doubling) {
  if (!b) return KPM_ERR_INVALID_ARG;
  return kpm_ell_props(b->op, hermitian, doubling);
}

int kpm_batch_set_doubling(kpm_batch* b, int on) {
  if (!b) return KPM_ERR_INVALID_ARG;
  return kpm_ell_set_doubling(b->op, on);
}

int kpm_batch_check(kpm_batch* b, void* stream) {
  if (!b) return KPM_ERR_INVALID_ARG;
  return kpm_ell_check(b->op, stream);
}

}  // extern "C"
