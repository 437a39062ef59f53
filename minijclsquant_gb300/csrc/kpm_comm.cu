// kpm_comm.cu -- fused commutator-series step (complex128).
//
// One launch advances both recursions of rec_com_A_vec
// (jclsquant/recurrence_functions.py:146-196; device version
// jclsquant/cuda_cython/cuda/recursions.cu:319-388) by one order:
//
//   C_{m} = 2H C_{m-1} - C_{m-2} + 2V T_{m-1}     (in place over C_{m-2})
//   T_{m} = 2H T_{m-1} - T_{m-2}                  (in place over T_{m-2})
//   acc  += c_m C_m
//
// and at m = 1: T_1 = H v, C_1 = V v, acc = c_1 C_1 (C_0 = 0).
// The reference needs three SpMV launches and one axpy per order; here every
// operator entry and every vector entry is touched once per order.
//
// The table form (TAB) serves rec_com_A_vec_tab (jclsquant/recurrence_functions.py:
// 202-250): instead of the accumulator it writes c_m C_m as row m of the caller's
// [R][M][n] table, straight from registers in the caller's unpacked layout.
#include "kpm_cheb.cuh"

namespace kpm {

struct CommParams {
  const void* val_h;
  const int32_t* col_h;
  const void* val_v;
  const int32_t* col_v;
  int64_t ld;
  int Lh, Lv;
  int64_t n_pad;
  const double2* tcur;  // T_{m-1}            [n_pad][R]
  double2* tout;        // T_{m-2} -> T_m
  const double2* ccur;  // C_{m-1}
  double2* cout;        // C_{m-2} -> C_m (FIRST: C_1)
  double2* acc;         // series accumulator
  const double2* coef;
  int m;
  // TAB: out[(r0 + r) * tab_vstride + m * n + row] = c_m C_m for rows < n
  double2* tab;
  int64_t n;
  int64_t tab_vstride;
  int r0;
};

template <bool RH, bool RV, int R, bool FIRST, bool TAB>
__global__ void __launch_bounds__(kBlock) comm_step_kernel(const CommParams p) {
  using MVH = typename MatV<double, RH>::type;
  using MVV = typename MatV<double, RV>::type;
  constexpr int RPB = kBlock / R;
  const int sub = threadIdx.x % R;
  const int rl = threadIdx.x / R;
  const MVH* __restrict__ vh = static_cast<const MVH*>(p.val_h);
  const MVV* __restrict__ vv = static_cast<const MVV*>(p.val_v);
  const double2 cm = p.coef[p.m];
  const int64_t stride = (int64_t)gridDim.x * RPB;
  for (int64_t row = (int64_t)blockIdx.x * RPB + rl; row < p.n_pad; row += stride) {
    const int64_t vi = row * R + sub;
    Cx<double, 1> t, c, x;
    if (FIRST) {
      t.re[0] = t.im[0] = 0.0;
      c.re[0] = c.im[0] = 0.0;
    } else {
      const double2 to = p.tout[vi];
      const double2 co = p.cout[vi];
      t.re[0] = -to.x; t.im[0] = -to.y;
      c.re[0] = -co.x; c.im[0] = -co.y;
    }
    for (int s = 0; s < p.Lh; ++s) {
      const int j = __ldcs(p.col_h + (int64_t)s * p.ld + row);
      const MVH hv = __ldcs(vh + (int64_t)s * p.ld + row);
      unpack(__ldg(p.tcur + (int64_t)j * R + sub), x);
      madd(t, hv, x);
      if (!FIRST) {
        unpack(__ldg(p.ccur + (int64_t)j * R + sub), x);
        madd(c, hv, x);
      }
    }
    for (int s = 0; s < p.Lv; ++s) {
      const int j = __ldcs(p.col_v + (int64_t)s * p.ld + row);
      const MVV w = __ldcs(vv + (int64_t)s * p.ld + row);
      unpack(__ldg(p.tcur + (int64_t)j * R + sub), x);
      madd(c, w, x);
    }
    if (FIRST) {
      t.re[0] *= 0.5; t.im[0] *= 0.5;
      c.re[0] *= 0.5; c.im[0] *= 0.5;
    }
    p.tout[vi] = pack(t);
    p.cout[vi] = pack(c);
    if (TAB) {
      if (row < p.n)
        p.tab[(int64_t)(p.r0 + sub) * p.tab_vstride + (int64_t)p.m * p.n + row] =
            make_double2(cm.x * c.re[0] - cm.y * c.im[0], cm.x * c.im[0] + cm.y * c.re[0]);
      continue;
    }
    double2 a;
    if (FIRST) {
      a = make_double2(cm.x * c.re[0] - cm.y * c.im[0], cm.x * c.im[0] + cm.y * c.re[0]);
    } else {  // acc += c_m C_m as two nested FMAs per component
      a = p.acc[vi];
      a.x = fma(cm.x, c.re[0], fma(-cm.y, c.im[0], a.x));
      a.y = fma(cm.x, c.im[0], fma(cm.y, c.re[0], a.y));
    }
    p.acc[vi] = a;
  }
}

template <bool RH, bool RV, int R>
static int launch_comm_r(bool first, const CommParams& p, int grid, cudaStream_t s) {
  const bool tab = p.tab != nullptr;
  if (first && tab)
    comm_step_kernel<RH, RV, R, true, true><<<grid, kBlock, 0, s>>>(p);
  else if (first)
    comm_step_kernel<RH, RV, R, true, false><<<grid, kBlock, 0, s>>>(p);
  else if (tab)
    comm_step_kernel<RH, RV, R, false, true><<<grid, kBlock, 0, s>>>(p);
  else
    comm_step_kernel<RH, RV, R, false, false><<<grid, kBlock, 0, s>>>(p);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_last_cuda_error(e);
    return KPM_ERR_CUDA;
  }
  return KPM_OK;
}

template <bool RH, bool RV>
static int launch_comm_hv(int R, bool first, const CommParams& p, int grid, cudaStream_t s) {
  switch (R) {
    case 1: return launch_comm_r<RH, RV, 1>(first, p, grid, s);
    case 2: return launch_comm_r<RH, RV, 2>(first, p, grid, s);
    case 4: return launch_comm_r<RH, RV, 4>(first, p, grid, s);
    case 8: return launch_comm_r<RH, RV, 8>(first, p, grid, s);
    default: return KPM_ERR_UNSUPPORTED;
  }
}

static int launch_comm(bool rh, bool rv, int R, bool first, const CommParams& p, int grid, cudaStream_t s) {
  if (rh && rv) return launch_comm_hv<true, true>(R, first, p, grid, s);
  if (rh && !rv) return launch_comm_hv<true, false>(R, first, p, grid, s);
  if (!rh && rv) return launch_comm_hv<false, true>(R, first, p, grid, s);
  return launch_comm_hv<false, false>(R, first, p, grid, s);
}

// Commutator series on one packed group: x ([n_pad][Rg] c128) in, result
// written to `result` ([n_pad][Rg] c128).  Uses ws.ta..td of h.
// With tab != nullptr the rows c_m C_m, m = 1 .. M-1, of vectors r0 .. r0+Rg-1 are written
// into tab ([R][M][n] c128, unpacked) instead, and `result` is not touched; row 0
// (c_0 C_0 = 0) is the caller's.
int comm_series_packed(kpm_ell_s* h, kpm_ell_s* v, int Rg, int M, const double2* coef, const double2* x,
                       double2* result, cudaStream_t s, double2* tab, int r0) {
  const size_t vb = (size_t)h->n_pad * Rg * sizeof(double2);
  KPM_TRY(ensure(h->ws.tc, vb));
  KPM_TRY(ensure(h->ws.td, vb));
  KPM_TRY(ensure(h->ws.ta, vb));
  double2* t_a = static_cast<double2*>(h->ws.ta.p);  // T_{m-2} slot
  double2* t_b = static_cast<double2*>(h->ws.tc.p);  // T_{m-1} slot
  double2* c_a = static_cast<double2*>(h->ws.td.p);  // C_{m-2} slot
  double2* c_b = result;                               // C_{m-1} slot is written into `result`'s partner
  // `result` doubles as the series accumulator; C needs two more buffers.
  KPM_TRY(ensure(h->ws.acc2, vb));
  c_b = static_cast<double2*>(h->ws.acc2.p);
  KPM_CUDA_TRY(cudaMemcpyAsync(t_a, x, vb, cudaMemcpyDeviceToDevice, s));
  const int grid = grid_for(h, Rg, 1);
  CommParams p;
  p.val_h = h->val64;
  p.col_h = h->col;
  p.val_v = v->val64;
  p.col_v = v->col;
  p.ld = h->n_pad;
  p.Lh = h->L;
  p.Lv = v->L;
  p.n_pad = h->n_pad;
  p.coef = coef;
  p.acc = result;
  p.tab = tab;
  p.n = h->n;
  p.tab_vstride = (int64_t)M * h->n;
  p.r0 = r0;
  // m = 1: T_1 = H v -> t_b ; C_1 = V v -> c_b ; acc = c_1 C_1
  p.tcur = t_a;
  p.tout = t_b;
  p.ccur = nullptr;
  p.cout = c_b;
  p.m = 1;
  KPM_TRY(launch_comm(h->is_real, v->is_real, Rg, true, p, grid, s));
  // C_0 = 0 lives in c_a.
  KPM_CUDA_TRY(cudaMemsetAsync(c_a, 0, vb, s));
  double2 *tp = t_a, *tc = t_b, *cp = c_a, *cc = c_b;
  for (int m = 2; m < M; ++m) {
    p.tcur = tc;
    p.tout = tp;
    p.ccur = cc;
    p.cout = cp;
    p.m = m;
    KPM_TRY(launch_comm(h->is_real, v->is_real, Rg, false, p, grid, s));
    double2* t = tp; tp = tc; tc = t;
    t = cp; cp = cc; cc = t;
  }
  return KPM_OK;
}

}  // namespace kpm
