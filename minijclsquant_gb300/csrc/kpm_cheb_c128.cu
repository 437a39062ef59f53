// Complex128 instantiations of the step kernels (the drop-in form).
#include "kpm_staged.cuh"
#include "kpm_ws.cuh"

namespace kpm {

int launch_step_f64(bool real, int R, int mode, int epi, const StepParams& p, int grid, cudaStream_t s) {
  switch (R) {
    case 1:
      return real ? launch_mode_epi<double, true, 1, 1>(mode, epi, p, grid, s)
                  : launch_mode_epi<double, false, 1, 1>(mode, epi, p, grid, s);
    case 2:
      return real ? launch_mode_epi<double, true, 2, 1>(mode, epi, p, grid, s)
                  : launch_mode_epi<double, false, 2, 1>(mode, epi, p, grid, s);
    case 4:
      return real ? launch_mode_epi<double, true, 4, 1>(mode, epi, p, grid, s)
                  : launch_mode_epi<double, false, 4, 1>(mode, epi, p, grid, s);
    case 8:
      return real ? launch_mode_epi<double, true, 8, 1>(mode, epi, p, grid, s)
                  : launch_mode_epi<double, false, 8, 1>(mode, epi, p, grid, s);
    default:
      return KPM_ERR_UNSUPPORTED;
  }
}

int launch_staged_f64(bool real, int R, int U, const StepParams& p, int grid, cudaStream_t s) {
  return Staged<double>::launch(real, R, U, p, grid, s);
}

int staged_ctas_f64(bool real, int R, int U, int L, int nvec) {
  return Staged<double>::ctas_per_sm(real, R, U, L, nvec);
}

int launch_ws_f64(bool real, int R, int U, const StepParams& p, int grid, cudaStream_t s, int sb) {
  return Ws<double>::launch(real, R, U, p, grid, s, sb);
}

int ws_ctas_f64(bool real, int R, int U, int L, int nvec, bool ff, int sb) {
  (void)nvec;
  return Ws<double>::ctas_per_sm(real, R, U, L, ff, sb);
}


}  // namespace kpm
