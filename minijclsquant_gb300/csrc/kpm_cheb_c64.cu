// Complex64 instantiations of the step kernels (mixed precision: complex64
// vectors and values, FP64 moment accumulation).  Two complex64 values per
// thread make every access a 16-byte vector load.
#include "kpm_staged.cuh"
#include "kpm_ws.cuh"

namespace kpm {

int launch_step_f32(bool real, int R, int mode, int epi, const StepParams& p, int grid, cudaStream_t s) {
  switch (R) {
    case 1:
      return real ? launch_mode_epi<float, true, 1, 1>(mode, epi, p, grid, s)
                  : launch_mode_epi<float, false, 1, 1>(mode, epi, p, grid, s);
    case 2:
      return real ? launch_mode_epi<float, true, 1, 2>(mode, epi, p, grid, s)
                  : launch_mode_epi<float, false, 1, 2>(mode, epi, p, grid, s);
    case 4:
      return real ? launch_mode_epi<float, true, 2, 2>(mode, epi, p, grid, s)
                  : launch_mode_epi<float, false, 2, 2>(mode, epi, p, grid, s);
    case 8:
      return real ? launch_mode_epi<float, true, 4, 2>(mode, epi, p, grid, s)
                  : launch_mode_epi<float, false, 4, 2>(mode, epi, p, grid, s);
    default:
      return KPM_ERR_UNSUPPORTED;
  }
}

int launch_staged_f32(bool real, int R, int U, const StepParams& p, int grid, cudaStream_t s) {
  return Staged<float>::launch(real, R, U, p, grid, s);
}

int staged_ctas_f32(bool real, int R, int U, int L, int nvec) {
  return Staged<float>::ctas_per_sm(real, R, U, L, nvec);
}

int launch_ws_f32(bool real, int R, int U, const StepParams& p, int grid, cudaStream_t s) {
  return Ws<float>::launch(real, R, U, p, grid, s);
}

int ws_ctas_f32(bool real, int R, int U, int L, int nvec) {
  (void)nvec;
  return Ws<float>::ctas_per_sm(real, R, U, L);
}

}  // namespace kpm
