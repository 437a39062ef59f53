// kpm_driven.cu -- time-dependent operators of driven systems on the device.
//
//   kpm_light_modifier : the Peierls substitution of a light pulse, the four forms of
//       light_modifier_cython (jclsquant/cython_modules/Extra_funs.pyx:236-342):
//         data_new = a * data * exp(i A0 (cx dx + cy dy) / ch)
//       with (cx, cy) = (0, sin wt) (linear) or (cos wt, eta sin wt) (circular), and
//       ch = cosh((t - 2 Tp) / (0.5673 Tp)) for the packed (pulse) forms, 1 otherwise.
//   kpm_ell_light_update : the same H(t) written straight into an operator's stored
//       values (the doubled SoA layout of kpm_ell_create), so a time-stepping caller
//       rewrites H(t) in one pass on the device instead of through host arrays.
//   kpm_phonon_modifier : hopping_pos_phonons_modifier (Extra_funs.pyx:540-560): bond
//       vectors displaced by a damped phonon, hoppings scaled by exp(-b (|d| / a0 - 1)).
//
// The time-dependent scalars (cos wt, sin wt, the pulse envelope) are evaluated once on
// the host in complex double arithmetic, as the reference evaluates them per element;
// per element the kernels do complex multiplies and one complex exponential
// exp(x + iy) = e^x (cos y + i sin y).  The light kernels take sin y and cos y from a
// 256-entry table and short polynomials (sincos_tab): the FP64 pipe, 1/64 of the FP32
// rate on GB300, bounds these kernels, and the table form needs fewer FP64 instructions.
// They run once per time step (recomputing the phases inside every recursion step would
// add that work per slot per step to an FP64-bound kernel).
#include <algorithm>
#include <cmath>
#include <complex>
#include <mutex>

#include "kpm_internal.cuh"

using namespace kpm;

namespace {

using cplx = std::complex<double>;

inline cudaStream_t stream_of(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline cplx param(const double* p, int k) { return cplx(p[2 * k], p[2 * k + 1]); }
inline double2 d2(cplx z) { return make_double2(z.real(), z.imag()); }

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 cexp2(double2 z) {
  double s, c;
  sincos(z.y, &s, &c);
  const double e = z.x == 0.0 ? 1.0 : exp(z.x);  // a pure phase (real pulse parameters): exp(0) = 1
  return make_double2(e * c, e * s);
}
// (sin, cos)(2 pi k / 256), k = 0 .. 255: each entry is the exact value rounded to the nearest
// double (computed in 60-digit arithmetic; a CPU test recomputes every entry).  A file-scope
// device constant: the kernels read it directly, so a light update needs no set-up.
__device__ const double2 g_sincos_tab[256] = {
    {0.0, 0x1.0000000000000p+0},
    {0x1.92155f7a3667ep-6, 0x1.ffd886084cd0dp-1},
    {0x1.91f65f10dd814p-5, 0x1.ff621e3796d7ep-1},
    {0x1.2d52092ce19f6p-4, 0x1.fe9cdad01883ap-1},
    {0x1.917a6bc29b42cp-4, 0x1.fd88da3d12526p-1},
    {0x1.f564e56a9730ep-4, 0x1.fc26470e19fd3p-1},
    {0x1.2c8106e8e613ap-3, 0x1.fa7557f08a517p-1},
    {0x1.5e214448b3fc6p-3, 0x1.f8764fa714ba9p-1},
    {0x1.8f8b83c69a60bp-3, 0x1.f6297cff75cb0p-1},
    {0x1.c0b826a7e4f63p-3, 0x1.f38f3ac64e589p-1},
    {0x1.f19f97b215f1bp-3, 0x1.f0a7efb9230d7p-1},
    {0x1.111d262b1f677p-2, 0x1.ed740e7684963p-1},
    {0x1.294062ed59f06p-2, 0x1.e9f4156c62ddap-1},
    {0x1.4135c94176601p-2, 0x1.e6288ec48e112p-1},
    {0x1.58f9a75ab1fddp-2, 0x1.e212104f686e5p-1},
    {0x1.7088530fa459fp-2, 0x1.ddb13b6ccc23cp-1},
    {0x1.87de2a6aea963p-2, 0x1.d906bcf328d46p-1},
    {0x1.9ef7943a8ed8ap-2, 0x1.d4134d14dc93ap-1},
    {0x1.b5d1009e15cc0p-2, 0x1.ced7af43cc773p-1},
    {0x1.cc66e9931c45ep-2, 0x1.c954b213411f5p-1},
    {0x1.e2b5d3806f63bp-2, 0x1.c38b2f180bdb1p-1},
    {0x1.f8ba4dbf89abap-2, 0x1.bd7c0ac6f952ap-1},
    {0x1.073879922ffeep-1, 0x1.b728345196e3ep-1},
    {0x1.11eb3541b4b23p-1, 0x1.b090a58150200p-1},
    {0x1.1c73b39ae68c8p-1, 0x1.a9b66290ea1a3p-1},
    {0x1.26d054cdd12dfp-1, 0x1.a29a7a0462782p-1},
    {0x1.30ff7fce17035p-1, 0x1.9b3e047f38741p-1},
    {0x1.3affa292050b9p-1, 0x1.93a22499263fbp-1},
    {0x1.44cf325091dd6p-1, 0x1.8bc806b151741p-1},
    {0x1.4e6cabbe3e5e9p-1, 0x1.83b0e0bff976ep-1},
    {0x1.57d69348ceca0p-1, 0x1.7b5df226aafafp-1},
    {0x1.610b7551d2cdfp-1, 0x1.72d0837efff96p-1},
    {0x1.6a09e667f3bcdp-1, 0x1.6a09e667f3bcdp-1},
    {0x1.72d0837efff96p-1, 0x1.610b7551d2cdfp-1},
    {0x1.7b5df226aafafp-1, 0x1.57d69348ceca0p-1},
    {0x1.83b0e0bff976ep-1, 0x1.4e6cabbe3e5e9p-1},
    {0x1.8bc806b151741p-1, 0x1.44cf325091dd6p-1},
    {0x1.93a22499263fbp-1, 0x1.3affa292050b9p-1},
    {0x1.9b3e047f38741p-1, 0x1.30ff7fce17035p-1},
    {0x1.a29a7a0462782p-1, 0x1.26d054cdd12dfp-1},
    {0x1.a9b66290ea1a3p-1, 0x1.1c73b39ae68c8p-1},
    {0x1.b090a58150200p-1, 0x1.11eb3541b4b23p-1},
    {0x1.b728345196e3ep-1, 0x1.073879922ffeep-1},
    {0x1.bd7c0ac6f952ap-1, 0x1.f8ba4dbf89abap-2},
    {0x1.c38b2f180bdb1p-1, 0x1.e2b5d3806f63bp-2},
    {0x1.c954b213411f5p-1, 0x1.cc66e9931c45ep-2},
    {0x1.ced7af43cc773p-1, 0x1.b5d1009e15cc0p-2},
    {0x1.d4134d14dc93ap-1, 0x1.9ef7943a8ed8ap-2},
    {0x1.d906bcf328d46p-1, 0x1.87de2a6aea963p-2},
    {0x1.ddb13b6ccc23cp-1, 0x1.7088530fa459fp-2},
    {0x1.e212104f686e5p-1, 0x1.58f9a75ab1fddp-2},
    {0x1.e6288ec48e112p-1, 0x1.4135c94176601p-2},
    {0x1.e9f4156c62ddap-1, 0x1.294062ed59f06p-2},
    {0x1.ed740e7684963p-1, 0x1.111d262b1f677p-2},
    {0x1.f0a7efb9230d7p-1, 0x1.f19f97b215f1bp-3},
    {0x1.f38f3ac64e589p-1, 0x1.c0b826a7e4f63p-3},
    {0x1.f6297cff75cb0p-1, 0x1.8f8b83c69a60bp-3},
    {0x1.f8764fa714ba9p-1, 0x1.5e214448b3fc6p-3},
    {0x1.fa7557f08a517p-1, 0x1.2c8106e8e613ap-3},
    {0x1.fc26470e19fd3p-1, 0x1.f564e56a9730ep-4},
    {0x1.fd88da3d12526p-1, 0x1.917a6bc29b42cp-4},
    {0x1.fe9cdad01883ap-1, 0x1.2d52092ce19f6p-4},
    {0x1.ff621e3796d7ep-1, 0x1.91f65f10dd814p-5},
    {0x1.ffd886084cd0dp-1, 0x1.92155f7a3667ep-6},
    {0x1.0000000000000p+0, 0.0},
    {0x1.ffd886084cd0dp-1, -0x1.92155f7a3667ep-6},
    {0x1.ff621e3796d7ep-1, -0x1.91f65f10dd814p-5},
    {0x1.fe9cdad01883ap-1, -0x1.2d52092ce19f6p-4},
    {0x1.fd88da3d12526p-1, -0x1.917a6bc29b42cp-4},
    {0x1.fc26470e19fd3p-1, -0x1.f564e56a9730ep-4},
    {0x1.fa7557f08a517p-1, -0x1.2c8106e8e613ap-3},
    {0x1.f8764fa714ba9p-1, -0x1.5e214448b3fc6p-3},
    {0x1.f6297cff75cb0p-1, -0x1.8f8b83c69a60bp-3},
    {0x1.f38f3ac64e589p-1, -0x1.c0b826a7e4f63p-3},
    {0x1.f0a7efb9230d7p-1, -0x1.f19f97b215f1bp-3},
    {0x1.ed740e7684963p-1, -0x1.111d262b1f677p-2},
    {0x1.e9f4156c62ddap-1, -0x1.294062ed59f06p-2},
    {0x1.e6288ec48e112p-1, -0x1.4135c94176601p-2},
    {0x1.e212104f686e5p-1, -0x1.58f9a75ab1fddp-2},
    {0x1.ddb13b6ccc23cp-1, -0x1.7088530fa459fp-2},
    {0x1.d906bcf328d46p-1, -0x1.87de2a6aea963p-2},
    {0x1.d4134d14dc93ap-1, -0x1.9ef7943a8ed8ap-2},
    {0x1.ced7af43cc773p-1, -0x1.b5d1009e15cc0p-2},
    {0x1.c954b213411f5p-1, -0x1.cc66e9931c45ep-2},
    {0x1.c38b2f180bdb1p-1, -0x1.e2b5d3806f63bp-2},
    {0x1.bd7c0ac6f952ap-1, -0x1.f8ba4dbf89abap-2},
    {0x1.b728345196e3ep-1, -0x1.073879922ffeep-1},
    {0x1.b090a58150200p-1, -0x1.11eb3541b4b23p-1},
    {0x1.a9b66290ea1a3p-1, -0x1.1c73b39ae68c8p-1},
    {0x1.a29a7a0462782p-1, -0x1.26d054cdd12dfp-1},
    {0x1.9b3e047f38741p-1, -0x1.30ff7fce17035p-1},
    {0x1.93a22499263fbp-1, -0x1.3affa292050b9p-1},
    {0x1.8bc806b151741p-1, -0x1.44cf325091dd6p-1},
    {0x1.83b0e0bff976ep-1, -0x1.4e6cabbe3e5e9p-1},
    {0x1.7b5df226aafafp-1, -0x1.57d69348ceca0p-1},
    {0x1.72d0837efff96p-1, -0x1.610b7551d2cdfp-1},
    {0x1.6a09e667f3bcdp-1, -0x1.6a09e667f3bcdp-1},
    {0x1.610b7551d2cdfp-1, -0x1.72d0837efff96p-1},
    {0x1.57d69348ceca0p-1, -0x1.7b5df226aafafp-1},
    {0x1.4e6cabbe3e5e9p-1, -0x1.83b0e0bff976ep-1},
    {0x1.44cf325091dd6p-1, -0x1.8bc806b151741p-1},
    {0x1.3affa292050b9p-1, -0x1.93a22499263fbp-1},
    {0x1.30ff7fce17035p-1, -0x1.9b3e047f38741p-1},
    {0x1.26d054cdd12dfp-1, -0x1.a29a7a0462782p-1},
    {0x1.1c73b39ae68c8p-1, -0x1.a9b66290ea1a3p-1},
    {0x1.11eb3541b4b23p-1, -0x1.b090a58150200p-1},
    {0x1.073879922ffeep-1, -0x1.b728345196e3ep-1},
    {0x1.f8ba4dbf89abap-2, -0x1.bd7c0ac6f952ap-1},
    {0x1.e2b5d3806f63bp-2, -0x1.c38b2f180bdb1p-1},
    {0x1.cc66e9931c45ep-2, -0x1.c954b213411f5p-1},
    {0x1.b5d1009e15cc0p-2, -0x1.ced7af43cc773p-1},
    {0x1.9ef7943a8ed8ap-2, -0x1.d4134d14dc93ap-1},
    {0x1.87de2a6aea963p-2, -0x1.d906bcf328d46p-1},
    {0x1.7088530fa459fp-2, -0x1.ddb13b6ccc23cp-1},
    {0x1.58f9a75ab1fddp-2, -0x1.e212104f686e5p-1},
    {0x1.4135c94176601p-2, -0x1.e6288ec48e112p-1},
    {0x1.294062ed59f06p-2, -0x1.e9f4156c62ddap-1},
    {0x1.111d262b1f677p-2, -0x1.ed740e7684963p-1},
    {0x1.f19f97b215f1bp-3, -0x1.f0a7efb9230d7p-1},
    {0x1.c0b826a7e4f63p-3, -0x1.f38f3ac64e589p-1},
    {0x1.8f8b83c69a60bp-3, -0x1.f6297cff75cb0p-1},
    {0x1.5e214448b3fc6p-3, -0x1.f8764fa714ba9p-1},
    {0x1.2c8106e8e613ap-3, -0x1.fa7557f08a517p-1},
    {0x1.f564e56a9730ep-4, -0x1.fc26470e19fd3p-1},
    {0x1.917a6bc29b42cp-4, -0x1.fd88da3d12526p-1},
    {0x1.2d52092ce19f6p-4, -0x1.fe9cdad01883ap-1},
    {0x1.91f65f10dd814p-5, -0x1.ff621e3796d7ep-1},
    {0x1.92155f7a3667ep-6, -0x1.ffd886084cd0dp-1},
    {0.0, -0x1.0000000000000p+0},
    {-0x1.92155f7a3667ep-6, -0x1.ffd886084cd0dp-1},
    {-0x1.91f65f10dd814p-5, -0x1.ff621e3796d7ep-1},
    {-0x1.2d52092ce19f6p-4, -0x1.fe9cdad01883ap-1},
    {-0x1.917a6bc29b42cp-4, -0x1.fd88da3d12526p-1},
    {-0x1.f564e56a9730ep-4, -0x1.fc26470e19fd3p-1},
    {-0x1.2c8106e8e613ap-3, -0x1.fa7557f08a517p-1},
    {-0x1.5e214448b3fc6p-3, -0x1.f8764fa714ba9p-1},
    {-0x1.8f8b83c69a60bp-3, -0x1.f6297cff75cb0p-1},
    {-0x1.c0b826a7e4f63p-3, -0x1.f38f3ac64e589p-1},
    {-0x1.f19f97b215f1bp-3, -0x1.f0a7efb9230d7p-1},
    {-0x1.111d262b1f677p-2, -0x1.ed740e7684963p-1},
    {-0x1.294062ed59f06p-2, -0x1.e9f4156c62ddap-1},
    {-0x1.4135c94176601p-2, -0x1.e6288ec48e112p-1},
    {-0x1.58f9a75ab1fddp-2, -0x1.e212104f686e5p-1},
    {-0x1.7088530fa459fp-2, -0x1.ddb13b6ccc23cp-1},
    {-0x1.87de2a6aea963p-2, -0x1.d906bcf328d46p-1},
    {-0x1.9ef7943a8ed8ap-2, -0x1.d4134d14dc93ap-1},
    {-0x1.b5d1009e15cc0p-2, -0x1.ced7af43cc773p-1},
    {-0x1.cc66e9931c45ep-2, -0x1.c954b213411f5p-1},
    {-0x1.e2b5d3806f63bp-2, -0x1.c38b2f180bdb1p-1},
    {-0x1.f8ba4dbf89abap-2, -0x1.bd7c0ac6f952ap-1},
    {-0x1.073879922ffeep-1, -0x1.b728345196e3ep-1},
    {-0x1.11eb3541b4b23p-1, -0x1.b090a58150200p-1},
    {-0x1.1c73b39ae68c8p-1, -0x1.a9b66290ea1a3p-1},
    {-0x1.26d054cdd12dfp-1, -0x1.a29a7a0462782p-1},
    {-0x1.30ff7fce17035p-1, -0x1.9b3e047f38741p-1},
    {-0x1.3affa292050b9p-1, -0x1.93a22499263fbp-1},
    {-0x1.44cf325091dd6p-1, -0x1.8bc806b151741p-1},
    {-0x1.4e6cabbe3e5e9p-1, -0x1.83b0e0bff976ep-1},
    {-0x1.57d69348ceca0p-1, -0x1.7b5df226aafafp-1},
    {-0x1.610b7551d2cdfp-1, -0x1.72d0837efff96p-1},
    {-0x1.6a09e667f3bcdp-1, -0x1.6a09e667f3bcdp-1},
    {-0x1.72d0837efff96p-1, -0x1.610b7551d2cdfp-1},
    {-0x1.7b5df226aafafp-1, -0x1.57d69348ceca0p-1},
    {-0x1.83b0e0bff976ep-1, -0x1.4e6cabbe3e5e9p-1},
    {-0x1.8bc806b151741p-1, -0x1.44cf325091dd6p-1},
    {-0x1.93a22499263fbp-1, -0x1.3affa292050b9p-1},
    {-0x1.9b3e047f38741p-1, -0x1.30ff7fce17035p-1},
    {-0x1.a29a7a0462782p-1, -0x1.26d054cdd12dfp-1},
    {-0x1.a9b66290ea1a3p-1, -0x1.1c73b39ae68c8p-1},
    {-0x1.b090a58150200p-1, -0x1.11eb3541b4b23p-1},
    {-0x1.b728345196e3ep-1, -0x1.073879922ffeep-1},
    {-0x1.bd7c0ac6f952ap-1, -0x1.f8ba4dbf89abap-2},
    {-0x1.c38b2f180bdb1p-1, -0x1.e2b5d3806f63bp-2},
    {-0x1.c954b213411f5p-1, -0x1.cc66e9931c45ep-2},
    {-0x1.ced7af43cc773p-1, -0x1.b5d1009e15cc0p-2},
    {-0x1.d4134d14dc93ap-1, -0x1.9ef7943a8ed8ap-2},
    {-0x1.d906bcf328d46p-1, -0x1.87de2a6aea963p-2},
    {-0x1.ddb13b6ccc23cp-1, -0x1.7088530fa459fp-2},
    {-0x1.e212104f686e5p-1, -0x1.58f9a75ab1fddp-2},
    {-0x1.e6288ec48e112p-1, -0x1.4135c94176601p-2},
    {-0x1.e9f4156c62ddap-1, -0x1.294062ed59f06p-2},
    {-0x1.ed740e7684963p-1, -0x1.111d262b1f677p-2},
    {-0x1.f0a7efb9230d7p-1, -0x1.f19f97b215f1bp-3},
    {-0x1.f38f3ac64e589p-1, -0x1.c0b826a7e4f63p-3},
    {-0x1.f6297cff75cb0p-1, -0x1.8f8b83c69a60bp-3},
    {-0x1.f8764fa714ba9p-1, -0x1.5e214448b3fc6p-3},
    {-0x1.fa7557f08a517p-1, -0x1.2c8106e8e613ap-3},
    {-0x1.fc26470e19fd3p-1, -0x1.f564e56a9730ep-4},
    {-0x1.fd88da3d12526p-1, -0x1.917a6bc29b42cp-4},
    {-0x1.fe9cdad01883ap-1, -0x1.2d52092ce19f6p-4},
    {-0x1.ff621e3796d7ep-1, -0x1.91f65f10dd814p-5},
    {-0x1.ffd886084cd0dp-1, -0x1.92155f7a3667ep-6},
    {-0x1.0000000000000p+0, 0.0},
    {-0x1.ffd886084cd0dp-1, 0x1.92155f7a3667ep-6},
    {-0x1.ff621e3796d7ep-1, 0x1.91f65f10dd814p-5},
    {-0x1.fe9cdad01883ap-1, 0x1.2d52092ce19f6p-4},
    {-0x1.fd88da3d12526p-1, 0x1.917a6bc29b42cp-4},
    {-0x1.fc26470e19fd3p-1, 0x1.f564e56a9730ep-4},
    {-0x1.fa7557f08a517p-1, 0x1.2c8106e8e613ap-3},
    {-0x1.f8764fa714ba9p-1, 0x1.5e214448b3fc6p-3},
    {-0x1.f6297cff75cb0p-1, 0x1.8f8b83c69a60bp-3},
    {-0x1.f38f3ac64e589p-1, 0x1.c0b826a7e4f63p-3},
    {-0x1.f0a7efb9230d7p-1, 0x1.f19f97b215f1bp-3},
    {-0x1.ed740e7684963p-1, 0x1.111d262b1f677p-2},
    {-0x1.e9f4156c62ddap-1, 0x1.294062ed59f06p-2},
    {-0x1.e6288ec48e112p-1, 0x1.4135c94176601p-2},
    {-0x1.e212104f686e5p-1, 0x1.58f9a75ab1fddp-2},
    {-0x1.ddb13b6ccc23cp-1, 0x1.7088530fa459fp-2},
    {-0x1.d906bcf328d46p-1, 0x1.87de2a6aea963p-2},
    {-0x1.d4134d14dc93ap-1, 0x1.9ef7943a8ed8ap-2},
    {-0x1.ced7af43cc773p-1, 0x1.b5d1009e15cc0p-2},
    {-0x1.c954b213411f5p-1, 0x1.cc66e9931c45ep-2},
    {-0x1.c38b2f180bdb1p-1, 0x1.e2b5d3806f63bp-2},
    {-0x1.bd7c0ac6f952ap-1, 0x1.f8ba4dbf89abap-2},
    {-0x1.b728345196e3ep-1, 0x1.073879922ffeep-1},
    {-0x1.b090a58150200p-1, 0x1.11eb3541b4b23p-1},
    {-0x1.a9b66290ea1a3p-1, 0x1.1c73b39ae68c8p-1},
    {-0x1.a29a7a0462782p-1, 0x1.26d054cdd12dfp-1},
    {-0x1.9b3e047f38741p-1, 0x1.30ff7fce17035p-1},
    {-0x1.93a22499263fbp-1, 0x1.3affa292050b9p-1},
    {-0x1.8bc806b151741p-1, 0x1.44cf325091dd6p-1},
    {-0x1.83b0e0bff976ep-1, 0x1.4e6cabbe3e5e9p-1},
    {-0x1.7b5df226aafafp-1, 0x1.57d69348ceca0p-1},
    {-0x1.72d0837efff96p-1, 0x1.610b7551d2cdfp-1},
    {-0x1.6a09e667f3bcdp-1, 0x1.6a09e667f3bcdp-1},
    {-0x1.610b7551d2cdfp-1, 0x1.72d0837efff96p-1},
    {-0x1.57d69348ceca0p-1, 0x1.7b5df226aafafp-1},
    {-0x1.4e6cabbe3e5e9p-1, 0x1.83b0e0bff976ep-1},
    {-0x1.44cf325091dd6p-1, 0x1.8bc806b151741p-1},
    {-0x1.3affa292050b9p-1, 0x1.93a22499263fbp-1},
    {-0x1.30ff7fce17035p-1, 0x1.9b3e047f38741p-1},
    {-0x1.26d054cdd12dfp-1, 0x1.a29a7a0462782p-1},
    {-0x1.1c73b39ae68c8p-1, 0x1.a9b66290ea1a3p-1},
    {-0x1.11eb3541b4b23p-1, 0x1.b090a58150200p-1},
    {-0x1.073879922ffeep-1, 0x1.b728345196e3ep-1},
    {-0x1.f8ba4dbf89abap-2, 0x1.bd7c0ac6f952ap-1},
    {-0x1.e2b5d3806f63bp-2, 0x1.c38b2f180bdb1p-1},
    {-0x1.cc66e9931c45ep-2, 0x1.c954b213411f5p-1},
    {-0x1.b5d1009e15cc0p-2, 0x1.ced7af43cc773p-1},
    {-0x1.9ef7943a8ed8ap-2, 0x1.d4134d14dc93ap-1},
    {-0x1.87de2a6aea963p-2, 0x1.d906bcf328d46p-1},
    {-0x1.7088530fa459fp-2, 0x1.ddb13b6ccc23cp-1},
    {-0x1.58f9a75ab1fddp-2, 0x1.e212104f686e5p-1},
    {-0x1.4135c94176601p-2, 0x1.e6288ec48e112p-1},
    {-0x1.294062ed59f06p-2, 0x1.e9f4156c62ddap-1},
    {-0x1.111d262b1f677p-2, 0x1.ed740e7684963p-1},
    {-0x1.f19f97b215f1bp-3, 0x1.f0a7efb9230d7p-1},
    {-0x1.c0b826a7e4f63p-3, 0x1.f38f3ac64e589p-1},
    {-0x1.8f8b83c69a60bp-3, 0x1.f6297cff75cb0p-1},
    {-0x1.5e214448b3fc6p-3, 0x1.f8764fa714ba9p-1},
    {-0x1.2c8106e8e613ap-3, 0x1.fa7557f08a517p-1},
    {-0x1.f564e56a9730ep-4, 0x1.fc26470e19fd3p-1},
    {-0x1.917a6bc29b42cp-4, 0x1.fd88da3d12526p-1},
    {-0x1.2d52092ce19f6p-4, 0x1.fe9cdad01883ap-1},
    {-0x1.91f65f10dd814p-5, 0x1.ff621e3796d7ep-1},
    {-0x1.92155f7a3667ep-6, 0x1.ffd886084cd0dp-1},
};

// sin x and cos x by table lookup: P. T. P. Tang, "Table-lookup algorithms for elementary
// functions and their error analysis" (1991), with the three-part argument reduction of
// W. J. Cody and W. Waite, "Software Manual for the Elementary Functions" (1980).
// x = k 2pi/256 + r with |r| <= pi/256 (2pi/256 split into parts of 32, 32 and 53
// significant bits, so k C1 and k C2 are exact for |k| < 2^21); then
//   sin x = S_k cos r + C_k sin r,   cos x = C_k cos r - S_k sin r,
// with (S_k, C_k) = (sin, cos)(2pi k / 256) from the table and the Taylor series of sin r
// to r^7 and of cos r to r^6 (the next terms are below 2e-20).  Absolute error about
// 1.5e-16.  Near a zero of sin or cos (x close to a multiple of pi/2) the error is also
// small relative to the result: the table holds exact zeros there and the reduction keeps
// r to a few ulps of itself (a restatement of these steps in 60-digit arithmetic gives
// 4e-16 relative for phases within 1e-9 of k pi).  |x| > 2e4, and NaN, go to sincos().
constexpr double kScC1 = 0x1.921fb54400000p-6;
constexpr double kScC2 = 0x1.0b4611a600000p-40;
constexpr double kScC3 = 0x1.3198a2e037073p-75;
constexpr double kScInv = 40.74366543152521;  // 256 / (2 pi)

__device__ __forceinline__ void sincos_tab(double x, double* s, double* c) {
  if (!(fabs(x) <= 2.0e4)) {
    sincos(x, s, c);
    return;
  }
  const double kd = rint(x * kScInv);
  double r = fma(-kd, kScC1, x);
  r = fma(-kd, kScC2, r);
  r = fma(-kd, kScC3, r);
  const double2 t = __ldg(g_sincos_tab + ((int)kd & 255));  // (S_k, C_k); k mod 256 in two's complement
  const double r2 = r * r;
  const double sr = fma(r * r2, fma(r2, fma(r2, -1.0 / 5040.0, 1.0 / 120.0), -1.0 / 6.0), r);
  const double cr = fma(r2, fma(r2, fma(r2, -1.0 / 720.0, 1.0 / 24.0), -0.5), 1.0);
  *s = fma(t.x, cr, t.y * sr);
  *c = fma(t.y, cr, -(t.x * sr));
}
__device__ __forceinline__ double2 cexp_tab(double2 z) {
  double s, c;
  sincos_tab(z.y, &s, &c);
  if (z.x == 0.0) return make_double2(c, s);  // a pure phase (real pulse parameters)
  const double e = exp(z.x);
  return make_double2(e * c, e * s);
}
// kx dx + ky dy; with real bond vectors (their usual form) two FMAs per component
__device__ __forceinline__ double2 light_arg(double2 kx, double2 ky, double2 dx, double2 dy) {
  if (dx.y == 0.0 && dy.y == 0.0)
    return make_double2(fma(kx.x, dx.x, ky.x * dy.x), fma(kx.y, dx.x, ky.y * dy.x));
  return cadd(cmul(kx, dx), cmul(ky, dy));
}


// cos(x + iy) = cos x cosh y - i sin x sinh y
__device__ __forceinline__ double2 ccos2(double2 z) {
  double s, c;
  sincos(z.x, &s, &c);
  return make_double2(c * cosh(z.y), -s * sinh(z.y));
}
// a / b for complex b
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

int grid_for_count(int64_t count) { return (int)std::max<int64_t>(1, std::min<int64_t>((count + 255) / 256, 65536)); }

// Per-element coefficients of the light modifier: z = kx dx + ky dy.
void light_coefficients(const double* params, double2* a, double2* kx, double2* ky) {
  const cplx A = param(params, 0), A0 = param(params, 1), t = param(params, 2), w = param(params, 3),
             Tp = param(params, 4), eta = param(params, 5);
  const cplx I(0.0, 1.0);
  const cplx ch = (Tp != 0.0) ? std::cosh((t - 2.0 * Tp) / (0.5673 * Tp)) : cplx(1.0, 0.0);
  const cplx sw = std::sin(w * t), cw = std::cos(w * t);
  if (eta == 0.0) {  // linear forms: the y component only
    *kx = make_double2(0.0, 0.0);
    *ky = d2(I * A0 * sw / ch);
  } else {
    *kx = d2(I * A0 * cw / ch);
    *ky = d2(I * A0 * eta * sw / ch);
  }
  *a = d2(A);
}

__global__ void light_kernel(int64_t count, double2 a, double2 kx, double2 ky, const double2* __restrict__ data,
                             const double2* __restrict__ dx, const double2* __restrict__ dy, double2* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 z = light_arg(kx, ky, dx[i], dy[i]);
    out[i] = cmul(cmul(a, data[i]), cexp_tab(z));
  }
}

// H(t) into the doubled SoA values of an operator, one thread per row.  Every lane runs
// the same slot loop, so a slot whose phase argument is zero on the whole warp (the
// on-site and padding slots: dx = dy = 0) skips the FP64 sincos together: exp(0) = 1
// exactly.  Stores are whole 128-byte segments of each slot plane s * n_pad + row; the
// row's L consecutive inputs come through L1.  Padding rows (row >= n) keep the zeros
// written at creation.
// a2 = 2a: the stored values are 2H (doubling is exact, so 2a data e = 2 (a data e) bit for bit).
__global__ void light_update_kernel(int64_t n, int64_t n_pad, int L, double2 a2, double2 kx, double2 ky,
                                    const double2* __restrict__ data, const double2* __restrict__ dx,
                                    const double2* __restrict__ dy, double2* __restrict__ val) {
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < n; row += (int64_t)gridDim.x * blockDim.x) {
    for (int s = 0; s < L; ++s) {
      const int64_t k = row * L + s;
      const double2 z = light_arg(kx, ky, dx[k], dy[k]);
      const double2 e = (z.x == 0.0 && z.y == 0.0) ? make_double2(1.0, 0.0) : cexp_tab(z);
      val[(int64_t)s * n_pad + row] = cmul(cmul(a2, data[k]), e);
    }
  }
}

// p[i] = e_pol[i] cos(wt - q Sx[i]), per site (both the row's and the column's term of
// every bond are read from here).
__global__ void phonon_site_kernel(int64_t n, double2 wt, double2 q0, double2 q1, const double2* __restrict__ ex,
                                   const double2* __restrict__ ey, const double2* __restrict__ sx,
                                   const double2* __restrict__ sy, double2* __restrict__ px, double2* __restrict__ py) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 ax = make_double2(wt.x, wt.y);
    const double2 qx = cmul(q0, sx[i]);
    const double2 qy = cmul(q1, sy[i]);
    px[i] = cmul(ex[i], ccos2(make_double2(ax.x - qx.x, ax.y - qx.y)));
    py[i] = cmul(ey[i], ccos2(make_double2(ax.x - qy.x, ax.y - qy.y)));
  }
}

__global__ void phonon_kernel(int64_t count, int64_t n, int L, double2 aq_over_ch, double2 a0, double2 b,
                              const double2* __restrict__ data, const int32_t* __restrict__ idx,
                              const double2* __restrict__ dx, const double2* __restrict__ dy,
                              const double2* __restrict__ px, const double2* __restrict__ py,
                              double2* __restrict__ data_new, double2* __restrict__ dx_new,
                              double2* __restrict__ dy_new, unsigned* bad) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = i / L;
    const int64_t col = idx[i];
    if (row == col) continue;  // diagonal slots are left as they are
    if (col < 0 || col >= n) {  // a column outside the operator: recorded, slot skipped
      atomicOr(bad, 1u);
      continue;
    }
    const double2 ddx = cmul(aq_over_ch, make_double2(px[row].x - px[col].x, px[row].y - px[col].y));
    const double2 ddy = cmul(aq_over_ch, make_double2(py[row].x - py[col].x, py[row].y - py[col].y));
    const double2 nx = cadd(dx[i], ddx), ny = cadd(dy[i], ddy);
    // r = sqrt(|dx|^2 + |dy|^2) / a0 - 1;  data_new = data exp(-b r)
    const double len = sqrt(nx.x * nx.x + nx.y * nx.y + ny.x * ny.x + ny.y * ny.y);
    double2 r = cdiv(make_double2(len, 0.0), a0);
    r.x -= 1.0;
    const double2 z = cmul(make_double2(-b.x, -b.y), r);
    dx_new[i] = nx;
    dy_new[i] = ny;
    data_new[i] = cmul(data[i], cexp2(z));
  }
}

}  // namespace

extern "C" {

int kpm_light_modifier(int64_t count, const double* params, const double* data, const double* dx, const double* dy,
                       double* data_new, void* stream) {
  if (count < 1 || !params || !data || !dx || !dy || !data_new) return KPM_ERR_INVALID_ARG;
  double2 a, kx, ky;
  light_coefficients(params, &a, &kx, &ky);
  cudaStream_t s = stream_of(stream);
  light_kernel<<<grid_for_count(count), 256, 0, s>>>(count, a, kx, ky, reinterpret_cast<const double2*>(data),
                                                     reinterpret_cast<const double2*>(dx),
                                                     reinterpret_cast<const double2*>(dy),
                                                     reinterpret_cast<double2*>(data_new));
  return check_cuda(cudaGetLastError());
}

int kpm_ell_light_update(kpm_ell* h, const double* params, const double* data0, const double* dx, const double* dy,
                         void* stream) {
  if (!h || !params || !data0 || !dx || !dy) return KPM_ERR_INVALID_ARG;
  if (h->is_real) return KPM_ERR_DTYPE;  // H(t) is complex: create the operator with KPM_FLAG_COMPLEX
  double2 a, kx, ky;
  light_coefficients(params, &a, &kx, &ky);
  cudaStream_t s = stream_of(stream);
  light_update_kernel<<<grid_for_count(h->n), 256, 0, s>>>(
      h->n, h->n_pad, h->L, make_double2(2.0 * a.x, 2.0 * a.y), kx, ky, reinterpret_cast<const double2*>(data0), reinterpret_cast<const double2*>(dx),
      reinterpret_cast<const double2*>(dy), static_cast<double2*>(h->val64));
  KPM_TRY(check_cuda(cudaGetLastError()));
  return values_changed(h, s);
}

int kpm_phonon_modifier(int64_t n, int len_row, const double* params, const double* data, const int32_t* indices,
                        const double* dx, const double* dy, const double* e_pol_x, const double* e_pol_y,
                        const double* Sx, const double* Sy, double* data_new, double* dx_new, double* dy_new,
                        void* stream) {
  if (n < 1 || len_row < 1 || !params || !data || !indices || !dx || !dy || !e_pol_x || !e_pol_y || !Sx || !Sy ||
      !data_new || !dx_new || !dy_new)
    return KPM_ERR_INVALID_ARG;
  const cplx a0 = param(params, 0), b = param(params, 1), Aq = param(params, 2), wq = param(params, 3),
             t = param(params, 4), q0 = param(params, 5), q1 = param(params, 6);
  if (wq == 0.0 || a0 == 0.0) return KPM_ERR_INVALID_ARG;
  const cplx Tp = 2.0 * M_PI / wq;
  const cplx ch = std::cosh((t - 2.0 * Tp) / (0.5673 * Tp));
  cudaStream_t s = stream_of(stream);
  DevBuf site;
  KPM_TRY(ensure(site, (size_t)2 * n * sizeof(double2) + sizeof(double2)));
  double2* px = static_cast<double2*>(site.p);
  double2* py = px + n;
  unsigned* bad = reinterpret_cast<unsigned*>(py + n);
  unsigned bad_host = 0;
  KPM_TRY(check_cuda(cudaMemsetAsync(bad, 0, sizeof(unsigned), s)));
  phonon_site_kernel<<<grid_for_count(n), 256, 0, s>>>(n, d2(wq * t), d2(q0), d2(q1),
                                                       reinterpret_cast<const double2*>(e_pol_x),
                                                       reinterpret_cast<const double2*>(e_pol_y),
                                                       reinterpret_cast<const double2*>(Sx),
                                                       reinterpret_cast<const double2*>(Sy), px, py);
  int st = check_cuda(cudaGetLastError());
  const int64_t count = n * (int64_t)len_row;
  if (st == KPM_OK) {
    phonon_kernel<<<grid_for_count(count), 256, 0, s>>>(
        count, n, len_row, d2(Aq / ch), d2(a0), d2(b), reinterpret_cast<const double2*>(data), indices,
        reinterpret_cast<const double2*>(dx), reinterpret_cast<const double2*>(dy), px, py,
        reinterpret_cast<double2*>(data_new), reinterpret_cast<double2*>(dx_new), reinterpret_cast<double2*>(dy_new),
        bad);
    st = check_cuda(cudaGetLastError());
  }
  if (st == KPM_OK) st = check_cuda(cudaMemcpyAsync(&bad_host, bad, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  if (st == KPM_OK) st = check_cuda(cudaStreamSynchronize(s));  // the per-site scratch is freed below
  release(site);
  if (st == KPM_OK && bad_host) st = KPM_ERR_INDEX;
  return st;
}

}  // extern "C"
