// Shared device helpers: complex arithmetic on float2/double2 and the
// parameter blocks passed from the plan to the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace lgb {

template <typename T> struct Cplx;
template <> struct Cplx<float> { using type = float2; };
template <> struct Cplx<double> { using type = double2; };

template <typename T2> __device__ __forceinline__ T2 mk(double re, double im);
template <> __device__ __forceinline__ float2 mk<float2>(double re, double im) {
  return make_float2((float)re, (float)im);
}
template <> __device__ __forceinline__ double2 mk<double2>(double re, double im) {
  return make_double2(re, im);
}

// c += a * b
template <typename T2> __device__ __forceinline__ void cmac(T2& c, const T2 a, const T2 b) {
  c.x = fma(a.x, b.x, c.x);
  c.x = fma(-a.y, b.y, c.x);
  c.y = fma(a.x, b.y, c.y);
  c.y = fma(a.y, b.x, c.y);
}
// c += a * conj(b)
template <typename T2> __device__ __forceinline__ void cmacc(T2& c, const T2 a, const T2 b) {
  c.x = fma(a.x, b.x, c.x);
  c.x = fma(a.y, b.y, c.x);
  c.y = fma(a.y, b.x, c.y);
  c.y = fma(-a.x, b.y, c.y);
}
template <typename T2> __device__ __forceinline__ T2 cmul(const T2 a, const T2 b) {
  T2 c;
  c.x = a.x * b.x - a.y * b.y;
  c.y = a.x * b.y + a.y * b.x;
  return c;
}
// a + s * b (real s)
template <typename T2, typename S> __device__ __forceinline__ T2 caxpy(const T2 a, S s, const T2 b) {
  T2 c;
  c.x = fma(s, b.x, a.x);
  c.y = fma(s, b.y, a.y);
  return c;
}
template <typename T2> __device__ __forceinline__ bool cfinite(const T2 a) {
  return isfinite(a.x) && isfinite(a.y);
}
__device__ __forceinline__ double2 to_d2(const float2 a) { return make_double2(a.x, a.y); }
__device__ __forceinline__ double2 to_d2(const double2 a) { return a; }

// Bounded spin budget for every device-side wait (mbarrier polls).  A wait
// that exceeds it records LGB_ERR_TIMEOUT and the kernel winds down.
constexpr long long kSpinLimit = 1LL << 26;

// Per-launch parameters of the CTA-resident (one instance per CTA) kernels.
struct CtaParams {
  int n_inst, n_cops, cops_kind, n_eops, n_drive, nt, obs_t0, store_every, drive_shared;
  double dt;
  const int* order;          // processing order, largest first
  const int* dims;           // N per instance
  const int* npad;           // padded N (multiple of 4)
  const long long* off;      // packed offset (complex elements) of N x N operators
  const long long* woff;     // offset of an NP x NPS working matrix (complex elements)
  const long long* soff;     // offset of the instance's stored states
  const unsigned char* place;// bit0: Lt in shared memory, bit1: Yt in shared memory
  const void* At;            // A^T, A = -i H_eff (trace-shifted), NP x NPS per instance
  const void* Lt;            // dense L_k^T, n_cops x NP x NPS per instance
  const void* Dm;            // diagonal-c_ops dissipator D_ij, NP x NPS per instance
  const void* Gt;            // drive terms (i H_d)^T, n_drive x NP x NPS per instance
  const double2* Ot;         // observables transposed (FP64), n_eops x NP x NPS per instance
  const float2* OtF;         // the same in FP32 (tensor-core kernel)
  const double* drive;       // drive samples
  const double2* rho0;       // packed initial states
  double2* obs_out;
  double2* rho_out;
  double2* states_out;
  void* state_ws;            // rho and RK4 sum, 2 x NP x NPS per instance (global-state variant)
  void* y_ws;                // Y_k^T scratch, n_cops x NP x NPS per instance (when not in smem)
  int* err;                  // per-instance status
  int smem_bytes;            // dynamic shared memory of the launch
  int drive_ld;              // samples per drive term and instance (0: nt)
  long long state_stride;    // complex elements between stored states (0: N*N)
  void* ystore;              // optional: every stage input, 4 * ycap x NP x NPS per instance
  int ycap;                  // steps held per instance in ystore
  int tc_pairs;              // tensor-core kernel: two instances per CTA for NP <= 32
  int test_stall;            // test hook: the first MMA commit is never issued
  long long spin;            // poll bound of the tensor-core kernel's waits (0: default)
  double check_tol;          // per-step trace/hermiticity check tolerance (0: off)
  double* chk;               // [n_inst][2]: max trace drift, max hermiticity deviation (-1: not checked)
};

}  // namespace lgb
