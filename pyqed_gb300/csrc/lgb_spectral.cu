// Eigen-decomposition (spectral) evaluation of Lindblad dynamics
// (pyqed/superoperator.py:455-770, Lindblad_solver).
//
// With the Liouvillian diagonalised on the host, L = sum_n lambda_n |r_n><l_n| / norm_n,
// every quantity the reference's Lindblad_solver returns is a sum over modes:
//   evolve / correlation_*_1t:  F(t) = sum_n W_n exp(lambda_n t)
//   correlation_*_1w:           S(w) = sum_n W_n (-1 / (lambda_n + i w))
//   correlation_3op_2t:         C(tau, t) = sum_{m,n} exp(lambda_m tau) coeff_mn exp(lambda_n t)
// with the mode weights W (and coeff) formed on the host from the
// eigenvectors.  spectral_sum_kernel evaluates up to 16 such sums at many
// points: a thread per point, the modes staged through shared memory in
// chunks and split over blockIdx.y so that a short point list still fills
// the GPU; the partial sums of the mode slices are added in a fixed order
// (spectral_reduce_kernel), so results are deterministic.  The two-time
// correlation is two complex128 GEMMs (cuBLAS) around the exponential
// tables that spectral_exp_kernel fills.  All arithmetic is FP64.
#include <cublas_v2.h>

#include <algorithm>
#include <mutex>

#include "lgb_common.cuh"
#include "lgb_internal.h"

namespace lgb {
namespace {

constexpr int kSThreads = 128;
constexpr int kSChunk = 128;
constexpr int kSMaxOut = 16;

__device__ __forceinline__ double2 mode_factor(int kind, double2 l, double x) {
  if (kind == 0) {  // exp(lambda x)
    const double e = exp(l.x * x);
    double s, c;
    sincos(l.y * x, &s, &c);
    return make_double2(e * c, e * s);
  }
  // -1 / (lambda + i x) = (-Re z + i Im z) / |z|^2, z = lambda + i x
  const double zr = l.x, zi = l.y + x;
  const double d = zr * zr + zi * zi;
  return make_double2(-zr / d, zi / d);
}

__global__ void __launch_bounds__(kSThreads) spectral_sum_kernel(int k, int n_out, int n_x, int kind, int mslice,
                                                                 const double2* __restrict__ lam,
                                                                 const double2* __restrict__ W,
                                                                 const double* __restrict__ x, double2* part) {
  extern __shared__ double2 sh[];  // lambda chunk [kSChunk], then W chunk [n_out][kSChunk]
  const int xi = blockIdx.x * kSThreads + threadIdx.x;
  const double xv = xi < n_x ? x[xi] : 0.0;
  double2 acc[kSMaxOut];
#pragma unroll
  for (int o = 0; o < kSMaxOut; ++o) acc[o] = make_double2(0.0, 0.0);
  const int m0 = blockIdx.y * mslice, m1 = min(k, m0 + mslice);
  for (int c0 = m0; c0 < m1; c0 += kSChunk) {
    const int cn = min(kSChunk, m1 - c0);
    __syncthreads();
    for (int q = threadIdx.x; q < cn; q += kSThreads) sh[q] = lam[c0 + q];
    for (int q = threadIdx.x; q < n_out * cn; q += kSThreads) {
      const int o = q / cn, j = q - o * cn;
      sh[kSChunk + o * kSChunk + j] = W[(long long)o * k + c0 + j];
    }
    __syncthreads();
    for (int j = 0; j < cn; ++j) {
      const double2 f = mode_factor(kind, sh[j], xv);
#pragma unroll
      for (int o = 0; o < kSMaxOut; ++o)
        if (o < n_out) cmac(acc[o], sh[kSChunk + o * kSChunk + j], f);
    }
  }
  if (xi < n_x) {
#pragma unroll
    for (int o = 0; o < kSMaxOut; ++o)
      if (o < n_out) part[((long long)blockIdx.y * n_x + xi) * n_out + o] = acc[o];
  }
}

__global__ void spectral_reduce_kernel(int nslice, long long n, const double2* part, double2* out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double2 s = make_double2(0.0, 0.0);
    for (int y = 0; y < nslice; ++y) {
      const double2 v = part[(long long)y * n + i];
      s.x += v.x;
      s.y += v.y;
    }
    out[i] = s;
  }
}

// out[r][c] = exp(lambda_{mode} x_{point}); modes along the rows when
// modes_on_rows, else along the columns
__global__ void spectral_exp_kernel(int rows, int cols, bool modes_on_rows, const double2* lam, const double* x,
                                    double2* out) {
  const long long n = (long long)rows * cols;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i / cols), c = (int)(i - (long long)r * cols);
    out[i] = modes_on_rows ? mode_factor(0, lam[r], x[c]) : mode_factor(0, lam[c], x[r]);
  }
}

std::mutex g_blas_mu;
cublasHandle_t g_blas[64] = {};

cublasHandle_t blas_for_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(g_blas_mu);
  if (g_blas[dev] == nullptr && cublasCreate(&g_blas[dev]) != CUBLAS_STATUS_SUCCESS) g_blas[dev] = nullptr;
  return g_blas[dev];
}

int grid_for(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 8192)); }

}  // namespace
}  // namespace lgb

extern "C" {

int lgb_spectral_sum(int32_t k, int32_t n_out, int32_t n_x, int32_t kind, const double* lambda, const double* W,
                     const double* x, double* out, void* stream) {
  if (k < 1 || n_out < 1 || n_out > lgb::kSMaxOut || n_x < 0 || (kind != 0 && kind != 1) || lambda == nullptr ||
      W == nullptr || (n_x > 0 && (x == nullptr || out == nullptr)))
    return LGB_ERR_INVALID_ARG;
  if (n_x == 0) return LGB_OK;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  int dev = 0, n_sm = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  const int bx = (n_x + lgb::kSThreads - 1) / lgb::kSThreads;
  // split the modes until the grid covers two waves of the SMs
  int ns = std::max(1, std::min((2 * n_sm + bx - 1) / bx, (k + lgb::kSChunk - 1) / lgb::kSChunk));
  const int mslice = (k + ns - 1) / ns;
  ns = (k + mslice - 1) / mslice;
  const long long npart = (long long)n_x * n_out;
  double2* part = nullptr;
  if (cudaMallocAsync(&part, (size_t)ns * npart * sizeof(double2), st) != cudaSuccess) return LGB_ERR_CUDA;
  const size_t smem = (size_t)(1 + n_out) * lgb::kSChunk * sizeof(double2);
  lgb::spectral_sum_kernel<<<dim3(bx, ns), lgb::kSThreads, smem, st>>>(
      k, n_out, n_x, kind, mslice, reinterpret_cast<const double2*>(lambda), reinterpret_cast<const double2*>(W), x,
      part);
  lgb::spectral_reduce_kernel<<<lgb::grid_for(npart), 256, 0, st>>>(ns, npart, part, reinterpret_cast<double2*>(out));
  const cudaError_t e = cudaGetLastError();
  cudaFreeAsync(part, st);
  return e == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

int lgb_spectral_2t(int32_t k, int32_t n_tau, int32_t n_t, const double* lambda, const double* coeff,
                    const double* tau, const double* t, double* cor, void* stream) {
  if (k < 1 || n_tau < 0 || n_t < 0 || lambda == nullptr || coeff == nullptr ||
      (n_tau > 0 && tau == nullptr) || (n_t > 0 && t == nullptr) || (n_tau > 0 && n_t > 0 && cor == nullptr))
    return LGB_ERR_INVALID_ARG;
  if (n_tau == 0 || n_t == 0) return LGB_OK;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  cublasHandle_t h = lgb::blas_for_device();
  if (h == nullptr) return LGB_ERR_CUDA;
  const double2* lam = reinterpret_cast<const double2*>(lambda);
  double2 *E1 = nullptr, *E2 = nullptr, *tmp = nullptr;
  // E1 [n_tau][k] = exp(lambda_m tau_a), E2 [k][n_t] = exp(lambda_n t_b), tmp [k][n_t]
  if (cudaMallocAsync(&E1, (size_t)n_tau * k * sizeof(double2), st) != cudaSuccess) return LGB_ERR_CUDA;
  if (cudaMallocAsync(&E2, (size_t)k * n_t * sizeof(double2), st) != cudaSuccess ||
      cudaMallocAsync(&tmp, (size_t)k * n_t * sizeof(double2), st) != cudaSuccess) {
    cudaFreeAsync(E1, st);
    if (E2 != nullptr) cudaFreeAsync(E2, st);
    return LGB_ERR_CUDA;
  }
  lgb::spectral_exp_kernel<<<lgb::grid_for((long long)n_tau * k), 256, 0, st>>>(n_tau, k, false, lam, tau, E1);
  lgb::spectral_exp_kernel<<<lgb::grid_for((long long)k * n_t), 256, 0, st>>>(k, n_t, true, lam, t, E2);
  int status = cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
  if (status == LGB_OK) {
    // row-major X (r x c) is the column-major X^T: with column-major views
    // tmp^T = E2^T coeff^T and cor^T = tmp^T E1^T, i.e. cor = E1 coeff E2
    std::lock_guard<std::mutex> lock(lgb::g_blas_mu);
    const cuDoubleComplex one = make_cuDoubleComplex(1.0, 0.0), zero = make_cuDoubleComplex(0.0, 0.0);
    bool ok = cublasSetStream(h, st) == CUBLAS_STATUS_SUCCESS;
    ok = ok && cublasZgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, n_t, k, k, &one, reinterpret_cast<const cuDoubleComplex*>(E2),
                           n_t, reinterpret_cast<const cuDoubleComplex*>(coeff), k, &zero,
                           reinterpret_cast<cuDoubleComplex*>(tmp), n_t) == CUBLAS_STATUS_SUCCESS;
    ok = ok && cublasZgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, n_t, n_tau, k, &one,
                           reinterpret_cast<const cuDoubleComplex*>(tmp), n_t,
                           reinterpret_cast<const cuDoubleComplex*>(E1), k, &zero,
                           reinterpret_cast<cuDoubleComplex*>(cor), n_t) == CUBLAS_STATUS_SUCCESS;
    if (!ok) status = LGB_ERR_CUDA;
  }
  cudaFreeAsync(E1, st);
  cudaFreeAsync(E2, st);
  cudaFreeAsync(tmp, st);
  return status;
}

}  // extern "C"
