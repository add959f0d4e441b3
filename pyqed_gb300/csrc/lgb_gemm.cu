// Grid-wide GEMM schedule for instances too large for one CTA (N > 88 in
// FP32, N > 68 in FP64): each RK4 stage of the rewritten RHS
// (pyqed/oqs.py:697-715)
//     R = A X + X A^dag + sum_k L_k X L_k^dag,   A = -i H_eff,
// is two complex GEMMs and one fused epilogue:
//   G1  T_k = L_k X                        (k = 1..K, one strided-batched GEMM)
//   G2  R = [A | X | T_1 .. T_K] . [X ; A^dag ; L_1^dag ; .. ; L_K^dag]
//   E   RK4 stage combination (pyqed/phys.py:1051-1064), next stage input
//       written into both operand slabs, diagonal-dissipator term D o X,
//       observables Tr[O rho] (pyqed/phys.py:1257-1264) reduced in FP64.
// G1 writes its outputs straight into the left operand slab, so G2 sees the
// whole RHS as a single GEMM with K-dimension (K + 2) N.  Algorithmic work
// per stage: (2K + 2) N^3 complex multiply-adds, the minimum for dense
// collapse operators.  The FP32 and FP64 paths call cuBLAS for G1/G2 (plain
// library GEMMs); the fused kernels below are this library's.
#include <cublas_v2.h>

#include <algorithm>
#include <type_traits>

#include "lgb_internal.h"

namespace lgb {

namespace {

constexpr int kEpiThreads = 256;
constexpr int kEpiElems = 4;  // elements per thread

template <typename T> struct Blas;
template <> struct Blas<float> {
  using C = cuComplex;
  static cublasStatus_t gemm(cublasHandle_t h, cublasOperation_t ta, cublasOperation_t tb, int m,
                             int n, int k, const C* al, const C* A, int lda, const C* B, int ldb,
                             const C* be, C* Cc, int ldc) {
    return cublasCgemm(h, ta, tb, m, n, k, al, A, lda, B, ldb, be, Cc, ldc);
  }
  static cublasStatus_t gemm_sb(cublasHandle_t h, int m, int n, int k, const C* al, const C* A,
                                int lda, long long sa, const C* B, int ldb, long long sb,
                                const C* be, C* Cc, int ldc, long long sc, int batch) {
    return cublasCgemmStridedBatched(h, CUBLAS_OP_N, CUBLAS_OP_N, m, n, k, al, A, lda, sa, B, ldb,
                                     sb, be, Cc, ldc, sc, batch);
  }
  static C one() { return make_cuComplex(1.f, 0.f); }
  static C zero() { return make_cuComplex(0.f, 0.f); }
};
template <> struct Blas<double> {
  using C = cuDoubleComplex;
  static cublasStatus_t gemm(cublasHandle_t h, cublasOperation_t ta, cublasOperation_t tb, int m,
                             int n, int k, const C* al, const C* A, int lda, const C* B, int ldb,
                             const C* be, C* Cc, int ldc) {
    return cublasZgemm(h, ta, tb, m, n, k, al, A, lda, B, ldb, be, Cc, ldc);
  }
  static cublasStatus_t gemm_sb(cublasHandle_t h, int m, int n, int k, const C* al, const C* A,
                                int lda, long long sa, const C* B, int ldb, long long sb,
                                const C* be, C* Cc, int ldc, long long sc, int batch) {
    return cublasZgemmStridedBatched(h, CUBLAS_OP_N, CUBLAS_OP_N, m, n, k, al, A, lda, sa, B, ldb,
                                     sb, be, Cc, ldc, sc, batch);
  }
  static C one() { return make_cuDoubleComplex(1.0, 0.0); }
  static C zero() { return make_cuDoubleComplex(0.0, 0.0); }
};

// Row-major C(M x N) = A(M x K) B(K x N) through column-major cuBLAS:
// C^T = B^T A^T, i.e. the operands are passed swapped.
template <typename T>
cublasStatus_t gemm_rm(cublasHandle_t h, int M, int N, int K, const void* A, int lda,
                       const void* B, int ldb, void* C, int ldc) {
  using B_ = Blas<T>;
  const typename B_::C one = B_::one(), zero = B_::zero();
  return B_::gemm(h, CUBLAS_OP_N, CUBLAS_OP_N, N, M, K, &one,
                  reinterpret_cast<const typename B_::C*>(B), ldb,
                  reinterpret_cast<const typename B_::C*>(A), lda, &zero,
                  reinterpret_cast<typename B_::C*>(C), ldc);
}

// ---- operator preparation ------------------------------------------------------
// G (FP64, N x N) = sum_k L_k^dag L_k has been formed by a ZGEMM; this kernel
// writes the working-precision slabs:
//   Lbuf[:, 0:N]          = A = -i (H - c I) - G / 2      (left operand, block 0)
//   Rbuf[N:2N, :]         = A^dag                          (right operand, block 1)
//   Rbuf[(2+k)N:(3+k)N,:] = L_k^dag, Lstk[k] = L_k         (dense collapse operators)
//   Dm                    = sum_k l_k l_k^dag              (diagonal collapse operators)
//   A0 / Gd               = A and i H_d for driven instances
//   Ot[e]                 = O_e^T (FP64)
template <typename T>
__global__ void gemm_setup_kernel(GemmInstance g, const double2* H, const double2* cops,
                                  int cops_kind, int K, const double2* eops, int E,
                                  const double2* dops, int D, const double2* G,
                                  const double* shift_ptr, long long doff_b) {
  using T2 = typename Cplx<T>::type;
  const int N = g.N;
  const long long NN = (long long)N * N;
  const int W = g.W;
  const double shift = *shift_ptr;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < NN;
       idx += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(idx / N), j = (int)(idx % N);
    double2 h = H[idx];
    const double hx = h.x - (i == j ? shift : 0.0);
    double2 gg = G != nullptr ? G[idx] : make_double2(0.0, 0.0);
    if (cops_kind == 2 && i == j) {
      double s = 0.0;
      for (int k = 0; k < K; ++k) {
        const double2 l = cops[doff_b * K + (long long)k * N + i];
        s += l.x * l.x + l.y * l.y;
      }
      gg.x += s;
    }
    // A_ij = -i (H_ij - c d_ij) - G_ij / 2
    const double2 a = make_double2(h.y - 0.5 * gg.x, -hx - 0.5 * gg.y);
    T2* L = reinterpret_cast<T2*>(g.Lbuf);
    T2* R = reinterpret_cast<T2*>(g.Rbuf);
    L[(long long)i * W + j] = mk<T2>(a.x, a.y);
    // (A^dag)_ji = conj(A_ij) -> Rbuf row N + j, column i
    R[(long long)(N + j) * N + i] = mk<T2>(a.x, -a.y);
    if (g.A0 != nullptr) reinterpret_cast<T2*>(g.A0)[idx] = mk<T2>(a.x, a.y);
    for (int d = 0; d < D; ++d) {
      const double2 hd = dops[(long long)d * NN + idx];
      reinterpret_cast<T2*>(g.Gd)[(long long)d * NN + idx] = mk<T2>(-hd.y, hd.x);  // i H_d
    }
    if (cops_kind == 1) {
      for (int k = 0; k < K; ++k) {
        const double2 l = cops[(long long)k * NN + idx];
        reinterpret_cast<T2*>(g.Lstk)[(long long)k * NN + idx] = mk<T2>(l.x, l.y);
        // (L_k^dag)_ji = conj(L_k,ij) -> Rbuf row (2+k)N + j, column i
        R[(long long)((2 + k) * N + j) * N + i] = mk<T2>(l.x, -l.y);
      }
    } else if (cops_kind == 2) {
      double dx = 0.0, dy = 0.0;
      for (int k = 0; k < K; ++k) {
        const double2 u = cops[doff_b * K + (long long)k * N + i];
        const double2 v = cops[doff_b * K + (long long)k * N + j];
        dx += u.x * v.x + u.y * v.y;
        dy += u.y * v.x - u.x * v.y;
      }
      reinterpret_cast<T2*>(g.Dm)[idx] = mk<T2>(dx, dy);
    }
    for (int e = 0; e < E; ++e) g.Ot[(long long)e * NN + (long long)j * N + i] = eops[(long long)e * NN + idx];
  }
}

// Driven instances: A(t) = A0 + sum_d f_d (i H_d) into Lbuf block 0 and its
// adjoint into Rbuf block 1.
template <typename T>
__global__ void gemm_drive_kernel(GemmInstance g, int D, const double* f, int nt, const int* ctr) {
  const int step = *ctr;
  using T2 = typename Cplx<T>::type;
  const int N = g.N;
  const long long NN = (long long)N * N;
  T fd[4];
#pragma unroll
  for (int d = 0; d < 4; ++d) fd[d] = d < D ? (T)f[(long long)d * nt + step] : (T)0;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < NN;
       idx += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(idx / N), j = (int)(idx % N);
    T2 a = reinterpret_cast<const T2*>(g.A0)[idx];
#pragma unroll
    for (int d = 0; d < 4; ++d)
      if (d < D) a = caxpy(a, fd[d], reinterpret_cast<const T2*>(g.Gd)[(long long)d * NN + idx]);
    reinterpret_cast<T2*>(g.Lbuf)[(long long)i * g.W + j] = a;
    T2 ad = a;
    ad.y = -ad.y;
    reinterpret_cast<T2*>(g.Rbuf)[(long long)(N + j) * N + i] = ad;
  }
}

// Initial state: rho = rho0, X = rho0 in both operand slabs, RK4 sum = 0.
template <typename T>
__global__ void gemm_init_kernel(GemmInstance g, const double2* rho0) {
  using T2 = typename Cplx<T>::type;
  const int N = g.N;
  const long long NN = (long long)N * N;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < NN;
       idx += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(idx / N), j = (int)(idx % N);
    const double2 v = rho0[idx];
    const T2 x = mk<T2>(v.x, v.y);
    reinterpret_cast<T2*>(g.rho)[idx] = x;
    reinterpret_cast<T2*>(g.racc)[idx] = mk<T2>(0.0, 0.0);
    reinterpret_cast<T2*>(g.Lbuf)[(long long)i * g.W + N + j] = x;
    reinterpret_cast<T2*>(g.Rbuf)[idx] = x;
  }
}

// Deterministic FP64 reduction of per-block observable partials: the last
// block to finish sums the partials in block order.
__device__ void finish_obs(GemmInstance& g, const double2* blk, int E, double2* obs_out,
                           long long row_index) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
    for (int e = 0; e < E; ++e) g.partial[(long long)e * gridDim.x + blockIdx.x] = blk[e];
    __threadfence();
    const int ticket = atomicAdd(g.counter, 1);
    last = ticket == (int)gridDim.x - 1;
  }
  __syncthreads();
  if (last) {
    __threadfence();
    if ((int)threadIdx.x < E) {
      double2 s = make_double2(0.0, 0.0);
      const double2* pp = g.partial + (long long)threadIdx.x * gridDim.x;
      for (int b = 0; b < (int)gridDim.x; ++b) {
        const volatile double* vp = reinterpret_cast<const volatile double*>(pp + b);
        s.x += vp[0];
        s.y += vp[1];
      }
      if (obs_out != nullptr) obs_out[row_index * E + threadIdx.x] = s;
    }
    if (threadIdx.x == 0) *g.counter = 0;
  }
}

__device__ __forceinline__ double block_sum(double v, double* sbuf) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sbuf[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += sbuf[k];
  return s;  // valid in thread 0
}

// Observables of the current rho (used for the t0 row).
template <typename T>
__global__ void gemm_obs_kernel(GemmInstance g, int E, double2* obs_out, long long row_index) {
  using T2 = typename Cplx<T>::type;
  __shared__ double sbuf[kEpiThreads / 32];
  __shared__ double2 blk[16];
  const long long NN = (long long)g.N * g.N;
  for (int e = 0; e < E; ++e) {
    double sx = 0.0, sy = 0.0;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < NN;
         idx += (long long)gridDim.x * blockDim.x) {
      const double2 x = to_d2(reinterpret_cast<const T2*>(g.rho)[idx]);
      const double2 o = g.Ot[(long long)e * NN + idx];
      sx += o.x * x.x - o.y * x.y;
      sy += o.x * x.y + o.y * x.x;
    }
    sx = block_sum(sx, sbuf);
    sy = block_sum(sy, sbuf);
    if (threadIdx.x == 0) blk[e] = make_double2(sx, sy);
  }
  finish_obs(g, blk, E, obs_out, row_index);
}

// Fused RK4 stage epilogue.  Stage s in 0..3 reads R = G2's output (+ D o X),
// updates the RK4 sum / rho and writes the next stage input X into Lbuf
// block 1 and Rbuf block 0.  After the fourth stage it also reduces the
// observables, checks finiteness and stores the state when asked.
template <typename T>
__global__ void __launch_bounds__(kEpiThreads) gemm_epilogue_kernel(
    GemmInstance g, int stage, double dt, int diag, int E, double2* obs_out, StepOut so) {
  using T2 = typename Cplx<T>::type;
  __shared__ double sbuf[kEpiThreads / 32];
  __shared__ double2 blk[16];
  const int N = g.N;
  const long long NN = (long long)N * N;
  const int step = *so.ctr;
  const long long row_index = (long long)step + so.obs_t0;
  double2* state_out = (stage == 3) ? so.state_at(step, NN) : nullptr;
  double2* rho_out = (stage == 3 && step == so.nt - 1) ? so.rho_out : nullptr;
  const T cst = (T)((stage == 2) ? dt : 0.5 * dt);
  const T sixth = (T)(dt / 6.0);
  double ox[16], oy[16];
#pragma unroll
  for (int e = 0; e < 16; ++e) ox[e] = oy[e] = 0.0;
  bool fin = true;
  const T2* Rout = reinterpret_cast<const T2*>(g.Rout);
  T2* rho = reinterpret_cast<T2*>(g.rho);
  T2* racc = reinterpret_cast<T2*>(g.racc);
  T2* L = reinterpret_cast<T2*>(g.Lbuf);
  T2* Rb = reinterpret_cast<T2*>(g.Rbuf);
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < NN;
       idx += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(idx / N), j = (int)(idx % N);
    T2 R = Rout[idx];
    if (diag) cmac(R, reinterpret_cast<const T2*>(g.Dm)[idx], Rb[idx]);
    T2 r = rho[idx];
    T2 ra = racc[idx];
    T2 xn;
    if (stage == 0) {
      ra = R;
      xn = caxpy(r, cst, R);
    } else if (stage < 3) {
      ra = caxpy(ra, (T)2, R);
      xn = caxpy(r, cst, R);
    } else {
      ra.x += R.x;
      ra.y += R.y;
      r = caxpy(r, sixth, ra);
      rho[idx] = r;
      xn = r;
      fin = fin && cfinite(r);
      const double2 rd = to_d2(r);
      for (int e = 0; e < E && e < 16; ++e) {
        const double2 o = g.Ot[(long long)e * NN + idx];
        ox[e] += o.x * rd.x - o.y * rd.y;
        oy[e] += o.x * rd.y + o.y * rd.x;
      }
      if (state_out != nullptr) state_out[idx] = rd;
      if (rho_out != nullptr) rho_out[idx] = rd;
    }
    if (stage < 3) racc[idx] = ra;
    L[(long long)i * g.W + N + j] = xn;
    Rb[idx] = xn;
  }
  if (stage == 3) {
    const int bad = __syncthreads_or(!fin);
    if (bad && threadIdx.x == 0) *g.err = 4;  // LGB_ERR_NONFINITE
    for (int e = 0; e < E; ++e) {
      const double sx = block_sum(ox[e], sbuf);
      const double sy = block_sum(oy[e], sbuf);
      if (threadIdx.x == 0) blk[e] = make_double2(sx, sy);
    }
    if (E > 0) finish_obs(g, blk, E, obs_out, row_index);
  }
}

__global__ void step_inc_kernel(int* ctr) { *ctr += 1; }

// Per-step check (optional): trace and hermiticity deviation of rho, in FP64.
// 32 x 32 tiles through shared memory (the transposed tile for rho_ji);
// the trace partials of the diagonal tiles and the largest |rho_ij -
// conj(rho_ji)| go to the instance's scratch by atomics (the order of the
// trace additions only moves its last bits; the check compares with a
// tolerance).  ws: [0..1] Tr rho0, [2] rho0 Hermitian, [3..4] Tr rho, [5] max
// deviation (as the bits of a non-negative double).
template <typename T>
__global__ void gemm_check_accum_kernel(const void* rho_, int N, double* ws) {
  using T2 = typename Cplx<T>::type;
  __shared__ double2 tile[32][33];
  const T2* rho = reinterpret_cast<const T2*>(rho_);
  const int ti = blockIdx.y * 32, tj = blockIdx.x * 32;
  // the transposed tile (rows tj.., columns ti..)
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int i = tj + r, j = ti + threadIdx.x;
    tile[r][threadIdx.x] = (i < N && j < N) ? to_d2(rho[(long long)i * N + j]) : make_double2(0.0, 0.0);
  }
  __syncthreads();
  double h = 0.0, tx = 0.0, ty = 0.0;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int i = ti + r, j = tj + threadIdx.x;
    if (i < N && j < N) {
      const double2 x = to_d2(rho[(long long)i * N + j]);
      const double2 xt = tile[threadIdx.x][r];  // rho[j][i]
      h = fmax(h, hypot(x.x - xt.x, x.y + xt.y));
      if (i == j) {
        tx += x.x;
        ty += x.y;
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    h = fmax(h, __shfl_xor_sync(0xffffffffu, h, o));
    tx += __shfl_xor_sync(0xffffffffu, tx, o);
    ty += __shfl_xor_sync(0xffffffffu, ty, o);
  }
  if (threadIdx.x == 0) {
    atomicMax(reinterpret_cast<unsigned long long*>(ws + 5), (unsigned long long)__double_as_longlong(h));
    if (ti == tj) {
      atomicAdd(ws + 3, tx);
      atomicAdd(ws + 4, ty);
    }
  }
}

__global__ void gemm_check_fold_kernel(double* ws, double* chk, int* err, double tol, int initial) {
  const double h = ws[5];
  if (initial) {
    ws[0] = ws[3];
    ws[1] = ws[4];
    ws[2] = h <= tol ? 1.0 : 0.0;
    chk[0] = 0.0;
    chk[1] = ws[2] != 0.0 ? 0.0 : -1.0;
  } else {
    const double dtr = hypot(ws[3] - ws[0], ws[4] - ws[1]);
    chk[0] = fmax(chk[0], dtr);
    bool bad = !(dtr <= tol);
    if (ws[2] != 0.0) {
      chk[1] = fmax(chk[1], h);
      bad = bad || !(h <= tol);
    }
    if (bad && *err == 0) *err = 9;  // LGB_ERR_CHECK
  }
  ws[3] = ws[4] = ws[5] = 0.0;
}

int epi_grid(int N) {
  const long long NN = (long long)N * N;
  long long b = (NN + (long long)kEpiThreads * kEpiElems - 1) / ((long long)kEpiThreads * kEpiElems);
  return (int)std::min<long long>(std::max<long long>(b, 1), 4096);
}

}  // namespace

size_t gemm_partial_slots(int N) { return (size_t)epi_grid(N); }

int gemm_setup(const GemmSetupArgs& a, cudaStream_t st) {
  const GemmInstance& g = a.g;
  const int N = g.N;
  const long long NN = (long long)N * N;
  cublasSetStream(a.blas, st);
  const double2* G = nullptr;
  if (a.cops_kind == 1 && a.K > 0) {
    // G^T (column-major view of row-major G) = M M^H with M the column-major
    // view (N x KN) of the row-major stack [L_1; ..; L_K]
    const cuDoubleComplex one = make_cuDoubleComplex(1.0, 0.0), zero = make_cuDoubleComplex(0.0, 0.0);
    if (cublasZgemm(a.blas, CUBLAS_OP_N, CUBLAS_OP_C, N, N, a.K * N, &one,
                    reinterpret_cast<const cuDoubleComplex*>(a.cops), N,
                    reinterpret_cast<const cuDoubleComplex*>(a.cops), N, &zero,
                    reinterpret_cast<cuDoubleComplex*>(a.Gtmp), N) != CUBLAS_STATUS_SUCCESS)
      return LGB_ERR_CUDA;
    G = a.Gtmp;
  }
  const int grid = (int)std::min<long long>((NN + 255) / 256, 4096);
  if (a.fp64) {
    gemm_setup_kernel<double><<<grid, 256, 0, st>>>(g, a.H, a.cops, a.cops_kind, a.K, a.eops, a.E,
                                                    a.dops, a.D, G, a.shift, a.doff);
  } else {
    gemm_setup_kernel<float><<<grid, 256, 0, st>>>(g, a.H, a.cops, a.cops_kind, a.K, a.eops, a.E,
                                                   a.dops, a.D, G, a.shift, a.doff);
  }
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

template <typename T>
static int gemm_propagate_t(const GemmRunArgs& a, cudaStream_t st) {
  GemmInstance g = a.g;
  const int N = g.N, K = a.Kdense, W = g.W;
  const long long NN = (long long)N * N;
  const int grid = (int)std::min<long long>((NN + 255) / 256, 4096);
  const int egrid = epi_grid(N);
  const size_t esz = sizeof(typename Cplx<T>::type);
  cublasSetStream(a.blas, st);
  gemm_init_kernel<T><<<grid, 256, 0, st>>>(g, a.rho0);
  const bool check = a.check_tol > 0.0 && a.chk != nullptr;
  if (check) gemm_check(a, std::is_same<T, double>::value, true, st);
  if (a.obs_t0 && a.E > 0) gemm_obs_kernel<T><<<egrid, kEpiThreads, 0, st>>>(g, a.E, a.obs_out, 0);
  if (cudaMemsetAsync(a.ctr, 0, sizeof(int), st) != cudaSuccess) return LGB_ERR_CUDA;
  if (cudaGetLastError() != cudaSuccess) return LGB_ERR_CUDA;
  using B_ = Blas<T>;
  StepOut so;
  so.ctr = a.ctr;
  so.obs_t0 = a.obs_t0;
  so.nt = a.nt;
  so.store_every = a.store_every;
  so.states_out = a.states_out;
  so.rho_out = a.rho_out;
  auto one_step = [&](cudaStream_t s) -> int {
    const typename B_::C one = B_::one(), zero = B_::zero();
    cublasSetStream(a.blas, s);
    if (a.D > 0) gemm_drive_kernel<T><<<grid, 256, 0, s>>>(g, a.D, a.drive, a.nt, a.ctr);
    for (int stage = 0; stage < 4; ++stage) {
      if (K > 0) {
        // T_k = L_k X -> Lbuf blocks 2..K+1 (row-major, ld W); X = Rbuf rows 0..N-1
        if (B_::gemm_sb(a.blas, N, N, N, &one, reinterpret_cast<const typename B_::C*>(g.Rbuf), N,
                        0, reinterpret_cast<const typename B_::C*>(g.Lstk), N, NN, &zero,
                        reinterpret_cast<typename B_::C*>((char*)g.Lbuf + 2 * (size_t)N * esz), W,
                        N, K) != CUBLAS_STATUS_SUCCESS)
          return LGB_ERR_CUDA;
      }
      // R = Lbuf (N x W) . Rbuf (W x N)
      if (gemm_rm<T>(a.blas, N, N, W, g.Lbuf, W, g.Rbuf, N, g.Rout, N) != CUBLAS_STATUS_SUCCESS)
        return LGB_ERR_CUDA;
      gemm_epilogue_kernel<T><<<egrid, kEpiThreads, 0, s>>>(g, stage, a.dt, a.diag, a.E, a.obs_out, so);
    }
    if (check) gemm_check(a, std::is_same<T, double>::value, false, s);
    step_inc_kernel<<<1, 1, 0, s>>>(a.ctr);
    return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
  };
  const int r = run_steps(a.nt, st, a.cap, one_step, a.graph_steps);
  cublasSetStream(a.blas, st);
  if (r != LGB_OK) return r;
  if (a.nt == 0 && a.rho_out != nullptr)
    cudaMemcpyAsync(a.rho_out, a.rho0, NN * sizeof(double2), cudaMemcpyDeviceToDevice, st);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

void gemm_check(const GemmRunArgs& a, bool fp64, bool initial, cudaStream_t st) {
  const int t = (a.g.N + 31) / 32;
  if (initial) cudaMemsetAsync(a.chk_ws, 0, 8 * sizeof(double), st);
  if (fp64) {
    gemm_check_accum_kernel<double><<<dim3(t, t), dim3(32, 8), 0, st>>>(a.g.rho, a.g.N, a.chk_ws);
  } else {
    gemm_check_accum_kernel<float><<<dim3(t, t), dim3(32, 8), 0, st>>>(a.g.rho, a.g.N, a.chk_ws);
  }
  gemm_check_fold_kernel<<<1, 1, 0, st>>>(a.chk_ws, a.chk, a.g.err, a.check_tol, initial ? 1 : 0);
}

int gemm_propagate(const GemmRunArgs& a, cudaStream_t st) {
  if (a.split) return split_propagate(a, st);
  return a.fp64 ? gemm_propagate_t<double>(a, st) : gemm_propagate_t<float>(a, st);
}

void gemm_init_split(const GemmInstance& g, const double2* rho0, cudaStream_t st) {
  const long long NN = (long long)g.N * g.N;
  gemm_init_kernel<float><<<(int)std::min<long long>((NN + 255) / 256, 4096), 256, 0, st>>>(g, rho0);
}
void gemm_obs_split(const GemmInstance& g, int E, double2* obs_out, cudaStream_t st) {
  gemm_obs_kernel<float><<<epi_grid(g.N), kEpiThreads, 0, st>>>(g, E, obs_out, 0);
}
void gemm_drive_split(const GemmInstance& g, int D, const double* f, int nt, const int* ctr, cudaStream_t st) {
  const long long NN = (long long)g.N * g.N;
  gemm_drive_kernel<float><<<(int)std::min<long long>((NN + 255) / 256, 4096), 256, 0, st>>>(g, D, f, nt, ctr);
}
void gemm_step_inc(int* ctr, cudaStream_t st) { step_inc_kernel<<<1, 1, 0, st>>>(ctr); }

}  // namespace lgb
