// Redfield master equation (pyqed/oqs.py:30-100, 364-459, 519-563) on the GPU.
//
// The reference builds, in the eigenbasis of H (row-major vec, left(a) =
// a (x) 1, right(a) = 1 (x) a^T), the N^2 x N^2 generator
//     R = -i [E, .] - sum_k [A_k, L_k . - . L_k^dag],   L_k = C_k o A_k,
// C_k[n][m] = S_k(e_m - e_n), and integrates d vec(rho)/dt = R vec(rho) with
// RK4 (pyqed/phys.py:1051-1064).
//
// redfield_tensor_kernel writes R element by element:
//     R[(a,b),(x,y)] = -i (e_a - e_b) d_ax d_by
//                      - sum_k [ (A L)_ax d_by - A_ax (L^dag)_yb - L_ax A_yb + d_ax (L^dag A)_yb ]
// (one thread per element, O(N^4 K) work).  redfield_rk4_kernel propagates
// a batch, one CTA per instance: the state, the stage input, the stage
// derivative and the RK4 sum live in shared memory, the generator too when it
// fits (else it streams from L2); each stage is a warp-per-row complex GEMV
// followed by the fused RK4 combination, and after every step the
// observables Tr[O rho] are reduced in FP64 and the state checked for
// non-finite values.  FP64 (the check path) and FP32.
#include <algorithm>
#include <vector>

#include "lgb_common.cuh"
#include "lgb_internal.h"

namespace lgb {

namespace {

constexpr int kRThreads = 256;
constexpr int kRWarps = kRThreads / 32;
constexpr int kRMaxEops = 16;

__global__ void redfield_tensor_kernel(int n, int K, const double* evals, const double2* A,
                                       const double* C, double2* R) {
  const long long M = (long long)n * n;
  const long long total = M * M;
  const long long nn = (long long)n * n;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(idx / M), q = (int)(idx % M);
    const int a = r / n, b = r % n, x = q / n, y = q % n;
    double vx = 0.0, vy = 0.0;
    if (a == x && b == y) vy = -(evals[a] - evals[b]);  // -i (e_a - e_b)
    for (int k = 0; k < K; ++k) {
      const double2* Ak = A + k * nn;
      const double* Ck = C + k * nn;
      // L = C o A; (L^dag)_yb = conj(L_by) = C_by conj(A_by)
      const double2 Aax = Ak[a * n + x], Ayb = Ak[y * n + b];
      const double cax = Ck[a * n + x], cby = Ck[b * n + y];
      const double2 Lax = make_double2(cax * Aax.x, cax * Aax.y);
      const double2 Aby = Ak[b * n + y];
      const double2 Ldyb = make_double2(cby * Aby.x, -cby * Aby.y);
      // + A_ax (L^dag)_yb + L_ax A_yb
      vx += Aax.x * Ldyb.x - Aax.y * Ldyb.y + Lax.x * Ayb.x - Lax.y * Ayb.y;
      vy += Aax.x * Ldyb.y + Aax.y * Ldyb.x + Lax.x * Ayb.y + Lax.y * Ayb.x;
      if (b == y) {  // - (A L)_ax
        for (int c = 0; c < n; ++c) {
          const double2 Aac = Ak[a * n + c], Acx = Ak[c * n + x];
          const double ccx = Ck[c * n + x];
          vx -= ccx * (Aac.x * Acx.x - Aac.y * Acx.y);
          vy -= ccx * (Aac.x * Acx.y + Aac.y * Acx.x);
        }
      }
      if (a == x) {  // - (L^dag A)_yb,  (L^dag)_yc = C_cy conj(A_cy)
        for (int c = 0; c < n; ++c) {
          const double2 Acy = Ak[c * n + y], Acb = Ak[c * n + b];
          const double ccy = Ck[c * n + y];
          vx -= ccy * (Acy.x * Acb.x + Acy.y * Acb.y);
          vy -= ccy * (Acy.x * Acb.y - Acy.y * Acb.x);
        }
      }
    }
    R[idx] = make_double2(vx, vy);
  }
}

// Generators of many systems in one launch: blockIdx.y is the system, whose
// eigenvalues, operators, spectra and R start at the given offsets.
__global__ void redfield_tensor_batch_kernel(int K, const int* dims, const long long* eoff, const long long* moff,
                                             const long long* roff, const double* evals, const double2* A,
                                             const double* C, double2* R) {
  const int sys = blockIdx.y;
  const int n = dims[sys];
  const long long M = (long long)n * n, total = M * M, nn = M;
  const double* ev = evals + eoff[sys];
  const double2* As = A + (long long)K * moff[sys];
  const double* Cs = C + (long long)K * moff[sys];
  double2* Rs = R + roff[sys];
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(idx / M), q = (int)(idx % M);
    const int a = r / n, b = r % n, x = q / n, y = q % n;
    double vx = 0.0, vy = 0.0;
    if (a == x && b == y) vy = -(ev[a] - ev[b]);
    for (int k = 0; k < K; ++k) {
      const double2* Ak = As + k * nn;
      const double* Ck = Cs + k * nn;
      const double2 Aax = Ak[a * n + x], Ayb = Ak[y * n + b];
      const double cax = Ck[a * n + x], cby = Ck[b * n + y];
      const double2 Lax = make_double2(cax * Aax.x, cax * Aax.y);
      const double2 Aby = Ak[b * n + y];
      const double2 Ldyb = make_double2(cby * Aby.x, -cby * Aby.y);
      vx += Aax.x * Ldyb.x - Aax.y * Ldyb.y + Lax.x * Ayb.x - Lax.y * Ayb.y;
      vy += Aax.x * Ldyb.y + Aax.y * Ldyb.x + Lax.x * Ayb.y + Lax.y * Ayb.x;
      if (b == y) {
        for (int c = 0; c < n; ++c) {
          const double2 Aac = Ak[a * n + c], Acx = Ak[c * n + x];
          const double ccx = Ck[c * n + x];
          vx -= ccx * (Aac.x * Acx.x - Aac.y * Acx.y);
          vy -= ccx * (Aac.x * Acx.y + Aac.y * Acx.x);
        }
      }
      if (a == x) {
        for (int c = 0; c < n; ++c) {
          const double2 Acy = Ak[c * n + y], Acb = Ak[c * n + b];
          const double ccy = Ck[c * n + y];
          vx -= ccy * (Acy.x * Acb.x + Acy.y * Acb.y);
          vy -= ccy * (Acy.x * Acb.y - Acy.y * Acb.x);
        }
      }
    }
    Rs[idx] = make_double2(vx, vy);
  }
}

template <typename T>
__global__ void redfield_convert_kernel(const double2* src, typename Cplx<T>::type* dst, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    dst[i] = mk<typename Cplx<T>::type>(src[i].x, src[i].y);
}

struct RedfieldParams {
  int n_inst, n_eops, nt, store_every;
  double dt;
  const int* dims;
  const long long* roff;     // generator offset (complex elements) per instance
  const long long* voff;     // vector offset (N^2) per instance
  const unsigned char* rsm;  // generator held in shared memory
  const void* R;             // working-precision generators
  const double2* Ot;         // vec(O_e^T) per instance (E x N^2), FP64
  const double2* rho0;       // vec(rho0) in the eigenbasis
  double2* obs_out;          // [n_inst][nt][E]
  double2* rho_out;          // vec(rho) after nt steps
  double2* states_out;       // [n_inst][nt / store_every][N^2]
  int* err;
};

template <typename T>
__global__ void __launch_bounds__(kRThreads) redfield_rk4_kernel(RedfieldParams p) {
  using T2 = typename Cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double red[kRWarps][kRMaxEops][2];
  const int b = blockIdx.x;
  const int N = p.dims[b];
  const int M = N * N;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  T2* y = reinterpret_cast<T2*>(smem);
  T2* x = y + M;
  T2* k = x + M;
  T2* acc = k + M;
  const T2* Rg = reinterpret_cast<const T2*>(p.R) + p.roff[b];
  const T2* R = Rg;
  if (p.rsm[b]) {
    T2* Rs = acc + M;
    for (long long i = tid; i < (long long)M * M; i += kRThreads) Rs[i] = Rg[i];
    R = Rs;
  }
  const double2* r0 = p.rho0 + p.voff[b];
  for (int i = tid; i < M; i += kRThreads) {
    const T2 v = mk<T2>(r0[i].x, r0[i].y);
    y[i] = v;
    x[i] = v;
  }
  if (tid == 0) p.err[b] = 0;
  __syncthreads();
  const T dt = (T)p.dt, hdt = (T)(0.5 * p.dt), sdt = (T)(p.dt / 6.0);
  const int E = p.n_eops;
  const double2* Ot = p.Ot + (long long)E * p.voff[b];
  for (int step = 0; step < p.nt; ++step) {
    for (int stage = 0; stage < 4; ++stage) {
      // k = R x (one warp per row, lanes along the row)
      for (int r = warp; r < M; r += kRWarps) {
        const T2* row = R + (long long)r * M;
        T2 s = mk<T2>(0.0, 0.0);
        for (int c = lane; c < M; c += 32) cmac(s, row[c], x[c]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
          s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
        }
        if (lane == 0) k[r] = s;
      }
      __syncthreads();
      for (int i = tid; i < M; i += kRThreads) {
        const T2 ki = k[i];
        if (stage == 0) {
          acc[i] = ki;
          x[i] = caxpy(y[i], hdt, ki);
        } else if (stage < 3) {
          acc[i] = caxpy(acc[i], (T)2, ki);
          x[i] = caxpy(y[i], stage == 2 ? dt : hdt, ki);
        } else {
          T2 s = acc[i];
          s.x += ki.x;
          s.y += ki.y;
          const T2 yn = caxpy(y[i], sdt, s);
          y[i] = yn;
          x[i] = yn;
        }
      }
      __syncthreads();
    }
    // observables and finiteness of rho(t_{step+1})
    bool fin = true;
    double ox[kRMaxEops], oy[kRMaxEops];
#pragma unroll
    for (int e = 0; e < kRMaxEops; ++e) ox[e] = oy[e] = 0.0;
    for (int i = tid; i < M; i += kRThreads) {
      const double2 v = to_d2(y[i]);
      fin = fin && isfinite(v.x) && isfinite(v.y);
#pragma unroll
      for (int e = 0; e < kRMaxEops; ++e) {
        if (e >= E) break;
        const double2 o = Ot[(long long)e * M + i];
        ox[e] += o.x * v.x - o.y * v.y;
        oy[e] += o.x * v.y + o.y * v.x;
      }
      if (p.store_every > 0 && p.states_out != nullptr && (step + 1) % p.store_every == 0) {
        // instance b's states are one contiguous block of (nt / store_every) x N^2
        const long long ns = p.nt / p.store_every;
        p.states_out[p.voff[b] * ns + (long long)((step + 1) / p.store_every - 1) * M + i] = v;
      }
    }
    for (int e = 0; e < E; ++e) {
      double sx = ox[e], sy = oy[e];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, o);
        sy += __shfl_xor_sync(0xffffffffu, sy, o);
      }
      if (lane == 0) {
        red[warp][e][0] = sx;
        red[warp][e][1] = sy;
      }
    }
    const bool bad = __syncthreads_or(!fin) != 0;
    if (tid < E && p.obs_out != nullptr) {
      double sx = 0.0, sy = 0.0;
      for (int w = 0; w < kRWarps; ++w) {
        sx += red[w][tid][0];
        sy += red[w][tid][1];
      }
      p.obs_out[((long long)b * p.nt + step) * E + tid] = make_double2(sx, sy);
    }
    if (bad) {
      if (tid == 0) p.err[b] = 4;  // LGB_ERR_NONFINITE
      return;
    }
    __syncthreads();
  }
  if (p.rho_out != nullptr)
    for (int i = tid; i < M; i += kRThreads) p.rho_out[p.voff[b] + i] = to_d2(y[i]);
}

constexpr size_t kRSmemBudget = 200 * 1024;

// FP32 systems with N^2 <= 64 (N <= 8): the generator lives in registers, four
// threads per row of R, sixteen complex entries each; a stage is the partial
// dot products of the four threads (the stage input broadcast from shared
// memory), a two-step shuffle sum, and the RK4 combination by the row's
// first thread, which keeps the row's state in registers.  One barrier per
// stage (the stage input is double-buffered); a row's four threads take the
// interleaved columns q, q + 4, .. so that their stage-input loads hit four
// banks.  The same arithmetic as redfield_rk4_kernel<float>; observables are
// reduced in FP32 with error-free TwoSum trees, staged as (hi, lo) pairs in
// the output slots and widened to FP64 after the run.
constexpr int kRRegM = 64;
constexpr int kRRegCols = kRRegM / 4;

__device__ __forceinline__ void rf_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

template <int MC>  // MC > 0: every system has N^2 = MC (compile-time column loop)
__global__ void __launch_bounds__(kRThreads, 4) redfield_rk4_reg_kernel(RedfieldParams p) {
  __shared__ float2 xs[2][kRRegM];
  __shared__ float2 ots[kRMaxEops][kRRegM];
  __shared__ float red[kRWarps][kRMaxEops][4];
  const int b = blockIdx.x;
  const int N = p.dims[b];
  const int M = MC > 0 ? MC : N * N;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int r = tid >> 2, q = tid & 3;
  const int cpt = MC > 0 ? (MC + 3) / 4 : (M + 3) >> 2;  // columns per thread: q, q + 4, q + 8, ..
  const bool owner = q == 0 && r < M;
  const float2* Rg = reinterpret_cast<const float2*>(p.R) + p.roff[b];
  float2 Rr[kRRegCols];
#pragma unroll
  for (int k = 0; k < kRRegCols; ++k) {
    const int c = q + 4 * k;  // interleaved: the four threads of a row read four banks
    Rr[k] = (r < M && k < cpt && c < M) ? Rg[(long long)r * M + c] : make_float2(0.f, 0.f);
  }
  const int E = p.n_eops;
  const double2* Ot = p.Ot + (long long)E * p.voff[b];
  for (int i = tid; i < kRMaxEops * kRRegM; i += kRThreads) {
    const int e = i / kRRegM, j = i - e * kRRegM;
    const double2 o = (e < E && j < M) ? Ot[(long long)e * M + j] : make_double2(0.0, 0.0);
    ots[e][j] = make_float2((float)o.x, (float)o.y);
  }
  float2 y = make_float2(0.f, 0.f), acc = make_float2(0.f, 0.f);
  if (owner) {
    const double2 v = p.rho0[p.voff[b] + r];
    y = make_float2((float)v.x, (float)v.y);
  }
  for (int i = tid; i < 2 * kRRegM; i += kRThreads) xs[i / kRRegM][i % kRRegM] = make_float2(0.f, 0.f);
  __syncthreads();
  if (owner) xs[0][r] = y;
  if (tid == 0) p.err[b] = 0;
  __syncthreads();
  const float dt = (float)p.dt, hdt = (float)(0.5 * p.dt), sdt = (float)(p.dt / 6.0);
  int cur = 0;
  int nsteps = p.nt;  // steps whose observables were written
  for (int step = 0; step < p.nt; ++step) {
    for (int stage = 0; stage < 4; ++stage) {
      const float2* x = xs[cur];
      // four independent accumulators (short dependency chains)
      float2 s4[4] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
      for (int k = 0; k < kRRegCols; ++k)
        if (k < cpt) cmac(s4[k & 3], Rr[k], x[q + 4 * k]);
      float2 s = make_float2((s4[0].x + s4[1].x) + (s4[2].x + s4[3].x), (s4[0].y + s4[1].y) + (s4[2].y + s4[3].y));
      s.x += __shfl_xor_sync(0xffffffffu, s.x, 1);
      s.y += __shfl_xor_sync(0xffffffffu, s.y, 1);
      s.x += __shfl_xor_sync(0xffffffffu, s.x, 2);
      s.y += __shfl_xor_sync(0xffffffffu, s.y, 2);
      if (owner) {
        float2 xn;
        if (stage == 0) {
          acc = s;
          xn = caxpy(y, hdt, s);
        } else if (stage < 3) {
          acc = caxpy(acc, 2.f, s);
          xn = caxpy(y, stage == 2 ? dt : hdt, s);
        } else {
          float2 t = acc;
          t.x += s.x;
          t.y += s.y;
          y = caxpy(y, sdt, t);
          xn = y;
        }
        xs[cur ^ 1][r] = xn;
      }
      __syncthreads();
      cur ^= 1;
    }
    // observables Tr[O rho] of rho(t_{step+1}) and its finiteness
    const bool fin = !owner || (isfinite(y.x) && isfinite(y.y));
#pragma unroll
    for (int e = 0; e < kRMaxEops; ++e) {
      if (e >= E) break;
      float hx = 0.f, hy = 0.f, lx = 0.f, ly = 0.f;
      if (owner) {
        const float2 o = ots[e][r];
        hx = fmaf(-o.y, y.y, o.x * y.x);
        hy = fmaf(o.y, y.x, o.x * y.y);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        float sum, er;
        rf_two_sum(hx, __shfl_xor_sync(0xffffffffu, hx, o), sum, er);
        lx += __shfl_xor_sync(0xffffffffu, lx, o) + er;
        hx = sum;
        rf_two_sum(hy, __shfl_xor_sync(0xffffffffu, hy, o), sum, er);
        ly += __shfl_xor_sync(0xffffffffu, ly, o) + er;
        hy = sum;
      }
      if (lane == 0) {
        red[warp][e][0] = hx;
        red[warp][e][1] = lx;
        red[warp][e][2] = hy;
        red[warp][e][3] = ly;
      }
    }
    if (p.store_every > 0 && p.states_out != nullptr && (step + 1) % p.store_every == 0 && owner) {
      const long long ns = p.nt / p.store_every;
      p.states_out[p.voff[b] * ns + (long long)((step + 1) / p.store_every - 1) * M + r] =
          make_double2(y.x, y.y);
    }
    const bool bad = __syncthreads_or(!fin) != 0;
    if (tid < E && p.obs_out != nullptr) {
      // FP32 (hi, lo) sums across the warps, staged in the 16-byte output
      // slot; widened to FP64 after the run (no FP64 arithmetic per step)
      float hx = red[0][tid][0], lx = red[0][tid][1], hy = red[0][tid][2], ly = red[0][tid][3];
      for (int w = 1; w < kRWarps; ++w) {
        float sum, er;
        rf_two_sum(hx, red[w][tid][0], sum, er);
        lx += red[w][tid][1] + er;
        hx = sum;
        rf_two_sum(hy, red[w][tid][2], sum, er);
        ly += red[w][tid][3] + er;
        hy = sum;
      }
      *reinterpret_cast<float4*>(p.obs_out + ((long long)b * p.nt + step) * E + tid) = make_float4(hx, lx, hy, ly);
    }
    if (bad) {
      if (tid == 0) p.err[b] = 4;  // LGB_ERR_NONFINITE
      nsteps = step + 1;
      break;
    }
    __syncthreads();
  }
  if (p.obs_out != nullptr) {
    __syncthreads();
    double2* o = p.obs_out + (long long)b * p.nt * E;
    for (long long i = tid; i < (long long)nsteps * E; i += kRThreads) {
      const float4 v = *reinterpret_cast<const float4*>(o + i);
      o[i] = make_double2((double)v.x + (double)v.y, (double)v.z + (double)v.w);
    }
  }
  if (nsteps < p.nt) return;
  if (p.rho_out != nullptr && owner) p.rho_out[p.voff[b] + r] = make_double2(y.x, y.y);
}

}  // namespace
}  // namespace lgb

// ---- C ABI -----------------------------------------------------------------------
struct lgb_redfield_plan {
  lgb_redfield_problem_t prob{};
  std::vector<int> dims;
  std::vector<long long> roff, voff;
  std::vector<unsigned char> rsm;
  long long tot_r = 0, tot_v = 0;
  size_t smem = 0;
  bool reg = false;  // FP32 and every N^2 <= 64: the register-resident kernel
  int* d_dims = nullptr;
  long long* d_roff = nullptr;
  long long* d_voff = nullptr;
  unsigned char* d_rsm = nullptr;
  void* d_R = nullptr;
  double2* d_Ot = nullptr;
  int* d_err = nullptr;
  bool ready = false;
};

namespace {

void rf_free(lgb_redfield_plan* pl) {
  cudaFree(pl->d_dims);
  cudaFree(pl->d_roff);
  cudaFree(pl->d_voff);
  cudaFree(pl->d_rsm);
  cudaFree(pl->d_R);
  cudaFree(pl->d_Ot);
  cudaFree(pl->d_err);
}

template <typename V>
bool rf_upload(V** d, const std::vector<V>& h) {
  if (cudaMalloc(d, std::max<size_t>(1, h.size()) * sizeof(V)) != cudaSuccess) return false;
  return cudaMemcpy(*d, h.data(), h.size() * sizeof(V), cudaMemcpyHostToDevice) == cudaSuccess;
}

}  // namespace

extern "C" {

int lgb_redfield_tensor(int32_t n, int32_t n_ops, const double* evals, const double* A,
                        const double* C, double* R_out, void* stream) {
  if (n < 1 || n > lgb_redfield_max_dim(LGB_PREC_FP32) || n_ops < 0 || evals == nullptr ||
      R_out == nullptr || (n_ops > 0 && (A == nullptr || C == nullptr)))
    return LGB_ERR_INVALID_ARG;
  const long long total = (long long)n * n * n * n;
  const int grid = (int)std::min<long long>((total + 255) / 256, 8192);
  lgb::redfield_tensor_kernel<<<grid, 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      n, n_ops, evals, reinterpret_cast<const double2*>(A), C, reinterpret_cast<double2*>(R_out));
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

int lgb_redfield_tensor_batch(int32_t n_sys, const int32_t* dims_host, int32_t n_ops, const double* evals,
                              const double* A, const double* C, double* R_out, void* stream) {
  if (n_sys < 1 || dims_host == nullptr || n_ops < 0 || evals == nullptr || R_out == nullptr ||
      (n_ops > 0 && (A == nullptr || C == nullptr)))
    return LGB_ERR_INVALID_ARG;
  std::vector<int> dims(n_sys);
  std::vector<long long> eoff(n_sys), moff(n_sys), roff(n_sys);
  long long te = 0, tm = 0, tr = 0, maxr = 1;
  for (int b = 0; b < n_sys; ++b) {
    const int n = dims_host[b];
    if (n < 1 || n > lgb_redfield_max_dim(LGB_PREC_FP32)) return LGB_ERR_INVALID_ARG;
    dims[b] = n;
    eoff[b] = te;
    moff[b] = tm;
    roff[b] = tr;
    te += n;
    tm += (long long)n * n;
    tr += (long long)n * n * n * n;
    maxr = std::max(maxr, (long long)n * n * n * n);
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  int* d_dims = nullptr;
  long long* d_off = nullptr;
  if (cudaMallocAsync(&d_dims, n_sys * sizeof(int), st) != cudaSuccess) return LGB_ERR_CUDA;
  if (cudaMallocAsync(&d_off, 3 * (size_t)n_sys * sizeof(long long), st) != cudaSuccess) {
    cudaFreeAsync(d_dims, st);
    return LGB_ERR_CUDA;
  }
  std::vector<long long> offs;
  offs.insert(offs.end(), eoff.begin(), eoff.end());
  offs.insert(offs.end(), moff.begin(), moff.end());
  offs.insert(offs.end(), roff.begin(), roff.end());
  bool ok = cudaMemcpyAsync(d_dims, dims.data(), n_sys * sizeof(int), cudaMemcpyHostToDevice, st) == cudaSuccess &&
            cudaMemcpyAsync(d_off, offs.data(), offs.size() * sizeof(long long), cudaMemcpyHostToDevice, st) ==
                cudaSuccess;
  if (ok) {
    const int gx = (int)std::min<long long>((maxr + 255) / 256, 64);
    lgb::redfield_tensor_batch_kernel<<<dim3(gx, n_sys), 256, 0, st>>>(
        n_ops, d_dims, d_off, d_off + n_sys, d_off + 2 * n_sys, evals, reinterpret_cast<const double2*>(A), C,
        reinterpret_cast<double2*>(R_out));
    ok = cudaGetLastError() == cudaSuccess;
  }
  // the host vectors must outlive the asynchronous copies
  cudaStreamSynchronize(st);
  cudaFreeAsync(d_dims, st);
  cudaFreeAsync(d_off, st);
  return ok ? LGB_OK : LGB_ERR_CUDA;
}

int lgb_redfield_max_dim(int32_t precision) { return precision == LGB_PREC_FP64 ? 48 : 64; }

int lgb_redfield_create(lgb_redfield_t* plan, const lgb_redfield_problem_t* prob, const int32_t* dims) {
  if (plan == nullptr || prob == nullptr || dims == nullptr) return LGB_ERR_INVALID_ARG;
  *plan = nullptr;
  const lgb_redfield_problem_t& pr = *prob;
  if (pr.n_inst < 1 || pr.n_eops < 0 || pr.n_eops > 16 || pr.nt < 0 || pr.store_every < 0 ||
      pr.reserved != 0 || !(pr.dt == pr.dt))
    return LGB_ERR_INVALID_ARG;
  if (pr.precision != LGB_PREC_FP64 && pr.precision != LGB_PREC_FP32) return LGB_ERR_UNSUPPORTED;
  auto* pl = new lgb_redfield_plan();
  pl->prob = pr;
  const size_t esz = pr.precision == LGB_PREC_FP64 ? 16 : 8;
  for (int b = 0; b < pr.n_inst; ++b) {
    const int N = dims[b];
    if (N < 1 || N > lgb_redfield_max_dim(pr.precision)) {
      delete pl;
      return N < 1 ? LGB_ERR_INVALID_ARG : LGB_ERR_UNSUPPORTED;
    }
    const long long M = (long long)N * N;
    pl->dims.push_back(N);
    pl->roff.push_back(pl->tot_r);
    pl->voff.push_back(pl->tot_v);
    pl->tot_r += M * M;
    pl->tot_v += M;
    const size_t vec = 4 * (size_t)M * esz, gen = (size_t)(M * M) * esz;
    const bool in_smem = vec + gen <= lgb::kRSmemBudget;
    pl->rsm.push_back(in_smem ? 1 : 0);
    pl->smem = std::max(pl->smem, vec + (in_smem ? gen : 0));
  }
  pl->reg = pr.precision == LGB_PREC_FP32 &&
            std::all_of(pl->dims.begin(), pl->dims.end(), [](int d) { return d * d <= lgb::kRRegM; });
  bool ok = rf_upload(&pl->d_dims, pl->dims) && rf_upload(&pl->d_roff, pl->roff) &&
            rf_upload(&pl->d_voff, pl->voff) && rf_upload(&pl->d_rsm, pl->rsm) &&
            cudaMalloc(&pl->d_R, std::max<long long>(1, pl->tot_r) * esz) == cudaSuccess &&
            cudaMalloc(&pl->d_Ot, std::max<long long>(1, (long long)pr.n_eops * pl->tot_v) * sizeof(double2)) ==
                cudaSuccess &&
            cudaMalloc(&pl->d_err, pr.n_inst * sizeof(int)) == cudaSuccess &&
            cudaMemset(pl->d_err, 0, pr.n_inst * sizeof(int)) == cudaSuccess;
  if (!ok) {
    rf_free(pl);
    delete pl;
    return LGB_ERR_CUDA;
  }
  *plan = pl;
  return LGB_OK;
}

int lgb_redfield_destroy(lgb_redfield_t plan) {
  if (plan == nullptr) return LGB_ERR_INVALID_ARG;
  cudaDeviceSynchronize();
  rf_free(plan);
  delete plan;
  return LGB_OK;
}

int lgb_redfield_set(lgb_redfield_t plan, const double* R, const double* eops, void* stream) {
  if (plan == nullptr || R == nullptr || (plan->prob.n_eops > 0 && eops == nullptr)) return LGB_ERR_INVALID_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const long long n = plan->tot_r;
  const int grid = (int)std::min<long long>((n + 255) / 256, 8192);
  if (plan->prob.precision == LGB_PREC_FP64) {
    if (cudaMemcpyAsync(plan->d_R, R, n * sizeof(double2), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
      return LGB_ERR_CUDA;
  } else {
    lgb::redfield_convert_kernel<float><<<grid, 256, 0, st>>>(reinterpret_cast<const double2*>(R),
                                                              reinterpret_cast<float2*>(plan->d_R), n);
  }
  if (plan->prob.n_eops > 0 &&
      cudaMemcpyAsync(plan->d_Ot, eops, (size_t)plan->prob.n_eops * plan->tot_v * sizeof(double2),
                      cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return LGB_ERR_CUDA;
  if (cudaGetLastError() != cudaSuccess) return LGB_ERR_CUDA;
  plan->ready = true;
  return LGB_OK;
}

int lgb_redfield_propagate(lgb_redfield_t plan, const double* rho0, double* obs_out, double* rho_out,
                           double* states_out, void* stream) {
  if (plan == nullptr || rho0 == nullptr) return LGB_ERR_INVALID_ARG;
  if (!plan->ready) return LGB_ERR_STATE;
  const lgb_redfield_problem_t& pr = plan->prob;
  if (states_out != nullptr && pr.store_every == 0) return LGB_ERR_INVALID_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  lgb::RedfieldParams p{};
  p.n_inst = pr.n_inst;
  p.n_eops = pr.n_eops;
  p.nt = pr.nt;
  p.store_every = pr.store_every;
  p.dt = pr.dt;
  p.dims = plan->d_dims;
  p.roff = plan->d_roff;
  p.voff = plan->d_voff;
  p.rsm = plan->d_rsm;
  p.R = plan->d_R;
  p.Ot = plan->d_Ot;
  p.rho0 = reinterpret_cast<const double2*>(rho0);
  p.obs_out = reinterpret_cast<double2*>(obs_out);
  p.rho_out = reinterpret_cast<double2*>(rho_out);
  p.states_out = reinterpret_cast<double2*>(states_out);
  p.err = plan->d_err;
  cudaError_t e;
  if (pr.precision == LGB_PREC_FP64) {
    e = cudaFuncSetAttribute(lgb::redfield_rk4_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)plan->smem);
    if (e == cudaSuccess)
      lgb::redfield_rk4_kernel<double><<<pr.n_inst, lgb::kRThreads, plan->smem, st>>>(p);
  } else if (plan->reg) {
    const bool all8 = std::all_of(plan->dims.begin(), plan->dims.end(), [](int d) { return d == 8; });
    if (all8)
      lgb::redfield_rk4_reg_kernel<64><<<pr.n_inst, lgb::kRThreads, 0, st>>>(p);
    else
      lgb::redfield_rk4_reg_kernel<0><<<pr.n_inst, lgb::kRThreads, 0, st>>>(p);
    e = cudaSuccess;
  } else {
    e = cudaFuncSetAttribute(lgb::redfield_rk4_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)plan->smem);
    if (e == cudaSuccess)
      lgb::redfield_rk4_kernel<float><<<pr.n_inst, lgb::kRThreads, plan->smem, st>>>(p);
  }
  if (e != cudaSuccess) return LGB_ERR_CUDA;
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

int lgb_redfield_errors(lgb_redfield_t plan, int32_t* flags_host) {
  if (plan == nullptr || flags_host == nullptr) return LGB_ERR_INVALID_ARG;
  const cudaError_t e =
      cudaMemcpy(flags_host, plan->d_err, plan->prob.n_inst * sizeof(int), cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

}  // extern "C"
