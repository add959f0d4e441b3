// Discrete adjoint of the frozen-H RK4 propagation (FP32, N <= 64, dense or
// no collapse operators, up to four drive terms).
//
// Forward step k (H frozen at t_{k+1}, pyqed/oqs.py:1792-1796):
//   Y1 = rho_k, Y2 = rho_k + h/2 L Y1, Y3 = rho_k + h/2 L Y2, Y4 = rho_k + h L Y3,
//   rho_{k+1} = rho_k + h/6 (L Y1 + 2 L Y2 + 2 L Y3 + L Y4),
// with L(X) = A X + X A^dag + sum_j L_j X L_j^dag.  With the Hilbert-Schmidt
// product <P, Q> = Re Tr[P^dag Q] and lambda' = dJ/drho_{k+1}, the exact
// adjoint of that step is
//   nu4 = h/6 lambda'                      w4 = L^dag nu4
//   nu3 = h/3 lambda' + h   w4             w3 = L^dag nu3
//   nu2 = h/3 lambda' + h/2 w3             w2 = L^dag nu2
//   nu1 = h/6 lambda' + h/2 w2             w1 = L^dag nu1
//   lambda_k = lambda' + w1 + w2 + w3 + w4 + g_k O^dag,
// where L^dag(X) = A^dag X + X A + sum_j L_j^dag X L_j has the forward form
// with A -> A^dag, L_j -> L_j^dag, and g_k is the gradient of the loss with
// respect to the observable Tr[O rho_k].  Parameter gradients are
// sum_stages Re<nu_s, (dL/dtheta) Y_s>:
//   drive f_d:      dL/df_d (Y) = i[H_d, Y]  -> Re sum_ij (i H_d)^T_ij M_ij,
//   H0:             Gamma = i M^dag accumulated (dJ = Re Tr[Gamma^dag dH0]),
//   rate scale s_j: (L_j -> sqrt(s_j) L_j) <L_j^dag nu L_j, Y> - 1/2 Re Tr[L_j^dag L_j (P + Q)],
// with P = Y nu^dag, Q = nu^dag Y, M = P - Q.  The stage inputs Y come from a
// recompute pass of the forward kernel over one checkpoint segment; this
// kernel walks that segment backwards, one CTA per instance, holding the
// costate in registers and the operands in shared memory.
#include "lgb_common.cuh"
#include "lgb_internal.h"

namespace lgb {

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;

__device__ __forceinline__ float2 cz() { return make_float2(0.f, 0.f); }
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 cscale(float s, float2 a) { return make_float2(s * a.x, s * a.y); }
// Re(conj(a) b)
__device__ __forceinline__ float redot(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }
// Re(a b)
__device__ __forceinline__ float remul(float2 a, float2 b) { return a.x * b.x - a.y * b.y; }

__device__ double block_sum(double v, double* sbuf) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sbuf[w] = v;
  __syncthreads();
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < kWarps; ++k) s += sbuf[k];
  return s;  // every thread
}

__global__ void __launch_bounds__(kThreads, 1) adjoint_segment_kernel(AdjParams p) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double sbuf[kWarps];
  const int b = p.order[blockIdx.x];
  const int N = p.dims[b];
  const int NP = p.npad[b];
  const int NPS = NP + 2;
  const int MS = NP * NPS;
  const int nT = NP >> 2;
  const int tid = threadIdx.x;
  const bool act = tid < nT * nT;
  const int ty = act ? tid / nT : 0, tx = act ? tid - (tid / nT) * nT : 0;
  const int i0 = 4 * ty;
  const int K = p.n_cops;
  const int D = p.n_drive;
  const int E = p.n_eops;
  const long long wo = p.woff[b];
  const float h = (float)p.dt;

  float2* sAdj = reinterpret_cast<float2*>(smem);  // conj(A) row-major = (A^dag)^T
  float2* sX = sAdj + MS;                          // nu
  float2* sXt = sX + MS;                           // nu^T
  float2* sB = sXt + MS;                           // max(K, 2) scratch slabs
  const float2* At0 = p.At + wo;
  const float2* Gt = p.Gt + (long long)D * wo;
  const float2* Lt = p.Lt + (long long)K * wo;
  float2* Lc = p.Lc + (long long)K * wo;
  float2* GkT = p.GkT + (long long)K * wo;
  float2* Macc = p.Macc + wo;
  float2* lamg = p.lam + wo;
  const float2* ys = p.ys + 4LL * p.ycap * wo;
  const double2* Ot = p.Ot + (long long)E * wo;
  const int dld = p.drive_ld;
  const double* drv = p.drive + (p.drive_shared ? 0 : (long long)b * D * dld);

  auto elem = [&](int ii, int jj, int& i, int& j) {
    i = i0 + ii;
    j = tx + nT * jj;
  };
  // observable gradient at state k: sum_e g[row(k)][e] O_e^dag, or zero
  auto obs_term = [&](int k, int ii, int jj) -> float2 {
    const int row = k - 1 + p.obs_t0;
    if (row < 0 || E == 0 || p.obs_grad == nullptr) return cz();
    int i, j;
    elem(ii, jj, i, j);
    double2 acc = make_double2(0.0, 0.0);
    for (int e = 0; e < E; ++e) {
      const double2 g = p.obs_grad[((long long)b * p.nt + row) * E + e];
      const double2 o = Ot[(long long)e * MS + i * NPS + j];  // O[j][i]; O^dag[i][j] = conj(o)
      acc.x += g.x * o.x + g.y * o.y;
      acc.y += g.y * o.x - g.x * o.y;
    }
    return make_float2((float)acc.x, (float)acc.y);
  };

  float2 lam[4][4];
  if (p.first_segment) {
    // operator-side scratch: conj(L_k) row-major and (L_k^dag L_k)^T
    for (int kc = 0; kc < K; ++kc) {
      for (int idx = tid; idx < MS; idx += kThreads) {
        const int r = idx / NPS, c = idx % NPS;
        Lc[(long long)kc * MS + idx] = (r < NP && c < NP) ? cconj(Lt[(long long)kc * MS + c * NPS + r]) : cz();
      }
    }
    if (act) {
      for (int kc = 0; kc < K; ++kc) {
        const float2* L = Lt + (long long)kc * MS;  // L^T: L[m][x] = L[x*NPS + m]... stored as Lt[m][x]
#pragma unroll
        for (int ii = 0; ii < 4; ++ii)
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            int i, j;
            elem(ii, jj, i, j);
            // G^T[i][j] = G[j][i] = sum_m conj(L[m][j]) L[m][i],  L[m][x] = Lt[x][m]
            float2 s = cz();
            for (int m = 0; m < NP; ++m) {
              const float2 u = L[j * NPS + m], v = L[i * NPS + m];
              s.x += u.x * v.x + u.y * v.y;
              s.y += u.x * v.y - u.y * v.x;
            }
            GkT[(long long)kc * MS + i * NPS + j] = s;
          }
      }
#pragma unroll
      for (int ii = 0; ii < 4; ++ii)
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          int i, j;
          elem(ii, jj, i, j);
          Macc[i * NPS + j] = cz();
          lam[ii][jj] = obs_term(p.nt, ii, jj);
        }
    }
    __syncthreads();
  } else if (act) {
#pragma unroll
    for (int ii = 0; ii < 4; ++ii)
#pragma unroll
      for (int jj = 0; jj < 4; ++jj) {
        int i, j;
        elem(ii, jj, i, j);
        lam[ii][jj] = lamg[i * NPS + j];
      }
  }

  double gscale[4] = {0.0, 0.0, 0.0, 0.0};  // per collapse operator (K <= 4)

  for (int kk = p.seg_len - 1; kk >= 0; --kk) {
    const int k = p.seg0 + kk;  // global step index
    // adjoint generator of step k: sAdj = conj(A_k) with A_k = A0 + sum_d f_d (i H_d)
    float f[4];
#pragma unroll
    for (int d = 0; d < 4; ++d) f[d] = d < D ? (float)drv[(long long)d * dld + k] : 0.f;
    __syncthreads();
    for (int idx = tid; idx < MS; idx += kThreads) {
      const int r = idx / NPS, c = idx % NPS;
      float2 a = cz();
      if (r < NP && c < NP) {
        a = At0[c * NPS + r];  // A[r][c]
#pragma unroll
        for (int d = 0; d < 4; ++d)
          if (d < D) {
            const float2 g = Gt[(long long)d * MS + c * NPS + r];
            a.x = fmaf(f[d], g.x, a.x);
            a.y = fmaf(f[d], g.y, a.y);
          }
      }
      sAdj[idx] = cconj(a);
    }
    float2 wprev[4][4], wsum[4][4];
#pragma unroll
    for (int ii = 0; ii < 4; ++ii)
#pragma unroll
      for (int jj = 0; jj < 4; ++jj) wprev[ii][jj] = wsum[ii][jj] = cz();
    double dE[4] = {0.0, 0.0, 0.0, 0.0};

#pragma unroll 1
    for (int s = 3; s >= 0; --s) {
      const float cs = h * ((s == 0 || s == 3) ? (1.f / 6.f) : (1.f / 3.f));
      const float ds = (s == 3) ? 0.f : (s == 2 ? h : 0.5f * h);
      const float2* Ys = ys + (long long)(kk * 4 + s) * MS;
      // nu_s -> sX, sXt
      __syncthreads();
      if (act) {
#pragma unroll
        for (int ii = 0; ii < 4; ++ii)
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            int i, j;
            elem(ii, jj, i, j);
            float2 nu = cscale(cs, lam[ii][jj]);
            nu.x = fmaf(ds, wprev[ii][jj].x, nu.x);
            nu.y = fmaf(ds, wprev[ii][jj].y, nu.y);
            sX[i * NPS + j] = nu;
            sXt[j * NPS + i] = nu;
          }
      }
      __syncthreads();
      // phase A: Y'_j = L_j^dag nu -> transposed into sB[j]
      if (act) {
        for (int kc = 0; kc < K; ++kc) {
          const float2* Ls = Lc + (long long)kc * MS;
          float2 t[4][4];
#pragma unroll
          for (int ii = 0; ii < 4; ++ii)
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) t[ii][jj] = cz();
          for (int m = 0; m < NP; ++m) {
            float2 a[4], x[4];
#pragma unroll
            for (int ii = 0; ii < 4; ++ii) a[ii] = Ls[m * NPS + i0 + ii];
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) x[jj] = sX[m * NPS + tx + nT * jj];
#pragma unroll
            for (int ii = 0; ii < 4; ++ii)
#pragma unroll
              for (int jj = 0; jj < 4; ++jj) cmac(t[ii][jj], a[ii], x[jj]);
          }
          float2* Y = sB + (long long)kc * MS;
#pragma unroll
          for (int ii = 0; ii < 4; ++ii)
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) Y[(tx + nT * jj) * NPS + i0 + ii] = t[ii][jj];
        }
      }
      __syncthreads();
      // phase B: w = A^dag nu + nu A + sum_j Y'_j L_j, with <L_j^dag nu L_j, Y_s> per j
      float2 acc[4][4];
#pragma unroll
      for (int ii = 0; ii < 4; ++ii)
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) acc[ii][jj] = cz();
      if (act) {
        for (int m = 0; m < NP; ++m) {
          float2 a[4], y[4], x[4], bb[4];
#pragma unroll
          for (int ii = 0; ii < 4; ++ii) {
            a[ii] = sAdj[m * NPS + i0 + ii];
            y[ii] = sXt[m * NPS + i0 + ii];
          }
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            x[jj] = sX[m * NPS + tx + nT * jj];
            bb[jj] = sAdj[m * NPS + tx + nT * jj];
          }
#pragma unroll
          for (int ii = 0; ii < 4; ++ii)
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) {
              cmac(acc[ii][jj], a[ii], x[jj]);
              cmacc(acc[ii][jj], y[ii], bb[jj]);
            }
        }
        for (int kc = 0; kc < K; ++kc) {
          const float2* Y = sB + (long long)kc * MS;
          const float2* Ls = Lc + (long long)kc * MS;
          float2 t[4][4];
#pragma unroll
          for (int ii = 0; ii < 4; ++ii)
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) t[ii][jj] = cz();
          for (int m = 0; m < NP; ++m) {
            float2 y[4], l[4];
#pragma unroll
            for (int ii = 0; ii < 4; ++ii) y[ii] = Y[m * NPS + i0 + ii];
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) l[jj] = Ls[m * NPS + tx + nT * jj];
#pragma unroll
            for (int ii = 0; ii < 4; ++ii)
#pragma unroll
              for (int jj = 0; jj < 4; ++jj) cmacc(t[ii][jj], y[ii], l[jj]);
          }
          float gz = 0.f;
#pragma unroll
          for (int ii = 0; ii < 4; ++ii)
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) {
              int i, j;
              elem(ii, jj, i, j);
              acc[ii][jj] = cadd(acc[ii][jj], t[ii][jj]);
              gz += redot(t[ii][jj], Ys[i * NPS + j]);
            }
          if (kc < 4) gscale[kc] += (double)gz;
        }
#pragma unroll
        for (int ii = 0; ii < 4; ++ii)
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            wprev[ii][jj] = acc[ii][jj];
            wsum[ii][jj] = cadd(wsum[ii][jj], acc[ii][jj]);
          }
      }
      // gradients: P = Y nu^dag, Q = nu^dag Y with Y = Y_s in sB[0] (row-major) / sB[1] (transposed)
      __syncthreads();
      float2* sY = sB;
      float2* sYt = sB + MS;
      if (act) {
#pragma unroll
        for (int ii = 0; ii < 4; ++ii)
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            int i, j;
            elem(ii, jj, i, j);
            const float2 v = Ys[i * NPS + j];
            sY[i * NPS + j] = v;
            sYt[j * NPS + i] = v;
          }
      }
      __syncthreads();
      if (act) {
        float2 P[4][4], Q[4][4];
#pragma unroll
        for (int ii = 0; ii < 4; ++ii)
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) P[ii][jj] = Q[ii][jj] = cz();
        for (int c = 0; c < NP; ++c) {
          float2 yt[4], nt4[4], nu[4], yv[4];
#pragma unroll
          for (int ii = 0; ii < 4; ++ii) {
            yt[ii] = sYt[c * NPS + i0 + ii];  // Y[i][c]
            nu[ii] = sX[c * NPS + i0 + ii];   // nu[c][i]
          }
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            nt4[jj] = sXt[c * NPS + tx + nT * jj];  // nu[j][c]
            yv[jj] = sY[c * NPS + tx + nT * jj];    // Y[c][j]
          }
#pragma unroll
          for (int ii = 0; ii < 4; ++ii)
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) {
              cmacc(P[ii][jj], yt[ii], nt4[jj]);             // Y[i][c] conj(nu[j][c])
              cmac(Q[ii][jj], cconj(nu[ii]), yv[jj]);        // conj(nu[c][i]) Y[c][j]
            }
        }
        float ge[4] = {0.f, 0.f, 0.f, 0.f};
        float gq[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int ii = 0; ii < 4; ++ii)
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            int i, j;
            elem(ii, jj, i, j);
            const float2 M = make_float2(P[ii][jj].x - Q[ii][jj].x, P[ii][jj].y - Q[ii][jj].y);
            const float2 S = cadd(P[ii][jj], Q[ii][jj]);
            Macc[i * NPS + j] = cadd(Macc[i * NPS + j], M);
#pragma unroll
            for (int d = 0; d < 4; ++d)
              if (d < D) ge[d] += remul(Gt[(long long)d * MS + i * NPS + j], M);
            for (int kc = 0; kc < K && kc < 4; ++kc)
              gq[kc] += remul(GkT[(long long)kc * MS + i * NPS + j], S);
          }
#pragma unroll
        for (int d = 0; d < 4; ++d) dE[d] += (double)ge[d];
#pragma unroll
        for (int kc = 0; kc < 4; ++kc) gscale[kc] -= 0.5 * (double)gq[kc];
      }
    }
    // lambda_k = lambda' + sum_s w_s + g_k O^dag
    if (act) {
#pragma unroll
      for (int ii = 0; ii < 4; ++ii)
#pragma unroll
        for (int jj = 0; jj < 4; ++jj)
          lam[ii][jj] = cadd(cadd(lam[ii][jj], wsum[ii][jj]), obs_term(k, ii, jj));
    }
    for (int d = 0; d < D; ++d) {
      const double v = block_sum(dE[d], sbuf);
      if (tid == 0 && p.dE != nullptr) p.dE[((long long)b * D + d) * p.nt + k] = v;
    }
  }

  if (act) {
#pragma unroll
    for (int ii = 0; ii < 4; ++ii)
#pragma unroll
      for (int jj = 0; jj < 4; ++jj) {
        int i, j;
        elem(ii, jj, i, j);
        lamg[i * NPS + j] = lam[ii][jj];
      }
  }
  for (int kc = 0; kc < K && kc < 4; ++kc) {
    const double v = block_sum(gscale[kc], sbuf);
    if (tid == 0 && p.dscale != nullptr) p.dscale[(long long)b * K + kc] += v;
  }
  (void)N;
}

// lambda_0 and Gamma = i M^dag out of the padded working layout (complex128, packed).
__global__ void adjoint_finish_kernel(AdjParams p, const long long* off, double2* drho0,
                                      double2* dH) {
  const int b = blockIdx.y;
  const int N = p.dims[b];
  const int NP = p.npad[b];
  const int NPS = NP + 2;
  const long long wo = p.woff[b];
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < N * N; idx += gridDim.x * blockDim.x) {
    const int i = idx / N, j = idx % N;
    if (drho0 != nullptr) {
      const float2 l = p.lam[wo + i * NPS + j];
      drho0[off[b] + idx] = make_double2(l.x, l.y);
    }
    if (dH != nullptr) {
      // Gamma[i][j] = i conj(M[j][i])
      const float2 m = p.Macc[wo + j * NPS + i];
      dH[off[b] + idx] = make_double2(m.y, m.x);
    }
  }
}

}  // namespace

int adjoint_smem_bytes(int npad, int K) {
  const long long ms = (long long)npad * (npad + 2) * sizeof(float2);
  return (int)((3 + (K > 2 ? K : 2)) * ms);
}

cudaError_t launch_adjoint_segment(const AdjParams& p, int n_blocks, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(adjoint_segment_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, p.smem_bytes);
  if (e != cudaSuccess) return e;
  adjoint_segment_kernel<<<n_blocks, kThreads, p.smem_bytes, st>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_adjoint_finish(const AdjParams& p, const long long* off, double2* drho0,
                                  double2* dH, cudaStream_t st) {
  dim3 grid(16, p.n_inst);
  adjoint_finish_kernel<<<grid, 256, 0, st>>>(p, off, drho0, dH);
  return cudaGetLastError();
}

}  // namespace lgb
