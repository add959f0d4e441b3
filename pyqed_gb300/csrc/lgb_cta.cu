// CTA-resident batched RK4 propagator on the FP32 / FP64 pipes.
//
// One CTA owns one instance for all Nt steps.  A^T (A = -i H_eff), the stage
// input X and its transpose X^T live in shared memory; each of the 256
// threads owns 4x4 tiles of the N x N state (rows 4*ty..4*ty+3, columns
// tx + nT*j) and keeps rho and the RK4 sum in registers (FP32, N <= 64) or in
// a private global workspace slab (FP64 and 64 < N <= 88).
//
// Per RK4 stage (pyqed/phys.py:1051-1064 with the RHS of pyqed/oqs.py:697-715
// rewritten as R = A X + X A^dag + sum_k L_k X L_k^dag, or + D o X for
// diagonal collapse operators):
//   [dense c_ops]  Y_k = L_k X  -> Y_k^T in shared memory        (sync)
//   R = A X + X A^dag + sum_k Y_k L_k^dag  (register-tiled)      (sync)
//   epilogue: RK4 stage combination, next stage input -> X, X^T  (sync)
// After the fourth stage the observables Tr[O rho] (pyqed/phys.py:1257-1264)
// are reduced in FP64 (warp shuffles + one shared-memory pass) and the state
// is checked for non-finite values.
#include <type_traits>

#include "lgb_common.cuh"
#include "lgb_internal.h"

namespace lgb {

namespace {

constexpr int kThreads = 256;      // default block: 4x4 tiles cover N <= 64 in one round
constexpr int kThreadsWide = 384;  // wide block: one round for 64 < N <= 76
constexpr int kMaxWarps = kThreadsWide / 32;
constexpr int kMaxEops = 16;

template <typename T2>
__device__ __forceinline__ void ld4(const T2* __restrict__ p, T2 v[4]) {
  if constexpr (sizeof(T2) == 8) {
    const float4 a = reinterpret_cast<const float4*>(p)[0];
    const float4 b = reinterpret_cast<const float4*>(p)[1];
    v[0] = make_float2(a.x, a.y);
    v[1] = make_float2(a.z, a.w);
    v[2] = make_float2(b.x, b.y);
    v[3] = make_float2(b.z, b.w);
  } else {
    v[0] = p[0];
    v[1] = p[1];
    v[2] = p[2];
    v[3] = p[3];
  }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename T, int NT, int ROUNDS, bool SREG, bool YS = false>
__device__ __forceinline__ void cta_body(const CtaParams& p, const int b, unsigned char* smem,
                                         double2 (*sRed)[kMaxEops], int* sFlag) {
  constexpr int kWarps = NT / 32;
  using T2 = typename Cplx<T>::type;
  constexpr int PADC = 16 / (int)sizeof(T2);
  const int N = p.dims[b];
  const int NP = p.npad[b];
  const int NPS = NP + PADC;
  const int MS = NP * NPS;
  const int nT = NP >> 2;
  const int ntiles = nT * nT;
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int K = p.n_cops;
  const bool dense = (p.cops_kind == 1) && K > 0;
  const bool diag = (p.cops_kind == 2) && K > 0;
  const int E = p.n_eops;
  const long long wo = p.woff[b];
  const T dt = (T)p.dt;
  const T half_dt = (T)(0.5 * p.dt);
  const T sixth_dt = (T)(p.dt / 6.0);

  T2* sAt = reinterpret_cast<T2*>(smem);
  T2* sX = sAt + MS;
  T2* sXt = sX + MS;
  T2* cursor = sXt + MS;
  const T2* Lt = nullptr;
  T2* Yt = nullptr;
  if (dense) {
    if (p.place[b] & 2) {
      Yt = cursor;
      cursor += (long long)K * MS;
    } else {
      Yt = reinterpret_cast<T2*>(p.y_ws) + (long long)K * wo;
    }
    const T2* Ltg = reinterpret_cast<const T2*>(p.Lt) + (long long)K * wo;
    if (p.place[b] & 1) {
      T2* sLt = cursor;
      for (int i = tid; i < K * MS; i += NT) sLt[i] = Ltg[i];
      Lt = sLt;
    } else {
      Lt = Ltg;
    }
  }
  const T2* At0 = reinterpret_cast<const T2*>(p.At) + wo;
  const T2* Dm = reinterpret_cast<const T2*>(p.Dm) + wo;
  const T2* Gt = reinterpret_cast<const T2*>(p.Gt) + (long long)p.n_drive * wo;
  const double2* Ot = p.Ot + (long long)E * wo;
  T2* wsRho = reinterpret_cast<T2*>(p.state_ws) + 2 * wo;
  T2* wsAcc = wsRho + MS;

  int ty[ROUNDS], tx[ROUNDS];
  bool act[ROUNDS];
#pragma unroll
  for (int r = 0; r < ROUNDS; ++r) {
    const int t = tid + r * NT;
    act[r] = t < ntiles;
    ty[r] = act[r] ? t / nT : 0;
    tx[r] = act[r] ? t - ty[r] * nT : 0;
  }

  // register state (SREG) -- unused otherwise
  T2 rrho[SREG ? ROUNDS : 1][4][4];
  T2 racc[SREG ? ROUNDS : 1][4][4];

  // ---- initial state -------------------------------------------------------
  const double2* r0 = p.rho0 + p.off[b];
#pragma unroll
  for (int r = 0; r < ROUNDS; ++r) {
    if (!act[r]) continue;
#pragma unroll
    for (int ii = 0; ii < 4; ++ii) {
#pragma unroll
      for (int jj = 0; jj < 4; ++jj) {
        const int i = 4 * ty[r] + ii, j = tx[r] + nT * jj;
        double2 v = make_double2(0.0, 0.0);
        if (i < N && j < N) v = r0[(long long)i * N + j];
        const T2 x = mk<T2>(v.x, v.y);
        sX[i * NPS + j] = x;
        sXt[j * NPS + i] = x;
        if constexpr (SREG) {
          rrho[r][ii][jj] = x;
        } else {
          wsRho[i * NPS + j] = x;
        }
      }
    }
  }
  if (p.n_drive == 0) {
    for (int i = tid; i < MS; i += NT) sAt[i] = At0[i];
  }

  // FP64 observables Tr[O rho] and a finiteness check of the current state.
  auto reduce_state = [&](int row) -> bool {
    bool fin = true;
#pragma unroll
    for (int r = 0; r < ROUNDS; ++r) {
      if (!act[r]) continue;
#pragma unroll
      for (int ii = 0; ii < 4; ++ii) {
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          const int i = 4 * ty[r] + ii, j = tx[r] + nT * jj;
          T2 x;
          if constexpr (SREG) {
            x = rrho[r][ii][jj];
          } else {
            x = wsRho[i * NPS + j];
          }
          fin = fin && cfinite(x);
        }
      }
    }
    for (int e = 0; e < E; ++e) {
      double sx = 0.0, sy = 0.0;
#pragma unroll
      for (int r = 0; r < ROUNDS; ++r) {
        if (!act[r]) continue;
#pragma unroll
        for (int ii = 0; ii < 4; ++ii) {
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            const int i = 4 * ty[r] + ii, j = tx[r] + nT * jj;
            T2 x;
            if constexpr (SREG) {
              x = rrho[r][ii][jj];
            } else {
              x = wsRho[i * NPS + j];
            }
            const double2 xd = to_d2(x);
            const double2 o = Ot[(long long)e * MS + i * NPS + j];
            sx += o.x * xd.x - o.y * xd.y;
            sy += o.x * xd.y + o.y * xd.x;
          }
        }
      }
      sx = warp_sum(sx);
      sy = warp_sum(sy);
      if (lane == 0) sRed[warp][e] = make_double2(sx, sy);
    }
    const unsigned bad = __ballot_sync(0xffffffffu, !fin);
    if (lane == 0) sFlag[warp] = bad != 0u;
    __syncthreads();
    bool anybad = false;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) anybad = anybad || sFlag[w];
    if (tid < E && p.obs_out != nullptr) {
      double2 s = make_double2(0.0, 0.0);
#pragma unroll
      for (int w = 0; w < kWarps; ++w) {
        s.x += sRed[w][tid].x;
        s.y += sRed[w][tid].y;
      }
      const long long nrows = (long long)p.nt + p.obs_t0;
      p.obs_out[((long long)b * nrows + row) * E + tid] = s;
    }
    return anybad;
  };

  // optional record of every stage input (the recompute pass of the adjoint)
  T2* ys = (YS && p.ystore != nullptr)
               ? reinterpret_cast<T2*>(p.ystore) + 4LL * p.ycap * wo : nullptr;
  auto ystore = [&](int slot, int i, int j, T2 v) {
    if constexpr (YS) {
      if (ys != nullptr) ys[(long long)slot * MS + i * NPS + j] = v;
    }
  };
  if (YS && ys != nullptr) {
#pragma unroll
    for (int r = 0; r < ROUNDS; ++r) {
      if (!act[r]) continue;
#pragma unroll
      for (int ii = 0; ii < 4; ++ii)
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          const int i = 4 * ty[r] + ii, j = tx[r] + nT * jj;
          ystore(0, i, j, sX[i * NPS + j]);
        }
    }
  }

  // Optional per-step check (p.check_tol > 0), accumulated in FP64: the drift
  // |Tr rho(t) - Tr rho0| and, when rho0 is Hermitian to the tolerance,
  // max_ij |rho_ij - conj(rho_ji)|, both read from the stage-input copy of
  // the state (X and X^T hold rho after the step).  Thread 0 keeps the
  // running maxima and writes them, and the LGB_ERR_CHECK flag, at the end.
  __shared__ double sChk[kMaxWarps][3];
  const bool checking = p.check_tol > 0.0 && p.chk != nullptr;
  double2 chk_tr0 = make_double2(0.0, 0.0);
  bool chk_herm = false, chk_bad = false;
  double chk_dtr = 0.0, chk_dh = 0.0;
  auto check_state = [&](bool initial) {
    double trx = 0.0, try_ = 0.0, hm = 0.0;
#pragma unroll
    for (int r = 0; r < ROUNDS; ++r) {
      if (!act[r]) continue;
#pragma unroll
      for (int ii = 0; ii < 4; ++ii) {
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          const int i = 4 * ty[r] + ii, j = tx[r] + nT * jj;
          if (i < N && j < N) {
            const double2 x = to_d2(sX[i * NPS + j]);
            const double2 xt = to_d2(sXt[i * NPS + j]);  // X^T[i][j] = X[j][i]
            if (i == j) {
              trx += x.x;
              try_ += x.y;
            }
            hm = fmax(hm, hypot(x.x - xt.x, x.y + xt.y));
          }
        }
      }
    }
    trx = warp_sum(trx);
    try_ = warp_sum(try_);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) hm = fmax(hm, __shfl_xor_sync(0xffffffffu, hm, o));
    if (lane == 0) {
      sChk[warp][0] = trx;
      sChk[warp][1] = try_;
      sChk[warp][2] = hm;
    }
    __syncthreads();
    if (tid == 0) {
      double2 tr = make_double2(0.0, 0.0);
      double h = 0.0;
      for (int w = 0; w < kWarps; ++w) {
        tr.x += sChk[w][0];
        tr.y += sChk[w][1];
        h = fmax(h, sChk[w][2]);
      }
      if (initial) {
        chk_tr0 = tr;
        chk_herm = h <= p.check_tol;
      } else {
        const double dtr = hypot(tr.x - chk_tr0.x, tr.y - chk_tr0.y);
        chk_dtr = fmax(chk_dtr, dtr);
        if (chk_herm) chk_dh = fmax(chk_dh, h);
        chk_bad = chk_bad || !(dtr <= p.check_tol) || (chk_herm && !(h <= p.check_tol));
      }
    }
  };

  if (tid == 0) p.err[b] = 0;
  __syncthreads();
  if (checking) check_state(true);
  if (p.obs_t0) reduce_state(0);

  const int dld = p.drive_ld > 0 ? p.drive_ld : p.nt;
  const double* drv = p.drive;
  if (p.n_drive > 0 && !p.drive_shared) drv += (long long)b * p.n_drive * dld;

  for (int step = 0; step < p.nt; ++step) {
    if (p.n_drive > 0) {
      // H(t_{k+1}) = H0 - sum_d f_d(t_{k+1}) H_d  ->  A = A0 + sum_d f_d (i H_d)
      T f[4];
#pragma unroll
      for (int d = 0; d < 4; ++d) f[d] = (d < p.n_drive) ? (T)drv[(long long)d * dld + step] : (T)0;
      for (int i = tid; i < MS; i += NT) {
        T2 a = At0[i];
#pragma unroll
        for (int d = 0; d < 4; ++d)
          if (d < p.n_drive) a = caxpy(a, f[d], Gt[(long long)d * MS + i]);
        sAt[i] = a;
      }
    }
    __syncthreads();

#pragma unroll 1
    for (int stage = 0; stage < 4; ++stage) {
      // ---- phase A: Y_k = L_k X -> Y_k^T --------------------------------
      if (dense) {
        for (int k = 0; k < K; ++k) {
          const T2* L = Lt + (long long)k * MS;
          T2* Y = Yt + (long long)k * MS;
#pragma unroll
          for (int r = 0; r < ROUNDS; ++r) {
            if (!act[r]) continue;
            T2 t[4][4];
#pragma unroll
            for (int ii = 0; ii < 4; ++ii)
#pragma unroll
              for (int jj = 0; jj < 4; ++jj) t[ii][jj] = mk<T2>(0.0, 0.0);
            const int i0 = 4 * ty[r];
#pragma unroll 2
            for (int m = 0; m < NP; ++m) {
              T2 a[4], x[4];
              ld4(L + m * NPS + i0, a);
#pragma unroll
              for (int jj = 0; jj < 4; ++jj) x[jj] = sX[m * NPS + tx[r] + nT * jj];
#pragma unroll
              for (int ii = 0; ii < 4; ++ii)
#pragma unroll
                for (int jj = 0; jj < 4; ++jj) cmac(t[ii][jj], a[ii], x[jj]);
            }
#pragma unroll
            for (int ii = 0; ii < 4; ++ii)
#pragma unroll
              for (int jj = 0; jj < 4; ++jj) Y[(tx[r] + nT * jj) * NPS + i0 + ii] = t[ii][jj];
          }
        }
        __syncthreads();
      }

      // ---- phase B: R = A X + X A^dag + sum_k Y_k L_k^dag ----------------
      T2 acc[ROUNDS][4][4];
#pragma unroll
      for (int r = 0; r < ROUNDS; ++r) {
#pragma unroll
        for (int ii = 0; ii < 4; ++ii)
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) acc[r][ii][jj] = mk<T2>(0.0, 0.0);
        if (!act[r]) continue;
        const int i0 = 4 * ty[r];
        const int c0 = tx[r];
#pragma unroll 4
        for (int k = 0; k < NP; ++k) {
          T2 a[4], y[4], x[4], bb[4];
          const T2* rowA = sAt + k * NPS;
          ld4(rowA + i0, a);
          ld4(sXt + k * NPS + i0, y);
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            x[jj] = sX[k * NPS + c0 + nT * jj];
            bb[jj] = rowA[c0 + nT * jj];
          }
#pragma unroll
          for (int ii = 0; ii < 4; ++ii)
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) {
              cmac(acc[r][ii][jj], a[ii], x[jj]);
              cmacc(acc[r][ii][jj], y[ii], bb[jj]);
            }
        }
        if (dense) {
          for (int k = 0; k < K; ++k) {
            const T2* L = Lt + (long long)k * MS;
            const T2* Y = Yt + (long long)k * MS;
#pragma unroll 2
            for (int m = 0; m < NP; ++m) {
              T2 y[4], l[4];
              ld4(Y + m * NPS + i0, y);
#pragma unroll
              for (int jj = 0; jj < 4; ++jj) l[jj] = L[m * NPS + c0 + nT * jj];
#pragma unroll
              for (int ii = 0; ii < 4; ++ii)
#pragma unroll
                for (int jj = 0; jj < 4; ++jj) cmacc(acc[r][ii][jj], y[ii], l[jj]);
            }
          }
        }
      }
      __syncthreads();

      // ---- phase C: RK4 stage combination --------------------------------
      const T cstage = (stage == 2) ? dt : half_dt;
#pragma unroll
      for (int r = 0; r < ROUNDS; ++r) {
        if (!act[r]) continue;
#pragma unroll
        for (int ii = 0; ii < 4; ++ii) {
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            const int i = 4 * ty[r] + ii, j = tx[r] + nT * jj;
            T2 R = acc[r][ii][jj];
            if (diag) {
              const T2 xc = sX[i * NPS + j];
              cmac(R, Dm[i * NPS + j], xc);
            }
            T2 rho, ra;
            if constexpr (SREG) {
              rho = rrho[r][ii][jj];
              ra = racc[r][ii][jj];
            } else {
              rho = wsRho[i * NPS + j];
              ra = (stage == 0) ? mk<T2>(0.0, 0.0) : wsAcc[i * NPS + j];
            }
            T2 xn;
            if (stage == 0) {
              ra = R;
              xn = caxpy(rho, cstage, R);
            } else if (stage < 3) {
              ra = caxpy(ra, (T)2, R);
              xn = caxpy(rho, cstage, R);
            } else {
              ra.x += R.x;
              ra.y += R.y;
              rho = caxpy(rho, sixth_dt, ra);
              xn = rho;
            }
            if constexpr (SREG) {
              rrho[r][ii][jj] = rho;
              racc[r][ii][jj] = ra;
            } else {
              if (stage < 3) {
                wsAcc[i * NPS + j] = ra;
              } else {
                wsRho[i * NPS + j] = rho;
              }
            }
            sX[i * NPS + j] = xn;
            sXt[j * NPS + i] = xn;
            if (stage < 3) {
              ystore(step * 4 + stage + 1, i, j, xn);
            } else if (step + 1 < p.nt) {
              ystore((step + 1) * 4, i, j, xn);
            }
          }
        }
      }
      if (stage < 3) __syncthreads();
    }

    // ---- after the step: observables, finiteness, stored states ----------
    const bool bad = reduce_state(step + p.obs_t0);
    if (bad) {
      if (tid == 0) p.err[b] = 4;  // LGB_ERR_NONFINITE
      break;
    }
    if (checking) check_state(false);
    if (p.store_every > 0 && p.states_out != nullptr && ((step + 1) % p.store_every) == 0) {
      const long long si = (step + 1) / p.store_every - 1;
      double2* dst = p.states_out + p.soff[b] +
                     si * (p.state_stride > 0 ? p.state_stride : (long long)N * N);
#pragma unroll
      for (int r = 0; r < ROUNDS; ++r) {
        if (!act[r]) continue;
#pragma unroll
        for (int ii = 0; ii < 4; ++ii)
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            const int i = 4 * ty[r] + ii, j = tx[r] + nT * jj;
            if (i < N && j < N) {
              T2 x;
              if constexpr (SREG) {
                x = rrho[r][ii][jj];
              } else {
                x = wsRho[i * NPS + j];
              }
              dst[(long long)i * N + j] = to_d2(x);
            }
          }
      }
    }
  }

  if (checking && tid == 0) {
    p.chk[2 * b] = chk_dtr;
    p.chk[2 * b + 1] = chk_herm ? chk_dh : -1.0;
    if (chk_bad && p.err[b] == 0) p.err[b] = 9;  // LGB_ERR_CHECK
  }
  if (p.rho_out != nullptr) {
    double2* dst = p.rho_out + p.off[b];
#pragma unroll
    for (int r = 0; r < ROUNDS; ++r) {
      if (!act[r]) continue;
#pragma unroll
      for (int ii = 0; ii < 4; ++ii)
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          const int i = 4 * ty[r] + ii, j = tx[r] + nT * jj;
          if (i < N && j < N) {
            T2 x;
            if constexpr (SREG) {
              x = rrho[r][ii][jj];
            } else {
              x = wsRho[i * NPS + j];
            }
            dst[(long long)i * N + j] = to_d2(x);
          }
        }
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads, 1) cta_rk4_kernel(CtaParams p) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double2 sRed[kThreads / 32][kMaxEops];
  __shared__ int sFlag[kThreads / 32];
  const int b = p.order[blockIdx.x];
  const int NP = p.npad[b];
  if constexpr (std::is_same<T, float>::value) {
    if (NP <= 64) {
      cta_body<T, kThreads, 1, true>(p, b, smem, sRed, sFlag);
    } else {
      cta_body<T, kThreads, 2, false>(p, b, smem, sRed, sFlag);
    }
  } else {
    if (NP <= 64) {
      cta_body<T, kThreads, 1, false>(p, b, smem, sRed, sFlag);
    } else {
      cta_body<T, kThreads, 2, false>(p, b, smem, sRed, sFlag);
    }
  }
}

// FP32, N <= 64, recording every stage input (the adjoint's recompute pass).
__global__ void __launch_bounds__(kThreads, 1) cta_rk4_record_kernel(CtaParams p) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double2 sRed[kThreads / 32][kMaxEops];
  __shared__ int sFlag[kThreads / 32];
  const int b = p.order[blockIdx.x];
  cta_body<float, kThreads, 1, true, true>(p, b, smem, sRed, sFlag);
}

// FP32, 64 < N <= 76: one 4x4 tile per thread, state in registers.
__global__ void __launch_bounds__(kThreadsWide, 1) cta_rk4_wide_kernel(CtaParams p) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double2 sRed[kThreadsWide / 32][kMaxEops];
  __shared__ int sFlag[kThreadsWide / 32];
  const int b = p.order[blockIdx.x];
  cta_body<float, kThreadsWide, 1, true>(p, b, smem, sRed, sFlag);
}

}  // namespace

int cta_max_npad() { return 88; }
int cta_wide_max_npad() { return 76; }

size_t cta_elem_bytes(int precision) { return precision == 0 ? sizeof(double2) : sizeof(float2); }

cudaError_t launch_cta_rk4(const CtaParams& p, int precision, int n_blocks, cudaStream_t stream,
                           bool wide) {
  if (n_blocks <= 0) return cudaSuccess;
  cudaError_t e;
  if (p.ystore != nullptr) {
    e = cudaFuncSetAttribute(cta_rk4_record_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             p.smem_bytes);
    if (e != cudaSuccess) return e;
    cta_rk4_record_kernel<<<n_blocks, kThreads, p.smem_bytes, stream>>>(p);
  } else if (wide) {
    e = cudaFuncSetAttribute(cta_rk4_wide_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             p.smem_bytes);
    if (e != cudaSuccess) return e;
    cta_rk4_wide_kernel<<<n_blocks, kThreadsWide, p.smem_bytes, stream>>>(p);
  } else if (precision == 0) {
    e = cudaFuncSetAttribute(cta_rk4_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             p.smem_bytes);
    if (e != cudaSuccess) return e;
    cta_rk4_kernel<double><<<n_blocks, kThreads, p.smem_bytes, stream>>>(p);
  } else {
    e = cudaFuncSetAttribute(cta_rk4_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             p.smem_bytes);
    if (e != cudaSuccess) return e;
    cta_rk4_kernel<float><<<n_blocks, kThreads, p.smem_bytes, stream>>>(p);
  }
  return cudaGetLastError();
}

}  // namespace lgb
