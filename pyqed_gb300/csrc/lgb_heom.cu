// Hierarchical equations of motion (pyqed/oqs.py:1332-1371, 1808-1935) on the GPU.
//
// The reference's HEOM keeps one exponential bath mode (correlation
// D(t) = D0 e^{-gamma t}) and a chain of nado auxiliary density operators
// X_0 .. X_{nado-1}, X_0 = rho, X_{nado-1} the zero terminator.  One explicit
// Euler step sweeps the levels in place, n = 0 .. nado-2:
//     X_n += dt ( -i[H, X_n] - [sz, X_{n+1}] - n gamma X_n
//                 + n (Re D0 [sz, X_{n-1}] + i Im D0 {sz, X_{n-1}}) ),
// where X_{n-1} is already the new value of this step and X_{n+1} the old one
// (pyqed/oqs.py:1854-1866).  The propagator form (pyqed/oqs.py:1877-1935) runs
// the same sweep on the Liouville-space propagator, which is the sweep applied
// to every basis matrix E_c, and advances level 0 twice per step
// (LGB_HEOM_DOUBLE_FIRST).
//
// heom_sweep_kernel: one thread group per system (G = 32..256 threads, a few
// groups per CTA, each with its own named barrier); a thread computes one
// column element of a pair of rows (r, r + ceil(N/2)), so both share the
// column loads and carry six independent accumulators each.  -iH, sz and,
// when they fit, all the levels stay in shared memory for the whole run; the
// levels otherwise live in a global workspace (L2-resident).  The in-place
// Gauss-Seidel sweep becomes a ring of nado slots: at step k level n lives in
// slot (n - k) mod nado and writes its new value into slot (n - k - 1) mod
// nado, the old slot of level n-1, which no later level of the step reads, so
// each level costs one group barrier.  A diagonal sz (LGB_HEOM_DIAG_SZ) turns
// its products into O(N^2) scalings.  FP32 compensates the update of level 0
// (Kahan); the deeper levels are small and enter level 0 only through
// dt [sz, X_1].  FP64 is the check path.  After every step the observables
// Tr[O X_0] are reduced in FP64 and X_0 is checked for non-finite values
// (LGB_ERR_NONFINITE stops that system).
#include <algorithm>
#include <vector>

#include "lgb_common.cuh"
#include "lgb_internal.h"

namespace lgb {

namespace {

constexpr int kHThreads = 256;
constexpr int kHWarps = kHThreads / 32;
constexpr int kHMaxEops = 16;
constexpr int kHMaxDim = 64;     // N^2 <= 16 x 256 elements per group
constexpr size_t kHSmemBudget = 200 * 1024;

struct HeomParams {
  int n_inst, n_eops, nt, nado, double_first;
  int G;       // threads per system (multiple of 32)
  int gpc;     // systems per CTA
  int NS;      // slot stride in elements (max N^2 of the batch)
  double dt;
  const int* dims;
  const long long* voff;  // packed N^2 offsets
  const double* bath;     // per system: gamma, Re D0, Im D0
  const double2* H;       // packed N x N (FP64)
  const double2* sz;
  const double2* Ot;      // vec(O_e^T), E x N^2 per system
  const float2* OtF;      // the same in FP32 (FP32 sweep)
  const double2* rho0;
  double2* obs_out;       // [n_inst][E][nt]
  double2* rho_out;       // X_0 after nt steps, packed
  double2* ado_out;       // all levels after nt steps: system b at nado * voff[b]
  void* ws;               // levels (and compensations) when they are not on chip
  int* err;
};

__device__ __forceinline__ void hbar(int id, int n) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}
__device__ __forceinline__ bool hbar_or(int id, int n, bool pred) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 q, %1, 0;\n\t"
      "bar.red.or.pred p, %2, %3, q;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)pred), "r"(id), "r"(n)
      : "memory");
  return r != 0;
}

// c -= a * b
template <typename T2> __device__ __forceinline__ void cmsub(T2& c, const T2 a, const T2 b) {
  c.x = fma(-a.x, b.x, c.x);
  c.x = fma(a.y, b.y, c.x);
  c.y = fma(-a.x, b.y, c.y);
  c.y = fma(-a.y, b.x, c.y);
}

// Products of one task, the column-c elements of rows r0 and r1 (two rows
// share every column load): acc[e] = {Am X, X Am, sz Y, Y sz, sz Z, Z sz}
// at (r_e, c), with Am = -iH, Y = X_{n+1} (old) and Z = X_{n-1} (new).  With
// DIAG, S holds the diagonal of sz and its products are O(1) per element.
template <typename T2, bool HY, bool HZ, bool DIAG, int NC>
__device__ __forceinline__ void task_products(int n_rt, int r0, int r1, int c, const T2* Am, const T2* S,
                                              const T2* X, const T2* Y, const T2* Z, T2 (&acc)[2][6]) {
  const int N = NC > 0 ? NC : n_rt;  // NC > 0: the dimension is a compile-time constant
#pragma unroll
  for (int e = 0; e < 2; ++e)
#pragma unroll
    for (int q = 0; q < 6; ++q) acc[e][q] = mk<T2>(0.0, 0.0);
  const int R0 = r0 * N, R1 = r1 * N;
  auto kstep = [&](int k) {
    const int kc = k * N + c;
    const T2 xk = X[kc], ak = Am[kc];
    cmac(acc[0][0], Am[R0 + k], xk);
    cmac(acc[1][0], Am[R1 + k], xk);
    cmac(acc[0][1], X[R0 + k], ak);
    cmac(acc[1][1], X[R1 + k], ak);
    if constexpr (!DIAG && (HY || HZ)) {
      const T2 sk = S[kc], s0 = S[R0 + k], s1 = S[R1 + k];
      if constexpr (HY) {
        const T2 yk = Y[kc];
        cmac(acc[0][2], s0, yk);
        cmac(acc[1][2], s1, yk);
        cmac(acc[0][3], Y[R0 + k], sk);
        cmac(acc[1][3], Y[R1 + k], sk);
      }
      if constexpr (HZ) {
        const T2 zk = Z[kc];
        cmac(acc[0][4], s0, zk);
        cmac(acc[1][4], s1, zk);
        cmac(acc[0][5], Z[R0 + k], sk);
        cmac(acc[1][5], Z[R1 + k], sk);
      }
    }
  };
  if constexpr (NC > 0) {
#pragma unroll
    for (int k = 0; k < NC; ++k) kstep(k);
  } else {
#pragma unroll 2
    for (int k = 0; k < N; ++k) kstep(k);
  }
  if constexpr (DIAG && (HY || HZ)) {
    const T2 sc = S[c];
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const int r = e ? r1 : r0;
      const T2 sr = S[r];
      if constexpr (HY) {
        const T2 y = Y[r * N + c];
        acc[e][2] = cmul(sr, y);
        acc[e][3] = cmul(y, sc);
      }
      if constexpr (HZ) {
        const T2 z = Z[r * N + c];
        acc[e][4] = cmul(sr, z);
        acc[e][5] = cmul(z, sc);
      }
    }
  }
}

// f = Am X - X Am - sz Y + Y sz - ng X + cr (sz Z - Z sz) + i ci (sz Z + Z sz)
// at (r0, c) and (r1, c).
template <typename T2, bool DIAG, int NC>
__device__ __forceinline__ void task_rhs(bool hy, bool hz, int N, int r0, int r1, int c, const T2* Am, const T2* S,
                                         const T2* X, const T2* Y, const T2* Z, decltype(T2{}.x) ng,
                                         decltype(T2{}.x) cr, decltype(T2{}.x) ci, T2& f0, T2& f1) {
  using T = decltype(T2{}.x);
  T2 acc[2][6];
  if (hy) {
    if (hz) task_products<T2, true, true, DIAG, NC>(N, r0, r1, c, Am, S, X, Y, Z, acc);
    else task_products<T2, true, false, DIAG, NC>(N, r0, r1, c, Am, S, X, Y, Z, acc);
  } else {
    if (hz) task_products<T2, false, true, DIAG, NC>(N, r0, r1, c, Am, S, X, Y, Z, acc);
    else task_products<T2, false, false, DIAG, NC>(N, r0, r1, c, Am, S, X, Y, Z, acc);
  }
  const T tng = ng, tcr = cr, tci = ci;
#pragma unroll
  for (int e = 0; e < 2; ++e) {
    const T2 x = X[(e ? r1 : r0) * N + c];
    const T2* a = acc[e];
    T2 f;
    f.x = a[0].x - a[1].x - a[2].x + a[3].x - tng * x.x + tcr * (a[4].x - a[5].x) - tci * (a[4].y + a[5].y);
    f.y = a[0].y - a[1].y - a[2].y + a[3].y - tng * x.y + tcr * (a[4].y - a[5].y) + tci * (a[4].x + a[5].x);
    if (e) f1 = f;
    else f0 = f;
  }
}

__device__ __forceinline__ int ring(int x, int L) {
  const int m = x % L;
  return m < 0 ? m + L : m;
}

// x + dt f; the FP32 path compensates level 0 (Kahan, in place: each element
// of the compensation belongs to one thread)
template <typename T2>
__device__ __forceinline__ T2 euler_comp(T2 x, T2 f, decltype(T2{}.x) dt, T2* cp) {
  using T = decltype(T2{}.x);
  if constexpr (sizeof(T) == 4) {
    const T2 c = *cp;
    const T yx = dt * f.x - c.x, yy = dt * f.y - c.y;
    const T tx = x.x + yx, ty = x.y + yy;
    *cp = make_float2((tx - x.x) - yx, (ty - x.y) - yy);
    return make_float2(tx, ty);
  } else {
    return make_double2(x.x + f.x * dt, x.y + f.y * dt);
  }
}
template <typename T2>
__device__ __forceinline__ T2 euler_plain(T2 x, T2 f, decltype(T2{}.x) dt) {
  T2 r;
  r.x = x.x + f.x * dt;
  r.y = x.y + f.y * dt;
  return r;
}

// Error-free sum s + e = a + b (Knuth's TwoSum): the FP32 observable reduction
// carries its rounding errors in a second word
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

template <typename T, bool ONCHIP, bool DIAG, int NC>
__global__ void __launch_bounds__(kHThreads, sizeof(T) == 4 ? (DIAG ? 4 : 3) : 2) heom_sweep_kernel(HeomParams p) {
  using T2 = typename Cplx<T>::type;
  constexpr bool KAHAN = sizeof(T) == 4;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double red[2][kHWarps][kHMaxEops][2];
  const int G = p.G;
  const int g = threadIdx.x / G, gt = threadIdx.x - g * G;
  const int b_slot = blockIdx.x * p.gpc + g;
  // G < 32: several systems share a warp (G a power of two) and sync with it
  const bool sub = G < 32;
  if (!sub && b_slot >= p.n_inst) return;  // no CTA-wide barrier below: each group syncs on its own
  // a sub-warp group past the end of the batch repeats the last system with
  // every global write off, so that all lanes keep taking part in the warp syncs
  const bool active = b_slot < p.n_inst;
  const int b = active ? b_slot : p.n_inst - 1;
  const int bid = 1 + g;
  const bool wg = G <= 32;  // a group within one warp syncs with warp primitives
  const unsigned gmask = sub ? (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1))) : 0xffffffffu;
  const int red0 = (G < 32 ? G : 32) >> 1;  // first offset of the in-group shuffle trees
  // NC > 0: every system has dimension NC (compile-time loops and strides)
  const int N = NC > 0 ? NC : p.dims[b], M = N * N, L = p.nado, NS = NC > 0 ? NC * NC : p.NS;
  const int h = (N + 1) >> 1, tasks = N * h;
  // levels (nado slots of NS) and, for FP32, the compensation of level 0
  const size_t lev_elems = (size_t)L * NS + (KAHAN ? NS : 0);
  T2* base = reinterpret_cast<T2*>(smem) + (size_t)g * (2 * NS + (ONCHIP ? lev_elems : 0));
  T2* Am = base;
  T2* S = base + NS;
  T2* lev = ONCHIP ? base + 2 * NS : reinterpret_cast<T2*>(p.ws) + (size_t)b * lev_elems;
  T2* cmp = lev + (size_t)L * NS;  // FP32 only
  const long long vo = p.voff[b];
  for (int i = gt; i < M; i += G) {
    const double2 hv = p.H[vo + i];
    Am[i] = mk<T2>(hv.y, -hv.x);  // -i H
    if (!DIAG) S[i] = mk<T2>(p.sz[vo + i].x, p.sz[vo + i].y);
  }
  if (DIAG)
    for (int r = gt; r < N; r += G) S[r] = mk<T2>(p.sz[vo + r * N + r].x, p.sz[vo + r * N + r].y);
  for (int l = 0; l < L; ++l)
    for (int i = gt; i < M; i += G) {
      const double2 v = l == 0 ? p.rho0[vo + i] : make_double2(0.0, 0.0);
      lev[(size_t)l * NS + i] = mk<T2>(v.x, v.y);
    }
  if constexpr (KAHAN)
    for (int i = gt; i < M; i += G) cmp[i] = mk<T2>(0.0, 0.0);
  if (gt == 0 && active) p.err[b] = 0;
  auto gsync = [&]() {
    if (wg) __syncwarp();
    else hbar(bid, G);
  };
  auto gsync_or = [&](bool pred) -> bool {
    if (wg) {
      __syncwarp();  // orders the level's shared-memory writes for the other lanes
      return __any_sync(gmask, pred) != 0;
    }
    return hbar_or(bid, G, pred);
  };
  gsync();
  // level coefficients in the working precision (no FP64 arithmetic in the
  // FP32 sweep: GB300's FP64 pipe is narrow)
  const T tg = (T)p.bath[3 * b], tr = (T)p.bath[3 * b + 1], ti = (T)p.bath[3 * b + 2];
  const T dt = (T)p.dt;
  const int E = p.n_eops;
  const T2* Ot = reinterpret_cast<const T2*>(KAHAN ? (const void*)p.OtF : (const void*)p.Ot) + (long long)E * vo;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w0 = (g * G) >> 5, nw = G >> 5;
  // FP32 one-warp groups: widen the staged observables of steps [0, nsteps)
  auto flush_obs = [&](int nsteps) {
    if constexpr (KAHAN) {
      if (wg && p.obs_out != nullptr) {
        __syncwarp();
        for (int e = 0; e < E && active; ++e) {
          double2* row = p.obs_out + ((long long)b * E + e) * p.nt;
          for (int st = gt; st < nsteps; st += G) {
            const float4 v = *reinterpret_cast<const float4*>(row + st);
            row[st] = make_double2((double)v.x + (double)v.y, (double)v.z + (double)v.w);
          }
        }
      }
    }
  };
  // this thread's (row pair, column) task when every task fits the group (N <= 22)
  const bool one = tasks <= G;
  const int rp1 = gt / N, c1 = gt - rp1 * N;
  int kk = 0;  // step mod L
  for (int step = 0; step < p.nt; ++step) {
    if (p.double_first) {
      // the propagator form advances level 0 once more before the sweep: into
      // the spare slot, then copied back (each thread copies its own elements)
      const int s0 = ring(-kk, L), sp = ring(-kk - 1, L);
      T2* X = lev + (size_t)s0 * NS;
      T2* Xs = lev + (size_t)sp * NS;
      const T2* Y = L > 2 ? lev + (size_t)ring(1 - kk, L) * NS : nullptr;
      for (int t = gt; t < tasks; t += G) {
        const int rp = t / N, c = t - rp * N, r1 = rp + h;
        const bool two = r1 < N;
        T2 f0, f1;
        task_rhs<T2, DIAG, NC>(Y != nullptr, false, N, rp, two ? r1 : rp, c, Am, S, X, Y, nullptr, (T)0, (T)0, (T)0,
                           f0, f1);
        const int i0 = rp * N + c, i1 = r1 * N + c;
        Xs[i0] = euler_comp(X[i0], f0, dt, cmp + i0);
        if (two) Xs[i1] = euler_comp(X[i1], f1, dt, cmp + i1);
      }
      gsync();
      for (int t = gt; t < tasks; t += G) {
        const int rp = t / N, c = t - rp * N, r1 = rp + h;
        X[rp * N + c] = Xs[rp * N + c];
        if (r1 < N) X[r1 * N + c] = Xs[r1 * N + c];
      }
      gsync();
    }
    // ring slots of level 0: its own, its new one, level 1's and (unused at n = 0) level -1's
    int so = kk == 0 ? 0 : L - kk;
    int sn = so == 0 ? L - 1 : so - 1;
    int sy = so + 1 == L ? 0 : so + 1;
    int sz2 = sn == 0 ? L - 1 : sn - 1;
    for (int n = 0; n <= L - 2; ++n) {
      const T2* X = lev + (size_t)so * NS;
      T2* Xn = lev + (size_t)sn * NS;
      const bool hy = n + 1 <= L - 2;
      const T2* Y = hy ? lev + (size_t)sy * NS : nullptr;
      const bool hz = n > 0;
      const T2* Z = hz ? lev + (size_t)sz2 * NS : nullptr;
      const T tn = (T)n;
      const T ng = tn * tg, cr = tn * tr, ci = tn * ti;
      bool fin = true;
      auto run_task = [&](int rp, int c) {
        const int r1 = rp + h;
        const bool two = r1 < N;
        T2 f0, f1;
        task_rhs<T2, DIAG, NC>(hy, hz, N, rp, two ? r1 : rp, c, Am, S, X, Y, Z, ng, cr, ci, f0, f1);
        const int i0 = rp * N + c, i1 = r1 * N + c;
        if (n == 0) {
          const T2 v0 = euler_comp(X[i0], f0, dt, cmp + i0);
          Xn[i0] = v0;
          fin = fin && cfinite(v0);
          if (two) {
            const T2 v1 = euler_comp(X[i1], f1, dt, cmp + i1);
            Xn[i1] = v1;
            fin = fin && cfinite(v1);
          }
        } else {
          Xn[i0] = euler_plain(X[i0], f0, dt);
          if (two) Xn[i1] = euler_plain(X[i1], f1, dt);
        }
      };
      if (one) {
        if (gt < tasks) run_task(rp1, c1);
      } else {
        for (int t = gt; t < tasks; t += G) run_task(t / N, t - (t / N) * N);
      }
      if (n == 0) {
        // observables of the new X_0 (this thread's own elements, read back)
        for (int e = 0; e < E; ++e) {
          const T2* O = Ot + (long long)e * M;
          double sx, sy;
          if constexpr (KAHAN) {
            float hx = 0.f, hyv = 0.f, lx = 0.f, ly = 0.f;
            for (int t = gt; t < tasks; t += G) {
              const int rp = one ? rp1 : t / N, c = one ? c1 : t - (t / N) * N;
#pragma unroll
              for (int q = 0; q < 2; ++q) {
                const int r = q ? rp + h : rp;
                if (r < N) {
                  const float2 o = O[r * N + c], v = Xn[r * N + c];
                  float s, er;
                  two_sum(hx, fmaf(-o.y, v.y, o.x * v.x), s, er);
                  hx = s;
                  lx += er;
                  two_sum(hyv, fmaf(o.y, v.x, o.x * v.y), s, er);
                  hyv = s;
                  ly += er;
                }
              }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
              if (o > red0) continue;  // shuffles stay inside the group
              float s, er;
              two_sum(hx, __shfl_xor_sync(0xffffffffu, hx, o), s, er);
              lx += __shfl_xor_sync(0xffffffffu, lx, o) + er;
              hx = s;
              two_sum(hyv, __shfl_xor_sync(0xffffffffu, hyv, o), s, er);
              ly += __shfl_xor_sync(0xffffffffu, ly, o) + er;
              hyv = s;
            }
            if (wg) {
              // staged as (hi, lo, hi, lo) in the 16-byte output slot and
              // widened to FP64 by whole warps after the run (flush_obs)
              if (gt == 0 && active && p.obs_out != nullptr)
                *reinterpret_cast<float4*>(p.obs_out + ((long long)b * E + e) * p.nt + step) =
                    make_float4(hx, lx, hyv, ly);
              continue;
            }
            sx = lane == 0 ? (double)hx + (double)lx : 0.0;
            sy = lane == 0 ? (double)hyv + (double)ly : 0.0;
          } else {
            sx = 0.0;
            sy = 0.0;
            for (int t = gt; t < tasks; t += G) {
              const int rp = one ? rp1 : t / N, c = one ? c1 : t - (t / N) * N;
#pragma unroll
              for (int q = 0; q < 2; ++q) {
                const int r = q ? rp + h : rp;
                if (r < N) {
                  const double2 o = to_d2(O[r * N + c]), v = to_d2(Xn[r * N + c]);
                  sx += o.x * v.x - o.y * v.y;
                  sy += o.x * v.y + o.y * v.x;
                }
              }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
              if (o > red0) continue;
              sx += __shfl_xor_sync(0xffffffffu, sx, o);
              sy += __shfl_xor_sync(0xffffffffu, sy, o);
            }
          }
          if (wg) {
            if (gt == 0 && active && p.obs_out != nullptr)
              p.obs_out[((long long)b * E + e) * p.nt + step] = make_double2(sx, sy);
          } else if (lane == 0) {
            red[step & 1][warp][e][0] = sx;
            red[step & 1][warp][e][1] = sy;
          }
        }
        const bool bad = gsync_or(!fin);
        if (!wg && gt < E && p.obs_out != nullptr) {
          double sx = 0.0, sy = 0.0;
          for (int w = 0; w < nw; ++w) {
            sx += red[step & 1][w0 + w][gt][0];
            sy += red[step & 1][w0 + w][gt][1];
          }
          p.obs_out[((long long)b * E + gt) * p.nt + step] = make_double2(sx, sy);
        }
        if (bad) {
          if (gt == 0 && active) p.err[b] = 4;  // LGB_ERR_NONFINITE
          if (!sub) {
            flush_obs(step + 1);
            return;
          }
          // a sub-warp group runs on with its warp; the error flag stands
        }
      } else {
        gsync();
      }
      so = so + 1 == L ? 0 : so + 1;
      sn = sn + 1 == L ? 0 : sn + 1;
      sy = sy + 1 == L ? 0 : sy + 1;
      sz2 = sz2 + 1 == L ? 0 : sz2 + 1;
    }
    kk = kk + 1 == L ? 0 : kk + 1;
  }
  flush_obs(p.nt);
  // outputs: level n sits in slot (n - nt) mod L
  if (!active) return;
  for (int l = 0; l < L; ++l) {
    const T2* X = lev + (size_t)ring(l - kk, L) * NS;
    for (int i = gt; i < M; i += G) {
      const double2 v = l < L - 1 ? to_d2(X[i]) : make_double2(0.0, 0.0);
      if (l == 0 && p.rho_out != nullptr) p.rho_out[vo + i] = v;
      if (p.ado_out != nullptr) p.ado_out[(long long)L * vo + (long long)l * M + i] = v;
    }
  }
}

template <typename T>
__global__ void heom_convert_kernel(const double2* src, typename Cplx<T>::type* dst, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[i] = mk<typename Cplx<T>::type>(src[i].x, src[i].y);
}

}  // namespace
}  // namespace lgb

// ---- C ABI -----------------------------------------------------------------------
struct lgb_heom_plan {
  lgb_heom_problem_t prob{};
  std::vector<int> dims;
  std::vector<long long> voff;
  long long tot_v = 0;
  int G = 32, gpc = 1, NS = 1;
  int nconst = 0;  // the common dimension when it has a compiled sweep, else 0
  bool on_chip = true;
  size_t smem = 0;
  int* d_dims = nullptr;
  long long* d_voff = nullptr;
  double* d_bath = nullptr;
  double2* d_H = nullptr;
  double2* d_sz = nullptr;
  double2* d_Ot = nullptr;
  float2* d_OtF = nullptr;
  void* d_ws = nullptr;
  int* d_err = nullptr;
  bool ready = false;
};

namespace {

void heom_free(lgb_heom_plan* pl) {
  cudaFree(pl->d_dims);
  cudaFree(pl->d_voff);
  cudaFree(pl->d_bath);
  cudaFree(pl->d_H);
  cudaFree(pl->d_sz);
  cudaFree(pl->d_Ot);
  cudaFree(pl->d_OtF);
  cudaFree(pl->d_ws);
  cudaFree(pl->d_err);
}

// the FP32 on-chip sweep with the dimension fixed at compile time (2, 4, 8,
// 16) when every system of the batch has it, else the general kernel
template <bool DIAG, typename F>
cudaError_t heom_launch_fp32(int nconst, F&& launch) {
  switch (nconst) {
    case 2: return launch(lgb::heom_sweep_kernel<float, true, DIAG, 2>);
    case 4: return launch(lgb::heom_sweep_kernel<float, true, DIAG, 4>);
    case 8: return launch(lgb::heom_sweep_kernel<float, true, DIAG, 8>);
    case 16: return launch(lgb::heom_sweep_kernel<float, true, DIAG, 16>);
    default: return launch(lgb::heom_sweep_kernel<float, true, DIAG, 0>);
  }
}

template <typename V>
bool heom_upload(V** d, const std::vector<V>& h) {
  if (cudaMalloc(d, std::max<size_t>(1, h.size()) * sizeof(V)) != cudaSuccess) return false;
  return cudaMemcpy(*d, h.data(), h.size() * sizeof(V), cudaMemcpyHostToDevice) == cudaSuccess;
}

// bytes of one system's levels: nado slots of NS elements, plus the level-0
// compensation of the FP32 path
size_t heom_level_bytes(int NS, int nado, int precision) {
  return precision == LGB_PREC_FP64 ? (size_t)nado * NS * 16 : ((size_t)nado + 1) * NS * 8;
}

// shared-memory bytes of one system's region
size_t heom_group_bytes(int NS, int nado, int precision, bool on_chip) {
  const size_t esz = precision == LGB_PREC_FP64 ? 16 : 8;
  return 2 * (size_t)NS * esz + (on_chip ? heom_level_bytes(NS, nado, precision) : 0);
}

}  // namespace

extern "C" {

int lgb_heom_max_dim(int32_t precision) {
  (void)precision;
  return lgb::kHMaxDim;
}

int lgb_heom_max_levels_on_chip(int32_t n, int32_t precision) {
  if (n < 1 || n > lgb::kHMaxDim) return 0;
  const size_t fixed = heom_group_bytes(n * n, 0, precision, true);
  if (fixed >= lgb::kHSmemBudget) return 0;
  const size_t per_level = precision == LGB_PREC_FP64 ? (size_t)n * n * 16 : (size_t)n * n * 8;
  return (int)((lgb::kHSmemBudget - fixed) / per_level);
}

int lgb_heom_create(lgb_heom_t* plan, const lgb_heom_problem_t* prob, const int32_t* dims) {
  if (plan == nullptr || prob == nullptr || dims == nullptr) return LGB_ERR_INVALID_ARG;
  *plan = nullptr;
  const lgb_heom_problem_t& pr = *prob;
  if (pr.n_inst < 1 || pr.n_eops < 0 || pr.n_eops > lgb::kHMaxEops || pr.nt < 0 || pr.nado < 2 ||
      (pr.flags & ~(LGB_HEOM_DOUBLE_FIRST | LGB_HEOM_DIAG_SZ)) != 0 || !(pr.dt == pr.dt))
    return LGB_ERR_INVALID_ARG;
  if (pr.precision != LGB_PREC_FP64 && pr.precision != LGB_PREC_FP32) return LGB_ERR_UNSUPPORTED;
  auto* pl = new lgb_heom_plan();
  pl->prob = pr;
  int nmax = 1;
  for (int b = 0; b < pr.n_inst; ++b) {
    const int N = dims[b];
    if (N < 1 || N > lgb::kHMaxDim) {
      delete pl;
      return N < 1 ? LGB_ERR_INVALID_ARG : LGB_ERR_UNSUPPORTED;
    }
    nmax = std::max(nmax, N);
    pl->dims.push_back(N);
    pl->voff.push_back(pl->tot_v);
    pl->tot_v += (long long)N * N;
  }
  pl->NS = nmax * nmax;
  const bool uniform = std::all_of(pl->dims.begin(), pl->dims.end(), [&](int d) { return d == nmax; });
  if (uniform && (nmax == 2 || nmax == 4 || nmax == 8 || nmax == 16)) pl->nconst = nmax;
  // one thread per (column, row pair) task; a batch of one small dimension
  // (at most 16 tasks) packs 32 / G systems into each warp
  const int tasks = nmax * ((nmax + 1) / 2);
  pl->G = std::min(lgb::kHThreads, std::max(32, (tasks + 31) / 32 * 32));
  size_t per = heom_group_bytes(pl->NS, pr.nado, pr.precision, true);
  if (per > lgb::kHSmemBudget) {
    pl->on_chip = false;
    per = heom_group_bytes(pl->NS, pr.nado, pr.precision, false);
  }
  pl->gpc = std::max(1, std::min<int>(lgb::kHThreads / pl->G, (int)(lgb::kHSmemBudget / per)));
  if (uniform && tasks <= 16 && pl->on_chip) {
    int g = 1;
    while (g < tasks) g <<= 1;
    const int per_warp = 32 / g;
    int gpc = std::min<int>(lgb::kHThreads / g, (int)(lgb::kHSmemBudget / per)) / per_warp * per_warp;
    // no more whole warps than the batch fills
    gpc = std::min(gpc, (pr.n_inst + per_warp - 1) / per_warp * per_warp);
    if (gpc >= per_warp) {
      pl->G = g;
      pl->gpc = gpc;
    }
  }
  pl->smem = per * pl->gpc;
  bool ok = heom_upload(&pl->d_dims, pl->dims) && heom_upload(&pl->d_voff, pl->voff) &&
            cudaMalloc(&pl->d_bath, 3 * sizeof(double) * pr.n_inst) == cudaSuccess &&
            cudaMalloc(&pl->d_H, std::max<long long>(1, pl->tot_v) * sizeof(double2)) == cudaSuccess &&
            cudaMalloc(&pl->d_sz, std::max<long long>(1, pl->tot_v) * sizeof(double2)) == cudaSuccess &&
            cudaMalloc(&pl->d_Ot, std::max<long long>(1, (long long)pr.n_eops * pl->tot_v) * sizeof(double2)) ==
                cudaSuccess &&
            cudaMalloc(&pl->d_OtF, std::max<long long>(1, (long long)pr.n_eops * pl->tot_v) * sizeof(float2)) ==
                cudaSuccess &&
            cudaMalloc(&pl->d_err, pr.n_inst * sizeof(int)) == cudaSuccess &&
            cudaMemset(pl->d_err, 0, pr.n_inst * sizeof(int)) == cudaSuccess;
  if (ok && !pl->on_chip)
    ok = cudaMalloc(&pl->d_ws, (size_t)pr.n_inst * heom_level_bytes(pl->NS, pr.nado, pr.precision)) ==
         cudaSuccess;
  if (!ok) {
    heom_free(pl);
    delete pl;
    return LGB_ERR_CUDA;
  }
  *plan = pl;
  return LGB_OK;
}

int lgb_heom_destroy(lgb_heom_t plan) {
  if (plan == nullptr) return LGB_ERR_INVALID_ARG;
  cudaDeviceSynchronize();
  heom_free(plan);
  delete plan;
  return LGB_OK;
}

int lgb_heom_layout(lgb_heom_t plan, int32_t* info) {
  if (plan == nullptr || info == nullptr) return LGB_ERR_INVALID_ARG;
  info[0] = plan->G;
  info[1] = plan->gpc;
  info[2] = plan->on_chip ? 1 : 0;
  info[3] = (int32_t)plan->smem;
  return LGB_OK;
}

int lgb_heom_set(lgb_heom_t plan, const double* H, const double* sz, const double* bath, const double* eops,
                 void* stream) {
  if (plan == nullptr || H == nullptr || sz == nullptr || bath == nullptr ||
      (plan->prob.n_eops > 0 && eops == nullptr))
    return LGB_ERR_INVALID_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const size_t v = (size_t)plan->tot_v * sizeof(double2);
  if (cudaMemcpyAsync(plan->d_H, H, v, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(plan->d_sz, sz, v, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(plan->d_bath, bath, 3 * sizeof(double) * plan->prob.n_inst, cudaMemcpyDeviceToDevice,
                      st) != cudaSuccess)
    return LGB_ERR_CUDA;
  if (plan->prob.n_eops > 0) {
    if (cudaMemcpyAsync(plan->d_Ot, eops, (size_t)plan->prob.n_eops * v, cudaMemcpyDeviceToDevice, st) !=
        cudaSuccess)
      return LGB_ERR_CUDA;
    const long long n = (long long)plan->prob.n_eops * plan->tot_v;
    lgb::heom_convert_kernel<float><<<(int)std::min<long long>((n + 255) / 256, 4096), 256, 0, st>>>(
        plan->d_Ot, plan->d_OtF, n);
    if (cudaGetLastError() != cudaSuccess) return LGB_ERR_CUDA;
  }
  plan->ready = true;
  return LGB_OK;
}

int lgb_heom_propagate(lgb_heom_t plan, const double* rho0, double* obs_out, double* rho_out, double* ado_out,
                       void* stream) {
  if (plan == nullptr || rho0 == nullptr) return LGB_ERR_INVALID_ARG;
  if (!plan->ready) return LGB_ERR_STATE;
  const lgb_heom_problem_t& pr = plan->prob;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  lgb::HeomParams p{};
  p.n_inst = pr.n_inst;
  p.n_eops = pr.n_eops;
  p.nt = pr.nt;
  p.nado = pr.nado;
  p.double_first = (pr.flags & LGB_HEOM_DOUBLE_FIRST) ? 1 : 0;
  p.G = plan->G;
  p.gpc = plan->gpc;
  p.NS = plan->NS;
  p.dt = pr.dt;
  p.dims = plan->d_dims;
  p.voff = plan->d_voff;
  p.bath = plan->d_bath;
  p.H = plan->d_H;
  p.sz = plan->d_sz;
  p.Ot = plan->d_Ot;
  p.OtF = plan->d_OtF;
  p.rho0 = reinterpret_cast<const double2*>(rho0);
  p.obs_out = reinterpret_cast<double2*>(obs_out);
  p.rho_out = reinterpret_cast<double2*>(rho_out);
  p.ado_out = reinterpret_cast<double2*>(ado_out);
  p.ws = plan->d_ws;
  p.err = plan->d_err;
  const int grid = (pr.n_inst + plan->gpc - 1) / plan->gpc;
  const int block = plan->gpc * plan->G;
  const int smem = (int)plan->smem;
  cudaError_t e;
  auto launch = [&](auto kern) {
    cudaError_t r = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (r == cudaSuccess) kern<<<grid, block, smem, st>>>(p);
    return r;
  };
  const bool diag = (pr.flags & LGB_HEOM_DIAG_SZ) != 0;
  if (pr.precision == LGB_PREC_FP64) {
    if (diag)
      e = plan->on_chip ? launch(lgb::heom_sweep_kernel<double, true, true, 0>)
                        : launch(lgb::heom_sweep_kernel<double, false, true, 0>);
    else
      e = plan->on_chip ? launch(lgb::heom_sweep_kernel<double, true, false, 0>)
                        : launch(lgb::heom_sweep_kernel<double, false, false, 0>);
  } else if (!plan->on_chip) {
    e = diag ? launch(lgb::heom_sweep_kernel<float, false, true, 0>)
             : launch(lgb::heom_sweep_kernel<float, false, false, 0>);
  } else if (diag) {
    e = heom_launch_fp32<true>(plan->nconst, launch);
  } else {
    e = heom_launch_fp32<false>(plan->nconst, launch);
  }
  if (e != cudaSuccess) return LGB_ERR_CUDA;
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

int lgb_heom_errors(lgb_heom_t plan, int32_t* flags_host) {
  if (plan == nullptr || flags_host == nullptr) return LGB_ERR_INVALID_ARG;
  const cudaError_t e =
      cudaMemcpy(flags_host, plan->d_err, plan->prob.n_inst * sizeof(int), cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

}  // extern "C"
