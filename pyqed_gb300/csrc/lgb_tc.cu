// CTA-resident batched RK4 propagator on the 5th-generation tensor cores
// (tcgen05, accumulators in tensor memory), split precision 3xTF32 or 3xBF16.
//
// One persistent CTA per SM pulls instances (N <= 64) from a work queue and
// keeps each one resident for all Nt steps.  The complex products of the
// rewritten RHS (pyqed/oqs.py:697-715)
//     R = A X + X A^dag + D o X,     A = -i H_eff,
// are real-embedded into one 128 x NP FP32 accumulator D in TMEM whose lanes
// 0..63 hold Re R and lanes 64..127 hold Im R (rows i):
//   group 1 (A X):     D += [[Ar, -Ai], [Ai, Ar]] . [Xr ; Xi]      (K = 2 NP)
//   group 2 (X A^dag): D += [[Xr,  Xi], [Xi, -Xr]] . [Ar | Ai]^T    (K = 2 NP)
// Both 128-row operands are 128-row windows of 192-row shared-memory stacks
//   SA = [-Ai ; Ar ; Ai]   (windows: rows 64..191 for k < NP, rows 0..127 for k >= NP)
//   SX = [ Xr ; Xi ; -Xr]  (windows: rows 0..127 for k < NP, rows 64..191 for k >= NP)
// and the N-side operands are views of the same stacks: [Xr ; Xi] as an
// MN-major view of SX blocks 0/1, [Ar | Ai] as K-major views of SA blocks 1/2.
// Every product runs three times on the split operands (hi*hi + hi*lo +
// lo*hi, correction terms first) with FP32 accumulation; the 64-bit
// algorithmic count is 64 N^3 real flops per instance-step.
//
// Each of the 512 threads owns a quarter of one TMEM lane's columns (a lane
// is one component of one row); it keeps rho, the RK4 sum, a Kahan compensation term
// and the stage input in registers, performs the RK4 stage combination
// (pyqed/phys.py:1051-1064) with a Kahan-compensated final update, splits the
// next stage input into hi/lo and writes it into SX.  Observables Tr[O rho]
// are reduced in FP64 after every step.  Every mbarrier wait is bounded; a
// wait that runs out marks the instance LGB_ERR_TIMEOUT and the CTA stops.
#include <cuda_bf16.h>

#include "lgb_common.cuh"
#include "lgb_internal.h"
#include "lgb_umma.cuh"

namespace lgb {

namespace {

using namespace umma;

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxEops = 16;

// TF32 or BF16 operand element
template <bool BF16> struct Elem;
template <> struct Elem<false> {
  using T = float;
  static constexpr int kSize = 4;
  static constexpr uint32_t kFmt = kFmtTF32;
  static constexpr int kK = 8;  // K per MMA instruction
  __device__ static void split(float x, float& hi, float& lo) {
    hi = to_tf32(x);
    lo = to_tf32(x - hi);
  }
};
template <> struct Elem<true> {
  using T = __nv_bfloat16;
  static constexpr int kSize = 2;
  static constexpr uint32_t kFmt = kFmtBF16;
  static constexpr int kK = 16;
  __device__ static void split(float x, float& hi, float& lo) {
    hi = __bfloat162float(__float2bfloat16_rn(x));
    lo = __bfloat162float(__float2bfloat16_rn(x - hi));
  }
};

// Byte offset of element (r, c) in a core-matrix tiled operand (see lgb_umma.cuh).
template <bool BF16>
__device__ __forceinline__ uint32_t toff(int r, int c, uint32_t sbo) {
  constexpr int EPC = 16 / Elem<BF16>::kSize;
  return (uint32_t)(r >> 3) * sbo + (uint32_t)(c / EPC) * 128u + (uint32_t)(r & 7) * 16u +
         (uint32_t)(c % EPC) * Elem<BF16>::kSize;
}


struct TcShared {
  uint64_t mbar;
  uint32_t tmem_base;
  int next;
  int flag[kWarps];
  double2 red[kWarps][kMaxEops];
};

// Shared-memory geometry of one instance (NP = padded dimension).
//   stacks SA, SX: 192 rows x NP columns, core matrices adjacent along K
//   (LBO 128 B), row groups SBO_S apart;
//   SXT (X^T, the N-side operand of A X): 2 NP rows x NP columns with the
//   K-direction core matrices 144 B apart, so that the column-wise scalar
//   stores of the epilogue hit 32 distinct banks.
template <bool BF16, int NP>
struct Geo {
  static constexpr int EPC = 16 / Elem<BF16>::kSize;      // elements per 16 bytes
  static constexpr uint32_t LBO_S = 128;
  static constexpr uint32_t SBO_S = (NP / EPC) * 128;
  static constexpr uint32_t STACK = 24 * SBO_S;           // 192 rows
  static constexpr uint32_t LBO_T = 144;
  static constexpr uint32_t SBO_T = (NP / EPC) * 144;
  static constexpr uint32_t XT = (2 * NP / 8) * SBO_T;    // 2 NP rows
  static constexpr int KS = NP / Elem<BF16>::kK;          // MMA K-steps per chunk
  static constexpr uint32_t KSTEP_S = (Elem<BF16>::kK / EPC) * LBO_S;
  static constexpr uint32_t KSTEP_T = (Elem<BF16>::kK / EPC) * LBO_T;
  // TF32 keeps one level of X resident (two MMA phases per stage); BF16 both.
  static constexpr int XLEVELS = BF16 ? 2 : 1;
  static constexpr uint32_t BYTES = 2 * STACK + XLEVELS * (STACK + XT);
};
// exchange buffer for a complex diagonal dissipator: [2][64][64] floats
constexpr uint32_t kXchgBytes = 2 * 64 * 64 * 4;

template <bool BF16>
__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
  if constexpr (BF16) {
    mma_f16(d, a, b, id, acc);
  } else {
    mma_tf32(d, a, b, id, acc);
  }
}

// Descriptor arithmetic: the start address is the low 14-bit field (in 16-byte
// units); shared-memory offsets below 256 KB never carry out of it, so a
// descriptor for base + off is the base descriptor + (off >> 4).
__device__ __forceinline__ uint64_t dadd(uint64_t d, uint32_t off) { return d + (off >> 4); }

// D (+)= Ahat . [Xr ; Xi]  with Ahat = SA windows (level a) and X^T from SXT.
template <bool BF16, int NP>
__device__ __forceinline__ void group_ax(uint32_t d, uint32_t sa, uint32_t sxt, uint32_t& acc) {
  using G = Geo<BF16, NP>;
  constexpr uint32_t id = idesc(Elem<BF16>::kFmt, 128, NP, false, false);
  const uint64_t da = sdesc(sa, G::LBO_S, G::SBO_S);
  const uint64_t db = sdesc(sxt, G::LBO_T, G::SBO_T);
  // the K loop is unrolled (descriptors = chunk base + compile-time constant,
  // no dependent address arithmetic between MMAs); the chunk loop is not, to
  // bound register pressure
#pragma unroll 1
  for (int chunk = 0; chunk < 2; ++chunk) {
    const uint32_t a_off = (chunk == 0 ? 8u : 0u) * G::SBO_S;       // [Ar;Ai] or [-Ai;Ar]
    const uint32_t b_off = (uint32_t)chunk * (NP / 8) * G::SBO_T;    // Xr^T or Xi^T
    const uint64_t ca = dadd(da, a_off), cb = dadd(db, b_off);
#pragma unroll
    for (int s = 0; s < G::KS; ++s) {
      mma<BF16>(d, dadd(ca, s * G::KSTEP_S), dadd(cb, s * G::KSTEP_T), id, acc);
      acc = 1;
    }
  }
}

// D (+)= Xhat . [Ar | Ai]^T  with Xhat = SX windows and [Ar | Ai] from SA blocks 1, 2.
template <bool BF16, int NP>
__device__ __forceinline__ void group_xa(uint32_t d, uint32_t sx, uint32_t sa, uint32_t& acc) {
  using G = Geo<BF16, NP>;
  constexpr uint32_t id = idesc(Elem<BF16>::kFmt, 128, NP, false, false);
  const uint64_t da = sdesc(sx, G::LBO_S, G::SBO_S);
  const uint64_t db = sdesc(sa, G::LBO_S, G::SBO_S);
#pragma unroll 1
  for (int chunk = 0; chunk < 2; ++chunk) {
    const uint32_t a_off = (chunk == 0 ? 0u : 8u) * G::SBO_S;        // [Xr;Xi] or [Xi;-Xr]
    const uint32_t b_off = (chunk == 0 ? 8u : 16u) * G::SBO_S;       // Ar or Ai block
    const uint64_t ca = dadd(da, a_off), cb = dadd(db, b_off);
#pragma unroll
    for (int s = 0; s < G::KS; ++s) {
      mma<BF16>(d, dadd(ca, s * G::KSTEP_S), dadd(cb, s * G::KSTEP_S), id, acc);
      acc = 1;
    }
  }
}

__device__ __forceinline__ void sync_for_mma() {
  fence_async_smem();
  fence_before_sync();
  __syncthreads();
}

// Store 4 consecutive columns of one operand row (16 bytes TF32, 8 bytes BF16).
template <bool BF16>
__device__ __forceinline__ void st4(unsigned char* base, const float* v) {
  if constexpr (!BF16) {
    *reinterpret_cast<float4*>(base) = make_float4(v[0], v[1], v[2], v[3]);
  } else {
    __nv_bfloat162 p0 = __floats2bfloat162_rn(v[0], v[1]);
    __nv_bfloat162 p1 = __floats2bfloat162_rn(v[2], v[3]);
    uint2 u;
    u.x = *reinterpret_cast<uint32_t*>(&p0);
    u.y = *reinterpret_cast<uint32_t*>(&p1);
    *reinterpret_cast<uint2*>(base) = u;
  }
}

template <int W>
__device__ __forceinline__ void tmem_ld_cols(uint32_t taddr, float* v) {
  if constexpr (W == 4) {
    tmem_ld4(taddr, v);
  } else if constexpr (W == 8) {
    tmem_ld8(taddr, v);
  } else if constexpr (W == 12) {
    tmem_ld8(taddr, v);
    tmem_ld4(taddr + 8, v + 8);
  } else {
    tmem_ld16(taddr, v);
  }
}

// One instance, all Nt steps.  Thread mapping: warp w reads TMEM lane quarter
// (w & 3) and owns columns [(w >> 2) NP/4, (w >> 2 + 1) NP/4) of its lane;
// lane l holds component l / 64 (0 real, 1 imaginary) of row l % 64.
template <bool BF16, int NP>
__device__ void tc_instance(const CtaParams& p, const int b, unsigned char* smem, TcShared& sh,
                            uint32_t& phase, bool& alive) {
  using El = Elem<BF16>;
  using G = Geo<BF16, NP>;
  using ET = typename El::T;
  constexpr int EPC = G::EPC;
  constexpr int NPQ = NP / 4;                 // columns per thread
  constexpr int NG = NPQ / 4;                 // groups of 4 columns
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int quarter = warp & 3, cg = warp >> 2;
  const int l = quarter * 32 + lane;  // TMEM lane
  const int comp = l >> 6;            // 0: real part, 1: imaginary part
  const int i = l & 63;               // row
  const int j0 = cg * NPQ;            // first owned column
  const int N = p.dims[b];
  const int NPS = NP + 2;             // row stride of the FP32 working matrices
  const long long wo = p.woff[b];
  const int E = p.n_eops;
  const bool diag = p.cops_kind == 2 && p.n_cops > 0;
  const float half_dt = (float)(0.5 * p.dt), dt = (float)p.dt, sixth_dt = (float)(p.dt / 6.0);

  unsigned char* SAh = smem;
  unsigned char* SAl = SAh + G::STACK;
  unsigned char* SX0 = SAl + G::STACK;        // X level 0 (TF32: the level in flight; BF16: hi)
  unsigned char* SXT0 = SX0 + G::STACK;
  unsigned char* SX1 = SXT0 + G::XT;          // BF16 only: lo
  unsigned char* SXT1 = SX1 + G::STACK;
  float* sXc = reinterpret_cast<float*>(smem + G::BYTES);  // complex-D exchange
  const uint32_t sa_hi = smem_u32(SAh), sa_lo = smem_u32(SAl);
  const uint32_t sx0 = smem_u32(SX0), sxt0 = smem_u32(SXT0);
  const uint32_t sx1 = smem_u32(SX1), sxt1 = smem_u32(SXT1);
  const float2* At0 = reinterpret_cast<const float2*>(p.At) + wo;
  const float2* Gt = reinterpret_cast<const float2*>(p.Gt) + (long long)p.n_drive * wo;
  const float2* Dm = reinterpret_cast<const float2*>(p.Dm) + wo;
  const float2* OtF = p.OtF + (long long)E * wo;
  const uint32_t taddr = sh.tmem_base + ((uint32_t)(quarter * 32) << 16) + (uint32_t)j0;

  // ---- A stack: SA = [-Ai ; Ar ; Ai] (hi / lo), rebuilt per step when driven --
  auto build_sa = [&](const float* f) {
    for (int idx = tid; idx < 64 * NP; idx += kThreads) {
      const int k = idx / 64, r = idx % 64;  // consecutive threads: consecutive rows
      float2 a = make_float2(0.f, 0.f);
      if (r < NP) {
        a = At0[k * NPS + r];  // A[r][k]
        if (f != nullptr) {
#pragma unroll
          for (int d = 0; d < 4; ++d)
            if (d < p.n_drive) {
              const float2 g = Gt[(long long)d * NP * NPS + k * NPS + r];
              a.x = fmaf(f[d], g.x, a.x);
              a.y = fmaf(f[d], g.y, a.y);
            }
        }
      }
      float h, lo;
      El::split(-a.y, h, lo);
      *reinterpret_cast<ET*>(SAh + toff<BF16>(r, k, G::SBO_S)) = (ET)h;
      *reinterpret_cast<ET*>(SAl + toff<BF16>(r, k, G::SBO_S)) = (ET)lo;
      El::split(a.x, h, lo);
      *reinterpret_cast<ET*>(SAh + toff<BF16>(64 + r, k, G::SBO_S)) = (ET)h;
      *reinterpret_cast<ET*>(SAl + toff<BF16>(64 + r, k, G::SBO_S)) = (ET)lo;
      El::split(a.y, h, lo);
      *reinterpret_cast<ET*>(SAh + toff<BF16>(128 + r, k, G::SBO_S)) = (ET)h;
      *reinterpret_cast<ET*>(SAl + toff<BF16>(128 + r, k, G::SBO_S)) = (ET)lo;
    }
  };

  // ---- X operands: SX = [Xr ; Xi ; -Xr] rows, SXT = [Xr^T ; Xi^T] -------------
  // level: 0 = hi part, 1 = lo part of the split of x.
  const int xrow = comp == 0 ? i : 64 + i;
  auto write_x = [&](const float* x, int level, unsigned char* SX, unsigned char* SXT) {
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      float v[4], nv[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        float h, lo;
        El::split(x[g * 4 + e], h, lo);
        v[e] = level == 0 ? h : lo;
        nv[e] = -v[e];
      }
      const int c = j0 + g * 4;
      st4<BF16>(SX + toff<BF16>(xrow, c, G::SBO_S), v);
      if (comp == 0) st4<BF16>(SX + toff<BF16>(128 + i, c, G::SBO_S), nv);
      if (i < NP) {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int rt = comp * NP + c + e;  // row of X^T (= column of X)
          const uint32_t o = (uint32_t)(rt >> 3) * G::SBO_T + (uint32_t)(i / EPC) * G::LBO_T +
                             (uint32_t)(rt & 7) * 16u + (uint32_t)(i % EPC) * El::kSize;
          *reinterpret_cast<ET*>(SXT + o) = (ET)v[e];
        }
      }
    }
  };

  // ---- observables Tr[O rho]: FP32 partials per thread and warp (pairwise
  // shuffle tree), FP64 across warps.  A per-thread mask skips the zero
  // entries of O (sparse observables such as a transition dipole).
  uint32_t omask = 0;  // bit e*NPQ+jj (E * NPQ <= 32 bits used)
  const bool use_mask = E * NPQ <= 32;
  if (use_mask && i < N) {
    for (int e = 0; e < E; ++e) {
      const float2* o = OtF + (long long)e * NP * NPS + (long long)i * NPS + j0;
#pragma unroll
      for (int jj = 0; jj < NPQ; ++jj) {
        const float2 ov = o[jj];
        if (ov.x != 0.f || ov.y != 0.f) omask |= 1u << (e * NPQ + jj);
      }
    }
  }
  auto reduce_state = [&](const float* rho, int row) -> bool {
    bool fin = true;
#pragma unroll
    for (int jj = 0; jj < NPQ; ++jj) fin = fin && isfinite(rho[jj]);
    for (int e = 0; e < E; ++e) {
      float fx = 0.f, fy = 0.f;
      const uint32_t m = use_mask ? (omask >> (e * NPQ)) : 0xffffffffu;
      if (i < N && (m & ((NPQ >= 32) ? 0xffffffffu : ((1u << NPQ) - 1u))) != 0u) {
        const float2* o = OtF + (long long)e * NP * NPS + (long long)i * NPS + j0;
#pragma unroll
        for (int jj = 0; jj < NPQ; ++jj) {
          if (!(m & (1u << jj))) continue;
          const float2 ov = o[jj];  // O[j][i]
          if (comp == 0) {
            fx = fmaf(ov.x, rho[jj], fx);
            fy = fmaf(ov.y, rho[jj], fy);
          } else {
            fx = fmaf(-ov.y, rho[jj], fx);
            fy = fmaf(ov.x, rho[jj], fy);
          }
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        fx += __shfl_xor_sync(0xffffffffu, fx, o);
        fy += __shfl_xor_sync(0xffffffffu, fy, o);
      }
      if (lane == 0) sh.red[warp][e] = make_double2((double)fx, (double)fy);
    }
    const unsigned bad = __ballot_sync(0xffffffffu, !fin);
    if (lane == 0) sh.flag[warp] = bad != 0u;
    __syncthreads();
    bool anybad = false;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) anybad = anybad || sh.flag[w];
    if (tid < E && p.obs_out != nullptr) {
      double2 sacc = make_double2(0.0, 0.0);
#pragma unroll
      for (int w = 0; w < kWarps; ++w) {
        sacc.x += sh.red[w][tid].x;
        sacc.y += sh.red[w][tid].y;
      }
      const long long nrows = (long long)p.nt + p.obs_t0;
      p.obs_out[((long long)b * nrows + row) * E + tid] = sacc;
    }
    return anybad;
  };

  // Bounded wait for the last commit; on time-out mark the instance and stop.
  auto wait_mma = [&]() -> bool {
    const bool ok = mbar_wait(&sh.mbar, phase, kSpinLimit);
    phase ^= 1u;
    if (__syncthreads_or(!ok)) {
      if (tid == 0) p.err[b] = 5;  // LGB_ERR_TIMEOUT
      mbar_wait(&sh.mbar, phase ^ 1u, kSpinLimit);
      alive = false;
      return false;
    }
    return true;
  };

  // ---- state -------------------------------------------------------------------
  float rho[NPQ], racc[NPQ], kc[NPQ], xin[NPQ];
  {
    const double2* r0 = p.rho0 + p.off[b];
#pragma unroll
    for (int jj = 0; jj < NPQ; ++jj) {
      const int j = j0 + jj;
      double v = 0.0;
      if (i < N && j < N) {
        const double2 z = r0[(long long)i * N + j];
        v = comp == 0 ? z.x : z.y;
      }
      rho[jj] = (float)v;
      xin[jj] = rho[jj];
      racc[jj] = 0.f;
      kc[jj] = 0.f;
    }
  }

  // Dissipator D o X of diagonal collapse operators.  Pure-dephasing type
  // (D diagonal and real) keeps D_ii in a register; a general D is read from
  // the working copy; a complex D couples the real and imaginary lanes, which
  // then exchange the stage input through shared memory.
  bool off = false, dc = false;
  if (diag && i < N) {
#pragma unroll
    for (int jj = 0; jj < NPQ; ++jj) {
      const float2 d = Dm[i * NPS + j0 + jj];
      off = off || ((j0 + jj != i) && (d.x != 0.f || d.y != 0.f));
      dc = dc || (d.y != 0.f);
    }
  }
  const bool dgeneral = __syncthreads_or(off) != 0;
  const bool dcomplex = __syncthreads_or(dc) != 0;
  const bool dfast = diag && !dgeneral && !dcomplex;
  const int dpos = (i >= j0 && i < j0 + NPQ) ? i - j0 : -1;
  const float dd = (dfast && dpos >= 0 && i < N) ? Dm[i * NPS + i].x : 0.f;
  auto publish_x = [&]() {
#pragma unroll
    for (int jj = 0; jj < NPQ; ++jj) sXc[(comp * 64 + i) * 64 + j0 + jj] = xin[jj];
  };
  if (dcomplex) publish_x();
  if (p.n_drive == 0) build_sa(nullptr);
  if (tid == 0) p.err[b] = 0;
  if (p.obs_t0) reduce_state(rho, 0);

  const double* drv = p.drive;
  if (p.n_drive > 0 && !p.drive_shared) drv += (long long)b * p.n_drive * p.nt;

  for (int step = 0; step < p.nt && alive; ++step) {
    if (p.n_drive > 0) {
      float f[4];
#pragma unroll
      for (int d = 0; d < 4; ++d) f[d] = (d < p.n_drive) ? (float)drv[(long long)d * p.nt + step] : 0.f;
      build_sa(f);
    }
#pragma unroll 1
    for (int stage = 0; stage < 4; ++stage) {
      if constexpr (!BF16) {
        // phase A: X_lo resident -> Ah Xl + Xl Ah
        write_x(xin, 1, SX0, SXT0);
        sync_for_mma();
        if (tid == 0) {
          fence_after_sync();
          uint32_t acc = 0;
          group_ax<BF16, NP>(sh.tmem_base, sa_hi, sxt0, acc);
          group_xa<BF16, NP>(sh.tmem_base, sx0, sa_hi, acc);
          mma_commit(&sh.mbar);
        }
        if (!wait_mma()) break;
        // phase B: X_hi resident -> Al Xh + Xh Al + Ah Xh + Xh Ah
        write_x(xin, 0, SX0, SXT0);
        sync_for_mma();
        if (tid == 0) {
          fence_after_sync();
          uint32_t acc = 1;
          group_ax<BF16, NP>(sh.tmem_base, sa_lo, sxt0, acc);
          group_xa<BF16, NP>(sh.tmem_base, sx0, sa_lo, acc);
          group_ax<BF16, NP>(sh.tmem_base, sa_hi, sxt0, acc);
          group_xa<BF16, NP>(sh.tmem_base, sx0, sa_hi, acc);
          mma_commit(&sh.mbar);
        }
        if (!wait_mma()) break;
      } else {
        write_x(xin, 0, SX0, SXT0);
        write_x(xin, 1, SX1, SXT1);
        sync_for_mma();
        if (tid == 0) {
          fence_after_sync();
          uint32_t acc = 0;
          group_ax<BF16, NP>(sh.tmem_base, sa_hi, sxt1, acc);
          group_xa<BF16, NP>(sh.tmem_base, sx1, sa_hi, acc);
          group_ax<BF16, NP>(sh.tmem_base, sa_lo, sxt0, acc);
          group_xa<BF16, NP>(sh.tmem_base, sx0, sa_lo, acc);
          group_ax<BF16, NP>(sh.tmem_base, sa_hi, sxt0, acc);
          group_xa<BF16, NP>(sh.tmem_base, sx0, sa_hi, acc);
          mma_commit(&sh.mbar);
        }
        if (!wait_mma()) break;
      }
      fence_after_sync();
      float v[NPQ];
      tmem_ld_cols<NPQ>(taddr, v);
      tmem_wait_ld();
      // RHS element R = v + (D o X); stages 0-2 form the RK4 sum and the next
      // stage input, stage 3 applies the Kahan-compensated update
      auto rhs = [&](int jj) -> float {
        float R = v[jj];
        if (dfast) {
          R = (jj == dpos) ? fmaf(dd, xin[jj], R) : R;
        } else if (diag && i < NP) {
          const float2 d = Dm[i * NPS + j0 + jj];
          R = fmaf(d.x, xin[jj], R);
          if (dcomplex) {
            const float xo = sXc[((1 - comp) * 64 + i) * 64 + j0 + jj];
            R = fmaf(comp == 0 ? -d.y : d.y, xo, R);
          }
        }
        return R;
      };
      if (stage < 3) {
        const float cst = (stage == 2) ? dt : half_dt;
        const float keep = (stage == 0) ? 0.f : 1.f;
        const float w = (stage == 0) ? 1.f : 2.f;
#pragma unroll
        for (int jj = 0; jj < NPQ; ++jj) {
          const float R = rhs(jj);
          racc[jj] = fmaf(w, R, keep * racc[jj]);
          xin[jj] = fmaf(cst, R, rho[jj]);
        }
      } else {
#pragma unroll
        for (int jj = 0; jj < NPQ; ++jj) {
          const float R = rhs(jj);
          // Kahan-compensated rho += dt/6 (k1 + 2 k2 + 2 k3 + k4)
          const float y = fmaf(sixth_dt, racc[jj] + R, -kc[jj]);
          const float t = rho[jj] + y;
          kc[jj] = (t - rho[jj]) - y;
          rho[jj] = t;
          xin[jj] = t;
        }
      }
      if (dcomplex) {
        __syncthreads();  // every partner has read the previous stage input
        publish_x();
      }
    }
    if (!alive) break;
    const bool bad = reduce_state(rho, step + p.obs_t0);
    if (bad) {
      if (tid == 0) p.err[b] = 4;  // LGB_ERR_NONFINITE
      break;
    }
    if (p.store_every > 0 && p.states_out != nullptr && ((step + 1) % p.store_every) == 0 &&
        i < N) {
      const long long si = (step + 1) / p.store_every - 1;
      double2* dst = p.states_out + p.soff[b] + si * (long long)N * N;
#pragma unroll
      for (int jj = 0; jj < NPQ; ++jj) {
        const int j = j0 + jj;
        if (j < N) reinterpret_cast<double*>(dst + (long long)i * N + j)[comp] = (double)rho[jj];
      }
    }
  }

  if (alive && p.rho_out != nullptr && i < N) {
    double2* dst = p.rho_out + p.off[b];
#pragma unroll
    for (int jj = 0; jj < NPQ; ++jj) {
      const int j = j0 + jj;
      if (j < N) reinterpret_cast<double*>(dst + (long long)i * N + j)[comp] = (double)rho[jj];
    }
  }
  // TMEM reads of this instance are done before the next instance's first MMA
  fence_before_sync();
  __syncthreads();
}

template <bool BF16>
__global__ void __launch_bounds__(kThreads, 1) tc_rk4_kernel(CtaParams p, const int* order,
                                                             int n_items, int* queue) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ TcShared sh;
  const int tid = threadIdx.x;
  if (tid == 0) {
    mbar_init(&sh.mbar, 1);
    mbar_fence_init();
  }
  if (tid < 32) {
    tmem_alloc(&sh.tmem_base, 64);
    tmem_relinquish();
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  uint32_t phase = 0;
  bool alive = true;
  while (alive) {
    if (tid == 0) sh.next = atomicAdd(queue, 1);
    __syncthreads();
    const int item = sh.next;
    __syncthreads();
    if (item >= n_items) break;
    const int b = order[item];
    switch (p.npad[b]) {
      case 16: tc_instance<BF16, 16>(p, b, smem, sh, phase, alive); break;
      case 32: tc_instance<BF16, 32>(p, b, smem, sh, phase, alive); break;
      case 48: tc_instance<BF16, 48>(p, b, smem, sh, phase, alive); break;
      default: tc_instance<BF16, 64>(p, b, smem, sh, phase, alive); break;
    }
  }
  fence_before_sync();
  __syncthreads();
  if (tid < 32) tmem_dealloc(sh.tmem_base, 64);
}

}  // namespace

int tc_max_dim() { return 64; }

int tc_smem_core(bool bf16, int npad) {
  switch (npad) {
    case 16: return bf16 ? (int)Geo<true, 16>::BYTES : (int)Geo<false, 16>::BYTES;
    case 32: return bf16 ? (int)Geo<true, 32>::BYTES : (int)Geo<false, 32>::BYTES;
    case 48: return bf16 ? (int)Geo<true, 48>::BYTES : (int)Geo<false, 48>::BYTES;
    default: return bf16 ? (int)Geo<true, 64>::BYTES : (int)Geo<false, 64>::BYTES;
  }
}

int tc_smem_bytes(int precision, int npad) {
  const bool bf16 = precision == LGB_PREC_BF16X3;
  return tc_smem_core(bf16, npad) + (int)kXchgBytes;
}

cudaError_t launch_tc_rk4(const CtaParams& p, int precision, const int* order, int n_items,
                          int* queue, int grid, cudaStream_t stream) {
  if (n_items <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(queue, 0, sizeof(int), stream);
  if (e != cudaSuccess) return e;
  if (precision == LGB_PREC_BF16X3) {
    e = cudaFuncSetAttribute(tc_rk4_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             p.smem_bytes);
    if (e != cudaSuccess) return e;
    tc_rk4_kernel<true><<<grid, kThreads, p.smem_bytes, stream>>>(p, order, n_items, queue);
  } else {
    e = cudaFuncSetAttribute(tc_rk4_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             p.smem_bytes);
    if (e != cudaSuccess) return e;
    tc_rk4_kernel<false><<<grid, kThreads, p.smem_bytes, stream>>>(p, order, n_items, queue);
  }
  return cudaGetLastError();
}

}  // namespace lgb
