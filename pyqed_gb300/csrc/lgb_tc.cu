// CTA-resident batched RK4 propagator on the 5th-generation tensor cores
// (tcgen05, accumulator in tensor memory), split precision 3xTF32 or 3xBF16.
//
// One persistent CTA per SM pulls instances (N <= 64, padded to NP, a multiple
// of 16) from a work queue and keeps each one resident for all Nt steps.  The
// rewritten RHS (pyqed/oqs.py:697-715)
//     R = A X + X A^dag + D o X,     A = -i H_eff,
// is two complex products, each evaluated as a real MMA whose M side carries
// the real and imaginary rows of one complex factor and whose N side carries
// the two parts of the other:
//   M row (c, i) = 32 (i / 16) + 16 c + i % 16        c = 0 real, 1 imaginary
//   N col (p, j) = 32 (j / 16) + 16 (1 - p) + j % 16   (p = 0 at the odd 16-block)
// With P = P0 + i P1 on the M side and Q = Q0 + i Q1 on the N side the
// accumulator holds D[(c,i)][(p,j)] = (P_c Q_p)[i][j], and
//   Re (P Q) = D[(0,i)][(0,j)] - D[(1,i)][(1,j)],  Im (P Q) = D[(1,i)][(0,j)] + D[(0,i)][(1,j)].
// The two lanes of a row i (c = 0, 1) sit 16 apart in one 32-lane TMEM
// quarter, so the combination is one warp shuffle.
//   A X:       P = A  (rows (Ar, Ai) of the A buffer),  Q = X   (X^T buffer: Xr^T, Xi^T)
//   X A^dag:   P = -i X  (rows (Xi, -Xr) of the XM buffer),  Q = i A^dag  (the same A
//              buffer read as the N side: part 0 = Ai, part 1 = Ar)
// so one A buffer serves both products.  Every operand is split into hi + lo
// (TF32 or BF16) and each product keeps the three leading terms, so a stage
// is 6 K-loops of NP/kK instructions at N = 2NP (48 instructions at NP = 64
// for TF32, against 96 at N = NP for the Re/Im-blocked embedding) into one
// accumulator, and one commit.
//
// Each of the 512 threads owns a quarter of the columns of one TMEM lane (one
// component of one row); it keeps rho, the RK4 sum, a Kahan compensation term
// and the stage input in registers, performs the RK4 stage combination
// (pyqed/phys.py:1051-1064) with a Kahan-compensated final update, splits the
// next stage input into hi/lo and writes it into the XM and X^T buffers.
// The diagonal of A stays out of the split products: its entries are of
// order one (the site energies) and a hi + lo split holds them only to
// ~2^-17 (BF16) or ~2^-21 (TF32) relative, which turns into a phase error
// growing with t.  Its term (a_i + conj(a_j)) X_ij is formed in FP32 from the
// FP32 stage input and written into the part-0 accumulator columns (part-1
// columns zeroed) before the stage's MMAs, which accumulate onto it; the
// off-diagonal couplings are small, so their split representation error is
// too.
// Observables Tr[O rho] (pyqed/phys.py:1257-1264) of step k are reduced while
// the tensor core runs the first stage of step k + 1.  Every mbarrier wait is
// bounded; a wait that runs out marks the instance LGB_ERR_TIMEOUT and the CTA
// stops.
#include <cuda_bf16.h>

#include <algorithm>
#include <type_traits>

#include "lgb_common.cuh"
#include "lgb_internal.h"
#include "lgb_umma.cuh"

namespace lgb {

namespace {

using namespace umma;

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxEops = 16;
constexpr uint32_t kTmemCols = 128;  // D: 2 NP <= 128 columns

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

// Two thread groups (the warps of TMEM lane quarters 0-1 and 2-3) run separate
// instances when NP <= 32; otherwise group 0 is the whole CTA.
struct TcShared {
  alignas(16) float2 adg[2][64];  // diagonal of A of each group's instance (applied in FP32)
  uint64_t mbar[2];
  uint32_t tmem_base;
  int next[2];
  float2 red[2][kMaxEops][kWarps];  // per-warp observable partials
  double chk[2][kWarps][3];         // per-warp check partials: Tr rho (re, im), max hermiticity deviation
  double chk_run[2][4];             // check state of each group's instance: Tr rho0 (re, im), max drift, max deviation
  int chk_flags[2];                 // bit 0: rho0 Hermitian (deviation checked), bit 1: tolerance exceeded
};

// N = 65 (static H): the 64 x 64 block runs on the tensor cores as above; the
// border row and column (index g = 64) run on the SIMT pipes while the MMAs
// of the block are in flight.  With c_i = X[i][g], r_j = X[g][j], z = X[g][g],
// a_i = A[i][g], b_j = A[g][j], alpha = A[g][g] and M the 64 x 64 block:
//   block:   R_ij += a_i r_j + c_i conj(a_j)                       (epilogue)
//   column:  R_ig = (A_M c)_i + a_i z + (M conj(b))_i + c_i conj(alpha) + D_ig c_i
//   row:     R_gj = (b^T M)_j + alpha r_j + (conj(A_M) r)_j + z conj(a_j) + D_gj r_j
//   corner:  R_gg = b.c + alpha z + r.conj(b) + z conj(alpha) + D_gg z
// (M conj(b)) is reduced by the epilogue of the previous stage from its
// registers; (b^T M) reads the X^T operand buffer; A_M c and conj(A_M) r read
// A from global memory (L1/L2).  The border's RK4 state sits in shared memory
// after the operand buffers.
constexpr int kBorder = 65;  // border index 64 plus one (the corner is entry 64 of the row arrays)
struct TcBorder {
  float2 bx[2][2][kBorder];   // stage input [buffer][0: column c_i, 1: row r_j and corner]
  float2 rho[2][kBorder], racc[2][kBorder], nkc[2][kBorder];
  float2 aB[kBorder], bB[kBorder];      // A[i][g], A[g][j] (entry 64: alpha)
  float2 dcol[kBorder], drow[kBorder];  // D[i][g], D[g][j]
  float2 t1[64], t3[64], t4[64];        // (A_M c)_i, (b^T M)_j, (conj(A_M) r)_j of the stage
  float2 t3p[2][64];                    // BF16: b^T M_p of the real (p = 0) and imaginary parts
  float2 t2p[2][64][4];                 // (M conj(b))_i partials of the four column groups, per bx buffer
  float2 csum[2];                       // corner sums b.c and r.conj(b)
};

// Shared-memory geometry of one instance.  Core matrices of 8 rows x 16 bytes.
//   "S" layout (A buffer, XM buffer), K-major: the K-direction core matrices
//   of an 8-row group are adjacent (LBO 128 B), row groups SBO_S apart;
//   X^T buffer (the N side of A X), TF32: the K-major "T" layout, K-direction
//   core matrices 144 B apart and row groups SBO_T apart, SBO_T = 32 mod
//   64 B, so that the column-wise scalar stores of a warp (16 rows i of each
//   of two row halves, 2 row groups apart) hit distinct banks;
//   X^T buffer, BF16: MN-major (the instruction descriptor's transpose-B
//   bit), i.e. X's own rows: core matrices of 8 K-rows (i) x 8 N-elements
//   (j), N-direction ones adjacent (SBO 128 B), K-direction ones SK_M apart
//   (LBO).  A thread's four columns of row i are then one 8-byte piece of a
//   core-matrix row (16 bytes for two groups) instead of four scalars.  The
//   descriptor reading (LBO = the K-direction stride for MN-major operands)
//   was checked by an in-bounds probe against a CPU product.
// Each buffer holds the hi level (2 NP rows) followed by the lo level.  An
// M-side operand reads 128 rows from its level base; the rows past 2 NP belong
// to lanes no thread uses and stay inside the buffer (BYTES covers the last
// window).
template <bool BF16, int NP>
struct Geo {
  static constexpr int EPC = 16 / Elem<BF16>::kSize;  // elements per 16 bytes
  static constexpr uint32_t SBO_S = (NP / EPC) * 128;
  static constexpr uint32_t LVL_S = (2 * NP / 8) * SBO_S;
  static constexpr uint32_t LBO_T = 144;
  static constexpr uint32_t SBO_T = (NP / EPC) * 144 + (96u - ((NP / EPC) * 144u) % 64u) % 64u;
  // BF16: the X^T buffer is the MN-major B operand instead: element (n, k)
  // at (n / 8) SN_M + (k / 8) SK_M + (k % 8) 16 + (n % 8) 2, core matrices of
  // 8 K-rows x 8 N-elements, N-direction ones adjacent
  static constexpr uint32_t SN_M = 128;
  static constexpr uint32_t SK_M = (2 * NP / 8) * 128;
  static constexpr uint32_t LVL_T = BF16 ? (NP / 8) * SK_M : (2 * NP / 8) * SBO_T;
  static constexpr int KS = NP / Elem<BF16>::kK;  // MMA K-steps
  static constexpr uint32_t KSTEP_S = (Elem<BF16>::kK / EPC) * 128;
  static constexpr uint32_t KSTEP_T = BF16 ? 2 * SK_M : (Elem<BF16>::kK / EPC) * LBO_T;
  static constexpr uint32_t OFF_A = 0;
  static constexpr uint32_t OFF_XM = 2 * LVL_S;
  static constexpr uint32_t OFF_XT = 4 * LVL_S;
  static constexpr uint32_t END = OFF_XT + 2 * LVL_T;
  static constexpr uint32_t WIN_END = OFF_XM + LVL_S + 16 * SBO_S;  // last M-side window
  static constexpr uint32_t BYTES = ((END > WIN_END ? END : WIN_END) + 127u) / 128u * 128u;
};

// M row of component c of row i, in the interleaved order.
__device__ __forceinline__ int mrow(int c, int i) { return ((i >> 4) << 5) + (c << 4) + (i & 15); }
// N column of part p (0: the odd 16-block) for index j.
__device__ __forceinline__ int ncol(int p, int j) { return ((j >> 4) << 5) + ((1 - p) << 4) + (j & 15); }

// Byte offset of element (r, k) in the S layout (row r, K index k).
template <bool BF16, int NP>
__device__ __forceinline__ uint32_t off_s(int r, int k) {
  using G = Geo<BF16, NP>;
  return (uint32_t)(r >> 3) * G::SBO_S + (uint32_t)(k / G::EPC) * 128u + (uint32_t)(r & 7) * 16u +
         (uint32_t)(k % G::EPC) * Elem<BF16>::kSize;
}
// Byte offset of element (r, k) of the X^T buffer (N row r, K index k): the
// T layout (TF32), the MN-major layout (BF16).
template <bool BF16, int NP>
__device__ __forceinline__ uint32_t off_t(int r, int k) {
  using G = Geo<BF16, NP>;
  if constexpr (BF16) {
    return (uint32_t)(r >> 3) * G::SN_M + (uint32_t)(k >> 3) * G::SK_M + (uint32_t)(k & 7) * 16u +
           (uint32_t)(r & 7) * 2u;
  } else {
    return (uint32_t)(r >> 3) * G::SBO_T + (uint32_t)(k / G::EPC) * G::LBO_T + (uint32_t)(r & 7) * 16u +
           (uint32_t)(k % G::EPC) * Elem<BF16>::kSize;
  }
}

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

// The 6 K-loops of one RK4 stage (single issuing thread), all at N = 2 NP
// into one accumulator.
// mshift: the M-side windows start this many bytes before the buffers, so
// that the instance's rows land in TMEM lanes 64..127 (second instance of a
// CTA that runs two).
template <bool BF16, int NP>
__device__ __forceinline__ void issue_stage(uint32_t d, uint32_t base, uint32_t mshift) {
  using G = Geo<BF16, NP>;
  constexpr uint32_t id = idesc(Elem<BF16>::kFmt, 128, 2 * NP, false, false);
  constexpr uint32_t idx = idesc(Elem<BF16>::kFmt, 128, 2 * NP, false, BF16);  // A X: B MN-major (BF16)
  const uint64_t dAm = sdesc(base + G::OFF_A - mshift, 128, G::SBO_S);  // A as M side
  const uint64_t dAn = sdesc(base + G::OFF_A, 128, G::SBO_S);           // A as N side
  const uint64_t dXM = sdesc(base + G::OFF_XM - mshift, 128, G::SBO_S);
  const uint64_t dXT = BF16 ? sdesc(base + G::OFF_XT, G::SK_M, G::SN_M)
                            : sdesc(base + G::OFF_XT, G::LBO_T, G::SBO_T);
  // A X: A_hi X_hi, A_hi X_lo, A_lo X_hi
  // (the accumulator already holds the diagonal term, so every MMA accumulates)
#pragma unroll
  for (int s = 0; s < G::KS; ++s)
    mma<BF16>(d, dadd(dAm, s * G::KSTEP_S), dadd(dXT, s * G::KSTEP_T), idx, 1u);
#pragma unroll
  for (int s = 0; s < G::KS; ++s)
    mma<BF16>(d, dadd(dAm, s * G::KSTEP_S), dadd(dXT, G::LVL_T + s * G::KSTEP_T), idx, 1u);
#pragma unroll
  for (int s = 0; s < G::KS; ++s)
    mma<BF16>(d, dadd(dAm, G::LVL_S + s * G::KSTEP_S), dadd(dXT, s * G::KSTEP_T), idx, 1u);
  // X A^dag = (-i X) (i A^dag): X_hi A_hi, X_hi A_lo, X_lo A_hi
#pragma unroll
  for (int s = 0; s < G::KS; ++s)
    mma<BF16>(d, dadd(dXM, s * G::KSTEP_S), dadd(dAn, s * G::KSTEP_S), id, 1u);
#pragma unroll
  for (int s = 0; s < G::KS; ++s)
    mma<BF16>(d, dadd(dXM, s * G::KSTEP_S), dadd(dAn, G::LVL_S + s * G::KSTEP_S), id, 1u);
#pragma unroll
  for (int s = 0; s < G::KS; ++s)
    mma<BF16>(d, dadd(dXM, G::LVL_S + s * G::KSTEP_S), dadd(dAn, s * G::KSTEP_S), id, 1u);
}

// Barriers of a thread group: the whole CTA (GR = 1) or one half of it (GR = 2,
// named barriers 1 and 2 of 256 threads).
template <int GR>
__device__ __forceinline__ void gsync(int g) {
  if constexpr (GR == 1) {
    __syncthreads();
  } else {
    asm volatile("bar.sync %0, %1;" ::"r"(g + 1), "r"(kThreads / GR) : "memory");
  }
}
template <int GR>
__device__ __forceinline__ bool gor(int g, bool pred) {
  if constexpr (GR == 1) {
    return __syncthreads_or(pred) != 0;
  } else {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 q, %1, 0;\n\t"
        "bar.red.or.pred p, %2, %3, q;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)pred), "r"(g + 1), "r"(kThreads / GR)
        : "memory");
    return r != 0;
  }
}
template <int GR>
__device__ __forceinline__ void sync_for_mma(int g) {
  fence_async_smem();
  fence_before_sync();
  gsync<GR>(g);
}

// Store 4 consecutive K elements of one operand row (16 bytes TF32, 8 bytes BF16).
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

// Store 8 consecutive K elements of one BF16 operand row (a, then b; 16 bytes).
__device__ __forceinline__ void st8_bf16(unsigned char* base, const float* a, const float* b) {
  const __nv_bfloat162 p0 = __floats2bfloat162_rn(a[0], a[1]), p1 = __floats2bfloat162_rn(a[2], a[3]);
  const __nv_bfloat162 p2 = __floats2bfloat162_rn(b[0], b[1]), p3 = __floats2bfloat162_rn(b[2], b[3]);
  uint4 u;
  u.x = *reinterpret_cast<const uint32_t*>(&p0);
  u.y = *reinterpret_cast<const uint32_t*>(&p1);
  u.z = *reinterpret_cast<const uint32_t*>(&p2);
  u.w = *reinterpret_cast<const uint32_t*>(&p3);
  *reinterpret_cast<uint4*>(base) = u;
}

// One instance, all Nt steps.  Thread mapping: warp w reads TMEM lane quarter
// q = w & 3 and owns columns [(w >> 2) NP/4, (w >> 2 + 1) NP/4) of its lane;
// lane l of the warp is TMEM lane 32 q + l = M row (c, i) with c = l >> 4,
// i = 16 q + (l & 15); its partner (1 - c, i) is lane l ^ 16.
template <bool BF16, int NP, int GR, bool BD = false>
__device__ void tc_instance(const CtaParams& p, const int b, unsigned char* smem, TcShared& sh,
                            const int grp, uint32_t& phase, bool& alive) {
  using El = Elem<BF16>;
  using G = Geo<BF16, NP>;
  using ET = typename El::T;
  constexpr int kT = kThreads / GR;  // threads of the group
  constexpr int kW = kT / 32;        // warps of the group
  constexpr int NPQ = NP / 4;        // columns per thread
  constexpr int NG = NPQ / 4;        // groups of 4 columns
  const int gwarp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int quarter = gwarp & 3, cg = gwarp >> 2;  // TMEM lane quarter, column group
  // group-local warp and thread index (GR = 2: the group holds quarters 2 grp, 2 grp + 1)
  const int warp = GR == 1 ? gwarp : (cg * 2 + (gwarp & 1));
  const int tid = warp * 32 + lane;
  const int c = lane >> 4;                              // 0: real part, 1: imaginary part
  const int i = (GR == 1 ? quarter : (quarter & 1)) * 16 + (lane & 15);  // row
  const bool row_ok = i < NP;
  const int j0 = cg * NPQ;                   // first owned column
  const int N = p.dims[b];
  // padded dimension and row stride of the FP32 working matrices (NP, or 68
  // for an instance with a border)
  const int NPD = BD ? p.npad[b] : NP;
  const int NPS = NPD + 2;
  const long long wo = p.woff[b];
  const int E = p.n_eops;
  const bool diag = p.cops_kind == 2 && p.n_cops > 0;
  const float half_dt = (float)(0.5 * p.dt), dt = (float)p.dt, sixth_dt = (float)(p.dt / 6.0);

  unsigned char* SA = smem + G::OFF_A;
  unsigned char* SXM = smem + G::OFF_XM;
  unsigned char* SXT = smem + G::OFF_XT;
  const uint32_t sbase = smem_u32(smem);
  const float2* At0 = reinterpret_cast<const float2*>(p.At) + wo;
  const float2* Gt = reinterpret_cast<const float2*>(p.Gt) + (long long)p.n_drive * wo;
  const float2* Dm = reinterpret_cast<const float2*>(p.Dm) + wo;
  const float2* OtF = p.OtF + (long long)E * wo;
  const uint32_t tmem_d = sh.tmem_base + (uint32_t)(grp * 64);
  const uint32_t mshift = (uint32_t)grp * 8u * G::SBO_S;  // 64 rows
  const uint32_t tlane = tmem_d + ((uint32_t)(quarter * 32) << 16);
  uint64_t* mbar = &sh.mbar[grp];
  TcBorder* bd = BD ? reinterpret_cast<TcBorder*>(smem + G::BYTES) : nullptr;
  constexpr int kG = NP;  // border index (BD)

  // ---- A buffer: rows (0, r) = Ar[r], (1, r) = Ai[r]; hi level then lo level.
  // Rebuilt every step when driven.
  auto build_a = [&](const float* f) {
    for (int idx = tid; idx < NP * NP; idx += kT) {
      const int k = idx / NP, r = idx % NP;  // consecutive threads: consecutive rows
      float2 a = At0[k * NPS + r];           // A[r][k]
      if (f != nullptr) {
#pragma unroll
        for (int d = 0; d < 4; ++d)
          if (d < p.n_drive) {
            const float2 g = Gt[(long long)d * NPD * NPS + k * NPS + r];
            a.x = fmaf(f[d], g.x, a.x);
            a.y = fmaf(f[d], g.y, a.y);
          }
      }
      if (k == r) {  // applied in FP32 by inject
        sh.adg[grp][r] = a;
        a = make_float2(0.f, 0.f);
      }
      float h, lo;
      El::split(a.x, h, lo);
      *reinterpret_cast<ET*>(SA + off_s<BF16, NP>(mrow(0, r), k)) = (ET)h;
      *reinterpret_cast<ET*>(SA + G::LVL_S + off_s<BF16, NP>(mrow(0, r), k)) = (ET)lo;
      El::split(a.y, h, lo);
      *reinterpret_cast<ET*>(SA + off_s<BF16, NP>(mrow(1, r), k)) = (ET)h;
      *reinterpret_cast<ET*>(SA + G::LVL_S + off_s<BF16, NP>(mrow(1, r), k)) = (ET)lo;
    }
  };

  // ---- X operands of a stage input x (this thread's component of row i):
  //   XM (M side of X A^dag): row (0, i) = Xi[i], row (1, i) = -Xr[i]
  //   X^T (N side of A X):    row (0, j) = Xr[.][j], row (1, j) = Xi[.][j], K index i
  // written 4 columns at a time (group g: columns j0 + 4g .. j0 + 4g + 3).
  const int xm_row = mrow(1 - c, i);
  const float xm_sign = c == 0 ? -1.f : 1.f;
  // BF16 with a multiple of 8 columns per thread: the XM values of an even
  // group wait for the odd one and both go out as one 16-byte store per level
  // (8-byte stores of the 32 rows of a warp, 1 KB apart per row group, would
  // share one bank set).  Every caller walks the groups in order.
  constexpr bool kXmPairs = BF16 && (NPQ % 8 == 0);
  [[maybe_unused]] uint32_t xph[2], xpl[2];  // BF16: packed XM values of the even group
  // XM row sign as a bit mask on packed BF16 pairs (c = 0: the row holds -Xr)
  [[maybe_unused]] const uint32_t xm_flip = c == 0 ? 0x80008000u : 0u;
  auto write_group = [&](int g, const float* x4) {
    if (!row_ok) return;
    const int col = j0 + g * 4;
    if constexpr (BF16) {
      // split on packed pairs: hi = bf16(x) (two at a time), lo = bf16(x - hi);
      // the same values as Elem<true>::split, with fewer conversions
      uint32_t h[2], l[2];
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const __nv_bfloat162 hb = __floats2bfloat162_rn(x4[2 * q], x4[2 * q + 1]);
        const float2 hf = __bfloat1622float2(hb);
        const float2 r = __fadd2_rn(make_float2(x4[2 * q], x4[2 * q + 1]), make_float2(-hf.x, -hf.y));
        const __nv_bfloat162 lb = __floats2bfloat162_rn(r.x, r.y);
        h[q] = *reinterpret_cast<const uint32_t*>(&hb);
        l[q] = *reinterpret_cast<const uint32_t*>(&lb);
      }
      // X^T (MN-major): the 4 columns are 4 consecutive N elements of K-row i
      // (one 8-byte piece of a core-matrix row; 16 bytes for a pair of groups)
      if constexpr (kXmPairs) {
        if ((g & 1) == 0) {
          xph[0] = h[0];
          xph[1] = h[1];
          xpl[0] = l[0];
          xpl[1] = l[1];
        } else {
          const uint32_t o = off_t<BF16, NP>(ncol(c, col - 4), i);
          *reinterpret_cast<uint4*>(SXT + o) = make_uint4(xph[0], xph[1], h[0], h[1]);
          *reinterpret_cast<uint4*>(SXT + G::LVL_T + o) = make_uint4(xpl[0], xpl[1], l[0], l[1]);
          // -bf16(x) = bf16(-x) exactly: the XM sign is a flip of the sign bits
          const uint32_t m = off_s<BF16, NP>(xm_row, col - 4);
          *reinterpret_cast<uint4*>(SXM + m) =
              make_uint4(xph[0] ^ xm_flip, xph[1] ^ xm_flip, h[0] ^ xm_flip, h[1] ^ xm_flip);
          *reinterpret_cast<uint4*>(SXM + G::LVL_S + m) =
              make_uint4(xpl[0] ^ xm_flip, xpl[1] ^ xm_flip, l[0] ^ xm_flip, l[1] ^ xm_flip);
        }
      } else {
        const uint32_t o = off_t<BF16, NP>(ncol(c, col), i);
        *reinterpret_cast<uint2*>(SXT + o) = make_uint2(h[0], h[1]);
        *reinterpret_cast<uint2*>(SXT + G::LVL_T + o) = make_uint2(l[0], l[1]);
        const uint32_t m = off_s<BF16, NP>(xm_row, col);
        *reinterpret_cast<uint2*>(SXM + m) = make_uint2(h[0] ^ xm_flip, h[1] ^ xm_flip);
        *reinterpret_cast<uint2*>(SXM + G::LVL_S + m) = make_uint2(l[0] ^ xm_flip, l[1] ^ xm_flip);
      }
    } else {
      float vh[4], vl[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) El::split(x4[e], vh[e], vl[e]);  // split(-x) = -split(x)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const uint32_t o = off_t<BF16, NP>(ncol(c, col + e), i);
        *reinterpret_cast<ET*>(SXT + o) = (ET)vh[e];
        *reinterpret_cast<ET*>(SXT + G::LVL_T + o) = (ET)vl[e];
        vh[e] *= xm_sign;
        vl[e] *= xm_sign;
      }
      st4<BF16>(SXM + off_s<BF16, NP>(xm_row, col), vh);
      st4<BF16>(SXM + G::LVL_S + off_s<BF16, NP>(xm_row, col), vl);
    }
  };
  // The diagonal term (a_i + conj(a_j)) X_ij of the stage input x (columns
  // j0 + 4g .. + 3; the partner lane holds the other component) into the
  // part-0 accumulator columns, the part-1 columns zeroed.  Warp-uniform.
  const float sgx = c == 0 ? -1.f : 1.f;
  // ai: a_i of this thread's row (adg_row())
  auto adg_row = [&]() -> float2 { return row_ok ? sh.adg[grp][i] : make_float2(0.f, 0.f); };
  auto inject = [&](int g, const float* x4, float2 ai) {
    {
      const int col = j0 + g * 4;
      float q[4];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const float4 aj = *reinterpret_cast<const float4*>(&sh.adg[grp][col + 2 * h]);
        const float2 x2 = make_float2(x4[2 * h], x4[2 * h + 1]);
        const float2 xp2 = make_float2(__shfl_xor_sync(0xffffffffu, x4[2 * h], 16),
                                       __shfl_xor_sync(0xffffffffu, x4[2 * h + 1], 16));
        // Re: (ar_i + ar_j) xr - (ai_i - ai_j) xi,  Im: (ar_i + ar_j) xi + (ai_i - ai_j) xr
        const float2 dx2 = __fadd2_rn(make_float2(ai.x, ai.x), make_float2(aj.x, aj.z));
        const float2 sdy2 = __ffma2_rn(make_float2(-sgx, -sgx), make_float2(aj.y, aj.w),
                                       make_float2(sgx * ai.y, sgx * ai.y));
        const float2 q2 = __ffma2_rn(sdy2, xp2, __fmul2_rn(dx2, x2));
        q[2 * h] = q2.x;
        q[2 * h + 1] = q2.y;
      }
      const float z[4] = {0.f, 0.f, 0.f, 0.f};
      tmem_st4(tlane + (uint32_t)ncol(0, col), q);
      tmem_st4(tlane + (uint32_t)ncol(1, col), z);
    }
  };
  // hi + lo of the current stage input of group g, read back from XM (used by
  // the general diagonal dissipator)
  auto read_group = [&](int g, float* x4) {
    const int col = j0 + g * 4;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      float v = 0.f;
      if (row_ok) {
        const uint32_t o = off_s<BF16, NP>(xm_row, col + e);
        v = (float)*reinterpret_cast<const ET*>(SXM + o) +
            (float)*reinterpret_cast<const ET*>(SXM + G::LVL_S + o);
      }
      x4[e] = xm_sign * v;
    }
  };

  // ---- state: element jj of this thread is component .x (jj even) or .y (jj
  // odd) of pair jj / 2, so the RK4 arithmetic runs on packed FP32x2 pairs;
  // nkc holds the negated Kahan compensation.
  float2 rho2[NPQ / 2], racc2[NPQ / 2], nkc2[NPQ / 2];
  auto rho_at = [&](int jj) -> float { return (jj & 1) ? rho2[jj >> 1].y : rho2[jj >> 1].x; };

  // ---- observables Tr[O rho]: FP32 partials per thread and warp (pairwise
  // shuffle tree), folded across warps by a second shuffle tree and written in
  // FP64.  A per-thread mask skips the zero entries of O (sparse observables
  // such as a transition dipole).
  uint32_t omask = 0;  // bit e*NPQ+jj (E * NPQ <= 32 bits used)
  const bool use_mask = E * NPQ <= 32;
  if (use_mask && i < N) {
    for (int e = 0; e < E; ++e) {
      const float2* o = OtF + (long long)e * NPD * NPS + (long long)i * NPS + j0;
#pragma unroll
      for (int jj = 0; jj < NPQ; ++jj) {
        const float2 ov = o[jj];
        if (ov.x != 0.f || ov.y != 0.f) omask |= 1u << (e * NPQ + jj);
      }
    }
  }
  // Part 1 (no barrier): per-warp partials of every Tr[O_e rho] into sh.red;
  // returns whether this thread's elements are finite.
  // ---- optional per-step check (p.check_tol > 0), FP64 accumulation: the
  // drift |Tr rho(t) - Tr rho0| and, for a Hermitian rho0, max_ij
  // |rho_ij - conj(rho_ji)|.  Both sides of the hermiticity test are read
  // from the X^T operand buffer (hi + lo, the stage input = rho after the
  // step), so that an exactly Hermitian FP32 state compares equal; the
  // resolution is that of the split operands.  Thread 0 of the group keeps
  // the running maxima.
  const bool checking = p.check_tol > 0.0 && p.chk != nullptr;
  auto xt_at = [&](int r, int k) -> float {  // component of X^T row r, K index k (hi + lo)
    const uint32_t o = off_t<BF16, NP>(r, k);
    return (float)*reinterpret_cast<const ET*>(SXT + o) + (float)*reinterpret_cast<const ET*>(SXT + G::LVL_T + o);
  };
  auto check_partials = [&]() {
    float tr = 0.f, hf = 0.f;
    if (i < N) {
#pragma unroll 1
      for (int jj = 0; jj < NPQ; ++jj) {
        const int j = j0 + jj;
        if (j < N) {
          const float a = xt_at(ncol(c, j), i), t = xt_at(ncol(c, i), j);  // rho_ij, rho_ji (component c)
          if (j == i) tr = a;
          hf = fmaxf(hf, fabsf(c == 0 ? a - t : a + t));  // exact for the split values of a Hermitian state
        }
      }
    }
    // both components of each element: the partner lane holds the other one
    const double hp = (double)__shfl_xor_sync(0xffffffffu, hf, 16);
    double hm = sqrt((double)hf * (double)hf + hp * hp);
    double trx = c == 0 ? (double)tr : 0.0, tri = c == 1 ? (double)tr : 0.0;
    if constexpr (BD) {
      if (tid < kG) {  // border column (t, g) against row (g, t); the corner in the trace
        const float2 a = bd->rho[0][tid], t = bd->rho[1][tid];
        const double dx = (double)a.x - (double)t.x, dy = (double)a.y + (double)t.y;
        hm = fmax(hm, sqrt(dx * dx + dy * dy));
      } else if (tid == kG) {
        const float2 z = bd->rho[1][kG];
        trx += (double)z.x;
        tri += (double)z.y;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      trx += __shfl_xor_sync(0xffffffffu, trx, o);
      tri += __shfl_xor_sync(0xffffffffu, tri, o);
      hm = fmax(hm, __shfl_xor_sync(0xffffffffu, hm, o));
    }
    if (lane == 0) {
      sh.chk[grp][warp][0] = trx;
      sh.chk[grp][warp][1] = tri;
      sh.chk[grp][warp][2] = hm;
    }
  };
  // after a barrier that follows check_partials
  auto check_fold = [&](bool initial) {
    if (tid != 0) return;
    double2 tr = make_double2(0.0, 0.0);
    double h = 0.0;
    for (int w = 0; w < kW; ++w) {
      tr.x += sh.chk[grp][w][0];
      tr.y += sh.chk[grp][w][1];
      h = fmax(h, sh.chk[grp][w][2]);
    }
    double* run = sh.chk_run[grp];
    if (initial) {
      run[0] = tr.x;
      run[1] = tr.y;
      run[2] = run[3] = 0.0;
      sh.chk_flags[grp] = h <= p.check_tol ? 1 : 0;
    } else {
      const double ex = tr.x - run[0], ey = tr.y - run[1];
      const double dtr = sqrt(ex * ex + ey * ey);
      const bool herm = (sh.chk_flags[grp] & 1) != 0;
      run[2] = fmax(run[2], dtr);
      if (herm) run[3] = fmax(run[3], h);
      if (!(dtr <= p.check_tol) || (herm && !(h <= p.check_tol))) sh.chk_flags[grp] |= 2;
    }
  };

  auto obs_partials = [&]() -> bool {
    if (checking) check_partials();
    bool fin = true;
    if (i < N) {
#pragma unroll
      for (int jj = 0; jj < NPQ; ++jj) fin = fin && isfinite(rho_at(jj));
    }
    for (int e = 0; e < E; ++e) {
      float fx = 0.f, fy = 0.f;
      const uint32_t m = use_mask ? (omask >> (e * NPQ)) : 0xffffffffu;
      if (i < N && (m & ((NPQ >= 32) ? 0xffffffffu : ((1u << NPQ) - 1u))) != 0u) {
        const float2* o = OtF + (long long)e * NPD * NPS + (long long)i * NPS + j0;
        float2 ov[NPQ];
        // all loads issued before the first FMA (independent, predicated)
#pragma unroll
        for (int jj = 0; jj < NPQ; ++jj)
          ov[jj] = (m & (1u << jj)) ? __ldg(o + jj) : make_float2(0.f, 0.f);  // O[j][i]
#pragma unroll
        for (int jj = 0; jj < NPQ; ++jj) {
          if (c == 0) {
            fx = fmaf(ov[jj].x, rho_at(jj), fx);
            fy = fmaf(ov[jj].y, rho_at(jj), fy);
          } else {
            fx = fmaf(-ov[jj].y, rho_at(jj), fx);
            fy = fmaf(ov[jj].x, rho_at(jj), fy);
          }
        }
      }
      if constexpr (BD) {
        // border element (t, g) for t < 64, (g, t - 64) otherwise: O^T entry
        // [i][j] = O[j][i] at i * NPS + j
        if (tid < 2 * kG + 1) {
          const bool col = tid < kG;
          const int t = col ? tid : tid - kG;
          const float2 ov = OtF[(long long)e * NPD * NPS + (col ? t * NPS + kG : kG * NPS + t)];
          const float2 rv = bd->rho[col ? 0 : 1][t];
          fx = fmaf(ov.x, rv.x, fmaf(-ov.y, rv.y, fx));
          fy = fmaf(ov.x, rv.y, fmaf(ov.y, rv.x, fy));
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        fx += __shfl_xor_sync(0xffffffffu, fx, o);
        fy += __shfl_xor_sync(0xffffffffu, fy, o);
      }
      if (lane == 0) sh.red[grp][e][warp] = make_float2(fx, fy);
    }
    if constexpr (BD) {
      if (tid < 2 * kG + 1) {
        const float2 rv = bd->rho[tid < kG ? 0 : 1][tid < kG ? tid : tid - kG];
        fin = fin && isfinite(rv.x) && isfinite(rv.y);
      }
    }
    return fin;
  };
  // Part 2 (its barrier follows part 1): warp w folds the per-warp partials of
  // observables w, w + kW, .. and writes row ``row``; returns whether any
  // element was not finite.
  auto obs_finish = [&](bool fin, int row) -> bool {
    const bool anybad = gor<GR>(grp, !fin);
    if (checking) check_fold(false);
    if (p.obs_out != nullptr) {
      for (int e = warp; e < E; e += kW) {
        float2 v = lane < kW ? sh.red[grp][e][lane] : make_float2(0.f, 0.f);
#pragma unroll
        for (int o = kW / 2; o > 0; o >>= 1) {
          v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
          v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
        }
        if (lane == 0) {
          const long long nrows = (long long)p.nt + p.obs_t0;
          p.obs_out[((long long)b * nrows + row) * E + e] = make_double2((double)v.x, (double)v.y);
        }
      }
    }
    return anybad;
  };

  // Bounded wait for the last commit; on time-out mark the instance and stop.
  // What follows a time-out is best effort: MMAs possibly still in flight get
  // one more bounded wait, and then the CTA goes on to free its tensor memory
  // whether or not they drained -- a CTA that exited still holding it would
  // make every later allocation on this SM wait forever, which is worse than
  // a stalled pipe writing into columns nobody reads any more.
  const long long spin = p.spin > 0 ? p.spin : kSpinLimit;
  auto wait_mma = [&]() -> bool {
    const bool ok = mbar_wait(mbar, phase, spin);
    phase ^= 1u;
    if (gor<GR>(grp, !ok)) {
      if (tid == 0) p.err[b] = 5;  // LGB_ERR_TIMEOUT
      mbar_wait(mbar, phase ^ 1u, spin);  // let MMAs still in flight finish (bounded)
      alive = false;
      return false;
    }
    return true;
  };

  // ---- state -------------------------------------------------------------------
  {
    const double2* r0 = p.rho0 + p.off[b];
#pragma unroll
    for (int jj = 0; jj < NPQ; ++jj) {
      const int j = j0 + jj;
      double v = 0.0;
      if (i < N && j < N) {
        const double2 z = r0[(long long)i * N + j];
        v = c == 0 ? z.x : z.y;
      }
      if (jj & 1) {
        rho2[jj >> 1].y = (float)v;
      } else {
        rho2[jj >> 1].x = (float)v;
        racc2[jj >> 1] = make_float2(0.f, 0.f);
        nkc2[jj >> 1] = make_float2(0.f, 0.f);
      }
    }
  }

  // Dissipator D o X of diagonal collapse operators.  Pure-dephasing type
  // (D diagonal and real) keeps D_ii in a register; a general D is read from
  // the working copy; a complex D couples the real and imaginary lanes, which
  // exchange the stage input with a warp shuffle.
  bool off = false, dc = false;
  if (diag && i < N) {
#pragma unroll
    for (int jj = 0; jj < NPQ; ++jj) {
      const float2 d = Dm[i * NPS + j0 + jj];
      off = off || ((j0 + jj != i) && (d.x != 0.f || d.y != 0.f));
      dc = dc || (d.y != 0.f);
    }
  }
  const bool dgeneral = gor<GR>(grp, off);
  const bool dcomplex = gor<GR>(grp, dc);
  const bool dfast = diag && !dgeneral && !dcomplex;
  const int dpos = (i >= j0 && i < j0 + NPQ) ? i - j0 : -1;
  const float dd = (dfast && dpos >= 0 && i < N) ? Dm[i * NPS + i].x : 0.f;
  // warps that hold diagonal elements; element (i, i) of the stage input
  const bool dwarp = __any_sync(0xffffffffu, dpos >= 0 && i < N) != 0;
  float xd = 0.f;
#pragma unroll
  for (int jj = 0; jj < NPQ; ++jj) xd = (jj == dpos) ? rho_at(jj) : xd;
  if (p.n_drive == 0) build_a(nullptr);
#pragma unroll
  for (int g = 0; g < NG; ++g) {
    const float x4[4] = {rho2[2 * g].x, rho2[2 * g].y, rho2[2 * g + 1].x, rho2[2 * g + 1].y};
    write_group(g, x4);
  }
  // ---- border (BD): constants, state, and the (M conj(b)) partials of rho0
  int bcur = 0;  // border buffer holding the current stage input
  if constexpr (BD) {
    const double2* r0 = p.rho0 + p.off[b];
    for (int t = tid; t < kBorder; t += kT) {
      bd->aB[t] = At0[kG * NPS + t];  // A[t][g]
      bd->bB[t] = At0[t * NPS + kG];  // A[g][t]
      bd->dcol[t] = diag ? Dm[t * NPS + kG] : make_float2(0.f, 0.f);
      bd->drow[t] = diag ? Dm[kG * NPS + t] : make_float2(0.f, 0.f);
    }
    if (tid < 2 * kG + 1) {  // thread t owns border element (t, g) or (g, t - 64)
      const bool col = tid < kG;
      const int t = col ? tid : tid - kG, sl = col ? 0 : 1;
      const double2 z = col ? r0[(long long)t * N + kG] : r0[(long long)kG * N + t];
      const float2 v = make_float2((float)z.x, (float)z.y);
      bd->rho[sl][t] = v;
      bd->bx[0][sl][t] = v;
      bd->racc[sl][t] = make_float2(0.f, 0.f);
      bd->nkc[sl][t] = make_float2(0.f, 0.f);
    }
    gsync<GR>(grp);
    float tx = 0.f, ty = 0.f;
#pragma unroll
    for (int jj = 0; jj < NPQ; ++jj) {
      const float2 bj = bd->bB[j0 + jj];
      const float v = rho_at(jj);  // c = 0: Re M_ij, c = 1: Im M_ij
      tx = fmaf(v, c == 0 ? bj.x : bj.y, tx);
      ty = fmaf(v, c == 0 ? -bj.y : bj.x, ty);
    }
    tx += __shfl_xor_sync(0xffffffffu, tx, 16);
    ty += __shfl_xor_sync(0xffffffffu, ty, 16);
    if (c == 0) bd->t2p[0][i][cg] = make_float2(tx, ty);
  }
  // Border work of one stage, run while the block's MMAs are in flight: the
  // mode sums, then (after a barrier) the RK4 update of the 129 border
  // elements into the other border buffer.
  auto border_phase = [&](int stage) {
    if constexpr (BD) {
      const float2* bc = bd->bx[bcur][0];
      const float2* br = bd->bx[bcur][1];
      {  // (A_M c)_i and (conj(A_M) r)_j: four threads per row, 16 k each
        const int d = tid >> 2, q = tid & 3;
        const int row = d & (kG - 1);
        const bool t4 = d >= kG;
        float sx = 0.f, sy = 0.f;
        // all sixteen loads of A (L2-resident) in flight at once
        float2 av[16];
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) av[kk] = __ldg(At0 + (q * 16 + kk) * NPS + row);  // A[row][k]
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
          const int k = q * 16 + kk;
          const float2 a = av[kk];
          const float2 v = t4 ? br[k] : bc[k];
          const float ay = t4 ? -a.y : a.y;
          sx = fmaf(a.x, v.x, fmaf(-ay, v.y, sx));
          sy = fmaf(a.x, v.y, fmaf(ay, v.x, sy));
        }
        sx += __shfl_xor_sync(0xffffffffu, sx, 1);
        sy += __shfl_xor_sync(0xffffffffu, sy, 1);
        sx += __shfl_xor_sync(0xffffffffu, sx, 2);
        sy += __shfl_xor_sync(0xffffffffu, sy, 2);
        if (q == 0) (t4 ? bd->t4 : bd->t1)[row] = make_float2(sx, sy);
      }
      if constexpr (BF16) {
        // (b^T M)_j from the MN-major X^T operand (hi + lo): warp w takes
        // N-group w (8 consecutive n, one part p of 8 columns j) and walks the
        // eight K-groups; lane l reads K-row l >> 2, N pair 2 (l & 3), so that
        // each load of the warp is one 128-byte core matrix.  The partial sums
        // over k meet across the eight lanes of an N pair.
        const int ng = warp;
        const int p_part = (ng & 3) < 2 ? 1 : 0;  // ncol: the odd 16-block holds part 0
        const int jbase = 16 * (ng >> 2) + 8 * (ng & 1);
        const int kr = lane >> 2, np2 = 2 * (lane & 3);
        float s0x = 0.f, s0y = 0.f, s1x = 0.f, s1y = 0.f;  // b_k M_p[k][j], j = jbase + np2 + {0, 1}
#pragma unroll
        for (int kg = 0; kg < NP / 8; ++kg) {
          const int k = kg * 8 + kr;
          const uint32_t o = (uint32_t)ng * G::SN_M + (uint32_t)kg * G::SK_M + (uint32_t)kr * 16u + (uint32_t)np2 * 2u;
          const __nv_bfloat162 hv = *reinterpret_cast<const __nv_bfloat162*>(SXT + o);
          const __nv_bfloat162 lv = *reinterpret_cast<const __nv_bfloat162*>(SXT + G::LVL_T + o);
          const float2 m = __fadd2_rn(__bfloat1622float2(hv), __bfloat1622float2(lv));
          const float2 bk = bd->bB[k];
          s0x = fmaf(bk.x, m.x, s0x);
          s0y = fmaf(bk.y, m.x, s0y);
          s1x = fmaf(bk.x, m.y, s1x);
          s1y = fmaf(bk.y, m.y, s1y);
        }
#pragma unroll
        for (int o = 4; o < 32; o <<= 1) {
          s0x += __shfl_xor_sync(0xffffffffu, s0x, o);
          s0y += __shfl_xor_sync(0xffffffffu, s0y, o);
          s1x += __shfl_xor_sync(0xffffffffu, s1x, o);
          s1y += __shfl_xor_sync(0xffffffffu, s1y, o);
        }
        if (kr == 0) {
          bd->t3p[p_part][jbase + np2] = make_float2(s0x, s0y);
          bd->t3p[p_part][jbase + np2 + 1] = make_float2(s1x, s1y);
        }
      } else {  // (b^T M)_j from the X^T operand (hi + lo): eight threads per column, 8 k each
        const int j = tid >> 3, q = tid & 7;
        const int rr = ncol(0, j), ri = ncol(1, j);
        float sx = 0.f, sy = 0.f;
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) {
          const int k = q * 8 + kk;
          const uint32_t o_r = off_t<BF16, NP>(rr, k), o_i = off_t<BF16, NP>(ri, k);
          const float mr = (float)*reinterpret_cast<const ET*>(SXT + o_r) +
                           (float)*reinterpret_cast<const ET*>(SXT + G::LVL_T + o_r);
          const float mi = (float)*reinterpret_cast<const ET*>(SXT + o_i) +
                           (float)*reinterpret_cast<const ET*>(SXT + G::LVL_T + o_i);
          const float2 bk = bd->bB[k];
          sx = fmaf(bk.x, mr, fmaf(-bk.y, mi, sx));
          sy = fmaf(bk.x, mi, fmaf(bk.y, mr, sy));
        }
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) {
          sx += __shfl_xor_sync(0xffffffffu, sx, o);
          sy += __shfl_xor_sync(0xffffffffu, sy, o);
        }
        if (q == 0) bd->t3[j] = make_float2(sx, sy);
      }
      if (warp == kW - 1) {  // corner sums b.c and r.conj(b)
        float ux = 0.f, uy = 0.f, vx = 0.f, vy = 0.f;
        for (int k = lane; k < kG; k += 32) {
          const float2 bk = bd->bB[k], ck = bc[k], rk = br[k];
          ux = fmaf(bk.x, ck.x, fmaf(-bk.y, ck.y, ux));
          uy = fmaf(bk.x, ck.y, fmaf(bk.y, ck.x, uy));
          vx = fmaf(rk.x, bk.x, fmaf(rk.y, bk.y, vx));
          vy = fmaf(rk.y, bk.x, fmaf(-rk.x, bk.y, vy));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          ux += __shfl_xor_sync(0xffffffffu, ux, o);
          uy += __shfl_xor_sync(0xffffffffu, uy, o);
          vx += __shfl_xor_sync(0xffffffffu, vx, o);
          vy += __shfl_xor_sync(0xffffffffu, vy, o);
        }
        if (lane == 0) {
          bd->csum[0] = make_float2(ux, uy);
          bd->csum[1] = make_float2(vx, vy);
        }
      }
      gsync<GR>(grp);
      if (tid < 2 * kG + 1) {
        const bool col = tid < kG;
        const int t = col ? tid : tid - kG, sl = col ? 0 : 1;
        const float2 z = br[kG], al = bd->aB[kG];
        const float2 alc = make_float2(al.x, -al.y);
        float2 R;
        if (col) {
          const float2 x = bc[t], a = bd->aB[t];
          const float2* tp = bd->t2p[bcur][t];
          R = bd->t1[t];
          R.x += (tp[0].x + tp[1].x) + (tp[2].x + tp[3].x);
          R.y += (tp[0].y + tp[1].y) + (tp[2].y + tp[3].y);
          cmac(R, a, z);
          cmac(R, x, alc);
          cmac(R, bd->dcol[t], x);
        } else if (t < kG) {
          const float2 x = br[t], a = bd->aB[t];
          if constexpr (BF16) {  // b^T M = b^T M_0 + i b^T M_1
            const float2 u = bd->t3p[0][t], v = bd->t3p[1][t];
            R = make_float2(u.x - v.y, u.y + v.x);
          } else {
            R = bd->t3[t];
          }
          R.x += bd->t4[t].x;
          R.y += bd->t4[t].y;
          cmac(R, al, x);
          cmac(R, z, make_float2(a.x, -a.y));
          cmac(R, bd->drow[t], x);
        } else {
          R = bd->csum[0];
          R.x += bd->csum[1].x;
          R.y += bd->csum[1].y;
          cmac(R, al, z);
          cmac(R, z, alc);
          cmac(R, bd->drow[kG], z);
        }
        const float2 rh = bd->rho[sl][t];
        float2 xn;
        if (stage == 0) {
          bd->racc[sl][t] = R;
          xn = make_float2(fmaf(half_dt, R.x, rh.x), fmaf(half_dt, R.y, rh.y));
        } else if (stage < 3) {
          const float2 ra = bd->racc[sl][t];
          bd->racc[sl][t] = make_float2(fmaf(2.f, R.x, ra.x), fmaf(2.f, R.y, ra.y));
          const float h = stage == 2 ? dt : half_dt;
          xn = make_float2(fmaf(h, R.x, rh.x), fmaf(h, R.y, rh.y));
        } else {
          // Kahan-compensated rho += dt/6 (k1 + 2 k2 + 2 k3 + k4), as the block
          const float2 ra = bd->racc[sl][t], nk = bd->nkc[sl][t];
          const float yx = fmaf(sixth_dt, ra.x + R.x, nk.x), yy = fmaf(sixth_dt, ra.y + R.y, nk.y);
          const float tx = rh.x + yx, ty = rh.y + yy;
          bd->nkc[sl][t] = make_float2(yx - (tx - rh.x), yy - (ty - rh.y));
          xn = make_float2(tx, ty);
          bd->rho[sl][t] = xn;
        }
        bd->bx[bcur ^ 1][sl][t] = xn;
      }
    }
  };
  if (tid == 0) p.err[b] = 0;
  if (checking) {  // the values of rho0 (the X^T buffer written above)
    gsync<GR>(grp);
    check_partials();
    gsync<GR>(grp);
    check_fold(true);
  }
  if (p.obs_t0) obs_finish(obs_partials(), 0);
  // The observables of step s are reduced while the MMAs of the first stage
  // of step s + 1 run (and after the loop for the last step).
  int pend_row = -1;
  bool pend_fin = true, nonfinite = false;

  const double* drv = p.drive;
  if (p.n_drive > 0 && !p.drive_shared) drv += (long long)b * p.n_drive * p.nt;

  for (int step = 0; step < p.nt && alive; ++step) {
    if (p.n_drive > 0) {
      float f[4];
#pragma unroll
      for (int d = 0; d < 4; ++d) f[d] = (d < p.n_drive) ? (float)drv[(long long)d * p.nt + step] : 0.f;
      build_a(f);
    }
    {
      // diagonal term of the first stage (later steps of a static H get it from
      // the last epilogue of the step before)
      if (step == 0 || p.n_drive > 0) {
        gsync<GR>(grp);  // the diagonal written by build_a
        const float2 ai = adg_row();
#pragma unroll
        for (int g = 0; g < NG; ++g) {
          const float x4[4] = {rho2[2 * g].x, rho2[2 * g].y, rho2[2 * g + 1].x, rho2[2 * g + 1].y};
          inject(g, x4, ai);
        }
        tmem_wait_st();
      }
    }
#pragma unroll 1
    for (int stage = 0; stage < 4; ++stage) {
      sync_for_mma<GR>(grp);
      // (test hook: with test_stall the first stage's MMAs and commit are not
      // issued, so that its bounded wait runs out)
      if (tid == 0 && !(p.test_stall && step == 0 && stage == 0)) {
        fence_after_sync();
        issue_stage<BF16, NP>(tmem_d, sbase, mshift);
        mma_commit(mbar);
      }
      border_phase(stage);
      if (stage == 0 && pend_row >= 0) pend_fin = obs_partials();
      if (!wait_mma()) break;
      if (stage == 0 && pend_row >= 0) {
        const bool bad = obs_finish(pend_fin, pend_row);
        pend_row = -1;
        if (bad) {
          nonfinite = true;
          break;
        }
      }
      fence_after_sync();
      // RHS element R = (combined accumulator) + (D o X); stages 0-2 form the
      // RK4 sum and the next stage input, stage 3 applies the Kahan-compensated
      // update.  Each group of 4 columns (never crossing a 16-block) is loaded
      // from TMEM, combined with the partner lane, updated and written straight
      // into the operand buffers of the next stage.
      const float2 cst2 = make_float2(stage == 2 ? dt : half_dt, stage == 2 ? dt : half_dt);
      // MODE 0: no diagonal dissipator term in this warp, 1: pure dephasing
      // (diagonal real D) in a warp that holds diagonal elements, 2: general
      // diagonal D.  STAGE 0, 1 (stages 1 and 2) or 3.  Mode and stage are
      // resolved outside the unrolled element loops.
      auto epilogue = [&](auto mode_tag, auto stage_tag) {
        constexpr int MODE = decltype(mode_tag)::value;
        constexpr int STAGE = decltype(stage_tag)::value;
        const float sg = c == 0 ? -1.f : 1.f;
        const float2 sg2 = make_float2(sg, sg), m1 = make_float2(-1.f, -1.f);
        const float ddxd = dd * xd;
        // BD: this thread's component of a_i r_j + c_i conj(a_j) is
        // u0 r_j.x + u1 r_j.y + u2 a_j.x + u3 a_j.y; tx, ty accumulate the
        // (M conj(b))_i partial of the next stage input
        [[maybe_unused]] float u0 = 0.f, u1 = 0.f, u2 = 0.f, u3 = 0.f, tx = 0.f, ty = 0.f;
        [[maybe_unused]] const float2* brow = nullptr;
        [[maybe_unused]] float2 ai_row = make_float2(0.f, 0.f);
        ai_row = adg_row();
        if constexpr (BD) {
          const float2 ai = bd->aB[i], ci = bd->bx[bcur][0][i];
          u0 = c == 0 ? ai.x : ai.y;
          u1 = c == 0 ? -ai.y : ai.x;
          u2 = c == 0 ? ci.x : ci.y;
          u3 = c == 0 ? ci.y : -ci.x;
          brow = bd->bx[bcur][1];
        }
        // the accumulator columns of group g + 1 are loaded while group g is
        // processed (one tcgen05.wait::ld per group, after the group's work)
        float pa1[2][4], pa0[2][4];
        tmem_ld4(tlane + (uint32_t)ncol(1, j0), pa1[0]);
        tmem_ld4(tlane + (uint32_t)ncol(0, j0), pa0[0]);
        tmem_wait_ld();
#pragma unroll
        for (int g = 0; g < NG; ++g) {
          const int col = j0 + g * 4;
          float xo[4];
          const float* a1 = pa1[g & 1];
          const float* a0 = pa0[g & 1];
          if (g + 1 < NG) {
            tmem_ld4(tlane + (uint32_t)ncol(1, col + 4), pa1[(g + 1) & 1]);
            tmem_ld4(tlane + (uint32_t)ncol(0, col + 4), pa0[(g + 1) & 1]);
          }
          if constexpr (MODE == 2) read_group(g, xo);
          float q1x[4];
#pragma unroll
          for (int e = 0; e < 4; ++e) q1x[e] = __shfl_xor_sync(0xffffffffu, a1[e], 16);
          float2 xn2[2];
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int k = 2 * g + h;  // pair index
            float2 R = __ffma2_rn(sg2, make_float2(q1x[2 * h], q1x[2 * h + 1]),
                                  make_float2(a0[2 * h], a0[2 * h + 1]));
            if constexpr (MODE == 1) {
              R = __fadd2_rn(R, make_float2(2 * k == dpos ? ddxd : 0.f, 2 * k + 1 == dpos ? ddxd : 0.f));
            } else if constexpr (MODE == 2) {
#pragma unroll
              for (int u = 0; u < 2; ++u) {
                const int e = 2 * h + u;
                const float xp = dcomplex ? __shfl_xor_sync(0xffffffffu, xo[e], 16) : 0.f;
                float r = u ? R.y : R.x;
                if (row_ok) {
                  const float2 d = Dm[i * NPS + col + e];
                  r = fmaf(d.x, xo[e], r);
                  if (dcomplex) r = fmaf(sg * d.y, xp, r);
                }
                if (u) R.y = r; else R.x = r;
              }
            }
            if constexpr (BD) {
              const int j = col + 2 * h;
              const float2 r0 = brow[j], r1 = brow[j + 1], a0 = bd->aB[j], a1 = bd->aB[j + 1];
              R.x = fmaf(u0, r0.x, fmaf(u1, r0.y, fmaf(u2, a0.x, fmaf(u3, a0.y, R.x))));
              R.y = fmaf(u0, r1.x, fmaf(u1, r1.y, fmaf(u2, a1.x, fmaf(u3, a1.y, R.y))));
            }
            if constexpr (STAGE == 0) {
              racc2[k] = R;
              xn2[h] = __ffma2_rn(cst2, R, rho2[k]);
            } else if constexpr (STAGE == 1) {
              racc2[k] = __ffma2_rn(make_float2(2.f, 2.f), R, racc2[k]);
              xn2[h] = __ffma2_rn(cst2, R, rho2[k]);
            } else {
              // Kahan-compensated rho += dt/6 (k1 + 2 k2 + 2 k3 + k4)
              const float2 y = __ffma2_rn(make_float2(sixth_dt, sixth_dt), __fadd2_rn(racc2[k], R), nkc2[k]);
              const float2 t = __fadd2_rn(rho2[k], y);
              nkc2[k] = __ffma2_rn(__ffma2_rn(rho2[k], m1, t), m1, y);  // y - (t - rho)
              rho2[k] = t;
              xn2[h] = t;
            }
            if constexpr (MODE == 1) {
              xd = (2 * k == dpos) ? xn2[h].x : xd;
              xd = (2 * k + 1 == dpos) ? xn2[h].y : xd;
            }
            if constexpr (BD) {
              const int j = col + 2 * h;
              const float2 b0 = bd->bB[j], b1 = bd->bB[j + 1];
              tx = fmaf(xn2[h].x, c == 0 ? b0.x : b0.y, tx);
              ty = fmaf(xn2[h].x, c == 0 ? -b0.y : b0.x, ty);
              tx = fmaf(xn2[h].y, c == 0 ? b1.x : b1.y, tx);
              ty = fmaf(xn2[h].y, c == 0 ? -b1.y : b1.x, ty);
            }
          }
          const float x4[4] = {xn2[0].x, xn2[0].y, xn2[1].x, xn2[1].y};
          write_group(g, x4);
          if (STAGE < 3 || p.n_drive == 0) inject(g, x4, ai_row);
          if (g + 1 < NG) tmem_wait_ld();
        }
        tmem_wait_st();
        if constexpr (BD) {
          tx += __shfl_xor_sync(0xffffffffu, tx, 16);
          ty += __shfl_xor_sync(0xffffffffu, ty, 16);
          if (c == 0) bd->t2p[bcur ^ 1][i][cg] = make_float2(tx, ty);
        }
      };
      using S0 = std::integral_constant<int, 0>;
      using S1 = std::integral_constant<int, 1>;
      using S3 = std::integral_constant<int, 3>;
      const int mode = !diag ? 0 : (dfast ? (dwarp ? 1 : 0) : 2);
      auto by_mode = [&](auto stage_tag) {
        if (mode == 0) epilogue(std::integral_constant<int, 0>{}, stage_tag);
        else if (mode == 1) epilogue(std::integral_constant<int, 1>{}, stage_tag);
        else epilogue(std::integral_constant<int, 2>{}, stage_tag);
      };
      if (stage == 0) by_mode(S0{});
      else if (stage < 3) by_mode(S1{});
      else by_mode(S3{});
      bcur ^= 1;
    }
    if (!alive || nonfinite) break;
    pend_row = step + p.obs_t0;
    if (p.store_every > 0 && p.states_out != nullptr && ((step + 1) % p.store_every) == 0 &&
        i < N) {
      const long long si = (step + 1) / p.store_every - 1;
      double2* dst = p.states_out + p.soff[b] + si * (long long)N * N;
#pragma unroll
      for (int jj = 0; jj < NPQ; ++jj) {
        const int j = j0 + jj;
        if (j < N) reinterpret_cast<double*>(dst + (long long)i * N + j)[c] = (double)rho_at(jj);
      }
      if constexpr (BD) {
        if (tid < 2 * kG + 1) {
          const bool col = tid < kG;
          const int t = col ? tid : tid - kG;
          const float2 v = bd->rho[col ? 0 : 1][t];
          dst[col ? (long long)t * N + kG : (long long)kG * N + t] = make_double2(v.x, v.y);
        }
      }
    }
  }

  if (alive && !nonfinite && pend_row >= 0) {
    if (checking) gsync<GR>(grp);  // the last epilogue's X^T writes
    nonfinite = obs_finish(obs_partials(), pend_row);
  }
  if (nonfinite && tid == 0) p.err[b] = 4;  // LGB_ERR_NONFINITE
  if (checking && tid == 0) {
    const int fl = sh.chk_flags[grp];
    p.chk[2 * b] = sh.chk_run[grp][2];
    p.chk[2 * b + 1] = (fl & 1) ? sh.chk_run[grp][3] : -1.0;
    if ((fl & 2) && p.err[b] == 0) p.err[b] = 9;  // LGB_ERR_CHECK
  }
  if (alive && p.rho_out != nullptr && i < N) {
    double2* dst = p.rho_out + p.off[b];
#pragma unroll
    for (int jj = 0; jj < NPQ; ++jj) {
      const int j = j0 + jj;
      if (j < N) reinterpret_cast<double*>(dst + (long long)i * N + j)[c] = (double)rho_at(jj);
    }
    if constexpr (BD) {
      if (tid < 2 * kG + 1) {
        const bool col = tid < kG;
        const int t = col ? tid : tid - kG;
        const float2 v = bd->rho[col ? 0 : 1][t];
        dst[col ? (long long)t * N + kG : (long long)kG * N + t] = make_double2(v.x, v.y);
      }
    }
  }
  // TMEM reads of this instance are done before the next instance's first MMA
  fence_before_sync();
  gsync<GR>(grp);
}

// Shared memory of one group in two-instance mode (NP <= 32), 1 KB aligned.
template <bool BF16>
__host__ __device__ constexpr uint32_t dual_bytes() {
  return (Geo<BF16, 32>::BYTES + 1023u) / 1024u * 1024u;
}

template <bool BF16>
__global__ void __launch_bounds__(kThreads, 1) tc_rk4_kernel(CtaParams p, const int* order,
                                                             int n_items, int* queue) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ TcShared sh;
  const int tid = threadIdx.x;
  if (tid == 0) {
    mbar_init(&sh.mbar[0], 1);
    mbar_init(&sh.mbar[1], 1);
    mbar_fence_init();
  }
  if (tid < 32) {
    tmem_alloc(&sh.tmem_base, kTmemCols);
    tmem_relinquish();
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  uint32_t phase = 0;
  bool alive = true;
  int small = -1;
  // Instances with NP >= 48 (the queue is sorted by size): the whole CTA.
  while (true) {
    if (tid == 0) sh.next[0] = atomicAdd(queue, 1);
    __syncthreads();
    const int item = sh.next[0];
    __syncthreads();
    if (item >= n_items) break;
    const int b = order[item];
    if (!alive) {
      // after a timed-out wait this CTA only marks the instances it takes
      if (tid == 0) p.err[b] = 5;  // LGB_ERR_TIMEOUT
      continue;
    }
    if (p.npad[b] <= 32 && p.tc_pairs) {
      small = item;
      break;
    }
    switch (p.npad[b]) {
      case 16: tc_instance<BF16, 16, 1>(p, b, smem, sh, 0, phase, alive); break;
      case 32: tc_instance<BF16, 32, 1>(p, b, smem, sh, 0, phase, alive); break;
      case 48: tc_instance<BF16, 48, 1>(p, b, smem, sh, 0, phase, alive); break;
      default: tc_instance<BF16, 64, 1>(p, b, smem, sh, 0, phase, alive); break;
    }
  }
  // NP <= 32: the warps of TMEM lane quarters 0-1 and those of quarters 2-3
  // each run their own instances (own shared memory, TMEM columns, mbarrier
  // and named barrier; the second group's M-side operand windows start 64
  // rows early so that its rows land in lanes 64..127), so that one group's
  // MMAs overlap the other's epilogue.
  if (alive && small >= 0) {
    const int g = (tid >> 5 & 3) >> 1;  // TMEM lane quarters 0-1 or 2-3
    unsigned char* sg = smem + g * dual_bytes<BF16>();
    uint32_t ph = g == 0 ? phase : 0u;
    int item = g == 0 ? small : -1;
    bool galive = true;
    while (true) {
      if (item < 0) {
        if ((tid & 0x1bf) == 0) sh.next[g] = atomicAdd(queue, 1);  // warp 0 / 2, lane 0
        gsync<2>(g);
        item = sh.next[g];
        gsync<2>(g);
      }
      if (item >= n_items) break;
      const int b = order[item];
      if (!galive) {
        if ((tid & 0x1bf) == 0) p.err[b] = 5;  // LGB_ERR_TIMEOUT (not propagated)
        item = -1;
        continue;
      }
      if (p.npad[b] == 16) {
        tc_instance<BF16, 16, 2>(p, b, sg, sh, g, ph, galive);
      } else {
        tc_instance<BF16, 32, 2>(p, b, sg, sh, g, ph, galive);
      }
      item = -1;
    }
  }
  fence_before_sync();
  __syncthreads();
  if (tid < 32) tmem_dealloc(sh.tmem_base, kTmemCols);
}

// N = 65 instances (64 x 64 block + SIMT border): one CTA each, a kernel of
// their own so that the border's register pressure stays out of the
// persistent kernel.  Launched ahead of it; the persistent CTAs take the
// remaining SMs from the work queue.
template <bool BF16>
__global__ void __launch_bounds__(kThreads, 1) tc_border_kernel(CtaParams p, const int* order) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ TcShared sh;
  const int tid = threadIdx.x;
  if (tid == 0) {
    mbar_init(&sh.mbar[0], 1);
    mbar_init(&sh.mbar[1], 1);
    mbar_fence_init();
  }
  if (tid < 32) {
    tmem_alloc(&sh.tmem_base, kTmemCols);
    tmem_relinquish();
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  uint32_t phase = 0;
  bool alive = true;
  tc_instance<BF16, 64, 1, true>(p, order[blockIdx.x], smem, sh, 0, phase, alive);
  fence_before_sync();
  __syncthreads();
  if (tid < 32) tmem_dealloc(sh.tmem_base, kTmemCols);
}

}  // namespace

int tc_max_dim() { return 64; }
int tc_border_dim() { return 65; }

int tc_smem_bytes(int precision, int npad) {
  const bool bf16 = precision == LGB_PREC_BF16X3;
  // instances of at most npad: one at a time for NP >= 48, two for NP <= 32
  const int dual = bf16 ? 2 * (int)dual_bytes<true>() : 2 * (int)dual_bytes<false>();
  switch (npad) {
    case 16:
    case 32: return dual;
    case 48: return std::max(dual, bf16 ? (int)Geo<true, 48>::BYTES : (int)Geo<false, 48>::BYTES);
    case kTcBorderNpad:
      return std::max(dual, (bf16 ? (int)Geo<true, 64>::BYTES : (int)Geo<false, 64>::BYTES) +
                                (int)sizeof(TcBorder));
    default: return std::max(dual, bf16 ? (int)Geo<true, 64>::BYTES : (int)Geo<false, 64>::BYTES);
  }
}

cudaError_t launch_tc_border(const CtaParams& p, int precision, const int* order, int n_items,
                             cudaStream_t stream) {
  if (n_items <= 0) return cudaSuccess;
  cudaError_t e;
  if (precision == LGB_PREC_BF16X3) {
    e = cudaFuncSetAttribute(tc_border_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, p.smem_bytes);
    if (e != cudaSuccess) return e;
    tc_border_kernel<true><<<n_items, kThreads, p.smem_bytes, stream>>>(p, order);
  } else {
    e = cudaFuncSetAttribute(tc_border_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, p.smem_bytes);
    if (e != cudaSuccess) return e;
    tc_border_kernel<false><<<n_items, kThreads, p.smem_bytes, stream>>>(p, order);
  }
  return cudaGetLastError();
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
