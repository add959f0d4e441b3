// Split-precision (3xTF32 / 3xBF16) GEMM schedule for large instances on the
// 5th-generation tensor cores: the same per-stage structure as the FP32/FP64
// schedule (lgb_gemm.cu; pyqed/oqs.py:697-715 rewritten as
//     G1  T_k = L_k X,   G2  R = [A | X | T_1..T_K] . [X ; A^dag ; L_1^dag ; ..],
// then the RK4 stage combination of pyqed/phys.py:1051-1064), with G1 and G2
// run by a hand-written TMA-fed tcgen05 GEMM.
//
// Complex GEMM C = P Q in the interleaved real form of the instance kernel
// (lgb_tc.cu): the M-side operand holds the rows of P as
//     M row (c, i) = 32 (i / 16) + 16 c + i % 16      (c = 0 real, 1 imaginary part)
// and the N-side operand the rows of Q^T as
//     N row (p, j) = 32 (j / 16) + 16 (1 - p) + j % 16,
// both K-major, each split into a hi and a lo array (TF32 or BF16).  One real
// MMA of M = 128, N = 256 then accumulates D[(c,i)][(p,j)] = (P_c Q_p)[i][j]
// for a 64 x 128 complex tile, and
//     Re C = D[(0,i)][(0,j)] - D[(1,i)][(1,j)],   Im C = D[(1,i)][(0,j)] + D[(0,i)][(1,j)]
// with the two lanes of row i 16 apart in one TMEM quarter (one shuffle).
// Every K-step issues the three leading split products hi*hi, hi*lo, lo*hi.
//
// Pipeline (one CTA of 128 threads per tile, one tile per SM at a time):
// thread 0 issues the TMA loads of 4-stage ring buffers (hi and lo of both
// operands; one 2D load per operand tile of 64 bytes of K per row, written
// with the 64-byte swizzle that the MMA descriptors name, so each row is one
// contiguous 64-byte read), thread 32 issues the MMAs and commits each stage back to
// the producer, and all four warps run the epilogue (TMEM -> registers ->
// partner combination -> shared-memory staging -> coalesced FP32 complex
// stores).  Large-K products can be split over CTAs (split-K); the consumer
// kernels add the partial tiles.  Every mbarrier wait is bounded and a wait
// that runs out sets LGB_ERR_TIMEOUT.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>

#include "lgb_common.cuh"
#include "lgb_internal.h"
#include "lgb_split.cuh"
#include "lgb_umma.cuh"

namespace lgb {

namespace {

using namespace umma;
using namespace splitk;

constexpr int kGThreads = 128;
constexpr int kStages = 4;
constexpr int kPRows = 128;                // M-side rows per tile (64 complex rows)
constexpr int kQRows = 256;                // N-side rows per tile (128 complex columns)
constexpr uint32_t kPBytes = kPRows * kRowBytes;  // one level of P per stage
constexpr uint32_t kQBytes = kQRows * kRowBytes;
constexpr uint32_t kStageBytes = 2 * kPBytes + 2 * kQBytes;
constexpr uint32_t kGemmSmem = kStages * kStageBytes;  // 192 KB
constexpr int kStagePitch = 129;                       // float2 per staged output row

struct CgArgs {
  int p_row0 = 0, p_batch_rows = 0;  // M-side: first row of this product, rows per batch
  int q_row0 = 0, q_batch_rows = 0;  // N-side
  int k0 = 0, klen = 0, ksplit = 1;  // K range of one split (multiple of the stage depth)
  float2* out = nullptr;             // complex FP32 output tiles
  long long out_ld = 0, out_batch = 0, out_split = 0;
  int* err = nullptr;
};

// C (+ split partials) = P Q for one 64 x 128 complex tile per CTA.
template <bool BF16>
__global__ void __launch_bounds__(kGThreads, 1)
    cgemm3_kernel(const __grid_constant__ CUtensorMap mPh, const __grid_constant__ CUtensorMap mPl,
                  const __grid_constant__ CUtensorMap mQh, const __grid_constant__ CUtensorMap mQl,
                  CgArgs a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t full[kStages], empty[kStages], done;
  __shared__ uint32_t tmem_base;
  __shared__ int bail;
  constexpr int KT = kRowBytes / (BF16 ? 2 : 4);  // K elements per stage
  constexpr int KSTEPS = KT / (BF16 ? 16 : 8);     // 32-byte MMA K-steps
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int batch = blockIdx.z / a.ksplit, kz = blockIdx.z % a.ksplit;
  const int prow = a.p_row0 + batch * a.p_batch_rows + blockIdx.y * kPRows;
  const int qrow = a.q_row0 + batch * a.q_batch_rows + blockIdx.x * kQRows;
  const int kbeg = a.k0 + kz * a.klen;
  const int nkb = a.klen / KT;
  const uint32_t sbase = smem_u32(smem);

  // after a timed-out wait anywhere in this instance, later launches return at once
  if (tid == 0) bail = *reinterpret_cast<volatile int*>(a.err) == 5;
  __syncthreads();
  if (bail) return;
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&done, 1);
    mbar_fence_init();
  }
  if (warp == 0) {
    tmem_alloc(&tmem_base, 256);
    tmem_relinquish();
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = tmem_base;
  bool ok = true;

  if (tid == 0) {
    // ---- producer ---------------------------------------------------------------
    for (int kb = 0; kb < nkb && ok; ++kb) {
      const int s = kb % kStages;
      const uint32_t par = ((kb / kStages) & 1) ^ 1;
      if (!mbar_wait(&empty[s], par, kGemmSpin)) {
        ok = false;
        break;
      }
      mbar_expect_tx(&full[s], kStageBytes);
      const uint32_t st = sbase + s * kStageBytes;
      const int x = kbeg + kb * KT;
      tma_load_2d(st, &mPh, x, prow, &full[s]);
      tma_load_2d(st + kPBytes, &mPl, x, prow, &full[s]);
      tma_load_2d(st + 2 * kPBytes, &mQh, x, qrow, &full[s]);
      tma_load_2d(st + 2 * kPBytes + kQBytes, &mQl, x, qrow, &full[s]);
    }
    if (!ok) atomicExch(a.err, 5);  // LGB_ERR_TIMEOUT
  } else if (tid == 32) {
    // ---- MMA issuer -----------------------------------------------------------------
    constexpr uint32_t id = idesc(BF16 ? kFmtBF16 : kFmtTF32, 128, 256, false, false);
    for (int kb = 0; kb < nkb && ok; ++kb) {
      const int s = kb % kStages;
      if (!mbar_wait(&full[s], (kb / kStages) & 1, kGemmSpin)) {
        ok = false;
        break;
      }
      fence_after_sync();
      const uint32_t st = sbase + s * kStageBytes;
#pragma unroll
      for (int ks = 0; ks < KSTEPS; ++ks) {
        // K-step ks = bytes 32 ks .. 32 ks + 31 of every row (inside the atom)
        const uint64_t ph = sdesc_sw64(st + 32 * ks);
        const uint64_t pl = sdesc_sw64(st + kPBytes + 32 * ks);
        const uint64_t qh = sdesc_sw64(st + 2 * kPBytes + 32 * ks);
        const uint64_t ql = sdesc_sw64(st + 2 * kPBytes + kQBytes + 32 * ks);
        mma_k<BF16>(tmem, ph, qh, id, (kb > 0 || ks > 0) ? 1u : 0u);
        mma_k<BF16>(tmem, ph, ql, id, 1u);
        mma_k<BF16>(tmem, pl, qh, id, 1u);
      }
      mma_commit(&empty[s]);  // stage s is free once these MMAs completed
    }
    mma_commit(&done);
    if (!ok) atomicExch(a.err, 5);
  }
  __syncwarp();
  // ---- epilogue -----------------------------------------------------------------------
  const bool fin = mbar_wait(&done, 0, kGemmSpin);
  const bool all = __syncthreads_and(fin) != 0;
  fence_after_sync();
  float2* stage = reinterpret_cast<float2*>(smem);  // [64][kStagePitch] complex, after the mainloop
  if (all) {
    const int c = lane >> 4;
    const int i = warp * 16 + (lane & 15);  // complex row within the tile
    const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);
    const float sg = c == 0 ? -1.f : 1.f;
#pragma unroll 1
    for (int h = 0; h < 8; ++h) {
      float p1[16], p0[16];
      tmem_ld16(tl + 32 * h, p1);
      tmem_ld16(tl + 32 * h + 16, p0);
      tmem_wait_ld();
#pragma unroll
      for (int e = 0; e < 16; ++e) {
        const float x = __shfl_xor_sync(0xffffffffu, p1[e], 16);
        reinterpret_cast<float*>(stage + i * kStagePitch + 16 * h + e)[c] = fmaf(sg, x, p0[e]);
      }
    }
  } else if (tid == 0) {
    atomicExch(a.err, 5);
  }
  __syncthreads();
  if (all) {
    float2* out = a.out + batch * a.out_batch + kz * a.out_split +
                  (long long)(blockIdx.y * 64) * a.out_ld + blockIdx.x * 128;
    for (int r = 0; r < 64; ++r) out[(long long)r * a.out_ld + tid] = stage[r * kStagePitch + tid];
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, 256);
}

// ---- split conversions ------------------------------------------------------------------
// Row block: dst row mrow(c, i), column coff + j  <-  component c of src[i][j]
// (batched: blockIdx.y = batch).
template <bool BF16>
__global__ void split_rows_kernel(const float2* src, long long src_ld, long long src_batch, int rows,
                                  int cols, void* dh, void* dl, long long pitch, long long dst_batch,
                                  long long coff) {
  using T = typename SElem<BF16>::T;
  const float2* s = src + blockIdx.y * src_batch;
  T* H = reinterpret_cast<T*>(dh) + blockIdx.y * dst_batch;
  T* L = reinterpret_cast<T*>(dl) + blockIdx.y * dst_batch;
  const long long n = (long long)rows * cols;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(idx / cols), j = (int)(idx % cols);
    const float2 v = s[(long long)i * src_ld + j];
    T h, l;
    SElem<BF16>::split(v.x, h, l);
    H[(long long)mrow(0, i) * pitch + coff + j] = h;
    L[(long long)mrow(0, i) * pitch + coff + j] = l;
    SElem<BF16>::split(v.y, h, l);
    H[(long long)mrow(1, i) * pitch + coff + j] = h;
    L[(long long)mrow(1, i) * pitch + coff + j] = l;
  }
}

// Transposed block: dst row ncol(p, j), column coff + k  <-  component p of
// src[k][j]; 32 x 32 tiles through shared memory, coalesced both ways.
template <bool BF16>
__global__ void split_trans_kernel(const float2* src, long long src_ld, int rows, int cols, void* dh,
                                   void* dl, long long pitch, long long coff) {
  using T = typename SElem<BF16>::T;
  __shared__ float2 tile[32][33];
  const int k0 = blockIdx.y * 32, j0 = blockIdx.x * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (int r = ty; r < 32; r += 8) {
    const int k = k0 + r, j = j0 + tx;
    tile[r][tx] = (k < rows && j < cols) ? src[(long long)k * src_ld + j] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  T* H = reinterpret_cast<T*>(dh);
  T* L = reinterpret_cast<T*>(dl);
  for (int r = ty; r < 32; r += 8) {
    const int j = j0 + r, k = k0 + tx;
    if (j >= cols || k >= rows) continue;
    const float2 v = tile[tx][r];
    T h, l;
    SElem<BF16>::split(v.x, h, l);
    H[(long long)ncol(0, j) * pitch + coff + k] = h;
    L[(long long)ncol(0, j) * pitch + coff + k] = l;
    SElem<BF16>::split(v.y, h, l);
    H[(long long)ncol(1, j) * pitch + coff + k] = h;
    L[(long long)ncol(1, j) * pitch + coff + k] = l;
  }
}

// G1 consumer: T_k = sum of the split partials -> M-side block 2 + k of G2.
template <bool BF16>
__global__ void tsum_split_kernel(const float2* part, int ksplit, long long split_stride, int Kd,
                                  int N, int NP, void* dh, void* dl, long long pitch) {
  using T = typename SElem<BF16>::T;
  const long long n = (long long)Kd * N * N;
  T* H = reinterpret_cast<T*>(dh);
  T* L = reinterpret_cast<T*>(dl);
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(idx / ((long long)N * N));
    const long long rem = idx % ((long long)N * N);
    const int i = (int)(rem / N), j = (int)(rem % N);
    const long long src = (long long)k * NP * NP + (long long)i * NP + j;
    float2 v = part[src];
    for (int z = 1; z < ksplit; ++z) {
      const float2 w = part[z * split_stride + src];
      v.x += w.x;
      v.y += w.y;
    }
    const long long col = (long long)(2 + k) * NP + j;
    T h, l;
    SElem<BF16>::split(v.x, h, l);
    H[(long long)mrow(0, i) * pitch + col] = h;
    L[(long long)mrow(0, i) * pitch + col] = l;
    SElem<BF16>::split(v.y, h, l);
    H[(long long)mrow(1, i) * pitch + col] = h;
    L[(long long)mrow(1, i) * pitch + col] = l;
  }
}

// Deterministic FP64 reduction of per-block observable partials (last block sums).
__device__ void finish_obs_split(const GemmInstance& g, const double2* blk, int E, double2* obs_out,
                                 long long row, int nblocks) {
  __shared__ bool last;
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    for (int e = 0; e < E; ++e) g.partial[(long long)e * nblocks + blockIdx.x] = blk[e];
    __threadfence();
    last = atomicAdd(g.counter, 1) == nblocks - 1;
  }
  __syncthreads();
  if (last) {
    __threadfence();
    const int t = threadIdx.y * 32 + threadIdx.x;
    if (t < E) {
      double2 s = make_double2(0.0, 0.0);
      const double2* pp = g.partial + (long long)t * nblocks;
      for (int q = 0; q < nblocks; ++q) {
        const volatile double* vp = reinterpret_cast<const volatile double*>(pp + q);
        s.x += vp[0];
        s.y += vp[1];
      }
      if (obs_out != nullptr) obs_out[row * E + t] = s;
    }
    if (t == 0) *g.counter = 0;
  }
}

// RK4 stage epilogue of the split schedule on 32 x 32 tiles (blockIdx.x =
// tile): R = sum of the G2 split partials (+ D o X), RK4 combination in FP32
// (Kahan-compensated final update), next stage input X into the FP32 slab
// (Rbuf block 0), the M-side block 1 (rows) and the N-side block 0
// (transposed) of the split operands; observables after stage 3.
template <bool BF16>
__global__ void __launch_bounds__(256) split_epilogue_kernel(GemmInstance g, GemmSplit sp, int stage,
                                                             double dt, int diag, int E,
                                                             double2* obs_out, StepOut so) {
  using T = typename SElem<BF16>::T;
  __shared__ float2 xt[32][33];
  __shared__ double red[8][16][2];
  __shared__ double2 blk[16];
  const int N = g.N, NP = sp.NP;
  const int tiles = (N + 31) / 32;
  const int i0 = (blockIdx.x / tiles) * 32, j0 = (blockIdx.x % tiles) * 32;
  const int step = *so.ctr;
  const long long row = (long long)step + so.obs_t0;
  double2* state_out = stage == 3 ? so.state_at(step, (long long)N * N) : nullptr;
  double2* rho_out = (stage == 3 && step == so.nt - 1) ? so.rho_out : nullptr;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const float cst = (float)((stage == 2) ? dt : 0.5 * dt);
  const float sixth = (float)(dt / 6.0);
  float2* rho = reinterpret_cast<float2*>(g.rho);
  float2* racc = reinterpret_cast<float2*>(g.racc);
  float2* Xf = reinterpret_cast<float2*>(g.Rbuf);  // block 0: X (N x N, ld N)
  float2* kcm = sp.kc;
  const long long NN = (long long)NP * NP;
  double ox[16], oy[16];
#pragma unroll
  for (int e = 0; e < 16; ++e) ox[e] = oy[e] = 0.0;
  bool fin = true;
  T* LH = reinterpret_cast<T*>(sp.Ls[0]);
  T* LL = reinterpret_cast<T*>(sp.Ls[1]);
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + r, j = j0 + tx;
    float2 xn = make_float2(0.f, 0.f);
    if (i < N && j < N) {
      const long long e2 = (long long)i * NP + j;
      float2 R = sp.Rpart[e2];
      for (int z = 1; z < sp.ks2; ++z) {
        const float2 w = sp.Rpart[z * NN + e2];
        R.x += w.x;
        R.y += w.y;
      }
      const long long idx = (long long)i * N + j;
      if (diag) cmac(R, reinterpret_cast<const float2*>(g.Dm)[idx], Xf[idx]);
      float2 rr = rho[idx];
      float2 ra = racc[idx];
      if (stage == 0) {
        ra = R;
        xn = caxpy(rr, cst, R);
      } else if (stage < 3) {
        ra = caxpy(ra, 2.f, R);
        xn = caxpy(rr, cst, R);
      } else {
        // Kahan-compensated rho += dt/6 (k1 + 2 k2 + 2 k3 + k4)
        const float2 kc = kcm[idx];
        const float yx = fmaf(sixth, ra.x + R.x, -kc.x), yy = fmaf(sixth, ra.y + R.y, -kc.y);
        const float tx_ = rr.x + yx, ty_ = rr.y + yy;
        kcm[idx] = make_float2((tx_ - rr.x) - yx, (ty_ - rr.y) - yy);
        rr = make_float2(tx_, ty_);
        rho[idx] = rr;
        xn = rr;
        fin = fin && isfinite(rr.x) && isfinite(rr.y);
        const double2 rd = make_double2(rr.x, rr.y);
        for (int e = 0; e < E && e < 16; ++e) {
          const double2 o = g.Ot[(long long)e * N * N + idx];
          ox[e] += o.x * rd.x - o.y * rd.y;
          oy[e] += o.x * rd.y + o.y * rd.x;
        }
        if (state_out != nullptr) state_out[idx] = rd;
        if (rho_out != nullptr) rho_out[idx] = rd;
      }
      if (stage < 3) racc[idx] = ra;
      Xf[idx] = xn;
      // M-side block 1 of G2: rows (c, i), column NP + j
      const long long col = (long long)NP + j;
      T h, l;
      SElem<BF16>::split(xn.x, h, l);
      LH[(long long)mrow(0, i) * sp.Wp + col] = h;
      LL[(long long)mrow(0, i) * sp.Wp + col] = l;
      SElem<BF16>::split(xn.y, h, l);
      LH[(long long)mrow(1, i) * sp.Wp + col] = h;
      LL[(long long)mrow(1, i) * sp.Wp + col] = l;
    }
    xt[r][tx] = xn;
  }
  __syncthreads();
  // N-side block 0 (X^T): row (p, j), column i
  T* RH = reinterpret_cast<T*>(sp.Rs[0]);
  T* RL = reinterpret_cast<T*>(sp.Rs[1]);
  for (int r = ty; r < 32; r += 8) {
    const int j = j0 + r, i = i0 + tx;
    if (i >= N || j >= N) continue;
    const float2 v = xt[tx][r];
    T h, l;
    SElem<BF16>::split(v.x, h, l);
    RH[(long long)ncol(0, j) * sp.Wp + i] = h;
    RL[(long long)ncol(0, j) * sp.Wp + i] = l;
    SElem<BF16>::split(v.y, h, l);
    RH[(long long)ncol(1, j) * sp.Wp + i] = h;
    RL[(long long)ncol(1, j) * sp.Wp + i] = l;
  }
  if (stage == 3) {
    const int t = ty * 32 + tx;
    const bool bad = __syncthreads_or(!fin) != 0;
    if (bad && t == 0) *g.err = 4;  // LGB_ERR_NONFINITE
    for (int e = 0; e < E && e < 16; ++e) {
      double sx = ox[e], sy = oy[e];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, o);
        sy += __shfl_xor_sync(0xffffffffu, sy, o);
      }
      if (tx == 0) {
        red[ty][e][0] = sx;
        red[ty][e][1] = sy;
      }
    }
    __syncthreads();
    if (t < E) {
      double sx = 0.0, sy = 0.0;
      for (int w = 0; w < 8; ++w) {
        sx += red[w][t][0];
        sy += red[w][t][1];
      }
      blk[t] = make_double2(sx, sy);
    }
    __syncthreads();
    if (E > 0) finish_obs_split(g, blk, E, obs_out, row, gridDim.x);
  }
}

// ---- tensor maps ---------------------------------------------------------------------------
using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*,
                              CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                              CUtensorMapFloatOOBfill);

EncodeFn encode_fn() {
  static EncodeFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeFn>(p);
  });
  return fn;
}

// 2D map over a K-major split array (rows x pitch elements), box = 64 bytes x
// box_rows, 64-byte swizzle.
bool make_map(CUtensorMap* m, void* base, bool bf16, long long rows, long long pitch, int box_rows) {
  EncodeFn fn = encode_fn();
  if (fn == nullptr) return false;
  const int esz = bf16 ? 2 : 4;
  cuuint64_t dims[2] = {(cuuint64_t)pitch, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(pitch * esz)};
  cuuint32_t box[2] = {(cuuint32_t)(kRowBytes / esz), (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  return fn(m, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base,
            dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// K-dimension split: the number of parts (dividing the stage count) that
// brings the grid closest to the SM count without exceeding it much.
int choose_ksplit(int tiles, int kblocks, int n_sm, int cap = 0) {
  int best = 1;
  const int smax = cap > 0 ? std::min(cap, 64) : 64;
  for (int s = 1; s <= kblocks && s <= smax; ++s) {
    if (kblocks % s) continue;
    if ((long long)tiles * s <= n_sm) best = s;
  }
  return best;
}

// (the kernel's shared-memory attribute is set once in split_setup, outside
// any stream capture)
template <bool BF16>
cudaError_t launch_cgemm(const CUtensorMap* maps, const CgArgs& a, int ntile_n, int ntile_m, int nz,
                         cudaStream_t st) {
  cgemm3_kernel<BF16><<<dim3(ntile_n, ntile_m, nz), kGThreads, kGemmSmem, st>>>(maps[0], maps[1], maps[2],
                                                                               maps[3], a);
  return cudaGetLastError();
}

template <bool BF16>
int split_propagate_t(const GemmRunArgs& a, cudaStream_t st) {
  const GemmInstance& g = a.g;
  const GemmSplit& sp = a.sp;
  const int N = g.N, NP = sp.NP, K = a.Kdense;
  const long long NN = (long long)N * N;
  const int grid = (int)std::min<long long>((NN + 255) / 256, 4096);
  const int tiles = (N + 31) / 32;
  const int KT = kRowBytes / (BF16 ? 2 : 4);
  cudaError_t e = cudaSuccess;
  // initial state: FP32 rho, RK4 sum, X in the FP32 slabs, then the split X blocks
  gemm_init_split(g, a.rho0, st);
  cudaMemsetAsync(sp.kc, 0, NN * sizeof(float2), st);
  split_rows_kernel<BF16><<<dim3(grid, 1), 256, 0, st>>>(reinterpret_cast<const float2*>(g.Rbuf), N, 0, N,
                                                         N, sp.Ls[0], sp.Ls[1], sp.Wp, 0, NP);
  split_trans_kernel<BF16><<<dim3(tiles, tiles), dim3(32, 8), 0, st>>>(
      reinterpret_cast<const float2*>(g.Rbuf), N, N, N, sp.Rs[0], sp.Rs[1], sp.Wp, 0);
  const bool check = a.check_tol > 0.0 && a.chk != nullptr;
  if (check) gemm_check(a, false, true, st);
  if (a.obs_t0 && a.E > 0) gemm_obs_split(g, a.E, a.obs_out, st);
  if (cudaMemsetAsync(a.ctr, 0, sizeof(int), st) != cudaSuccess) return LGB_ERR_CUDA;
  if ((e = cudaGetLastError()) != cudaSuccess) return LGB_ERR_CUDA;
  if (a.persist && sp.persist && a.D == 0 && a.nt > 0) {
    // one persistent launch (after converting the operands into its blocked layout)
    const int r = persist_propagate(a, st);
    if (r != LGB_ERR_UNSUPPORTED) return r;
  }
  // G1: T_k = L_k X, batched over k; G2: R = Ls . Rs^T
  CgArgs g1, g2;
  g1.p_row0 = 0;
  g1.p_batch_rows = 2 * NP;
  g1.q_row0 = 0;
  g1.q_batch_rows = 0;
  g1.k0 = 0;
  g1.ksplit = sp.ks1;
  g1.klen = NP / sp.ks1;
  g1.out = sp.Tpart;
  g1.out_ld = NP;
  g1.out_batch = (long long)NP * NP;
  g1.out_split = (long long)K * NP * NP;
  g1.err = g.err;
  g2.p_row0 = 0;
  g2.q_row0 = 0;
  g2.k0 = 0;
  g2.ksplit = sp.ks2;
  g2.klen = (int)(sp.Wp / sp.ks2);
  g2.out = sp.Rpart;
  g2.out_ld = NP;
  g2.out_split = (long long)NP * NP;
  g2.err = g.err;
  if (g1.klen % KT || g2.klen % KT) return LGB_ERR_INVALID_ARG;
  StepOut so;
  so.ctr = a.ctr;
  so.obs_t0 = a.obs_t0;
  so.nt = a.nt;
  so.store_every = a.store_every;
  so.states_out = a.states_out;
  so.rho_out = a.rho_out;
  auto one_step = [&](cudaStream_t s) -> int {
    if (a.D > 0) {
      gemm_drive_split(g, a.D, a.drive, a.nt, a.ctr, s);
      // A -> M-side block 0 (rows); A^dag -> N-side block 1 (transposed)
      split_rows_kernel<BF16><<<dim3(grid, 1), 256, 0, s>>>(reinterpret_cast<const float2*>(g.Lbuf), g.W,
                                                            0, N, N, sp.Ls[0], sp.Ls[1], sp.Wp, 0, 0);
      split_trans_kernel<BF16><<<dim3(tiles, tiles), dim3(32, 8), 0, s>>>(
          reinterpret_cast<const float2*>(g.Rbuf) + NN, N, N, N, sp.Rs[0], sp.Rs[1], sp.Wp, NP);
    }
    for (int stage = 0; stage < 4; ++stage) {
      if (K > 0) {
        if (launch_cgemm<BF16>(sp.map_g1, g1, NP / 128, NP / 64, K * sp.ks1, s) != cudaSuccess)
          return LGB_ERR_CUDA;
        tsum_split_kernel<BF16><<<(int)std::min<long long>((K * NN + 255) / 256, 8192), 256, 0, s>>>(
            sp.Tpart, sp.ks1, (long long)K * NP * NP, K, N, NP, sp.Ls[0], sp.Ls[1], sp.Wp);
      }
      if (launch_cgemm<BF16>(sp.map_g2, g2, NP / 128, NP / 64, sp.ks2, s) != cudaSuccess)
        return LGB_ERR_CUDA;
      split_epilogue_kernel<BF16><<<tiles * tiles, dim3(32, 8), 0, s>>>(g, sp, stage, a.dt, a.diag, a.E,
                                                                        a.obs_out, so);
    }
    if (check) gemm_check(a, false, false, s);
    gemm_step_inc(a.ctr, s);
    return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
  };
  const int r = run_steps(a.nt, st, a.cap, one_step, a.graph_steps);
  if (r != LGB_OK) return r;
  if (a.nt == 0 && a.rho_out != nullptr)
    cudaMemcpyAsync(a.rho_out, a.rho0, NN * sizeof(double2), cudaMemcpyDeviceToDevice, st);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

}  // namespace

int split_padded_dim(int N) { return (N + 127) / 128 * 128; }

size_t split_partial_slots(int N) {
  const size_t t = (size_t)((N + 31) / 32);
  return t * t;
}

int split_setup(GemmSplit& sp, const GemmInstance& g, int Kd, bool bf16, int n_sm, cudaStream_t st) {
  const int N = g.N, NP = sp.NP;
  const int tiles = (N + 31) / 32;
  const int grid = (int)std::min<long long>(((long long)N * N + 255) / 256, 4096);
  const long long NN = (long long)N * N;
  // zero padding everywhere, then the static blocks
  const size_t esz = bf16 ? 2 : 4;
  for (int l = 0; l < 2; ++l) {
    if (cudaMemsetAsync(sp.Ls[l], 0, (size_t)2 * NP * sp.Wp * esz, st) != cudaSuccess) return LGB_ERR_CUDA;
    if (cudaMemsetAsync(sp.Rs[l], 0, (size_t)2 * NP * sp.Wp * esz, st) != cudaSuccess) return LGB_ERR_CUDA;
    if (Kd > 0 && cudaMemsetAsync(sp.Lks[l], 0, (size_t)Kd * 2 * NP * NP * esz, st) != cudaSuccess)
      return LGB_ERR_CUDA;
  }
  const float2* Lb = reinterpret_cast<const float2*>(g.Lbuf);
  const float2* Rb = reinterpret_cast<const float2*>(g.Rbuf);
  for (int blk = 1; blk < Kd + 2; ++blk) {
    // N-side blocks 1 .. Kd+1 (A^dag, L_k^dag) from the FP32 right slab
    if (bf16)
      split_trans_kernel<true><<<dim3(tiles, tiles), dim3(32, 8), 0, st>>>(Rb + blk * NN, N, N, N, sp.Rs[0],
                                                                        sp.Rs[1], sp.Wp, (long long)blk * NP);
    else
      split_trans_kernel<false><<<dim3(tiles, tiles), dim3(32, 8), 0, st>>>(Rb + blk * NN, N, N, N, sp.Rs[0],
                                                                         sp.Rs[1], sp.Wp, (long long)blk * NP);
  }
  // M-side block 0 (A)
  if (bf16)
    split_rows_kernel<true><<<dim3(grid, 1), 256, 0, st>>>(Lb, g.W, 0, N, N, sp.Ls[0], sp.Ls[1], sp.Wp, 0, 0);
  else
    split_rows_kernel<false><<<dim3(grid, 1), 256, 0, st>>>(Lb, g.W, 0, N, N, sp.Ls[0], sp.Ls[1], sp.Wp, 0, 0);
  // G1 M side: L_k rows
  if (Kd > 0) {
    if (bf16)
      split_rows_kernel<true><<<dim3(grid, Kd), 256, 0, st>>>(reinterpret_cast<const float2*>(g.Lstk), N, NN, N,
                                                              N, sp.Lks[0], sp.Lks[1], NP,
                                                              (long long)2 * NP * NP, 0);
    else
      split_rows_kernel<false><<<dim3(grid, Kd), 256, 0, st>>>(reinterpret_cast<const float2*>(g.Lstk), N, NN,
                                                               N, N, sp.Lks[0], sp.Lks[1], NP,
                                                               (long long)2 * NP * NP, 0);
  }
  if (cudaGetLastError() != cudaSuccess) return LGB_ERR_CUDA;
  // tensor maps: G2 (Ls rows 2NP x Wp, Rs rows 2NP x Wp), G1 (Lks rows Kd 2NP x NP, Rs)
  bool ok = make_map(&sp.map_g2[0], sp.Ls[0], bf16, 2LL * NP, sp.Wp, kPRows) &&
            make_map(&sp.map_g2[1], sp.Ls[1], bf16, 2LL * NP, sp.Wp, kPRows) &&
            make_map(&sp.map_g2[2], sp.Rs[0], bf16, 2LL * NP, sp.Wp, kQRows) &&
            make_map(&sp.map_g2[3], sp.Rs[1], bf16, 2LL * NP, sp.Wp, kQRows);
  if (ok && Kd > 0)
    ok = make_map(&sp.map_g1[0], sp.Lks[0], bf16, (long long)Kd * 2 * NP, NP, kPRows) &&
         make_map(&sp.map_g1[1], sp.Lks[1], bf16, (long long)Kd * 2 * NP, NP, kPRows) &&
         make_map(&sp.map_g1[2], sp.Rs[0], bf16, 2LL * NP, sp.Wp, kQRows) &&
         make_map(&sp.map_g1[3], sp.Rs[1], bf16, 2LL * NP, sp.Wp, kQRows);
  if (!ok) return LGB_ERR_UNSUPPORTED;
  // persistent kernel: blocked operands allocated and its clusters co-resident
  sp.persist = sp.Lsb[0] != nullptr && persist_supported(NP, bf16);
  split_set_ksplit(sp, Kd, n_sm);
  const cudaError_t e = bf16 ? cudaFuncSetAttribute(cgemm3_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    (int)kGemmSmem)
                             : cudaFuncSetAttribute(cgemm3_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    (int)kGemmSmem);
  return e == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

void split_set_ksplit(GemmSplit& sp, int Kd, int cta_budget, int cap) {
  // (a cap only lowers the factors, so the partial-tile buffers sized for the
  // largest budget stay large enough)
  const int KT = kRowBytes / (sp.bf16 ? 2 : 4);
  const int t2 = (sp.NP / 128) * (sp.NP / 64);
  sp.ks2 = choose_ksplit(t2, (int)(sp.Wp / KT), cta_budget, cap);
  sp.ks1 = Kd > 0 ? choose_ksplit(t2 * Kd, sp.NP / KT, cta_budget, cap) : 1;
}

size_t split_tpart_elems(int NP, int Kd, int n_sm, bool bf16) {
  // upper bound of ks1 * Kd * NP^2 (ks1 <= n_sm / tiles)
  const int KT = kRowBytes / (bf16 ? 2 : 4);
  const int t = (NP / 128) * (NP / 64) * std::max(Kd, 1);
  const int ks = choose_ksplit(t, NP / KT, n_sm);
  return (size_t)ks * std::max(Kd, 1) * NP * NP;
}
size_t split_rpart_elems(int NP, int Kd, int n_sm, bool bf16) {
  const int KT = kRowBytes / (bf16 ? 2 : 4);
  const int t = (NP / 128) * (NP / 64);
  const int ks = choose_ksplit(t, (Kd + 2) * NP / KT, n_sm);
  return (size_t)ks * NP * NP;
}

int split_propagate(const GemmRunArgs& a, cudaStream_t st) {
  return a.sp.bf16 ? split_propagate_t<true>(a, st) : split_propagate_t<false>(a, st);
}

}  // namespace lgb
