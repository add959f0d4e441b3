// Persistent split-precision (3xTF32 / 3xBF16) schedule for one instance of
// 64 < N <= 256 (padded NP = 128 or 256): the whole propagation in one launch.
//
// The graph-replayed schedule (lgb_gemm_tc.cu) spends a launch per GEMM,
// split-K sum and epilogue, 17 per RK4 step; at NP = 256 those dependent
// launches, not the tensor pipe, set its speed.  Here the same products of
// pyqed/oqs.py:697-715,
//     G1  T_k = L_k X,      G2  R = [A | X | T_1..T_K] . [X ; A^dag ; L_1^dag ; ..],
// and the RK4 combination of pyqed/phys.py:1051-1064 run as two phases per
// stage separated by grid-wide barriers (8 per step):
//
// * The grid is one cluster of 4 CTAs per 64 x 32 complex tile of R
//   ((NP/64)(NP/32) clusters, 128 CTAs at NP = 256, one CTA per SM; clusters
//   of 4 because a GB300 holds 15 clusters of 8 such CTAs, 36 of 4).  Every
//   work item is an M = 128, N = 64 tcgen05 product (64 x 32 complex, the
//   interleaved real form of lgb_tc.cu) over a K range, fed by a 4-stage
//   ring of bulk copies from the blocked operand layout below (thread 0) and
//   issued by one thread (thread 32) as the three leading split products
//   hi*hi, hi*lo, lo*hi.
// * G2: the 4 CTAs of a cluster split its tile's K extent (K + 2) NP four
//   ways; G1: they take the K products of the tile position, each split
//   s1 = 4 / K ways (rounded down to a power of two).  The split partials
//   are summed through distributed shared memory: every CTA stores its
//   combined rows (FP32) into the receive buffer of the CTA that owns them,
//   one hardware cluster barrier, and the owner adds the sources in a fixed
//   order (deterministic; no partial tiles in global memory, no extra phase).
// * The owner of rows [16r, 16r + 16) of the G2 tile keeps rho, the RK4 sum,
//   the Kahan compensation and the stage input of its 512 elements in
//   registers for the whole run; it applies the stage combination, writes
//   the next stage input into both split operand layouts and, after stage 3,
//   the observables' partials, the stored states and the final rho.
// * The operands live in blocked copies of the K-major split arrays (see
//   boff), converted at launch; Ls and Rs have two copies: stage s reads
//   copy s % 2 and writes the next X into the other, so no CTA overwrites an
//   operand that another CTA may still be loading.
//
// Every mbarrier wait and every grid-barrier wait is bounded (a grid barrier
// gives up after 1 s of global-timer time).  A wait that runs out sets
// LGB_ERR_TIMEOUT; from the next grid barrier on the CTA skips all work but
// still takes part in every cluster barrier, so that the hardware cluster
// barriers always complete and the kernel ends.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>

#include "lgb_common.cuh"
#include "lgb_internal.h"
#include "lgb_split.cuh"
#include "lgb_umma.cuh"

namespace lgb {

namespace {

using namespace umma;
using namespace splitk;

constexpr int kPsThreads = 128;
constexpr int kPsCluster = 4;
constexpr int kPsCols = 32;                              // complex columns of a tile (64 rows)
constexpr int kPsOwn = 64 / kPsCluster;                  // G2 tile rows owned by one CTA
constexpr int kPsStages = 4;
constexpr int kPsRowBytes = 128;                         // K bytes per operand row and ring stage
constexpr uint32_t kPsTileP = 128 * kPsRowBytes;         // 16 KB: one level of the M-side operand
constexpr uint32_t kPsTileQ = 2 * kPsCols * kPsRowBytes; // 8 KB: one level of the N-side operand
constexpr uint32_t kPsStageBytes = 2 * kPsTileP + 2 * kPsTileQ;  // P hi, P lo, Q hi, Q lo
constexpr uint32_t kPsRing = kPsStages * kPsStageBytes;  // 192 KB
constexpr uint32_t kPsRecv = 64 * 2 * kPsCols * 4;       // 16 KB: tile rows x parts x columns, FP32
constexpr uint32_t kPsXs = kPsOwn * kPsCols * sizeof(float2);  // 4 KB: the owner's next X rows
constexpr uint32_t kPsSmem = kPsRing + kPsRecv + kPsXs + 1024;  // + alignment slack (213 KB)
constexpr unsigned long long kPsBarNs = 1000000000ull;   // grid-barrier wait bound (1 s)

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_idx() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
  return r;
}
// shared::cta address of this CTA -> the same offset in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t mapa(uint32_t addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
__device__ __forceinline__ void st_cluster4(uint32_t addr, float a, float b, float c, float d) {
  asm volatile("st.shared::cluster.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "f"(a), "f"(b), "f"(c),
               "f"(d)
               : "memory");
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void red_release_add(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
// order this thread's generic global writes before later async-proxy (bulk copy) reads
__device__ __forceinline__ void fence_proxy_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

// hi and lo parts of 8 consecutive values -> 16-byte-aligned vector stores
template <bool BF16>
__device__ __forceinline__ void store8_split(typename SElem<BF16>::T* hd, typename SElem<BF16>::T* ld,
                                             const float* v) {
  using T = typename SElem<BF16>::T;
  constexpr int W = 8 * (int)sizeof(T) / 4;  // 32-bit words per part
  uint32_t hw[W], lw[W];
  if constexpr (BF16) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      T h0, l0, h1, l1;
      SElem<true>::split(v[2 * k], h0, l0);
      SElem<true>::split(v[2 * k + 1], h1, l1);
      hw[k] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
      lw[k] = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
    }
  } else {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      float h, l;
      SElem<false>::split(v[k], h, l);
      hw[k] = __float_as_uint(h);
      lw[k] = __float_as_uint(l);
    }
  }
#pragma unroll
  for (int w = 0; w < W / 4; ++w) {
    reinterpret_cast<uint4*>(hd)[w] = make_uint4(hw[4 * w], hw[4 * w + 1], hw[4 * w + 2], hw[4 * w + 3]);
    reinterpret_cast<uint4*>(ld)[w] = make_uint4(lw[4 * w], lw[4 * w + 1], lw[4 * w + 2], lw[4 * w + 3]);
  }
}

// Blocked operand layout: an operand of R rows and K columns is stored as
// 64-row x 128-byte blocks, block (row block rb, K block kb) at position
// kb * nrb + rb (nrb = R / 64), each laid out as the 128-byte-swizzled
// K-major shared-memory tile (row r at r * 128 B, 16-byte chunk c at chunk
// c ^ (r % 8)).  A 128-row M-side tile of one K block is then 16 KB and a
// 64-row N-side tile 8 KB of contiguous memory, one bulk copy each.
template <int ESZ>
__device__ __forceinline__ long long boff(int r, long long k, int nrb) {
  constexpr int KT = kPsRowBytes / ESZ, CE = 16 / ESZ;  // elements per block row, per chunk
  const long long kb = k / KT;
  const int kk = (int)(k - kb * KT);
  return ((kb * nrb + (r >> 6)) * 64 + (r & 63)) * KT + ((kk / CE) ^ (r & 7)) * CE + kk % CE;
}

// 8 consecutive values of row r from column k (a multiple of 8) -> hi and lo
// blocked arrays (one 16-byte chunk at BF16, two at TF32)
template <bool BF16>
__device__ __forceinline__ void store8_blk(typename SElem<BF16>::T* H, typename SElem<BF16>::T* L, int r,
                                           long long k, int nrb, const float* v) {
  constexpr int ESZ = BF16 ? 2 : 4;
  if constexpr (BF16) {
    const long long o = boff<ESZ>(r, k, nrb);
    store8_split<true>(H + o, L + o, v);
  } else {
    float h[4], l[4];
    for (int half = 0; half < 2; ++half) {
#pragma unroll
      for (int u = 0; u < 4; ++u) SElem<false>::split(v[4 * half + u], h[u], l[u]);
      const long long o = boff<ESZ>(r, k + 4 * half, nrb);
      *reinterpret_cast<uint4*>(H + o) =
          make_uint4(__float_as_uint(h[0]), __float_as_uint(h[1]), __float_as_uint(h[2]), __float_as_uint(h[3]));
      *reinterpret_cast<uint4*>(L + o) =
          make_uint4(__float_as_uint(l[0]), __float_as_uint(l[1]), __float_as_uint(l[2]), __float_as_uint(l[3]));
    }
  }
}

__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint64_t* mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(smem_u32(mbar))
               : "memory");
}

struct PsArgs {
  int N = 0, NP = 0, K = 0, E = 0, nt = 0, diag = 0, obs_t0 = 0;
  int s1 = 1, nkb1 = 0, nkb2 = 0, tn = 0;  // tn: column tiles (NP / 32)
  double dt = 0.0;
  const void* Lks[2] = {nullptr, nullptr};  // blocked operands (hi, lo): L_k rows (nrb1 row blocks)
  void* Ls[2] = {nullptr, nullptr};         // Ls, two copies of copy_elems (nrb2 row blocks each)
  void* Rs[2] = {nullptr, nullptr};         // Rs, the same
  int nrb1 = 0, nrb2 = 0;
  long long copy_elems = 0;
  float2* rho = nullptr;         // FP32 state (read at the start, written at the end)
  const float2* Dm = nullptr;    // diagonal-collapse dissipator (diag)
  const double2* Ot = nullptr;   // E x N x N observables transposed
  double2* obs_out = nullptr;    // this instance's rows
  double2* part = nullptr;       // [2][kPsSlots][grid] observable and check partials
  unsigned* bar = nullptr;       // grid-barrier counter, zero at launch
  int* err = nullptr;
  StepOut so;
  // per-step check (check_tol > 0): the state's trace drift and hermiticity
  // deviation folded into chk[2] against the rho0 values in chk_ws[0..2]
  double check_tol = 0.0;
  double* chk = nullptr;
  const double* chk_ws = nullptr;
};

constexpr int kPsSlots = 18;  // partial slots per step parity: 16 observables, trace, hermiticity

template <bool BF16>
__global__ void __cluster_dims__(kPsCluster, 1, 1) __launch_bounds__(kPsThreads, 1)
    persist_rk4_kernel(const PsArgs a) {
  using T = typename SElem<BF16>::T;
  extern __shared__ unsigned char ps_smem[];
  __shared__ uint64_t full[kPsStages], empty[kPsStages], done;
  __shared__ uint32_t tmem_base;
  __shared__ int s_dead;
  __shared__ double s_red[4][16][2];
  __shared__ double s_chk[4][3];
  constexpr int KT = kPsRowBytes / (BF16 ? 2 : 4);  // K elements per ring stage
  constexpr int KSTEPS = KT / (BF16 ? 16 : 8);      // MMA K-steps per ring stage (32 B each)
  constexpr uint32_t id = idesc(BF16 ? kFmtBF16 : kFmtTF32, 128, 2 * kPsCols, false, false);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int rank = (int)cluster_rank();
  const int cid = (int)cluster_idx();
  const int I = cid / a.tn, J = cid % a.tn;  // the cluster's G2 tile
  const int N = a.N, NP = a.NP;
  const uint32_t sraw = smem_u32(ps_smem);
  const uint32_t sb = (sraw + 1023u) & ~1023u;  // ring base (1 KB aligned for the swizzled tiles)
  unsigned char* gb = ps_smem + (sb - sraw);
  // one receive buffer: its reuse by the next phase is ordered by the grid
  // barrier between the phases
  const uint32_t recv = sb + kPsRing;
  const float* recvf = reinterpret_cast<const float*>(gb + kPsRing);
  float2* xs = reinterpret_cast<float2*>(gb + kPsRing + kPsRecv);

  if (tid == 0) {
    for (int s = 0; s < kPsStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&done, 1);
    mbar_fence_init();
    s_dead = *reinterpret_cast<volatile int*>(a.err) == 5;
  }
  if (warp == 0) {
    tmem_alloc(&tmem_base, 2 * kPsCols);
    tmem_relinquish();
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  cluster_sync_all();  // every CTA of the cluster runs before the first remote store
  const uint32_t tmem = tmem_base;
  bool dead = s_dead != 0;

  // owned elements of the G2 tile: rows orow + (tid >> 5) + 4q, column tid & 31
  const int orow = kPsOwn * rank, ocol = tid & 31;
  float2 rr[4], ra[4], kc[4], xc[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int i = 64 * I + orow + (tid >> 5) + 4 * q, j = kPsCols * J + ocol;
    rr[q] = (i < N && j < N) ? a.rho[(long long)i * N + j] : make_float2(0.f, 0.f);
    ra[q] = kc[q] = make_float2(0.f, 0.f);
    xc[q] = rr[q];
  }
  uint32_t kit = 0, nitem = 0, nbar = 0;

  // One product over ring stages [kb0, kb1) into the TMEM accumulator: the
  // M-side blocks from P (row block rbp of nrbp), the N-side from Q (row
  // block rbq of nrb2), hi and lo.
  auto item = [&](const T* ph, const T* pl, int rbp, int nrbp, const T* qh, const T* ql, int rbq, int kb0,
                  int kb1) {
    if (tid == 0) {
      fence_proxy_global();
      bool ok = true;
      for (int kb = kb0; kb < kb1; ++kb) {
        const uint32_t it = kit + (uint32_t)(kb - kb0);
        const int s = (int)(it % kPsStages);
        if (!mbar_wait(&empty[s], ((it / kPsStages) & 1) ^ 1, kGemmSpin)) {
          ok = false;
          break;
        }
        mbar_expect_tx(&full[s], kPsStageBytes);
        const uint32_t st = sb + s * kPsStageBytes;
        const long long po = ((long long)kb * nrbp + rbp) * 64 * KT;
        const long long qo = ((long long)kb * a.nrb2 + rbq) * 64 * KT;
        bulk_load(st, ph + po, kPsTileP, &full[s]);
        bulk_load(st + kPsTileP, pl + po, kPsTileP, &full[s]);
        bulk_load(st + 2 * kPsTileP, qh + qo, kPsTileQ, &full[s]);
        bulk_load(st + 2 * kPsTileP + kPsTileQ, ql + qo, kPsTileQ, &full[s]);
      }
      if (!ok) atomicExch(a.err, 5);  // LGB_ERR_TIMEOUT
    } else if (tid == 32) {
      fence_after_sync();
      bool ok = true;
      for (int kb = kb0; kb < kb1; ++kb) {
        const uint32_t it = kit + (uint32_t)(kb - kb0);
        const int s = (int)(it % kPsStages);
        if (!mbar_wait(&full[s], (it / kPsStages) & 1, kGemmSpin)) {
          ok = false;
          break;
        }
        fence_after_sync();
        const uint32_t st = sb + s * kPsStageBytes;
#pragma unroll
        for (int ks = 0; ks < KSTEPS; ++ks) {
          const uint64_t dph = sdesc_sw128(st + 32 * ks);
          const uint64_t dpl = sdesc_sw128(st + kPsTileP + 32 * ks);
          const uint64_t dqh = sdesc_sw128(st + 2 * kPsTileP + 32 * ks);
          const uint64_t dql = sdesc_sw128(st + 2 * kPsTileP + kPsTileQ + 32 * ks);
          mma_k<BF16>(tmem, dph, dqh, id, (kb > kb0 || ks > 0) ? 1u : 0u);
          mma_k<BF16>(tmem, dph, dql, id, 1u);
          mma_k<BF16>(tmem, dpl, dqh, id, 1u);
        }
        mma_commit(&empty[s]);  // ring stage s is free once these MMAs completed
      }
      mma_commit(&done);
      if (!ok) atomicExch(a.err, 5);
    }
    __syncwarp();
    kit += (uint32_t)(kb1 - kb0);
  };

  // Wait for the item's MMAs, combine the partner lanes and store this CTA's
  // rows (split source `src`) into the receive buffers of their owners:
  // tile row i belongs to CTA owner0 + i / rows_per.  A row's 8 four-float
  // chunks are stored at chunk ^ (i % 8), which spreads one store
  // instruction of a warp over the banks.
  auto push = [&](int src, int rows_per, int owner0) {
    const uint32_t buf = recv;
    if (!mbar_wait(&done, nitem & 1, kGemmSpin)) atomicExch(a.err, 5);
    ++nitem;
    fence_after_sync();
    const int c = lane >> 4, i = warp * 16 + (lane & 15);
    const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);
    const float sg = c == 0 ? -1.f : 1.f;
    float v[kPsCols];
#pragma unroll
    for (int h = 0; h < kPsCols / 16; ++h) {
      float p1[16], p0[16];
      tmem_ld16(tl + 32 * h, p1);
      tmem_ld16(tl + 32 * h + 16, p0);
      tmem_wait_ld();
#pragma unroll
      for (int e = 0; e < 16; ++e) {
        const float x = __shfl_xor_sync(0xffffffffu, p1[e], 16);
        v[16 * h + e] = fmaf(sg, x, p0[e]);
      }
    }
    fence_before_sync();
    const int ow = owner0 + i / rows_per, rl = i % rows_per, sw = i & 7;
    const uint32_t dst = mapa(buf + (uint32_t)(((src * rows_per + rl) * 2 + c) * kPsCols * 4), (uint32_t)ow);
#pragma unroll
    for (int q = 0; q < kPsCols / 4; ++q)
      st_cluster4(dst + 16u * (uint32_t)(q ^ sw), v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
  };

  // Grid barrier: the CTA's writes are ordered before thread 0's release-add
  // by the CTA barrier, and the acquire polls before the CTA's later reads by
  // the second one (no separate fences: they cost 6 % of a step).
  auto gsync = [&]() {
    fence_proxy_global();
    __syncthreads();
    ++nbar;
    if (tid == 0) {
      int d = s_dead;
      if (!d) {
        red_release_add(a.bar, 1u);
        const unsigned target = nbar * gridDim.x;
        const unsigned long long t0 = gtimer();
        while (ld_acquire(a.bar) < target) {
          if (gtimer() - t0 > kPsBarNs) {
            d = 1;
            atomicExch(a.err, 5);
            break;
          }
        }
        if (*reinterpret_cast<volatile int*>(a.err) == 5) d = 1;
      }
      s_dead = d;
    }
    __syncthreads();
    dead = s_dead != 0;
  };

  T* const LH = reinterpret_cast<T*>(a.Ls[0]);
  T* const LL = reinterpret_cast<T*>(a.Ls[1]);
  T* const RH = reinterpret_cast<T*>(a.Rs[0]);
  T* const RL = reinterpret_cast<T*>(a.Rs[1]);
  const T* const KH = reinterpret_cast<const T*>(a.Lks[0]);
  const T* const KL = reinterpret_cast<const T*>(a.Lks[1]);
  const long long CE = a.copy_elems;
  const float sixth = (float)(a.dt / 6.0);
  const bool check = a.check_tol > 0.0;

  // Per-step check of step `step`'s state: this CTA's elements against their
  // transposes (the FP32 state every owner wrote at that step's last stage)
  // and its share of the trace, into the partial slots of the step's parity.
  auto check_partials = [&](int step) {
    double h = 0.0, tx = 0.0, ty = 0.0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int ig = 64 * I + orow + (tid >> 5) + 4 * q, jg = kPsCols * J + ocol;
      if (ig < N && jg < N) {
        // (written by another CTA one grid barrier ago: read past L1)
        const volatile float* vt = reinterpret_cast<const volatile float*>(a.rho + (long long)jg * N + ig);
        const float xtx = vt[0], xty = vt[1];
        h = fmax(h, hypot((double)rr[q].x - (double)xtx, (double)rr[q].y + (double)xty));
        if (ig == jg) {
          tx += rr[q].x;
          ty += rr[q].y;
        }
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      h = fmax(h, __shfl_xor_sync(0xffffffffu, h, o));
      tx += __shfl_xor_sync(0xffffffffu, tx, o);
      ty += __shfl_xor_sync(0xffffffffu, ty, o);
    }
    if (lane == 0) {
      s_chk[warp][0] = h;
      s_chk[warp][1] = tx;
      s_chk[warp][2] = ty;
    }
    __syncthreads();
    if (tid == 0) {
      const double hh = fmax(fmax(s_chk[0][0], s_chk[1][0]), fmax(s_chk[2][0], s_chk[3][0]));
      const double sx = (s_chk[0][1] + s_chk[1][1]) + (s_chk[2][1] + s_chk[3][1]);
      const double sy = (s_chk[0][2] + s_chk[1][2]) + (s_chk[2][2] + s_chk[3][2]);
      a.part[((long long)(step & 1) * kPsSlots + 16) * gridDim.x + blockIdx.x] = make_double2(sx, sy);
      a.part[((long long)(step & 1) * kPsSlots + 17) * gridDim.x + blockIdx.x] = make_double2(hh, 0.0);
    }
  };
  // (CTA 0, once every CTA's partials of `step` are in) fold into the maxima
  auto check_fold = [&](int step) {
    if (blockIdx.x != 0 || tid != 0) return;
    const double2* pt = a.part + ((long long)(step & 1) * kPsSlots + 16) * gridDim.x;
    const double2* ph = a.part + ((long long)(step & 1) * kPsSlots + 17) * gridDim.x;
    double sx = 0.0, sy = 0.0, h = 0.0;
    for (unsigned b = 0; b < gridDim.x; ++b) {
      const volatile double* vt = reinterpret_cast<const volatile double*>(pt + b);
      const volatile double* vh = reinterpret_cast<const volatile double*>(ph + b);
      sx += vt[0];
      sy += vt[1];
      h = fmax(h, vh[0]);
    }
    const double dtr = hypot(sx - a.chk_ws[0], sy - a.chk_ws[1]);
    a.chk[0] = fmax(a.chk[0], dtr);
    bool bad = !(dtr <= a.check_tol);
    if (a.chk_ws[2] != 0.0) {
      a.chk[1] = fmax(a.chk[1], h);
      bad = bad || !(h <= a.check_tol);
    }
    if (bad) atomicCAS(a.err, 0, 9);  // LGB_ERR_CHECK
  };
  int fold_step = -1;  // a step whose check partials await the fold after the next grid barrier
  auto gsync_fold = [&]() {
    gsync();
    if (fold_step >= 0 && !dead) check_fold(fold_step);
    fold_step = -1;
  };

  // tile row i, column col of an owner's receive buffer (rows_per rows per source)
  auto roff = [](int src, int rows_per, int rl, int c, int i, int col) {
    return ((src * rows_per + rl) * 2 + c) * kPsCols + 4 * ((col >> 2) ^ (i & 7)) + (col & 3);
  };

  for (int step = 0; step < a.nt; ++step) {
    for (int stage = 0; stage < 4; ++stage) {
      const int cp = stage & 1, nx = cp ^ 1;  // operand copy read / written by this stage
      if (check && stage == 0 && step > 0 && !dead) {
        check_partials(step - 1);
        fold_step = step - 1;
      }
      // ---- G1: T_k = L_k X, K products of the tile position split s1 ways ----------
      if (a.K > 0) {
        const int groups = kPsCluster / a.s1, g = rank / a.s1, zz = rank % a.s1;
        const int rows_per = 64 / a.s1;
        for (int k0 = 0; k0 < a.K; k0 += groups) {
          const int k = k0 + g;
          const bool act = k < a.K && !dead;
          if (act) {
            item(KH, KL, (k * 2 * NP + 128 * I) / 64, a.nrb1, RH + cp * CE, RL + cp * CE, J,
                 zz * a.nkb1 / a.s1, (zz + 1) * a.nkb1 / a.s1);
            push(zz, rows_per, g * a.s1);
          }
          cluster_sync_all();
          const float* rb = recvf;
          if (act) {
            // owned rows [zz rows_per, +rows_per) of T_k -> M-side block 2 + k of this
            // copy, 8 columns of one row part per task
            for (int q = 0; q < rows_per / 16; ++q) {
              const int e = tid + 128 * q;
              const int oct = e & 3, c = (e >> 2) & 1, rl = e >> 3;
              const int i = zz * rows_per + rl;
              float v[8];
#pragma unroll
              for (int u = 0; u < 8; ++u) v[u] = 0.f;
              for (int src = 0; src < a.s1; ++src) {
                const float* b = rb + ((src * rows_per + rl) * 2 + c) * kPsCols;
                const float4 lo4 = *reinterpret_cast<const float4*>(b + 4 * ((2 * oct) ^ (i & 7)));
                const float4 hi4 = *reinterpret_cast<const float4*>(b + 4 * ((2 * oct + 1) ^ (i & 7)));
                v[0] += lo4.x, v[1] += lo4.y, v[2] += lo4.z, v[3] += lo4.w;
                v[4] += hi4.x, v[5] += hi4.y, v[6] += hi4.z, v[7] += hi4.w;
              }
              const long long colg = (long long)(2 + k) * NP + kPsCols * J + 8 * oct;
              store8_blk<BF16>(LH + cp * CE, LL + cp * CE, mrow(c, 64 * I + i), colg, a.nrb2, v);
            }
          }
          // (one receive buffer: the next round's stores wait until every owner has read)
          if (k0 + groups < a.K) cluster_sync_all();
        }
        gsync_fold();
      }
      // ---- G2: R = Ls . Rs^T, the tile's K extent split over the cluster -----------
      if (!dead) {
        item(LH + cp * CE, LL + cp * CE, 2 * I, a.nrb2, RH + cp * CE, RL + cp * CE, J,
             rank * a.nkb2 / kPsCluster, (rank + 1) * a.nkb2 / kPsCluster);
        push(rank, kPsOwn, 0);
      }
      cluster_sync_all();
      const float* rb = recvf;
      bool fin = true;
      if (!dead) {
        const float cst = (float)((stage == 2) ? a.dt : 0.5 * a.dt);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int r = (tid >> 5) + 4 * q, i = orow + r;
          float2 R = make_float2(0.f, 0.f);
#pragma unroll
          for (int src = 0; src < kPsCluster; ++src) {
            R.x += rb[roff(src, kPsOwn, r, 0, i, ocol)];
            R.y += rb[roff(src, kPsOwn, r, 1, i, ocol)];
          }
          const int ig = 64 * I + i, jg = kPsCols * J + ocol;
          const bool in = ig < N && jg < N;
          if (a.diag && in) cmac(R, a.Dm[(long long)ig * N + jg], xc[q]);
          float2 xn;
          if (stage == 0) {
            ra[q] = R;
            xn = caxpy(rr[q], cst, R);
          } else if (stage < 3) {
            ra[q] = caxpy(ra[q], 2.f, R);
            xn = caxpy(rr[q], cst, R);
          } else {
            // Kahan-compensated rho += dt/6 (k1 + 2 k2 + 2 k3 + k4)
            const float yx = fmaf(sixth, ra[q].x + R.x, -kc[q].x), yy = fmaf(sixth, ra[q].y + R.y, -kc[q].y);
            const float tx = rr[q].x + yx, ty = rr[q].y + yy;
            kc[q] = make_float2((tx - rr[q].x) - yx, (ty - rr[q].y) - yy);
            rr[q] = make_float2(tx, ty);
            xn = rr[q];
            fin = fin && isfinite(tx) && isfinite(ty);
          }
          if (!in) xn = make_float2(0.f, 0.f);
          xc[q] = xn;
          xs[r * kPsCols + ocol] = xn;
        }
      }
      __syncthreads();
      if (!dead) {
        // N-side block 0 (X^T) of the next copy: row (p, j), 8 of the owner's 16 columns
        {
          const int p = (tid >> 5) & 1, col = tid & 31, half = tid >> 6;
          const long long c0 = 64LL * I + orow + 8 * half;
          float v[8];
#pragma unroll
          for (int r = 0; r < 8; ++r) {
            const float2 x = xs[(8 * half + r) * kPsCols + col];
            v[r] = p == 0 ? x.x : x.y;
          }
          store8_blk<BF16>(RH + nx * CE, RL + nx * CE, ncol(p, kPsCols * J + col), c0, a.nrb2, v);
        }
        // M-side block 1 (X rows) of the next copy: row (c, i), 8 of the tile's 32 columns
        {
          const int oct = tid & 3, c = (tid >> 2) & 1, r = tid >> 3;
          const long long c0 = (long long)NP + kPsCols * J + 8 * oct;
          float v[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const float2 x = xs[r * kPsCols + 8 * oct + u];
            v[u] = c == 0 ? x.x : x.y;
          }
          store8_blk<BF16>(LH + nx * CE, LL + nx * CE, mrow(c, 64 * I + orow + r), c0, a.nrb2, v);
        }
      }
      if (stage == 3 && !dead) {
        if (__syncthreads_or(!fin) && tid == 0) atomicCAS(a.err, 0, 4);  // LGB_ERR_NONFINITE
        if (check) {
          // the state of this step, for the transposed reads of its check
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int ig = 64 * I + orow + (tid >> 5) + 4 * q, jg = kPsCols * J + ocol;
            if (ig < N && jg < N) a.rho[(long long)ig * N + jg] = rr[q];
          }
        }
        double2* state_out = a.so.state_at(step, (long long)N * N);
        double2* rho_out = step == a.nt - 1 ? a.so.rho_out : nullptr;
        if (state_out != nullptr || rho_out != nullptr) {
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int ig = 64 * I + orow + (tid >> 5) + 4 * q, jg = kPsCols * J + ocol;
            if (ig < N && jg < N) {
              const double2 rd = make_double2(rr[q].x, rr[q].y);
              if (state_out != nullptr) state_out[(long long)ig * N + jg] = rd;
              if (rho_out != nullptr) rho_out[(long long)ig * N + jg] = rd;
            }
          }
        }
        for (int e = 0; e < a.E; ++e) {
          double sx = 0.0, sy = 0.0;
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int ig = 64 * I + orow + (tid >> 5) + 4 * q, jg = kPsCols * J + ocol;
            if (ig < N && jg < N) {
              const double2 o = a.Ot[(long long)e * N * N + (long long)ig * N + jg];
              sx += o.x * rr[q].x - o.y * rr[q].y;
              sy += o.x * rr[q].y + o.y * rr[q].x;
            }
          }
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            sx += __shfl_xor_sync(0xffffffffu, sx, o);
            sy += __shfl_xor_sync(0xffffffffu, sy, o);
          }
          if (lane == 0) {
            s_red[warp][e][0] = sx;
            s_red[warp][e][1] = sy;
          }
        }
        __syncthreads();
        if (tid < a.E) {
          const double sx = (s_red[0][tid][0] + s_red[1][tid][0]) + (s_red[2][tid][0] + s_red[3][tid][0]);
          const double sy = (s_red[0][tid][1] + s_red[1][tid][1]) + (s_red[2][tid][1] + s_red[3][tid][1]);
          a.part[((long long)(step & 1) * kPsSlots + tid) * gridDim.x + blockIdx.x] = make_double2(sx, sy);
        }
      }
      gsync_fold();
      if (stage == 3 && !dead && blockIdx.x == 0 && tid < a.E) {
        // every CTA's partial of this step is in: fixed-order FP64 sum
        const double2* pp = a.part + ((long long)(step & 1) * kPsSlots + tid) * gridDim.x;
        double sx = 0.0, sy = 0.0;
        for (unsigned b = 0; b < gridDim.x; ++b) {
          const volatile double* vp = reinterpret_cast<const volatile double*>(pp + b);
          sx += vp[0];
          sy += vp[1];
        }
        a.obs_out[((long long)step + a.obs_t0) * a.E + tid] = make_double2(sx, sy);
      }
    }
  }
  if (check && a.nt > 0 && !dead) {
    // the last step's check
    check_partials(a.nt - 1);
    fold_step = a.nt - 1;
    gsync_fold();
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int ig = 64 * I + orow + (tid >> 5) + 4 * q, jg = kPsCols * J + ocol;
    if (!dead && ig < N && jg < N) a.rho[(long long)ig * N + jg] = rr[q];
  }
  fence_before_sync();
  __syncthreads();
  cluster_sync_all();  // no CTA leaves while a peer may still address its shared memory
  if (warp == 0) tmem_dealloc(tmem, 2 * kPsCols);
}

// K-major hi/lo arrays (rows x pitch elements) -> the blocked layout, into
// `copies` copies copy_elems apart; one 16-byte chunk per thread and step.
template <bool BF16>
__global__ void to_blocks_kernel(const void* src_h, const void* src_l, long long rows, long long pitch,
                                 void* dst_h, void* dst_l, int nrb, long long copy_elems, int copies) {
  using T = typename SElem<BF16>::T;
  constexpr int CE = 16 / (int)sizeof(T);
  const long long cpr = pitch / CE, n = rows * cpr;
  const T* sh = reinterpret_cast<const T*>(src_h);
  const T* sl = reinterpret_cast<const T*>(src_l);
  T* dh = reinterpret_cast<T*>(dst_h);
  T* dl = reinterpret_cast<T*>(dst_l);
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long r = idx / cpr, k = (idx - r * cpr) * CE;
    const uint4 vh = *reinterpret_cast<const uint4*>(sh + r * pitch + k);
    const uint4 vl = *reinterpret_cast<const uint4*>(sl + r * pitch + k);
    const long long o = boff<(int)sizeof(T)>((int)r, k, nrb);
    for (int c = 0; c < copies; ++c) {
      *reinterpret_cast<uint4*>(dh + c * copy_elems + o) = vh;
      *reinterpret_cast<uint4*>(dl + c * copy_elems + o) = vl;
    }
  }
}

int grid_of(int NP) { return kPsCluster * (NP / 64) * (NP / kPsCols); }

}  // namespace

bool persist_supported(int NP, bool bf16) {
  if (NP != 128 && NP != 256) return false;
  const void* fn = bf16 ? reinterpret_cast<const void*>(&persist_rk4_kernel<true>)
                        : reinterpret_cast<const void*>(&persist_rk4_kernel<false>);
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPsSmem) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid_of(NP));
  cfg.blockDim = dim3(kPsThreads);
  cfg.dynamicSmemBytes = kPsSmem;
  int nc = 0;
  if (cudaOccupancyMaxActiveClusters(&nc, fn, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  // every cluster co-resident: the grid barriers need all CTAs running at once
  return nc * kPsCluster >= grid_of(NP);
}

int persist_part_elems(int NP) { return 2 * kPsSlots * grid_of(NP); }

int persist_propagate(const GemmRunArgs& a, cudaStream_t st) {
  const GemmSplit& sp = a.sp;
  const int NP = sp.NP;
  const int KT = kPsRowBytes / (sp.bf16 ? 2 : 4);
  PsArgs p;
  p.N = a.g.N;
  p.NP = NP;
  p.K = a.Kdense;
  p.E = a.E;
  p.nt = a.nt;
  p.diag = a.diag;
  p.obs_t0 = a.obs_t0;
  p.nkb1 = NP / KT;
  p.nkb2 = (int)(sp.Wp / KT);
  int s1 = kPsCluster;
  while (s1 > 1 && (a.Kdense * s1 > kPsCluster || s1 > p.nkb1)) s1 >>= 1;
  p.s1 = s1;
  p.tn = NP / kPsCols;
  p.dt = a.dt;
  p.nrb1 = a.Kdense * 2 * NP / 64;
  p.nrb2 = 2 * NP / 64;
  p.copy_elems = 2LL * NP * sp.Wp;
  for (int l = 0; l < 2; ++l) {
    p.Lks[l] = sp.Lksb[l];
    p.Ls[l] = sp.Lsb[l];
    p.Rs[l] = sp.Rsb[l];
  }
  p.rho = reinterpret_cast<float2*>(a.g.rho);
  p.Dm = reinterpret_cast<const float2*>(a.g.Dm);
  p.Ot = a.g.Ot;
  p.obs_out = a.obs_out;
  p.part = sp.part;
  p.bar = sp.bar;
  p.err = a.g.err;
  p.so.obs_t0 = a.obs_t0;
  p.so.nt = a.nt;
  p.so.store_every = a.store_every;
  p.so.states_out = a.states_out;
  p.so.rho_out = a.rho_out;
  if (a.check_tol > 0.0 && a.chk != nullptr) {
    p.check_tol = a.check_tol;
    p.chk = a.chk;
    p.chk_ws = a.chk_ws;
  }
  const int grid = grid_of(NP);
  if (p.nkb2 < kPsCluster || (p.K > 0 && p.nkb1 < p.s1) || (long long)a.nt * 9 * grid >= (1LL << 31))
    return LGB_ERR_UNSUPPORTED;
  // the operands (set up and initialised in the K-major arrays) into the
  // blocked layout: L_k once, Ls and Rs into both copies
  const int cgrid = 1024;  // (grid-stride loops)
  if (sp.bf16) {
    if (p.K > 0)
      to_blocks_kernel<true><<<cgrid, 256, 0, st>>>(sp.Lks[0], sp.Lks[1], (long long)p.K * 2 * NP, NP, sp.Lksb[0],
                                                    sp.Lksb[1], p.nrb1, 0, 1);
    to_blocks_kernel<true><<<cgrid, 256, 0, st>>>(sp.Ls[0], sp.Ls[1], 2LL * NP, sp.Wp, sp.Lsb[0], sp.Lsb[1], p.nrb2,
                                                  p.copy_elems, 2);
    to_blocks_kernel<true><<<cgrid, 256, 0, st>>>(sp.Rs[0], sp.Rs[1], 2LL * NP, sp.Wp, sp.Rsb[0], sp.Rsb[1], p.nrb2,
                                                  p.copy_elems, 2);
  } else {
    if (p.K > 0)
      to_blocks_kernel<false><<<cgrid, 256, 0, st>>>(sp.Lks[0], sp.Lks[1], (long long)p.K * 2 * NP, NP, sp.Lksb[0],
                                                     sp.Lksb[1], p.nrb1, 0, 1);
    to_blocks_kernel<false><<<cgrid, 256, 0, st>>>(sp.Ls[0], sp.Ls[1], 2LL * NP, sp.Wp, sp.Lsb[0], sp.Lsb[1], p.nrb2,
                                                   p.copy_elems, 2);
    to_blocks_kernel<false><<<cgrid, 256, 0, st>>>(sp.Rs[0], sp.Rs[1], 2LL * NP, sp.Wp, sp.Rsb[0], sp.Rsb[1], p.nrb2,
                                                   p.copy_elems, 2);
  }
  if (cudaMemsetAsync(sp.bar, 0, sizeof(unsigned), st) != cudaSuccess) return LGB_ERR_CUDA;
  if (sp.bf16)
    persist_rk4_kernel<true><<<grid, kPsThreads, kPsSmem, st>>>(p);
  else
    persist_rk4_kernel<false><<<grid, kPsThreads, kPsSmem, st>>>(p);
  return cudaGetLastError() == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

}  // namespace lgb
