// Internal plan structure and kernel launchers shared by the C-ABI layer.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "../../include/lindblad_gb300.h"

struct cublasContext;
#include "lgb_common.cuh"

namespace lgb {

// ---- CTA-resident schedule (lgb_cta.cu) -------------------------------------
int cta_max_npad();
int cta_wide_max_npad();
size_t cta_elem_bytes(int precision);
cudaError_t launch_cta_rk4(const CtaParams& p, int precision, int n_blocks, cudaStream_t stream,
                           bool wide);

// ---- tensor-core CTA-resident schedule (lgb_tc.cu) --------------------------
// N <= tc_max_dim() runs as one padded block; N = tc_border_dim() with a static
// H runs as a 64 x 64 block plus a SIMT border row and column, its working
// matrices padded to kTcBorderNpad.
constexpr int kTcBorderNpad = 68;
int tc_max_dim();
int tc_border_dim();
int tc_smem_bytes(int precision, int npad);
cudaError_t launch_tc_rk4(const CtaParams& p, int precision, const int* order, int n_items,
                          int* queue, int grid, cudaStream_t stream);
cudaError_t launch_tc_border(const CtaParams& p, int precision, const int* order, int n_items,
                             cudaStream_t stream);

// ---- discrete adjoint (lgb_adjoint.cu) ------------------------------------------
struct AdjParams {
  int n_inst, n_cops, n_drive, n_eops, nt, seg0, seg_len, ycap, drive_ld, drive_shared, obs_t0;
  int first_segment, smem_bytes;
  double dt;
  const int* order;
  const int* dims;
  const int* npad;
  const long long* woff;
  const float2* At;      // forward A0^T (working FP32)
  const float2* Gt;      // (i H_d)^T
  const float2* Lt;      // L_k^T
  float2* Lc;            // scratch: conj(L_k) row-major
  float2* GkT;           // scratch: (L_k^dag L_k)^T
  float2* Macc;          // sum over stages of P - Q (the H0 gradient before Gamma = i M^dag)
  float2* lam;           // costate
  const float2* ys;      // stage inputs of the segment
  const double2* Ot;     // observables transposed (FP64)
  const double* drive;   // drive samples, [inst][n_drive][drive_ld]
  const double2* obs_grad;
  double* dE;            // [n_inst][n_drive][nt]
  double* dscale;        // [n_inst][n_cops], accumulated
};
int adjoint_smem_bytes(int npad, int K);
cudaError_t launch_adjoint_segment(const AdjParams& p, int n_blocks, cudaStream_t st);
cudaError_t launch_adjoint_finish(const AdjParams& p, const long long* off, double2* drho0,
                                  double2* dH, cudaStream_t st);

// ---- operator preparation (lgb_setup.cu) -------------------------------------
struct SetupParams {
  int n_inst, n_cops, cops_kind, n_eops, n_drive, padc;
  int max_npad;  // the largest padded dimension (sizes the setup grid)
  const int* dims;
  const int* npad;
  const long long* off;
  const long long* doff;
  const long long* woff;
  const double2* H;
  const double2* cops;
  const double2* eops;
  const double2* dops;
  double* shift;  // per-instance trace shift Re Tr(H)/N
  void* At;
  void* Lt;
  void* Dm;
  void* Gt;
  double2* Ot;
  float2* OtF;  // FP32 copy of Ot (FP32-working plans only)
};
cudaError_t launch_setup(const SetupParams& p, int precision, cudaStream_t stream);
cudaError_t launch_trace_shift(const SetupParams& p, cudaStream_t stream);

// ---- grid-wide GEMM schedule (lgb_gemm.cu) ----------------------------------------
struct GemmInstance {
  int N = 0, W = 0;              // dimension; W = (K_dense + 2) N, the GEMM K extent
  void* Lbuf = nullptr;          // N x W   [A | X | T_1 .. T_K]      (working precision)
  void* Rbuf = nullptr;          // W x N   [X ; A^dag ; L_k^dag]
  void* Rout = nullptr;          // N x N   RHS
  void* Lstk = nullptr;          // K x N x N collapse operators
  void* Dm = nullptr;            // N x N   diagonal-collapse dissipator matrix
  void* A0 = nullptr;            // N x N   static A of a driven instance
  void* Gd = nullptr;            // D x N x N drive terms i H_d
  void* rho = nullptr;           // N x N
  void* racc = nullptr;          // N x N   RK4 sum
  double2* Ot = nullptr;         // E x N x N observables transposed (FP64)
  double2* partial = nullptr;    // E x grid observable partials
  int* counter = nullptr;        // last-block ticket
  int* err = nullptr;            // instance status
};
// Step-dependent outputs of the stage-3 epilogue, resolved on the device from
// the step counter (so that a captured step can be replayed).
struct StepOut {
  const int* ctr = nullptr;
  int obs_t0 = 0, nt = 0, store_every = 0;
  double2* states_out = nullptr;
  double2* rho_out = nullptr;
  __host__ __device__ double2* state_at(int step, long long NN) const {
    if (store_every <= 0 || states_out == nullptr || (step + 1) % store_every != 0) return nullptr;
    return states_out + (long long)((step + 1) / store_every - 1) * NN;
  }
};
struct GemmSetupArgs {
  GemmInstance g;
  cublasContext* blas = nullptr;
  bool fp64 = false;
  const double2* H = nullptr;
  const double2* cops = nullptr;  // this instance's collapse operators
  const double2* eops = nullptr;
  const double2* dops = nullptr;
  int cops_kind = 0, K = 0, E = 0, D = 0;
  const double* shift = nullptr;  // device, Re Tr(H)/N
  long long doff = 0;             // packed-diagonal base of this instance (diag kind)
  double2* Gtmp = nullptr;        // N x N FP64 scratch for sum_k L_k^dag L_k
};
// Split-precision operands of the GEMM schedule (lgb_gemm_tc.cu): the
// interleaved K-major hi/lo arrays of G2 (Ls: M side [A | X | T_k], Rs: N side
// [X ; A^dag ; L_k^dag] transposed) and of G1 (Lks: the L_k), the split-K
// partial outputs, the Kahan compensation and the TMA tensor maps.
struct GemmSplit {
  int NP = 0;                    // dimension padded to a multiple of 128
  long long Wp = 0;              // (K_dense + 2) NP, the K extent of G2
  bool bf16 = false;
  void* Ls[2] = {nullptr, nullptr};   // 2 NP x Wp
  void* Rs[2] = {nullptr, nullptr};   // 2 NP x Wp
  void* Lks[2] = {nullptr, nullptr};  // K x 2 NP x NP
  float2* Tpart = nullptr;       // ks1 x K x NP x NP
  float2* Rpart = nullptr;       // ks2 x NP x NP
  float2* kc = nullptr;          // N x N
  int ks1 = 1, ks2 = 1;
  // persistent kernel (NP <= 256): the same operands in 64-row x 128-byte
  // blocks laid out as the swizzled shared-memory tiles, Ls and Rs twice
  bool persist = false;          // it applies (its clusters co-resident)
  void* Lsb[2] = {nullptr, nullptr};
  void* Rsb[2] = {nullptr, nullptr};
  void* Lksb[2] = {nullptr, nullptr};
  unsigned* bar = nullptr;       // grid-barrier counter
  double2* part = nullptr;       // observable and check partials
  CUtensorMap map_g1[4];         // Lks hi, lo; Rs hi, lo
  CUtensorMap map_g2[4];         // Ls hi, lo; Rs hi, lo
};
struct GemmRunArgs {
  GemmInstance g;
  bool split = false;
  GemmSplit sp;
  int* ctr = nullptr;              // device step counter (step-dependent kernel arguments)
  cudaStream_t cap = nullptr;      // private stream for CUDA-graph capture (null: no graphs)
  cublasContext* blas = nullptr;
  bool fp64 = false;
  int Kdense = 0, D = 0, E = 0, nt = 0, obs_t0 = 0, store_every = 0, diag = 0;
  double dt = 0.0;
  const double2* rho0 = nullptr;
  const double* drive = nullptr;   // [D][nt] for this instance
  double2* obs_out = nullptr;      // this instance's rows
  double2* rho_out = nullptr;
  double2* states_out = nullptr;
  int graph_steps = 16;            // RK4 steps per captured CUDA graph
  bool persist = true;             // split precision: the persistent kernel where it applies
  double check_tol = 0.0;          // per-step check (0: off)
  double* chk = nullptr;           // this instance's [2] check maxima
  double* chk_ws = nullptr;        // this instance's [8] check scratch
};
size_t gemm_partial_slots(int N);
// per-step trace / hermiticity check of the GEMM schedule's state (g.rho,
// FP32 or FP64): accumulate, then fold into the maxima (initial: the rho0 values)
void gemm_check(const GemmRunArgs& a, bool fp64, bool initial, cudaStream_t st);
int gemm_setup(const GemmSetupArgs& a, cudaStream_t st);
int gemm_propagate(const GemmRunArgs& a, cudaStream_t st);
// FP32 pieces of the GEMM schedule reused by the split-precision one
void gemm_init_split(const GemmInstance& g, const double2* rho0, cudaStream_t st);
void gemm_obs_split(const GemmInstance& g, int E, double2* obs_out, cudaStream_t st);
void gemm_drive_split(const GemmInstance& g, int D, const double* f, int nt, const int* ctr, cudaStream_t st);
void gemm_step_inc(int* ctr, cudaStream_t st);
// nt RK4 steps: eagerly, or as CUDA graphs of up to 16 steps captured once on
// `cap` and replayed on `st` (one_step launches one step on the stream given)
template <typename F>
int run_steps(int nt, cudaStream_t st, cudaStream_t cap, F&& one_step, int graph_steps = 16);
// split-precision schedule (lgb_gemm_tc.cu)
int split_padded_dim(int N);
size_t split_partial_slots(int N);
size_t split_tpart_elems(int NP, int Kd, int n_sm, bool bf16);
size_t split_rpart_elems(int NP, int Kd, int n_sm, bool bf16);
int split_setup(GemmSplit& sp, const GemmInstance& g, int Kd, bool bf16, int n_sm, cudaStream_t st);
// split-K factors of one instance for a CTA budget (SM count x waves)
void split_set_ksplit(GemmSplit& sp, int Kd, int cta_budget, int cap = 0);
int split_propagate(const GemmRunArgs& a, cudaStream_t st);
// persistent split-precision kernel (lgb_gemm_persist.cu): one launch for all
// steps of a static instance with NP = 128 or 256
bool persist_supported(int NP, bool bf16);
int persist_part_elems(int NP);
int persist_propagate(const GemmRunArgs& a, cudaStream_t st);

}  // namespace lgb

struct lgb_plan {
  lgb_problem_t prob{};
  int device = 0;
  int schedule = LGB_SCHED_CTA;
  int smem_bytes = 0;
  int padc = 2;
  bool ops_set = false;
  long long n_store = 0;
  std::vector<int> dims, npad, order;      // order: CTA-kernel instances, largest first
  std::vector<int> order_w;                // 384-thread FP32 CTA-kernel instances (64 < N <= 76)
  std::vector<int> tc_order;               // tensor-core kernel instances, largest first
  std::vector<int> tcb_order;              // N = 65 instances of the tensor-core border kernel
  int tc_smem = 0;
  int tcb_smem = 0;
  int opt_pairs = 1;                       // LGB_OPT_TC_PAIRS
  int opt_waves = 1;                       // LGB_OPT_GEMM_WAVES
  int opt_stall = 0;                       // LGB_OPT_TEST_STALL
  int opt_check = 0;                       // LGB_OPT_CHECK: 0 off, v: tolerance 10^-v
  int opt_kcap = 0;                        // LGB_OPT_GEMM_KSPLIT: split-K cap (0: none)
  int opt_gsteps = 16;                     // LGB_OPT_GRAPH_STEPS: RK4 steps per CUDA graph
  int opt_persist = 1;                     // LGB_OPT_GEMM_PERSIST: persistent split kernel where it applies
  cudaStream_t cap_stream = nullptr;       // GEMM schedule: CUDA-graph capture
  int* d_ctr = nullptr;                    // GEMM schedule: device step counter
  void* blas_ws = nullptr;                 // cuBLAS workspace (graph capture allocates nothing)
  int smem_w = 0;
  int n_sm = 0;
  cudaStream_t side[3] = {nullptr, nullptr, nullptr};  // streams for kernels that run beside the first
  cudaEvent_t ev_fork = nullptr;
  cudaEvent_t ev_join[3] = {nullptr, nullptr, nullptr};
  std::vector<long long> off, doff, woff, soff;
  std::vector<unsigned char> place;
  long long tot_off = 0, tot_doff = 0, tot_woff = 0;
  int64_t flops_per_step = 0;
  size_t ws_bytes = 0;
  cudaStream_t last_stream = nullptr;
  // device buffers (owned)
  int* d_dims = nullptr;
  int* d_npad = nullptr;
  int* d_order = nullptr;
  int* d_order_w = nullptr;
  int* d_tc_order = nullptr;
  int* d_tcb_order = nullptr;
  int* d_queue = nullptr;
  long long* d_off = nullptr;
  long long* d_doff = nullptr;
  long long* d_woff = nullptr;
  long long* d_soff = nullptr;
  unsigned char* d_place = nullptr;
  double* d_shift = nullptr;
  void* d_At = nullptr;
  void* d_Lt = nullptr;
  void* d_Dm = nullptr;
  void* d_Gt = nullptr;
  double2* d_Ot = nullptr;
  float2* d_OtF = nullptr;
  void* d_state = nullptr;
  void* d_y = nullptr;
  int* d_err = nullptr;
  double* d_chk = nullptr;                 // [n_inst][2] per-step check maxima
  double* d_chkws = nullptr;               // [n_inst][8] GEMM schedule: check scratch
  std::vector<void*> allocations;
  // adjoint (plans created with LGB_FLAG_ADJOINT)
  bool adjoint = false;
  int ckpt_every = 0;
  double2* d_ckpt = nullptr;     // [n_ckpt][packed] checkpoints rho_C, rho_2C, ...
  void* d_ybuf = nullptr;        // stage inputs of one segment, 4 C x NP x NPS per instance
  float2* d_lam = nullptr;
  float2* d_lc = nullptr;
  float2* d_gkt = nullptr;
  float2* d_macc = nullptr;
  int adj_smem = 0;
  // grid-wide GEMM schedule
  cublasContext* blas = nullptr;
  std::vector<lgb::GemmInstance> gemm;
  std::vector<lgb::GemmSplit> gsplit;     // split-precision operands (3xTF32 / 3xBF16 GEMM schedule)
  double2* d_gtmp = nullptr;
};

// ---- CUDA-graph step runner of the GEMM schedule (header-defined template) -------
namespace lgb {
template <typename F>
int run_steps(int nt, cudaStream_t st, cudaStream_t cap, F&& one_step, int graph_steps) {
  const int kGraphSteps = graph_steps > 0 ? graph_steps : 16;
  const int kGraphMin = 2 * kGraphSteps;
  if (cap == nullptr || nt < kGraphMin) {
    for (int s = 0; s < nt; ++s) {
      const int r = one_step(st);
      if (r != LGB_OK) return r;
    }
    return LGB_OK;
  }
  // capture `steps` steps on the private stream (nothing executes there) and
  // replay the instantiated graph on the caller's stream
  auto build = [&](int steps, cudaGraphExec_t* ex) -> int {
    if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return LGB_ERR_CUDA;
    int r = LGB_OK;
    for (int s = 0; s < steps && r == LGB_OK; ++s) r = one_step(cap);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(cap, &g);
    if (r != LGB_OK || e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return r != LGB_OK ? r : LGB_ERR_CUDA;
    }
    const cudaError_t ei = cudaGraphInstantiate(ex, g, 0);
    cudaGraphDestroy(g);
    return ei == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
  };
  const int S = nt < kGraphSteps ? nt : kGraphSteps;
  cudaGraphExec_t full = nullptr, rest = nullptr;
  int r = build(S, &full);
  if (r == LGB_OK && nt % S) r = build(nt % S, &rest);
  for (int k = 0; k < nt / S && r == LGB_OK; ++k)
    if (cudaGraphLaunch(full, st) != cudaSuccess) r = LGB_ERR_CUDA;
  if (r == LGB_OK && rest != nullptr && cudaGraphLaunch(rest, st) != cudaSuccess) r = LGB_ERR_CUDA;
  // an executable graph destroyed while in flight is freed when it completes
  if (full) cudaGraphExecDestroy(full);
  if (rest) cudaGraphExecDestroy(rest);
  return r;
}
}  // namespace lgb
