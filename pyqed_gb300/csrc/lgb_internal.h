// Internal plan structure and kernel launchers shared by the C-ABI layer.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "../../include/lindblad_gb300.h"
#include "lgb_common.cuh"

namespace lgb {

// ---- CTA-resident schedule (lgb_cta.cu) -------------------------------------
int cta_max_npad();
int cta_wide_max_npad();
size_t cta_elem_bytes(int precision);
cudaError_t launch_cta_rk4(const CtaParams& p, int precision, int n_blocks, cudaStream_t stream,
                           bool wide);

// ---- tensor-core CTA-resident schedule (lgb_tc.cu) --------------------------
int tc_max_dim();
int tc_smem_bytes(int precision, int npad);
cudaError_t launch_tc_rk4(const CtaParams& p, int precision, const int* order, int n_items,
                          int* queue, int grid, cudaStream_t stream);

// ---- operator preparation (lgb_setup.cu) -------------------------------------
struct SetupParams {
  int n_inst, n_cops, cops_kind, n_eops, n_drive, padc;
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
  int tc_smem = 0;
  int smem_w = 0;
  int n_sm = 0;
  cudaStream_t side[2] = {nullptr, nullptr};  // streams for kernels that run beside the first
  cudaEvent_t ev_fork = nullptr;
  cudaEvent_t ev_join[2] = {nullptr, nullptr};
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
  std::vector<void*> allocations;
};
