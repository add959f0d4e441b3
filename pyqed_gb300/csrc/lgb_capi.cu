// C-ABI entry points (include/lindblad_gb300.h): plan set-up, operator
// upload, propagation and error reporting.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <numeric>

#include <cublas_v2.h>

#include "lgb_internal.h"

using lgb::CtaParams;

namespace {

constexpr int kVersion = 1 * 10000 + 0 * 100 + 0;
constexpr int kSmemBudget = 224 * 1024;  // dynamic shared memory per CTA we plan with

int cuda_status(cudaError_t e) { return e == cudaSuccess ? LGB_OK : LGB_ERR_CUDA; }

template <typename P>
int dalloc(lgb_plan* pl, P** ptr, size_t bytes) {
  *ptr = nullptr;
  if (bytes == 0) return LGB_OK;
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) return LGB_ERR_CUDA;
  pl->allocations.push_back(p);
  pl->ws_bytes += bytes;
  *ptr = reinterpret_cast<P*>(p);
  return LGB_OK;
}

template <typename T>
int upload(lgb_plan* pl, T** dptr, const std::vector<T>& v) {
  int s = dalloc(pl, dptr, v.size() * sizeof(T));
  if (s != LGB_OK || v.empty()) return s;
  return cuda_status(cudaMemcpy(*dptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
}

void free_plan(lgb_plan* pl) {
  if (pl->blas) cublasDestroy(pl->blas);
  if (pl->cap_stream) cudaStreamDestroy(pl->cap_stream);
  pl->cap_stream = nullptr;
  pl->blas = nullptr;
  for (void* p : pl->allocations) cudaFree(p);
  pl->allocations.clear();
  for (int k = 0; k < 3; ++k) {
    if (pl->side[k]) cudaStreamDestroy(pl->side[k]);
    if (pl->ev_join[k]) cudaEventDestroy(pl->ev_join[k]);
    pl->side[k] = nullptr;
    pl->ev_join[k] = nullptr;
  }
  if (pl->ev_fork) cudaEventDestroy(pl->ev_fork);
  pl->ev_fork = nullptr;
}

int validate(const lgb_problem_t* pr, const int32_t* dims) {
  if (pr == nullptr || dims == nullptr) return LGB_ERR_INVALID_ARG;
  if (pr->n_inst < 1 || pr->n_cops < 0 || pr->n_eops < 0 || pr->n_eops > 16 || pr->n_drive < 0 ||
      pr->n_drive > 4 || pr->nt < 0 || pr->store_every < 0 ||
      (pr->flags & ~LGB_FLAG_ADJOINT) != 0 || pr->checkpoint_every < 0 || pr->reserved != 0)
    return LGB_ERR_INVALID_ARG;
  if (pr->flags & LGB_FLAG_ADJOINT) {
    // the adjoint runs on the FP32 CTA kernel with dense (or no) collapse operators
    if (pr->precision != LGB_PREC_FP32 || pr->cops_kind == LGB_COPS_DIAG || pr->store_every != 0 ||
        pr->schedule == LGB_SCHED_GEMM || pr->n_cops > 4)
      return LGB_ERR_UNSUPPORTED;
    for (int b = 0; b < pr->n_inst; ++b)
      if (dims[b] > 64) return LGB_ERR_UNSUPPORTED;
  }
  if (pr->cops_kind < LGB_COPS_NONE || pr->cops_kind > LGB_COPS_DIAG) return LGB_ERR_INVALID_ARG;
  if (pr->cops_kind == LGB_COPS_NONE && pr->n_cops != 0) return LGB_ERR_INVALID_ARG;
  if (pr->cops_kind != LGB_COPS_NONE && pr->n_cops == 0) return LGB_ERR_INVALID_ARG;
  if (pr->precision < LGB_PREC_FP64 || pr->precision > LGB_PREC_BF16X3) return LGB_ERR_INVALID_ARG;
  if (pr->schedule < LGB_SCHED_AUTO || pr->schedule > LGB_SCHED_GEMM) return LGB_ERR_INVALID_ARG;
  if (!(pr->dt == pr->dt)) return LGB_ERR_INVALID_ARG;
  for (int b = 0; b < pr->n_inst; ++b)
    if (dims[b] < 1 || dims[b] > 65536) return LGB_ERR_INVALID_ARG;
  return LGB_OK;
}

}  // namespace

extern "C" {

int lgb_get_version(void) { return kVersion; }

const char* lgb_status_string(int status) {
  switch (status) {
    case LGB_OK: return "ok";
    case LGB_ERR_INVALID_ARG: return "invalid argument";
    case LGB_ERR_UNSUPPORTED: return "unsupported by this build";
    case LGB_ERR_CUDA: return "CUDA runtime error";
    case LGB_ERR_NONFINITE: return "state became non-finite";
    case LGB_ERR_TIMEOUT: return "bounded device wait timed out";
    case LGB_ERR_NO_DEVICE: return "no CUDA device";
    case LGB_ERR_STATE: return "call order violated";
    case LGB_ERR_TOO_LARGE: return "size exceeds the no-allocation scratch limit";
    case LGB_ERR_CHECK: return "per-step trace/hermiticity check exceeded its tolerance";
    default: return "unknown status";
  }
}

int lgb_plan_create(lgb_plan_t* plan, const lgb_problem_t* problem, const int32_t* dims_host) {
  if (plan == nullptr) return LGB_ERR_INVALID_ARG;
  *plan = nullptr;
  int s = validate(problem, dims_host);
  if (s != LGB_OK) return s;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return LGB_ERR_NO_DEVICE;
  }
  lgb_plan* pl = new (std::nothrow) lgb_plan();
  if (pl == nullptr) return LGB_ERR_INVALID_ARG;
  pl->prob = *problem;
  cudaGetDevice(&pl->device);
  const lgb_problem_t& pr = pl->prob;
  const int n = pr.n_inst;
  const int prec = pr.precision;
  const size_t esz = lgb::cta_elem_bytes(prec == LGB_PREC_FP64 ? 0 : 1);
  pl->padc = (int)(16 / esz);

  pl->dims.assign(dims_host, dims_host + n);
  pl->npad.resize(n);
  pl->off.resize(n);
  pl->doff.resize(n);
  pl->woff.resize(n);
  pl->soff.resize(n);
  pl->place.assign(n, 0);
  pl->adjoint = (pr.flags & LGB_FLAG_ADJOINT) != 0;
  if (pl->adjoint) {
    int c = pr.checkpoint_every;
    if (c <= 0) c = std::max(1, (int)std::lround(std::sqrt((double)std::max(pr.nt, 1))));
    pl->ckpt_every = c;
    pl->n_store = pr.nt / c;  // checkpoints rho_C, rho_2C, ...
  } else {
    pl->n_store = pr.store_every > 0 ? pr.nt / pr.store_every : 0;
  }
  const int K = pr.n_cops;
  const bool dense = pr.cops_kind == LGB_COPS_DENSE;
  const bool split = prec == LGB_PREC_TF32X3 || prec == LGB_PREC_BF16X3;
  cudaDeviceGetAttribute(&pl->n_sm, cudaDevAttrMultiProcessorCount, pl->device);

  // Tensor-core kernel: N <= 64 (padded to a multiple of 16), and N = 65 with
  // a static H (a 64 x 64 block plus a SIMT border, padded to 68); no dense
  // collapse operators (those keep the FP32 CTA kernel).
  std::vector<char> on_tc(n, 0);
  for (int b = 0; b < n; ++b)
    on_tc[b] = split && !dense && pr.schedule != LGB_SCHED_GEMM &&
               (pl->dims[b] <= lgb::tc_max_dim() || (pl->dims[b] == lgb::tc_border_dim() && pr.n_drive == 0));
  for (int b = 0; b < n; ++b) {
    const long long N = pl->dims[b];
    const int NP = !on_tc[b] ? (int)((N + 3) / 4 * 4)
                             : (N > lgb::tc_max_dim() ? lgb::kTcBorderNpad : (int)((N + 15) / 16 * 16));
    pl->npad[b] = NP;
    pl->off[b] = pl->tot_off;
    pl->doff[b] = pl->tot_doff;
    pl->woff[b] = pl->tot_woff;
    // user states: per instance contiguous; adjoint checkpoints: [n_ckpt][packed]
    pl->soff[b] = pl->adjoint ? pl->tot_off : pl->n_store * pl->tot_off;
    pl->tot_off += N * N;
    pl->tot_doff += N;
    pl->tot_woff += (long long)NP * (NP + pl->padc);
    pl->flops_per_step += 64LL * (1 + (dense ? K : 0)) * N * N * N;
  }

  // ---- schedule ---------------------------------------------------------------
  // The CTA-resident kernels need the instance in shared memory; anything
  // larger goes to the grid-wide GEMM schedule.
  int sched = pr.schedule;
  bool cta_ok = true;
  int smem = 0, smem_w = 0, tc_smem = 0, tc_maxnp = 0;
  std::vector<char> wide(n, 0);
  for (int b = 0; b < n && cta_ok; ++b) {
    if (on_tc[b]) {
      if (pl->npad[b] != lgb::kTcBorderNpad) tc_maxnp = std::max(tc_maxnp, pl->npad[b]);
      continue;
    }
    if (pl->npad[b] > lgb::cta_max_npad()) {
      cta_ok = false;
      break;
    }
    // FP32 instances with 64 < N <= 76 take the 384-thread single-round block
    wide[b] = prec != LGB_PREC_FP64 && pl->npad[b] > 64 && pl->npad[b] <= lgb::cta_wide_max_npad();
    const long long ms = (long long)pl->npad[b] * (pl->npad[b] + pl->padc) * esz;
    long long used = 3 * ms;
    unsigned char pf = 0;
    if (used > kSmemBudget) {
      cta_ok = false;
      break;
    }
    if (dense) {
      if (used + K * ms <= kSmemBudget) {
        used += K * ms;
        pf |= 2;
      }
      if (used + K * ms <= kSmemBudget) {
        used += K * ms;
        pf |= 1;
      }
    }
    pl->place[b] = pf;
    if (wide[b]) {
      smem_w = std::max<long long>(smem_w, used);
    } else {
      smem = std::max<long long>(smem, used);
    }
  }
  if (tc_maxnp > 0) tc_smem = lgb::tc_smem_bytes(prec, tc_maxnp);
  pl->tcb_smem = lgb::tc_smem_bytes(prec, lgb::kTcBorderNpad);
  if (sched == LGB_SCHED_AUTO) sched = cta_ok ? LGB_SCHED_CTA : LGB_SCHED_GEMM;
  if (sched == LGB_SCHED_CTA && !cta_ok) {
    delete pl;
    return LGB_ERR_UNSUPPORTED;
  }
  pl->schedule = sched;
  pl->smem_bytes = smem;
  pl->smem_w = smem_w;
  pl->tc_smem = tc_smem;

  // Largest instances first: with one CTA per instance the hardware block
  // scheduler then performs longest-processing-time-first list scheduling;
  // the tensor-core kernel's work queue hands them out in the same order.
  for (int b = 0; b < n; ++b)
    (on_tc[b] ? (pl->npad[b] == lgb::kTcBorderNpad ? pl->tcb_order : pl->tc_order)
              : (wide[b] ? pl->order_w : pl->order)).push_back(b);
  auto by_size = [&](int a, int c) { return pl->dims[a] > pl->dims[c]; };
  std::stable_sort(pl->order.begin(), pl->order.end(), by_size);
  std::stable_sort(pl->order_w.begin(), pl->order_w.end(), by_size);
  std::stable_sort(pl->tc_order.begin(), pl->tc_order.end(), by_size);
  if (sched == LGB_SCHED_GEMM) {
    // every instance goes through the GEMM schedule, in order
    pl->order.clear();
    pl->order_w.clear();
    pl->tc_order.clear();
    pl->tcb_order.clear();
  }
  const int n_launch = (pl->order.empty() ? 0 : 1) + (pl->order_w.empty() ? 0 : 1) +
                       (pl->tc_order.empty() ? 0 : 1) + (pl->tcb_order.empty() ? 0 : 1);
  bool ok = cudaEventCreateWithFlags(&pl->ev_fork, cudaEventDisableTiming) == cudaSuccess;
  for (int k = 0; k + 1 < n_launch && ok; ++k) {
    ok = cudaStreamCreateWithFlags(&pl->side[k], cudaStreamNonBlocking) == cudaSuccess &&
         cudaEventCreateWithFlags(&pl->ev_join[k], cudaEventDisableTiming) == cudaSuccess;
  }
  if (!ok) {
    free_plan(pl);
    delete pl;
    return LGB_ERR_CUDA;
  }

  // ---- device buffers ---------------------------------------------------------
  s = LGB_OK;
  const long long W = pl->tot_woff;
  s = s ? s : upload(pl, &pl->d_dims, pl->dims);
  s = s ? s : upload(pl, &pl->d_npad, pl->npad);
  s = s ? s : upload(pl, &pl->d_order, pl->order);
  s = s ? s : upload(pl, &pl->d_order_w, pl->order_w);
  s = s ? s : upload(pl, &pl->d_tc_order, pl->tc_order);
  s = s ? s : upload(pl, &pl->d_tcb_order, pl->tcb_order);
  s = s ? s : dalloc(pl, &pl->d_queue, sizeof(int));
  s = s ? s : upload(pl, &pl->d_off, pl->off);
  s = s ? s : upload(pl, &pl->d_doff, pl->doff);
  s = s ? s : upload(pl, &pl->d_woff, pl->woff);
  s = s ? s : upload(pl, &pl->d_soff, pl->soff);
  s = s ? s : upload(pl, &pl->d_place, pl->place);
  s = s ? s : dalloc(pl, &pl->d_shift, n * sizeof(double));
  s = s ? s : dalloc(pl, &pl->d_At, W * esz);
  s = s ? s : dalloc(pl, &pl->d_Lt, dense ? (size_t)K * W * esz : 0);
  s = s ? s : dalloc(pl, &pl->d_Dm, pr.cops_kind == LGB_COPS_DIAG ? W * esz : 0);
  s = s ? s : dalloc(pl, &pl->d_Gt, (size_t)pr.n_drive * W * esz);
  s = s ? s : dalloc(pl, &pl->d_Ot, (size_t)pr.n_eops * W * sizeof(double2));
  s = s ? s : dalloc(pl, &pl->d_OtF, prec == LGB_PREC_FP64 ? 0 : (size_t)pr.n_eops * W * sizeof(float2));
  s = s ? s : dalloc(pl, &pl->d_state, 2 * W * esz);
  s = s ? s : dalloc(pl, &pl->d_y, dense ? (size_t)K * W * esz : 0);
  s = s ? s : dalloc(pl, &pl->d_err, n * sizeof(int));
  s = s ? s : dalloc(pl, &pl->d_chk, 2 * n * sizeof(double));
  s = s ? s : dalloc(pl, &pl->d_chkws, sched == LGB_SCHED_GEMM ? 8 * n * sizeof(double) : 0);
  if (s == LGB_OK && pl->d_err) s = cuda_status(cudaMemset(pl->d_err, 0, n * sizeof(int)));
  if (s == LGB_OK && pl->adjoint) {
    const long long W = pl->tot_woff;
    const int C = pl->ckpt_every;
    s = s ? s : dalloc(pl, &pl->d_ckpt, (size_t)std::max<long long>(pl->n_store, 1) * pl->tot_off * sizeof(double2));
    s = s ? s : dalloc(pl, &pl->d_ybuf, (size_t)4 * C * W * sizeof(float2));
    s = s ? s : dalloc(pl, &pl->d_lam, (size_t)W * sizeof(float2));
    s = s ? s : dalloc(pl, &pl->d_lc, (size_t)std::max(K, 1) * W * sizeof(float2));
    s = s ? s : dalloc(pl, &pl->d_gkt, (size_t)std::max(K, 1) * W * sizeof(float2));
    s = s ? s : dalloc(pl, &pl->d_macc, (size_t)W * sizeof(float2));
    int maxnp = 0;
    for (int b = 0; b < n; ++b) maxnp = std::max(maxnp, pl->npad[b]);
    pl->adj_smem = lgb::adjoint_smem_bytes(maxnp, K);
  }
  if (s == LGB_OK && sched == LGB_SCHED_GEMM) {
    // per-instance operand slabs of the GEMM schedule (working precision)
    const int E = pr.n_eops, D = pr.n_drive;
    const int Kd = dense ? K : 0;
    int maxn = 0;
    for (int b = 0; b < n; ++b) maxn = std::max(maxn, pl->dims[b]);
    double2* partial = nullptr;
    int* counter = nullptr;
    const size_t slots = split ? std::max(lgb::gemm_partial_slots(maxn), lgb::split_partial_slots(maxn))
                               : lgb::gemm_partial_slots(maxn);
    s = s ? s : dalloc(pl, &partial, (size_t)std::max(E, 1) * slots * sizeof(double2));
    s = s ? s : dalloc(pl, &counter, sizeof(int));
    if (s == LGB_OK) s = cuda_status(cudaMemset(counter, 0, sizeof(int)));
    s = s ? s : dalloc(pl, &pl->d_gtmp, dense ? (size_t)maxn * maxn * sizeof(double2) : 0);
    pl->gemm.resize(n);
    for (int b = 0; b < n && s == LGB_OK; ++b) {
      lgb::GemmInstance& g = pl->gemm[b];
      const size_t NN = (size_t)pl->dims[b] * pl->dims[b];
      g.N = pl->dims[b];
      g.W = (Kd + 2) * g.N;
      s = s ? s : dalloc(pl, &g.Lbuf, NN * (Kd + 2) * esz);
      s = s ? s : dalloc(pl, &g.Rbuf, NN * (Kd + 2) * esz);
      s = s ? s : dalloc(pl, &g.Rout, NN * esz);
      s = s ? s : dalloc(pl, &g.Lstk, NN * Kd * esz);
      s = s ? s : dalloc(pl, &g.Dm, pr.cops_kind == LGB_COPS_DIAG ? NN * esz : 0);
      s = s ? s : dalloc(pl, &g.A0, D > 0 ? NN * esz : 0);
      s = s ? s : dalloc(pl, &g.Gd, NN * D * esz);
      s = s ? s : dalloc(pl, &g.rho, NN * esz);
      s = s ? s : dalloc(pl, &g.racc, NN * esz);
      s = s ? s : dalloc(pl, &g.Ot, NN * E * sizeof(double2));
      g.partial = partial;
      g.counter = counter;
      g.err = pl->d_err + b;
    }
    if (split) {
      // split operands: interleaved hi/lo arrays padded to NP = 128 k
      const bool bf16 = prec == LGB_PREC_BF16X3;
      const size_t ses = bf16 ? 2 : 4;
      pl->gsplit.resize(n);
      for (int b = 0; b < n && s == LGB_OK; ++b) {
        lgb::GemmSplit& q = pl->gsplit[b];
        q.NP = lgb::split_padded_dim(pl->dims[b]);
        q.Wp = (long long)(Kd + 2) * q.NP;
        q.bf16 = bf16;
        for (int l = 0; l < 2; ++l) {
          s = s ? s : dalloc(pl, &q.Ls[l], (size_t)2 * q.NP * q.Wp * ses);
          s = s ? s : dalloc(pl, &q.Rs[l], (size_t)2 * q.NP * q.Wp * ses);
          s = s ? s : dalloc(pl, &q.Lks[l], (size_t)Kd * 2 * q.NP * q.NP * ses);
        }
        if (q.NP <= 256) {
          // the persistent kernel's blocked operands (two copies of Ls and Rs)
          for (int l = 0; l < 2; ++l) {
            s = s ? s : dalloc(pl, &q.Lsb[l], (size_t)2 * 2 * q.NP * q.Wp * ses);
            s = s ? s : dalloc(pl, &q.Rsb[l], (size_t)2 * 2 * q.NP * q.Wp * ses);
            s = s ? s : dalloc(pl, &q.Lksb[l], (size_t)Kd * 2 * q.NP * q.NP * ses);
          }
          s = s ? s : dalloc(pl, &q.bar, sizeof(unsigned));
          s = s ? s : dalloc(pl, &q.part, (size_t)lgb::persist_part_elems(q.NP) * sizeof(double2));
        }
        s = s ? s : dalloc(pl, &q.Tpart, Kd ? lgb::split_tpart_elems(q.NP, Kd, 2 * pl->n_sm, bf16) * sizeof(float2) : 0);
        s = s ? s : dalloc(pl, &q.Rpart, lgb::split_rpart_elems(q.NP, Kd, 2 * pl->n_sm, bf16) * sizeof(float2));
        s = s ? s : dalloc(pl, &q.kc, (size_t)pl->dims[b] * pl->dims[b] * sizeof(float2));
      }
    }
    if (s == LGB_OK) {
      if (cublasCreate(&pl->blas) != CUBLAS_STATUS_SUCCESS) {
        pl->blas = nullptr;
        s = LGB_ERR_CUDA;
      } else {
        // plain library GEMMs: no reduced-precision tensor-op substitutions
        cublasSetMathMode(pl->blas, CUBLAS_PEDANTIC_MATH);
      }
    }
    // step counter, a private capture stream and a fixed cuBLAS workspace, so
    // that blocks of RK4 steps can be captured into CUDA graphs
    constexpr size_t kBlasWs = 32u << 20;
    s = s ? s : dalloc(pl, &pl->d_ctr, sizeof(int));
    s = s ? s : dalloc(pl, &pl->blas_ws, kBlasWs);
    if (s == LGB_OK && cublasSetWorkspace(pl->blas, pl->blas_ws, kBlasWs) != CUBLAS_STATUS_SUCCESS)
      s = LGB_ERR_CUDA;
    if (s == LGB_OK && cudaStreamCreateWithFlags(&pl->cap_stream, cudaStreamNonBlocking) != cudaSuccess) {
      pl->cap_stream = nullptr;
      s = LGB_ERR_CUDA;
    }
  }
  if (s != LGB_OK) {
    free_plan(pl);
    delete pl;
    return s;
  }
  *plan = pl;
  return LGB_OK;
}

int lgb_plan_destroy(lgb_plan_t plan) {
  if (plan == nullptr) return LGB_ERR_INVALID_ARG;
  free_plan(plan);
  delete plan;
  return LGB_OK;
}

int lgb_plan_set_operators(lgb_plan_t plan, const double* H, const double* cops,
                           const double* eops, const double* drive_ops, void* stream) {
  if (plan == nullptr || H == nullptr) return LGB_ERR_INVALID_ARG;
  const lgb_problem_t& pr = plan->prob;
  if (pr.n_cops > 0 && cops == nullptr) return LGB_ERR_INVALID_ARG;
  if (pr.n_eops > 0 && eops == nullptr) return LGB_ERR_INVALID_ARG;
  if (pr.n_drive > 0 && drive_ops == nullptr) return LGB_ERR_INVALID_ARG;
  lgb::SetupParams sp{};
  sp.n_inst = pr.n_inst;
  sp.n_cops = pr.n_cops;
  sp.cops_kind = pr.cops_kind;
  sp.n_eops = pr.n_eops;
  sp.n_drive = pr.n_drive;
  sp.padc = plan->padc;
  sp.max_npad = 0;
  for (int np_ : plan->npad) sp.max_npad = std::max(sp.max_npad, np_);
  sp.dims = plan->d_dims;
  sp.npad = plan->d_npad;
  sp.off = plan->d_off;
  sp.doff = plan->d_doff;
  sp.woff = plan->d_woff;
  sp.H = reinterpret_cast<const double2*>(H);
  sp.cops = reinterpret_cast<const double2*>(cops);
  sp.eops = reinterpret_cast<const double2*>(eops);
  sp.dops = reinterpret_cast<const double2*>(drive_ops);
  sp.shift = plan->d_shift;
  sp.At = plan->d_At;
  sp.Lt = plan->d_Lt;
  sp.Dm = plan->d_Dm;
  sp.Gt = plan->d_Gt;
  sp.Ot = plan->d_Ot;
  sp.OtF = plan->d_OtF;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  plan->last_stream = st;
  int s = LGB_OK;
  if (plan->schedule == LGB_SCHED_GEMM) {
    s = cuda_status(lgb::launch_trace_shift(sp, st));
    const int K = pr.n_cops;
    for (int b = 0; b < pr.n_inst && s == LGB_OK; ++b) {
      const long long o = plan->off[b];
      lgb::GemmSetupArgs a;
      a.g = plan->gemm[b];
      a.blas = plan->blas;
      a.fp64 = pr.precision == LGB_PREC_FP64;
      a.H = sp.H + o;
      a.cops = pr.cops_kind == LGB_COPS_DENSE ? sp.cops + K * o
               : pr.cops_kind == LGB_COPS_DIAG ? sp.cops + K * plan->doff[b] : nullptr;
      a.eops = pr.n_eops ? sp.eops + (long long)pr.n_eops * o : nullptr;
      a.dops = pr.n_drive ? sp.dops + (long long)pr.n_drive * o : nullptr;
      a.cops_kind = pr.cops_kind;
      a.K = K;
      a.E = pr.n_eops;
      a.D = pr.n_drive;
      a.shift = plan->d_shift + b;
      a.doff = 0;
      a.Gtmp = plan->d_gtmp;
      s = lgb::gemm_setup(a, st);
      if (s == LGB_OK && !plan->gsplit.empty())
        s = lgb::split_setup(plan->gsplit[b], plan->gemm[b], pr.cops_kind == LGB_COPS_DENSE ? K : 0,
                             pr.precision == LGB_PREC_BF16X3, plan->n_sm * plan->opt_waves, st);
    }
  } else {
    s = cuda_status(lgb::launch_setup(sp, pr.precision == LGB_PREC_FP64 ? 0 : 1, st));
  }
  if (s == LGB_OK) plan->ops_set = true;
  return s;
}

int lgb_plan_propagate(lgb_plan_t plan, const double* rho0, const double* drive_samples,
                       double* obs_out, double* rho_out, double* states_out, void* stream) {
  if (plan == nullptr || rho0 == nullptr) return LGB_ERR_INVALID_ARG;
  if (!plan->ops_set) return LGB_ERR_STATE;
  const lgb_problem_t& pr = plan->prob;
  if (pr.n_drive > 0 && pr.nt > 0 && drive_samples == nullptr) return LGB_ERR_INVALID_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  plan->last_stream = st;
  CtaParams p{};
  p.tc_pairs = plan->opt_pairs;
  p.test_stall = plan->opt_stall;
  p.check_tol = plan->opt_check > 0 ? std::pow(10.0, -plan->opt_check) : 0.0;
  p.chk = plan->d_chk;
  p.spin = plan->opt_stall ? 4096 : 0;  // the test hook's waits give up after 4096 polls
  p.n_inst = pr.n_inst;
  p.n_cops = pr.n_cops;
  p.cops_kind = pr.cops_kind;
  p.n_eops = pr.n_eops;
  p.n_drive = pr.n_drive;
  p.nt = pr.nt;
  p.obs_t0 = pr.obs_t0;
  p.store_every = pr.store_every;
  p.drive_shared = pr.drive_shared;
  p.dt = pr.dt;
  p.order = plan->d_order;
  p.dims = plan->d_dims;
  p.npad = plan->d_npad;
  p.off = plan->d_off;
  p.woff = plan->d_woff;
  p.soff = plan->d_soff;
  p.place = plan->d_place;
  p.At = plan->d_At;
  p.Lt = plan->d_Lt;
  p.Dm = plan->d_Dm;
  p.Gt = plan->d_Gt;
  p.Ot = plan->d_Ot;
  p.OtF = plan->d_OtF;
  p.drive = drive_samples;
  p.rho0 = reinterpret_cast<const double2*>(rho0);
  p.obs_out = reinterpret_cast<double2*>(obs_out);
  p.rho_out = reinterpret_cast<double2*>(rho_out);
  p.states_out = reinterpret_cast<double2*>(states_out);
  p.state_ws = plan->d_state;
  p.y_ws = plan->d_y;
  p.err = plan->d_err;
  if (plan->adjoint) {
    // checkpoints for lgb_plan_adjoint: rho_C, rho_2C, ... for the whole batch
    if (states_out != nullptr) return LGB_ERR_INVALID_ARG;
    p.store_every = plan->ckpt_every;
    p.states_out = plan->d_ckpt;
    p.state_stride = plan->tot_off;
  }
  if (plan->schedule == LGB_SCHED_GEMM) {
    cudaMemsetAsync(plan->d_err, 0, pr.n_inst * sizeof(int), st);
    const long long nrows = (long long)pr.nt + pr.obs_t0;
    for (int b = 0; b < pr.n_inst; ++b) {
      lgb::GemmRunArgs a;
      a.g = plan->gemm[b];
      a.blas = plan->blas;
      a.fp64 = pr.precision == LGB_PREC_FP64;
      a.split = !plan->gsplit.empty();
      if (a.split) a.sp = plan->gsplit[b];
      a.ctr = plan->d_ctr;
      a.cap = plan->cap_stream;
      a.Kdense = pr.cops_kind == LGB_COPS_DENSE ? pr.n_cops : 0;
      a.D = pr.n_drive;
      a.E = pr.n_eops;
      a.nt = pr.nt;
      a.obs_t0 = pr.obs_t0;
      a.store_every = pr.store_every;
      a.diag = pr.cops_kind == LGB_COPS_DIAG && pr.n_cops > 0;
      a.dt = pr.dt;
      a.rho0 = p.rho0 + plan->off[b];
      a.drive = pr.n_drive ? drive_samples + (pr.drive_shared ? 0 : (long long)b * pr.n_drive * pr.nt) : nullptr;
      a.obs_out = p.obs_out ? p.obs_out + (long long)b * nrows * pr.n_eops : nullptr;
      a.rho_out = p.rho_out ? p.rho_out + plan->off[b] : nullptr;
      a.states_out = p.states_out ? p.states_out + plan->soff[b] : nullptr;
      a.graph_steps = plan->opt_gsteps;
      a.persist = plan->opt_persist != 0;
      a.check_tol = p.check_tol;
      a.chk = plan->d_chk + 2 * b;
      a.chk_ws = plan->d_chkws + 8 * b;
      const int r = lgb::gemm_propagate(a, st);
      if (r != LGB_OK) return r;
    }
    return LGB_OK;
  }
  // Up to four kernels (tensor-core border, wide FP32 CTA, FP32 CTA,
  // tensor-core) cover the batch; the first runs on the caller's stream, the
  // others on forked streams joined back before return.
  struct Launch {
    int kind;  // 0 tensor core, 1 CTA, 2 wide CTA, 3 tensor-core border
    int count;
  };
  Launch ls[4];
  int nl = 0;
  // The per-instance kernels hold the longest single instances; they are
  // launched first so that their blocks are resident from the start, and the
  // persistent tensor-core blocks fill the remaining SMs from the work queue.
  if (!plan->tcb_order.empty()) ls[nl++] = {3, (int)plan->tcb_order.size()};
  if (!plan->order_w.empty()) ls[nl++] = {2, (int)plan->order_w.size()};
  if (!plan->order.empty()) ls[nl++] = {1, (int)plan->order.size()};
  if (!plan->tc_order.empty()) ls[nl++] = {0, (int)plan->tc_order.size()};
  const int wprec = pr.precision == LGB_PREC_FP64 ? 0 : 1;
  cudaError_t e = cudaSuccess;
  if (nl > 1) {
    e = cudaEventRecord(plan->ev_fork, st);
    for (int k = 1; k < nl && e == cudaSuccess; ++k)
      e = cudaStreamWaitEvent(plan->side[k - 1], plan->ev_fork, 0);
  }
  for (int k = 0; k < nl && e == cudaSuccess; ++k) {
    cudaStream_t s_k = k == 0 ? st : plan->side[k - 1];
    if (ls[k].kind == 0) {
      p.smem_bytes = plan->tc_smem;
      e = lgb::launch_tc_rk4(p, pr.precision, plan->d_tc_order, ls[k].count, plan->d_queue,
                             std::min(plan->n_sm, ls[k].count), s_k);
    } else if (ls[k].kind == 3) {
      p.smem_bytes = plan->tcb_smem;
      e = lgb::launch_tc_border(p, pr.precision, plan->d_tcb_order, ls[k].count, s_k);
    } else {
      p.order = ls[k].kind == 1 ? plan->d_order : plan->d_order_w;
      p.smem_bytes = ls[k].kind == 1 ? plan->smem_bytes : plan->smem_w;
      e = lgb::launch_cta_rk4(p, wprec, ls[k].count, s_k, ls[k].kind == 2);
    }
    if (e == cudaSuccess && k > 0) e = cudaEventRecord(plan->ev_join[k - 1], s_k);
  }
  for (int k = 1; k < nl && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(st, plan->ev_join[k - 1], 0);
  return cuda_status(e);
}

int lgb_plan_adjoint(lgb_plan_t plan, const double* rho0, const double* drive,
                     const double* obs_grad, double* dE_out, double* dscale_out, double* dH_out,
                     double* drho0_out, void* stream) {
  if (plan == nullptr || rho0 == nullptr) return LGB_ERR_INVALID_ARG;
  if (!plan->adjoint) return LGB_ERR_STATE;
  if (!plan->ops_set) return LGB_ERR_STATE;
  const lgb_problem_t& pr = plan->prob;
  if (pr.n_drive > 0 && pr.nt > 0 && drive == nullptr) return LGB_ERR_INVALID_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  plan->last_stream = st;
  const int n = pr.n_inst;
  const int K = pr.cops_kind == LGB_COPS_DENSE ? pr.n_cops : 0;
  const int C = plan->ckpt_every;
  const int nseg = (pr.nt + C - 1) / C;
  cudaError_t e = cudaSuccess;
  if (dscale_out != nullptr && K > 0) e = cudaMemsetAsync(dscale_out, 0, (size_t)n * K * sizeof(double), st);
  if (dE_out != nullptr && pr.n_drive > 0 && e == cudaSuccess)
    e = cudaMemsetAsync(dE_out, 0, (size_t)n * pr.n_drive * pr.nt * sizeof(double), st);
  if (e != cudaSuccess) return LGB_ERR_CUDA;

  CtaParams f{};  // recompute pass: the forward kernel recording stage inputs
  f.n_inst = n;
  f.n_cops = pr.n_cops;
  f.cops_kind = pr.cops_kind;
  f.n_eops = 0;
  f.n_drive = pr.n_drive;
  f.obs_t0 = 0;
  f.store_every = 0;
  f.drive_shared = pr.drive_shared;
  f.dt = pr.dt;
  f.order = plan->d_order;
  f.dims = plan->d_dims;
  f.npad = plan->d_npad;
  f.off = plan->d_off;
  f.woff = plan->d_woff;
  f.soff = plan->d_soff;
  f.place = plan->d_place;
  f.At = plan->d_At;
  f.Lt = plan->d_Lt;
  f.Dm = plan->d_Dm;
  f.Gt = plan->d_Gt;
  f.Ot = plan->d_Ot;
  f.OtF = plan->d_OtF;
  f.state_ws = plan->d_state;
  f.y_ws = plan->d_y;
  f.err = plan->d_err;
  f.smem_bytes = plan->smem_bytes;
  f.drive_ld = pr.nt;
  f.ystore = plan->d_ybuf;
  f.ycap = C;

  lgb::AdjParams a{};
  a.n_inst = n;
  a.n_cops = K;
  a.n_drive = pr.n_drive;
  a.n_eops = pr.n_eops;
  a.nt = pr.nt;
  a.ycap = C;
  a.drive_ld = pr.nt;
  a.drive_shared = pr.drive_shared;
  a.obs_t0 = pr.obs_t0;
  a.smem_bytes = plan->adj_smem;
  a.dt = pr.dt;
  a.order = plan->d_order;
  a.dims = plan->d_dims;
  a.npad = plan->d_npad;
  a.woff = plan->d_woff;
  a.At = reinterpret_cast<const float2*>(plan->d_At);
  a.Gt = reinterpret_cast<const float2*>(plan->d_Gt);
  a.Lt = reinterpret_cast<const float2*>(plan->d_Lt);
  a.Lc = plan->d_lc;
  a.GkT = plan->d_gkt;
  a.Macc = plan->d_macc;
  a.lam = plan->d_lam;
  a.ys = reinterpret_cast<const float2*>(plan->d_ybuf);
  a.Ot = plan->d_Ot;
  a.drive = drive;
  a.obs_grad = reinterpret_cast<const double2*>(obs_grad);
  a.dE = dE_out;
  a.dscale = dscale_out;
  for (int sg = nseg - 1; sg >= 0 && e == cudaSuccess; --sg) {
    const int seg0 = sg * C;
    const int len = std::min(C, pr.nt - seg0);
    f.nt = len;
    f.rho0 = sg == 0 ? reinterpret_cast<const double2*>(rho0)
                     : plan->d_ckpt + (long long)(sg - 1) * plan->tot_off;
    f.drive = drive != nullptr ? drive + seg0 : nullptr;
    e = lgb::launch_cta_rk4(f, 1, n, st, false);
    a.seg0 = seg0;
    a.seg_len = len;
    a.first_segment = sg == nseg - 1;
    if (e == cudaSuccess) e = lgb::launch_adjoint_segment(a, n, st);
  }
  if (e == cudaSuccess && (drho0_out != nullptr || dH_out != nullptr))
    e = lgb::launch_adjoint_finish(a, plan->d_off, reinterpret_cast<double2*>(drho0_out),
                                   reinterpret_cast<double2*>(dH_out), st);
  return cuda_status(e);
}

int lgb_plan_errors(lgb_plan_t plan, int32_t* flags_host) {
  if (plan == nullptr || flags_host == nullptr) return LGB_ERR_INVALID_ARG;
  cudaError_t e = cudaStreamSynchronize(plan->last_stream);
  if (e != cudaSuccess) return LGB_ERR_CUDA;
  e = cudaMemcpy(flags_host, plan->d_err, plan->prob.n_inst * sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return LGB_ERR_CUDA;
  for (int b = 0; b < plan->prob.n_inst; ++b)
    if (flags_host[b] != LGB_OK) return flags_host[b];
  return LGB_OK;
}

int lgb_plan_check_stats(lgb_plan_t plan, double* stats_host) {
  if (plan == nullptr || stats_host == nullptr) return LGB_ERR_INVALID_ARG;
  if (plan->opt_check == 0) return LGB_ERR_STATE;
  cudaError_t e = cudaStreamSynchronize(plan->last_stream);
  if (e != cudaSuccess) return LGB_ERR_CUDA;
  e = cudaMemcpy(stats_host, plan->d_chk, 2 * plan->prob.n_inst * sizeof(double), cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? LGB_OK : LGB_ERR_CUDA;
}

int lgb_plan_set_option(lgb_plan_t plan, int32_t option, int32_t value) {
  if (plan == nullptr) return LGB_ERR_INVALID_ARG;
  switch (option) {
    case LGB_OPT_CHECK:
      if (value < 0 || value > 15) return LGB_ERR_INVALID_ARG;
      plan->opt_check = value;
      return LGB_OK;
    case LGB_OPT_TC_PAIRS:
      if (value != 0 && value != 1) return LGB_ERR_INVALID_ARG;
      plan->opt_pairs = value;
      return LGB_OK;
    case LGB_OPT_GEMM_WAVES: {
      if (value != 1 && value != 2) return LGB_ERR_INVALID_ARG;
      plan->opt_waves = value;
      const int Kd = plan->prob.cops_kind == LGB_COPS_DENSE ? plan->prob.n_cops : 0;
      for (auto& q : plan->gsplit) lgb::split_set_ksplit(q, Kd, plan->n_sm * value, plan->opt_kcap);
      return LGB_OK;
    }
    case LGB_OPT_GEMM_KSPLIT: {
      if (value != 0 && (value < 1 || value > 64 || (value & (value - 1)) != 0)) return LGB_ERR_INVALID_ARG;
      plan->opt_kcap = value;
      const int Kd = plan->prob.cops_kind == LGB_COPS_DENSE ? plan->prob.n_cops : 0;
      for (auto& q : plan->gsplit) lgb::split_set_ksplit(q, Kd, plan->n_sm * plan->opt_waves, value);
      return LGB_OK;
    }
    case LGB_OPT_GRAPH_STEPS:
      if (value < 1 || value > 64) return LGB_ERR_INVALID_ARG;
      plan->opt_gsteps = value;
      return LGB_OK;
    case LGB_OPT_TEST_STALL:
      if (value != 0 && value != 1) return LGB_ERR_INVALID_ARG;
      plan->opt_stall = value;
      return LGB_OK;
    case LGB_OPT_GEMM_PERSIST:
      if (value != 0 && value != 1) return LGB_ERR_INVALID_ARG;
      plan->opt_persist = value;
      return LGB_OK;
    default:
      return LGB_ERR_INVALID_ARG;
  }
}

int lgb_plan_get_info(lgb_plan_t plan, lgb_plan_info_t* info) {
  if (plan == nullptr || info == nullptr) return LGB_ERR_INVALID_ARG;
  info->schedule = plan->schedule;
  info->precision = plan->prob.precision;
  info->smem_bytes = std::max(std::max(plan->smem_bytes, plan->smem_w),
                              plan->tcb_order.empty() ? plan->tc_smem : std::max(plan->tc_smem, plan->tcb_smem));
  info->launches_per_propagate = (plan->order.empty() ? 0 : 1) + (plan->order_w.empty() ? 0 : 1) +
                                 (plan->tc_order.empty() ? 0 : 1) + (plan->tcb_order.empty() ? 0 : 1);
  info->persistent_instances = 0;
  info->reserved = 0;
  if (plan->schedule == LGB_SCHED_GEMM) {
    // per instance: init (+ t0 observables) + per step (drive) + 4 x (G1, G2, epilogue);
    // split precision: init also converts X (2 kernels), the drive step also
    // converts A and A^dag (2), and G1 has its split consumer
    const lgb_problem_t& pr = plan->prob;
    const bool split = !plan->gsplit.empty();
    const bool dense = pr.cops_kind == LGB_COPS_DENSE;
    const int per_stage = (dense ? (split ? 2 : 1) : 0) + 2;
    const int per_drive = pr.n_drive > 0 ? (split ? 3 : 1) : 0;
    const int init = 1 + (split ? 2 : 0) + (pr.obs_t0 && pr.n_eops ? 1 : 0);
    // (+1 per step: the step-counter increment; steps run as CUDA-graph replays when nt >= 32)
    int n_ps = 0;
    if (split && plan->opt_persist && pr.n_drive == 0 && pr.nt > 0)
      for (const auto& q : plan->gsplit) n_ps += q.persist ? 1 : 0;
    info->persistent_instances = n_ps;
    info->launches_per_propagate =
        (pr.n_inst - n_ps) * (init + pr.nt * (4 * per_stage + per_drive + 1)) + n_ps * (init + 1);
  }
  info->workspace_bytes = (int64_t)plan->ws_bytes;
  info->flops_per_step = plan->flops_per_step;
  return LGB_OK;
}

}  // extern "C"
