// lgb_propagate_noalloc: one FP64 propagation that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a process whose device heap was
// handed to another allocator at start-up (a framework's caching allocator
// or a fixed arena in a serving process), or an embedding whose memory
// budget is fixed before this library is loaded.  For them this entry point
// runs the FP64 CTA-resident kernel (the check path of lgb_plan_propagate)
// with every piece of working memory -- the prepared operators, the RK4
// state slabs, the dense-collapse scratch and the small per-instance tables
// -- placed in one file-scope __device__ array of fixed size.  The caller
// still passes its inputs and outputs as device pointers.
//
// The array lives as long as the library is loaded, on every device that
// loads it.  Its device address is looked up once per device and CUDA
// context (the first call on that device, which therefore should come
// before any stream capture; a call after the device's context was reset
// looks it up again).  Every call reuses the same array: concurrent calls on
// different streams of the same device race and must be serialised by the
// caller.
#include <cuda.h>

#include <mutex>

#include "lgb_internal.h"

namespace {

// Limits of the no-allocation entry point (they bound the scratch size).
constexpr int kMaxDim = LGB_NOALLOC_MAX_DIM;    // N <= 64
constexpr int kMaxCops = LGB_NOALLOC_MAX_COPS;  // collapse operators
constexpr int kMaxEops = LGB_NOALLOC_MAX_EOPS;  // observables
constexpr int kNP = (kMaxDim + 3) / 4 * 4;
constexpr long long kMS = (long long)kNP * (kNP + 1);  // FP64 working matrix (padc = 1)
// At, Lt (K), Dm, Ot (E), state (2), Y (K) -- all complex128
constexpr long long kComplexElems = (1 + kMaxCops + 1 + kMaxEops + 2 + kMaxCops) * kMS;
constexpr size_t kTableBytes = 4096;
constexpr size_t kScratchBytes = kComplexElems * sizeof(double2) + kTableBytes;

static __device__ __align__(256) unsigned char g_lgb_noalloc_scratch[kScratchBytes];

struct DevScratch {
  unsigned char* base = nullptr;
  unsigned long long ctx_id = 0;  // the context the address belongs to
  bool ready = false;
};
DevScratch g_dev[64];
std::mutex g_mu;

// ID of the current CUDA context (0 if the driver cannot tell).  The
// runtime is linked statically and the driver library is not linked, so
// the two driver calls are looked up through the runtime.
unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext*);
  using GetId = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
    cudaGetLastError();
    looked_up = true;
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current == nullptr || get_id == nullptr || get_current(&ctx) != CUDA_SUCCESS ||
      ctx == nullptr || get_id(ctx, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

// Small per-instance tables (one instance) written by a kernel from its
// arguments, so that no host-to-device copy is needed.
struct Tables {
  int order, dims, npad, err;
  long long off, doff, woff, soff;
  unsigned char place;
  double shift;
};

__global__ void noalloc_tables_kernel(Tables* t, int N, int NP, unsigned char place) {
  t->order = 0;
  t->dims = N;
  t->npad = NP;
  t->err = 0;
  t->off = t->doff = t->woff = t->soff = 0;
  t->place = place;
  t->shift = 0.0;  // overwritten by the trace-shift kernel of launch_setup (Re Tr(H) / N)
}

int scratch_for_current_device(unsigned char** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return LGB_ERR_CUDA;
  if (dev < 0 || dev >= 64) return LGB_ERR_UNSUPPORTED;
  // (the caller's device pointers imply that the device's context exists;
  // if the driver cannot name it, the address is looked up on every call)
  const unsigned long long ctx = current_context_id();
  std::lock_guard<std::mutex> lock(g_mu);
  // a reset of the device (cudaDeviceReset) unloads the module: the address
  // belongs to the context it was looked up in
  if (g_dev[dev].ready && (ctx == 0 || g_dev[dev].ctx_id != ctx)) g_dev[dev].ready = false;
  if (!g_dev[dev].ready) {
    void* p = nullptr;
    // the array's name is a host-side stand-in: its device address must be
    // looked up with the device current
    if (cudaGetSymbolAddress(&p, g_lgb_noalloc_scratch) != cudaSuccess) {
      cudaGetLastError();
      return LGB_ERR_CUDA;
    }
    g_dev[dev].base = static_cast<unsigned char*>(p);
    g_dev[dev].ctx_id = ctx != 0 ? ctx : current_context_id();
    g_dev[dev].ready = true;
  }
  *out = g_dev[dev].base;
  return LGB_OK;
}

}  // namespace

extern "C" int lgb_propagate_noalloc(const double* H, int32_t n, const double* cops,
                                     int32_t n_cops, int32_t cops_kind, const double* eops,
                                     int32_t n_eops, const double* rho0, int32_t nt, double dt,
                                     int32_t obs_t0, double* obs_out, double* rho_out,
                                     int32_t* status_out, void* stream) {
  if (H == nullptr || rho0 == nullptr || n < 1 || nt < 0 || n_cops < 0 || n_eops < 0 ||
      !(dt == dt))
    return LGB_ERR_INVALID_ARG;
  if (n > kMaxDim || n_cops > kMaxCops || n_eops > kMaxEops) return LGB_ERR_TOO_LARGE;
  if (cops_kind < LGB_COPS_NONE || cops_kind > LGB_COPS_DIAG) return LGB_ERR_INVALID_ARG;
  if ((cops_kind == LGB_COPS_NONE) != (n_cops == 0)) return LGB_ERR_INVALID_ARG;
  if (n_cops > 0 && cops == nullptr) return LGB_ERR_INVALID_ARG;
  if (n_eops > 0 && eops == nullptr) return LGB_ERR_INVALID_ARG;
  unsigned char* base = nullptr;
  int s = scratch_for_current_device(&base);
  if (s != LGB_OK) return s;

  const int NP = (n + 3) / 4 * 4;
  const long long ms = (long long)NP * (NP + 1);
  const bool dense = cops_kind == LGB_COPS_DENSE;
  const int K = n_cops;
  // carve the scratch array (complex128 slabs, then the tables)
  double2* c = reinterpret_cast<double2*>(base);
  double2* At = c;
  c += ms;
  double2* Lt = dense ? c : nullptr;
  c += dense ? K * ms : 0;
  double2* Dm = cops_kind == LGB_COPS_DIAG ? c : nullptr;
  c += cops_kind == LGB_COPS_DIAG ? ms : 0;
  double2* Ot = c;
  c += (long long)n_eops * ms;
  double2* state = c;
  c += 2 * ms;
  double2* Y = dense ? c : nullptr;
  Tables* t = reinterpret_cast<Tables*>(base + kComplexElems * sizeof(double2));

  // shared-memory placement of the dense-collapse slabs, as lgb_plan_create
  const long long mb = ms * (long long)sizeof(double2);
  constexpr long long kBudget = 224 * 1024;
  long long used = 3 * mb;
  unsigned char place = 0;
  if (dense) {
    if (used + K * mb <= kBudget) {
      used += K * mb;
      place |= 2;
    }
    if (used + K * mb <= kBudget) {
      used += K * mb;
      place |= 1;
    }
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  noalloc_tables_kernel<<<1, 1, 0, st>>>(t, n, NP, place);
  if (cudaGetLastError() != cudaSuccess) return LGB_ERR_CUDA;

  lgb::SetupParams sp{};
  sp.n_inst = 1;
  sp.n_cops = K;
  sp.cops_kind = cops_kind;
  sp.n_eops = n_eops;
  sp.n_drive = 0;
  sp.padc = 1;
  sp.max_npad = NP;
  sp.dims = &t->dims;
  sp.npad = &t->npad;
  sp.off = &t->off;
  sp.doff = &t->doff;
  sp.woff = &t->woff;
  sp.H = reinterpret_cast<const double2*>(H);
  sp.cops = reinterpret_cast<const double2*>(cops);
  sp.eops = reinterpret_cast<const double2*>(eops);
  sp.dops = nullptr;
  sp.shift = &t->shift;
  sp.At = At;
  sp.Lt = Lt;
  sp.Dm = Dm;
  sp.Gt = nullptr;
  sp.Ot = Ot;
  sp.OtF = nullptr;
  if (lgb::launch_setup(sp, 0, st) != cudaSuccess) return LGB_ERR_CUDA;

  lgb::CtaParams p{};
  p.n_inst = 1;
  p.n_cops = K;
  p.cops_kind = cops_kind;
  p.n_eops = n_eops;
  p.n_drive = 0;
  p.nt = nt;
  p.obs_t0 = obs_t0 ? 1 : 0;
  p.store_every = 0;
  p.drive_shared = 1;
  p.dt = dt;
  p.order = &t->order;
  p.dims = &t->dims;
  p.npad = &t->npad;
  p.off = &t->off;
  p.woff = &t->woff;
  p.soff = &t->soff;
  p.place = &t->place;
  p.At = At;
  p.Lt = Lt;
  p.Dm = Dm;
  p.Gt = nullptr;
  p.Ot = Ot;
  p.OtF = nullptr;
  p.drive = nullptr;
  p.rho0 = reinterpret_cast<const double2*>(rho0);
  p.obs_out = reinterpret_cast<double2*>(obs_out);
  p.rho_out = reinterpret_cast<double2*>(rho_out);
  p.states_out = nullptr;
  p.state_ws = state;
  p.y_ws = Y;
  p.err = status_out != nullptr ? status_out : &t->err;
  p.smem_bytes = (int)used;
  if (lgb::launch_cta_rk4(p, 0, 1, st, false) != cudaSuccess) return LGB_ERR_CUDA;
  return LGB_OK;
}
