/*
 * lindblad_gb300.h -- C ABI of the GB300-native Lindblad RK4 propagator.
 *
 * The reference (binggu56/pyqed, pure Python) has no native interface: its
 * Lindblad path is the Python class pyqed.oqs.LindbladSolver
 * (pyqed/oqs.py:1114-1330).  Each entry point below replaces one piece of
 * that class's call stack; the Python mirror pyqed_gb300.oqs.LindbladSolver
 * binds them with ctypes exactly as a maintainer of the reference would
 * (pyqed_gb300/_capi.py is that binding).
 *
 * Conventions
 *  - All matrices are complex128, interleaved (re, im) doubles, row-major.
 *  - A batch holds n_inst independent instances of dimensions dims[b].
 *    Instance b's N x N operators start at complex offset off[b] =
 *    sum_{a<b} dims[a]^2 ("packed layout").  Per-instance families use
 *    count * off[b] + k * dims[b]^2 (collapse operators, observables,
 *    drive operators, stored states); diagonal collapse operators use
 *    n_cops * doff[b] + k * dims[b] with doff[b] = sum_{a<b} dims[a].
 *  - Every pointer passed to lgb_plan_set_operators / lgb_plan_propagate is
 *    a DEVICE pointer owned by the caller.  The plan owns its workspace.
 *  - Every call returns an lgb status code; nothing throws across the ABI and
 *    no device code traps.  Per-instance failures (a non-finite state) are
 *    reported through lgb_plan_errors.
 *  - One plan per stream at a time; distinct plans are independent.
 */
#ifndef LINDBLAD_GB300_H
#define LINDBLAD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
enum {
  LGB_OK = 0,
  LGB_ERR_INVALID_ARG = 1,  /* bad size, null pointer, unsupported combination */
  LGB_ERR_UNSUPPORTED = 2,  /* valid request this build cannot serve            */
  LGB_ERR_CUDA = 3,         /* a CUDA runtime call failed                        */
  LGB_ERR_NONFINITE = 4,    /* some instance's state became NaN/Inf              */
  LGB_ERR_TIMEOUT = 5,      /* a bounded device wait gave up                     */
  LGB_ERR_NO_DEVICE = 6,    /* no CUDA device visible                            */
  LGB_ERR_STATE = 7,        /* call order violated (e.g. propagate before set)   */
  LGB_ERR_TOO_LARGE = 8,    /* request exceeds the no-allocation scratch limits  */
  LGB_ERR_CHECK = 9         /* the per-step state check (LGB_OPT_CHECK) exceeded
                               its tolerance; the propagation itself completed  */
};

/* ---- precisions ------------------------------------------------------------ */
enum {
  LGB_PREC_FP64 = 0,    /* complex128 arithmetic: the check path               */
  LGB_PREC_FP32 = 1,    /* complex64 arithmetic on the FP32 pipes ("plain")    */
  LGB_PREC_TF32X3 = 2,  /* split 3xTF32 tensor-core products, FP32 accumulate  */
  LGB_PREC_BF16X3 = 3   /* split 3xBF16 tensor-core products, FP32 accumulate  */
};

/* ---- collapse-operator storage -------------------------------------------- */
enum {
  LGB_COPS_NONE = 0,
  LGB_COPS_DENSE = 1,  /* n_cops dense N x N operators per instance            */
  LGB_COPS_DIAG = 2    /* n_cops diagonals (length N) per instance             */
};

/* ---- schedules ----------------------------------------------------------------- */
enum {
  LGB_SCHED_AUTO = 0,
  LGB_SCHED_CTA = 1,   /* one CTA holds an instance in shared memory for all steps */
  LGB_SCHED_GEMM = 2   /* grid-wide tiled complex GEMMs per RK4 stage               */
};

typedef struct lgb_plan* lgb_plan_t;

/* Problem description, copied by lgb_plan_create. */
typedef struct {
  int32_t n_inst;       /* number of independent instances (>= 1)                */
  int32_t n_cops;       /* collapse operators per instance                        */
  int32_t cops_kind;    /* LGB_COPS_*                                              */
  int32_t n_eops;       /* observables per instance (<= 16)                        */
  int32_t n_drive;      /* drive terms: H(t) = H0 - sum_i f_i(t) H_i (<= 4)        */
  int32_t nt;           /* RK4 steps (>= 0)                                        */
  int32_t obs_t0;       /* 1: observable row 0 holds Tr[O rho0] (Nt+1 rows)        */
  int32_t store_every;  /* store the state every s steps into states_out (0: no)  */
  int32_t precision;    /* LGB_PREC_*                                              */
  int32_t schedule;     /* LGB_SCHED_*                                             */
  int32_t drive_shared; /* 1: one sample set f_i(t_k) for all instances           */
  int32_t flags;        /* LGB_FLAG_* (0 or LGB_FLAG_ADJOINT)                      */
  double dt;            /* time step                                               */
  int32_t checkpoint_every; /* adjoint plans: keep rho every C steps (0: ~sqrt(nt)) */
  int32_t reserved;     /* must be 0                                               */
} lgb_problem_t;

/* Plan flags. */
enum {
  LGB_FLAG_ADJOINT = 1  /* keep checkpoints during propagate for lgb_plan_adjoint */
};

/* Library version: major*10000 + minor*100 + patch. */
int lgb_get_version(void);

/* Static, human-readable text for a status code. */
const char* lgb_status_string(int status);

/* Create a plan for a batch.  dims_host[n_inst] are the instance dimensions
 * (host memory).  Chooses the schedule, sorts the instances by cost and
 * allocates the device workspace on the current device.
 * Replaces the set-up half of LindbladSolver.__init__/run
 * (pyqed/oqs.py:1115-1147, 1149-1187). */
int lgb_plan_create(lgb_plan_t* plan, const lgb_problem_t* problem, const int32_t* dims_host);

/* Release the plan and its workspace. */
int lgb_plan_destroy(lgb_plan_t plan);

/* Upload the operators (device pointers, packed layout, complex128):
 *   H         Hamiltonian (static part H0 when n_drive > 0)       required
 *   cops      collapse operators (dense or diagonals)              if n_cops > 0
 *   eops      observables                                          if n_eops > 0
 *   drive_ops H_1..H_n_drive of H(t) = H0 - sum_i f_i(t) H_i       if n_drive > 0
 * Forms H_eff = H - (i/2) sum_k L_k^dag L_k once, in the plan's precision.
 * Replaces the operator set-up of liouvillian/lindbladian
 * (pyqed/oqs.py:697-715) that the reference repeats at every RHS call. */
int lgb_plan_set_operators(lgb_plan_t plan, const double* H, const double* cops,
                           const double* eops, const double* drive_ops, void* stream);

/* Propagate nt RK4 steps from rho0 (device, packed complex128).
 *   drive_samples  f_i(t0 + (k+1) dt), k = 0..nt-1: [n_drive][nt] when
 *                  drive_shared, else [n_inst][n_drive][nt] (doubles)
 *   obs_out        [n_inst][nt + obs_t0][n_eops] complex128, or NULL
 *   rho_out        final states, packed complex128, or NULL
 *   states_out     [per instance: nt/store_every states of N x N], or NULL
 * Replaces the time loops of _lindblad (pyqed/oqs.py:1596-1696),
 * _lindblad_driven (pyqed/oqs.py:1699-1806), _fast_lindblad
 * (pyqed/oqs.py:1492-1594) and _correlation_2p_1t (pyqed/oqs.py:717-791),
 * with rk4 (pyqed/phys.py:1051-1064) and obs_dm (pyqed/phys.py:1257-1264)
 * fused into the kernels.  Asynchronous on `stream`. */
int lgb_plan_propagate(lgb_plan_t plan, const double* rho0, const double* drive_samples,
                       double* obs_out, double* rho_out, double* states_out, void* stream);

/* Copy the per-instance status flags (LGB_OK or LGB_ERR_NONFINITE /
 * LGB_ERR_TIMEOUT / LGB_ERR_CHECK) of the last propagate into
 * flags_host[n_inst]; synchronises the plan's last stream.  Returns the
 * first non-OK flag. */
int lgb_plan_errors(lgb_plan_t plan, int32_t* flags_host);

/* The largest deviations the per-step check (LGB_OPT_CHECK) saw in the last
 * propagate, per instance: stats_host[2 b] = max over steps of
 * |Tr rho(t) - Tr rho0|, stats_host[2 b + 1] = max over steps and elements of
 * |rho_ij - conj(rho_ji)|, or -1 where rho0 itself is not Hermitian (a
 * correlation seed such as B rho0) and hermiticity is not checked.
 * Synchronises the plan's last stream.  LGB_ERR_STATE when the check is off.
 * No counterpart in the reference, which checks neither. */
int lgb_plan_check_stats(lgb_plan_t plan, double* stats_host);

/* Discrete adjoint of the last lgb_plan_propagate (plans created with
 * LGB_FLAG_ADJOINT: FP32, N <= 64, dense or no collapse operators, no stored
 * states).  Propagates the costate backwards with the adjoint generator,
 * recomputing the stage inputs segment by segment from the checkpoints kept
 * by propagate.  No counterpart in the reference, which has no gradients;
 * the forward map it differentiates is _lindblad_driven
 * (pyqed/oqs.py:1699-1806) with rk4 (pyqed/phys.py:1051-1064).
 *   rho0        the initial states given to propagate (device, packed c128)
 *   drive       the drive samples given to propagate
 *   obs_grad    [n_inst][nt + obs_t0][n_eops] complex128: dJ/dRe(o) + i dJ/dIm(o)
 *               for every observable o = Tr[O rho]
 *   dE_out      [n_inst][n_drive][nt] doubles: dJ/df_d(t_{k+1}) per instance, or NULL
 *   dscale_out  [n_inst][n_cops] doubles: dJ/ds_j for L_j -> sqrt(s_j) L_j at s_j = 1
 *               (divide by gamma_j for dJ/dgamma_j when L_j = sqrt(gamma_j) L^_j), or NULL
 *   dH_out      packed complex128 Gamma per instance, dJ = Re Tr[Gamma^dag dH0], or NULL
 *   drho0_out   packed complex128 dJ/drho0 in the same convention, or NULL
 * Asynchronous on `stream`. */
int lgb_plan_adjoint(lgb_plan_t plan, const double* rho0, const double* drive,
                     const double* obs_grad, double* dE_out, double* dscale_out, double* dH_out,
                     double* drho0_out, void* stream);

/* Plan introspection: the schedule and precision in use, the bytes of
 * device workspace, the dynamic shared memory per CTA, the number of
 * kernel launches one propagate issues and the number of instances that a
 * propagate runs on the persistent split-precision kernel
 * (LGB_OPT_GEMM_PERSIST). */
typedef struct {
  int32_t schedule;
  int32_t precision;
  int32_t smem_bytes;
  int32_t launches_per_propagate;
  int64_t workspace_bytes;
  int64_t flops_per_step;   /* algorithmic real flops of one RK4 step, whole batch */
  int32_t persistent_instances;
  int32_t reserved;
} lgb_plan_info_t;

int lgb_plan_get_info(lgb_plan_t plan, lgb_plan_info_t* info);

/* Tuning options of a plan; no counterpart in the reference.  They change
 * how the work is scheduled, never the arithmetic's result beyond rounding
 * order, and stay in force until changed.  pyqed_gb300.autotune picks them
 * by timing candidates.
 *   LGB_OPT_TC_PAIRS   tensor-core kernel: 1 (default) runs two instances per
 *                      CTA when NP <= 32, 0 one at a time
 *   LGB_OPT_GEMM_WAVES split-precision GEMM schedule: the split-K factors fill
 *                      1 (default) or 2 waves of CTAs on the SMs
 *   LGB_OPT_TEST_STALL test hook of the error path: 1 makes the tensor-core
 *                      kernel skip its first MMA commit, so that its bounded
 *                      wait (4096 polls) runs out and every instance it was
 *                      given reports LGB_ERR_TIMEOUT; nothing faults or hangs
 *   LGB_OPT_GEMM_KSPLIT split-precision GEMM schedule: cap on the split-K
 *                      factors (0: none, else a power of two <= 64)
 *   LGB_OPT_GRAPH_STEPS GEMM schedule: RK4 steps captured per CUDA graph
 *                      (1..64, default 16; propagations of fewer than two
 *                      graphs' worth of steps launch directly)
 *   LGB_OPT_GEMM_PERSIST split-precision GEMM schedule: 1 (default) runs a
 *                      static instance with 64 < N <= 256 as one persistent
 *                      launch (clusters of 8 CTAs, two grid barriers per RK4
 *                      stage) when the device holds all its CTAs at once;
 *                      0 always uses the graph-replayed kernels (use 0 when
 *                      other kernels occupy SMs during the propagation: the
 *                      kernel's grid barriers then give up after 1 s with
 *                      LGB_ERR_TIMEOUT rather than wait for SMs)
 *   LGB_OPT_CHECK      per-step check of the state, accumulated in FP64:
 *                      0 (default) off; v = 1..15 checks after every step
 *                      that |Tr rho(t) - Tr rho0| <= 10^-v and, for
 *                      instances whose rho0 is Hermitian to 10^-v,
 *                      max_ij |rho_ij - conj(rho_ji)| <= 10^-v.  An instance
 *                      that exceeds either is flagged LGB_ERR_CHECK; its
 *                      propagation completes and its outputs are written
 *                      (lgb_plan_check_stats gives the deviations).  The
 *                      state is never renormalised (the RK4 map of a
 *                      Lindblad generator keeps the trace up to rounding,
 *                      and trace-zero correlation seeds must stay so).  It
 *                      is a check, not tuning: it adds one reduction per step.
 * Returns LGB_ERR_INVALID_ARG for an unknown option or value. */
typedef enum {
  LGB_OPT_TC_PAIRS = 1,
  LGB_OPT_GEMM_WAVES = 2,
  LGB_OPT_TEST_STALL = 3,
  LGB_OPT_CHECK = 4,
  LGB_OPT_GEMM_KSPLIT = 5,
  LGB_OPT_GRAPH_STEPS = 6,
  LGB_OPT_GEMM_PERSIST = 7
} lgb_option_t;

int lgb_plan_set_option(lgb_plan_t plan, int32_t option, int32_t value);

/* ---- Redfield master equation ------------------------------------------------
 * Replaces RedfieldSolver.redfield_tensor / evolve / _redfield
 * (pyqed/oqs.py:30-100, 364-459, 519-563).  Everything lives in the
 * eigenbasis of H; vec is row-major (vec(rho)[a*N + b] = rho[a][b]).
 *
 * lgb_redfield_tensor builds, for one system of dimension n with n_ops
 * system-bath operators, the N^2 x N^2 generator (complex128, row-major)
 *     R = -i [E, .] - sum_k [A_k, L_k . - . L_k^dag],   L_k = C_k o A_k,
 * from the eigenvalues E (n FP64), the operators A_k = V^dag a_k V
 * (n_ops x n x n complex128) and the bath spectra C_k[m][l] = S_k(e_l - e_m)
 * (n_ops x n x n FP64) -- the reference's redfield_tensor (pyqed/oqs.py:519-563).
 * All pointers are device pointers.  n <= lgb_redfield_max_dim(LGB_PREC_FP32). */
int lgb_redfield_tensor(int32_t n, int32_t n_ops, const double* evals, const double* A,
                        const double* C, double* R_out, void* stream);

/* The generators of n_sys systems in one launch: dims_host[n_sys] (host),
 * evals packed (system b at sum_{c<b} N_c), A and C packed n_ops x N_b^2 at
 * n_ops * sum_{c<b} N_c^2, R_out packed N_b^4 at sum_{c<b} N_c^4.  Device
 * pointers for the data.  Synchronous: returns when the generators are built. */
int lgb_redfield_tensor_batch(int32_t n_sys, const int32_t* dims_host, int32_t n_ops, const double* evals,
                              const double* A, const double* C, double* R_out, void* stream);

/* Largest supported dimension per precision (64 for FP32, 48 for FP64). */
int lgb_redfield_max_dim(int32_t precision);

typedef struct lgb_redfield_plan* lgb_redfield_t;

typedef struct {
  int32_t n_inst;       /* independent systems in the batch                          */
  int32_t n_eops;       /* observables per system, <= 16                              */
  int32_t nt;           /* RK4 steps                                                  */
  int32_t precision;    /* LGB_PREC_FP64 or LGB_PREC_FP32                             */
  int32_t store_every;  /* keep vec(rho) every this many steps (0: none)              */
  int32_t reserved;     /* 0                                                          */
  double dt;
} lgb_redfield_problem_t;

/* A batch of systems of dimensions dims[n_inst] (host array). */
int lgb_redfield_create(lgb_redfield_t* plan, const lgb_redfield_problem_t* prob, const int32_t* dims);
int lgb_redfield_destroy(lgb_redfield_t plan);

/* Generators (packed: system b at offset sum_{c<b} N_c^4, complex128) and the
 * observables as vec(O_e^T) in the eigenbasis (packed: system b at
 * n_eops * sum_{c<b} N_c^2, e-major).  Device pointers. */
int lgb_redfield_set(lgb_redfield_t plan, const double* R, const double* eops, void* stream);

/* nt RK4 steps of d vec(rho)/dt = R vec(rho) (pyqed/phys.py:1051-1064).
 *   rho0       vec(rho0) in the eigenbasis, packed (sum N^2, complex128)
 *   obs_out    [n_inst][nt][n_eops] complex128 (Tr[O rho] after every step), or NULL
 *   rho_out    vec(rho) after nt steps, packed, or NULL
 *   states_out vec(rho) every store_every steps: system b holds a contiguous
 *              block of (nt / store_every) x N_b^2 at (nt / store_every) * sum_{c<b} N_c^2
 * A state that becomes NaN/Inf stops its system with LGB_ERR_NONFINITE
 * (lgb_redfield_errors). */
int lgb_redfield_propagate(lgb_redfield_t plan, const double* rho0, double* obs_out, double* rho_out,
                           double* states_out, void* stream);
int lgb_redfield_errors(lgb_redfield_t plan, int32_t* flags_host);

/* ---- HEOM (hierarchical equations of motion) ----------------------------------
 * Replaces HEOMSolver.run / propagator, _heom and _heom_propagator
 * (pyqed/oqs.py:1332-1371, 1808-1935): one exponential bath mode coupled
 * through one system operator sz, nado auxiliary density operators (the last
 * one the zero terminator), explicit Euler steps swept level by level in place:
 *     X_n += dt ( -i[H, X_n] - [sz, X_{n+1}] - n gamma X_n
 *                 + n (Re D0 [sz, X_{n-1}] + i Im D0 {sz, X_{n-1}}) ),
 * X_{n-1} already advanced in this step, X_{n+1} not yet. */
typedef struct lgb_heom_plan* lgb_heom_t;

enum {
  LGB_HEOM_DOUBLE_FIRST = 1, /* advance level 0 twice per step (_heom_propagator)             */
  LGB_HEOM_DIAG_SZ = 2       /* every sz is diagonal: its off-diagonal entries are not read */
};

typedef struct {
  int32_t n_inst;       /* independent systems in the batch                          */
  int32_t n_eops;       /* observables per system, <= 16                              */
  int32_t nt;           /* Euler steps                                                */
  int32_t nado;         /* levels per system including the zero terminator, >= 2     */
  int32_t precision;    /* LGB_PREC_FP64 or LGB_PREC_FP32                             */
  int32_t flags;        /* LGB_HEOM_DOUBLE_FIRST | LGB_HEOM_DIAG_SZ, or 0             */
  double dt;
} lgb_heom_problem_t;

/* Largest supported system dimension (64). */
int lgb_heom_max_dim(int32_t precision);
/* Most levels whose hierarchy stays in shared memory at dimension n; deeper
 * hierarchies run from a global workspace. */
int lgb_heom_max_levels_on_chip(int32_t n, int32_t precision);

int lgb_heom_create(lgb_heom_t* plan, const lgb_heom_problem_t* prob, const int32_t* dims);
int lgb_heom_destroy(lgb_heom_t plan);
/* info[4]: threads per system, systems per CTA, levels on chip (1/0), shared bytes per CTA. */
int lgb_heom_layout(lgb_heom_t plan, int32_t* info);

/* Device pointers, complex128 row-major, system b at offset sum_{c<b} N_c^2:
 *   H, sz  the Hamiltonian and the system-bath operator
 *   bath   n_inst x 3 FP64: gamma, Re D0, Im D0
 *   eops   vec(O_e^T) per system, e-major (n_eops x N_b^2 at n_eops * offset) */
int lgb_heom_set(lgb_heom_t plan, const double* H, const double* sz, const double* bath, const double* eops,
                 void* stream);

/* nt steps from X_0 = rho0 (packed), the other levels zero.
 *   obs_out [n_inst][n_eops][nt] complex128, Tr[O X_0] after every step, or NULL
 *   rho_out X_0 after nt steps (packed), or NULL
 *   ado_out all nado levels after nt steps, system b at nado * offset
 *           (level-major, the terminator written as zeros), or NULL
 * A system whose X_0 becomes NaN/Inf stops with LGB_ERR_NONFINITE. */
int lgb_heom_propagate(lgb_heom_t plan, const double* rho0, double* obs_out, double* rho_out, double* ado_out,
                       void* stream);
int lgb_heom_errors(lgb_heom_t plan, int32_t* flags_host);

/* ---- spectral (eigen-decomposition) evaluation ---------------------------------
 * Replaces the mode sums of Lindblad_solver.evolve / correlation_2op_1t /
 * correlation_2op_1w / correlation_3op_1t / correlation_3op_1w /
 * correlation_3op_2t / correlation_4op_2t (pyqed/superoperator.py:455-770);
 * the Liouvillian is diagonalised by the caller.  Device pointers, complex128
 * interleaved, row-major; FP64 arithmetic; results are deterministic.
 *
 * lgb_spectral_sum: out[p][o] = sum_n W[o][n] f(lambda_n, x_p), p < n_x, o < n_out <= 16,
 *   kind 0: f = exp(lambda x)          (time points)
 *   kind 1: f = -1 / (lambda + i x)    (frequencies)
 * x holds n_x real points (FP64). */
int lgb_spectral_sum(int32_t k, int32_t n_out, int32_t n_x, int32_t kind, const double* lambda, const double* W,
                     const double* x, double* out, void* stream);

/* lgb_spectral_2t: cor[a][b] = sum_{m,n} exp(lambda_m tau_a) coeff[m][n] exp(lambda_n t_b),
 * an n_tau x n_t matrix (the (len(taulist), len(tlist)) shape the reference returns). */
int lgb_spectral_2t(int32_t k, int32_t n_tau, int32_t n_t, const double* lambda, const double* coeff,
                    const double* tau, const double* t, double* cor, void* stream);

/* ---- propagation without device allocation ---------------------------------
 * No counterpart in the reference: pyqed is pure Python and never manages
 * device memory.
 *
 * For callers that cannot call cudaMalloc -- a process whose device memory
 * was handed to another allocator up front (a framework's caching allocator,
 * a fixed arena in a serving process), or an embedding whose device-memory
 * budget is fixed before this library is loaded.
 * It propagates ONE instance in complex128 (the same FP64 kernel as
 * lgb_plan_propagate with LGB_PREC_FP64) and keeps every working buffer in a
 * fixed array compiled into the library (about 1.1 MB, held on every device
 * that loads the library until the process exits); it never allocates.
 *
 *   H          N x N Hamiltonian (device, complex128)
 *   cops       n_cops collapse operators, dense (N x N each) or diagonals
 *              (N each) per cops_kind; NULL when n_cops == 0
 *   eops       n_eops observables (N x N each); NULL when n_eops == 0
 *   rho0       initial state (N x N)
 *   obs_out    [nt + obs_t0][n_eops] complex128, or NULL
 *   rho_out    final state (N x N), or NULL
 *   status_out one int32 on the device receiving LGB_OK or LGB_ERR_NONFINITE
 *              for this propagation, or NULL
 * Limits: N <= LGB_NOALLOC_MAX_DIM, n_cops <= LGB_NOALLOC_MAX_COPS,
 * n_eops <= LGB_NOALLOC_MAX_EOPS; larger requests return LGB_ERR_TOO_LARGE.
 * The first call on a device looks up the array's device address (once per
 * device and context: again after a reset of the device); make that first
 * call before any stream capture begins.  All calls
 * share the one array, so calls that overlap on the GPU (different streams,
 * or different host threads on the same device) race: serialise them.
 * Asynchronous on `stream`. */
#define LGB_NOALLOC_MAX_DIM 64
#define LGB_NOALLOC_MAX_COPS 4
#define LGB_NOALLOC_MAX_EOPS 4
int lgb_propagate_noalloc(const double* H, int32_t n, const double* cops, int32_t n_cops,
                          int32_t cops_kind, const double* eops, int32_t n_eops,
                          const double* rho0, int32_t nt, double dt, int32_t obs_t0,
                          double* obs_out, double* rho_out, int32_t* status_out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* LINDBLAD_GB300_H */
