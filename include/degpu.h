/* degpu -- C ABI of the GB300 EnsembleGPUKernel engine (libdegpu.so).
 *
 * Drop-in boundary for DiffEqGPU.jl's lower-level kernel API: a Julia shim (ccall) or any
 * C caller passes caller-owned DEVICE buffers and a CUDA stream; every solve is
 * stream-ordered (no host synchronisation inside), returns 0 or a negative DEGPU_E*
 * code, and reports per-trajectory failures in retcode[] instead of trapping.
 * Plain C types only; the stream is a cudaStream_t passed as void*.
 *
 * Layouts (B trajectories, N states, P parameters, L saved rows, Tt = time type):
 *   u0 [B][N] f32, p [B][P] f32, tspan [B][2] Tt, saveat [L] or [B][L] Tt,
 *   ts [B][L] Tt, us [B][L][N] f32  -- ts/us are the column-major Julia matrices
 *   Matrix{Tt}(L, B) and Matrix{SVector{N,Float32}}(L, B) of the reference.
 */
#ifndef DEGPU_H
#define DEGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DEGPU_VERSION "0.1.0"

/* return codes */
#define DEGPU_OK 0
#define DEGPU_E_INVALID (-1)   /* bad argument (sizes, pointers, options) */
#define DEGPU_E_COMPILE (-2)   /* NVRTC failed on the right-hand side or kernels */
#define DEGPU_E_CUDA (-3)      /* CUDA driver/runtime error */
#define DEGPU_E_UNSUPPORTED (-4) /* combination the reference also rejects */

/* algorithms: GPUTsit5, GPUVern7, GPURosenbrock23, GPURodas5P (alias GPURodas5), GPUEM,
 * GPURodas4 (src/ensemblegpukernel/gpukernel_algorithms.jl:30, 57, 112, 162, 243, 137) */
#define DEGPU_ALG_TSIT5 0
#define DEGPU_ALG_VERN7 1
#define DEGPU_ALG_ROSENBROCK23 2
#define DEGPU_ALG_RODAS5P 3
#define DEGPU_ALG_EM 4
#define DEGPU_ALG_RODAS4 5 /* GPURodas4 (gpukernel_algorithms.jl:137, perform_step/gpu_rodas4_perform_step.jl) */
#define DEGPU_ALG_VERN9 6  /* GPUVern9 (gpukernel_algorithms.jl:83, perform_step/gpu_vern9_perform_step.jl) */
#define DEGPU_ALG_SIEA 7   /* GPUSIEA, weak order 2 SDE (gpukernel_algorithms.jl:266, perform_step/gpu_siea_perform_step.jl) */
#define DEGPU_ALG_KVAERNO3 8 /* GPUKvaerno3 (gpukernel_algorithms.jl:187, perform_step/gpu_kvaerno3_perform_step.jl) */
#define DEGPU_ALG_KVAERNO5 9 /* GPUKvaerno5 (gpukernel_algorithms.jl:212, perform_step/gpu_kvaerno5_perform_step.jl) */

#define DEGPU_TIME_F32 0 /* Float32 tspan: every operation is the reference's Float32 one */
#define DEGPU_TIME_F64 1 /* FP64 time accumulation / end detection, FP32 state */

#define DEGPU_MODE_FAST 0   /* FMA contraction, hardware pow, LU + refinement */
#define DEGPU_MODE_PARITY 1 /* strict IEEE order of the reference, portable pow, Cramer solves */

#define DEGPU_DRIVER_AUTO 0       /* fixed: one trajectory/thread; adaptive: persistent */
#define DEGPU_DRIVER_NAIVE 1      /* one trajectory per thread (ode_asolve_kernel shape) */
#define DEGPU_DRIVER_PERSISTENT 2 /* warp lane refill + work stealing */

#define DEGPU_JAC_AUTO 0       /* user Jacobian/tgrad if given, else forward-mode AD */
#define DEGPU_JAC_AD 1
#define DEGPU_JAC_FINITEDIFF 2 /* alg_utils.jl:17-27 */

/* per-trajectory retcodes */
#define DEGPU_RET_DEFAULT 0
#define DEGPU_RET_SUCCESS 1
#define DEGPU_RET_TERMINATED 2
#define DEGPU_RET_DTLESSTHANMIN 3
#define DEGPU_RET_MAXITERS 4
#define DEGPU_RET_UNSTABLE 5

/* right-hand side flags */
#define DEGPU_RHS_HAS_JAC 1   /* source defines degpu_jac(float* J, const float* u, const float* p, float t), J column-major */
#define DEGPU_RHS_HAS_TGRAD 2 /* source defines degpu_tgrad(float* dT, const float* u, const float* p, float t) */
#define DEGPU_RHS_HAS_NOISE 4 /* source defines template<class T> degpu_g(T* g, const T* u, const float* p, T t) (diagonal noise) */
#define DEGPU_RHS_HAS_MASS 8  /* source defines degpu_mass(float* M): the constant mass matrix (column-major),
                                 taken by GPURosenbrock23 / GPURodas4 / GPURodas5P (ODEFunction mass_matrix) */

typedef struct degpu_rhs_s degpu_rhs;
typedef struct degpu_plan_s degpu_plan;

/* ---- callbacks (src/ensemblegpukernel/callbacks.jl, integrators/integrator_utils.jl) ----
 * The callback functions are CUDA C in the same source as the right-hand side:
 *   continuous:  float degpu_ccb_condition(int fn, const float* u, const float* p, degpu_time t);
 *                void  degpu_ccb_affect(int fn, degpu_integrator& I);
 *                void  degpu_ccb_affect_neg(int fn, degpu_integrator& I);
 *   discrete:    bool  degpu_dcb_condition(int fn, const float* u, const float* p, degpu_time t);
 *                void  degpu_dcb_affect(int fn, degpu_integrator& I);
 * degpu_time is float (DEGPU_TIME_F32) or double (DEGPU_TIME_F64); an affect may change
 * I.u in place and call degpu_terminate(I) (terminate!, retcode Terminated).  Each member of
 * a set names the function index fn it passes to those functions.  save_positions must be
 * (false, false), as in the reference (callbacks.jl:13, 72). */
#define DEGPU_MAX_CALLBACKS 8
#define DEGPU_ROOTFIND_LEFT 0  /* SciMLBase.LeftRootFind (default) */
#define DEGPU_ROOTFIND_RIGHT 1 /* SciMLBase.RightRootFind */
#define DEGPU_ROOTFIND_NONE 2  /* SciMLBase.NoRootFind: the event is placed at the step end */
typedef struct degpu_continuous_callback {
  int fn;               /* function index passed to degpu_ccb_* */
  int has_affect;       /* 0: affect! === nothing (upcrossings are ignored) */
  int has_affect_neg;   /* 0: affect_neg! === nothing (downcrossings are ignored) */
  int rootfind;         /* DEGPU_ROOTFIND_* */
  double abstol;        /* repeat-event tolerance: 100 eps(Float32) when converted from a ContinuousCallback */
  double repeat_nudge;  /* 1/100 */
  double dtrelax;       /* 1 */
} degpu_continuous_callback;
typedef struct degpu_callbacks {
  int n_continuous;                              /* <= DEGPU_MAX_CALLBACKS */
  const degpu_continuous_callback* continuous;   /* host array [n_continuous] */
  int n_discrete;                                /* <= DEGPU_MAX_CALLBACKS */
  const int* discrete;                           /* host array [n_discrete]: function indices */
} degpu_callbacks;

/* The isbits ImmutableODEProblem array of the reference, flattened (device pointers). */
typedef struct degpu_problems {
  const float* u0;    /* [B][N] */
  const float* p;     /* [B][P] */
  const void* tspan;  /* [B][2] of the time type */
  long long B;
} degpu_problems;

/* keyword arguments of vectorized_solve / vectorized_asolve */
typedef struct degpu_options {
  int alg;              /* DEGPU_ALG_* */
  int time_type;        /* DEGPU_TIME_* */
  int mode;             /* DEGPU_MODE_* */
  int driver;           /* DEGPU_DRIVER_* */
  int jac;              /* DEGPU_JAC_* */
  int save_everystep;
  int nsaveat;          /* 0 = no saveat */
  int saveat_per_traj;
  const void* saveat;   /* device, time type */
  double dt;            /* fixed dt, or initial dt of the adaptive controller */
  double abstol;
  double reltol;
  long long maxiters;   /* cap on step attempts per trajectory (0 = 10^7) */
  const float* dt0;     /* optional device [B]: per-trajectory initial dt (learned controller) */
  const float* tolscale;/* optional device [B]: per-trajectory tolerance multiplier */
  unsigned long long seed; /* EM noise key */
  long long traj_offset;   /* global index of trajectory 0 (noise streams of shards) */
  int block;            /* threads per block (0 = autotuned/default) */
  int chunk;            /* persistent driver: trajectories per warp refill (0 = default) */
  int ntstops;          /* tstops: 0 = none */
  const void* tstops;   /* device [ntstops] of the time type, ascending, shared by all trajectories */
  const degpu_callbacks* callbacks; /* NULL = no callbacks (CallbackSet(nothing)) */
  const int* order;     /* optional device [B]: the persistent driver (the default adaptive
                           driver) visits trajectory order[w] as its w-th work item, e.g. the
                           permutation of degpu_work_order; results are the same in any order.
                           Entries outside [0, B) are skipped.  Other drivers, and the
                           host-buffer API (which rejects it), run trajectories in index order. */
} degpu_options;

/* outputs (caller-owned device buffers) */
typedef struct degpu_outputs {
  void* ts;             /* [B][L] time type */
  float* us;            /* [B][L][N] */
  int L;
  signed char* retcode; /* optional [B] */
  int* naccept;         /* optional [B] */
  int* nreject;         /* optional [B] */
  float* dt_first;      /* optional [B]: first accepted step size (accepted-step trace) */
} degpu_outputs;

const char* degpu_version(void);
/* sizeof of the ABI structs (options, outputs, problems, continuous callback, callback set),
 * so that bindings can check their mirrors of these layouts */
void degpu_abi_struct_sizes(int* options, int* outputs, int* problems, int* continuous_callback, int* callbacks);
/* The library keeps the device scratch of earlier solves (work counters, the host API's
 * staging arena) in a per-device memory pool for reuse; this returns it to the device. */
void degpu_trim_memory(void);
/* last error message of the calling thread */
const char* degpu_last_error(void);

/* Register a right-hand side written in CUDA C:
 *   template <class T> __device__ void degpu_f(T* du, const T* u, const float* p, T t);
 * (T is float or a forward-mode dual), plus the optional functions named by flags.  It is
 * compiled with NVRTC for sm_103a together with the steppers, so it is inlined into
 * them.  Replaces the Julia RHS that the reference compiles into its KernelAbstractions
 * kernel (src/ensemblegpukernel/kernels.jl:1-152 via prob.f). */
int degpu_rhs_create(const char* cuda_source, int n_state, int n_param, int flags, degpu_rhs** out);
void degpu_rhs_destroy(degpu_rhs* f);
/* Source of a built-in model ("lorenz", "robertson", "decay", "growth", "linear15",
 * "gbm", "lorenz_addnoise", "osc"); NULL if unknown.  Also returns N, P, flags. */
const char* degpu_builtin_rhs(const char* name, int* n_state, int* n_param, int* flags);

/* vectorized_solve(probs, prob::ODEProblem, alg; dt, saveat, save_everystep)
 * -- src/ensemblegpukernel/lowerlevel_solve.jl:53-131 (fixed step). */
int degpu_vectorized_solve(const degpu_rhs* f, const degpu_problems* probs, const degpu_options* opt,
                           degpu_outputs* out, void* stream);

/* vectorized_asolve(probs, prob::ODEProblem, alg; dt, saveat, abstol, reltol)
 * -- src/ensemblegpukernel/lowerlevel_solve.jl:253-346 (adaptive). */
int degpu_vectorized_asolve(const degpu_rhs* f, const degpu_problems* probs, const degpu_options* opt,
                            degpu_outputs* out, void* stream);

/* vectorized_solve(probs, prob::SDEProblem, GPUEM(); dt, saveat, save_everystep)
 * -- src/ensemblegpukernel/lowerlevel_solve.jl:134-199 with em_kernel
 * (perform_step/gpu_em_perform_step.jl:1-74).  Adaptive EM is rejected like
 * lowerlevel_solve.jl:348-356. */
int degpu_vectorized_solve_sde(const degpu_rhs* f, const degpu_problems* probs, const degpu_options* opt,
                               degpu_outputs* out, void* stream);

/* batch_solve_up_kernel (src/solve.jl:382-419) with HOST buffers: copies the problems
 * to the device, runs vectorized_(a)solve, copies ts/us (and retcodes) back and
 * synchronises.  adaptive selects vectorized_asolve.  Host arrays use the layouts above
 * opt->saveat is a host array here, opt->dt0 / opt->tolscale stay device arrays.  Outputs
 * in page-locked memory (cudaHostAlloc / cudaHostRegister) are written by the solver kernel
 * directly (environment DEGPU_HOST_DIRECT=0 turns that off); pageable outputs are staged on
 * the device and, from 524,288 trajectories, pipelined in chunks (two compute streams and one
 * copy-back stream; environment DEGPU_HOST_CHUNK sets the chunk size).  Results do not depend
 * on the path or the chunking. */
int degpu_batch_solve_host(const degpu_rhs* f, const float* u0, const float* p, const void* tspan, long long B,
                           const degpu_options* opt, int adaptive, void* ts, float* us, int L,
                           signed char* retcode, int* naccept, int* nreject, void* stream);

/* Solve plan: compiles, autotunes block size and trajectories-per-warp (when
 * opt->block == 0), allocates the work counter and captures the whole solve (counter
 * reset + kernel) in a CUDA graph, so that repeated solves over the same buffers are one
 * graph launch.  adaptive selects vectorized_asolve semantics. */
int degpu_plan_create(const degpu_rhs* f, const degpu_problems* probs, const degpu_options* opt, int adaptive,
                      degpu_outputs* out, void* stream, degpu_plan** plan);
int degpu_plan_launch(degpu_plan* plan, void* stream);
/* the configuration the plan chose: block, chunk, grid, driver, registers per thread */
int degpu_plan_info(const degpu_plan* plan, int* block, int* chunk, int* grid, int* driver, int* regs);
void degpu_plan_destroy(degpu_plan* plan);

/* Autotuner (block size, trajectories per warp refill) on the first sample_B
 * trajectories; results are cached per kernel and size class. */
int degpu_autotune(const degpu_rhs* f, const degpu_problems* probs, const degpu_options* opt, int adaptive,
                   degpu_outputs* out, long long sample_B, void* stream, int* best_block, int* best_chunk);

/* Compile (NVRTC, sm_103a) the kernel a solve with these options would use, without
 * loading it -- needs no GPU.  Reports the compiler log on failure through
 * degpu_last_error().  *cubin_bytes receives the size of the compiled image. */
int degpu_rhs_check(const degpu_rhs* f, const degpu_options* opt, int adaptive, long long* cubin_bytes);

/* Registers/thread and spill bytes of the kernel a solve with these options would use
 * (compiles it if needed). */
int degpu_kernel_info(const degpu_rhs* f, const degpu_options* opt, int adaptive, int* regs, int* local_bytes,
                      int* max_threads);

/* ---- learned step control (no counterpart in the reference) ----
 * A BF16 MLP  x -> 64 SiLU -> 64 SiLU -> 2  predicting, per trajectory, log(initial dt) and
 * log(tolerance scale) from x = (u0, p, log10 reltol) (n_in <= 16).  Its outputs feed
 * degpu_options.dt0 / .tolscale; the embedded error estimate still accepts or rejects
 * every step.  Parameters are one packed FP32 vector (W1 [64][n_in], b1 [64], W2 [64][64],
 * b2 [64], W3 [2][64], b3 [2]); inputs are standardised with (mean, std) inside. */
#define DEGPU_MLP_HIDDEN 64
#define DEGPU_MLP_OUT 2
typedef struct degpu_mlp_s degpu_mlp;
int degpu_mlp_create(int n_in, unsigned long long seed, degpu_mlp** out);
void degpu_mlp_destroy(degpu_mlp* m);
int degpu_mlp_param_count(const degpu_mlp* m);
/* host arrays; any may be NULL */
int degpu_mlp_set_params(degpu_mlp* m, const float* host_params, const float* host_mean, const float* host_std);
int degpu_mlp_get_params(const degpu_mlp* m, float* host_params, float* host_grads, float* host_mean, float* host_std);
/* Tensor-core inference (mma.sync m16n8k16 bf16, fp32 accumulate) over device x [B][n_in]:
 * y [B][2] raw outputs (optional), dt0 = clamp(exp(y0), dt_lo, dt_hi), tolscale =
 * clamp(exp(y1), s_lo, s_hi) (each optional). */
int degpu_mlp_infer(const degpu_mlp* m, const float* x, long long B, float* y, float* dt0, float* tolscale,
                    float dt_lo, float dt_hi, float s_lo, float s_hi, void* stream);
/* Same, with the features read straight from a problem batch: x = (u0 [B][n_state],
 * p [B][n_param], log10 reltol); requires n_in == n_state + n_param + 1. */
int degpu_mlp_infer_problems(const degpu_mlp* m, const float* u0, int n_state, const float* p, int n_param, float reltol,
                             long long B, float* dt0, float* tolscale, float dt_lo, float dt_hi, float s_lo, float s_hi,
                             void* stream);
/* Learned-controller adaptive solve: degpu_mlp_infer_problems into per-trajectory dt0 and
 * tolerance-scale arrays (8 bytes per trajectory of scratch, from the stream-ordered
 * allocator), then degpu_vectorized_asolve with them.  opt->dt0 / opt->tolscale are
 * ignored; dt0 is clamped to [dt_lo, dt_hi], the scale to [1, s_max]. */
int degpu_learned_asolve(const degpu_rhs* f, const degpu_mlp* m, const degpu_problems* probs, const degpu_options* opt,
                         float dt_lo, float dt_hi, float s_max, degpu_outputs* out, void* stream);
/* degpu_learned_asolve for callers that cannot allocate device memory during a solve
 * (host callbacks, fixed-budget or real-time runtimes that own all device memory).  No
 * counterpart in the reference.  Same arguments and results as degpu_learned_asolve, but
 * its scratch (dt0 and tolerance scale, 8 bytes per trajectory, plus the work counter)
 * is a static array in the library's device image sized for at most
 * DEGPU_NOALLOC_MAX_TRAJECTORIES trajectories per call (larger calls return
 * DEGPU_E_INVALID).  It calls no allocator.  The first call on a device resolves the
 * array's address (cudaGetSymbolAddress), and the first call with a new right-hand side or
 * option set compiles and loads its kernels: make those first calls before any stream
 * capture.  All calls share the one array: calls that overlap on the GPU race and must be
 * serialised by the caller. */
#define DEGPU_NOALLOC_MAX_TRAJECTORIES 262144
int degpu_learned_asolve_noalloc(const degpu_rhs* f, const degpu_mlp* m, const degpu_problems* probs,
                                 const degpu_options* opt, float dt_lo, float dt_hi, float s_max, degpu_outputs* out,
                                 void* stream);
/* Visiting order for the persistent driver from a per-trajectory work estimate (device
 * work [B], e.g. predicted step attempts): order [B] (device) lists the trajectories by
 * descending work in quarter-octave classes of the estimate (floor(4 log2 work), clamped
 * to 0..127; NaN and work < 1 fall in class 0), in unspecified order inside a class.
 * Longest-first visiting shortens the tail of an ensemble with uneven step counts, where
 * each warp drains its last lanes one by one.  Scratch: 1 KB from the stream-ordered
 * allocator.  No counterpart in the reference. */
int degpu_work_order(const float* work, long long B, int* order, void* stream);
/* degpu_learned_asolve with optional parts: `m` (may be NULL: plain controller) predicts
 * dt0 and the tolerance scale as above; `work_model` (may be NULL: index order) is a
 * degpu_mlp whose first output is the predicted log step attempts of this solve, turned
 * into a visiting order by degpu_work_order.  Either model may take one more input after
 * log10 reltol, the span tf - t0 of each trajectory's tspan (input width N + P + 2), for
 * ensembles with per-trajectory tspans.  Scratch: 8 bytes per trajectory per model (the
 * work model's 8 are its prediction and the order), from the stream-ordered allocator.
 * opt->dt0 / tolscale / order are ignored. */
int degpu_learned_asolve_ex(const degpu_rhs* f, const degpu_mlp* m, const degpu_mlp* work_model,
                            const degpu_problems* probs, const degpu_options* opt, float dt_lo, float dt_hi,
                            float s_max, degpu_outputs* out, void* stream);
/* degpu_batch_solve_host (adaptive ODE solves) with the learned parts of
 * degpu_learned_asolve_ex: host buffers in and out, the models' inference and the
 * longest-first order run on the device copies of the inputs (per chunk on the pipelined
 * path).  Either model may be NULL.  With a work model the outputs are staged in device
 * memory and copied back in pipelined chunks even when they are page-locked (an ordered
 * solve's direct writes into host memory arrive scattered; DEGPU_HOST_DIRECT=1 forces
 * them). */
int degpu_learned_batch_solve_host(const degpu_rhs* f, const degpu_mlp* step_model, const degpu_mlp* work_model,
                                   const float* u0, const float* p, const void* tspan, long long B,
                                   const degpu_options* opt, float dt_lo, float dt_hi, float s_max, void* ts,
                                   float* us, int L, signed char* retcode, int* naccept, int* nreject, void* stream);
/* Gradient of the weighted mean squared error over a device batch (target, weight [B][2];
 * weight may be NULL) into the model's gradient buffer; *loss (device scalar, optional). */
int degpu_mlp_grad(degpu_mlp* m, const float* x, const float* target, const float* weight, long long B, float* loss,
                   void* stream);
/* One Adam step (bias-corrected) with decoupled-into-gradient weight decay. */
int degpu_mlp_adam_step(degpu_mlp* m, float lr, float beta1, float beta2, float eps, float weight_decay, void* stream);

/* ---- measurement utilities (no counterpart in the reference) ---- */
/* Sustained FP32 FMA throughput of the current device in TFLOP/s (8 independent FMA
 * chains per thread over a grid that fills every SM); the roofline denominator that
 * bench.py reports the stepping kernels against. */
int degpu_fp32_peak(double* tflops, void* stream);

#ifdef __cplusplus
}
#endif
#endif
