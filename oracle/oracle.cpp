/* CPU oracle for the EnsembleGPUKernel hot path of DiffEqGPU.jl -- TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py (CPU-baseline leg and the
 * `--impl reference` arm) load this library, and only as the checker / the timed CPU
 * reference.  The product (libdegpu.so + its kernels) never links or calls it.
 *
 * What it restates (all paths relative to the DiffEqGPU.jl checkout):
 *   driver loops        src/ensemblegpukernel/kernels.jl:1-152 (ode_solve_kernel, ode_asolve_kernel)
 *   saveat / sizing     src/ensemblegpukernel/lowerlevel_solve.jl:53-131, 253-346
 *   savevalues!         src/ensemblegpukernel/integrators/integrator_utils.jl:13-50
 *   controller consts   src/ensemblegpukernel/integrators/integrator_utils.jl:1-11
 *   Tsit5 step!         src/ensemblegpukernel/perform_step/gpu_tsit5_perform_step.jl:1-175
 *   Vern7 step!         src/ensemblegpukernel/perform_step/gpu_vern7_perform_step.jl:1-210
 *   Rosenbrock23 step!  src/ensemblegpukernel/perform_step/gpu_rosenbrock23_perform_step.jl:1-201
 *   Rodas5P step!       src/ensemblegpukernel/perform_step/gpu_rodas5P_perform_step.jl:1-351
 *   EM kernel           src/ensemblegpukernel/perform_step/gpu_em_perform_step.jl:1-74
 *   interpolants        src/ensemblegpukernel/integrators/nonstiff/interpolants.jl:28-190, 372-399,
 *                       src/ensemblegpukernel/integrators/stiff/interpolants.jl:13-23
 *   3x3 linear solve    src/ensemblegpukernel/linalg/linsolve.jl:31-57 (Cramer's rule)
 *   J / tgrad           src/ensemblegpukernel/nlsolve/type.jl:129-157, alg_utils.jl:17-27
 *   norm                DiffEqBase.ODE_DEFAULT_NORM for static arrays: sqrt(sum(abs2,u)/length(u))
 *
 * Arithmetic is FP32 in the reference's operation order (n-ary `+` folds left,
 * `dt*a*k` = `(dt*a)*k`), built with -ffp-contract=off.  Coefficients come from
 * tableaus_gen.h (Vern7, Rodas5P, Vern9; generated from the reference's tableau files)
 * and, for Tsit5, from Tsitouras (2011) -- the reference takes them from the un-vendored
 * SimpleDiffEq 1.11 (`_build_tsit5_caches`, `bθs`); their order conditions are checked
 * in tests/test_oracle.py.
 *
 * Documented deviations from the reference (the same in the kernels' parity mode):
 *   - `EEst^beta1`, `qold^beta2` use pm_powf (portable_math.h), not libm/CUDA pow;
 *   - interpolants (`@muladd` in the reference) are evaluated without FMA;
 *   - `error("dt<dtmin")` becomes retcode DtLessThanMin, and an attempt cap (maxiters)
 *     ends runaway trajectories with retcode MaxIters instead of looping forever;
 *   - with an FP64 tspan, time is held as an unevaluated float pair (hi, lo) advanced by
 *     error-free TwoSum/Fast2Sum (the kernels' FP64-time mode, ~48-bit time on FP32
 *     pipes); with a Float32 tspan every time operation is the reference's Float32 one.
 * Parity status: bit-faithful restatement for the fixed-step explicit RK path (only
 * +,-,* in a fixed order); adaptive paths pinned by the FP64 Vern9 solution and the
 * reference's own test tolerances -- the reference (Julia) cannot run in this build.
 *
 * Also here: an FP64 Vern9 solver (tableau: tableaus/verner_tableaus.jl:1198-1332) used
 * as the high-accuracy error oracle, and OpenMP ensemble drivers (the timed CPU baseline).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#include "portable_math.h"
#include "tableaus_gen.h"

/* ------------------------------------------------------------------ constants */
enum { ALG_TSIT5 = 0, ALG_VERN7 = 1, ALG_RB23 = 2, ALG_RODAS5P = 3, ALG_EM = 4, ALG_RODAS4 = 5, ALG_VERN9 = 6, ALG_SIEA = 7, ALG_KVAERNO3 = 8, ALG_KVAERNO5 = 9 };
enum { RET_DEFAULT = 0, RET_SUCCESS = 1, RET_TERMINATED = 2, RET_DTMIN = 3, RET_MAXITERS = 4, RET_UNSTABLE = 5 };
enum { JAC_AD = 0, JAC_ANALYTIC = 1, JAC_FINITEDIFF = 2 };
enum {
  M_LORENZ = 0, M_ROBERTSON = 1, M_DECAY = 2, M_GROWTH = 3, M_LINEAR15 = 4,
  M_GBM = 5, M_LORENZ_ADDNOISE = 6, M_OSC = 7, M_BALL = 8, M_ROBER_DAE = 9
};
#define MAXN 16
#define MAXP 8

/* ------------------------------------------------------------------ dual numbers
 * Forward-mode duals with NP partials, product rule ordered like ForwardDiff's
 * `x*y -> (vx*vy, partials(x)*vy + partials(y)*vx)`. */
template <int NP> struct Dual {
  float v; float d[NP];
  Dual() : v(0.f) { for (int i = 0; i < NP; i++) d[i] = 0.f; }
  Dual(float x) : v(x) { for (int i = 0; i < NP; i++) d[i] = 0.f; }
};
template <int NP> static inline Dual<NP> operator+(Dual<NP> a, Dual<NP> b) { Dual<NP> r; r.v = a.v + b.v; for (int i = 0; i < NP; i++) r.d[i] = a.d[i] + b.d[i]; return r; }
template <int NP> static inline Dual<NP> operator-(Dual<NP> a, Dual<NP> b) { Dual<NP> r; r.v = a.v - b.v; for (int i = 0; i < NP; i++) r.d[i] = a.d[i] - b.d[i]; return r; }
template <int NP> static inline Dual<NP> operator-(Dual<NP> a) { Dual<NP> r; r.v = -a.v; for (int i = 0; i < NP; i++) r.d[i] = -a.d[i]; return r; }
template <int NP> static inline Dual<NP> operator*(Dual<NP> a, Dual<NP> b) { Dual<NP> r; r.v = a.v * b.v; for (int i = 0; i < NP; i++) r.d[i] = a.d[i] * b.v + b.d[i] * a.v; return r; }
template <int NP> static inline Dual<NP> operator*(float a, Dual<NP> b) { Dual<NP> r; r.v = a * b.v; for (int i = 0; i < NP; i++) r.d[i] = a * b.d[i]; return r; }
template <int NP> static inline Dual<NP> operator*(Dual<NP> b, float a) { Dual<NP> r; r.v = b.v * a; for (int i = 0; i < NP; i++) r.d[i] = b.d[i] * a; return r; }
template <int NP> static inline Dual<NP> operator+(float a, Dual<NP> b) { Dual<NP> r = b; r.v = a + b.v; return r; }
template <int NP> static inline Dual<NP> operator+(Dual<NP> b, float a) { Dual<NP> r = b; r.v = b.v + a; return r; }
template <int NP> static inline Dual<NP> operator-(float a, Dual<NP> b) { Dual<NP> r; r.v = a - b.v; for (int i = 0; i < NP; i++) r.d[i] = -b.d[i]; return r; }
template <int NP> static inline Dual<NP> operator-(Dual<NP> b, float a) { Dual<NP> r = b; r.v = b.v - a; return r; }

/* ------------------------------------------------------------------ models
 * Right-hand sides written with the same operation order as the CUDA C sources the
 * tests hand to the library (diffeqgpu.jl_gb300/degpu/models.py).  S is float or Dual.
 *   lorenz     test/gpu_kernel_de/gpu_ode_regression.jl:4-12
 *   robertson  test/gpu_kernel_de/stiff_ode/gpu_ode_mass_matrix.jl (ODE form of its kinetics)
 *   decay      test/gpu_kernel_de/stiff_ode/gpu_ode_regression.jl:5-8   (u' = -p1 u)
 *   growth     test/public_interface.jl:9-11                           (u' = u)
 *   linear15   test/gpu_kernel_de/stiff_ode/gpu_ode_regression.jl:24-26 (u' = 1.01 u, N=15)
 *   gbm        test/gpu_kernel_de/gpu_sde_convergence.jl:6-8           (f = p1 u, g = p2 u)
 *   lorenz+additive noise  test/gpu_kernel_de/gpu_sde_regression.jl:47-58
 *   osc        harmonic oscillator u1' = u2, u2' = -p1^2 u1 (non-chaotic known answer)
 *   ball       bouncing ball u1' = u2, u2' = -p1 (test/gpu_kernel_de/gpu_ode_continuous_callbacks.jl:6-10)
 *   robertson_dae  Robertson with the constraint y1 + y2 + y3 = 1 and mass matrix diag(1,1,0)
 *              (test/gpu_kernel_de/stiff_ode/gpu_ode_mass_matrix.jl:5-31) */
struct ModelInfo { int N, P, has_jac, has_tgrad, is_sde; };
static ModelInfo model_info(int m) {
  switch (m) {
    case M_LORENZ: return {3, 3, 1, 1, 0};
    case M_ROBERTSON: return {3, 3, 1, 1, 0};
    case M_DECAY: return {1, 1, 1, 1, 0};
    case M_GROWTH: return {1, 1, 0, 0, 0};
    case M_LINEAR15: return {15, 1, 0, 0, 0};
    case M_GBM: return {1, 2, 0, 0, 1};
    case M_LORENZ_ADDNOISE: return {3, 3, 0, 0, 1};
    case M_OSC: return {2, 1, 1, 1, 0};
    case M_BALL: return {2, 1, 0, 0, 0};
    case M_ROBER_DAE: return {3, 3, 0, 0, 0};
  }
  return {0, 0, 0, 0, 0};
}

template <class S>
static void model_f(int m, S* du, const S* u, const float* p, float t) {
  (void)t;
  switch (m) {
    case M_LORENZ:
    case M_LORENZ_ADDNOISE: {
      du[0] = p[0] * (u[1] - u[0]);
      du[1] = u[0] * (p[1] - u[2]) - u[1];
      du[2] = u[0] * u[1] - p[2] * u[2];
    } break;
    case M_ROBERTSON: {
      du[0] = -p[0] * u[0] + p[2] * u[1] * u[2];
      du[1] = p[0] * u[0] - p[1] * u[1] * u[1] - p[2] * u[1] * u[2];
      du[2] = p[1] * u[1] * u[1];
    } break;
    case M_DECAY: du[0] = -p[0] * u[0]; break;
    case M_GROWTH: du[0] = u[0]; break;
    case M_LINEAR15: for (int i = 0; i < 15; i++) du[i] = 1.01f * u[i]; break;
    case M_GBM: du[0] = p[0] * u[0]; break;
    case M_OSC: { du[0] = u[1]; du[1] = -(p[0] * p[0]) * u[0]; } break;
    case M_BALL: { du[0] = u[1]; du[1] = S(-p[0]); } break;
    case M_ROBER_DAE: {
      du[0] = -p[0] * u[0] + p[2] * u[1] * u[2];
      du[1] = p[0] * u[0] - p[1] * (u[1] * u[1]) - p[2] * u[1] * u[2];
      du[2] = u[0] + u[1] + u[2] - 1.0f;
    } break;
  }
}

/* constant mass matrix (column-major) of the models that have one; returns 0 for M = I */
static int model_mass(int m, float* M) {
  if (m != M_ROBER_DAE) return 0;
  for (int i = 0; i < 9; i++) M[i] = 0.0f;
  M[0] = 1.0f; M[4] = 1.0f;
  return 1;
}
/* mass_matrix * v, rows summed left to right */
static void mass_mul(int N, const float* M, const float* v, float* out) {
  for (int i = 0; i < N; i++) {
    float acc = M[i] * v[0];
    for (int j = 1; j < N; j++) acc = acc + M[i + N * j] * v[j];
    out[i] = acc;
  }
}

/* analytic Jacobian (column-major J[i + N*j] = d f_i / d u_j) */
static void model_jac(int m, float* J, const float* u, const float* p, float t) {
  (void)t;
  switch (m) {
    case M_LORENZ:
      J[0] = -p[0]; J[1] = p[1] - u[2]; J[2] = u[1];
      J[3] = p[0]; J[4] = -1.0f; J[5] = u[0];
      J[6] = 0.0f; J[7] = -u[0]; J[8] = -p[2];
      break;
    case M_ROBERTSON:
      J[0] = -p[0]; J[1] = p[0]; J[2] = 0.0f;
      J[3] = p[2] * u[2]; J[4] = -(p[1] * u[1] + p[1] * u[1]) - p[2] * u[2]; J[5] = p[1] * u[1] + p[1] * u[1];
      J[6] = p[2] * u[1]; J[7] = -(p[2] * u[1]); J[8] = 0.0f;
      break;
    case M_DECAY: J[0] = -p[0]; break;
    case M_OSC: J[0] = 0.0f; J[1] = -(p[0] * p[0]); J[2] = 1.0f; J[3] = 0.0f; break;
  }
}
static void model_tgrad(int m, float* dT, int N) { (void)m; for (int i = 0; i < N; i++) dT[i] = 0.0f; }

/* callbacks of the models that define them, with the expressions of their CUDA C sources
 *   ball   continuous fn 0: condition u1, affect! = affect_neg! : u += (0, -2) .* u
 *                         (gpu_ode_continuous_callbacks.jl:18-24); fn 1: terminate! at contact
 *   decay  discrete fn 0: t == 2.4, fn 1: t == 4.0 (u += 10; gpu_ode_discrete_callbacks.jl:16-22
 *          with tstops at those times); fn 2: terminate! once u < 1 */
struct CbInteg { float* u; const float* p; double t; float dt; int terminated; };
static float model_ccb_condition(int m, int fn, const float* u, const float* p, double t) {
  (void)fn; (void)p; (void)t;
  if (m == M_BALL) return u[0];
  return 0.0f;
}
static void model_ccb_affect(int m, int fn, CbInteg& I) {
  if (m == M_BALL) {
    if (fn == 1) { I.terminated = 1; return; }
    I.u[0] = I.u[0] + 0.0f * I.u[0];
    I.u[1] = I.u[1] + -2.0f * I.u[1];
  }
}
static int model_dcb_condition(int m, int fn, const float* u, const float* p, double t) {
  (void)p;
  if (m != M_DECAY) return 0;
  if (fn == 0) return (float)t == 2.4f;
  if (fn == 1) return (float)t == 4.0f;
  return u[0] < 1.0f;
}
static void model_dcb_affect(int m, int fn, CbInteg& I) {
  if (m != M_DECAY) return;
  if (fn == 2) { I.terminated = 1; return; }
  I.u[0] = I.u[0] + 10.0f;
}

/* SDE noise g (diagonal) */
static void model_g(int m, float* g, const float* u, const float* p) {
  switch (m) {
    case M_GBM: g[0] = p[1] * u[0]; break;
    case M_LORENZ_ADDNOISE: g[0] = 3.0f; g[1] = 3.0f; g[2] = 3.0f; break;
  }
}

/* Jacobian and time-gradient per build_J_W / build_tgrad (nlsolve/type.jl:129-157). */
static void compute_J(int m, int jacmode, int N, float* J, const float* u, const float* p, float t) {
  ModelInfo mi = model_info(m);
  if (jacmode == JAC_ANALYTIC && mi.has_jac) { model_jac(m, J, u, p, t); return; }
  if (jacmode == JAC_FINITEDIFF) {
    /* finite_diff_jac, alg_utils.jl:17-27: dx = sqrt(eps(T)), column i = (f(x+dx e_i) - f(x)) / dx */
    const float dx = sqrtf(1.1920929e-07f);
    float f0[MAXN], f1[MAXN], x[MAXN];
    model_f<float>(m, f0, u, p, t);
    for (int j = 0; j < N; j++) {
      for (int i = 0; i < N; i++) x[i] = u[i];
      x[j] = x[j] + dx;
      model_f<float>(m, f1, x, p, t);
      for (int i = 0; i < N; i++) J[i + N * j] = (f1[i] - f0[i]) / dx;
    }
    return;
  }
  /* ForwardDiff.jacobian: one chunk with N partials (N <= MAXN) */
  Dual<MAXN> ud[MAXN], fd[MAXN];
  for (int i = 0; i < N; i++) { ud[i] = Dual<MAXN>(u[i]); ud[i].d[i] = 1.0f; }
  model_f<Dual<MAXN>>(m, fd, ud, p, t);
  for (int j = 0; j < N; j++)
    for (int i = 0; i < N; i++) J[i + N * j] = fd[i].d[j];
}
static void compute_tgrad(int m, int jacmode, int N, float* dT, const float* u, const float* p, float t) {
  ModelInfo mi = model_info(m);
  if (jacmode == JAC_ANALYTIC && mi.has_tgrad) { model_tgrad(m, dT, N); return; }
  if (jacmode == JAC_FINITEDIFF) {
    const float h = sqrtf(1.1920929e-07f);
    float f0[MAXN], f1[MAXN];
    model_f<float>(m, f1, u, p, t + h);
    model_f<float>(m, f0, u, p, t);
    for (int i = 0; i < N; i++) dT[i] = (f1[i] - f0[i]) / h;
    return;
  }
  /* ForwardDiff.derivative w.r.t. t: all built-in models are autonomous */
  for (int i = 0; i < N; i++) dT[i] = 0.0f;
}

/* ------------------------------------------------------------------ helpers */
/* Julia's min/max propagate NaN (Base.min for AbstractFloat) */
static inline float jl_min(float x, float y) { if (x != x) return x; if (y != y) return y; return y < x ? y : x; }
static inline float jl_max(float x, float y) { if (x != x) return x; if (y != y) return y; return y > x ? y : x; }
static inline double jl_mind(double x, double y) { if (x != x) return x; if (y != y) return y; return y < x ? y : x; }

/* ------------------------------------------------------------------ time arithmetic
 * float: the reference's Float32 time.  DF: hi + lo exactly, TwoSum (Knuth) + Fast2Sum
 * (Dekker) accumulation -- the same operations, in the same order, as the kernels. */
struct DF { float hi, lo; };
template <class Tt> struct TOut;
template <> struct TOut<float> { typedef float T; };
template <> struct TOut<DF> { typedef double T; };
template <class Tt> static inline Tt t_from(double x);
template <> inline float t_from<float>(double x) { return (float)x; }
template <> inline DF t_from<DF>(double x) { DF r; r.hi = (float)x; r.lo = (float)(x - (double)r.hi); return r; }
static inline float t_out(float t) { return t; }
static inline double t_out(DF t) { return (double)t.hi + (double)t.lo; }
static inline float t_add(float t, float d) { return t + d; }
static inline DF t_add(DF t, float d) {
  float s = t.hi + d;
  float bb = s - t.hi;
  float e = (t.hi - (s - bb)) + (d - bb);
  e = e + t.lo;
  DF r;
  r.hi = s + e;
  r.lo = e - (r.hi - s);
  return r;
}
static inline float t_rem(float tf, float t, float dt) { return tf - t - dt; }
static inline float t_rem(DF tf, DF t, float dt) { return ((tf.hi - t.hi) + (tf.lo - t.lo)) - dt; }
static inline bool t_lt(float a, float b) { return a < b; }
static inline bool t_lt(DF a, DF b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
static inline bool t_le(float a, float b) { return a <= b; }
static inline bool t_le(DF a, DF b) { return a.hi < b.hi || (a.hi == b.hi && a.lo <= b.lo); }
static inline float t_stage(float t, float c, float dt) { return t + c * dt; }
static inline float t_stage(DF t, float c, float dt) { return t.hi + (t.lo + c * dt); }
static inline float t_theta(float s, float tp, float dt) { return (s - tp) / dt; }
static inline float t_theta(DF s, DF tp, float dt) { return ((s.hi - tp.hi) + (s.lo - tp.lo)) / dt; }
static inline float t_em_theta(float s, float t, float dt) { return (s - (t - dt)) / dt; }
static inline float t_em_theta(DF s, DF t, float dt) { return (((s.hi - t.hi) + (s.lo - t.lo)) + dt) / dt; }
static inline float t_f32(float t) { return t; }
static inline float t_f32(DF t) { return t.hi + t.lo; }

/* DiffEqBase.ODE_DEFAULT_NORM for a static vector: sqrt(sum(abs2, u) / length(u)) */
static inline float ode_norm(const float* x, int N) {
  float s = x[0] * x[0];
  for (int i = 1; i < N; i++) s = s + x[i] * x[i];
  return sqrtf(s / (float)N);
}

/* Tsitouras (2011) 5(4) coefficients, as SimpleDiffEq builds them (convert(T, Float64)). */
struct Tsit5Tab {
  float c1, c2, c3, c4, c5, c6;
  float a21, a31, a32, a41, a42, a43, a51, a52, a53, a54, a61, a62, a63, a64, a65, a71, a72, a73, a74, a75, a76;
  float bt1, bt2, bt3, bt4, bt5, bt6, bt7;
  float r11, r12, r13, r14, r22, r23, r24, r32, r33, r34, r42, r43, r44, r52, r53, r54, r62, r63, r64, r72, r73, r74;
};
static Tsit5Tab make_tsit5() {
  Tsit5Tab T;
  T.c1 = (float)0.161; T.c2 = (float)0.327; T.c3 = (float)0.9; T.c4 = (float)0.9800255409045097; T.c5 = 1.0f; T.c6 = 1.0f;
  T.a21 = (float)0.161;
  T.a31 = (float)-0.008480655492356989; T.a32 = (float)0.335480655492357;
  T.a41 = (float)2.897153057105493; T.a42 = (float)-6.359448489975075; T.a43 = (float)4.3622954328695815;
  T.a51 = (float)5.325864828439257; T.a52 = (float)-11.748883564062828; T.a53 = (float)7.4955393428898365; T.a54 = (float)-0.09249506636175525;
  T.a61 = (float)5.86145544294642; T.a62 = (float)-12.92096931784711; T.a63 = (float)8.159367898576159; T.a64 = (float)-0.071584973281401; T.a65 = (float)-0.028269050394068383;
  T.a71 = (float)0.09646076681806523; T.a72 = (float)0.01; T.a73 = (float)0.4798896504144996; T.a74 = (float)1.379008574103742; T.a75 = (float)-3.290069515436081; T.a76 = (float)2.324710524099774;
  T.bt1 = (float)-0.00178001105222577714; T.bt2 = (float)-0.0008164344596567469; T.bt3 = (float)0.007880878010261995;
  T.bt4 = (float)-0.1447110071732629; T.bt5 = (float)0.5823571654525552; T.bt6 = (float)-0.45808210592918697; T.bt7 = (float)0.015151515151515152;
  T.r11 = 1.0f; T.r12 = (float)-2.763706197274826; T.r13 = (float)2.9132554618219126; T.r14 = (float)-1.0530884977290216;
  T.r22 = (float)0.13169999999999998; T.r23 = (float)-0.2234; T.r24 = (float)0.1017;
  T.r32 = (float)3.9302962368947516; T.r33 = (float)-5.941033872131505; T.r34 = (float)2.490627285651253;
  T.r42 = (float)-12.411077166933676; T.r43 = (float)30.33818863028232; T.r44 = (float)-16.548102889244902;
  T.r52 = (float)37.50931341651104; T.r53 = (float)-88.1789048947664; T.r54 = (float)47.37952196281928;
  T.r62 = (float)-27.896526289197286; T.r63 = (float)65.09189467479366; T.r64 = (float)-34.87065786149661;
  T.r72 = 1.5f; T.r73 = -4.0f; T.r74 = 2.5f;
  return T;
}
static const Tsit5Tab TS5 = make_tsit5();

static float V7[OR_VERN7_COUNT], V7X[OR_VERN7X_COUNT], V7I[OR_VERN7I_COUNT], R5P[OR_RODAS5P_COUNT], R4T[OR_RODAS4_COUNT];
static float F9[OR_VERN9_COUNT], F9X[OR_VERN9X_COUNT], F9I[OR_VERN9I_COUNT], FK3[OR_KVAERNO3_COUNT], FK5[OR_KVAERNO5_COUNT];
static int tabs_ready = 0;
static void init_tabs() {
  if (tabs_ready) return;
#pragma omp critical(oracle_tabs)
  {
    if (!tabs_ready) {
      for (int i = 0; i < OR_VERN7_COUNT; i++) V7[i] = (float)OR_VERN7[i];
      for (int i = 0; i < OR_VERN7X_COUNT; i++) V7X[i] = (float)OR_VERN7X[i];
      for (int i = 0; i < OR_VERN7I_COUNT; i++) V7I[i] = (float)OR_VERN7I[i];
      for (int i = 0; i < OR_RODAS5P_COUNT; i++) R5P[i] = (float)OR_RODAS5P[i];
      for (int i = 0; i < OR_RODAS4_COUNT; i++) R4T[i] = (float)OR_RODAS4[i];
      for (int i = 0; i < OR_VERN9_COUNT; i++) F9[i] = (float)OR_VERN9[i];
      for (int i = 0; i < OR_VERN9X_COUNT; i++) F9X[i] = (float)OR_VERN9X[i];
      for (int i = 0; i < OR_VERN9I_COUNT; i++) F9I[i] = (float)OR_VERN9I[i];
      for (int i = 0; i < OR_KVAERNO3_COUNT; i++) FK3[i] = (float)OR_KVAERNO3[i];
      for (int i = 0; i < OR_KVAERNO5_COUNT; i++) FK5[i] = (float)OR_KVAERNO5[i];
      tabs_ready = 1;
    }
  }
}
#define V7C(n) V7[OR_VERN7_##n]
#define V7XC(n) V7X[OR_VERN7X_##n]
#define V7IC(n) V7I[OR_VERN7I_##n]
#define RPC(n) R5P[OR_RODAS5P_##n]
#define R4C(n) R4T[OR_RODAS4_##n]
#define F9C(n) F9[OR_VERN9_##n]
#define F9XC(n) F9X[OR_VERN9X_##n]
#define F9IC(n) F9I[OR_VERN9I_##n]
#define K3C(n) FK3[OR_KVAERNO3_##n]
#define K5C(n) FK5[OR_KVAERNO5_##n]

/* ------------------------------------------------------------------ configuration */
extern "C" {
typedef struct {
  int alg;             /* ALG_* */
  int adaptive;        /* 0: vectorized_solve, 1: vectorized_asolve */
  int time_f64;        /* time type Tt: 0 = Float32 (the reference's Float32 tspan), 1 = Float64 */
  int save_everystep;
  int L;               /* saved points per trajectory (output rows) */
  int nsaveat;         /* 0: no saveat */
  int saveat_per_traj; /* saveat is [B][nsaveat] instead of [nsaveat] */
  int jac;             /* JAC_* */
  const double* saveat;
  double dt;           /* fixed dt / initial dt (converted to Tt as convert(eltype(tspan), dt)) */
  float abstol, reltol;
  long long maxiters;  /* cap on step attempts per trajectory */
  unsigned long long seed; /* EM: key of the counter-based generator */
  const float* dt0;    /* optional per-trajectory initial dt (overrides dt) */
  const float* tolscale; /* optional per-trajectory multiplier of abstol and reltol */
  int ntstops;         /* tstops (ascending, shared by all trajectories) */
  const double* tstops;
  int nccb;            /* continuous callbacks: function index, flags (bit 0 affect!, bit 1
                        * affect_neg!, bits 2-3 root-find mode), abstol, repeat nudge, dtrelax */
  int ccb_fn[8], ccb_flags[8];
  float ccb_abstol[8], ccb_nudge[8], ccb_dtrelax[8];
  int ndcb;            /* discrete callbacks: function index */
  int dcb_fn[8];
} oracle_cfg;
}

/* ------------------------------------------------------------------ integrator state
 * One struct for all algorithms (the reference's GPU*Integrator structs, types.jl). */
template <class Tt> struct Integ {
  int N;
  float u[MAXN], uprev[MAXN];
  float k[10][MAXN];      /* Tsit5 k1..k7, Vern7 k1..k10, RB23 k1..k3, Rodas5P dense k1..k3 */
  float J[MAXN * MAXN], dT[MAXN]; /* Rodas5P: per-step Jacobian (computed once per step) */
  Tt t, tprev, tf;
  float dt, dtnew, qold;
  float abstol, reltol;
  int u_modified;
  int cur_t, step_idx;
  int retcode;
  long long nattempt, naccept, nreject;
  int tstops_idx;          /* next tstop, 0-based */
  int event_last;          /* event_last_time (1-based callback index, 0 = none) */
  float last_event_error;  /* condition residual at the last located event */
};

/* time argument handed to f: `t + c*dt` in Tt, passed to the FP32 right-hand side */
template <class Tt> static inline float tstage(Tt t, float c, float dt) { return t_stage(t, c, dt); }

/* ------------------------------------------------------------------ Tsit5 */
/* stage block shared by gpu_tsit5_perform_step.jl:36-49 (fixed) and :104-115 (adaptive).
 * `last6` selects the fixed-step grouping of the final combination (:47-48). */
template <class Tt>
static void tsit5_stages(int m, Integ<Tt>& ig, const float* p, Tt t, float dt, const float* k1, float* u, float (*k)[MAXN], int fixed_grouping) {
  const Tsit5Tab& T = TS5;
  int N = ig.N;
  const float* up = ig.uprev;
  float tmp[MAXN], k2[MAXN], k3[MAXN], k4[MAXN], k5[MAXN], k6[MAXN], k7[MAXN];
  for (int i = 0; i < N; i++) tmp[i] = up[i] + (dt * T.a21) * k1[i];
  model_f<float>(m, k2, tmp, p, tstage(t, T.c1, dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (T.a31 * k1[i] + T.a32 * k2[i]);
  model_f<float>(m, k3, tmp, p, tstage(t, T.c2, dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (T.a41 * k1[i] + T.a42 * k2[i] + T.a43 * k3[i]);
  model_f<float>(m, k4, tmp, p, tstage(t, T.c3, dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (T.a51 * k1[i] + T.a52 * k2[i] + T.a53 * k3[i] + T.a54 * k4[i]);
  model_f<float>(m, k5, tmp, p, tstage(t, T.c4, dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (T.a61 * k1[i] + T.a62 * k2[i] + T.a63 * k3[i] + T.a64 * k4[i] + T.a65 * k5[i]);
  model_f<float>(m, k6, tmp, p, t_stage(t, 1.0f, dt));
  for (int i = 0; i < N; i++) {
    if (fixed_grouping)
      u[i] = up[i] + dt * ((T.a71 * k1[i] + T.a72 * k2[i] + T.a73 * k3[i] + T.a74 * k4[i]) + T.a75 * k5[i] + T.a76 * k6[i]);
    else
      u[i] = up[i] + dt * (T.a71 * k1[i] + T.a72 * k2[i] + T.a73 * k3[i] + T.a74 * k4[i] + T.a75 * k5[i] + T.a76 * k6[i]);
  }
  model_f<float>(m, k7, u, p, t_stage(t, 1.0f, dt));
  for (int i = 0; i < N; i++) {
    k[0][i] = k1[i]; k[1][i] = k2[i]; k[2][i] = k3[i]; k[3][i] = k4[i];
    k[4][i] = k5[i]; k[5][i] = k6[i]; k[6][i] = k7[i];
  }
}

/* SimpleDiffEq.bθs: b_iθ by Horner from the highest coefficient */
static void tsit5_btheta(float th, float* b) {
  const Tsit5Tab& T = TS5;
  b[0] = (((T.r14 * th + T.r13) * th + T.r12) * th + T.r11) * th;
  b[1] = (((T.r24 * th + T.r23) * th + T.r22) * th) * th;
  b[2] = (((T.r34 * th + T.r33) * th + T.r32) * th) * th;
  b[3] = (((T.r44 * th + T.r43) * th + T.r42) * th) * th;
  b[4] = (((T.r54 * th + T.r53) * th + T.r52) * th) * th;
  b[5] = (((T.r64 * th + T.r63) * th + T.r62) * th) * th;
  b[6] = (((T.r74 * th + T.r73) * th + T.r72) * th) * th;
}

/* ------------------------------------------------------------------ Vern7 (k1 recomputed: not FSAL) */
template <class Tt>
static void vern7_stages(int m, Integ<Tt>& ig, const float* p, Tt t, float dt, float* u, float (*k)[MAXN]) {
  int N = ig.N;
  const float* up = ig.uprev;
  float tmp[MAXN];
  float* k1 = k[0]; float* k2 = k[1]; float* k3 = k[2]; float* k4 = k[3]; float* k5 = k[4];
  float* k6 = k[5]; float* k7 = k[6]; float* k8 = k[7]; float* k9 = k[8]; float* k10 = k[9];
  model_f<float>(m, k1, up, p, t_f32(t));
  float a = dt * V7C(a021);
  for (int i = 0; i < N; i++) tmp[i] = up[i] + a * k1[i];
  model_f<float>(m, k2, tmp, p, tstage(t, V7C(c2), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (V7C(a031) * k1[i] + V7C(a032) * k2[i]);
  model_f<float>(m, k3, tmp, p, tstage(t, V7C(c3), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (V7C(a041) * k1[i] + V7C(a043) * k3[i]);
  model_f<float>(m, k4, tmp, p, tstage(t, V7C(c4), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (V7C(a051) * k1[i] + V7C(a053) * k3[i] + V7C(a054) * k4[i]);
  model_f<float>(m, k5, tmp, p, tstage(t, V7C(c5), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (V7C(a061) * k1[i] + V7C(a063) * k3[i] + V7C(a064) * k4[i] + V7C(a065) * k5[i]);
  model_f<float>(m, k6, tmp, p, tstage(t, V7C(c6), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (V7C(a071) * k1[i] + V7C(a073) * k3[i] + V7C(a074) * k4[i] + V7C(a075) * k5[i] + V7C(a076) * k6[i]);
  model_f<float>(m, k7, tmp, p, tstage(t, V7C(c7), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (V7C(a081) * k1[i] + V7C(a083) * k3[i] + V7C(a084) * k4[i] + V7C(a085) * k5[i] + V7C(a086) * k6[i] + V7C(a087) * k7[i]);
  model_f<float>(m, k8, tmp, p, tstage(t, V7C(c8), dt));
  float g9[MAXN], g10[MAXN];
  for (int i = 0; i < N; i++) {
    g9[i] = up[i] + dt * (V7C(a091) * k1[i] + V7C(a093) * k3[i] + V7C(a094) * k4[i] + V7C(a095) * k5[i] + V7C(a096) * k6[i] + V7C(a097) * k7[i] + V7C(a098) * k8[i]);
    g10[i] = up[i] + dt * (V7C(a101) * k1[i] + V7C(a103) * k3[i] + V7C(a104) * k4[i] + V7C(a105) * k5[i] + V7C(a106) * k6[i] + V7C(a107) * k7[i]);
  }
  model_f<float>(m, k9, g9, p, t_stage(t, 1.0f, dt));
  model_f<float>(m, k10, g10, p, t_stage(t, 1.0f, dt));
  for (int i = 0; i < N; i++)
    u[i] = up[i] + dt * (V7C(b1) * k1[i] + V7C(b4) * k4[i] + V7C(b5) * k5[i] + V7C(b6) * k6[i] + V7C(b7) * k7[i] + V7C(b8) * k8[i] + V7C(b9) * k9[i]);
}

/* q_i(Θ) tail-sum polynomials, nonstiff/interpolants.jl:28-88 (Horner, no FMA) */
static inline float horner6(float th, float a0, float a1, float a2, float a3, float a4, float a5) {
  return ((((a5 * th + a4) * th + a3) * th + a2) * th + a1) * th + a0;
}
static void vern7_q(float th, float* q) {
#define SYN(II, OUT)                                                       \
  {                                                                        \
    float s5 = V7IC(r##II##7), s4 = V7IC(r##II##6) + s5, s3 = V7IC(r##II##5) + s4; \
    float s2 = V7IC(r##II##4) + s3, s1 = V7IC(r##II##3) + s2;                \
    OUT = horner6(th, V7IC(r##II##2) + s1, s1, s2, s3, s4, s5);             \
  }
  {
    float s15 = V7IC(r017), s14 = V7IC(r016) + s15, s13 = V7IC(r015) + s14, s12 = V7IC(r014) + s13;
    float s11 = V7IC(r013) + s12, s10 = V7IC(r012) + s11;
    q[0] = horner6(th, s10, s11, s12, s13, s14, s15);
  }
  SYN(04, q[1]) SYN(05, q[2]) SYN(06, q[3]) SYN(07, q[4]) SYN(08, q[5]) SYN(09, q[6])
  SYN(11, q[7]) SYN(12, q[8]) SYN(13, q[9]) SYN(14, q[10]) SYN(15, q[11]) SYN(16, q[12])
#undef SYN
}

template <class Tt>
static void vern7_interp(int m, const Integ<Tt>& ig, const float* p, float th, float dt, float* out) {
  int N = ig.N;
  const float* up = ig.uprev;
  const float(*k)[MAXN] = ig.k;
  float k11[MAXN], k12[MAXN], k13[MAXN], k14[MAXN], k15[MAXN], k16[MAXN], tmp[MAXN];
  const float *k1 = k[0], *k4 = k[3], *k5 = k[4], *k6 = k[5], *k7 = k[6], *k8 = k[7], *k9 = k[8];
  Tt tp = ig.tprev;
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (V7XC(a1101) * k1[i] + V7XC(a1104) * k4[i] + V7XC(a1105) * k5[i] + V7XC(a1106) * k6[i] + V7XC(a1107) * k7[i] + V7XC(a1108) * k8[i] + V7XC(a1109) * k9[i]);
  model_f<float>(m, k11, tmp, p, tstage(tp, V7XC(c11), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (V7XC(a1201) * k1[i] + V7XC(a1204) * k4[i] + V7XC(a1205) * k5[i] + V7XC(a1206) * k6[i] + V7XC(a1207) * k7[i] + V7XC(a1208) * k8[i] + V7XC(a1209) * k9[i] + V7XC(a1211) * k11[i]);
  model_f<float>(m, k12, tmp, p, tstage(tp, V7XC(c12), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (V7XC(a1301) * k1[i] + V7XC(a1304) * k4[i] + V7XC(a1305) * k5[i] + V7XC(a1306) * k6[i] + V7XC(a1307) * k7[i] + V7XC(a1308) * k8[i] + V7XC(a1309) * k9[i] + V7XC(a1311) * k11[i] + V7XC(a1312) * k12[i]);
  model_f<float>(m, k13, tmp, p, tstage(tp, V7XC(c13), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (V7XC(a1401) * k1[i] + V7XC(a1404) * k4[i] + V7XC(a1405) * k5[i] + V7XC(a1406) * k6[i] + V7XC(a1407) * k7[i] + V7XC(a1408) * k8[i] + V7XC(a1409) * k9[i] + V7XC(a1411) * k11[i] + V7XC(a1412) * k12[i] + V7XC(a1413) * k13[i]);
  model_f<float>(m, k14, tmp, p, tstage(tp, V7XC(c14), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (V7XC(a1501) * k1[i] + V7XC(a1504) * k4[i] + V7XC(a1505) * k5[i] + V7XC(a1506) * k6[i] + V7XC(a1507) * k7[i] + V7XC(a1508) * k8[i] + V7XC(a1509) * k9[i] + V7XC(a1511) * k11[i] + V7XC(a1512) * k12[i] + V7XC(a1513) * k13[i]);
  model_f<float>(m, k15, tmp, p, tstage(tp, V7XC(c15), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (V7XC(a1601) * k1[i] + V7XC(a1604) * k4[i] + V7XC(a1605) * k5[i] + V7XC(a1606) * k6[i] + V7XC(a1607) * k7[i] + V7XC(a1608) * k8[i] + V7XC(a1609) * k9[i] + V7XC(a1611) * k11[i] + V7XC(a1612) * k12[i] + V7XC(a1613) * k13[i]);
  model_f<float>(m, k16, tmp, p, tstage(tp, V7XC(c16), dt));
  float q[13];
  vern7_q(th, q);
  for (int i = 0; i < N; i++) {
    float step_sum = dt * (V7C(b1) * k1[i] + V7C(b4) * k4[i] + V7C(b5) * k5[i] + V7C(b6) * k6[i] + V7C(b7) * k7[i] + V7C(b8) * k8[i] + V7C(b9) * k9[i]);
    float corr = dt * (k1[i] * q[0] + k4[i] * q[1] + k5[i] * q[2] + k6[i] * q[3] + k7[i] * q[4] + k8[i] * q[5] + k9[i] * q[6] +
                       k11[i] * q[7] + k12[i] * q[8] + k13[i] * q[9] + k14[i] * q[10] + k15[i] * q[11] + k16[i] * q[12]);
    out[i] = up[i] + th * step_sum + th * (th - 1.0f) * corr;
  }
}

/* ------------------------------------------------------------------ linear algebra
 * linear_solve for N <= 3 (linsolve.jl:8-57): Cramer's rule with StaticArrays' det;
 * N > 3: partial-pivot LU (lu.jl) + triangular solves. */
static float det3(const float* a) { /* column-major; det = dot(c1, cross(c2, c3)) */
  float x0 = a[0], x1 = a[1], x2 = a[2];
  float y0 = a[3], y1 = a[4], y2 = a[5];
  float z0 = a[6], z1 = a[7], z2 = a[8];
  float c0 = y1 * z2 - y2 * z1, c1 = y2 * z0 - y0 * z2, c2 = y0 * z1 - y1 * z0;
  return x0 * c0 + x1 * c1 + x2 * c2;
}
#define A_(i, j) a[(i - 1) + N * (j - 1)]
static void linear_solve(int N, const float* a, const float* b, float* x) {
  if (N == 1) { x[0] = b[0] / a[0]; return; }
  if (N == 2) {
    float d = a[0] * a[3] - a[2] * a[1];
    x[0] = (A_(2, 2) * b[0] - A_(1, 2) * b[1]) / d;
    x[1] = (A_(1, 1) * b[1] - A_(2, 1) * b[0]) / d;
    return;
  }
  if (N == 3) {
    float d = det3(a);
    x[0] = ((A_(2, 2) * A_(3, 3) - A_(2, 3) * A_(3, 2)) * b[0] + (A_(1, 3) * A_(3, 2) - A_(1, 2) * A_(3, 3)) * b[1] + (A_(1, 2) * A_(2, 3) - A_(1, 3) * A_(2, 2)) * b[2]) / d;
    x[1] = ((A_(2, 3) * A_(3, 1) - A_(2, 1) * A_(3, 3)) * b[0] + (A_(1, 1) * A_(3, 3) - A_(1, 3) * A_(3, 1)) * b[1] + (A_(1, 3) * A_(2, 1) - A_(1, 1) * A_(2, 3)) * b[2]) / d;
    x[2] = ((A_(2, 1) * A_(3, 2) - A_(2, 2) * A_(3, 1)) * b[0] + (A_(1, 2) * A_(3, 1) - A_(1, 1) * A_(3, 2)) * b[1] + (A_(1, 1) * A_(2, 2) - A_(1, 2) * A_(2, 1)) * b[2]) / d;
    return;
  }
  /* partial pivoting LU, row-major working copy */
  float LU[MAXN][MAXN], y[MAXN];
  int piv[MAXN];
  for (int i = 0; i < N; i++) { piv[i] = i; for (int j = 0; j < N; j++) LU[i][j] = a[i + N * j]; }
  for (int kk = 0; kk < N; kk++) {
    int pr = kk; float best = fabsf(LU[kk][kk]);
    for (int i = kk + 1; i < N; i++) if (fabsf(LU[i][kk]) > best) { best = fabsf(LU[i][kk]); pr = i; }
    if (pr != kk) { for (int j = 0; j < N; j++) { float t = LU[kk][j]; LU[kk][j] = LU[pr][j]; LU[pr][j] = t; } int t = piv[kk]; piv[kk] = piv[pr]; piv[pr] = t; }
    for (int i = kk + 1; i < N; i++) {
      LU[i][kk] = LU[i][kk] / LU[kk][kk];
      for (int j = kk + 1; j < N; j++) LU[i][j] = LU[i][j] - LU[i][kk] * LU[kk][j];
    }
  }
  for (int i = 0; i < N; i++) { float s = b[piv[i]]; for (int j = 0; j < i; j++) s = s - LU[i][j] * y[j]; y[i] = s; }
  for (int i = N - 1; i >= 0; i--) { float s = y[i]; for (int j = i + 1; j < N; j++) s = s - LU[i][j] * x[j]; x[i] = s / LU[i][i]; }
}
#undef A_

/* ------------------------------------------------------------------ controller (integrator_utils.jl:1-11) */
struct Ctrl { float beta1, beta2, qmax, qmin, gamma, qoldinit; };
static Ctrl make_ctrl(int order) {
  Ctrl c;
  c.beta1 = (float)(7.0 / (10.0 * order));
  c.beta2 = (float)(2.0 / (5.0 * order));
  c.qmax = 10.0f; c.qmin = (float)(1.0 / 5.0); c.gamma = (float)(9.0 / 10.0); c.qoldinit = (float)1.0e-4;
  return c;
}
static int alg_order(int alg) {
  return alg == ALG_TSIT5 ? 5 : alg == ALG_VERN7 ? 7 : alg == ALG_RB23 ? 2 : alg == ALG_RODAS5P ? 5 : alg == ALG_RODAS4 ? 4 : alg == ALG_VERN9 ? 9 : alg == ALG_KVAERNO3 ? 3 : alg == ALG_KVAERNO5 ? 5 : 1;
}

/* PI controller decision, shared by every adaptive step! (e.g. gpu_tsit5_perform_step.jl:124-170).
 * Returns 1 if accepted; updates dt (reject) or dt_accepted/dtnew/qold (accept). */
template <class Tt>
static int controller(Integ<Tt>& ig, const Ctrl& C, float EEst, float& dt, Tt t) {
  float q11 = 0.0f, q;
  if (EEst == 0.0f) q = 1.0f / C.qmax;
  else { q11 = pm_powf(EEst, C.beta1); q = q11 / pm_powf(ig.qold, C.beta2); }
  if (EEst > 1.0f) {
    dt = dt / jl_min(1.0f / C.qmin, q11 / C.gamma);
    return 0;
  }
  q = jl_max(1.0f / C.qmax, jl_min(1.0f / C.qmin, q / C.gamma));
  ig.qold = jl_max(EEst, C.qoldinit);
  float dtnew = dt / q;
  float rem = t_rem(ig.tf, t, dt);
  ig.dtnew = jl_min(fabsf(dtnew), fabsf(rem));
  ig.dt = dt;
  ig.tprev = t;
  if (rem < 1.0e-14f) ig.t = ig.tf;
  else ig.t = t_add(t, dt);
  return 1;
}

/* error weights: tmp ./ (abstol .+ max.(abs.(uprev), abs.(u)) * reltol) */
static inline float scaled_norm(const float* e, const float* up, const float* u, int N, float abstol, float reltol) {
  float tmp[MAXN];
  for (int i = 0; i < N; i++) tmp[i] = e[i] / (abstol + jl_max(fabsf(up[i]), fabsf(u[i])) * reltol);
  return ode_norm(tmp, N);
}

/* ------------------------------------------------------------------ Vern9
 * gpu_vern9_perform_step.jl:1-319 (16 stages, k1 recomputed every attempt; the dense output
 * keeps k1, k8..k16) and nonstiff/interpolants.jl:192-371 (10 extra stages, bΘs by
 * Horner as Julia's evalpoly, evaluated without FMA). */
template <class Tt>
static void vern9_stages(int m, Integ<Tt>& ig, const float* p, Tt t, float dt, float* u, float (*k)[MAXN]) {
  int N = ig.N;
  float tmp[MAXN], k2[MAXN], k3[MAXN], k4[MAXN], k5[MAXN], k6[MAXN], k7[MAXN];
  const float* up = ig.uprev;
  model_f<float>(m, k[0], up, p, t_f32(t));
  float a = dt * F9C(a0201);
  for (int i = 0; i < N; i++) tmp[i] = up[i] + a * k[0][i];
  model_f<float>(m, k2, tmp, p, tstage(t, F9C(c1), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (F9C(a0301) * k[0][i] + F9C(a0302) * k2[i]);
  model_f<float>(m, k3, tmp, p, tstage(t, F9C(c2), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (F9C(a0401) * k[0][i] + F9C(a0403) * k3[i]);
  model_f<float>(m, k4, tmp, p, tstage(t, F9C(c3), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (F9C(a0501) * k[0][i] + F9C(a0503) * k3[i] + F9C(a0504) * k4[i]);
  model_f<float>(m, k5, tmp, p, tstage(t, F9C(c4), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (F9C(a0601) * k[0][i] + F9C(a0604) * k4[i] + F9C(a0605) * k5[i]);
  model_f<float>(m, k6, tmp, p, tstage(t, F9C(c5), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (F9C(a0701) * k[0][i] + F9C(a0704) * k4[i] + F9C(a0705) * k5[i] + F9C(a0706) * k6[i]);
  model_f<float>(m, k7, tmp, p, tstage(t, F9C(c6), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (F9C(a0801) * k[0][i] + F9C(a0806) * k6[i] + F9C(a0807) * k7[i]);
  model_f<float>(m, k[1], tmp, p, tstage(t, F9C(c7), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (F9C(a0901) * k[0][i] + F9C(a0906) * k6[i] + F9C(a0907) * k7[i] + F9C(a0908) * k[1][i]);
  model_f<float>(m, k[2], tmp, p, tstage(t, F9C(c8), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (F9C(a1001) * k[0][i] + F9C(a1006) * k6[i] + F9C(a1007) * k7[i] + F9C(a1008) * k[1][i] + F9C(a1009) * k[2][i]);
  model_f<float>(m, k[3], tmp, p, tstage(t, F9C(c9), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (F9C(a1101) * k[0][i] + F9C(a1106) * k6[i] + F9C(a1107) * k7[i] + F9C(a1108) * k[1][i] + F9C(a1109) * k[2][i] + F9C(a1110) * k[3][i]);
  model_f<float>(m, k[4], tmp, p, tstage(t, F9C(c10), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (F9C(a1201) * k[0][i] + F9C(a1206) * k6[i] + F9C(a1207) * k7[i] + F9C(a1208) * k[1][i] + F9C(a1209) * k[2][i] + F9C(a1210) * k[3][i] + F9C(a1211) * k[4][i]);
  model_f<float>(m, k[5], tmp, p, tstage(t, F9C(c11), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (F9C(a1301) * k[0][i] + F9C(a1306) * k6[i] + F9C(a1307) * k7[i] + F9C(a1308) * k[1][i] + F9C(a1309) * k[2][i] + F9C(a1310) * k[3][i] + F9C(a1311) * k[4][i] + F9C(a1312) * k[5][i]);
  model_f<float>(m, k[6], tmp, p, tstage(t, F9C(c12), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (F9C(a1401) * k[0][i] + F9C(a1406) * k6[i] + F9C(a1407) * k7[i] + F9C(a1408) * k[1][i] + F9C(a1409) * k[2][i] + F9C(a1410) * k[3][i] + F9C(a1411) * k[4][i] + F9C(a1412) * k[5][i] + F9C(a1413) * k[6][i]);
  model_f<float>(m, k[7], tmp, p, tstage(t, F9C(c13), dt));
  float g16[MAXN];
  for (int i = 0; i < N; i++) {
    tmp[i] = up[i] + dt * (F9C(a1501) * k[0][i] + F9C(a1506) * k6[i] + F9C(a1507) * k7[i] + F9C(a1508) * k[1][i] + F9C(a1509) * k[2][i] + F9C(a1510) * k[3][i] + F9C(a1511) * k[4][i] + F9C(a1512) * k[5][i] + F9C(a1513) * k[6][i] + F9C(a1514) * k[7][i]);
    g16[i] = up[i] + dt * (F9C(a1601) * k[0][i] + F9C(a1606) * k6[i] + F9C(a1607) * k7[i] + F9C(a1608) * k[1][i] + F9C(a1609) * k[2][i] + F9C(a1610) * k[3][i] + F9C(a1611) * k[4][i] + F9C(a1612) * k[5][i] + F9C(a1613) * k[6][i]);
  }
  model_f<float>(m, k[8], tmp, p, tstage(t, 1.0f, dt));
  model_f<float>(m, k[9], g16, p, tstage(t, 1.0f, dt));
  for (int i = 0; i < N; i++) u[i] = up[i] + dt * (F9C(b1) * k[0][i] + F9C(b8) * k[1][i] + F9C(b9) * k[2][i] + F9C(b10) * k[3][i] + F9C(b11) * k[4][i] + F9C(b12) * k[5][i] + F9C(b13) * k[6][i] + F9C(b14) * k[7][i] + F9C(b15) * k[8][i]);
}
// Julia's @evalpoly (Horner from the highest coefficient; no FMA in parity mode)
template <class Tt>
static void vern9_interp(int m, const Integ<Tt>& ig, const float* p, float th, float dt, float* out) {
  int N = ig.N;
  const float* up = ig.uprev;
  const float(*k)[MAXN] = ig.k;
  const Tt tp = ig.tprev;
  float tmp[MAXN], e17[MAXN], e18[MAXN], e19[MAXN], e20[MAXN], e21[MAXN], e22[MAXN], e23[MAXN], e24[MAXN], e25[MAXN], e26[MAXN];
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (F9XC(a1701) * k[0][i] + F9XC(a1708) * k[1][i] + F9XC(a1709) * k[2][i] + F9XC(a1710) * k[3][i] + F9XC(a1711) * k[4][i] + F9XC(a1712) * k[5][i] + F9XC(a1713) * k[6][i] + F9XC(a1714) * k[7][i] + F9XC(a1715) * k[8][i]);
  model_f<float>(m, e17, tmp, p, tstage(tp, F9XC(c17), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (F9XC(a1801) * k[0][i] + F9XC(a1808) * k[1][i] + F9XC(a1809) * k[2][i] + F9XC(a1810) * k[3][i] + F9XC(a1811) * k[4][i] + F9XC(a1812) * k[5][i] + F9XC(a1813) * k[6][i] + F9XC(a1814) * k[7][i] + F9XC(a1815) * k[8][i] + F9XC(a1817) * e17[i]);
  model_f<float>(m, e18, tmp, p, tstage(tp, F9XC(c18), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (F9XC(a1901) * k[0][i] + F9XC(a1908) * k[1][i] + F9XC(a1909) * k[2][i] + F9XC(a1910) * k[3][i] + F9XC(a1911) * k[4][i] + F9XC(a1912) * k[5][i] + F9XC(a1913) * k[6][i] + F9XC(a1914) * k[7][i] + F9XC(a1915) * k[8][i] + F9XC(a1917) * e17[i] + F9XC(a1918) * e18[i]);
  model_f<float>(m, e19, tmp, p, tstage(tp, F9XC(c19), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (F9XC(a2001) * k[0][i] + F9XC(a2008) * k[1][i] + F9XC(a2009) * k[2][i] + F9XC(a2010) * k[3][i] + F9XC(a2011) * k[4][i] + F9XC(a2012) * k[5][i] + F9XC(a2013) * k[6][i] + F9XC(a2014) * k[7][i] + F9XC(a2015) * k[8][i] + F9XC(a2017) * e17[i] + F9XC(a2018) * e18[i] + F9XC(a2019) * e19[i]);
  model_f<float>(m, e20, tmp, p, tstage(tp, F9XC(c20), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (F9XC(a2101) * k[0][i] + F9XC(a2108) * k[1][i] + F9XC(a2109) * k[2][i] + F9XC(a2110) * k[3][i] + F9XC(a2111) * k[4][i] + F9XC(a2112) * k[5][i] + F9XC(a2113) * k[6][i] + F9XC(a2114) * k[7][i] + F9XC(a2115) * k[8][i] + F9XC(a2117) * e17[i] + F9XC(a2118) * e18[i] + F9XC(a2119) * e19[i] + F9XC(a2120) * e20[i]);
  model_f<float>(m, e21, tmp, p, tstage(tp, F9XC(c21), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (F9XC(a2201) * k[0][i] + F9XC(a2208) * k[1][i] + F9XC(a2209) * k[2][i] + F9XC(a2210) * k[3][i] + F9XC(a2211) * k[4][i] + F9XC(a2212) * k[5][i] + F9XC(a2213) * k[6][i] + F9XC(a2214) * k[7][i] + F9XC(a2215) * k[8][i] + F9XC(a2217) * e17[i] + F9XC(a2218) * e18[i] + F9XC(a2219) * e19[i] + F9XC(a2220) * e20[i] + F9XC(a2221) * e21[i]);
  model_f<float>(m, e22, tmp, p, tstage(tp, F9XC(c22), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (F9XC(a2301) * k[0][i] + F9XC(a2308) * k[1][i] + F9XC(a2309) * k[2][i] + F9XC(a2310) * k[3][i] + F9XC(a2311) * k[4][i] + F9XC(a2312) * k[5][i] + F9XC(a2313) * k[6][i] + F9XC(a2314) * k[7][i] + F9XC(a2315) * k[8][i] + F9XC(a2317) * e17[i] + F9XC(a2318) * e18[i] + F9XC(a2319) * e19[i] + F9XC(a2320) * e20[i] + F9XC(a2321) * e21[i]);
  model_f<float>(m, e23, tmp, p, tstage(tp, F9XC(c23), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (F9XC(a2401) * k[0][i] + F9XC(a2408) * k[1][i] + F9XC(a2409) * k[2][i] + F9XC(a2410) * k[3][i] + F9XC(a2411) * k[4][i] + F9XC(a2412) * k[5][i] + F9XC(a2413) * k[6][i] + F9XC(a2414) * k[7][i] + F9XC(a2415) * k[8][i] + F9XC(a2417) * e17[i] + F9XC(a2418) * e18[i] + F9XC(a2419) * e19[i] + F9XC(a2420) * e20[i] + F9XC(a2421) * e21[i]);
  model_f<float>(m, e24, tmp, p, tstage(tp, F9XC(c24), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (F9XC(a2501) * k[0][i] + F9XC(a2508) * k[1][i] + F9XC(a2509) * k[2][i] + F9XC(a2510) * k[3][i] + F9XC(a2511) * k[4][i] + F9XC(a2512) * k[5][i] + F9XC(a2513) * k[6][i] + F9XC(a2514) * k[7][i] + F9XC(a2515) * k[8][i] + F9XC(a2517) * e17[i] + F9XC(a2518) * e18[i] + F9XC(a2519) * e19[i] + F9XC(a2520) * e20[i] + F9XC(a2521) * e21[i]);
  model_f<float>(m, e25, tmp, p, tstage(tp, F9XC(c25), dt));
  for (int i = 0; i < N; i++) tmp[i] = up[i] + dt * (F9XC(a2601) * k[0][i] + F9XC(a2608) * k[1][i] + F9XC(a2609) * k[2][i] + F9XC(a2610) * k[3][i] + F9XC(a2611) * k[4][i] + F9XC(a2612) * k[5][i] + F9XC(a2613) * k[6][i] + F9XC(a2614) * k[7][i] + F9XC(a2615) * k[8][i] + F9XC(a2617) * e17[i] + F9XC(a2618) * e18[i] + F9XC(a2619) * e19[i] + F9XC(a2620) * e20[i] + F9XC(a2621) * e21[i]);
  model_f<float>(m, e26, tmp, p, tstage(tp, F9XC(c26), dt));
  float b1 = F9IC(r019);
  b1 = th * b1 + F9IC(r018);
  b1 = th * b1 + F9IC(r017);
  b1 = th * b1 + F9IC(r016);
  b1 = th * b1 + F9IC(r015);
  b1 = th * b1 + F9IC(r014);
  b1 = th * b1 + F9IC(r013);
  b1 = th * b1 + F9IC(r012);
  b1 = th * b1 + F9IC(r011);
  b1 = th * b1 + 0.0f;
  float b8 = F9IC(r089);
  b8 = th * b8 + F9IC(r088);
  b8 = th * b8 + F9IC(r087);
  b8 = th * b8 + F9IC(r086);
  b8 = th * b8 + F9IC(r085);
  b8 = th * b8 + F9IC(r084);
  b8 = th * b8 + F9IC(r083);
  b8 = th * b8 + F9IC(r082);
  b8 = th * b8 + 0.0f;
  b8 = th * b8 + 0.0f;
  float b9 = F9IC(r099);
  b9 = th * b9 + F9IC(r098);
  b9 = th * b9 + F9IC(r097);
  b9 = th * b9 + F9IC(r096);
  b9 = th * b9 + F9IC(r095);
  b9 = th * b9 + F9IC(r094);
  b9 = th * b9 + F9IC(r093);
  b9 = th * b9 + F9IC(r092);
  b9 = th * b9 + 0.0f;
  b9 = th * b9 + 0.0f;
  float b10 = F9IC(r109);
  b10 = th * b10 + F9IC(r108);
  b10 = th * b10 + F9IC(r107);
  b10 = th * b10 + F9IC(r106);
  b10 = th * b10 + F9IC(r105);
  b10 = th * b10 + F9IC(r104);
  b10 = th * b10 + F9IC(r103);
  b10 = th * b10 + F9IC(r102);
  b10 = th * b10 + 0.0f;
  b10 = th * b10 + 0.0f;
  float b11 = F9IC(r119);
  b11 = th * b11 + F9IC(r118);
  b11 = th * b11 + F9IC(r117);
  b11 = th * b11 + F9IC(r116);
  b11 = th * b11 + F9IC(r115);
  b11 = th * b11 + F9IC(r114);
  b11 = th * b11 + F9IC(r113);
  b11 = th * b11 + F9IC(r112);
  b11 = th * b11 + 0.0f;
  b11 = th * b11 + 0.0f;
  float b12 = F9IC(r129);
  b12 = th * b12 + F9IC(r128);
  b12 = th * b12 + F9IC(r127);
  b12 = th * b12 + F9IC(r126);
  b12 = th * b12 + F9IC(r125);
  b12 = th * b12 + F9IC(r124);
  b12 = th * b12 + F9IC(r123);
  b12 = th * b12 + F9IC(r122);
  b12 = th * b12 + 0.0f;
  b12 = th * b12 + 0.0f;
  float b13 = F9IC(r139);
  b13 = th * b13 + F9IC(r138);
  b13 = th * b13 + F9IC(r137);
  b13 = th * b13 + F9IC(r136);
  b13 = th * b13 + F9IC(r135);
  b13 = th * b13 + F9IC(r134);
  b13 = th * b13 + F9IC(r133);
  b13 = th * b13 + F9IC(r132);
  b13 = th * b13 + 0.0f;
  b13 = th * b13 + 0.0f;
  float b14 = F9IC(r149);
  b14 = th * b14 + F9IC(r148);
  b14 = th * b14 + F9IC(r147);
  b14 = th * b14 + F9IC(r146);
  b14 = th * b14 + F9IC(r145);
  b14 = th * b14 + F9IC(r144);
  b14 = th * b14 + F9IC(r143);
  b14 = th * b14 + F9IC(r142);
  b14 = th * b14 + 0.0f;
  b14 = th * b14 + 0.0f;
  float b15 = F9IC(r159);
  b15 = th * b15 + F9IC(r158);
  b15 = th * b15 + F9IC(r157);
  b15 = th * b15 + F9IC(r156);
  b15 = th * b15 + F9IC(r155);
  b15 = th * b15 + F9IC(r154);
  b15 = th * b15 + F9IC(r153);
  b15 = th * b15 + F9IC(r152);
  b15 = th * b15 + 0.0f;
  b15 = th * b15 + 0.0f;
  float b17 = F9IC(r179);
  b17 = th * b17 + F9IC(r178);
  b17 = th * b17 + F9IC(r177);
  b17 = th * b17 + F9IC(r176);
  b17 = th * b17 + F9IC(r175);
  b17 = th * b17 + F9IC(r174);
  b17 = th * b17 + F9IC(r173);
  b17 = th * b17 + F9IC(r172);
  b17 = th * b17 + 0.0f;
  b17 = th * b17 + 0.0f;
  float b18 = F9IC(r189);
  b18 = th * b18 + F9IC(r188);
  b18 = th * b18 + F9IC(r187);
  b18 = th * b18 + F9IC(r186);
  b18 = th * b18 + F9IC(r185);
  b18 = th * b18 + F9IC(r184);
  b18 = th * b18 + F9IC(r183);
  b18 = th * b18 + F9IC(r182);
  b18 = th * b18 + 0.0f;
  b18 = th * b18 + 0.0f;
  float b19 = F9IC(r199);
  b19 = th * b19 + F9IC(r198);
  b19 = th * b19 + F9IC(r197);
  b19 = th * b19 + F9IC(r196);
  b19 = th * b19 + F9IC(r195);
  b19 = th * b19 + F9IC(r194);
  b19 = th * b19 + F9IC(r193);
  b19 = th * b19 + F9IC(r192);
  b19 = th * b19 + 0.0f;
  b19 = th * b19 + 0.0f;
  float b20 = F9IC(r209);
  b20 = th * b20 + F9IC(r208);
  b20 = th * b20 + F9IC(r207);
  b20 = th * b20 + F9IC(r206);
  b20 = th * b20 + F9IC(r205);
  b20 = th * b20 + F9IC(r204);
  b20 = th * b20 + F9IC(r203);
  b20 = th * b20 + F9IC(r202);
  b20 = th * b20 + 0.0f;
  b20 = th * b20 + 0.0f;
  float b21 = F9IC(r219);
  b21 = th * b21 + F9IC(r218);
  b21 = th * b21 + F9IC(r217);
  b21 = th * b21 + F9IC(r216);
  b21 = th * b21 + F9IC(r215);
  b21 = th * b21 + F9IC(r214);
  b21 = th * b21 + F9IC(r213);
  b21 = th * b21 + F9IC(r212);
  b21 = th * b21 + 0.0f;
  b21 = th * b21 + 0.0f;
  float b22 = F9IC(r229);
  b22 = th * b22 + F9IC(r228);
  b22 = th * b22 + F9IC(r227);
  b22 = th * b22 + F9IC(r226);
  b22 = th * b22 + F9IC(r225);
  b22 = th * b22 + F9IC(r224);
  b22 = th * b22 + F9IC(r223);
  b22 = th * b22 + F9IC(r222);
  b22 = th * b22 + 0.0f;
  b22 = th * b22 + 0.0f;
  float b23 = F9IC(r239);
  b23 = th * b23 + F9IC(r238);
  b23 = th * b23 + F9IC(r237);
  b23 = th * b23 + F9IC(r236);
  b23 = th * b23 + F9IC(r235);
  b23 = th * b23 + F9IC(r234);
  b23 = th * b23 + F9IC(r233);
  b23 = th * b23 + F9IC(r232);
  b23 = th * b23 + 0.0f;
  b23 = th * b23 + 0.0f;
  float b24 = F9IC(r249);
  b24 = th * b24 + F9IC(r248);
  b24 = th * b24 + F9IC(r247);
  b24 = th * b24 + F9IC(r246);
  b24 = th * b24 + F9IC(r245);
  b24 = th * b24 + F9IC(r244);
  b24 = th * b24 + F9IC(r243);
  b24 = th * b24 + F9IC(r242);
  b24 = th * b24 + 0.0f;
  b24 = th * b24 + 0.0f;
  float b25 = F9IC(r259);
  b25 = th * b25 + F9IC(r258);
  b25 = th * b25 + F9IC(r257);
  b25 = th * b25 + F9IC(r256);
  b25 = th * b25 + F9IC(r255);
  b25 = th * b25 + F9IC(r254);
  b25 = th * b25 + F9IC(r253);
  b25 = th * b25 + F9IC(r252);
  b25 = th * b25 + 0.0f;
  b25 = th * b25 + 0.0f;
  float b26 = F9IC(r269);
  b26 = th * b26 + F9IC(r268);
  b26 = th * b26 + F9IC(r267);
  b26 = th * b26 + F9IC(r266);
  b26 = th * b26 + F9IC(r265);
  b26 = th * b26 + F9IC(r264);
  b26 = th * b26 + F9IC(r263);
  b26 = th * b26 + F9IC(r262);
  b26 = th * b26 + 0.0f;
  b26 = th * b26 + 0.0f;
  for (int i = 0; i < N; i++) out[i] = up[i] + dt * (k[0][i] * b1 + k[1][i] * b8 + k[2][i] * b9 + k[3][i] * b10 + k[4][i] * b11 + k[5][i] * b12 + k[6][i] * b13 + k[7][i] * b14 + k[8][i] * b15 + e17[i] * b17 + e18[i] * b18 + e19[i] * b19 + e20[i] * b20 + e21[i] * b21 + e22[i] * b22 + e23[i] * b23 + e24[i] * b24 + e25[i] * b25 + e26[i] * b26);
}

/* ------------------------------------------------------------------ Rosenbrock23 */
template <class Tt>
static void rb23_attempt(int m, int jacmode, Integ<Tt>& ig, const float* p, Tt t, float dt, float* u, float* k1o, float* k2o, float* err, int adaptive) {
  int N = ig.N;
  const float d = 1.0f / (2.0f + sqrtf(2.0f));
  float J[MAXN * MAXN], dT[MAXN], W[MAXN * MAXN], F0[MAXN], F1[MAXN], F2[MAXN], rhs[MAXN], tmp[MAXN], k1[MAXN], k2[MAXN], k3[MAXN];
  float tf_ = t_f32(t);
  float gam = dt * d, dto2 = dt / 2.0f, dto6 = dt / 6.0f;
  compute_J(m, jacmode, N, J, ig.uprev, p, tf_);
  compute_tgrad(m, jacmode, N, dT, ig.uprev, p, tf_);
  float Mm[MAXN * MAXN];
  const int has_mass = model_mass(m, Mm);
  for (int j = 0; j < N; j++)
    for (int i = 0; i < N; i++) W[i + N * j] = (has_mass ? Mm[i + N * j] : (i == j ? 1.0f : 0.0f)) - gam * J[i + N * j];
  model_f<float>(m, F0, ig.uprev, p, tf_);
  for (int i = 0; i < N; i++) rhs[i] = F0[i] + gam * dT[i];
  linear_solve(N, W, rhs, k1);
  for (int i = 0; i < N; i++) tmp[i] = ig.uprev[i] + dto2 * k1[i];
  model_f<float>(m, F1, tmp, p, t_stage(t, 1.0f, dto2));
  if (has_mass) { float mk[MAXN]; mass_mul(N, Mm, k1, mk); for (int i = 0; i < N; i++) rhs[i] = F1[i] - mk[i]; }
  else for (int i = 0; i < N; i++) rhs[i] = F1[i] - k1[i];
  linear_solve(N, W, rhs, k2);
  for (int i = 0; i < N; i++) k2[i] = k2[i] + k1[i];
  for (int i = 0; i < N; i++) u[i] = ig.uprev[i] + dt * k2[i];
  for (int i = 0; i < N; i++) { k1o[i] = k1[i]; k2o[i] = k2[i]; }
  if (!adaptive) return;
  const float e32 = 6.0f + sqrtf(2.0f);
  model_f<float>(m, F2, u, p, t_stage(t, 1.0f, dt));
  if (has_mass) {
    float cv[MAXN], mv[MAXN];
    for (int i = 0; i < N; i++) cv[i] = e32 * k2[i] + 2.0f * k1[i];
    mass_mul(N, Mm, cv, mv);
    for (int i = 0; i < N; i++) rhs[i] = F2[i] - mv[i] + e32 * F1[i] + 2.0f * F0[i] + dt * dT[i];
  } else {
    for (int i = 0; i < N; i++) rhs[i] = F2[i] - e32 * (k2[i] - F1[i]) - 2.0f * (k1[i] - F0[i]) + dt * dT[i];
  }
  linear_solve(N, W, rhs, k3);
  for (int i = 0; i < N; i++) err[i] = dto6 * (k1[i] - 2.0f * k2[i] + k3[i]);
}

/* linsolve_tmp = base + mass_matrix * (combination) of the Rodas stages */
#define MASS_LT_O(LT, BASE, COMBO)                                             \
  {                                                                            \
    if (has_mass) {                                                            \
      float cv_[MAXN], mv_[MAXN];                                              \
      for (int i = 0; i < N; i++) cv_[i] = (COMBO);                            \
      mass_mul(N, Mm, cv_, mv_);                                               \
      for (int i = 0; i < N; i++) LT[i] = (BASE) + mv_[i];                     \
    } else {                                                                   \
      for (int i = 0; i < N; i++) LT[i] = (BASE) + (COMBO);                    \
    }                                                                          \
  }

/* ------------------------------------------------------------------ Rodas5P */
template <class Tt>
static void rodas5p_attempt(int m, Integ<Tt>& ig, const float* p, Tt t, float dt, float* uout, float* k8o, float (*dense)[MAXN]) {
  int N = ig.N;
  const float* J = ig.J; const float* dT = ig.dT; const float* up = ig.uprev;
  float dtC21 = RPC(C21) / dt, dtC31 = RPC(C31) / dt, dtC32 = RPC(C32) / dt, dtC41 = RPC(C41) / dt, dtC42 = RPC(C42) / dt, dtC43 = RPC(C43) / dt;
  float dtC51 = RPC(C51) / dt, dtC52 = RPC(C52) / dt, dtC53 = RPC(C53) / dt, dtC54 = RPC(C54) / dt;
  float dtC61 = RPC(C61) / dt, dtC62 = RPC(C62) / dt, dtC63 = RPC(C63) / dt, dtC64 = RPC(C64) / dt, dtC65 = RPC(C65) / dt;
  float dtC71 = RPC(C71) / dt, dtC72 = RPC(C72) / dt, dtC73 = RPC(C73) / dt, dtC74 = RPC(C74) / dt, dtC75 = RPC(C75) / dt, dtC76 = RPC(C76) / dt;
  float dtC81 = RPC(C81) / dt, dtC82 = RPC(C82) / dt, dtC83 = RPC(C83) / dt, dtC84 = RPC(C84) / dt, dtC85 = RPC(C85) / dt, dtC86 = RPC(C86) / dt, dtC87 = RPC(C87) / dt;
  float dtd1 = dt * RPC(d1), dtd2 = dt * RPC(d2), dtd3 = dt * RPC(d3), dtd4 = dt * RPC(d4), dtd5 = dt * RPC(d5);
  float dtgamma = dt * RPC(gamma);
  float W[MAXN * MAXN];
  float inv_dtg = 1.0f / dtgamma;
  float Mm[MAXN * MAXN];
  const int has_mass = model_mass(m, Mm);
  for (int j = 0; j < N; j++)
    for (int i = 0; i < N; i++) W[i + N * j] = J[i + N * j] - (has_mass ? Mm[i + N * j] : (i == j ? 1.0f : 0.0f)) * inv_dtg;
  float du[MAXN], u[MAXN], lt[MAXN], neg[MAXN];
  float k1[MAXN], k2[MAXN], k3[MAXN], k4[MAXN], k5[MAXN], k6[MAXN], k7[MAXN], k8[MAXN];
  float tf_ = t_f32(t);
#define SOLVE(K) { for (int i = 0; i < N; i++) neg[i] = -lt[i]; linear_solve(N, W, neg, K); }
  model_f<float>(m, du, up, p, tf_);
  for (int i = 0; i < N; i++) lt[i] = du[i] + dtd1 * dT[i];
  SOLVE(k1);
  for (int i = 0; i < N; i++) u[i] = up[i] + RPC(a21) * k1[i];
  model_f<float>(m, du, u, p, tstage(t, RPC(c2), dt));
  MASS_LT_O(lt, du[i] + dtd2 * dT[i], dtC21 * k1[i]);
  SOLVE(k2);
  for (int i = 0; i < N; i++) u[i] = up[i] + RPC(a31) * k1[i] + RPC(a32) * k2[i];
  model_f<float>(m, du, u, p, tstage(t, RPC(c3), dt));
  MASS_LT_O(lt, du[i] + dtd3 * dT[i], (dtC31 * k1[i] + dtC32 * k2[i]));
  SOLVE(k3);
  for (int i = 0; i < N; i++) u[i] = up[i] + RPC(a41) * k1[i] + RPC(a42) * k2[i] + RPC(a43) * k3[i];
  model_f<float>(m, du, u, p, tstage(t, RPC(c4), dt));
  MASS_LT_O(lt, du[i] + dtd4 * dT[i], (dtC41 * k1[i] + dtC42 * k2[i] + dtC43 * k3[i]));
  SOLVE(k4);
  for (int i = 0; i < N; i++) u[i] = up[i] + RPC(a51) * k1[i] + RPC(a52) * k2[i] + RPC(a53) * k3[i] + RPC(a54) * k4[i];
  model_f<float>(m, du, u, p, tstage(t, RPC(c5), dt));
  MASS_LT_O(lt, du[i] + dtd5 * dT[i], (dtC52 * k2[i] + dtC54 * k4[i] + dtC51 * k1[i] + dtC53 * k3[i]));
  SOLVE(k5);
  for (int i = 0; i < N; i++) u[i] = up[i] + RPC(a61) * k1[i] + RPC(a62) * k2[i] + RPC(a63) * k3[i] + RPC(a64) * k4[i] + RPC(a65) * k5[i];
  model_f<float>(m, du, u, p, t_stage(t, 1.0f, dt));
  MASS_LT_O(lt, du[i], (dtC61 * k1[i] + dtC62 * k2[i] + dtC63 * k3[i] + dtC64 * k4[i] + dtC65 * k5[i]));
  SOLVE(k6);
  for (int i = 0; i < N; i++) u[i] = u[i] + k6[i];
  model_f<float>(m, du, u, p, t_stage(t, 1.0f, dt));
  MASS_LT_O(lt, du[i], (dtC71 * k1[i] + dtC72 * k2[i] + dtC73 * k3[i] + dtC74 * k4[i] + dtC75 * k5[i] + dtC76 * k6[i]));
  SOLVE(k7);
  for (int i = 0; i < N; i++) u[i] = u[i] + k7[i];
  model_f<float>(m, du, u, p, t_stage(t, 1.0f, dt));
  MASS_LT_O(lt, du[i], (dtC81 * k1[i] + dtC82 * k2[i] + dtC83 * k3[i] + dtC84 * k4[i] + dtC85 * k5[i] + dtC86 * k6[i] + dtC87 * k7[i]));
  SOLVE(k8);
#undef SOLVE
  for (int i = 0; i < N; i++) { uout[i] = u[i] + k8[i]; k8o[i] = k8[i]; }
  for (int i = 0; i < N; i++) {
    dense[0][i] = RPC(h21) * k1[i] + RPC(h22) * k2[i] + RPC(h23) * k3[i] + RPC(h24) * k4[i] + RPC(h25) * k5[i] + RPC(h26) * k6[i] + RPC(h27) * k7[i] + RPC(h28) * k8[i];
    dense[1][i] = RPC(h31) * k1[i] + RPC(h32) * k2[i] + RPC(h33) * k3[i] + RPC(h34) * k4[i] + RPC(h35) * k5[i] + RPC(h36) * k6[i] + RPC(h37) * k7[i] + RPC(h38) * k8[i];
    dense[2][i] = RPC(h41) * k1[i] + RPC(h42) * k2[i] + RPC(h43) * k3[i] + RPC(h44) * k4[i] + RPC(h45) * k5[i] + RPC(h46) * k6[i] + RPC(h47) * k7[i] + RPC(h48) * k8[i];
  }
}

/* ------------------------------------------------------------------ Rodas4
 * gpu_rodas4_perform_step.jl:1-114 (fixed) / :116-277 (adaptive): 6 stages, error estimate
 * k6, two dense-output vectors; J and dT once per step (:36-40, :145-149). */
template <class Tt>
static void rodas4_attempt(int m, Integ<Tt>& ig, const float* p, Tt t, float dt, float* uout, float* k6o, float (*dense)[MAXN]) {
  int N = ig.N;
  const float* J = ig.J; const float* dT = ig.dT; const float* up = ig.uprev;
  float dtC21 = R4C(C21) / dt, dtC31 = R4C(C31) / dt, dtC32 = R4C(C32) / dt, dtC41 = R4C(C41) / dt, dtC42 = R4C(C42) / dt, dtC43 = R4C(C43) / dt;
  float dtC51 = R4C(C51) / dt, dtC52 = R4C(C52) / dt, dtC53 = R4C(C53) / dt, dtC54 = R4C(C54) / dt;
  float dtC61 = R4C(C61) / dt, dtC62 = R4C(C62) / dt, dtC63 = R4C(C63) / dt, dtC64 = R4C(C64) / dt, dtC65 = R4C(C65) / dt;
  float dtd1 = dt * R4C(d1), dtd2 = dt * R4C(d2), dtd3 = dt * R4C(d3), dtd4 = dt * R4C(d4);
  float dtgamma = dt * R4C(gamma);
  float W[MAXN * MAXN];
  float inv_dtg = 1.0f / dtgamma;
  float Mm[MAXN * MAXN];
  const int has_mass = model_mass(m, Mm);
  for (int j = 0; j < N; j++)
    for (int i = 0; i < N; i++) W[i + N * j] = J[i + N * j] - (has_mass ? Mm[i + N * j] : (i == j ? 1.0f : 0.0f)) * inv_dtg;
  float du[MAXN], u[MAXN], lt[MAXN], neg[MAXN];
  float k1[MAXN], k2[MAXN], k3[MAXN], k4[MAXN], k5[MAXN], k6[MAXN];
  float tf_ = t_f32(t);
#define SOLVE(K) { for (int i = 0; i < N; i++) neg[i] = -lt[i]; linear_solve(N, W, neg, K); }
  model_f<float>(m, du, up, p, tf_);
  for (int i = 0; i < N; i++) lt[i] = du[i] + dtd1 * dT[i];
  SOLVE(k1);
  for (int i = 0; i < N; i++) u[i] = up[i] + R4C(a21) * k1[i];
  model_f<float>(m, du, u, p, tstage(t, R4C(c2), dt));
  MASS_LT_O(lt, du[i] + dtd2 * dT[i], dtC21 * k1[i]);
  SOLVE(k2);
  for (int i = 0; i < N; i++) u[i] = up[i] + R4C(a31) * k1[i] + R4C(a32) * k2[i];
  model_f<float>(m, du, u, p, tstage(t, R4C(c3), dt));
  MASS_LT_O(lt, du[i] + dtd3 * dT[i], (dtC31 * k1[i] + dtC32 * k2[i]));
  SOLVE(k3);
  for (int i = 0; i < N; i++) u[i] = up[i] + R4C(a41) * k1[i] + R4C(a42) * k2[i] + R4C(a43) * k3[i];
  model_f<float>(m, du, u, p, tstage(t, R4C(c4), dt));
  MASS_LT_O(lt, du[i] + dtd4 * dT[i], (dtC41 * k1[i] + dtC42 * k2[i] + dtC43 * k3[i]));
  SOLVE(k4);
  for (int i = 0; i < N; i++) u[i] = up[i] + R4C(a51) * k1[i] + R4C(a52) * k2[i] + R4C(a53) * k3[i] + R4C(a54) * k4[i];
  model_f<float>(m, du, u, p, t_stage(t, 1.0f, dt));
  MASS_LT_O(lt, du[i], (dtC52 * k2[i] + dtC54 * k4[i] + dtC51 * k1[i] + dtC53 * k3[i]));
  SOLVE(k5);
  for (int i = 0; i < N; i++) u[i] = u[i] + k5[i];
  model_f<float>(m, du, u, p, t_stage(t, 1.0f, dt));
  MASS_LT_O(lt, du[i], (dtC61 * k1[i] + dtC62 * k2[i] + dtC65 * k5[i] + dtC64 * k4[i] + dtC63 * k3[i]));
  SOLVE(k6);
#undef SOLVE
  for (int i = 0; i < N; i++) { uout[i] = u[i] + k6[i]; k6o[i] = k6[i]; }
  for (int i = 0; i < N; i++) {
    dense[0][i] = R4C(h21) * k1[i] + R4C(h22) * k2[i] + R4C(h23) * k3[i] + R4C(h24) * k4[i] + R4C(h25) * k5[i];
    dense[1][i] = R4C(h31) * k1[i] + R4C(h32) * k2[i] + R4C(h33) * k3[i] + R4C(h34) * k4[i] + R4C(h35) * k5[i];
  }
}

/* ------------------------------------------------------------------ Kvaerno3 / Kvaerno5
 * gpu_kvaerno3_perform_step.jl, gpu_kvaerno5_perform_step.jl with nlsolve (nlsolve/utils.jl:1-26)
 * and W = -I + (γ dt) J from build_J_W (nlsolve/type.jl:129-140). */
static void sdirk_w(int N, const float* J, float gdt, float* W) {
  for (int j = 0; j < N; j++)
    for (int i = 0; i < N; i++) W[i + N * j] = (i == j) ? gdt * J[i + N * j] + -1.0f : gdt * J[i + N * j];
}
template <class Tt>
static void nlsolve_o(int m, int jacmode, int N, const float* p, float* z, const float* tmp, float gam, float c, Tt tn, float dtn) {
  const float tc = t_stage(tn, c, dtn);
  const float gdt = gam * dtn;
  float x[MAXN], fx[MAXN], J[MAXN * MAXN], W[MAXN * MAXN], r[MAXN], dz[MAXN];
  for (int i = 0; i < N; i++) x[i] = tmp[i] + gam * z[i];
  model_f<float>(m, fx, x, p, tc);
  for (int it = 0; it < 30; it++) {
    compute_J(m, jacmode, N, J, x, p, tc);
    sdirk_w(N, J, gdt, W);
    for (int i = 0; i < N; i++) r[i] = dtn * fx[i] - z[i];
    linear_solve(N, W, r, dz);
    for (int i = 0; i < N; i++) { z[i] = z[i] - dz[i]; x[i] = tmp[i] + gam * z[i]; }
    model_f<float>(m, fx, x, p, tc);
    for (int i = 0; i < N; i++) r[i] = dtn * fx[i] - z[i];
    if (ode_norm(r, N) < 1.1920928955078125e-05f) break; /* diffeqgpunorm < 100 eps(Float32) */
  }
}
/* One attempt.  k1: the step's k1; tn/dtn: the nonlinear solver's time and step (the
 * attempt's when adaptive; integ.t after the advance and integ.dt for fixed steps).
 * Writes u, k2 = z_last / dt and, when adaptive, err. */
template <class Tt>
static void kvaerno_attempt(int m, int jacmode, int alg, Integ<Tt>& ig, const float* p, Tt t, float dt, Tt tn, float dtn,
                            const float* k1, float* u, float* k2, float* err, int adaptive) {
  const int N = ig.N;
  const float* up = ig.uprev;
  float tmp[MAXN], z1[MAXN], z2[MAXN], z3[MAXN], z4[MAXN], z5[MAXN], z6[MAXN], z7[MAXN], e[MAXN], zl[MAXN];
  float g;
  for (int i = 0; i < N; i++) z1[i] = dt * k1[i];
  if (alg == ALG_KVAERNO3) {
    g = K3C(gamma);
    for (int i = 0; i < N; i++) { z2[i] = z1[i]; tmp[i] = up[i] + g * z1[i]; }
    nlsolve_o(m, jacmode, N, p, z2, tmp, g, g, tn, dtn);
    for (int i = 0; i < N; i++) { z3[i] = K3C(alpha31) * z1[i] + K3C(alpha32) * z2[i]; tmp[i] = up[i] + K3C(a31) * z1[i] + K3C(a32) * z2[i]; }
    nlsolve_o(m, jacmode, N, p, z3, tmp, g, K3C(c3), tn, dtn);
    for (int i = 0; i < N; i++) {
      z4[i] = K3C(a31) * z1[i] + K3C(a32) * z2[i] + g * z3[i];
      tmp[i] = up[i] + K3C(a41) * z1[i] + K3C(a42) * z2[i] + K3C(a43) * z3[i];
    }
    nlsolve_o(m, jacmode, N, p, z4, tmp, g, 1.0f, tn, dtn);
    for (int i = 0; i < N; i++) {
      zl[i] = z4[i];
      e[i] = K3C(btilde1) * z1[i] + K3C(btilde2) * z2[i] + K3C(btilde3) * z3[i] + K3C(btilde4) * z4[i];
    }
  } else {
    g = K5C(gamma);
    for (int i = 0; i < N; i++) { z2[i] = z1[i]; tmp[i] = up[i] + g * z1[i]; }
    nlsolve_o(m, jacmode, N, p, z2, tmp, g, g, tn, dtn);
    for (int i = 0; i < N; i++) { z3[i] = K5C(alpha31) * z1[i] + K5C(alpha32) * z2[i]; tmp[i] = up[i] + K5C(a31) * z1[i] + K5C(a32) * z2[i]; }
    nlsolve_o(m, jacmode, N, p, z3, tmp, g, K5C(c3), tn, dtn);
    for (int i = 0; i < N; i++) {
      z4[i] = K5C(alpha41) * z1[i] + K5C(alpha42) * z2[i] + K5C(alpha43) * z3[i];
      tmp[i] = up[i] + K5C(a41) * z1[i] + K5C(a42) * z2[i] + K5C(a43) * z3[i];
    }
    nlsolve_o(m, jacmode, N, p, z4, tmp, g, K5C(c4), tn, dtn);
    for (int i = 0; i < N; i++) {
      z5[i] = K5C(alpha51) * z1[i] + K5C(alpha52) * z2[i] + K5C(alpha53) * z3[i];
      tmp[i] = up[i] + K5C(a51) * z1[i] + K5C(a52) * z2[i] + K5C(a53) * z3[i] + K5C(a54) * z4[i];
    }
    nlsolve_o(m, jacmode, N, p, z5, tmp, g, K5C(c5), tn, dtn);
    for (int i = 0; i < N; i++) {
      z6[i] = K5C(alpha61) * z1[i] + K5C(alpha62) * z2[i] + K5C(alpha63) * z3[i];
      tmp[i] = up[i] + K5C(a61) * z1[i] + K5C(a63) * z3[i] + K5C(a64) * z4[i] + K5C(a65) * z5[i];
    }
    nlsolve_o(m, jacmode, N, p, z6, tmp, g, K5C(c6), tn, dtn);
    for (int i = 0; i < N; i++) {
      z7[i] = K5C(a61) * z1[i] + K5C(a63) * z3[i] + K5C(a64) * z4[i] + K5C(a65) * z5[i] + g * z6[i];
      tmp[i] = up[i] + K5C(a71) * z1[i] + K5C(a73) * z3[i] + K5C(a74) * z4[i] + K5C(a75) * z5[i] + K5C(a76) * z6[i];
    }
    nlsolve_o(m, jacmode, N, p, z7, tmp, g, 1.0f, tn, dtn);
    for (int i = 0; i < N; i++) {
      zl[i] = z7[i];
      e[i] = K5C(btilde1) * z1[i] + K5C(btilde3) * z3[i] + K5C(btilde4) * z4[i] + K5C(btilde5) * z5[i] + K5C(btilde6) * z6[i] + K5C(btilde7) * z7[i];
    }
  }
  for (int i = 0; i < N; i++) { u[i] = tmp[i] + g * zl[i]; k2[i] = zl[i] / dt; }
  if (adaptive) {
    float J[MAXN * MAXN], W[MAXN * MAXN];
    compute_J(m, jacmode, N, J, u, p, t_stage(t, 1.0f, dt));
    sdirk_w(N, J, g * dt, W);
    linear_solve(N, W, e, err);
  }
}

/* default Hermite interpolation (nonstiff/interpolants.jl:1-21) */
template <class Tt>
static void hermite_interp(const Integ<Tt>& ig, float th, float dt, float* out) {
  const float a = 1.0f - th, b = th * (th - 1.0f), c = 1.0f - 2.0f * th, d = (th - 1.0f) * dt, e = th * dt;
  for (int i = 0; i < ig.N; i++)
    out[i] = (a * ig.uprev[i] + th * ig.u[i]) + b * ((c * (ig.u[i] - ig.uprev[i]) + d * ig.k[0][i]) + e * ig.k[1][i]);
}

/* ------------------------------------------------------------------ interpolation (savevalues!) */
template <class Tt>
static void interpolate(int m, int alg, const Integ<Tt>& ig, const float* p, float th, float dt, float* out) {
  int N = ig.N;
  const float* y0 = ig.uprev;
  switch (alg) {
    case ALG_TSIT5: { /* nonstiff/interpolants.jl:372-387 */
      float b[7];
      tsit5_btheta(th, b);
      for (int i = 0; i < N; i++)
        out[i] = y0[i] + dt * (b[0] * ig.k[0][i] + b[1] * ig.k[1][i] + b[2] * ig.k[2][i] + b[3] * ig.k[3][i] + b[4] * ig.k[4][i] + b[5] * ig.k[5][i] + b[6] * ig.k[6][i]);
    } break;
    case ALG_VERN7: vern7_interp(m, ig, p, th, dt, out); break;
    case ALG_VERN9: vern9_interp(m, ig, p, th, dt, out); break;
    case ALG_KVAERNO3:
    case ALG_KVAERNO5: hermite_interp(ig, th, dt, out); break;
    case ALG_RB23: { /* nonstiff/interpolants.jl:389-399 */
      const float d = 1.0f / (2.0f + sqrtf(2.0f));
      float c1 = th * (1.0f - th) / (1.0f - 2.0f * d);
      float c2 = th * (th - 2.0f * d) / (1.0f - 2.0f * d);
      for (int i = 0; i < N; i++) out[i] = y0[i] + dt * (c1 * ig.k[0][i] + c2 * ig.k[1][i]);
    } break;
    case ALG_RODAS4: { /* stiff/interpolants.jl:1-11 */
      float th1 = 1.0f - th;
      for (int i = 0; i < N; i++) out[i] = th1 * y0[i] + th * (ig.u[i] + th1 * (ig.k[0][i] + th * ig.k[1][i]));
    } break;
    case ALG_RODAS5P: { /* stiff/interpolants.jl:13-23 */
      float th1 = 1.0f - th;
      for (int i = 0; i < N; i++) out[i] = th1 * y0[i] + th * (ig.u[i] + th1 * (ig.k[0][i] + th * (ig.k[1][i] + th * ig.k[2][i])));
    } break;
  }
}

/* ------------------------------------------------------------------ callbacks (integrator_utils.jl:52-479)
 * Julia's sign / eps / nextfloat / max on Float32, the ITP root finder, event location and
 * application.  Event times: with a Float32 tspan absolute Float32 times (the reference's
 * arithmetic); with an FP64 tspan float offsets x from tprev, the event at tprev + x in the
 * pair time (the kernels do the same: the FP32 interpolant resolves no finer). */
static inline float jl_sign(float x) { return (x == 0.0f || x != x) ? x : copysignf(1.0f, x); }
static inline float o_max(float x, float y) { if (x != x) return x; if (y != y) return y; return y > x ? y : x; }
static inline float o_eps(float x) { /* ldexp(eps(Float32), exponent(x)); nextfloat(0) below floatmin */
  uint32_t b; memcpy(&b, &x, 4);
  uint32_t e = (b >> 23) & 0xffu, r;
  if (e == 0xffu) r = 0x7fc00000u;
  else if (e > 23u) r = (e - 23u) << 23;
  else r = e == 0u ? 1u : (1u << (e - 1u));
  float y; memcpy(&y, &r, 4); return y;
}
static inline float o_nextfloat(float x) {
  if (x != x || x == INFINITY) return x;
  uint32_t b;
  if (x == 0.0f) b = 1u; else { memcpy(&b, &x, 4); b = x > 0.0f ? b + 1u : b - 1u; }
  float y; memcpy(&y, &b, 4); return y;
}

template <class Tt> struct CbClock;
template <> struct CbClock<float> {
  static float bottom(const Integ<float>& ig) { return ig.tprev; }
  static float top(const Integ<float>& ig) { return ig.t; }
  static float theta(const Integ<float>& ig, float x) { return (x - ig.tprev) / ig.dt; }
  static float time(const Integ<float>& ig, float x) { (void)ig; return x; }
};
template <> struct CbClock<DF> {
  static float bottom(const Integ<DF>& ig) { (void)ig; return 0.0f; }
  static float top(const Integ<DF>& ig) { return t_rem(ig.t, ig.tprev, 0.0f); }
  static float theta(const Integ<DF>& ig, float x) { return x / ig.dt; }
  static DF time(const Integ<DF>& ig, float x) { return t_add(ig.tprev, x); }
};

/* get_condition (integrator_utils.jl:461-479): u at t, uprev at tprev, else integ(abst) */
template <class Tt>
static float cond_at(int m, int alg, const Integ<Tt>& ig, const float* p, int fn, float x) {
  typedef CbClock<Tt> K;
  float v[MAXN];
  if (x == K::top(ig)) for (int c = 0; c < ig.N; c++) v[c] = ig.u[c];
  else if (x == K::bottom(ig)) for (int c = 0; c < ig.N; c++) v[c] = ig.uprev[c];
  else interpolate(m, alg, ig, p, K::theta(ig, x), ig.dt, v);
  return model_ccb_condition(m, fn, v, p, (double)t_out(K::time(ig, x)));
}

/* gpu_find_root (integrator_utils.jl:302-355): ITP, scaled_k1 = 0.2, k2 = 2, n0 = 10 */
template <class Tt>
static float itp_root(int m, int alg, const Integ<Tt>& ig, const float* p, int fn, float left, float right,
                      int rootfind) {
  float fl = cond_at(m, alg, ig, p, fn, left), fr = cond_at(m, alg, ig, p, fn, right);
  const float span0 = right - left;
  const float k1 = 0.2f / span0;
  float eps_s = span0 * 512.0f;
  for (int it = 0; it < 100; it++) {
    const float span = right - left;
    const float mid = (left + right) / 2.0f;
    const float r = eps_s - span / 2.0f;
    const float x_f = left + (span * fl) / (fl - fr);
    const float delta = o_max(k1 * span * span, o_eps(x_f));
    const float diff = mid - x_f;
    const float xt = (delta <= fabsf(diff)) ? x_f + copysignf(delta, diff) : mid;
    const float xp = (fabsf(xt - mid) <= r) ? xt : mid - copysignf(r, diff);
    const float yp = cond_at(m, alg, ig, p, fn, xp);
    const float yps = yp * jl_sign(fr);
    if (yps > 0.0f) { right = xp; fr = yp; }
    else if (yps < 0.0f) { left = xp; fl = yp; }
    else { left = xp; right = xp; break; }
    eps_s = eps_s / 2.0f;
    if (o_nextfloat(left) >= right) break;
  }
  return rootfind == 1 ? right : left;
}

/* savevalues! (integrator_utils.jl:13-50) */
template <class Tt>
static void save_values(int m, int alg, Integ<Tt>& ig, const float* p, const double* sa, int nsa, int L,
                        int save_every, typename TOut<Tt>::T* ts, float* us) {
  const int N = ig.N;
  if (!sa && save_every) {
    if (ig.step_idx >= 0 && ig.step_idx < L) {
      for (int i = 0; i < N; i++) us[(size_t)ig.step_idx * N + i] = ig.u[i];
      ts[ig.step_idx] = t_out(ig.t);
    }
    ig.step_idx++;
  } else if (sa) {
    while (ig.cur_t < nsa && t_le(t_from<Tt>(sa[ig.cur_t]), ig.t)) {
      Tt savet = t_from<Tt>(sa[ig.cur_t]);
      float th = t_theta(savet, ig.tprev, ig.dt);
      if (ig.cur_t < L) {
        interpolate(m, alg, ig, p, th, ig.dt, us + (size_t)ig.cur_t * N);
        ts[ig.cur_t] = (typename TOut<Tt>::T)sa[ig.cur_t];
      }
      ig.cur_t++;
    }
  }
}

template <class Tt>
static void run_affect(int m, Integ<Tt>& ig, const float* p, int kind, int fn) {
  CbInteg I{ig.u, p, (double)t_out(ig.t), ig.dt, 0};
  if (kind == 2) model_dcb_affect(m, fn, I);
  else model_ccb_affect(m, fn, I);  /* the built-in models use affect! as affect_neg! */
  if (I.terminated) ig.retcode = RET_TERMINATED;
}

/* handle_callbacks! (:258-300) with find_callback_time (:357-428), apply_callback! (:212-256),
 * change_t_via_interpolation! (:180-209) and apply_discrete_callback! (:67-150).
 * Returns saved_in_cb. */
template <class Tt>
static int handle_callbacks(int m, const oracle_cfg* cfg, Integ<Tt>& ig, const float* p, const double* sa,
                            int nsa, int L, int save_every, typename TOut<Tt>::T* ts, float* us) {
  typedef CbClock<Tt> K;
  const int alg = cfg->alg, N = ig.N;
  int saved = 0;
  if (cfg->nccb > 0) {
    int occ_best = 0, idx = 0;
    float t_best = 0.0f, sign_best = 0.0f, res_best = 0.0f;
    for (int j = 0; j < cfg->nccb; j++) {
      const int fn = cfg->ccb_fn[j], fl = cfg->ccb_flags[j];
      float bottom_t = K::bottom(ig);
      float bottom_c = model_ccb_condition(m, fn, ig.uprev, p, (double)t_out(ig.tprev));
      if (ig.event_last == j + 1 && fabsf(bottom_c - ig.last_event_error) <= cfg->ccb_abstol[j]) {
        bottom_t = bottom_t + ig.dt * cfg->ccb_nudge[j];
        bottom_c = cond_at(m, alg, ig, p, fn, bottom_t);
      }
      const float bs = jl_sign(bottom_c);
      const float top_t = K::top(ig);
      const float tsg = jl_sign(cond_at(m, alg, ig, p, fn, top_t));
      const int occ = ((bs < 0.0f && (fl & 1)) || (bs > 0.0f && (fl & 2))) && bs * tsg <= 0.0f;
      float te = top_t, res = 0.0f;
      const int rootfind = (fl >> 2) & 3;
      if (occ && rootfind != 2 && tsg != 0.0f) {
        te = itp_root(m, alg, ig, p, fn, bottom_t, top_t, rootfind);
        res = cond_at(m, alg, ig, p, fn, te);
      }
      if (occ && (!occ_best || te < t_best)) { occ_best = 1; t_best = te; sign_best = bs; res_best = res; idx = j + 1; }
    }
    if (occ_best) {
      ig.event_last = idx;
      ig.last_event_error = res_best;
      const float xcur = K::top(ig);
      if (t_best != xcur) { /* change_t_via_interpolation! (:180-209) */
        float v[MAXN];
        interpolate(m, alg, ig, p, K::theta(ig, t_best), ig.dt, v);
        for (int c = 0; c < N; c++) ig.u[c] = v[c];
        ig.step_idx -= (int)rintf((xcur - t_best) / ig.dt);
        ig.t = K::time(ig, t_best);
      }
      if (cfg->adaptive && ig.dtnew < 1.0e-12f) { /* :226-234 */
        const float remaining = fabsf(t_rem(ig.tf, ig.t, 0.0f));
        const float relaxed = cfg->ccb_dtrelax[0] * ig.dt;
        ig.dtnew = (remaining < relaxed) ? remaining : relaxed;
      }
      save_values(m, alg, ig, p, sa, nsa, L, save_every, ts, us);
      saved = 1;
      ig.u_modified = 1;
      const int f0 = cfg->ccb_flags[0];
      if (sign_best < 0.0f) { if (f0 & 1) run_affect(m, ig, p, 0, cfg->ccb_fn[0]); else ig.u_modified = 0; }
      else if (sign_best > 0.0f) { if (f0 & 2) run_affect(m, ig, p, 1, cfg->ccb_fn[0]); else ig.u_modified = 0; }
    } else {
      ig.event_last = 0;
    }
  }
  if (cfg->ndcb > 0) {
    int dsaved = 0;
    for (int j = 0; j < cfg->ndcb; j++) {
      const int fn = cfg->dcb_fn[j];
      if (model_dcb_condition(m, fn, ig.u, p, (double)t_out(ig.t))) {
        save_values(m, alg, ig, p, sa, nsa, L, save_every, ts, us);
        dsaved = 1;
        ig.u_modified = 1;
        run_affect(m, ig, p, 2, fn);
      }
    }
    saved = dsaved;
  }
  return saved;
}

/* `tstops[idx] - t - dt - 100 eps(T) < 0` (gpu_tsit5_perform_step.jl:18-19, :158-160) */
template <class Tt>
static int tstop_due(const oracle_cfg* cfg, const Integ<Tt>& ig, Tt t, float dt, Tt* s) {
  if (ig.tstops_idx >= cfg->ntstops) return 0;
  const float tol = sizeof(typename TOut<Tt>::T) == 8 ? (float)(100.0 * 2.220446049250313e-16) : 100.0f * 1.1920928955078125e-07f;
  *s = t_from<Tt>(cfg->tstops[ig.tstops_idx]);
  return t_rem(*s, t, dt) - tol < 0.0f;
}

/* ------------------------------------------------------------------ one trajectory (kernels.jl) */
template <class Tt>
static void solve_one(int m, const oracle_cfg* cfg, long long idx, const float* u0, const float* p, const double* tsp,
                      typename TOut<Tt>::T* ts, float* us, signed char* retcode, int* nacc, int* nrej) {
  typedef typename TOut<Tt>::T Out;
  ModelInfo mi = model_info(m);
  const int N = mi.N, L = cfg->L, alg = cfg->alg;
  Integ<Tt> ig;
  memset(&ig, 0, sizeof(ig));
  ig.N = N;
  Tt t0 = t_from<Tt>(tsp[0]), tf = t_from<Tt>(tsp[1]);
  for (int i = 0; i < N; i++) { ig.u[i] = u0[i]; ig.uprev[i] = u0[i]; for (int s = 0; s < 10; s++) ig.k[s][i] = u0[i]; }
  ig.t = t0; ig.tprev = t0; ig.tf = tf;
  float dt_in = cfg->dt0 ? cfg->dt0[idx] : (float)cfg->dt;
  ig.dt = dt_in; ig.dtnew = dt_in;
  float tsc = cfg->tolscale ? cfg->tolscale[idx] : 1.0f;
  ig.abstol = cfg->abstol * tsc; ig.reltol = cfg->reltol * tsc;
  ig.u_modified = 1; ig.retcode = RET_DEFAULT;
  ig.tstops_idx = 0; ig.event_last = 1; ig.last_event_error = 0.0f; /* stiff/types.jl:44-46 */
  Ctrl C = make_ctrl(alg_order(alg));
  ig.qold = C.qoldinit;

  /* fill! ts with tspan[1] (lowerlevel_solve.jl:82, 107, 318, 322) */
  for (int l = 0; l < L; l++) ts[l] = (Out)tsp[0];
  const double* sa = cfg->nsaveat ? (cfg->saveat_per_traj ? cfg->saveat + idx * cfg->nsaveat : cfg->saveat) : NULL;
  int nsa = cfg->nsaveat;
#define US(l) (us + (size_t)(l) * N)
#define SA(l) (t_from<Tt>(sa[(l)]))
  /* kernels.jl:35-47 / :116-126 (0-based cur_t here == 1-based cur_t - 1) */
  ig.cur_t = 0; ig.step_idx = 0;
  if (sa) {
    if ((Out)tsp[0] == (Out)sa[0]) { ig.cur_t = 1; for (int i = 0; i < N; i++) US(0)[i] = u0[i]; }
  } else {
    ts[0] = (Out)tsp[0]; for (int i = 0; i < N; i++) US(0)[i] = u0[i];
  }
  ig.step_idx = 1;

  const int save_every = cfg->save_everystep && !cfg->adaptive; /* adaptive init stores save_everystep=false (types.jl) */
  while (t_lt(ig.t, tf) && ig.retcode != RET_TERMINATED && ig.retcode != RET_DTMIN && ig.retcode != RET_MAXITERS) {
    /* ---------------- step! ---------------- */
    Tt t = ig.t;
    for (int i = 0; i < N; i++) ig.uprev[i] = ig.u[i];
    if (!cfg->adaptive) {
      if (++ig.nattempt > cfg->maxiters) { ig.retcode = RET_MAXITERS; break; }
      float dt = ig.dt;
      ig.tprev = t;
      Tt tstop;
      if (tstop_due(cfg, ig, t, dt, &tstop)) { ig.t = tstop; dt = t_rem(tstop, t, 0.0f); ig.tstops_idx++; }
      else ig.t = t_add(t, dt);
      float u[MAXN];
      if (alg == ALG_TSIT5) {
        float k1[MAXN];
        if (ig.u_modified) { model_f<float>(m, k1, ig.uprev, p, t_f32(t)); ig.u_modified = 0; }
        else for (int i = 0; i < N; i++) k1[i] = ig.k[6][i];
        tsit5_stages(m, ig, p, t, dt, k1, u, ig.k, 1);
      } else if (alg == ALG_VERN7) {
        vern7_stages(m, ig, p, t, dt, u, ig.k);
      } else if (alg == ALG_VERN9) {
        vern9_stages(m, ig, p, t, dt, u, ig.k);
      } else if (alg == ALG_RB23) {
        float err[MAXN];
        rb23_attempt(m, cfg->jac, ig, p, t, dt, u, ig.k[0], ig.k[1], err, 0);
      } else if (alg == ALG_RODAS5P) {
        float k8[MAXN];
        compute_J(m, cfg->jac, N, ig.J, ig.uprev, p, t_f32(t));
        compute_tgrad(m, cfg->jac, N, ig.dT, ig.uprev, p, t_f32(t));
        rodas5p_attempt(m, ig, p, t, dt, u, k8, ig.k);
      } else if (alg == ALG_KVAERNO3 || alg == ALG_KVAERNO5) {
        /* FSAL k1 = integ.k1 unless u was modified; the nonlinear solver takes integ.t (already
         * advanced) and integ.dt (gpu_kvaerno3_perform_step.jl:26-38) */
        float k1[MAXN], err[MAXN];
        if (ig.u_modified) { model_f<float>(m, k1, ig.uprev, p, t_f32(t)); ig.u_modified = 0; }
        else for (int i = 0; i < N; i++) k1[i] = ig.k[0][i];
        kvaerno_attempt(m, cfg->jac, alg, ig, p, t, dt, ig.t, ig.dt, k1, u, ig.k[1], err, 0);
        model_f<float>(m, ig.k[0], u, p, t_f32(t)); /* integ.k1 = f(u, p, t) (:83-86) */
      } else if (alg == ALG_RODAS4) {
        float k6[MAXN];
        compute_J(m, cfg->jac, N, ig.J, ig.uprev, p, t_f32(t));
        compute_tgrad(m, cfg->jac, N, ig.dT, ig.uprev, p, t_f32(t));
        rodas4_attempt(m, ig, p, t, dt, u, k6, ig.k);
      }
      for (int i = 0; i < N; i++) ig.u[i] = u[i];
      ig.naccept++;
    } else {
      float dt = ig.dtnew;
      float k1[MAXN];
      if (alg == ALG_TSIT5) {
        if (ig.u_modified) { model_f<float>(m, k1, ig.uprev, p, t_f32(t)); ig.u_modified = 0; }
        else for (int i = 0; i < N; i++) k1[i] = ig.k[6][i];
      }
      if (alg == ALG_KVAERNO3 || alg == ALG_KVAERNO5) model_f<float>(m, k1, ig.uprev, p, t_f32(t)); /* k1 = f(uprev, p, t) */
      if (alg == ALG_RODAS5P || alg == ALG_RODAS4) { /* J, dT once per step, outside the reject loop */
        compute_J(m, cfg->jac, N, ig.J, ig.uprev, p, t_f32(t));
        compute_tgrad(m, cfg->jac, N, ig.dT, ig.uprev, p, t_f32(t));
      }
      float EEst = INFINITY;
      while (EEst > 1.0f) {
        if (dt < 1.0e-14f) { ig.retcode = RET_DTMIN; break; }
        if (++ig.nattempt > cfg->maxiters) { ig.retcode = RET_MAXITERS; break; }
        float u[MAXN], err[MAXN], kk[10][MAXN];
        if (alg == ALG_TSIT5) {
          tsit5_stages(m, ig, p, t, dt, k1, u, kk, 0);
          for (int i = 0; i < N; i++)
            err[i] = dt * (TS5.bt1 * kk[0][i] + TS5.bt2 * kk[1][i] + TS5.bt3 * kk[2][i] + TS5.bt4 * kk[3][i] + TS5.bt5 * kk[4][i] + TS5.bt6 * kk[5][i] + TS5.bt7 * kk[6][i]);
        } else if (alg == ALG_VERN7) {
          vern7_stages(m, ig, p, t, dt, u, kk);
          for (int i = 0; i < N; i++)
            err[i] = dt * (V7C(btilde1) * kk[0][i] + V7C(btilde4) * kk[3][i] + V7C(btilde5) * kk[4][i] + V7C(btilde6) * kk[5][i] + V7C(btilde7) * kk[6][i] + V7C(btilde8) * kk[7][i] + V7C(btilde9) * kk[8][i] + V7C(btilde10) * kk[9][i]);
        } else if (alg == ALG_VERN9) {
          vern9_stages(m, ig, p, t, dt, u, kk);
          for (int i = 0; i < N; i++)
            err[i] = dt * (F9C(btilde1) * kk[0][i] + F9C(btilde8) * kk[1][i] + F9C(btilde9) * kk[2][i] + F9C(btilde10) * kk[3][i] + F9C(btilde11) * kk[4][i] + F9C(btilde12) * kk[5][i] + F9C(btilde13) * kk[6][i] + F9C(btilde14) * kk[7][i] + F9C(btilde15) * kk[8][i] + F9C(btilde16) * kk[9][i]);
        } else if (alg == ALG_RB23) {
          rb23_attempt(m, cfg->jac, ig, p, t, dt, u, kk[0], kk[1], err, 1);
        } else if (alg == ALG_KVAERNO3 || alg == ALG_KVAERNO5) {
          for (int i = 0; i < N; i++) kk[0][i] = k1[i];
          kvaerno_attempt(m, cfg->jac, alg, ig, p, t, dt, t, dt, k1, u, kk[1], err, 1);
        } else if (alg == ALG_RODAS4) { /* error estimate is k6 */
          rodas4_attempt(m, ig, p, t, dt, u, err, kk);
        } else { /* Rodas5P: error estimate is k8 */
          rodas5p_attempt(m, ig, p, t, dt, u, err, kk);
        }
        EEst = scaled_norm(err, ig.uprev, u, N, ig.abstol, ig.reltol);
        if (controller(ig, C, EEst, dt, t)) {
          int ns = alg == ALG_TSIT5 ? 7 : (alg == ALG_VERN7 || alg == ALG_VERN9) ? 10
                   : (alg == ALG_RB23 || alg == ALG_RODAS4 || alg == ALG_KVAERNO3 || alg == ALG_KVAERNO5) ? 2 : 3;
          for (int s = 0; s < ns; s++) for (int i = 0; i < N; i++) ig.k[s][i] = kk[s][i];
          for (int i = 0; i < N; i++) ig.u[i] = u[i];
          /* not snapped to tf: stop at the next tstop, u = integ(tstop) (:157-167) */
          Tt tstop;
          if (!(t_rem(ig.tf, t, dt) < 1.0e-14f) && tstop_due(cfg, ig, t, dt, &tstop)) {
            ig.t = tstop;
            ig.tstops_idx++;
            float v[MAXN];
            interpolate(m, alg, ig, p, t_theta(ig.t, ig.tprev, ig.dt), ig.dt, v);
            for (int i = 0; i < N; i++) ig.u[i] = v[i];
          }
          ig.naccept++;
        } else {
          ig.nreject++;
        }
      }
      if (ig.retcode == RET_DTMIN || ig.retcode == RET_MAXITERS) break;
    }
    /* ---------------- callbacks, then savevalues! unless a callback saved (kernels.jl:50-51) */
    int saved_in_cb = 0;
    if (cfg->nccb > 0 || cfg->ndcb > 0) saved_in_cb = handle_callbacks(m, cfg, ig, p, sa, nsa, L, save_every, ts, us);
    if (!saved_in_cb) save_values(m, alg, ig, p, sa, nsa, L, save_every, ts, us);
  }
  /* kernels.jl:53-62 / :133-142 */
  if (t_lt(tf, ig.t) && !sa) {
    if (cfg->save_everystep) { /* with !save_everystep slot 2 is overwritten right below */
      float th = t_theta(tf, ig.tprev, ig.dt);
      interpolate(m, alg, ig, p, th, ig.dt, US(L - 1));
      ts[L - 1] = (Out)tsp[1];
    }
  }
  if (!sa && !cfg->save_everystep) {
    for (int i = 0; i < N; i++) US(1)[i] = ig.u[i];
    ts[1] = t_out(ig.t);
  }
#undef US
#undef SA
  int finite = 1;
  for (int i = 0; i < N; i++) if (!isfinite(ig.u[i])) finite = 0;
  if (ig.retcode == RET_DEFAULT) ig.retcode = finite ? RET_SUCCESS : RET_UNSTABLE;
  if (retcode) retcode[idx] = (signed char)ig.retcode;
  if (nacc) nacc[idx] = (int)ig.naccept;
  if (nrej) nrej[idx] = (int)ig.nreject;
}

/* ------------------------------------------------------------------ EM (gpu_em_perform_step.jl:1-74)
 * Counter-based normals: Philox4x32-10 (Salmon et al., SC'11) keyed by the seed,
 * counter (step, trajectory, block, 0); Box-Muller with portable log / sincos. */
static inline uint32_t mulhi32(uint32_t a, uint32_t b) { return (uint32_t)(((uint64_t)a * b) >> 32); }
static void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; r++) {
    uint32_t hi0 = mulhi32(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
    uint32_t hi1 = mulhi32(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
    uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
}
static void normals4(uint64_t seed, uint32_t step, uint32_t traj, uint32_t blk, float* z) {
  uint32_t c[4] = {step, traj, blk, 0u};
  philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  for (int h = 0; h < 2; h++) {
    float u1 = (float)((c[2 * h] >> 8) + 1u) * 5.9604645e-08f;  /* (0, 1] */
    float u2 = (float)(c[2 * h + 1] >> 8) * 5.9604645e-08f;     /* [0, 1) */
    float r = sqrtf(-2.0f * pm_logf(u1));
    float s, co;
    pm_sincos_turns(u2, &s, &co);
    z[2 * h] = r * co; z[2 * h + 1] = r * s;
  }
}

template <class Tt>
static void em_one(int m, const oracle_cfg* cfg, long long idx, const float* u0, const float* p, const double* tsp,
                   typename TOut<Tt>::T* ts, float* us, signed char* retcode) {
  typedef typename TOut<Tt>::T Out;
  ModelInfo mi = model_info(m);
  const int N = mi.N, L = cfg->L;
  const Out t0_in = (Out)tsp[0], tf_in = (Out)tsp[1];
  const float dt = (float)cfg->dt;
  for (int l = 0; l < L; l++) ts[l] = t0_in;
  const double* sa = cfg->nsaveat ? (cfg->saveat_per_traj ? cfg->saveat + idx * cfg->nsaveat : cfg->saveat) : NULL;
  int nsa = cfg->nsaveat, cur_t = 0;
#define US(l) (us + (size_t)(l) * N)
  if (sa) { if (t0_in == (Out)sa[0]) { cur_t = 1; for (int i = 0; i < N; i++) US(0)[i] = u0[i]; } }
  else { ts[0] = t0_in; for (int i = 0; i < N; i++) US(0)[i] = u0[i]; }
  float sqdt = sqrtf(dt);
  float u[MAXN], up[MAXN], f[MAXN], g[MAXN], z[MAXN + 4];
  for (int i = 0; i < N; i++) u[i] = u0[i];
  Tt t = t_from<Tt>(tsp[0]);
  const Out span = tf_in - t0_in, dtb = (Out)dt;
  const Out ratio = (span < 0 ? -span : span) / (dtb < 0 ? -dtb : dtb); /* floor(Int, abs(tf - t0) / abs(dt)) */
  long long n = (long long)floor((double)ratio) + 1;
  if (n - 1 > cfg->maxiters) n = cfg->maxiters + 1;
  for (long long j = 2; j <= n; j++) {
    for (int i = 0; i < N; i++) up[i] = u[i];
    model_f<float>(m, f, up, p, t_f32(t));
    model_g(m, g, up, p);
    for (int b = 0; b < (N + 3) / 4; b++) normals4(cfg->seed, (uint32_t)(j - 2), (uint32_t)idx, (uint32_t)b, z + 4 * b);
    if (cfg->alg == ALG_SIEA) { /* gpu_siea_perform_step.jl:48-139, coefficients :23-47 */
      float dW[MAXN], W2[MAXN], W3[MAXN], x[MAXN], k1[MAXN], g1[MAXN], g2[MAXN];
      for (int i = 0; i < N; i++) {
        dW[i] = sqdt * z[i];
        W2[i] = (dW[i] * dW[i]) / sqdt;
        W3[i] = (0.0f * (dW[i] * dW[i] * dW[i])) / dt;
      }
      const float tstg = t_stage(t, 1.0f, dt);
      for (int i = 0; i < N; i++) x[i] = up[i] + (1.0f * f[i]) * dt + (1.0f * g[i]) * dW[i] + g[i] * W3[i];
      model_f<float>(m, k1, x, p, tstg);
      for (int i = 0; i < N; i++) x[i] = up[i] + (1.0f * f[i]) * dt + (1.0f * g[i]) * sqdt + (0.0f * g[i]) * W2[i];
      model_g(m, g1, x, p);
      for (int i = 0; i < N; i++) x[i] = up[i] + (1.0f * f[i]) * dt + (-1.0f * g[i]) * sqdt + (0.0f * g[i]) * W2[i];
      model_g(m, g2, x, p);
      for (int i = 0; i < N; i++) {
        u[i] = up[i] + (0.5f * f[i] + 0.5f * k1[i]) * dt;
        u[i] = u[i] + ((0.5f * g[i]) * dW[i] + ((0.25f * dW[i] + -0.25f * sqdt) + 0.25f * W2[i]) * g1[i] +
                       ((0.25f * dW[i] + 0.25f * sqdt) + -0.25f * W2[i]) * g2[i]);
      }
    } else {
      for (int i = 0; i < N; i++) u[i] = up[i] + f[i] * dt + (sqdt * g[i]) * z[i];
    }
    t = t_add(t, dt);
    if (!sa && cfg->save_everystep) {
      if (j - 1 < L) { for (int i = 0; i < N; i++) US(j - 1)[i] = u[i]; ts[j - 1] = t_out(t); }
    } else if (sa) {
      while (cur_t < nsa && t_le(t_from<Tt>(sa[cur_t]), t)) {
        Tt savet = t_from<Tt>(sa[cur_t]);
        float th = t_em_theta(savet, t, dt);
        if (cur_t < L) { for (int i = 0; i < N; i++) US(cur_t)[i] = up[i] + (u[i] - up[i]) * th; ts[cur_t] = (Out)sa[cur_t]; }
        cur_t++;
      }
    }
  }
  if (!sa && !cfg->save_everystep) { for (int i = 0; i < N; i++) US(1)[i] = u[i]; ts[1] = t_out(t); }
#undef US
  int finite = 1;
  for (int i = 0; i < N; i++) if (!isfinite(u[i])) finite = 0;
  if (retcode) retcode[idx] = finite ? RET_SUCCESS : RET_UNSTABLE;
}

/* ------------------------------------------------------------------ public C API */
extern "C" {

int oracle_model_dims(int model, int* N, int* P) {
  ModelInfo mi = model_info(model);
  if (!mi.N) return -1;
  *N = mi.N; *P = mi.P;
  return 0;
}

/* Ensemble solve on the host cores.  Layouts match the library's: u0 [B][N], p [B][P],
 * tspan [B][2] (f64, converted to Tt), ts [B][L] (Tt), us [B][L][N] (f32). */
int oracle_solve(int model, long long B, const float* u0, const float* p, const double* tspan,
                 const oracle_cfg* cfg, void* ts, float* us, signed char* retcode, int* naccept, int* nreject,
                 int nthreads) {
  ModelInfo mi = model_info(model);
  if (!mi.N || B < 0 || cfg->L < 1) return -1;
  if (!cfg->adaptive && !cfg->nsaveat && !cfg->save_everystep && cfg->L != 2) return -2;
  init_tabs();
  const int N = mi.N, P = mi.P, L = cfg->L;
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
  for (long long i = 0; i < B; i++) {
    const float* pi = p + (size_t)i * P;
    const double* tsp = tspan + 2 * (size_t)i;
    float* usi = us + (size_t)i * L * N;
    if (cfg->alg == ALG_EM || cfg->alg == ALG_SIEA) {
      if (cfg->time_f64) em_one<DF>(model, cfg, i, u0 + (size_t)i * N, pi, tsp, (double*)ts + (size_t)i * L, usi, retcode);
      else em_one<float>(model, cfg, i, u0 + (size_t)i * N, pi, tsp, (float*)ts + (size_t)i * L, usi, retcode);
    } else {
      if (cfg->time_f64) solve_one<DF>(model, cfg, i, u0 + (size_t)i * N, pi, tsp, (double*)ts + (size_t)i * L, usi, retcode, naccept, nreject);
      else solve_one<float>(model, cfg, i, u0 + (size_t)i * N, pi, tsp, (float*)ts + (size_t)i * L, usi, retcode, naccept, nreject);
    }
  }
  return 0;
}

/* the portable math used by parity mode, exported so tests can check its accuracy */
float oracle_pm_powf(float x, float y) { return pm_powf(x, y); }
float oracle_pm_logf(float x) { return pm_logf(x); }
float oracle_pm_expf(float x) { return pm_expf(x); }
void oracle_philox4x32_10(const unsigned* ctr, unsigned k0, unsigned k1, unsigned* out) {
  uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
  philox4x32_10(c, k0, k1);
  for (int i = 0; i < 4; i++) out[i] = c[i];
}
void oracle_normals4(unsigned long long seed, unsigned step, unsigned traj, unsigned blk, float* z) { normals4(seed, step, traj, blk, z); }

/* ------------------------------------------------------------------ FP64 Vern9 error oracle
 * Explicit 16-stage Verner 9(8) pair (tableaus/verner_tableaus.jl:1198-1332), generic
 * stage loop, standard PI-free controller with safety 0.9; saves land exactly on the
 * requested times (the step is clipped), so no interpolation error enters the oracle. */
static double V9A[17][17], V9C[17], V9B[17], V9BT[17];
static int v9_ready = 0;
static void init_v9() {
  if (v9_ready) return;
#pragma omp critical(oracle_v9)
  if (!v9_ready) {
    memset(V9A, 0, sizeof(V9A)); memset(V9C, 0, sizeof(V9C)); memset(V9B, 0, sizeof(V9B)); memset(V9BT, 0, sizeof(V9BT));
#define AV(r, c, n) V9A[r][c] = OR_VERN9[OR_VERN9_##n];
    AV(2, 1, a0201) AV(3, 1, a0301) AV(3, 2, a0302) AV(4, 1, a0401) AV(4, 3, a0403) AV(5, 1, a0501) AV(5, 3, a0503) AV(5, 4, a0504)
    AV(6, 1, a0601) AV(6, 4, a0604) AV(6, 5, a0605) AV(7, 1, a0701) AV(7, 4, a0704) AV(7, 5, a0705) AV(7, 6, a0706)
    AV(8, 1, a0801) AV(8, 6, a0806) AV(8, 7, a0807) AV(9, 1, a0901) AV(9, 6, a0906) AV(9, 7, a0907) AV(9, 8, a0908)
    AV(10, 1, a1001) AV(10, 6, a1006) AV(10, 7, a1007) AV(10, 8, a1008) AV(10, 9, a1009)
    AV(11, 1, a1101) AV(11, 6, a1106) AV(11, 7, a1107) AV(11, 8, a1108) AV(11, 9, a1109) AV(11, 10, a1110)
    AV(12, 1, a1201) AV(12, 6, a1206) AV(12, 7, a1207) AV(12, 8, a1208) AV(12, 9, a1209) AV(12, 10, a1210) AV(12, 11, a1211)
    AV(13, 1, a1301) AV(13, 6, a1306) AV(13, 7, a1307) AV(13, 8, a1308) AV(13, 9, a1309) AV(13, 10, a1310) AV(13, 11, a1311) AV(13, 12, a1312)
    AV(14, 1, a1401) AV(14, 6, a1406) AV(14, 7, a1407) AV(14, 8, a1408) AV(14, 9, a1409) AV(14, 10, a1410) AV(14, 11, a1411) AV(14, 12, a1412) AV(14, 13, a1413)
    AV(15, 1, a1501) AV(15, 6, a1506) AV(15, 7, a1507) AV(15, 8, a1508) AV(15, 9, a1509) AV(15, 10, a1510) AV(15, 11, a1511) AV(15, 12, a1512) AV(15, 13, a1513) AV(15, 14, a1514)
    AV(16, 1, a1601) AV(16, 6, a1606) AV(16, 7, a1607) AV(16, 8, a1608) AV(16, 9, a1609) AV(16, 10, a1610) AV(16, 11, a1611) AV(16, 12, a1612) AV(16, 13, a1613)
#undef AV
#define CV(s, n) V9C[s] = OR_VERN9[OR_VERN9_##n];
    CV(2, c1) CV(3, c2) CV(4, c3) CV(5, c4) CV(6, c5) CV(7, c6) CV(8, c7) CV(9, c8) CV(10, c9) CV(11, c10) CV(12, c11) CV(13, c12) CV(14, c13)
#undef CV
    V9C[15] = 1.0; V9C[16] = 1.0;
#define BV(s, n) V9B[s] = OR_VERN9[OR_VERN9_##n];
    BV(1, b1) BV(8, b8) BV(9, b9) BV(10, b10) BV(11, b11) BV(12, b12) BV(13, b13) BV(14, b14) BV(15, b15)
#undef BV
#define BT(s, n) V9BT[s] = OR_VERN9[OR_VERN9_##n];
    BT(1, btilde1) BT(8, btilde8) BT(9, btilde9) BT(10, btilde10) BT(11, btilde11) BT(12, btilde12) BT(13, btilde13) BT(14, btilde14) BT(15, btilde15) BT(16, btilde16)
#undef BT
    v9_ready = 1;
  }
}

static void f64_rhs(int m, double* du, const double* u, const double* p, double t) {
  (void)t;
  switch (m) {
    case M_LORENZ: case M_LORENZ_ADDNOISE:
      du[0] = p[0] * (u[1] - u[0]); du[1] = u[0] * (p[1] - u[2]) - u[1]; du[2] = u[0] * u[1] - p[2] * u[2]; break;
    case M_ROBERTSON:
      du[0] = -p[0] * u[0] + p[2] * u[1] * u[2]; du[1] = p[0] * u[0] - p[1] * u[1] * u[1] - p[2] * u[1] * u[2]; du[2] = p[1] * u[1] * u[1]; break;
    case M_DECAY: du[0] = -p[0] * u[0]; break;
    case M_GROWTH: du[0] = u[0]; break;
    case M_LINEAR15: for (int i = 0; i < 15; i++) du[i] = 1.01 * u[i]; break;
    case M_GBM: du[0] = p[0] * u[0]; break;
    case M_OSC: du[0] = u[1]; du[1] = -(p[0] * p[0]) * u[0]; break;
  }
}

/* Integrate one trajectory from t0 through the increasing times `stops` (the last is tf);
 * writes the state at each stop.  Returns the number of accepted steps, or -1. */
static long long vern9_traj(int m, int N, const double* u0, const double* p, double t0, int nstop, const double* stops,
                            double rtol, double atol, double* out, long long maxsteps) {
  double u[MAXN], k[17][MAXN], y[MAXN], un[MAXN];
  for (int i = 0; i < N; i++) u[i] = u0[i];
  double t = t0, h = 1e-3 * (stops[nstop - 1] - t0 > 0 ? 1.0 : 1.0);
  if (nstop > 0 && stops[nstop - 1] - t0 > 0 && h > stops[nstop - 1] - t0) h = stops[nstop - 1] - t0;
  long long nacc = 0, tries = 0;
  int si = 0;
  while (si < nstop && stops[si] <= t) { for (int i = 0; i < N; i++) out[si * N + i] = u[i]; si++; }
  while (si < nstop) {
    if (++tries > maxsteps) return -1;
    double target = stops[si];
    int land = 0;
    double hh = h;
    if (t + hh >= target) { hh = target - t; land = 1; }
    f64_rhs(m, k[1], u, p, t);
    for (int s = 2; s <= 16; s++) {
      for (int i = 0; i < N; i++) { double acc = 0.0; for (int j = 1; j < s; j++) acc += V9A[s][j] * k[j][i]; y[i] = u[i] + hh * acc; }
      f64_rhs(m, k[s], y, p, t + V9C[s] * hh);
    }
    double err = 0.0;
    for (int i = 0; i < N; i++) {
      double acc = 0.0, ea = 0.0;
      for (int s = 1; s <= 16; s++) { acc += V9B[s] * k[s][i]; ea += V9BT[s] * k[s][i]; }
      un[i] = u[i] + hh * acc;
      double sc = atol + rtol * fmax(fabs(u[i]), fabs(un[i]));
      double e = hh * ea / sc;
      err += e * e;
    }
    err = sqrt(err / N);
    if (!(err == err)) return -1;
    if (err <= 1.0) {
      for (int i = 0; i < N; i++) u[i] = un[i];
      t = land ? target : t + hh;
      nacc++;
      while (si < nstop && stops[si] <= t) { for (int i = 0; i < N; i++) out[si * N + i] = u[i]; si++; }
      double fac = err == 0.0 ? 5.0 : fmin(5.0, fmax(0.2, 0.9 * pow(err, -1.0 / 9.0)));
      if (!land || hh >= h) h = hh * fac; /* a clipped landing step does not shrink h */
    } else {
      h = hh * fmax(0.2, 0.9 * pow(err, -1.0 / 9.0));
    }
    if (h < 1e-15) return -1;
  }
  return nacc;
}

/* FP64 reference solutions.  stops: shared [nstop] (per_traj=0) or [B][nstop] (per_traj=1);
 * out [B][nstop][N].  Returns the number of trajectories that failed. */
long long oracle_vern9_f64(int model, long long B, const double* u0, const double* p, const double* t0,
                           int nstop, const double* stops, int per_traj, double rtol, double atol,
                           double* out, long long* nsteps, int nthreads) {
  ModelInfo mi = model_info(model);
  if (!mi.N) return -1;
  init_v9();
  const int N = mi.N, P = mi.P;
  long long fails = 0;
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads) reduction(+ : fails)
  for (long long i = 0; i < B; i++) {
    const double* st = per_traj ? stops + (size_t)i * nstop : stops;
    long long r = vern9_traj(model, N, u0 + (size_t)i * N, p + (size_t)i * P, t0[i], nstop, st, rtol, atol,
                             out + (size_t)i * nstop * N, 50000000LL);
    if (nsteps) nsteps[i] = r;
    if (r < 0) fails++;
  }
  return fails;
}

/* ------------------------------------------------------------------ FP64 stiff error oracle
 * An explicit Vern9 would need ~1e12 steps on Robertson over (0, 1e5), so stiff problems
 * are checked against FP64 Rodas5P (tableau rodas_tableaus.jl:186-283) with partial-pivot
 * LU, the analytic Jacobian and tight tolerances; tests cross-check it with scipy Radau. */
static void f64_jac(int m, double* J, const double* u, const double* p) {
  switch (m) {
    case M_ROBERTSON:
      J[0] = -p[0]; J[1] = p[0]; J[2] = 0.0;
      J[3] = p[2] * u[2]; J[4] = -2.0 * p[1] * u[1] - p[2] * u[2]; J[5] = 2.0 * p[1] * u[1];
      J[6] = p[2] * u[1]; J[7] = -p[2] * u[1]; J[8] = 0.0;
      break;
    case M_LORENZ: case M_LORENZ_ADDNOISE:
      J[0] = -p[0]; J[1] = p[1] - u[2]; J[2] = u[1]; J[3] = p[0]; J[4] = -1.0; J[5] = u[0]; J[6] = 0.0; J[7] = -u[0]; J[8] = -p[2];
      break;
    case M_DECAY: J[0] = -p[0]; break;
    case M_GROWTH: J[0] = 1.0; break;
    case M_OSC: J[0] = 0.0; J[1] = -(p[0] * p[0]); J[2] = 1.0; J[3] = 0.0; break;
    case M_LINEAR15: for (int i = 0; i < 225; i++) J[i] = 0.0; for (int i = 0; i < 15; i++) J[i * 16] = 1.01; break;
    case M_GBM: J[0] = p[0]; break;
  }
}
static void lu_f64(int N, double* A, int* piv) { /* column-major in place */
  for (int k = 0; k < N; k++) {
    int pr = k; double best = fabs(A[k + N * k]);
    for (int i = k + 1; i < N; i++) if (fabs(A[i + N * k]) > best) { best = fabs(A[i + N * k]); pr = i; }
    piv[k] = pr;
    if (pr != k) for (int j = 0; j < N; j++) { double t = A[k + N * j]; A[k + N * j] = A[pr + N * j]; A[pr + N * j] = t; }
    for (int i = k + 1; i < N; i++) {
      A[i + N * k] /= A[k + N * k];
      for (int j = k + 1; j < N; j++) A[i + N * j] -= A[i + N * k] * A[k + N * j];
    }
  }
}
static void lus_f64(int N, const double* A, const int* piv, double* b) {
  for (int k = 0; k < N; k++) if (piv[k] != k) { double t = b[k]; b[k] = b[piv[k]]; b[piv[k]] = t; }
  for (int i = 0; i < N; i++) for (int j = 0; j < i; j++) b[i] -= A[i + N * j] * b[j];
  for (int i = N - 1; i >= 0; i--) { for (int j = i + 1; j < N; j++) b[i] -= A[i + N * j] * b[j]; b[i] /= A[i + N * i]; }
}
static long long rodas5p_f64_traj(int m, int N, const double* u0, const double* p, double t0, int nstop, const double* stops,
                                  double rtol, double atol, double* out, long long maxsteps) {
#define R(n) OR_RODAS5P[OR_RODAS5P_##n]
  const double a[6][6] = {{0}, {R(a21)}, {R(a31), R(a32)}, {R(a41), R(a42), R(a43)}, {R(a51), R(a52), R(a53), R(a54)}, {R(a61), R(a62), R(a63), R(a64), R(a65)}};
  const double C[8][8] = {{0}, {R(C21)}, {R(C31), R(C32)}, {R(C41), R(C42), R(C43)}, {R(C51), R(C52), R(C53), R(C54)},
                          {R(C61), R(C62), R(C63), R(C64), R(C65)}, {R(C71), R(C72), R(C73), R(C74), R(C75), R(C76)},
                          {R(C81), R(C82), R(C83), R(C84), R(C85), R(C86), R(C87)}};
  const double cc[6] = {0.0, R(c2), R(c3), R(c4), R(c5), 1.0};
  const double dd[6] = {R(d1), R(d2), R(d3), R(d4), R(d5), 0.0};
  const double gam = R(gamma);
#undef R
  double u[MAXN], J[MAXN * MAXN], W[MAXN * MAXN], k[8][MAXN], du[MAXN], y[MAXN];
  int piv[MAXN];
  for (int i = 0; i < N; i++) u[i] = u0[i];
  double t = t0, h = 1e-8;
  long long nacc = 0, tries = 0;
  int si = 0;
  while (si < nstop && stops[si] <= t) { for (int i = 0; i < N; i++) out[si * N + i] = u[i]; si++; }
  while (si < nstop) {
    if (++tries > maxsteps) return -1;
    double target = stops[si];
    int land = 0;
    double hh = h;
    if (t + hh >= target) { hh = target - t; land = 1; }
    f64_jac(m, J, u, p);
    for (int j = 0; j < N; j++) for (int i = 0; i < N; i++) W[i + N * j] = J[i + N * j] - (i == j ? 1.0 / (hh * gam) : 0.0);
    lu_f64(N, W, piv);
    for (int s = 0; s < 8; s++) {
      if (s < 6) for (int i = 0; i < N; i++) { double acc = u[i]; for (int j = 0; j < s; j++) acc += a[s][j] * k[j][i]; y[i] = acc; }
      else for (int i = 0; i < N; i++) y[i] = y[i] + k[s - 1][i];
      f64_rhs(m, du, y, p, t + (s < 6 ? cc[s] : 1.0) * hh);
      for (int i = 0; i < N; i++) {
        double acc = du[i] + (s < 5 ? dd[s] * hh * 0.0 : 0.0); /* autonomous models: dT = 0 */
        for (int j = 0; j < s; j++) acc += C[s][j] / hh * k[j][i];
        k[s][i] = -acc;
      }
      lus_f64(N, W, piv, k[s]);
    }
    double err = 0.0, un[MAXN];
    for (int i = 0; i < N; i++) {
      un[i] = y[i] + k[7][i];
      double sc = atol + rtol * fmax(fabs(u[i]), fabs(un[i]));
      err += (k[7][i] / sc) * (k[7][i] / sc);
    }
    err = sqrt(err / N);
    if (!(err == err)) { h = hh * 0.2; continue; }
    if (err <= 1.0) {
      for (int i = 0; i < N; i++) u[i] = un[i];
      t = land ? target : t + hh;
      nacc++;
      while (si < nstop && stops[si] <= t) { for (int i = 0; i < N; i++) out[si * N + i] = u[i]; si++; }
      double fac = err == 0.0 ? 5.0 : fmin(5.0, fmax(0.2, 0.9 * pow(err, -1.0 / 5.0)));
      if (!land || hh >= h) h = hh * fac;
    } else {
      h = hh * fmax(0.2, 0.9 * pow(err, -1.0 / 5.0));
    }
    if (h < 1e-18) return -1;
  }
  return nacc;
}

long long oracle_rodas5p_f64(int model, long long B, const double* u0, const double* p, const double* t0,
                             int nstop, const double* stops, int per_traj, double rtol, double atol,
                             double* out, long long* nsteps, int nthreads) {
  ModelInfo mi = model_info(model);
  if (!mi.N) return -1;
  const int N = mi.N, P = mi.P;
  long long fails = 0;
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads) reduction(+ : fails)
  for (long long i = 0; i < B; i++) {
    const double* st = per_traj ? stops + (size_t)i * nstop : stops;
    long long r = rodas5p_f64_traj(model, N, u0 + (size_t)i * N, p + (size_t)i * P, t0[i], nstop, st, rtol, atol,
                                   out + (size_t)i * nstop * N, 50000000LL);
    if (nsteps) nsteps[i] = r;
    if (r < 0) fails++;
  }
  return fails;
}

} /* extern "C" */
