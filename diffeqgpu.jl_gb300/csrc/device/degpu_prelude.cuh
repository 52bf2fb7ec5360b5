// Device prelude: included by every NVRTC translation unit before the user's
// right-hand side, so that `template <class T> degpu_f(T* du, const T* u, const float* p, T t)`
// can be instantiated with float and with forward-mode dual numbers.
#pragma once

#ifdef __CUDACC_RTC__
typedef unsigned int uint32_t;
typedef unsigned long long uint64_t;
typedef int int32_t;
typedef long long int64_t;
#else
#include <stdint.h>
#endif

#include "degpu_params.h"

#define DEGPU_DEV __device__ __forceinline__

namespace degpu {

// ------------------------------------------------------------------ forward-mode duals
// Product rule ordered like ForwardDiff: (x*y).d = x.d * y.v + y.d * x.v.  Used for
// ForwardDiff-style Jacobians (nlsolve/type.jl:129-140) and time gradients (:142-157).
template <int NP>
struct Dual {
  float v;
  float d[NP];
  DEGPU_DEV Dual() : v(0.f) {
#pragma unroll
    for (int i = 0; i < NP; i++) d[i] = 0.f;
  }
  DEGPU_DEV Dual(float x) : v(x) {
#pragma unroll
    for (int i = 0; i < NP; i++) d[i] = 0.f;
  }
};
#define DEGPU_DUAL_BINOP(OP, VEXPR, DEXPR)                                   \
  template <int NP>                                                          \
  DEGPU_DEV Dual<NP> operator OP(const Dual<NP>& a, const Dual<NP>& b) {     \
    Dual<NP> r;                                                              \
    r.v = VEXPR;                                                             \
    _Pragma("unroll") for (int i = 0; i < NP; i++) r.d[i] = DEXPR;           \
    return r;                                                                \
  }
DEGPU_DUAL_BINOP(+, a.v + b.v, a.d[i] + b.d[i])
DEGPU_DUAL_BINOP(-, a.v - b.v, a.d[i] - b.d[i])
DEGPU_DUAL_BINOP(*, a.v * b.v, a.d[i] * b.v + b.d[i] * a.v)
#undef DEGPU_DUAL_BINOP
template <int NP> DEGPU_DEV Dual<NP> operator/(const Dual<NP>& a, const Dual<NP>& b) {
  Dual<NP> r;
  r.v = a.v / b.v;
  float inv2 = b.v * b.v;
#pragma unroll
  for (int i = 0; i < NP; i++) r.d[i] = (a.d[i] * b.v - b.d[i] * a.v) / inv2;
  return r;
}
template <int NP> DEGPU_DEV Dual<NP> operator-(const Dual<NP>& a) {
  Dual<NP> r; r.v = -a.v;
#pragma unroll
  for (int i = 0; i < NP; i++) r.d[i] = -a.d[i];
  return r;
}
template <int NP> DEGPU_DEV Dual<NP> operator*(float a, const Dual<NP>& b) {
  Dual<NP> r; r.v = a * b.v;
#pragma unroll
  for (int i = 0; i < NP; i++) r.d[i] = a * b.d[i];
  return r;
}
template <int NP> DEGPU_DEV Dual<NP> operator*(const Dual<NP>& b, float a) {
  Dual<NP> r; r.v = b.v * a;
#pragma unroll
  for (int i = 0; i < NP; i++) r.d[i] = b.d[i] * a;
  return r;
}
template <int NP> DEGPU_DEV Dual<NP> operator/(const Dual<NP>& b, float a) {
  Dual<NP> r; r.v = b.v / a;
#pragma unroll
  for (int i = 0; i < NP; i++) r.d[i] = b.d[i] / a;
  return r;
}
template <int NP> DEGPU_DEV Dual<NP> operator+(float a, const Dual<NP>& b) { Dual<NP> r = b; r.v = a + b.v; return r; }
template <int NP> DEGPU_DEV Dual<NP> operator+(const Dual<NP>& b, float a) { Dual<NP> r = b; r.v = b.v + a; return r; }
template <int NP> DEGPU_DEV Dual<NP> operator-(float a, const Dual<NP>& b) {
  Dual<NP> r; r.v = a - b.v;
#pragma unroll
  for (int i = 0; i < NP; i++) r.d[i] = -b.d[i];
  return r;
}
template <int NP> DEGPU_DEV Dual<NP> operator-(const Dual<NP>& b, float a) { Dual<NP> r = b; r.v = b.v - a; return r; }

// elementary functions usable inside right-hand sides (value + chain rule)
DEGPU_DEV float dsin(float x) { return sinf(x); }
DEGPU_DEV float dcos(float x) { return cosf(x); }
DEGPU_DEV float dexp(float x) { return expf(x); }
template <int NP> DEGPU_DEV Dual<NP> dsin(const Dual<NP>& a) {
  Dual<NP> r; r.v = sinf(a.v); float c = cosf(a.v);
#pragma unroll
  for (int i = 0; i < NP; i++) r.d[i] = a.d[i] * c;
  return r;
}
template <int NP> DEGPU_DEV Dual<NP> dcos(const Dual<NP>& a) {
  Dual<NP> r; r.v = cosf(a.v); float s = -sinf(a.v);
#pragma unroll
  for (int i = 0; i < NP; i++) r.d[i] = a.d[i] * s;
  return r;
}
template <int NP> DEGPU_DEV Dual<NP> dexp(const Dual<NP>& a) {
  Dual<NP> r; r.v = expf(a.v);
#pragma unroll
  for (int i = 0; i < NP; i++) r.d[i] = a.d[i] * r.v;
  return r;
}

// ------------------------------------------------------------------ portable math
// Bit-reproducible log / exp / pow / sincos built from IEEE +,-,*,/ and exact bit
// manipulation (range reduction + atanh and Taylor series, Muller "Elementary
// Functions" ch. 6).  Parity mode uses them so that the controller's `EEst^beta1`
// and the EM normals match a strict-IEEE CPU evaluation bit for bit.
DEGPU_DEV float pm_logf(float x) {
  int e = 0;
  if (x < 1.17549435e-38f) { x = x * 16777216.0f; e = -24; }
  uint32_t b = __float_as_uint(x);
  e += (int)((b >> 23) & 0xff) - 127;
  float m = __uint_as_float((b & 0x007fffffu) | 0x3f800000u);
  if (m > 1.41421356f) { m = m * 0.5f; e += 1; }
  float s = (m - 1.0f) / (m + 1.0f);
  float s2 = s * s;
  float poly = 1.0f / 13.0f;
  poly = poly * s2 + 1.0f / 11.0f;
  poly = poly * s2 + 1.0f / 9.0f;
  poly = poly * s2 + 1.0f / 7.0f;
  poly = poly * s2 + 1.0f / 5.0f;
  poly = poly * s2 + 1.0f / 3.0f;
  poly = poly * s2 + 1.0f;
  float lnm = 2.0f * s * poly;
  float ef = (float)e;
  return ef * 0.693145752f + (ef * 1.42860677e-06f + lnm);
}
DEGPU_DEV float pm_expf(float y) {
  if (y > 88.7f) return __uint_as_float(0x7f800000u);
  if (y < -103.0f) return 0.0f;
  float t = y * 1.44269504f;
  int n = (int)(t >= 0.0f ? t + 0.5f : t - 0.5f);
  float nf = (float)n;
  float r = (y - nf * 0.693145752f) - nf * 1.42860677e-06f;
  float p = 1.0f / 362880.0f;
  p = p * r + 1.0f / 40320.0f;
  p = p * r + 1.0f / 5040.0f;
  p = p * r + 1.0f / 720.0f;
  p = p * r + 1.0f / 120.0f;
  p = p * r + 1.0f / 24.0f;
  p = p * r + 1.0f / 6.0f;
  p = p * r + 0.5f;
  p = p * r + 1.0f;
  p = p * r + 1.0f;
  int n1 = n / 2, n2 = n - n1;
  float s1 = __uint_as_float((uint32_t)(n1 + 127) << 23);
  float s2 = __uint_as_float((uint32_t)(n2 + 127) << 23);
  return (p * s1) * s2;
}
DEGPU_DEV float pm_powf(float x, float y) {
  if (x == 0.0f) return 0.0f;
  if (!(x == x)) return x;
  if (x > 3.40282347e38f) return x;
  return pm_expf(y * pm_logf(x));
}
DEGPU_DEV void pm_sincos_turns(float v, float* s, float* c) {
  float w = v >= 0.5f ? v - 1.0f : v;
  float w4 = w * 4.0f;
  int q = (int)(w4 >= 0.0f ? w4 + 0.5f : w4 - 0.5f);
  float r = (w4 - (float)q) * 1.57079633f;
  float r2 = r * r;
  float sp = -1.0f / 39916800.0f;
  sp = sp * r2 + 1.0f / 362880.0f;
  sp = sp * r2 - 1.0f / 5040.0f;
  sp = sp * r2 + 1.0f / 120.0f;
  sp = sp * r2 - 1.0f / 6.0f;
  sp = sp * r2 + 1.0f;
  float sr = r * sp;
  float cp = 1.0f / 3628800.0f;
  cp = cp * r2 - 1.0f / 40320.0f;
  cp = cp * r2 + 1.0f / 720.0f;
  cp = cp * r2 - 1.0f / 24.0f;
  cp = cp * r2 + 0.5f;
  float cr = 1.0f - r2 * cp;
  int qm = q & 3;
  if (qm == 0) { *s = sr; *c = cr; }
  else if (qm == 1) { *s = cr; *c = -sr; }
  else if (qm == 2) { *s = -sr; *c = -cr; }
  else { *s = -cr; *c = sr; }
}

// Julia's Base.min/max for floats propagate NaN (fminf/fmaxf would drop it).  Parity mode
// keeps that; fast mode uses the single-instruction min/max: a NaN state then reaches the
// end of the span with finite step sizes instead of a NaN step size, and still ends with
// retcode Unstable.
#if DEGPU_PARITY
DEGPU_DEV float jl_min(float x, float y) { if (x != x) return x; if (y != y) return y; return y < x ? y : x; }
DEGPU_DEV float jl_max(float x, float y) { if (x != x) return x; if (y != y) return y; return y > x ? y : x; }
#else
DEGPU_DEV float jl_min(float x, float y) { return fminf(x, y); }
DEGPU_DEV float jl_max(float x, float y) { return fmaxf(x, y); }
#endif
DEGPU_DEV double jl_mind(double x, double y) { if (x != x) return x; if (y != y) return y; return y < x ? y : x; }

}  // namespace degpu

using degpu::Dual;
using degpu::dsin;
using degpu::dcos;
using degpu::dexp;

// ------------------------------------------------------------------ callbacks (user side)
// The affect functions of GPUContinuousCallback / GPUDiscreteCallback
// (src/ensemblegpukernel/callbacks.jl) receive the fields of the integrator that the
// reference's affects use: the state (modifiable in place), the parameters, the time, the
// step, and terminate! (integrator_utils.jl:52-65).  degpu_time is the time type of the
// solve (float for a Float32 tspan, double for FP64 time).
typedef DEGPU_TT degpu_time;
struct degpu_integrator {
  float* u;
  const float* p;
  degpu_time t;
  float dt;
  int terminated;
};
__device__ __forceinline__ void degpu_terminate(degpu_integrator& I) { I.terminated = 1; }
