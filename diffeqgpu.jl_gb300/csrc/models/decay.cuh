// degpu-model: decay 1 1 3
// u' = -p1 u with analytic Jacobian and time gradient
// (test/gpu_kernel_de/stiff_ode/gpu_ode_regression.jl:5-22)
template <class T>
__device__ __forceinline__ void degpu_f(T* du, const T* u, const float* p, T t) {
  du[0] = -p[0] * u[0];
}
__device__ __forceinline__ void degpu_jac(float* J, const float* u, const float* p, float t) { J[0] = -p[0]; }
__device__ __forceinline__ void degpu_tgrad(float* dT, const float* u, const float* p, float t) { dT[0] = 0.0f; }
// Discrete callbacks (test/gpu_kernel_de/gpu_ode_discrete_callbacks.jl:16-22, with tstops
// at the event times): fn 0 fires at t == 2.4 and fn 1 at t == 4.0, each adding 10 to u;
// fn 2 ends the trajectory once u < 1 (terminate!).  Times compare in Float32, which is
// exact for both time types.
__device__ __forceinline__ bool degpu_dcb_condition(int fn, const float* u, const float* p, degpu_time t) {
  if (fn == 0) return (float)t == 2.4f;
  if (fn == 1) return (float)t == 4.0f;
  return u[0] < 1.0f;
}
__device__ __forceinline__ void degpu_dcb_affect(int fn, degpu_integrator& I) {
  if (fn == 2) {
    degpu_terminate(I);
    return;
  }
  I.u[0] = I.u[0] + 10.0f;
}
