// degpu-model: ball 2 1 0
// Bouncing ball, u = (height, velocity), gravity p1 (test/gpu_kernel_de/gpu_ode_continuous_callbacks.jl:6-26)
template <class T>
__device__ __forceinline__ void degpu_f(T* du, const T* u, const float* p, T t) {
  du[0] = u[1];
  du[1] = T(-p[0]);
}
// Continuous callbacks.  fn 0: bounce -- the event is the height crossing zero and
// affect! reverses the velocity, u += (0, -2) .* u (the reference test's affect!); it is
// also the affect_neg!.  fn 1: the first ground contact ends the trajectory (terminate!).
__device__ __forceinline__ float degpu_ccb_condition(int fn, const float* u, const float* p, degpu_time t) {
  return u[0];
}
__device__ __forceinline__ void degpu_ccb_affect(int fn, degpu_integrator& I) {
  if (fn == 1) {
    degpu_terminate(I);
    return;
  }
  I.u[0] = I.u[0] + 0.0f * I.u[0];
  I.u[1] = I.u[1] + -2.0f * I.u[1];
}
__device__ __forceinline__ void degpu_ccb_affect_neg(int fn, degpu_integrator& I) { degpu_ccb_affect(fn, I); }
