// degpu-model: decay 1 1 3
// u' = -p1 u with analytic Jacobian and time gradient
// (test/gpu_kernel_de/stiff_ode/gpu_ode_regression.jl:5-22)
template <class T>
__device__ __forceinline__ void degpu_f(T* du, const T* u, const float* p, T t) {
  du[0] = -p[0] * u[0];
}
__device__ __forceinline__ void degpu_jac(float* J, const float* u, const float* p, float t) { J[0] = -p[0]; }
__device__ __forceinline__ void degpu_tgrad(float* dT, const float* u, const float* p, float t) { dT[0] = 0.0f; }
