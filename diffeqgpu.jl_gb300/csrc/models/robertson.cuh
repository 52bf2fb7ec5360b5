// degpu-model: robertson 3 3 3
// Robertson chemical kinetics in ODE form (the kinetics of
// test/gpu_kernel_de/stiff_ode/gpu_ode_mass_matrix.jl), p = (k1, k2, k3):
//   y1' = -k1 y1 + k3 y2 y3,  y2' = k1 y1 - k2 y2^2 - k3 y2 y3,  y3' = k2 y2^2
template <class T>
__device__ __forceinline__ void degpu_f(T* du, const T* u, const float* p, T t) {
  du[0] = -p[0] * u[0] + p[2] * u[1] * u[2];
  du[1] = p[0] * u[0] - p[1] * u[1] * u[1] - p[2] * u[1] * u[2];
  du[2] = p[1] * u[1] * u[1];
}
__device__ __forceinline__ void degpu_jac(float* J, const float* u, const float* p, float t) {
  J[0] = -p[0]; J[1] = p[0]; J[2] = 0.0f;
  J[3] = p[2] * u[2]; J[4] = -(p[1] * u[1] + p[1] * u[1]) - p[2] * u[2]; J[5] = p[1] * u[1] + p[1] * u[1];
  J[6] = p[2] * u[1]; J[7] = -(p[2] * u[1]); J[8] = 0.0f;
}
__device__ __forceinline__ void degpu_tgrad(float* dT, const float* u, const float* p, float t) {
  dT[0] = 0.0f; dT[1] = 0.0f; dT[2] = 0.0f;
}
