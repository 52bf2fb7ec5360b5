// degpu-model: lorenz 3 3 0
// Lorenz system, the reference's regression problem (test/gpu_kernel_de/gpu_ode_regression.jl:4-12):
//   du1 = s (u2 - u1),  du2 = u1 (r - u3) - u2,  du3 = u1 u2 - b u3,   p = (s, r, b)
template <class T>
__device__ __forceinline__ void degpu_f(T* du, const T* u, const float* p, T t) {
  du[0] = p[0] * (u[1] - u[0]);
  du[1] = u[0] * (p[1] - u[2]) - u[1];
  du[2] = u[0] * u[1] - p[2] * u[2];
}
