// degpu-model: lorenz_addnoise 3 3 4
// Lorenz drift with additive diagonal noise 3 (test/gpu_kernel_de/gpu_sde_regression.jl:47-58)
template <class T>
__device__ __forceinline__ void degpu_f(T* du, const T* u, const float* p, T t) {
  du[0] = p[0] * (u[1] - u[0]);
  du[1] = u[0] * (p[1] - u[2]) - u[1];
  du[2] = u[0] * u[1] - p[2] * u[2];
}
template <class T>
__device__ __forceinline__ void degpu_g(T* g, const T* u, const float* p, T t) {
  g[0] = 3.0f; g[1] = 3.0f; g[2] = 3.0f;
}
