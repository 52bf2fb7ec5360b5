// degpu-model: gbm 1 2 4
// geometric Brownian motion du = p1 u dt + p2 u dW (test/gpu_kernel_de/gpu_sde_convergence.jl:6-8)
template <class T>
__device__ __forceinline__ void degpu_f(T* du, const T* u, const float* p, T t) {
  du[0] = p[0] * u[0];
}
template <class T>
__device__ __forceinline__ void degpu_g(T* g, const T* u, const float* p, T t) {
  g[0] = p[1] * u[0];
}
