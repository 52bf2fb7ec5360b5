// degpu-model: linear15 15 1 0
// u' = 1.01 u in 15 dimensions (test/gpu_kernel_de/stiff_ode/gpu_ode_regression.jl:24-29),
// exercises the N > 3 linear-solve path
template <class T>
__device__ __forceinline__ void degpu_f(T* du, const T* u, const float* p, T t) {
#pragma unroll
  for (int i = 0; i < 15; i++) du[i] = 1.01f * u[i];
}
