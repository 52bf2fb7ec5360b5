// degpu-model: growth 1 1 0
// u' = u (test/public_interface.jl:9-11)
template <class T>
__device__ __forceinline__ void degpu_f(T* du, const T* u, const float* p, T t) {
  du[0] = u[0];
}
