// degpu-model: osc 2 1 3
// harmonic oscillator u1' = u2, u2' = -w^2 u1 (p = w): a non-chaotic known-answer problem
template <class T>
__device__ __forceinline__ void degpu_f(T* du, const T* u, const float* p, T t) {
  du[0] = u[1];
  du[1] = -(p[0] * p[0]) * u[0];
}
__device__ __forceinline__ void degpu_jac(float* J, const float* u, const float* p, float t) {
  J[0] = 0.0f; J[1] = -(p[0] * p[0]); J[2] = 1.0f; J[3] = 0.0f;
}
__device__ __forceinline__ void degpu_tgrad(float* dT, const float* u, const float* p, float t) { dT[0] = 0.0f; dT[1] = 0.0f; }
