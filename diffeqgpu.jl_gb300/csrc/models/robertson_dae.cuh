// degpu-model: robertson_dae 3 3 8
// Robertson kinetics as a semi-explicit DAE: the third equation is the conservation
// constraint y1 + y2 + y3 - 1 = 0 with a singular mass matrix diag(1, 1, 0)
// (test/gpu_kernel_de/stiff_ode/gpu_ode_mass_matrix.jl:5-31); p = (k1, k2, k3).
template <class T>
__device__ __forceinline__ void degpu_f(T* du, const T* u, const float* p, T t) {
  du[0] = -p[0] * u[0] + p[2] * u[1] * u[2];
  du[1] = p[0] * u[0] - p[1] * (u[1] * u[1]) - p[2] * u[1] * u[2];
  du[2] = u[0] + u[1] + u[2] - 1.0f;
}
__device__ __forceinline__ void degpu_mass(float* M) {
  M[0] = 1.0f; M[1] = 0.0f; M[2] = 0.0f;
  M[3] = 0.0f; M[4] = 1.0f; M[5] = 0.0f;
  M[6] = 0.0f; M[7] = 0.0f; M[8] = 0.0f;
}
