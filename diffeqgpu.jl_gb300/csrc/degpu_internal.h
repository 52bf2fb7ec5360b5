// Internal entry points shared between the host library's translation units (not part of
// the public C ABI in include/degpu.h).
#pragma once
#include "degpu.h"

// State and parameter dimensions of a registered right-hand side.
int degpu_internal_rhs_dims(const degpu_rhs* f, int* n_state, int* n_param);
// Record an error message for degpu_last_error() and return `code`.
int degpu_internal_fail(int code, const char* msg);
// Stream-ordered device scratch from the library's memory pool (free with cudaFreeAsync).
int degpu_internal_alloc(void** p, size_t n, void* stream);
// degpu_vectorized_asolve with a caller-provided persistent-driver work counter (8 bytes of
// device memory, zeroed on the stream before the launch) instead of one from the
// stream-ordered allocator.
int degpu_internal_asolve_with_work(const degpu_rhs* f, const degpu_problems* probs, const degpu_options* opt,
                                    degpu_outputs* out, unsigned long long* work, void* stream);
// degpu_mlp_infer_problems whose model may take one more feature after log10 reltol: the
// span tf - t0 of each trajectory's tspan [B][2] (FP64 when tspan_f64, else FP32), used
// when the model's input width is n_state + n_param + 2.
int degpu_internal_mlp_infer_problems(const degpu_mlp* m, const float* u0, int n_state, const float* p, int n_param,
                                      const void* tspan, int tspan_f64, float reltol, long long B, float* dt0,
                                      float* tolscale, float dt_lo, float dt_hi, float s_lo, float s_hi, void* stream);
