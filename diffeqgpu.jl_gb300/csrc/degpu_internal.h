// Internal entry points shared between the host library's translation units (not part of
// the public C ABI in include/degpu.h).
#pragma once
#include "degpu.h"

// State and parameter dimensions of a registered right-hand side.
int degpu_internal_rhs_dims(const degpu_rhs* f, int* n_state, int* n_param);
// Record an error message for degpu_last_error() and return `code`.
int degpu_internal_fail(int code, const char* msg);
// degpu_vectorized_asolve with a caller-provided persistent-driver work counter (8 bytes of
// device memory, zeroed on the stream before the launch) instead of one from the
// stream-ordered allocator.
int degpu_internal_asolve_with_work(const degpu_rhs* f, const degpu_problems* probs, const degpu_options* opt,
                                    degpu_outputs* out, unsigned long long* work, void* stream);
