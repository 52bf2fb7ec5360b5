// Learned-controller solve for callers that cannot allocate device memory.
//
// Some callers of this library must not call cudaMalloc (or any allocator) while they
// solve: code that runs inside a host callback or a library with a fixed memory budget,
// real-time loops that may not enter the driver's allocator, and runtimes that own all
// device memory themselves.  degpu_learned_asolve needs scratch memory besides the
// caller's inputs and outputs -- the per-trajectory initial step and tolerance scale the
// step-size model writes for the solver (8 bytes per trajectory) and the persistent
// driver's work counter -- and takes it from the stream-ordered allocator.  The variant
// below takes it instead from one fixed array that lives in this library's device image,
// sized for DEGPU_NOALLOC_MAX_TRAJECTORIES trajectories per call (2 MiB + 256 bytes, held
// by every GPU that loads the library until the process exits).
//
// Sharing rules: every call uses the same array, which keeps the previous call's
// contents.  The work counter is cleared on the stream before each solve and the model
// writes every dt0/scale entry the solve reads, so stale contents never leak into a
// result; but two calls whose work overlaps on the GPU (different streams, or different
// host threads on one device) race on the array and must be serialised by the caller.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "degpu.h"
#include "degpu_internal.h"

namespace {

constexpr long long kMaxTraj = DEGPU_NOALLOC_MAX_TRAJECTORIES;
constexpr size_t kCounterBytes = 256;  // work counter, padded to the array's alignment

// [0, 256): persistent-driver work counter | dt0 [kMaxTraj] f32 | tolerance scale [kMaxTraj] f32
static __device__ __align__(256) unsigned char g_noalloc_scratch[kCounterBytes + 8 * kMaxTraj];

std::mutex g_mu;
void* g_addr[64] = {};  // device address of g_noalloc_scratch, per device

// Set-up, once per device with that device current: the array's name is a host-side
// stand-in, so its device address must come from cudaGetSymbolAddress.
int scratch_address(char** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return degpu_internal_fail(DEGPU_E_CUDA, "cudaGetDevice failed");
  if (dev < 0 || dev >= 64) return degpu_internal_fail(DEGPU_E_UNSUPPORTED, "device index >= 64");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      return degpu_internal_fail(DEGPU_E_CUDA, (std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") +
                                                cudaGetErrorString(e)).c_str());
    }
    g_addr[dev] = p;
  }
  *out = static_cast<char*>(g_addr[dev]);
  return 0;
}

}  // namespace

extern "C" int degpu_learned_asolve_noalloc(const degpu_rhs* f, const degpu_mlp* m, const degpu_problems* probs,
                                            const degpu_options* opt, float dt_lo, float dt_hi, float s_max,
                                            degpu_outputs* out, void* stream) {
  if (!f || !m || !probs || !opt || !out) return degpu_internal_fail(DEGPU_E_INVALID, "null argument");
  if (probs->B < 0) return degpu_internal_fail(DEGPU_E_INVALID, "negative trajectory count");
  if (probs->B > kMaxTraj)
    return degpu_internal_fail(DEGPU_E_INVALID,
                               "degpu_learned_asolve_noalloc: more than DEGPU_NOALLOC_MAX_TRAJECTORIES (262144) "
                               "trajectories in one call; split the ensemble into batches of at most 262144");
  if (probs->B == 0) return 0;
  if (!(s_max >= 1.0f) || !(dt_lo > 0.0f) || !(dt_hi >= dt_lo))
    return degpu_internal_fail(DEGPU_E_INVALID, "bad dt / scale clamp");
  int n_state = 0, n_param = 0;
  int rc = degpu_internal_rhs_dims(f, &n_state, &n_param);
  if (rc) return rc;
  char* base = nullptr;
  rc = scratch_address(&base);
  if (rc) return rc;
  unsigned long long* work = reinterpret_cast<unsigned long long*>(base);
  float* dt0 = reinterpret_cast<float*>(base + kCounterBytes);
  float* tolscale = dt0 + probs->B;
  rc = degpu_mlp_infer_problems(m, probs->u0, n_state, probs->p, n_param, (float)opt->reltol, probs->B, dt0, tolscale,
                                dt_lo, dt_hi, 1.0f, s_max, stream);
  if (rc) return degpu_internal_fail(rc, "step-size model inference failed (does the model's input width match N + P + 1?)");
  degpu_options o = *opt;
  o.dt0 = dt0;
  o.tolscale = tolscale;
  o.order = nullptr;  // ignored, as in degpu_learned_asolve
  return degpu_internal_asolve_with_work(f, probs, &o, out, work, stream);
}
