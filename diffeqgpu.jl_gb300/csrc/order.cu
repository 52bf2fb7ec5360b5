// Longest-first visiting order for the persistent driver (no counterpart in the reference).
//
// The persistent driver refills a lane as soon as its trajectory ends, so lanes stay busy
// until the work queue runs dry; from then on every warp drains its last 32 trajectories
// and runs with fewer and fewer active lanes.  On an adaptive ensemble whose step counts
// vary several-fold that drain is a sizeable share of the solve.  Visiting the longest
// trajectories first leaves only short ones for the drain.  The order comes from a
// per-trajectory work estimate (the learned work model's predicted attempts): a counting
// sort into 128 quarter-octave classes of the estimate, highest class first.
//
//   work_hist_kernel     class histogram (shared-memory counts, one global add per class)
//   work_scan_kernel     class offsets, highest class first (one block)
//   work_scatter_kernel  order[offset(class) + rank within class] = trajectory; per tile
//                        one global add per class reserves the tile's slots
// Three launches, ~12 bytes of HBM traffic per trajectory.
#include <cuda_runtime.h>

#include "degpu.h"
#include "degpu_internal.h"

namespace {

constexpr int NCLS = 128;    // quarter-octaves of the work estimate: 2^0 .. 2^32
constexpr int THREADS = 256;
constexpr int ITEMS = 8;     // trajectories per thread and tile
constexpr int TILE = THREADS * ITEMS;

// rank of a work estimate's class, 0 = the largest estimates
__device__ __forceinline__ int class_rank(float w) {
  int c = 0;
  if (w >= 1.0f) {  // false for NaN
    const float q = 4.0f * __log2f(w);
    c = q < (float)(NCLS - 1) ? (int)q : NCLS - 1;
  }
  return NCLS - 1 - c;
}

__global__ void __launch_bounds__(THREADS) work_hist_kernel(const float* __restrict__ work, long long B, int* __restrict__ hist) {
  __shared__ int h[NCLS];
  for (int c = threadIdx.x; c < NCLS; c += blockDim.x) h[c] = 0;
  __syncthreads();
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < B; i += (long long)gridDim.x * blockDim.x)
    atomicAdd(&h[class_rank(work[i])], 1);
  __syncthreads();
  for (int c = threadIdx.x; c < NCLS; c += blockDim.x)
    if (h[c]) atomicAdd(&hist[c], h[c]);
}

// exclusive prefix sum over the class ranks (one block of NCLS threads)
__global__ void __launch_bounds__(NCLS) work_scan_kernel(const int* __restrict__ hist, int* __restrict__ cursor) {
  __shared__ int s[NCLS];
  const int c = threadIdx.x;
  s[c] = hist[c];
  __syncthreads();
  for (int off = 1; off < NCLS; off <<= 1) {
    const int v = c >= off ? s[c - off] : 0;
    __syncthreads();
    s[c] += v;
    __syncthreads();
  }
  cursor[c] = s[c] - hist[c];
}

__global__ void __launch_bounds__(THREADS) work_scatter_kernel(const float* __restrict__ work, long long B,
                                                                int* __restrict__ cursor, int* __restrict__ order) {
  __shared__ int cnt[NCLS], base[NCLS];
  for (long long t0 = (long long)blockIdx.x * TILE; t0 < B; t0 += (long long)gridDim.x * TILE) {
    for (int c = threadIdx.x; c < NCLS; c += blockDim.x) cnt[c] = 0;
    __syncthreads();
    int cls[ITEMS], pos[ITEMS];
#pragma unroll
    for (int j = 0; j < ITEMS; j++) {
      const long long i = t0 + (long long)j * THREADS + threadIdx.x;  // coalesced reads
      cls[j] = -1;
      if (i < B) {
        cls[j] = class_rank(work[i]);
        pos[j] = atomicAdd(&cnt[cls[j]], 1);
      }
    }
    __syncthreads();
    for (int c = threadIdx.x; c < NCLS; c += blockDim.x) base[c] = cnt[c] ? atomicAdd(&cursor[c], cnt[c]) : 0;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < ITEMS; j++)
      if (cls[j] >= 0) order[base[cls[j]] + pos[j]] = (int)(t0 + (long long)j * THREADS + threadIdx.x);
    __syncthreads();
  }
}

int sm_count_here() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

}  // namespace

extern "C" int degpu_work_order(const float* work, long long B, int* order, void* stream) {
  if (B < 0) return degpu_internal_fail(DEGPU_E_INVALID, "negative trajectory count");
  if (B > 0x7fffffffLL) return degpu_internal_fail(DEGPU_E_INVALID, "more than 2^31-1 trajectories in one call");
  if (B == 0) return 0;
  if (!work || !order) return degpu_internal_fail(DEGPU_E_INVALID, "null device buffer");
  cudaStream_t s = (cudaStream_t)stream;
  int* scratch = nullptr;  // hist [NCLS], cursor [NCLS]
  int rc = degpu_internal_alloc((void**)&scratch, 2 * NCLS * sizeof(int), stream);
  if (rc) return rc;
  cudaError_t e = cudaMemsetAsync(scratch, 0, NCLS * sizeof(int), s);
  const long long tiles = (B + TILE - 1) / TILE;
  const int grid = (int)(tiles < 4LL * sm_count_here() ? tiles : 4LL * sm_count_here());
  if (e == cudaSuccess) {
    work_hist_kernel<<<grid, THREADS, 0, s>>>(work, B, scratch);
    work_scan_kernel<<<1, NCLS, 0, s>>>(scratch, scratch + NCLS);
    work_scatter_kernel<<<grid, THREADS, 0, s>>>(work, B, scratch + NCLS, order);
    e = cudaGetLastError();
  }
  cudaFreeAsync(scratch, s);
  if (e != cudaSuccess) return degpu_internal_fail(DEGPU_E_CUDA, cudaGetErrorString(e));
  return 0;
}
