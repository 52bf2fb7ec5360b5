// Learned step control: a small BF16 MLP  x (n_in <= 16) -> 64 SiLU -> 64 SiLU -> 2
// predicting, per trajectory, log(initial dt) and log(tolerance scale) from (u0, p, log tol).
// No counterpart in the reference (its controller starts every trajectory from the user's
// dt and the same tolerances); the embedded error estimate still accepts or rejects every
// step, so the plain controller remains the judge of every step.
//
// Numerics (the same rounding points in inference and training, quantisation-aware):
//   xn = bf16((x - mean) / std);  z1 = W1q xn + b1;  h1 = bf16(silu(z1));
//   z2 = W2q h1 + b2;  h2 = bf16(silu(z2));  y = W3q h2 + b3      (Wq = bf16(W), fp32 accumulate)
// Inference runs on the tensor cores (mma.sync m16n8k16, bf16 in, fp32 accumulate: the
// layers are 16-64 wide, far below a tcgen05 tile).  Its 128 activations per trajectory
// would otherwise bound it on the special-function unit (a quarter of the FP32 rate): SiLU
// there is z/2 + z/2 tanh(z/2) with the hardware tanh (one SFU op, relative error below
// 2^-10, ahead of the bf16 rounding of h), ~0.07 ms per 10^6 trajectories.  Training is
// FP32 SIMT with the exp/reciprocal logistic: forward with the same bf16 rounding points,
// backward with straight-through rounding, weight gradients as per-tile shared-memory
// GEMMs, Adam.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>

#include "degpu.h"
#include "degpu_internal.h"

namespace {

constexpr int H = DEGPU_MLP_HIDDEN;  // 64
constexpr int KIN = 16;              // padded input width
constexpr int NOUT = DEGPU_MLP_OUT;  // 2

// packed FP32 parameter vector: W1 [H][n_in], b1 [H], W2 [H][H], b2 [H], W3 [NOUT][H], b3 [NOUT]
struct Layout {
  int n_in, oW1, ob1, oW2, ob2, oW3, ob3, count;
  __host__ __device__ explicit Layout(int n) : n_in(n) {
    oW1 = 0; ob1 = oW1 + H * n; oW2 = ob1 + H; ob2 = oW2 + H * H; oW3 = ob2 + H; ob3 = oW3 + NOUT * H;
    count = ob3 + NOUT;
  }
};

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }
// logistic function with the SFU's exp2 and reciprocal (a few ulp; the hidden activations
// are rounded to bf16 right after, and training and inference share this function).  For
// z < -87 the denominator overflows and the quotient is 0, the limit.
__device__ __forceinline__ float sigm(float z) { return __fdividef(1.0f, 1.0f + __expf(-z)); }
__device__ __forceinline__ float silu(float z) { return z * sigm(z); }
// inference activation: z sigma(z) = h + h tanh(h), h = z/2, with tanh.approx.f32 (PTX ISA,
// sm_75 and later)
__device__ __forceinline__ float silu_fast(float z) {
  const float h = 0.5f * z;
  float t;
  asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(h));
  return fmaf(h, t, h);
}
__device__ __forceinline__ float dsilu(float z) { float s = sigm(z); return s + z * s * (1.0f - s); }

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}

// D (16x8, f32) += A (16x16, bf16, row) * B (16x8, bf16, col)
__device__ __forceinline__ void mma16816(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// ------------------------------------------------------------------ inference (tensor cores)
// One warp per tile of 16 trajectories; weights staged once per CTA in shared memory as
// bf16 [out][in] rows, which is exactly the "col" B-operand layout of mma.m16n8k16.
// Rows are padded by 8 bf16 (16 bytes): a warp's B-fragment load reads row g = lane / 4,
// column pair tig = lane % 4 of eight consecutive rows, and with unpadded 128-byte W2 rows
// all eight rows start in the same bank (an 8-way conflict on every load); with 144-byte
// (W2, W3) and 48-byte (W1) rows the 32 lanes hit 32 different banks.
constexpr int WPAD = 8;
struct InferSmem {
  __nv_bfloat16 W1[H][KIN + WPAD];
  __nv_bfloat16 W2[H][H + WPAD];
  __nv_bfloat16 W3[8][H + WPAD];  // rows >= NOUT are zero
  float b1[H], b2[H], b3[8];
  float mean[KIN], rstd[KIN];
};

// Features come either from x [B][n_in] or, when x is null, straight from the problem batch:
// (u0 [B][Nu], p [B][Np], logtol), n_in = Nu + Np + 1, optionally followed by the span
// tf - t0 of the trajectory's tspan [B][2] (n_in = Nu + Np + 2; FP64 or FP32 tspan).
struct FeatSrc {
  const float* x;
  const float* u0;
  const float* p;
  int Nu, Np;
  float logtol;
  const void* tspan;
  int tspan_f64;
};

__global__ void __launch_bounds__(128) mlp_infer_kernel(const float* __restrict__ P, int n_in, const float* __restrict__ mean,
                                                        const float* __restrict__ stdv, const FeatSrc src, long long B,
                                                        float* __restrict__ y, float* __restrict__ dt0, float* __restrict__ tsc,
                                                        float dt_lo, float dt_hi, float s_lo, float s_hi) {
  __shared__ InferSmem S;
  const Layout Lo(n_in);
  for (int i = threadIdx.x; i < H * KIN; i += blockDim.x) {
    int o = i / KIN, k = i % KIN;
    S.W1[o][k] = __float2bfloat16_rn(k < n_in ? P[Lo.oW1 + o * n_in + k] : 0.0f);
  }
  for (int i = threadIdx.x; i < H * H; i += blockDim.x) S.W2[i / H][i % H] = __float2bfloat16_rn(P[Lo.oW2 + i]);
  for (int i = threadIdx.x; i < 8 * H; i += blockDim.x) {
    int o = i / H, k = i % H;
    S.W3[o][k] = __float2bfloat16_rn(o < NOUT ? P[Lo.oW3 + o * H + k] : 0.0f);
  }
  for (int i = threadIdx.x; i < H; i += blockDim.x) { S.b1[i] = P[Lo.ob1 + i]; S.b2[i] = P[Lo.ob2 + i]; }
  for (int i = threadIdx.x; i < 8; i += blockDim.x) S.b3[i] = i < NOUT ? P[Lo.ob3 + i] : 0.0f;
  for (int i = threadIdx.x; i < KIN; i += blockDim.x) {
    S.mean[i] = i < n_in ? mean[i] : 0.0f;
    S.rstd[i] = i < n_in ? 1.0f / stdv[i] : 0.0f;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
  const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
  const long long ntiles = (B + 15) / 16;
  // raw feature k of row r (unnormalised); 0 outside the batch and the input width
  auto raw = [&](long long r, int k) -> float {
    if (r >= B || k >= n_in) return 0.0f;
    if (src.x) return src.x[r * n_in + k];
    if (k < src.Nu) return src.u0[r * src.Nu + k];
    if (k < src.Nu + src.Np) return src.p[r * src.Np + (k - src.Nu)];
    if (k == src.Nu + src.Np) return src.logtol;
    if (src.tspan_f64) return (float)(((const double*)src.tspan)[2 * r + 1] - ((const double*)src.tspan)[2 * r]);
    return ((const float*)src.tspan)[2 * r + 1] - ((const float*)src.tspan)[2 * r];
  };
  // this lane's 8 A-fragment features of a tile: rows g and g + 8, columns 2 tig + {0, 1, 8, 9}
  auto load_tile = [&](long long tile, float* f) {
    const long long r0 = tile * 16 + g, r1 = r0 + 8;
    f[0] = raw(r0, tig * 2); f[1] = raw(r0, tig * 2 + 1); f[2] = raw(r1, tig * 2); f[3] = raw(r1, tig * 2 + 1);
    f[4] = raw(r0, tig * 2 + 8); f[5] = raw(r0, tig * 2 + 9); f[6] = raw(r1, tig * 2 + 8); f[7] = raw(r1, tig * 2 + 9);
  };
  const int c0 = tig * 2, c1 = tig * 2 + 1, c8 = tig * 2 + 8, c9 = tig * 2 + 9;
  const float m0 = S.mean[c0], m1 = S.mean[c1], m8 = S.mean[c8], m9 = S.mean[c9];
  const float s0 = S.rstd[c0], s1 = S.rstd[c1], s8 = S.rstd[c8], s9 = S.rstd[c9];
  long long tile = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  float fnext[8];
  if (tile < ntiles) load_tile(tile, fnext);
  for (; tile < ntiles; tile += warps) {
    const long long r0 = tile * 16 + g, r1 = r0 + 8;
    // the next tile's features are loaded before this tile's layers run (their global-memory
    // latency overlaps the tensor-core and activation work)
    float f[8];
#pragma unroll
    for (int j = 0; j < 8; j++) f[j] = fnext[j];
    if (tile + warps < ntiles) load_tile(tile + warps, fnext);
    uint32_t a[4];
    a[0] = pack_bf16((f[0] - m0) * s0, (f[1] - m1) * s1);
    a[1] = pack_bf16((f[2] - m0) * s0, (f[3] - m1) * s1);
    a[2] = pack_bf16((f[4] - m8) * s8, (f[5] - m9) * s9);
    a[3] = pack_bf16((f[6] - m8) * s8, (f[7] - m9) * s9);
    // layer 1: 8 n-tiles of 8 outputs
    float h[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      // the accumulator starts at the bias (z = b + W x, the training kernel's order)
      const float bb0 = S.b1[nt * 8 + tig * 2], bb1 = S.b1[nt * 8 + tig * 2 + 1];
      h[nt][0] = bb0; h[nt][1] = bb1; h[nt][2] = bb0; h[nt][3] = bb1;
      const __nv_bfloat16* w = &S.W1[nt * 8 + g][0];
      mma16816(h[nt], a, *reinterpret_cast<const uint32_t*>(w + tig * 2), *reinterpret_cast<const uint32_t*>(w + tig * 2 + 8));
      h[nt][0] = silu_fast(h[nt][0]); h[nt][1] = silu_fast(h[nt][1]);
      h[nt][2] = silu_fast(h[nt][2]); h[nt][3] = silu_fast(h[nt][3]);
    }
    // layer 2: accumulator fragments of layer 1 become the A fragments (k-tile kt = n-tiles 2kt, 2kt+1)
    uint32_t ha[4][4];
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
      ha[kt][0] = pack_bf16(h[2 * kt][0], h[2 * kt][1]);
      ha[kt][1] = pack_bf16(h[2 * kt][2], h[2 * kt][3]);
      ha[kt][2] = pack_bf16(h[2 * kt + 1][0], h[2 * kt + 1][1]);
      ha[kt][3] = pack_bf16(h[2 * kt + 1][2], h[2 * kt + 1][3]);
    }
    float h2[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      const float bb0 = S.b2[nt * 8 + tig * 2], bb1 = S.b2[nt * 8 + tig * 2 + 1];
      h2[nt][0] = bb0; h2[nt][1] = bb1; h2[nt][2] = bb0; h2[nt][3] = bb1;
      const __nv_bfloat16* w = &S.W2[nt * 8 + g][0];
#pragma unroll
      for (int kt = 0; kt < 4; kt++)
        mma16816(h2[nt], ha[kt], *reinterpret_cast<const uint32_t*>(w + kt * 16 + tig * 2),
                 *reinterpret_cast<const uint32_t*>(w + kt * 16 + tig * 2 + 8));
      h2[nt][0] = silu_fast(h2[nt][0]); h2[nt][1] = silu_fast(h2[nt][1]);
      h2[nt][2] = silu_fast(h2[nt][2]); h2[nt][3] = silu_fast(h2[nt][3]);
    }
    float o[4] = {S.b3[tig * 2], S.b3[tig * 2 + 1], S.b3[tig * 2], S.b3[tig * 2 + 1]};
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
      uint32_t a2[4] = {pack_bf16(h2[2 * kt][0], h2[2 * kt][1]), pack_bf16(h2[2 * kt][2], h2[2 * kt][3]),
                        pack_bf16(h2[2 * kt + 1][0], h2[2 * kt + 1][1]), pack_bf16(h2[2 * kt + 1][2], h2[2 * kt + 1][3])};
      const __nv_bfloat16* w = &S.W3[g][0];
      mma16816(o, a2, *reinterpret_cast<const uint32_t*>(w + kt * 16 + tig * 2),
               *reinterpret_cast<const uint32_t*>(w + kt * 16 + tig * 2 + 8));
    }
    if (tig == 0) {  // columns 0 and 1 live in lanes with tig == 0
      const float y00 = o[0], y01 = o[1], y10 = o[2], y11 = o[3];
      if (r0 < B) {
        if (y) { y[r0 * 2] = y00; y[r0 * 2 + 1] = y01; }
        if (dt0) dt0[r0] = fminf(fmaxf(__expf(y00), dt_lo), dt_hi);
        if (tsc) tsc[r0] = fminf(fmaxf(__expf(y01), s_lo), s_hi);
      }
      if (r1 < B) {
        if (y) { y[r1 * 2] = y10; y[r1 * 2 + 1] = y11; }
        if (dt0) dt0[r1] = fminf(fmaxf(__expf(y10), dt_lo), dt_hi);
        if (tsc) tsc[r1] = fminf(fmaxf(__expf(y11), s_lo), s_hi);
      }
    }
  }
}

// ------------------------------------------------------------------ training (FP32 SIMT)
constexpr int TT = 128;  // samples per tile == threads per block
constexpr int LD = H + 1;

__global__ void __launch_bounds__(TT) mlp_grad_kernel(const float* __restrict__ P, int n_in, const float* __restrict__ mean,
                                                      const float* __restrict__ stdv, const float* __restrict__ x,
                                                      const float* __restrict__ tgt, const float* __restrict__ wgt, long long B,
                                                      float inv_total, float* __restrict__ G, float* __restrict__ loss) {
  extern __shared__ float sm[];
  const Layout Lo(n_in);
  float* W2q = sm;                  // [H][H]
  float* W1q = W2q + H * H;         // [H][KIN]
  float* W3q = W1q + H * KIN;       // [NOUT][H]
  float* bia = W3q + NOUT * H;      // b1[H], b2[H], b3[NOUT], mean[KIN], rstd[KIN]
  float* H1 = bia + 2 * H + NOUT + 2 * KIN;  // [TT][LD] h1 (bf16-valued)
  float* G1 = H1 + TT * LD;          // [TT][LD] silu'(z1), later dz1
  float* H2 = G1 + TT * LD;          // [TT][LD] h2 (bf16-valued)
  float* DZ2 = H2 + TT * LD;         // [TT][LD]
  float* XQ = DZ2 + TT * LD;         // [TT][KIN+1]
  float* DY = XQ + TT * (KIN + 1);   // [TT][NOUT]
  const int t = threadIdx.x;
  for (int i = t; i < H * H; i += TT) W2q[i] = bf16r(P[Lo.oW2 + i]);
  for (int i = t; i < H * KIN; i += TT) { int o = i / KIN, k = i % KIN; W1q[i] = k < n_in ? bf16r(P[Lo.oW1 + o * n_in + k]) : 0.0f; }
  for (int i = t; i < NOUT * H; i += TT) W3q[i] = bf16r(P[Lo.oW3 + i]);
  for (int i = t; i < H; i += TT) { bia[i] = P[Lo.ob1 + i]; bia[H + i] = P[Lo.ob2 + i]; }
  if (t < NOUT) bia[2 * H + t] = P[Lo.ob3 + t];
  if (t < KIN) {
    bia[2 * H + NOUT + t] = t < n_in ? mean[t] : 0.0f;
    bia[2 * H + NOUT + KIN + t] = t < n_in ? 1.0f / stdv[t] : 0.0f;
  }
  __syncthreads();
  const float* b1 = bia;
  const float* b2 = bia + H;
  const float* b3 = bia + 2 * H;
  const float* mu = bia + 2 * H + NOUT;
  const float* rs = mu + KIN;
  // per-thread gradient accumulators: thread t owns dW2 rows j = t/2 (32 of its 64 columns),
  // dW1 row k = t/2 (8 of 16 columns), dW3 entry t, and one bias entry each
  float gW2[32], gW1[8], gW3 = 0.f, gb1 = 0.f, gb2 = 0.f, gb3 = 0.f, lsum = 0.f;
#pragma unroll
  for (int c = 0; c < 32; c++) gW2[c] = 0.f;
#pragma unroll
  for (int c = 0; c < 8; c++) gW1[c] = 0.f;
  const int jrow = t >> 1, half = t & 1;
  const long long ntiles = (B + TT - 1) / TT;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long m = tile * TT + t;
    const bool valid = m < B;
    // ---- forward (one sample per thread)
    float xq[KIN];
#pragma unroll
    for (int k = 0; k < KIN; k++) xq[k] = (valid && k < n_in) ? bf16r((x[m * n_in + k] - mu[k]) * rs[k]) : 0.0f;
#pragma unroll
    for (int k = 0; k < KIN; k++) XQ[t * (KIN + 1) + k] = xq[k];
    for (int j = 0; j < H; j++) {
      float z = b1[j];
#pragma unroll
      for (int k = 0; k < KIN; k++) z += W1q[j * KIN + k] * xq[k];
      H1[t * LD + j] = bf16r(silu(z));
      G1[t * LD + j] = dsilu(z);
    }
    float y[NOUT];
#pragma unroll
    for (int o = 0; o < NOUT; o++) y[o] = b3[o];
    for (int j = 0; j < H; j++) {
      float z = b2[j];
      for (int k = 0; k < H; k++) z += W2q[j * H + k] * H1[t * LD + k];
      float h2 = bf16r(silu(z));
      H2[t * LD + j] = h2;
      DZ2[t * LD + j] = dsilu(z);  // holds silu'(z2) until dy is known
#pragma unroll
      for (int o = 0; o < NOUT; o++) y[o] += W3q[o * H + j] * h2;
    }
    // ---- loss: weighted squared error, mean over the whole training set
    float dy[NOUT];
#pragma unroll
    for (int o = 0; o < NOUT; o++) {
      float w = valid ? (wgt ? wgt[m * NOUT + o] : 1.0f) : 0.0f;
      float r = valid ? (y[o] - tgt[m * NOUT + o]) : 0.0f;
      lsum += w * r * r * inv_total;
      dy[o] = 2.0f * w * r * inv_total;
      DY[t * NOUT + o] = dy[o];
    }
    for (int j = 0; j < H; j++) {
      float dh = 0.f;
#pragma unroll
      for (int o = 0; o < NOUT; o++) dh += dy[o] * W3q[o * H + j];
      DZ2[t * LD + j] = dh * DZ2[t * LD + j];
    }
    // dz1 = (dz2 W2) * silu'(z1), own sample
    for (int k = 0; k < H; k++) {
      float dh = 0.f;
      for (int j = 0; j < H; j++) dh += DZ2[t * LD + j] * W2q[j * H + k];
      G1[t * LD + k] = dh * G1[t * LD + k];
    }
    __syncthreads();
    // ---- weight gradients over the tile (shared-memory GEMMs, reduction over samples)
    for (int s = 0; s < TT; s++) {
      const float dz = DZ2[s * LD + jrow];
#pragma unroll
      for (int c = 0; c < 32; c++) gW2[c] += dz * H1[s * LD + half * 32 + c];
      const float d1 = G1[s * LD + jrow];
#pragma unroll
      for (int c = 0; c < 8; c++) gW1[c] += d1 * XQ[s * (KIN + 1) + half * 8 + c];
      gW3 += DY[s * NOUT + (t >> 6)] * H2[s * LD + (t & 63)];
      if (t < H) gb1 += G1[s * LD + t];
      else gb2 += DZ2[s * LD + (t - H)];
      if (t < NOUT) gb3 += DY[s * NOUT + t];
    }
    __syncthreads();
  }
  // ---- one atomic per owned entry
#pragma unroll
  for (int c = 0; c < 32; c++) atomicAdd(&G[Lo.oW2 + jrow * H + half * 32 + c], gW2[c]);
#pragma unroll
  for (int c = 0; c < 8; c++) {
    int k = half * 8 + c;
    if (k < n_in) atomicAdd(&G[Lo.oW1 + jrow * n_in + k], gW1[c]);
  }
  atomicAdd(&G[Lo.oW3 + (t >> 6) * H + (t & 63)], gW3);
  if (t < H) atomicAdd(&G[Lo.ob1 + t], gb1);
  else atomicAdd(&G[Lo.ob2 + (t - H)], gb2);
  if (t < NOUT) atomicAdd(&G[Lo.ob3 + t], gb3);
  // loss: warp reduce then one atomic per warp
  for (int off = 16; off; off >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, off);
  if ((t & 31) == 0) atomicAdd(loss, lsum);
}

__global__ void adam_kernel(float* __restrict__ P, const float* __restrict__ G, float* __restrict__ M, float* __restrict__ V, int n,
                            float lr, float b1, float b2, float eps, float c1, float c2, float wd) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float g = G[i] + wd * P[i];
  float m = b1 * M[i] + (1.0f - b1) * g;
  float v = b2 * V[i] + (1.0f - b2) * g * g;
  M[i] = m;
  V[i] = v;
  P[i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
}

size_t grad_smem_bytes() {
  return sizeof(float) * (H * H + H * KIN + NOUT * H + 2 * H + NOUT + 2 * KIN + 4 * TT * LD + TT * (KIN + 1) + TT * NOUT);
}

}  // namespace

struct degpu_mlp_s {
  int n_in = 0;
  int count = 0;
  float* P = nullptr;     // device master weights
  float* G = nullptr;     // device gradients
  float* M = nullptr;     // Adam first moment
  float* V = nullptr;     // Adam second moment
  float* mean = nullptr;  // device input normalisation
  float* stdv = nullptr;
  float* loss = nullptr;  // device scalar
  int steps = 0;
};

extern "C" {

int degpu_mlp_create(int n_in, unsigned long long seed, degpu_mlp** out) {
  if (!out || n_in < 1 || n_in > KIN) return DEGPU_E_INVALID;
  Layout Lo(n_in);
  auto* m = new degpu_mlp_s;
  m->n_in = n_in;
  m->count = Lo.count;
  size_t bytes = sizeof(float) * (4 * (size_t)Lo.count + 2 * KIN + 1);
  char* base = nullptr;
  if (cudaMalloc((void**)&base, bytes) != cudaSuccess) { delete m; return DEGPU_E_CUDA; }
  m->P = (float*)base;
  m->G = m->P + Lo.count;
  m->M = m->G + Lo.count;
  m->V = m->M + Lo.count;
  m->mean = m->V + Lo.count;
  m->stdv = m->mean + KIN;
  m->loss = m->stdv + KIN;
  // He-style init on the host (deterministic), zero biases, zero Adam state
  std::vector<float> h(4 * (size_t)Lo.count + 2 * KIN + 1, 0.0f);
  std::mt19937_64 rng(seed);
  std::normal_distribution<float> nd(0.0f, 1.0f);
  for (int i = 0; i < H * n_in; i++) h[Lo.oW1 + i] = nd(rng) * std::sqrt(2.0f / n_in);
  for (int i = 0; i < H * H; i++) h[Lo.oW2 + i] = nd(rng) * std::sqrt(2.0f / H);
  for (int i = 0; i < NOUT * H; i++) h[Lo.oW3 + i] = nd(rng) * std::sqrt(1.0f / H) * 0.1f;
  for (int i = 0; i < KIN; i++) h[4 * (size_t)Lo.count + KIN + i] = 1.0f;  // std = 1
  if (cudaMemcpy(base, h.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(base);
    delete m;
    return DEGPU_E_CUDA;
  }
  *out = m;
  return 0;
}

void degpu_mlp_destroy(degpu_mlp* m) {
  if (!m) return;
  cudaFree(m->P);
  delete m;
}

int degpu_mlp_param_count(const degpu_mlp* m) { return m ? m->count : DEGPU_E_INVALID; }

int degpu_mlp_set_params(degpu_mlp* m, const float* host_params, const float* host_mean, const float* host_std) {
  if (!m) return DEGPU_E_INVALID;
  if (host_params && cudaMemcpy(m->P, host_params, sizeof(float) * m->count, cudaMemcpyHostToDevice) != cudaSuccess) return DEGPU_E_CUDA;
  if (host_mean && cudaMemcpy(m->mean, host_mean, sizeof(float) * m->n_in, cudaMemcpyHostToDevice) != cudaSuccess) return DEGPU_E_CUDA;
  if (host_std && cudaMemcpy(m->stdv, host_std, sizeof(float) * m->n_in, cudaMemcpyHostToDevice) != cudaSuccess) return DEGPU_E_CUDA;
  return 0;
}

int degpu_mlp_get_params(const degpu_mlp* m, float* host_params, float* host_grads, float* host_mean, float* host_std) {
  if (!m) return DEGPU_E_INVALID;
  if (host_params && cudaMemcpy(host_params, m->P, sizeof(float) * m->count, cudaMemcpyDeviceToHost) != cudaSuccess) return DEGPU_E_CUDA;
  if (host_grads && cudaMemcpy(host_grads, m->G, sizeof(float) * m->count, cudaMemcpyDeviceToHost) != cudaSuccess) return DEGPU_E_CUDA;
  if (host_mean && cudaMemcpy(host_mean, m->mean, sizeof(float) * m->n_in, cudaMemcpyDeviceToHost) != cudaSuccess) return DEGPU_E_CUDA;
  if (host_std && cudaMemcpy(host_std, m->stdv, sizeof(float) * m->n_in, cudaMemcpyDeviceToHost) != cudaSuccess) return DEGPU_E_CUDA;
  return 0;
}

// resident inference blocks per SM: one wave of blocks, each staging the weights once and
// striding over the 16-trajectory tiles
static int infer_blocks_per_sm() {
  static int n = 0;
  if (!n) {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, mlp_infer_kernel, 128, 0) != cudaSuccess || b < 1) b = 1;
    n = b;
  }
  return n;
}

int degpu_mlp_infer(const degpu_mlp* m, const float* x, long long B, float* y, float* dt0, float* tolscale,
                    float dt_lo, float dt_hi, float s_lo, float s_hi, void* stream) {
  if (!m || B < 0 || (B > 0 && !x)) return DEGPU_E_INVALID;
  if (B == 0) return 0;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long tiles = (B + 15) / 16;
  long long grid = std::min<long long>((tiles + 3) / 4, (long long)sms * infer_blocks_per_sm());
  FeatSrc src{x, nullptr, nullptr, 0, 0, 0.0f, nullptr, 0};
  mlp_infer_kernel<<<(int)grid, 128, 0, (cudaStream_t)stream>>>(m->P, m->n_in, m->mean, m->stdv, src, B, y, dt0, tolscale,
                                                                 dt_lo, dt_hi, s_lo, s_hi);
  return cudaGetLastError() == cudaSuccess ? 0 : DEGPU_E_CUDA;
}

int degpu_mlp_infer_problems(const degpu_mlp* m, const float* u0, int n_state, const float* p, int n_param, float reltol,
                             long long B, float* dt0, float* tolscale, float dt_lo, float dt_hi, float s_lo, float s_hi,
                             void* stream) {
  return degpu_internal_mlp_infer_problems(m, u0, n_state, p, n_param, nullptr, 0, reltol, B, dt0, tolscale, dt_lo, dt_hi,
                                           s_lo, s_hi, stream);
}

int degpu_mlp_grad(degpu_mlp* m, const float* x, const float* target, const float* weight, long long B, float* loss_out,
                   void* stream) {
  if (!m || B <= 0 || !x || !target) return DEGPU_E_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  static bool attr_set = false;
  size_t smem = grad_smem_bytes();
  if (!attr_set) {
    if (cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
      return DEGPU_E_CUDA;
    attr_set = true;
  }
  if (cudaMemsetAsync(m->G, 0, sizeof(float) * m->count, s) != cudaSuccess) return DEGPU_E_CUDA;
  if (cudaMemsetAsync(m->loss, 0, sizeof(float), s) != cudaSuccess) return DEGPU_E_CUDA;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long tiles = (B + TT - 1) / TT;
  int grid = (int)std::min<long long>(tiles, (long long)sms);
  mlp_grad_kernel<<<grid, TT, smem, s>>>(m->P, m->n_in, m->mean, m->stdv, x, target, weight, B, 1.0f / (float)B, m->G, m->loss);
  if (cudaGetLastError() != cudaSuccess) return DEGPU_E_CUDA;
  if (loss_out && cudaMemcpyAsync(loss_out, m->loss, sizeof(float), cudaMemcpyDeviceToDevice, s) != cudaSuccess) return DEGPU_E_CUDA;
  return 0;
}

int degpu_mlp_adam_step(degpu_mlp* m, float lr, float beta1, float beta2, float eps, float weight_decay, void* stream) {
  if (!m) return DEGPU_E_INVALID;
  m->steps++;
  float c1 = 1.0f - std::pow(beta1, (float)m->steps), c2 = 1.0f - std::pow(beta2, (float)m->steps);
  adam_kernel<<<(m->count + 255) / 256, 256, 0, (cudaStream_t)stream>>>(m->P, m->G, m->M, m->V, m->count, lr, beta1, beta2,
                                                                        eps, c1, c2, weight_decay);
  return cudaGetLastError() == cudaSuccess ? 0 : DEGPU_E_CUDA;
}

}  // extern "C"

int degpu_internal_mlp_infer_problems(const degpu_mlp* m, const float* u0, int n_state, const float* p, int n_param,
                                      const void* tspan, int tspan_f64, float reltol, long long B, float* dt0,
                                      float* tolscale, float dt_lo, float dt_hi, float s_lo, float s_hi, void* stream) {
  if (!m || B < 0 || !(reltol > 0.0f)) return DEGPU_E_INVALID;
  const int base = n_state + n_param + 1;
  if (m->n_in != base && !(m->n_in == base + 1 && tspan)) return DEGPU_E_INVALID;
  if (B == 0) return 0;
  if (!u0 || (n_param > 0 && !p)) return DEGPU_E_INVALID;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long tiles = (B + 15) / 16;
  long long grid = std::min<long long>((tiles + 3) / 4, (long long)sms * infer_blocks_per_sm());
  FeatSrc src{nullptr, u0, p, n_state, n_param, log10f(reltol), m->n_in == base + 1 ? tspan : nullptr, tspan_f64};
  mlp_infer_kernel<<<(int)grid, 128, 0, (cudaStream_t)stream>>>(m->P, m->n_in, m->mean, m->stdv, src, B, nullptr, dt0,
                                                                 tolscale, dt_lo, dt_hi, s_lo, s_hi);
  return cudaGetLastError() == cudaSuccess ? 0 : DEGPU_E_CUDA;
}
