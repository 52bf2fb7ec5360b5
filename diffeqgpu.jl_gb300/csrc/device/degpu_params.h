/* Kernel parameter block, shared verbatim by the host library and the NVRTC-compiled
 * kernels (plain C, no CUDA types).  One struct, passed by value to every driver kernel.
 *
 * HBM layout (B trajectories, N states, P parameters, L saved points, Tt = time type):
 *   u0      [B][N]    f32   trajectory-major, i.e. Julia's Vector{SVector{N,Float32}}
 *   p       [B][P]    f32
 *   tspan   [B][2]    Tt    per-trajectory (t0, tf)
 *   saveat  [L] or [B][L] Tt
 *   ts      [B][L]    Tt    column i = trajectory i  (Julia Matrix{Tt}(L, B))
 *   us      [B][L][N] f32   column i = trajectory i  (Julia Matrix{SVector{N,Float32}}(L, B))
 */
#ifndef DEGPU_PARAMS_H
#define DEGPU_PARAMS_H

#define DEGPU_RET_DEFAULT 0
#define DEGPU_RET_SUCCESS 1
#define DEGPU_RET_TERMINATED 2
#define DEGPU_RET_DTLESSTHANMIN 3
#define DEGPU_RET_MAXITERS 4
#define DEGPU_RET_UNSTABLE 5

typedef struct degpu_kparams {
  const float* u0;
  const float* p;
  const void* tspan;
  const void* saveat;
  void* ts;
  float* us;
  signed char* retcode;   /* [B] or null */
  int* naccept;           /* [B] or null */
  int* nreject;           /* [B] or null */
  const float* dt0;       /* [B] per-trajectory initial dt (learned controller) or null */
  const float* tolscale;  /* [B] per-trajectory tolerance multiplier (learned controller) or null */
  float* dt_first;         /* [B] or null: first accepted dt (step-size trace) */
  unsigned long long* work; /* persistent driver: work[0] = next unclaimed trajectory */
  long long B;
  int maxiters;           /* cap on step attempts per trajectory (host-clamped to 2^31-1) */
  long long traj_offset;  /* global index of trajectory 0 (noise streams, shards) */
  unsigned long long seed;/* EM noise key */
  double dt;              /* fixed dt or initial dt, converted to Tt in the kernel */
  float abstol;
  float reltol;
  int L;                  /* rows of ts/us */
  int nsaveat;            /* 0 = no saveat */
  int saveat_per_traj;
  int save_everystep;
  int chunk;              /* persistent driver: trajectories claimed per warp refill */
  int stage_cols;         /* saved rows staged per lane in shared memory (blockDim*L*N floats) */
  int shared_saveat;      /* shared saveat grid converted once per block into shared memory */
  int ntstops;            /* 0 = no tstops */
  const void* tstops;     /* [ntstops] Tt, ascending, shared by all trajectories */
  /* callbacks (at most DEGPU_KP_MAX_CB of each kind): source function index, flags
   * (bit 0 affect!, bit 1 affect_neg!, bits 2-3 root-find mode), repeat-event tolerance,
   * repeat nudge and dt relaxation of each continuous callback; function index of each
   * discrete callback */
  int ccb_fn[8];
  int ccb_flags[8];
  float ccb_abstol[8];
  float ccb_nudge[8];
  float ccb_dtrelax[8];
  int dcb_fn[8];
  const int* order;       /* persistent driver: work item w runs trajectory order[w] (null: w);
                             entries outside [0, B) are skipped */
} degpu_kparams;
#define DEGPU_KP_MAX_CB 8

#endif
