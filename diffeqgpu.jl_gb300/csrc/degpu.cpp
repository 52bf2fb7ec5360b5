// libdegpu: host side of the GB300 EnsembleGPUKernel engine (C ABI in include/degpu.h).
//
// Replaces the reference's lower-level kernel API (src/ensemblegpukernel/lowerlevel_solve.jl)
// and its launch of ode_solve_kernel / ode_asolve_kernel / em_kernel (kernels.jl,
// perform_step/gpu_em_perform_step.jl).  Each (right-hand side, algorithm, driver, time
// type, mode) combination is one NVRTC translation unit: the user's CUDA C right-hand
// side followed by the stepper/driver templates, compiled for sm_103a, cached in memory
// and on disk, loaded once per device.  Launches are stream-ordered; plans capture the
// whole solve in a CUDA graph.
#include "degpu.h"

#include <cuda.h>
#include <cuda_runtime.h>
#include <nvrtc.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <sys/stat.h>
#include <unistd.h>
#include <vector>

#include "degpu_internal.h"
#include "device/degpu_params.h"

// embedded device sources (generated by build.py from csrc/device and csrc/models)
struct degpu_embedded_file { const char* name; const char* text; };
struct degpu_embedded_model { const char* name; int n, p, flags; const char* text; };
extern "C" const degpu_embedded_file degpu_embedded_headers[];
extern "C" const int degpu_embedded_nheaders;
extern "C" const degpu_embedded_model degpu_embedded_models[];
extern "C" const int degpu_embedded_nmodels;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}
#define CU_TRY(expr)                                                                   \
  do {                                                                                 \
    CUresult _r = (expr);                                                              \
    if (_r != CUDA_SUCCESS) {                                                          \
      const char* _s = nullptr;                                                        \
      if (g_drv.GetErrorString) g_drv.GetErrorString(_r, &_s);                         \
      return fail(DEGPU_E_CUDA, std::string(#expr) + ": " + (_s ? _s : "CUDA error")); \
    }                                                                                  \
  } while (0)
#define CUDA_TRY(expr)                                                                       \
  do {                                                                                       \
    cudaError_t _e = (expr);                                                                 \
    if (_e != cudaSuccess) return fail(DEGPU_E_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
  } while (0)

// Driver-API entry points, resolved at run time through the CUDA runtime
// (cudaGetDriverEntryPointByVersion) so that the library loads on machines without a
// driver (build and CPU-only test hosts) and needs no link against libcuda.
struct Driver {
  CUresult (*ModuleLoadData)(CUmodule*, const void*) = nullptr;
  CUresult (*ModuleGetFunction)(CUfunction*, CUmodule, const char*) = nullptr;
  CUresult (*LaunchKernel)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                           CUstream, void**, void**) = nullptr;
  CUresult (*FuncGetAttribute)(int*, CUfunction_attribute, CUfunction) = nullptr;
  CUresult (*OccupancyMaxActiveBlocksPerMultiprocessor)(int*, CUfunction, int, size_t) = nullptr;
  CUresult (*GetErrorString)(CUresult, const char**) = nullptr;
  CUresult (*FuncSetAttribute)(CUfunction, CUfunction_attribute, int) = nullptr;
  bool ok = false;
};
Driver g_drv;

template <class F>
bool resolve(const char* name, F*& fn) {
  void* p = nullptr;
  cudaDriverEntryPointQueryResult st;
  if (cudaGetDriverEntryPointByVersion(name, &p, 13000, cudaEnableDefault, &st) != cudaSuccess || !p) return false;
  fn = reinterpret_cast<F*>(p);
  return true;
}

int load_driver() {
  static std::once_flag once;
  static std::string err;
  std::call_once(once, [] {
    cudaError_t e = cudaFree(0);
    if (e != cudaSuccess) { err = std::string("CUDA initialisation failed: ") + cudaGetErrorString(e); return; }
    bool ok = resolve("cuModuleLoadData", g_drv.ModuleLoadData) && resolve("cuModuleGetFunction", g_drv.ModuleGetFunction) &&
              resolve("cuLaunchKernel", g_drv.LaunchKernel) && resolve("cuFuncGetAttribute", g_drv.FuncGetAttribute) &&
              resolve("cuOccupancyMaxActiveBlocksPerMultiprocessor", g_drv.OccupancyMaxActiveBlocksPerMultiprocessor) &&
              resolve("cuGetErrorString", g_drv.GetErrorString) &&
              resolve("cuFuncSetAttribute", g_drv.FuncSetAttribute);
    if (!ok) err = "could not resolve CUDA driver entry points";
    g_drv.ok = ok;
  });
  if (!g_drv.ok) return fail(DEGPU_E_CUDA, err);
  return 0;
}

uint64_t fnv1a(const std::string& s, uint64_t h = 1469598103934665603ULL) {
  for (unsigned char c : s) { h ^= c; h *= 1099511628211ULL; }
  return h;
}

}  // namespace

struct degpu_rhs_s {
  std::string src;
  int N, P, flags;
};

namespace {

bool is_sde_alg(int alg) { return alg == DEGPU_ALG_EM || alg == DEGPU_ALG_SIEA; }

struct KernelSpec {
  int alg, driver, tt, parity, jac, tgrad, refine;
  int tstops = 0, nccb = 0, ndcb = 0;  // tstops / callback set compiled into the kernel
  int mass = 0;                        // constant mass matrix (DEGPU_RHS_HAS_MASS)
  int lbt = 0, lbm = 0;                // launch bounds (threads, min blocks per SM); 0 = default
  std::string key() const {
    char b[160];
    snprintf(b, sizeof b, "a%d_d%d_t%d_m%d_j%d_g%d_r%d_s%d_c%d_e%d_M%d_L%d.%d", alg, driver, tt, parity, jac, tgrad,
             refine, tstops, nccb, ndcb, mass, lbt, lbm);
    return b;
  }
};

struct Kernel {
  CUfunction fn = nullptr;
  int regs = 0, local_bytes = 0, max_threads = 0;
};

std::mutex g_mu;
std::map<std::string, std::vector<char>> g_cubins;  // source-key -> cubin
std::map<std::string, CUmodule> g_modules;          // source-key + device -> module
std::map<std::string, Kernel> g_kernels;
std::map<std::string, std::pair<int, int>> g_tuned;  // autotune cache

std::string cache_dir() {
  const char* d = getenv("DEGPU_CACHE_DIR");
  std::string dir;
  if (d && *d) dir = d;
  else {
    const char* h = getenv("HOME");
    dir = std::string(h && *h ? h : "/tmp") + "/.cache/degpu";
  }
  return dir;
}

void mkdirs(const std::string& path) {
  std::string cur;
  for (size_t i = 0; i < path.size(); i++) {
    cur += path[i];
    if (path[i] == '/' && cur.size() > 1) mkdir(cur.c_str(), 0755);
  }
  mkdir(path.c_str(), 0755);
}

std::string build_source(const degpu_rhs_s* f, const KernelSpec& k) {
  char defs[640];
  snprintf(defs, sizeof defs,
           "#define DEGPU_N %d\n#define DEGPU_P %d\n#define DEGPU_TT %s\n#define DEGPU_ALG %d\n"
           "#define DEGPU_DRIVER %d\n#define DEGPU_PARITY %d\n#define DEGPU_JAC %d\n#define DEGPU_TGRAD %d\n"
           "#define DEGPU_LINSOLVE_REFINE %d\n#define DEGPU_TIME_DF %d\n"
           "#define DEGPU_TSTOPS %d\n#define DEGPU_NCCB %d\n#define DEGPU_NDCB %d\n#define DEGPU_MASS %d\n",
           f->N, f->P, k.tt ? "double" : "float", k.alg, k.driver, k.parity, k.jac, k.tgrad, k.refine, k.tt,
           k.tstops, k.nccb, k.ndcb, k.mass);
  std::string s = defs;
  if (k.lbt > 0) {  // launch bounds chosen by the occupancy step of get_kernel
    char b[96];
    snprintf(b, sizeof b, "#define DEGPU_LB_THREADS %d\n#define DEGPU_LB_MINBLOCKS %d\n", k.lbt, k.lbm);
    s += b;
  } else if (const char* lb = getenv("DEGPU_LB")) {  // developer override (register budget experiments)
    int thr = 0, mb = 0;
    if (sscanf(lb, "%d,%d", &thr, &mb) == 2 && thr > 0 && mb > 0) {
      char b[96];
      snprintf(b, sizeof b, "#define DEGPU_LB_THREADS %d\n#define DEGPU_LB_MINBLOCKS %d\n", thr, mb);
      s += b;
    }
  }
  s += "#include \"degpu_prelude.cuh\"\n#line 1 \"user_rhs.cu\"\n";
  s += f->src;
  s += "\n#include \"degpu_kernels.cuh\"\n";
  return s;
}

int compile_cubin(const std::string& src, bool parity, std::vector<char>& cubin) {
  int major = 0, minor = 0;
  nvrtcVersion(&major, &minor);
  std::string opts_key = std::string(parity ? "fmad0" : "fmad1") + "|sm_103a|" + std::to_string(major) + "." + std::to_string(minor);
  if (const char* mr = getenv("DEGPU_MAXRREG")) opts_key += std::string("|maxrreg=") + mr;
  uint64_t h = fnv1a(opts_key, fnv1a(src));
  char hex[32];
  snprintf(hex, sizeof hex, "%016llx", (unsigned long long)h);
  std::string path = cache_dir() + "/" + hex + ".cubin";
  if (!getenv("DEGPU_NO_DISK_CACHE")) {
    FILE* fp = fopen(path.c_str(), "rb");
    if (fp) {
      fseek(fp, 0, SEEK_END);
      long n = ftell(fp);
      fseek(fp, 0, SEEK_SET);
      if (n > 0) {
        cubin.resize(n);
        size_t got = fread(cubin.data(), 1, n, fp);
        fclose(fp);
        if ((long)got == n) return 0;
      } else {
        fclose(fp);
      }
    }
  }
  std::vector<const char*> hdr_txt, hdr_names;
  for (int i = 0; i < degpu_embedded_nheaders; i++) {
    hdr_names.push_back(degpu_embedded_headers[i].name);
    hdr_txt.push_back(degpu_embedded_headers[i].text);
  }
  nvrtcProgram prog;
  nvrtcResult r = nvrtcCreateProgram(&prog, src.c_str(), "degpu_tu.cu", (int)hdr_txt.size(), hdr_txt.data(), hdr_names.data());
  if (r != NVRTC_SUCCESS) return fail(DEGPU_E_COMPILE, std::string("nvrtcCreateProgram: ") + nvrtcGetErrorString(r));
  // parity: strict IEEE (no contraction, correctly rounded / and sqrt); fast: FMA
  // contraction and the approximate divide / square root of the SFU
  std::vector<const char*> opts = {"--gpu-architecture=sm_103a", "-std=c++17", "-lineinfo",
                                   parity ? "--fmad=false" : "--fmad=true",
                                   parity ? "--prec-div=true" : "--prec-div=false",
                                   parity ? "--prec-sqrt=true" : "--prec-sqrt=false"};
  // developer override of the register cap (occupancy experiments), part of the cache key
  std::string maxrreg;
  if (const char* mr = getenv("DEGPU_MAXRREG")) {
    if (atoi(mr) > 0) {
      maxrreg = std::string("--maxrregcount=") + mr;
      opts.push_back(maxrreg.c_str());
    }
  }
  r = nvrtcCompileProgram(prog, (int)opts.size(), opts.data());
  if (r != NVRTC_SUCCESS) {
    size_t n = 0;
    nvrtcGetProgramLogSize(prog, &n);
    std::string log(n, '\0');
    nvrtcGetProgramLog(prog, &log[0]);
    nvrtcDestroyProgram(&prog);
    return fail(DEGPU_E_COMPILE, "NVRTC compile failed:\n" + log);
  }
  size_t n = 0;
  nvrtcGetCUBINSize(prog, &n);
  cubin.resize(n);
  nvrtcGetCUBIN(prog, cubin.data());
  nvrtcDestroyProgram(&prog);
  if (!getenv("DEGPU_NO_DISK_CACHE")) {
    mkdirs(cache_dir());
    std::string tmp = path + ".tmp" + std::to_string(getpid());
    FILE* fp = fopen(tmp.c_str(), "wb");
    if (fp) {
      fwrite(cubin.data(), 1, n, fp);
      fclose(fp);
      rename(tmp.c_str(), path.c_str());
    }
  }
  return 0;
}

const char* kernel_name(int driver) {
  switch (driver) {
    case 2: return "degpu_persistent_kernel";
    case 3: return "degpu_em_kernel";
    default: return "degpu_solve_kernel";
  }
}

int ensure_context() {
  int rc = load_driver();
  if (rc) return rc;
  // make the runtime's primary context of the current device current -- once per device,
  // so that later solves (possibly inside a stream capture) issue no context calls
  static std::mutex mu;
  static unsigned long long done = 0;
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  if (dev < 64 && (done >> dev) & 1ULL) return 0;
  CUDA_TRY(cudaFree(0));
  if (dev < 64) done |= 1ULL << dev;
  return 0;
}

// Device scratch of the library (persistent-driver work counters, the learned solve's
// scratch, the host API's staging arena) comes from one memory pool per device that keeps
// its memory between calls (release threshold unlimited; degpu_trim_memory returns it), so
// repeated solves do not map and unmap device memory at every synchronisation as the
// default pool (threshold 0) does.  Inside a stream capture the allocation goes to the
// stream-ordered allocator's default pool instead (a graph allocation node).
std::mutex g_pool_mu;
cudaMemPool_t g_pools[64] = {};
int lib_alloc(void** p, size_t n, cudaStream_t s) {
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
    CUDA_TRY(cudaMallocAsync(p, n, s));
    return 0;
  }
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  cudaMemPool_t pool = nullptr;
  if (dev >= 0 && dev < 64) {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (!g_pools[dev]) {
      cudaMemPoolProps props;
      memset(&props, 0, sizeof props);
      props.allocType = cudaMemAllocationTypePinned;
      props.handleTypes = cudaMemHandleTypeNone;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = dev;
      cudaMemPool_t np = nullptr;
      if (cudaMemPoolCreate(&np, &props) == cudaSuccess) {
        unsigned long long keep = ~0ULL;
        cudaMemPoolSetAttribute(np, cudaMemPoolAttrReleaseThreshold, &keep);
        g_pools[dev] = np;
      }
    }
    pool = g_pools[dev];
  }
  if (pool) CUDA_TRY(cudaMallocFromPoolAsync(p, n, pool, s));
  else CUDA_TRY(cudaMallocAsync(p, n, s));
  return 0;
}

int load_kernel(const degpu_rhs_s* f, const KernelSpec& k, Kernel* out) {
  int rc = ensure_context();
  if (rc) return rc;
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  std::string src = build_source(f, k);
  std::string skey = std::to_string(fnv1a(src)) + "|" + k.key();
  std::string mkey = skey + "|dev" + std::to_string(dev);
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_kernels.find(mkey);
  if (it != g_kernels.end()) { *out = it->second; return 0; }
  auto cit = g_cubins.find(skey);
  if (cit == g_cubins.end()) {
    std::vector<char> cubin;
    rc = compile_cubin(src, k.parity != 0, cubin);
    if (rc) return rc;
    cit = g_cubins.emplace(skey, std::move(cubin)).first;
  }
  CUmodule mod;
  CU_TRY(g_drv.ModuleLoadData(&mod, cit->second.data()));
  g_modules[mkey] = mod;
  Kernel kern;
  CU_TRY(g_drv.ModuleGetFunction(&kern.fn, mod, kernel_name(k.driver)));
  g_drv.FuncGetAttribute(&kern.regs, CU_FUNC_ATTRIBUTE_NUM_REGS, kern.fn);
  g_drv.FuncGetAttribute(&kern.local_bytes, CU_FUNC_ATTRIBUTE_LOCAL_SIZE_BYTES, kern.fn);
  g_drv.FuncGetAttribute(&kern.max_threads, CU_FUNC_ATTRIBUTE_MAX_THREADS_PER_BLOCK, kern.fn);
  g_kernels[mkey] = kern;
  *out = kern;
  return 0;
}

// Warps one SM sub-partition (16,384 registers) holds at R registers per thread; registers
// are allocated per warp in units of 256 (8 per thread).
int warps_per_smsp(int regs) { return regs > 0 ? 16384 / (((regs + 7) / 8) * 8 * 32) : 0; }

// The fast-mode persistent driver is latency-bound at the occupancy its register count
// allows (ncu: ~72 % issue active, "wait" stalls dominant), so the kernel is also compiled
// under tighter launch bounds (128 threads, 5..7 blocks per SM) and the variant with the
// most resident warps that needs no local memory (no spills) is used.  Measured on the
// adaptive Lorenz ensemble: 102 -> 80 registers, 16 -> 24 warps per SM, 9-11 % faster;
// the next cap (72 registers) spills and is slower.  Each variant compiles once per process
// (and is cached on disk).
std::mutex g_occ_mu;
std::map<std::string, Kernel> g_occ;
int get_kernel(const degpu_rhs_s* f, const KernelSpec& k, Kernel* out) {
  const bool tune = k.driver == 2 && !k.parity && k.lbt == 0 && !getenv("DEGPU_LB") && !getenv("DEGPU_NO_OCC_TUNE");
  if (!tune) return load_kernel(f, k, out);
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  const std::string okey = std::to_string((uintptr_t)f) + "|" + std::to_string(fnv1a(f->src)) + "|" + k.key() + "|" +
                           std::to_string(dev);
  {
    std::lock_guard<std::mutex> lk(g_occ_mu);
    auto it = g_occ.find(okey);
    if (it != g_occ.end()) { *out = it->second; return 0; }
  }
  Kernel best;
  int rc = load_kernel(f, k, &best);
  if (rc) return rc;
  int bw = warps_per_smsp(best.regs);
  for (int mb = 5; mb <= 7; mb++) {
    KernelSpec k2 = k;
    k2.lbt = 128;
    k2.lbm = mb;
    Kernel c;
    if (load_kernel(f, k2, &c)) break;  // keep what compiled so far
    if (c.local_bytes > 0) break;        // spills: tighter caps only get worse
    const int w = warps_per_smsp(c.regs);
    if (w > bw) { best = c; bw = w; }
  }
  std::lock_guard<std::mutex> lk(g_occ_mu);
  g_occ[okey] = best;
  *out = best;
  return 0;
}

// ------------------------------------------------------------------ request validation
struct Request {
  const degpu_rhs_s* f;
  KernelSpec spec;
  degpu_kparams kp;
  int block, chunk;
};

int resolve_driver(const degpu_options* o, int adaptive) {
  if (is_sde_alg(o->alg)) return 3;
  if (!adaptive) return 0;
  if (o->driver == DEGPU_DRIVER_NAIVE) return 1;
  return 2;
}

int make_request(const degpu_rhs* f, const degpu_problems* pr, const degpu_options* o, int adaptive,
                 const degpu_outputs* out, Request* rq) {
  if (!f || !pr || !o || !out) return fail(DEGPU_E_INVALID, "null argument");
  if (pr->B < 0) return fail(DEGPU_E_INVALID, "negative trajectory count");
  if (pr->B > 0x7fffffffLL) return fail(DEGPU_E_INVALID, "more than 2^31-1 trajectories in one call; split into batches");
  if (o->alg < 0 || o->alg > 9) return fail(DEGPU_E_INVALID, "unknown algorithm");
  if (is_sde_alg(o->alg) && adaptive)
    return fail(DEGPU_E_UNSUPPORTED, o->alg == DEGPU_ALG_EM ? "Adaptive time-stepping is not supported yet with GPUEM."
                                                            : "Adaptive time-stepping is not supported yet with GPUSIEA.");
  if (is_sde_alg(o->alg) && !(f->flags & DEGPU_RHS_HAS_NOISE))
    return fail(DEGPU_E_INVALID, "GPUEM / GPUSIEA need a right-hand side with a noise function (DEGPU_RHS_HAS_NOISE)");
  if (o->time_type != DEGPU_TIME_F32 && o->time_type != DEGPU_TIME_F64) return fail(DEGPU_E_INVALID, "time_type");
  if (o->mode != DEGPU_MODE_FAST && o->mode != DEGPU_MODE_PARITY) return fail(DEGPU_E_INVALID, "mode");
  if (!(o->dt > 0.0) && !o->dt0) return fail(DEGPU_E_INVALID, "dt must be positive");
  if (out->L < 1) return fail(DEGPU_E_INVALID, "L must be >= 1");
  if (o->nsaveat < 0) return fail(DEGPU_E_INVALID, "nsaveat < 0");
  if (o->nsaveat > 0 && !o->saveat) return fail(DEGPU_E_INVALID, "saveat pointer missing");
  if (o->nsaveat > 0 && out->L != o->nsaveat)
    return fail(DEGPU_E_INVALID, "L must equal the number of saveat points (lowerlevel_solve.jl:106, 321)");
  if (o->nsaveat == 0 && !o->save_everystep && out->L != 2)
    return fail(DEGPU_E_INVALID, "without saveat and with save_everystep=false the output has L=2 rows (lowerlevel_solve.jl:79, 315)");
  if (pr->B > 0 && (!pr->u0 || !pr->tspan || !out->ts || !out->us)) return fail(DEGPU_E_INVALID, "null device buffer");
  if (pr->B > 0 && f->P > 0 && !pr->p) return fail(DEGPU_E_INVALID, "null parameter buffer");
  if (o->block < 0 || o->block > 1024 || (o->block % 32) != 0) return fail(DEGPU_E_INVALID, "block must be a multiple of 32 in [32, 1024]");
  if (o->chunk < 0 || o->chunk > 4096) return fail(DEGPU_E_INVALID, "chunk must be in [0, 4096]");
  rq->f = f;
  KernelSpec& k = rq->spec;
  k.alg = o->alg;
  k.driver = resolve_driver(o, adaptive);
  k.tt = o->time_type;
  k.parity = o->mode == DEGPU_MODE_PARITY;
  int jac_user = (f->flags & DEGPU_RHS_HAS_JAC) ? 1 : 0, tg_user = (f->flags & DEGPU_RHS_HAS_TGRAD) ? 1 : 0;
  if (o->jac == DEGPU_JAC_AUTO) { k.jac = jac_user ? 1 : 0; k.tgrad = tg_user ? 1 : 0; }
  else if (o->jac == DEGPU_JAC_AD) { k.jac = 0; k.tgrad = 0; }
  else if (o->jac == DEGPU_JAC_FINITEDIFF) { k.jac = 2; k.tgrad = 2; }
  else return fail(DEGPU_E_INVALID, "jac");
  // algorithms that build Jacobians and solve linear systems: Rosenbrock and ESDIRK (Newton)
  const bool implicit = o->alg == DEGPU_ALG_ROSENBROCK23 || o->alg == DEGPU_ALG_RODAS5P || o->alg == DEGPU_ALG_RODAS4 ||
                        o->alg == DEGPU_ALG_KVAERNO3 || o->alg == DEGPU_ALG_KVAERNO5;
  if (!implicit) { k.jac = 0; k.tgrad = 0; }
  if (f->flags & DEGPU_RHS_HAS_MASS) {
    if (o->alg != DEGPU_ALG_ROSENBROCK23 && o->alg != DEGPU_ALG_RODAS4 && o->alg != DEGPU_ALG_RODAS5P)
      return fail(DEGPU_E_UNSUPPORTED, "a mass matrix needs GPURosenbrock23, GPURodas4 or GPURodas5P");
    k.mass = 1;
  }
  k.refine = implicit && !k.parity ? 1 : 0;
  degpu_kparams& P = rq->kp;
  memset(&P, 0, sizeof P);
  P.u0 = pr->u0;
  P.p = pr->p;
  P.tspan = pr->tspan;
  P.saveat = o->nsaveat ? o->saveat : nullptr;
  P.ts = out->ts;
  P.us = out->us;
  P.retcode = out->retcode;
  P.naccept = out->naccept;
  P.nreject = out->nreject;
  P.dt_first = out->dt_first;
  P.dt0 = o->dt0;
  P.tolscale = o->tolscale;
  P.B = pr->B;
  P.maxiters = (int)std::min<long long>(o->maxiters > 0 ? o->maxiters : 10000000LL, 0x7fffffffLL);
  P.traj_offset = o->traj_offset;
  P.seed = o->seed;
  P.dt = o->dt;
  P.abstol = (float)o->abstol;
  P.reltol = (float)o->reltol;
  P.L = out->L;
  P.nsaveat = o->nsaveat;
  P.saveat_per_traj = o->saveat_per_traj;
  P.save_everystep = o->save_everystep;
  // tstops and callbacks (vectorized_(a)solve kwargs tstops / callback)
  if (o->ntstops < 0) return fail(DEGPU_E_INVALID, "ntstops < 0");
  if (o->ntstops > 0 && !o->tstops) return fail(DEGPU_E_INVALID, "tstops pointer missing");
  const degpu_callbacks* cb = o->callbacks;
  const int nc = cb ? cb->n_continuous : 0, nd = cb ? cb->n_discrete : 0;
  if (nc < 0 || nd < 0 || nc > DEGPU_MAX_CALLBACKS || nd > DEGPU_MAX_CALLBACKS)
    return fail(DEGPU_E_INVALID, "at most 8 continuous and 8 discrete callbacks per set");
  if ((nc && !cb->continuous) || (nd && !cb->discrete)) return fail(DEGPU_E_INVALID, "callback array missing");
  if (is_sde_alg(o->alg) && (nc || nd || o->ntstops))
    return fail(DEGPU_E_UNSUPPORTED, "GPUEM / GPUSIEA take no callbacks or tstops (em_kernel, siea_kernel)");
  for (int j = 0; j < nc; j++) {
    const degpu_continuous_callback& c = cb->continuous[j];
    if (c.fn < 0 || c.rootfind < 0 || c.rootfind > 2 || !(c.abstol >= 0.0) || !(c.dtrelax > 0.0))
      return fail(DEGPU_E_INVALID, "bad continuous callback (fn >= 0, rootfind in 0..2, abstol >= 0, dtrelax > 0)");
    P.ccb_fn[j] = c.fn;
    P.ccb_flags[j] = (c.has_affect ? 1 : 0) | (c.has_affect_neg ? 2 : 0) | (c.rootfind << 2);
    P.ccb_abstol[j] = (float)c.abstol;
    P.ccb_nudge[j] = (float)c.repeat_nudge;
    P.ccb_dtrelax[j] = (float)c.dtrelax;
  }
  for (int j = 0; j < nd; j++) {
    if (cb->discrete[j] < 0) return fail(DEGPU_E_INVALID, "bad discrete callback function index");
    P.dcb_fn[j] = cb->discrete[j];
  }
  P.ntstops = o->ntstops;
  P.tstops = o->ntstops ? o->tstops : nullptr;
  P.order = k.driver == 2 ? o->order : nullptr;  // visiting order: persistent driver only
  k.tstops = o->ntstops > 0 ? 1 : 0;
  k.nccb = nc;
  k.ndcb = nd;
  rq->block = o->block;
  rq->chunk = o->chunk;
  return 0;
}

int sm_count() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

// Dynamic shared memory of the ODE drivers: the shared saveat grid (once per block, in the
// kernels' time type) and, when they fit, one staged output column of L*N floats per lane.
struct SmemCfg {
  int shared_saveat = 0, stage_cols = 0;
  size_t bytes = 0;
};
SmemCfg smem_for(const Request& rq, int block, int N) {
  SmemCfg c;
  const degpu_kparams& P = rq.kp;
  if (rq.spec.driver == 3 || P.nsaveat == 0) return c;
  const size_t tsz = rq.spec.tt ? 8 : 4;
  if (!P.saveat_per_traj && (size_t)P.nsaveat * tsz <= 16384) {
    c.shared_saveat = 1;
    c.bytes = ((size_t)P.nsaveat * tsz + 15) & ~(size_t)15;
  }
  const size_t cols = (size_t)block * P.L * N * sizeof(float);
  if (!getenv("DEGPU_NO_STAGING") && cols <= 96 * 1024) {
    c.stage_cols = 1;
    c.bytes += cols;
  }
  return c;
}

int grid_for(const Request& rq, const Kernel& K, int block) {
  long long B = rq.kp.B;
  if (rq.spec.driver != 2) return (int)((B + block - 1) / block);
  // persistent: fill the machine once (a multiple of the SM count), never more than needed
  int per_sm = 0;
  const SmemCfg sc = smem_for(rq, block, rq.f->N);
  g_drv.OccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, K.fn, block, sc.bytes);
  if (per_sm < 1) per_sm = 1;
  long long g = (long long)per_sm * sm_count();
  long long need = (B + block - 1) / block;
  return (int)std::max(1LL, std::min(g, need));
}

int default_block(const Request& rq) { return rq.spec.driver == 2 ? 128 : 128; }
int default_chunk() { return 32; }

int launch(const Request& rq, const Kernel& K, int block, int chunk, unsigned long long* work, CUstream s) {
  if (block > K.max_threads)
    return fail(DEGPU_E_INVALID, "block larger than the kernel's launch bounds (" + std::to_string(K.max_threads) + " threads)");
  degpu_kparams P = rq.kp;
  P.chunk = chunk;
  P.work = work;
  const SmemCfg sc = smem_for(rq, block, rq.f->N);
  P.shared_saveat = sc.shared_saveat;
  P.stage_cols = sc.stage_cols;
  if (sc.bytes > 48 * 1024)
    CU_TRY(g_drv.FuncSetAttribute(K.fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)sc.bytes));
  int grid = grid_for(rq, K, block);
  if (rq.spec.driver == 2) {
    if (!work) return fail(DEGPU_E_INVALID, "persistent driver without a work counter");
    CUDA_TRY(cudaMemsetAsync(work, 0, sizeof(unsigned long long), (cudaStream_t)s));
  }
  void* args[] = {(void*)&P};
  CU_TRY(g_drv.LaunchKernel(K.fn, grid, 1, 1, block, 1, 1, (unsigned)sc.bytes, s, args, nullptr));
  return 0;
}

// Stream-ordered solve with a per-call work counter from the stream-ordered allocator.
int run(const degpu_rhs* f, const degpu_problems* pr, const degpu_options* o, int adaptive, degpu_outputs* out, void* stream) {
  Request rq;
  int rc = make_request(f, pr, o, adaptive, out, &rq);
  if (rc) return rc;
  if (rq.kp.B == 0) return 0;  // empty ensemble: nothing to do
  Kernel K;
  rc = get_kernel(f, rq.spec, &K);
  if (rc) return rc;
  int block = rq.block ? rq.block : default_block(rq);
  int chunk = rq.chunk ? rq.chunk : default_chunk();
  {
    std::lock_guard<std::mutex> lk(g_mu);
    char key[64];
    snprintf(key, sizeof key, "%p|%lld", (void*)K.fn, (long long)(rq.kp.B >> 16));
    auto it = g_tuned.find(key);
    if (!rq.block && it != g_tuned.end()) { block = it->second.first; if (!rq.chunk) chunk = it->second.second; }
  }
  unsigned long long* work = nullptr;
  cudaStream_t s = (cudaStream_t)stream;
  if (rq.spec.driver == 2) {
    rc = lib_alloc((void**)&work, 256, s);
    if (rc) return rc;
  }
  rc = launch(rq, K, block, chunk, work, (CUstream)s);
  if (work) cudaFreeAsync(work, s);
  return rc;
}

}  // namespace

// ====================================================================== C ABI
extern "C" {

const char* degpu_version(void) { return DEGPU_VERSION; }
void degpu_trim_memory(void) {
  std::lock_guard<std::mutex> lk(g_pool_mu);
  for (int d = 0; d < 64; d++)
    if (g_pools[d]) cudaMemPoolTrimTo(g_pools[d], 0);
}
void degpu_abi_struct_sizes(int* options, int* outputs, int* problems, int* continuous_callback, int* callbacks) {
  if (options) *options = (int)sizeof(degpu_options);
  if (outputs) *outputs = (int)sizeof(degpu_outputs);
  if (problems) *problems = (int)sizeof(degpu_problems);
  if (continuous_callback) *continuous_callback = (int)sizeof(degpu_continuous_callback);
  if (callbacks) *callbacks = (int)sizeof(degpu_callbacks);
}
const char* degpu_last_error(void) { return g_err.c_str(); }

int degpu_rhs_create(const char* cuda_source, int n_state, int n_param, int flags, degpu_rhs** out) {
  if (!cuda_source || !out) return fail(DEGPU_E_INVALID, "null argument");
  if (n_state < 1 || n_state > 32) return fail(DEGPU_E_INVALID, "state dimension must be in [1, 32]");
  if (n_param < 0 || n_param > 64) return fail(DEGPU_E_INVALID, "parameter count must be in [0, 64]");
  if (flags & ~(DEGPU_RHS_HAS_JAC | DEGPU_RHS_HAS_TGRAD | DEGPU_RHS_HAS_NOISE | DEGPU_RHS_HAS_MASS))
    return fail(DEGPU_E_INVALID, "unknown flags");
  auto* f = new degpu_rhs_s;
  f->src = cuda_source;
  f->N = n_state;
  f->P = n_param;
  f->flags = flags;
  *out = f;
  return 0;
}

void degpu_rhs_destroy(degpu_rhs* f) { delete f; }

const char* degpu_builtin_rhs(const char* name, int* n_state, int* n_param, int* flags) {
  if (!name) return nullptr;
  for (int i = 0; i < degpu_embedded_nmodels; i++) {
    if (strcmp(degpu_embedded_models[i].name, name) == 0) {
      if (n_state) *n_state = degpu_embedded_models[i].n;
      if (n_param) *n_param = degpu_embedded_models[i].p;
      if (flags) *flags = degpu_embedded_models[i].flags;
      return degpu_embedded_models[i].text;
    }
  }
  return nullptr;
}

int degpu_vectorized_solve(const degpu_rhs* f, const degpu_problems* probs, const degpu_options* opt,
                           degpu_outputs* out, void* stream) {
  if (opt && is_sde_alg(opt->alg)) return fail(DEGPU_E_INVALID, "GPUEM / GPUSIEA solve SDE problems: use degpu_vectorized_solve_sde");
  return run(f, probs, opt, 0, out, stream);
}

int degpu_vectorized_asolve(const degpu_rhs* f, const degpu_problems* probs, const degpu_options* opt,
                            degpu_outputs* out, void* stream) {
  return run(f, probs, opt, 1, out, stream);
}

int degpu_vectorized_solve_sde(const degpu_rhs* f, const degpu_problems* probs, const degpu_options* opt,
                               degpu_outputs* out, void* stream) {
  if (opt && !is_sde_alg(opt->alg)) return fail(DEGPU_E_INVALID, "SDE problems are solved with GPUEM or GPUSIEA");
  return run(f, probs, opt, 0, out, stream);
}

namespace {
// The learned parts of a host-buffer solve (both null: the plain solve).
struct HostModels {
  const degpu_mlp* step;
  const degpu_mlp* work;
  float dt_lo, dt_hi, s_max;
};

int batch_solve_host(const degpu_rhs* f, const HostModels& hm, const float* u0, const float* p, const void* tspan,
                     long long B, const degpu_options* opt, int adaptive, void* ts, float* us, int L,
                     signed char* retcode, int* naccept, int* nreject, void* stream) {
  if (!f || !opt) return fail(DEGPU_E_INVALID, "null argument");
  if (B < 0) return fail(DEGPU_E_INVALID, "negative trajectory count");
  if (opt->order) return fail(DEGPU_E_INVALID, "the host-buffer API takes no visiting order (options.order)");
  const bool learned = hm.step || hm.work;
  if (learned && (!adaptive || is_sde_alg(opt->alg)))
    return fail(DEGPU_E_INVALID, "step and work models apply to adaptive ODE solves");
  if (B == 0) return 0;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t tsz = opt->time_type == DEGPU_TIME_F64 ? 8 : 4;
  const size_t N = f->N, P = f->P;
  const size_t n_u0 = (size_t)B * N * 4, n_p = (size_t)B * P * 4, n_tsp = (size_t)B * 2 * tsz;
  const size_t n_ts = (size_t)B * L * tsz, n_us = (size_t)B * L * N * 4;
  const size_t sa_rows = opt->nsaveat ? (opt->saveat_per_traj ? (size_t)B : 1) : 0;
  const size_t n_sa = sa_rows * (size_t)opt->nsaveat * tsz;

  // Output buffers in page-locked host memory are addressable by the GPU (unified addressing
  // maps them into its address space; on GB300 they sit across the coherent NVLink-C2C
  // link), so the solver kernel writes ts/us/retcodes into them itself: no device staging of
  // the outputs and no copy pass after the solve.  Pageable outputs take the staged,
  // pipelined path below.
  auto device_view = [](const void* h) -> void* {
    if (!h) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    return (a.type == cudaMemoryTypeHost && a.devicePointer) ? a.devicePointer : nullptr;
  };
  // A visiting order (work model) scatters the trajectories' completion over the batch, and
  // with it the kernel's writes into host memory: column edges that neighbouring
  // trajectories share are written at different times, as partial lines over the link.
  // Measured on 1,048,576 Lorenz trajectories (441 MB of outputs): direct 4.98 ms against
  // 4.13 ms staged in HBM and copied back in pipelined chunks (4.80 / 5.13 ms in index
  // order).  So ordered solves take the staged path unless DEGPU_HOST_DIRECT=1.
  const char* direct_env = getenv("DEGPU_HOST_DIRECT");
  const bool direct_ok = hm.work ? (direct_env && direct_env[0] == '1') : !(direct_env && direct_env[0] == '0');
  if (direct_ok) {
    void* v_ts = device_view(ts);
    void* v_us = device_view(us);
    void* v_rc = device_view(retcode);
    void* v_na = device_view(naccept);
    void* v_nr = device_view(nreject);
    if (v_ts && v_us && (!retcode || v_rc) && (!naccept || v_na) && (!nreject || v_nr)) {
      size_t o_u0 = 0, o_p = (o_u0 + n_u0 + 255) & ~(size_t)255, o_tsp = (o_p + n_p + 255) & ~(size_t)255;
      size_t o_sa = (o_tsp + n_tsp + 255) & ~(size_t)255, o_work = (o_sa + n_sa + 255) & ~(size_t)255;
      char* d = nullptr;
      int rc = lib_alloc((void**)&d, o_work + 256, s);
      if (rc) return rc;
      if (cudaMemcpyAsync(d + o_u0, u0, n_u0, cudaMemcpyHostToDevice, s) != cudaSuccess ||
          (n_p && cudaMemcpyAsync(d + o_p, p, n_p, cudaMemcpyHostToDevice, s) != cudaSuccess) ||
          cudaMemcpyAsync(d + o_tsp, tspan, n_tsp, cudaMemcpyHostToDevice, s) != cudaSuccess ||
          (n_sa && cudaMemcpyAsync(d + o_sa, opt->saveat, n_sa, cudaMemcpyHostToDevice, s) != cudaSuccess))
        rc = fail(DEGPU_E_CUDA, "host-to-device copy failed");
      if (!rc) {
        degpu_problems pr{(const float*)(d + o_u0), (const float*)(d + o_p), d + o_tsp, B};
        degpu_options o = *opt;
        if (n_sa) o.saveat = d + o_sa;
        degpu_outputs out{v_ts, (float*)v_us, L, (signed char*)v_rc, (int*)v_na, (int*)v_nr, nullptr};
        unsigned long long* work = reinterpret_cast<unsigned long long*>(d + o_work);
        rc = learned ? degpu_learned_asolve_ex(f, hm.step, hm.work, &pr, &o, hm.dt_lo, hm.dt_hi, hm.s_max, &out, s)
             : is_sde_alg(opt->alg) ? degpu_vectorized_solve_sde(f, &pr, &o, &out, s)
                                    : (adaptive ? degpu_internal_asolve_with_work(f, &pr, &o, &out, work, s)
                                                : degpu_vectorized_solve(f, &pr, &o, &out, s));
      }
      cudaFreeAsync(d, s);
      cudaError_t e = cudaStreamSynchronize(s);
      if (!rc && e != cudaSuccess) rc = fail(DEGPU_E_CUDA, std::string("solve failed: ") + cudaGetErrorString(e));
      return rc;
    }
  }

  // one device arena for inputs + outputs, freed stream-ordered at the end
  size_t off_u0 = 0, off_p = (off_u0 + n_u0 + 255) & ~(size_t)255, off_tsp = (off_p + n_p + 255) & ~(size_t)255;
  size_t off_sa = (off_tsp + n_tsp + 255) & ~(size_t)255, off_ts = (off_sa + n_sa + 255) & ~(size_t)255;
  size_t off_us = (off_ts + n_ts + 255) & ~(size_t)255, off_rc = (off_us + n_us + 255) & ~(size_t)255;
  size_t off_na = (off_rc + B + 255) & ~(size_t)255, off_nr = (off_na + 4 * B + 255) & ~(size_t)255;
  long long chunk = B;
  if (B >= 2 * 262144) chunk = std::max<long long>(262144, (B + 7) / 8);
  if (const char* e = getenv("DEGPU_HOST_CHUNK")) {
    long long v = atoll(e);
    if (v > 0) chunk = v;
  }
  const long long nchunks = (B + chunk - 1) / chunk;
  // one 256-byte persistent-driver work counter per chunk, so no chunk allocates on its own
  size_t off_work = (off_nr + 4 * B + 255) & ~(size_t)255;
  size_t total = off_work + 256 * (size_t)nchunks;
  char* d = nullptr;
  {
    int arc = lib_alloc((void**)&d, total, s);
    if (arc) return arc;
  }
  // Pipelined: the batch is cut into chunks of contiguous trajectories.  The chunks' solves
  // alternate between two compute streams (so one chunk's tail overlaps the next chunk's
  // start), and a third stream copies each finished chunk back while later chunks solve (the
  // copy engines and the SMs work at once).  Chunking changes no result: trajectories are
  // independent and the noise streams are keyed by the global trajectory index
  // (traj_offset).
  const bool piped = nchunks > 1;
  cudaStream_t comp[2] = {s, s}, out_s = s;
  cudaEvent_t ev_start = nullptr, ev_k[2] = {nullptr, nullptr}, ev_end[3] = {nullptr, nullptr, nullptr};
  int rc = 0;
  auto cleanup_streams = [&]() {
    for (int k = 0; k < 2; k++) {
      if (ev_k[k]) cudaEventDestroy(ev_k[k]);
      if (comp[k] != s) cudaStreamDestroy(comp[k]);
    }
    for (int k = 0; k < 3; k++)
      if (ev_end[k]) cudaEventDestroy(ev_end[k]);
    if (out_s != s) cudaStreamDestroy(out_s);
    if (ev_start) cudaEventDestroy(ev_start);
  };
  if (!rc && n_sa && !opt->saveat_per_traj &&
      cudaMemcpyAsync(d + off_sa, opt->saveat, n_sa, cudaMemcpyHostToDevice, s) != cudaSuccess)
    rc = fail(DEGPU_E_CUDA, "host-to-device copy failed");
  if (!rc && piped) {
    bool ok = cudaEventCreateWithFlags(&ev_start, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventRecord(ev_start, s) == cudaSuccess &&
              cudaStreamCreateWithFlags(&out_s, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamWaitEvent(out_s, ev_start, 0) == cudaSuccess;
    for (int k = 0; k < 2 && ok; k++)
      ok = cudaStreamCreateWithFlags(&comp[k], cudaStreamNonBlocking) == cudaSuccess &&
           cudaEventCreateWithFlags(&ev_k[k], cudaEventDisableTiming) == cudaSuccess &&
           cudaStreamWaitEvent(comp[k], ev_start, 0) == cudaSuccess;
    for (int k = 0; k < 3 && ok; k++) ok = cudaEventCreateWithFlags(&ev_end[k], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) rc = fail(DEGPU_E_CUDA, "pipeline stream set-up failed");
  }
  for (long long c0 = 0, ci = 0; c0 < B && !rc; c0 += chunk, ci++) {
    const long long nb = std::min(chunk, B - c0);
    cudaStream_t cs = comp[ci & 1];
    auto h2d = [&](size_t off, const void* src, size_t unit) {
      return unit == 0 || cudaMemcpyAsync(d + off + c0 * unit, (const char*)src + c0 * unit, nb * unit,
                                          cudaMemcpyHostToDevice, cs) == cudaSuccess;
    };
    auto d2h = [&](void* dst, size_t off, size_t unit) {
      return !dst || cudaMemcpyAsync((char*)dst + c0 * unit, d + off + c0 * unit, nb * unit, cudaMemcpyDeviceToHost,
                                     out_s) == cudaSuccess;
    };
    const size_t sa_unit = opt->saveat_per_traj ? (size_t)opt->nsaveat * tsz : 0;
    if (!h2d(off_u0, u0, N * 4) || !(P == 0 || h2d(off_p, p, P * 4)) || !h2d(off_tsp, tspan, 2 * tsz) ||
        !(sa_unit == 0 || h2d(off_sa, opt->saveat, sa_unit))) {
      rc = fail(DEGPU_E_CUDA, "host-to-device copy failed");
      break;
    }
    degpu_problems pr{(const float*)(d + off_u0) + c0 * N, (const float*)(d + off_p) + c0 * P,
                      d + off_tsp + c0 * 2 * tsz, nb};
    degpu_options o = *opt;
    o.traj_offset = opt->traj_offset + c0;
    if (n_sa) o.saveat = d + off_sa + c0 * sa_unit;
    if (o.dt0) o.dt0 = opt->dt0 + c0;  // per-trajectory device arrays of the whole batch
    if (o.tolscale) o.tolscale = opt->tolscale + c0;
    degpu_outputs out{d + off_ts + c0 * L * tsz, (float*)(d + off_us) + c0 * L * N, L,
                      retcode ? (signed char*)(d + off_rc) + c0 : nullptr, naccept ? (int*)(d + off_na) + c0 : nullptr,
                      nreject ? (int*)(d + off_nr) + c0 : nullptr, nullptr};
    unsigned long long* work = reinterpret_cast<unsigned long long*>(d + off_work + 256 * (size_t)ci);
    rc = learned ? degpu_learned_asolve_ex(f, hm.step, hm.work, &pr, &o, hm.dt_lo, hm.dt_hi, hm.s_max, &out, cs)
         : is_sde_alg(opt->alg) ? degpu_vectorized_solve_sde(f, &pr, &o, &out, cs)
                                : (adaptive ? degpu_internal_asolve_with_work(f, &pr, &o, &out, work, cs)
                                            : degpu_vectorized_solve(f, &pr, &o, &out, cs));
    if (rc) break;
    if (piped && (cudaEventRecord(ev_k[ci & 1], cs) != cudaSuccess ||
                  cudaStreamWaitEvent(out_s, ev_k[ci & 1], 0) != cudaSuccess)) {
      rc = fail(DEGPU_E_CUDA, "pipeline event failed");
      break;
    }
    if (!d2h(ts, off_ts, L * tsz) || !d2h(us, off_us, L * N * 4) || !d2h(retcode, off_rc, 1) ||
        !d2h(naccept, off_na, 4) || !d2h(nreject, off_nr, 4)) {
      rc = fail(DEGPU_E_CUDA, "device-to-host copy failed");
      break;
    }
  }
  if (piped && ev_end[2]) {  // join every pipeline stream back into the caller's stream
    cudaStream_t js[3] = {comp[0], comp[1], out_s};
    for (int k = 0; k < 3; k++) {
      cudaEventRecord(ev_end[k], js[k]);
      cudaStreamWaitEvent(s, ev_end[k], 0);
    }
  }
  cudaFreeAsync(d, s);
  cudaError_t e = cudaStreamSynchronize(s);
  cleanup_streams();
  if (!rc && e != cudaSuccess) rc = fail(DEGPU_E_CUDA, std::string("solve failed: ") + cudaGetErrorString(e));
  return rc;
}
}  // namespace

int degpu_batch_solve_host(const degpu_rhs* f, const float* u0, const float* p, const void* tspan, long long B,
                           const degpu_options* opt, int adaptive, void* ts, float* us, int L,
                           signed char* retcode, int* naccept, int* nreject, void* stream) {
  return batch_solve_host(f, HostModels{nullptr, nullptr, 0.0f, 0.0f, 0.0f}, u0, p, tspan, B, opt, adaptive, ts, us,
                          L, retcode, naccept, nreject, stream);
}

int degpu_learned_batch_solve_host(const degpu_rhs* f, const degpu_mlp* step_model, const degpu_mlp* work_model,
                                   const float* u0, const float* p, const void* tspan, long long B,
                                   const degpu_options* opt, float dt_lo, float dt_hi, float s_max, void* ts,
                                   float* us, int L, signed char* retcode, int* naccept, int* nreject, void* stream) {
  return batch_solve_host(f, HostModels{step_model, work_model, dt_lo, dt_hi, s_max}, u0, p, tspan, B, opt, 1, ts, us,
                          L, retcode, naccept, nreject, stream);
}

int degpu_rhs_check(const degpu_rhs* f, const degpu_options* opt, int adaptive, long long* cubin_bytes) {
  if (!f || !opt) return fail(DEGPU_E_INVALID, "null argument");
  Request rq;
  degpu_problems pr{nullptr, nullptr, nullptr, 0};
  degpu_outputs out{nullptr, nullptr, opt->nsaveat ? opt->nsaveat : 2, nullptr, nullptr, nullptr, nullptr};
  degpu_options o = *opt;
  if (!(o.dt > 0)) o.dt = 1.0;
  if (!o.nsaveat) o.save_everystep = 0;
  int rc = make_request(f, &pr, &o, adaptive, &out, &rq);
  if (rc) return rc;
  std::vector<char> cubin;
  rc = compile_cubin(build_source(f, rq.spec), rq.spec.parity != 0, cubin);
  if (rc) return rc;
  if (cubin_bytes) *cubin_bytes = (long long)cubin.size();
  return 0;
}

int degpu_kernel_info(const degpu_rhs* f, const degpu_options* opt, int adaptive, int* regs, int* local_bytes,
                      int* max_threads) {
  if (!f || !opt) return fail(DEGPU_E_INVALID, "null argument");
  Request rq;
  degpu_problems pr{nullptr, nullptr, nullptr, 0};
  degpu_outputs out{nullptr, nullptr, opt->nsaveat ? opt->nsaveat : 2, nullptr, nullptr, nullptr, nullptr};
  degpu_options o = *opt;
  if (!(o.dt > 0)) o.dt = 1.0;
  int rc = make_request(f, &pr, &o, adaptive, &out, &rq);
  if (rc) return rc;
  Kernel K;
  rc = get_kernel(f, rq.spec, &K);
  if (rc) return rc;
  if (regs) *regs = K.regs;
  if (local_bytes) *local_bytes = K.local_bytes;
  if (max_threads) *max_threads = K.max_threads;
  return 0;
}

int degpu_learned_asolve(const degpu_rhs* f, const degpu_mlp* m, const degpu_problems* probs, const degpu_options* opt,
                         float dt_lo, float dt_hi, float s_max, degpu_outputs* out, void* stream) {
  if (!m) return fail(DEGPU_E_INVALID, "null argument");
  return degpu_learned_asolve_ex(f, m, nullptr, probs, opt, dt_lo, dt_hi, s_max, out, stream);
}

int degpu_learned_asolve_ex(const degpu_rhs* f, const degpu_mlp* m, const degpu_mlp* work_model,
                            const degpu_problems* probs, const degpu_options* opt, float dt_lo, float dt_hi,
                            float s_max, degpu_outputs* out, void* stream) {
  if (!f || !probs || !opt || !out) return fail(DEGPU_E_INVALID, "null argument");
  if (probs->B < 0) return fail(DEGPU_E_INVALID, "negative trajectory count");
  if (probs->B == 0) return 0;
  if (m && (!(s_max >= 1.0f) || !(dt_lo > 0.0f) || !(dt_hi >= dt_lo))) return fail(DEGPU_E_INVALID, "bad dt / scale clamp");
  cudaStream_t s = (cudaStream_t)stream;
  const size_t B = (size_t)probs->B;
  // scratch: [dt0 | tolscale] (step model), [predicted work | order] (work model)
  const size_t n_step = m ? 2 * B : 0, n_work = work_model ? 2 * B : 0;
  float* scratch = nullptr;
  int rc = lib_alloc((void**)&scratch, sizeof(float) * (n_step + n_work), s);
  if (rc) return rc;
  degpu_options o = *opt;
  o.dt0 = nullptr;
  o.tolscale = nullptr;
  o.order = nullptr;
  const int span_f64 = opt->time_type == DEGPU_TIME_F64;
  if (m) {
    rc = degpu_internal_mlp_infer_problems(m, probs->u0, f->N, probs->p, f->P, probs->tspan, span_f64,
                                           (float)opt->reltol, probs->B, scratch, scratch + B, dt_lo, dt_hi, 1.0f,
                                           s_max, stream);
    if (rc) rc = fail(rc, "step-size model inference failed (input width must be N + P + 1, or N + P + 2 with the span)");
    o.dt0 = scratch;
    o.tolscale = scratch + B;
  }
  if (!rc && work_model) {
    // predicted attempts = exp(first output), clamped to [1, 2^31]; the second output is unused
    float* work = scratch + n_step;
    int* order = reinterpret_cast<int*>(scratch + n_step + B);
    rc = degpu_internal_mlp_infer_problems(work_model, probs->u0, f->N, probs->p, f->P, probs->tspan, span_f64,
                                           (float)opt->reltol, probs->B, work, nullptr, 1.0f, 2147483648.0f, 1.0f,
                                           1.0f, stream);
    if (rc) rc = fail(rc, "work model inference failed (input width must be N + P + 1, or N + P + 2 with the span)");
    if (!rc) rc = degpu_work_order(work, probs->B, order, stream);
    o.order = order;
  }
  if (!rc) rc = degpu_vectorized_asolve(f, probs, &o, out, stream);
  cudaFreeAsync(scratch, s);
  return rc;
}

// ------------------------------------------------------------------ autotuner
int degpu_autotune(const degpu_rhs* f, const degpu_problems* probs, const degpu_options* opt, int adaptive,
                   degpu_outputs* out, long long sample_B, void* stream, int* best_block, int* best_chunk) {
  Request rq;
  int rc = make_request(f, probs, opt, adaptive, out, &rq);
  if (rc) return rc;
  if (rq.kp.B == 0) return fail(DEGPU_E_INVALID, "cannot autotune an empty ensemble");
  Kernel K;
  rc = get_kernel(f, rq.spec, &K);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  Request sample = rq;
  if (sample_B > 0 && sample_B < sample.kp.B) sample.kp.B = sample_B;
  const int blocks[] = {64, 128, 256};
  std::vector<int> chunks = {0};
  if (rq.spec.driver == 2) chunks = {32, 64, 128};
  unsigned long long* work = nullptr;
  rc = lib_alloc((void**)&work, 256, s);
  if (rc) return rc;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  int bb = default_block(rq), bc = default_chunk();
  for (int b : blocks) {
    if (b > K.max_threads) continue;
    for (int c : chunks) {
      int cc = c ? c : default_chunk();
      rc = launch(sample, K, b, cc, work, (CUstream)s);  // warm-up
      if (rc) break;
      float tot = 0.f;
      for (int rep = 0; rep < 2 && !rc; rep++) {
        cudaEventRecord(e0, s);
        rc = launch(sample, K, b, cc, work, (CUstream)s);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        tot += ms;
      }
      if (rc) break;
      if (tot < best) { best = tot; bb = b; bc = cc; }
    }
    if (rc) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(work, s);
  if (rc) return rc;
  CUDA_TRY(cudaStreamSynchronize(s));
  {
    std::lock_guard<std::mutex> lk(g_mu);
    char key[64];
    snprintf(key, sizeof key, "%p|%lld", (void*)K.fn, (long long)(rq.kp.B >> 16));
    g_tuned[key] = {bb, bc};
  }
  if (best_block) *best_block = bb;
  if (best_chunk) *best_chunk = bc;
  return 0;
}

}  // extern "C"

// ------------------------------------------------------------------ plans (CUDA graphs)
struct degpu_plan_s {
  Request rq;
  Kernel K;
  int block = 0, chunk = 0, grid = 0;
  unsigned long long* work = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

extern "C" {

int degpu_plan_create(const degpu_rhs* f, const degpu_problems* probs, const degpu_options* opt, int adaptive,
                      degpu_outputs* out, void* stream, degpu_plan** plan) {
  if (!plan) return fail(DEGPU_E_INVALID, "null plan");
  std::unique_ptr<degpu_plan_s> pl(new degpu_plan_s);
  int rc = make_request(f, probs, opt, adaptive, out, &pl->rq);
  if (rc) return rc;
  if (pl->rq.kp.B == 0) return fail(DEGPU_E_INVALID, "cannot plan an empty ensemble");
  rc = get_kernel(f, pl->rq.spec, &pl->K);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  pl->block = opt->block;
  pl->chunk = opt->chunk;
  if (!pl->block) {
    long long sample = std::min<long long>(pl->rq.kp.B, 1LL << 18);
    rc = degpu_autotune(f, probs, opt, adaptive, out, sample, stream, &pl->block, &pl->chunk);
    if (rc) return rc;
  }
  if (!pl->chunk) pl->chunk = default_chunk();
  CUDA_TRY(cudaMalloc((void**)&pl->work, 256));
  pl->grid = grid_for(pl->rq, pl->K, pl->block);
  cudaStream_t cap;
  CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
  CUDA_TRY(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
  rc = launch(pl->rq, pl->K, pl->block, pl->chunk, pl->work, (CUstream)cap);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(cap, &g);
  cudaStreamDestroy(cap);
  if (rc) { if (g) cudaGraphDestroy(g); cudaFree(pl->work); return rc; }
  if (e != cudaSuccess) { cudaFree(pl->work); return fail(DEGPU_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(e)); }
  pl->graph = g;
  e = cudaGraphInstantiate(&pl->exec, g, 0);
  if (e != cudaSuccess) { cudaGraphDestroy(g); cudaFree(pl->work); return fail(DEGPU_E_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e)); }
  (void)s;
  *plan = pl.release();
  return 0;
}

int degpu_plan_launch(degpu_plan* plan, void* stream) {
  if (!plan) return fail(DEGPU_E_INVALID, "null plan");
  CUDA_TRY(cudaGraphLaunch(plan->exec, (cudaStream_t)stream));
  return 0;
}

int degpu_plan_info(const degpu_plan* plan, int* block, int* chunk, int* grid, int* driver, int* regs) {
  if (!plan) return fail(DEGPU_E_INVALID, "null plan");
  if (block) *block = plan->block;
  if (chunk) *chunk = plan->chunk;
  if (grid) *grid = plan->grid;
  if (driver) *driver = plan->rq.spec.driver;
  if (regs) *regs = plan->K.regs;
  return 0;
}

void degpu_plan_destroy(degpu_plan* plan) {
  if (!plan) return;
  if (plan->exec) cudaGraphExecDestroy(plan->exec);
  if (plan->graph) cudaGraphDestroy(plan->graph);
  if (plan->work) cudaFree(plan->work);
  delete plan;
}

}  // extern "C"

// ------------------------------------------------------------------ internal helpers
int degpu_internal_rhs_dims(const degpu_rhs* f, int* n_state, int* n_param) {
  if (!f) return fail(DEGPU_E_INVALID, "null right-hand side");
  if (n_state) *n_state = f->N;
  if (n_param) *n_param = f->P;
  return 0;
}

int degpu_internal_fail(int code, const char* msg) { return fail(code, msg ? msg : ""); }

int degpu_internal_alloc(void** p, size_t n, void* stream) { return lib_alloc(p, n, (cudaStream_t)stream); }

int degpu_internal_asolve_with_work(const degpu_rhs* f, const degpu_problems* probs, const degpu_options* opt,
                                    degpu_outputs* out, unsigned long long* work, void* stream) {
  Request rq;
  int rc = make_request(f, probs, opt, 1, out, &rq);
  if (rc) return rc;
  if (rq.kp.B == 0) return 0;
  Kernel K;
  rc = get_kernel(f, rq.spec, &K);
  if (rc) return rc;
  int block = rq.block ? rq.block : default_block(rq);
  int chunk = rq.chunk ? rq.chunk : default_chunk();
  {
    std::lock_guard<std::mutex> lk(g_mu);
    char key[64];
    snprintf(key, sizeof key, "%p|%lld", (void*)K.fn, (long long)(rq.kp.B >> 16));
    auto it = g_tuned.find(key);
    if (!rq.block && it != g_tuned.end()) { block = it->second.first; if (!rq.chunk) chunk = it->second.second; }
  }
  if (rq.spec.driver == 2 && !work) return fail(DEGPU_E_INVALID, "persistent driver needs a work counter");
  return launch(rq, K, block, chunk, work, (CUstream)stream);
}
