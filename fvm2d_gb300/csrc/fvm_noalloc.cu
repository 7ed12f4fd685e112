// fvm_noalloc.cu -- the density-residual norm of conres.f:11-31 for callers
// that cannot allocate device memory.
//
// Some drivers own every byte of device memory themselves: a Fortran code
// whose state lives in OpenACC or CUDA Fortran data regions, or a process
// whose memory is managed by another framework's pool.  They cannot let a
// library call cudaMalloc (which also synchronises the whole device and can
// fail under memory pressure in the middle of a run).  This entry point
// takes the driver's own device arrays and needs no allocation: its scratch
// (one partial sum per 256 vertices) is the file-scope array below, which
// every GPU that loads this library holds until the process exits.
#include <climits>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/fvm_gpu.h"

namespace {

constexpr int kThreads = 256;
constexpr int kMaxParts = FVM_NOALLOC_MAX_POINTS / kThreads;
constexpr int kMaxDevices = 64;

struct Partial {
  double sumsq;
  double maxabs;
  int argmax;   // 1-based point index; INT_MAX when no change
  int pad;
};

struct Result {
  double sumsq;
  double maxabs;
  int argmax;
  int pad;
};
static_assert(sizeof(Partial) == 24 && sizeof(Result) == 24, "scratch record sizes");

// The scratch: partials of the first pass, and the reduced result.  Shared
// by every call on a device; each call overwrites the partials it reads.
static __device__ __align__(256) Partial g_parts[kMaxParts];
static __device__ __align__(256) Result g_result;

std::mutex g_mu;
Partial *g_parts_addr[kMaxDevices];
Result *g_result_addr[kMaxDevices];
bool g_ready[kMaxDevices];

__device__ __forceinline__ void combine(double &s, double &m, int &a, double os, double om, int oa) {
  s += os;
  if (om > m || (om == m && oa < a)) {
    m = om;
    a = oa;
  }
}

// pass 1: one partial per CTA of kThreads consecutive points
__global__ void __launch_bounds__(kThreads) k_parts(const double *__restrict__ prim,
                                                    const double *__restrict__ prim_old, int np,
                                                    Partial *parts) {
  __shared__ double s_s[kThreads / 32], s_m[kThreads / 32];
  __shared__ int s_a[kThreads / 32];
  const int i = blockIdx.x * kThreads + threadIdx.x;
  double s = 0.0, m = 0.0;
  int a = INT_MAX;
  if (i < np) {
    const double gra = prim[4 * (size_t)i] - prim_old[4 * (size_t)i];   // conres.f:15
    s = gra * gra;
    m = fabs(gra);
    // conres.f:17-21 takes a point only when |gra| > fresi, which a NaN
    // never is: a NaN poisons the sum of squares but not the maximum
    if (m > 0.0) a = i + 1;
    else m = 0.0;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
    combine(s, m, a, __shfl_down_sync(0xffffffffu, s, off), __shfl_down_sync(0xffffffffu, m, off),
            __shfl_down_sync(0xffffffffu, a, off));
  if ((threadIdx.x & 31) == 0) {
    s_s[threadIdx.x >> 5] = s;
    s_m[threadIdx.x >> 5] = m;
    s_a[threadIdx.x >> 5] = a;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < kThreads / 32; w++) combine(s, m, a, s_s[w], s_m[w], s_a[w]);
    Partial p;
    p.sumsq = s;
    p.maxabs = m;
    p.argmax = a;
    p.pad = 0;
    parts[blockIdx.x] = p;
  }
}

// pass 2: one CTA folds the partials of this call in a fixed order
__global__ void __launch_bounds__(kThreads) k_final(const Partial *parts, int nparts, Result *out) {
  __shared__ double s_s[kThreads], s_m[kThreads];
  __shared__ int s_a[kThreads];
  double s = 0.0, m = 0.0;
  int a = INT_MAX;
  for (int k = threadIdx.x; k < nparts; k += kThreads) combine(s, m, a, parts[k].sumsq, parts[k].maxabs, parts[k].argmax);
  s_s[threadIdx.x] = s;
  s_m[threadIdx.x] = m;
  s_a[threadIdx.x] = a;
  __syncthreads();
  for (int st = kThreads / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) {
      double ss = s_s[threadIdx.x], mm = s_m[threadIdx.x];
      int aa = s_a[threadIdx.x];
      combine(ss, mm, aa, s_s[threadIdx.x + st], s_m[threadIdx.x + st], s_a[threadIdx.x + st]);
      s_s[threadIdx.x] = ss;
      s_m[threadIdx.x] = mm;
      s_a[threadIdx.x] = aa;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    Result r;
    r.sumsq = s_s[0];
    r.maxabs = s_m[0];
    r.argmax = s_a[0];
    r.pad = 0;
    *out = r;
  }
}

// Device addresses of the scratch on the current device (looked up once per
// device, with that device current).
cudaError_t scratch_of(Partial **parts, Result **result) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_ready[dev]) {
    void *p = nullptr, *r = nullptr;
    e = cudaGetSymbolAddress(&p, g_parts);
    if (e != cudaSuccess) return e;
    e = cudaGetSymbolAddress(&r, g_result);
    if (e != cudaSuccess) return e;
    g_parts_addr[dev] = static_cast<Partial *>(p);
    g_result_addr[dev] = static_cast<Result *>(r);
    g_ready[dev] = true;
  }
  *parts = g_parts_addr[dev];
  *result = g_result_addr[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" int32_t fvm_gpu_conres_noalloc(const double *prim, const double *prim_old, int32_t np,
                                          int32_t first, double *fres1, double *fres,
                                          double *fresi, int32_t *iresi) {
  if (!prim || !prim_old || !fres1 || np < 1) return FVM_ERR_ARG;
  if (np > FVM_NOALLOC_MAX_POINTS) return FVM_ERR_ARG;   // beyond the static scratch
  Partial *parts = nullptr;
  Result *res = nullptr;
  cudaError_t e = scratch_of(&parts, &res);
  if (e != cudaSuccess) return FVM_ERR_CUDA;
  const int nparts = (np + kThreads - 1) / kThreads;
  k_parts<<<nparts, kThreads, 0, 0>>>(prim, prim_old, np, parts);
  k_final<<<1, kThreads, 0, 0>>>(parts, nparts, res);
  if ((e = cudaGetLastError()) != cudaSuccess) return FVM_ERR_CUDA;
  Result r;
  if ((e = cudaMemcpy(&r, res, sizeof(r), cudaMemcpyDeviceToHost)) != cudaSuccess) return FVM_ERR_CUDA;
  const double raw = sqrt(r.sumsq / np);             // conres.f:23
  if (fresi) *fresi = r.maxabs;
  if (iresi) *iresi = r.maxabs > 0.0 ? r.argmax : 0;
  if (first) {                                       // conres.f:25-29
    *fres1 = raw;
    if (raw == 0.0) {
      if (fres) *fres = raw;
      return FVM_ERR_ZERO_FIRST_RES;
    }
  } else if (!(*fres1 > 0.0)) {
    return FVM_ERR_ARG;
  }
  if (fres) *fres = raw / *fres1;                    // conres.f:31
  return FVM_OK;
}
