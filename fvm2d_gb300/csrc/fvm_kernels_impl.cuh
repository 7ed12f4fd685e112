// fvm_kernels_impl.cuh -- launcher definitions for one state precision R.
// Included once per precision translation unit.
#pragma once

#include "fvm_kernels.cuh"
#include "fvm_launch.h"

namespace fvm {

#define FVM_DEFINE_LAUNCHERS(R)                                                            \
  size_t smem_grad(const LaunchCfg &c, R *) {                                              \
    return size_t(c.max_tri) * (sizeof(TriSmem<R>) + (c.viscous ? 9 * sizeof(R) : 0));     \
  }                                                                                        \
  size_t smem_flux(const LaunchCfg &c, R *) { return size_t(c.max_slots) * sizeof(R4<R>); } \
  size_t smem_sa(const LaunchCfg &c, R *) {                                                \
    return size_t(3 * c.max_tri + c.max_slots) * sizeof(R) + 16;                           \
  }                                                                                        \
  cudaError_t launch_visc(const ArenaPtrs<R> &A, const LaunchCfg &c, int stage, int do_dt,  \
                          int routine) {                                                   \
    k_visc<R><<<c.grid, kBlockVerts, 0, c.stream>>>(A, stage, do_dt, routine);             \
    return cudaGetLastError();                                                             \
  }                                                                                        \
  cudaError_t launch_grad(const ArenaPtrs<R> &A, const LaunchCfg &c, int stage, int do_dt,  \
                          int routine) {                                                   \
    size_t sm = smem_grad(c, (R *)nullptr);                                                \
    if (sm > kMaxSmem) return cudaErrorInvalidConfiguration;                              \
    k_grad<R><<<c.grid, kBlockVerts, sm, c.stream>>>(A, stage, do_dt, routine, c.max_tri);  \
    return cudaGetLastError();                                                             \
  }                                                                                        \
  cudaError_t launch_flux(const ArenaPtrs<R> &A, const LaunchCfg &c, int stage, int mode,   \
                          int irk, int routine) {                                          \
    size_t sm = smem_flux(c, (R *)nullptr);                                                \
    if (sm > kMaxSmem) return cudaErrorInvalidConfiguration;                              \
    switch (c.flux) {                                                                      \
      case 1: k_flux<R, 1><<<c.grid, kBlockVerts, sm, c.stream>>>(A, stage, mode, irk, routine); break; \
      case 2: k_flux<R, 2><<<c.grid, kBlockVerts, sm, c.stream>>>(A, stage, mode, irk, routine); break; \
      case 3: k_flux<R, 3><<<c.grid, kBlockVerts, sm, c.stream>>>(A, stage, mode, irk, routine); break; \
      default: k_flux<R, 0><<<c.grid, kBlockVerts, sm, c.stream>>>(A, stage, mode, irk, routine); \
    }                                                                                      \
    return cudaGetLastError();                                                             \
  }                                                                                        \
  cudaError_t launch_sa(const ArenaPtrs<R> &A, const LaunchCfg &c, int stage, int routine) {\
    size_t sm = smem_sa(c, (R *)nullptr);                                                  \
    if (sm > kMaxSmem) return cudaErrorInvalidConfiguration;                              \
    k_sa<R><<<c.grid, kBlockVerts, sm, c.stream>>>(A, stage, routine, c.max_tri);           \
    return cudaGetLastError();                                                             \
  }                                                                                        \
  cudaError_t launch_monitor(const ArenaPtrs<R> &A, const LaunchCfg &c, int serial_clcd) {  \
    if (A.nslots <= 0) return cudaSuccess;                                                 \
    k_monitor<R><<<A.nslots, 256, 0, c.stream>>>(A, serial_clcd);                          \
    return cudaGetLastError();                                                             \
  }                                                                                        \
  cudaError_t launch_update(const ArenaPtrs<R> &A, const LaunchCfg &c, int irk) {           \
    k_update<R><<<c.grid, kBlockVerts, 0, c.stream>>>(A, irk);                             \
    return cudaGetLastError();                                                             \
  }                                                                                        \
  cudaError_t launch_time_step(const ArenaPtrs<R> &A, const LaunchCfg &c) {                 \
    k_time_step<R><<<c.grid, kBlockVerts, 0, c.stream>>>(A);                               \
    return cudaGetLastError();                                                             \
  }                                                                                        \
  cudaError_t launch_positivity(const ArenaPtrs<R> &A, const LaunchCfg &c) {                \
    k_positivity<R><<<c.grid, kBlockVerts, 0, c.stream>>>(A);                              \
    return cudaGetLastError();                                                             \
  }                                                                                        \
  cudaError_t launch_conres(const ArenaPtrs<R> &A, const LaunchCfg &c, int mesh, int first) {\
    k_conres_part<R><<<c.grid, kBlockVerts, 0, c.stream>>>(A);                             \
    k_routine_monitor<R><<<1, 256, 0, c.stream>>>(A, mesh, 0, first, 0);                    \
    return cudaGetLastError();                                                             \
  }                                                                                        \
  cudaError_t launch_clcd(const ArenaPtrs<R> &A, const LaunchCfg &c, int mesh, int serial) { \
    k_routine_monitor<R><<<1, 256, 0, c.stream>>>(A, mesh, 1, 0, serial);                   \
    return cudaGetLastError();                                                             \
  }                                                                                        \
  cudaError_t launch_limitgrad(const ArenaPtrs<R> &A, const LaunchCfg &c) {                 \
    k_limitgrad<R><<<c.grid, kBlockVerts, 0, c.stream>>>(A);                               \
    return cudaGetLastError();                                                             \
  }                                                                                        \
  cudaError_t prepare_attributes(const LaunchCfg &c, R *) {                                \
    const size_t g = smem_grad(c, (R *)nullptr), f = smem_flux(c, (R *)nullptr),           \
                 s = smem_sa(c, (R *)nullptr);                                             \
    if (g > kMaxSmem || f > kMaxSmem || s > kMaxSmem) return cudaErrorInvalidConfiguration; \
    cudaError_t e = cudaFuncSetAttribute(k_grad<R>,                                        \
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g); \
    if (e == cudaSuccess)                                                                  \
      e = cudaFuncSetAttribute(k_flux<R, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)f); \
    if (e == cudaSuccess)                                                                  \
      e = cudaFuncSetAttribute(k_flux<R, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)f); \
    if (e == cudaSuccess)                                                                  \
      e = cudaFuncSetAttribute(k_flux<R, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)f); \
    if (e == cudaSuccess)                                                                  \
      e = cudaFuncSetAttribute(k_flux<R, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)f); \
    if (e == cudaSuccess)                                                                  \
      e = cudaFuncSetAttribute(k_sa<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s); \
    return e;                                                                              \
  }

}  // namespace fvm
