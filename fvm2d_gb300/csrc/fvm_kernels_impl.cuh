// fvm_kernels_impl.cuh -- launcher definitions for one state precision R.
// Included once per precision translation unit.
#pragma once

#include "fvm_kernels.cuh"
#include "fvm_launch.h"

namespace fvm {

// Grid of a persistent per-block kernel: one wave of the CTAs that fit on
// the device at once (its occupancy with this shared memory), so that no
// partial second wave idles most SMs at the end of a launch.
template <typename K>
inline int fit_grid(const LaunchCfg &c, K kern, size_t smem, int threads = kBlockVerts) {
  if (!c.fit) return c.grid;
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, smem) != cudaSuccess) {
    (void)cudaGetLastError();
    occ = 1;
  }
  const int g = (occ < 1 ? 1 : occ) * c.sms;
  return g < c.grid ? g : c.grid;
}

// The flux pass for template code F (Riemann solver | kFluxStd).
template <typename R, int F>
inline void launch_flux_code(const ArenaPtrs<R> &A, const LaunchCfg &c, size_t sm, int nt,
                             int stage, int mode, int irk, int routine) {
  k_flux<R, F><<<fit_grid(c, k_flux<R, F>, sm, nt), nt, sm, c.stream>>>(A, stage, mode, irk,
                                                                         routine);
}
template <typename R>
inline void launch_flux_any(const ArenaPtrs<R> &A, const LaunchCfg &c, size_t sm, int nt,
                            int stage, int mode, int irk, int routine) {
  if constexpr (sizeof(R) == 4) {
    if (c.std_const) {
      switch (c.flux) {
        case 1: launch_flux_code<R, 1 | kFluxStd>(A, c, sm, nt, stage, mode, irk, routine); return;
        case 2: launch_flux_code<R, 2 | kFluxStd>(A, c, sm, nt, stage, mode, irk, routine); return;
        case 3: launch_flux_code<R, 3 | kFluxStd>(A, c, sm, nt, stage, mode, irk, routine); return;
        default: launch_flux_code<R, kFluxStd>(A, c, sm, nt, stage, mode, irk, routine); return;
      }
    }
  }
  switch (c.flux) {
    case 1: launch_flux_code<R, 1>(A, c, sm, nt, stage, mode, irk, routine); return;
    case 2: launch_flux_code<R, 2>(A, c, sm, nt, stage, mode, irk, routine); return;
    case 3: launch_flux_code<R, 3>(A, c, sm, nt, stage, mode, irk, routine); return;
    default: launch_flux_code<R, 0>(A, c, sm, nt, stage, mode, irk, routine); return;
  }
}
// dynamic shared memory attribute of every flux-pass instantiation
template <typename R>
inline cudaError_t flux_attributes(size_t f) {
  const int b = (int)f;
  cudaError_t e = cudaFuncSetAttribute(k_flux<R, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_flux<R, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_flux<R, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_flux<R, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  if constexpr (sizeof(R) == 4) {
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_flux<R, kFluxStd>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_flux<R, 1 | kFluxStd>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_flux<R, 2 | kFluxStd>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_flux<R, 3 | kFluxStd>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  }
  return e;
}

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
    k_visc<R><<<fit_grid(c, k_visc<R>, 0), kBlockVerts, 0, c.stream>>>(A, stage, do_dt, routine);             \
    return cudaGetLastError();                                                             \
  }                                                                                        \
  cudaError_t launch_grad_pipe(const ArenaPtrs<R> &A, const LaunchCfg &c, int stage,       \
                               int do_dt, int routine, long long budget, int inject,      \
                               int skip_inviscid) {                                       \
    if (sizeof(R) != 4 || !c.tri_loc) return cudaErrorNotSupported;                      \
    const GradPipeLayout pl = grad_pipe_layout(c.max_tri, c.max_halo, c.viscous);         \
    const int groups = c.pipe_groups == 1 ? 1 : 2;                                        \
    const int ns = pipe_stage_count(pl.stage, groups, c.pipe_stages);                      \
    if (!ns) return cudaErrorNotSupported;                                                 \
    const size_t sb = (size_t)ns * pl.stage;                                               \
    const int vis = c.viscous ? 1 : 0;                                                     \
    if (groups == 1)                                                                       \
      k_grad_pipe<R, 1><<<fit_grid(c, k_grad_pipe<R, 1>, sb, 32 + kBlockVerts),            \
                          32 + kBlockVerts, sb, c.stream>>>(A, stage, do_dt, routine,      \
                          c.max_tri, c.max_halo, vis, ns, budget, inject, skip_inviscid);  \
    else                                                                                   \
      k_grad_pipe<R, 2><<<fit_grid(c, k_grad_pipe<R, 2>, sb, 32 + 2 * kBlockVerts),        \
                          32 + 2 * kBlockVerts, sb, c.stream>>>(A, stage, do_dt, routine,  \
                          c.max_tri, c.max_halo, vis, ns, budget, inject, skip_inviscid);  \
    return cudaGetLastError();                                                             \
  }                                                                                        \
  cudaError_t launch_grad(const ArenaPtrs<R> &A, const LaunchCfg &c, int stage, int do_dt,  \
                          int routine) {                                                   \
    size_t sm = smem_grad(c, (R *)nullptr);                                                \
    if (sm > kMaxSmem) return cudaErrorInvalidConfiguration;                              \
    /* FP32: inviscid meshes take the vertex-stencil pass, viscous ones the */             \
    /* triangle pass below */                                                              \
    int skip = 0;                                                                          \
    if (sizeof(R) == 4 && c.stencil) {                                                     \
      if (c.any_inviscid) {                                                                \
        k_grad_stencil<R><<<fit_grid(c, k_grad_stencil<R>, 0), kBlockVerts, 0, c.stream>>>( \
            A, stage, do_dt, routine);                                                     \
        const cudaError_t se = cudaGetLastError();                                         \
        if (se != cudaSuccess) return se;                                                  \
      }                                                                                    \
      if (!c.viscous) return cudaSuccess;                                                  \
      skip = 1;                                                                            \
    }                                                                                      \
    if (c.grad_mode == 4 && sizeof(R) == 4 && c.tri_loc) {                                 \
      const cudaError_t pe = launch_grad_pipe(A, c, stage, do_dt, routine, kPipeBudget, 0, \
                                              skip);                                       \
      if (pe != cudaErrorNotSupported) return pe;                                          \
    }                                                                                      \
    if (c.grad_mode == 2) {                                                                \
      k_grad_v<R><<<fit_grid(c, k_grad_v<R>, 0), kBlockVerts, 0, c.stream>>>(A, stage, do_dt, routine, skip); \
      return cudaGetLastError();                                                           \
    }                                                                                      \
    if (c.grad_mode >= 3 && c.tri_loc) {  /* else the per-thread form, same sums */      \
      if (sizeof(R) != 4) return cudaErrorNotSupported;                                    \
      const size_t sb = grad_bulk_layout(c.max_tri, c.max_halo, c.viscous).total;          \
      if (sb > kMaxSmem) return cudaErrorInvalidConfiguration;                            \
      k_grad_bulk<R><<<fit_grid(c, k_grad_bulk<R>, sb), kBlockVerts, sb, c.stream>>>(       \
          A, stage, do_dt, routine, c.max_tri, c.max_halo, c.viscous ? 1 : 0, skip);       \
      return cudaGetLastError();                                                           \
    }                                                                                      \
    k_grad<R><<<fit_grid(c, k_grad<R>, sm), kBlockVerts, sm, c.stream>>>(A, stage, do_dt, routine, c.max_tri, skip);  \
    return cudaGetLastError();                                                             \
  }                                                                                        \
  cudaError_t launch_flux(const ArenaPtrs<R> &A, const LaunchCfg &c, int stage, int mode,   \
                          int irk, int routine) {                                          \
    size_t sm = smem_flux(c, (R *)nullptr);                                                \
    if (sm > kMaxSmem) return cudaErrorInvalidConfiguration;                              \
    const int nt = sizeof(R) == 4 ? kFluxThreads : kBlockVerts;                           \
    launch_flux_any<R>(A, c, sm, nt, stage, mode, irk, routine);                           \
    return cudaGetLastError();                                                             \
  }                                                                                        \
  size_t smem_step(const LaunchCfg &c, R *) {                                              \
    const size_t tri = size_t(c.max_tri2) * sizeof(TriSmem<R>) +                           \
                       (c.viscous ? size_t(c.max_tri) * 9 * sizeof(R) : 0);                 \
    const size_t flx = size_t(c.max_slots) * sizeof(R4<R>);                                \
    const size_t r1 = ((tri > flx ? tri : flx) + 63) & ~size_t(63);                        \
    return r1 + size_t(c.max_loc) * sizeof(Grad<R>);                                       \
  }                                                                                        \
  cudaError_t launch_step(const ArenaPtrs<R> &A, const LaunchCfg &c, int stage) {           \
    const size_t sm = smem_step(c, (R *)nullptr);                                          \
    if (sm > kMaxSmem) return cudaErrorInvalidConfiguration;                              \
    const int v = c.viscous ? 1 : 0;                                                       \
    switch (c.flux) {                                                                      \
      case 1: k_step<R, 1><<<fit_grid(c, k_step<R, 1>, sm), kBlockVerts, sm, c.stream>>>(A, stage, c.max_tri, c.max_tri2, c.max_slots, c.max_loc, v); break; \
      case 2: k_step<R, 2><<<fit_grid(c, k_step<R, 2>, sm), kBlockVerts, sm, c.stream>>>(A, stage, c.max_tri, c.max_tri2, c.max_slots, c.max_loc, v); break; \
      case 3: k_step<R, 3><<<fit_grid(c, k_step<R, 3>, sm), kBlockVerts, sm, c.stream>>>(A, stage, c.max_tri, c.max_tri2, c.max_slots, c.max_loc, v); break; \
      default: k_step<R, 0><<<fit_grid(c, k_step<R, 0>, sm), kBlockVerts, sm, c.stream>>>(A, stage, c.max_tri, c.max_tri2, c.max_slots, c.max_loc, v); \
    }                                                                                      \
    return cudaGetLastError();                                                             \
  }                                                                                        \
  cudaError_t launch_sa(const ArenaPtrs<R> &A, const LaunchCfg &c, int stage, int routine) {\
    size_t sm = smem_sa(c, (R *)nullptr);                                                  \
    if (sm > kMaxSmem) return cudaErrorInvalidConfiguration;                              \
    k_sa<R><<<fit_grid(c, k_sa<R>, sm), kBlockVerts, sm, c.stream>>>(A, stage, routine, c.max_tri);           \
    return cudaGetLastError();                                                             \
  }                                                                                        \
  cudaError_t launch_monitor(const ArenaPtrs<R> &A, const LaunchCfg &c, int serial_clcd) {  \
    if (A.nslots <= 0) return cudaSuccess;                                                 \
    k_monitor<R><<<A.nslots, monitor_threads<R>(), 0, c.stream>>>(A, serial_clcd);         \
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
  cudaError_t launch_gradient_edge(const ArenaPtrs<R> &A, const LaunchCfg &c) {             \
    const size_t sm = size_t(c.max_slots) * sizeof(Grad<R>);                                 \
    if (sm > kMaxSmem) return cudaErrorInvalidConfiguration;                              \
    k_gradient_edge<R><<<c.grid, kBlockVerts, sm, c.stream>>>(A);                          \
    return cudaGetLastError();                                                             \
  }                                                                                        \
  cudaError_t launch_shockind(const ArenaPtrs<R> &A, const LaunchCfg &c) {                  \
    k_shockind<R><<<c.grid, kBlockVerts, 0, c.stream>>>(A);                                \
    return cudaGetLastError();                                                             \
  }                                                                                        \
  cudaError_t launch_limitgrad(const ArenaPtrs<R> &A, const LaunchCfg &c) {                 \
    k_limitgrad<R><<<c.grid, kBlockVerts, 0, c.stream>>>(A);                               \
    return cudaGetLastError();                                                             \
  }                                                                                        \
  cudaError_t prepare_attributes(const LaunchCfg &c, R *) {                                \
    const size_t g = smem_grad(c, (R *)nullptr), f = smem_flux(c, (R *)nullptr),           \
                 s = smem_sa(c, (R *)nullptr);                                             \
    const size_t st = smem_step(c, (R *)nullptr);                                          \
    if (g > kMaxSmem || f > kMaxSmem || s > kMaxSmem || st > kMaxSmem)                     \
      return cudaErrorInvalidConfiguration;                                                \
    for (int k = 0; k < 4; k++) {                                                          \
      cudaError_t e2 = cudaSuccess;                                                        \
      if (k == 0) e2 = cudaFuncSetAttribute(k_step<R, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)st); \
      if (k == 1) e2 = cudaFuncSetAttribute(k_step<R, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)st); \
      if (k == 2) e2 = cudaFuncSetAttribute(k_step<R, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)st); \
      if (k == 3) e2 = cudaFuncSetAttribute(k_step<R, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)st); \
      if (e2 != cudaSuccess) return e2;                                                    \
    }                                                                                      \
    cudaError_t e = cudaFuncSetAttribute(k_grad<R>,                                        \
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g); \
    if (e == cudaSuccess) e = flux_attributes<R>(f);                                       \
    if (e == cudaSuccess)                                                                  \
      e = cudaFuncSetAttribute(k_sa<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s); \
    const size_t gb = grad_bulk_layout(c.max_tri, kTriLocMax, c.viscous).total;            \
    if (e == cudaSuccess && sizeof(R) == 4 && gb <= kMaxSmem)                              \
      e = cudaFuncSetAttribute(k_grad_bulk<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gb); \
    const size_t ge = size_t(c.max_slots) * sizeof(Grad<R>);                                 \
    if (e == cudaSuccess && ge <= kMaxSmem)                                                \
      e = cudaFuncSetAttribute(k_gradient_edge<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ge); \
    const int pmax = (int)(kMaxSmem - kPipeStaticSmem);                                    \
    if (e == cudaSuccess && sizeof(R) == 4)                                                \
      e = cudaFuncSetAttribute(k_grad_pipe<R, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, pmax); \
    if (e == cudaSuccess && sizeof(R) == 4)                                                \
      e = cudaFuncSetAttribute(k_grad_pipe<R, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, pmax); \
    return e;                                                                              \
  }

}  // namespace fvm
