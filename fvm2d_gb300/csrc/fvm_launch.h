// fvm_launch.h -- host-callable launchers of the hot-path kernels, one set
// per state precision (definitions in fvm_kernels_fp64.cu / _fp32.cu).
#pragma once

#include <cuda_runtime.h>

#include "fvm_internal.h"

namespace fvm {

constexpr size_t kMaxSmem = 227 * 1024;   // dynamic shared memory per CTA

struct LaunchCfg {
  int grid;          // CTAs of the per-block kernels (persistent loop)
  int max_tri;       // max triangle entries of any block
  int max_slots;     // max edge slots (interior + 2 x boundary) of any block
  bool viscous;      // any mesh viscous (gradient-pass shared memory)
  int flux;          // 1/2/3: every mesh uses that Riemann solver; 0: mixed
  int max_tri2;      // max triangles of a block plus those of its halo
  int max_loc;       // max own + halo vertices of a block
  int sms;           // multiprocessors of the device
  bool fit;          // grid = CTAs resident at once (occupancy x sms), capped by grid
  int grad_mode;     // gradient pass: 1 loads per thread (k_grad), 2 per vertex
                     // (k_grad_v), 3 bulk copies to shared memory (k_grad_bulk, FP32)
  int max_halo;      // max halo vertices of a block (k_grad_bulk's halo ids)
  bool tri_loc;      // every resident block's triangle records carry local slots
  bool stencil;      // FP32: inviscid meshes take the vertex-stencil gradient pass
  bool any_inviscid; // an inviscid mesh is resident
  int pipe_groups;   // consumer groups of a pipelined kernel's CTA (1 or 2)
  int pipe_stages;   // stages of its ring (0: as many as fit, at most kPipeMaxStages)
  bool std_const;    // every resident mesh has math.f's constants (FP32 flux pass folds them)
  cudaStream_t stream;
};

// Stages of a pipelined kernel's ring for stages of `stage_bytes`: as many as
// fit the shared memory (at most `want` when want > 0), 0 when fewer than
// groups + 1 fit.
inline int pipe_stage_count(uint32_t stage_bytes, int groups, int want) {
  int n = (int)((kMaxSmem - kPipeStaticSmem) / stage_bytes);
  if (n > kPipeMaxStages) n = kPipeMaxStages;
  if (want > 0 && n > want) n = want;
  return n >= groups + 1 ? n : 0;
}

#define FVM_DECLARE_LAUNCHERS(R)                                                          \
  cudaError_t launch_visc(const ArenaPtrs<R> &A, const LaunchCfg &c, int stage, int do_dt, \
                          int routine);                                                   \
  cudaError_t launch_grad(const ArenaPtrs<R> &A, const LaunchCfg &c, int stage, int do_dt, \
                          int routine);                                                   \
  cudaError_t launch_grad_pipe(const ArenaPtrs<R> &A, const LaunchCfg &c, int stage,       \
                               int do_dt, int routine, long long budget, int inject,      \
                               int skip_inviscid);                                        \
  cudaError_t launch_flux(const ArenaPtrs<R> &A, const LaunchCfg &c, int stage, int mode,  \
                          int irk, int routine);                                          \
  cudaError_t launch_sa(const ArenaPtrs<R> &A, const LaunchCfg &c, int stage, int routine);\
  cudaError_t launch_step(const ArenaPtrs<R> &A, const LaunchCfg &c, int stage);           \
  size_t smem_step(const LaunchCfg &c, R *);                                              \
  cudaError_t launch_monitor(const ArenaPtrs<R> &A, const LaunchCfg &c, int serial_clcd); \
  cudaError_t launch_update(const ArenaPtrs<R> &A, const LaunchCfg &c, int irk);           \
  cudaError_t launch_time_step(const ArenaPtrs<R> &A, const LaunchCfg &c);                 \
  cudaError_t launch_positivity(const ArenaPtrs<R> &A, const LaunchCfg &c);                \
  cudaError_t launch_conres(const ArenaPtrs<R> &A, const LaunchCfg &c, int mesh, int first);\
  cudaError_t launch_clcd(const ArenaPtrs<R> &A, const LaunchCfg &c, int mesh, int serial);\
  cudaError_t launch_limitgrad(const ArenaPtrs<R> &A, const LaunchCfg &c);                 \
  cudaError_t launch_gradient_edge(const ArenaPtrs<R> &A, const LaunchCfg &c);             \
  cudaError_t launch_shockind(const ArenaPtrs<R> &A, const LaunchCfg &c);                  \
  size_t smem_grad(const LaunchCfg &c, R *);                                              \
  size_t smem_flux(const LaunchCfg &c, R *);                                              \
  size_t smem_sa(const LaunchCfg &c, R *);                                                \
  cudaError_t prepare_attributes(const LaunchCfg &c, R *);

FVM_DECLARE_LAUNCHERS(double)
FVM_DECLARE_LAUNCHERS(float)

// set-up kernels (FP64)
cudaError_t launch_edge_csl(const double2 *ds, D4 *csl, int n, cudaStream_t s);
cudaError_t launch_dtlength(int np, int nt, const double2 *coord, const int *elem,
                            const double *elarea, double *drmin, cudaStream_t s);
cudaError_t launch_wall_dist(int np, int nsedge, const double2 *coord, const int2 *sedge,
                             const int *ptype, int bugcompat, double *wd, cudaStream_t s);
// driver-order FP64 <-> arena-order per-vertex arrays of one mesh (fvm_setup.cu)
cudaError_t launch_get_vertex(int rsz, double *dst, const unsigned char *src, size_t stride,
                              const int *orig, int np, int k, int c0, cudaStream_t s);
cudaError_t launch_fill_vertex(int rsz, unsigned char *dst, size_t stride, int np, int k,
                               const double *values, cudaStream_t s);
// the same into / out of buffer b[*sel] (sel: a field of the mesh's control
// block on the device), from byte offset off
cudaError_t launch_put_vertex_sel(int rsz, unsigned char *const b[3], const int *sel, size_t off,
                                  size_t stride, const double *src, const int *orig, int np,
                                  int k, cudaStream_t s);
cudaError_t launch_get_vertex_sel(int rsz, double *dst, unsigned char *const b[3], const int *sel,
                                  size_t off, size_t stride, const int *orig, int np, int k,
                                  int c0, cudaStream_t s);
// a mesh's control block set on the device for a new state (what 0) or a
// start (what 1)
cudaError_t launch_ctl_update(MeshCtl *c, int what, int n, double minres, cudaStream_t s);
cudaError_t launch_gather_blocks(const int *work, const BlockInfo *blocks, BlockInfo *out, int n,
                                 cudaStream_t s);

}  // namespace fvm
