// fvm_kernels.cuh -- CUDA kernels of the fvm2d hot path, templated on the
// state type R.  Included by fvm_kernels_fp64.cu (compiled without FMA
// contraction) and fvm_kernels_fp32.cu.
//
// Every per-block kernel walks the work list (a persistent grid-stride loop
// over blocks of every active mesh in the arena), skips meshes whose control
// block is inactive, and picks the state buffers from the mesh's phase:
//   iterate mode, stage s = 1,2,3 (old = buffer p):
//     s1: p -> p+1      s2: p+1 -> p+2      s3: p+2 -> p+1   (mod 3)
//   routine mode (stage 0): state = p, prim_old = p+2, updates in place.
#pragma once

#include <climits>

#include "fvm_device.cuh"

#ifndef FVM_FLUX_THREADS
#define FVM_FLUX_THREADS 256  // threads of the FP32 flux pass's CTAs (one block of vertices each)
#endif
#ifndef FVM_FLUX_MINB32
#define FVM_FLUX_MINB32 6   // resident CTAs per SM asked of the FP32 flux kernel
#endif
#ifndef FVM_GRAD_MINB32
#define FVM_GRAD_MINB32 5   // resident CTAs per SM asked of the FP32 gradient kernel
#endif
#ifndef FVM_GRADV_MINB32
#define FVM_GRADV_MINB32 4  // the same for its per-vertex form
#endif
#ifndef FVM_STENCIL_MINB
#define FVM_STENCIL_MINB 6  // resident CTAs per SM asked of the stencil gradient kernel
#endif
#ifndef FVM_GATHER_BATCH
#define FVM_GATHER_BATCH 1  // FP32 flux pass: incidences loaded together in the per-vertex gather
#endif
#ifndef FVM_FLUX_PIPE
#define FVM_FLUX_PIPE 1     // FP32 flux pass: the next edge entry's ends in flight with this entry's gathers
#endif
#ifndef FVM_STENCIL_PIPE
#define FVM_STENCIL_PIPE 1  // stencil pass: next trip's neighbour ids in flight with this trip's states
#endif
#ifndef FVM_STENCIL_BATCH
#define FVM_STENCIL_BATCH 2 // edges whose loads are in flight at once per thread
#endif

namespace fvm {

// FP32 flux pass: threads per CTA (one block of kBlockVerts vertices; the
// edge trips spread over all of them, the per-vertex gather uses the first
// kBlockVerts)
constexpr int kFluxThreads = FVM_FLUX_THREADS;
static_assert(kFluxThreads % 32 == 0 && kFluxThreads >= kBlockVerts && kFluxThreads <= 1024,
              "flux CTA size");

enum { MODE_RESIDUAL = 0, MODE_UPDATE = 1 };

__device__ __forceinline__ int cur_buf(int p, int stage) {
  return stage <= 1 ? p : (p + stage - 1) % 3;
}
__device__ __forceinline__ int out_buf(int p, int stage) {
  return stage == 2 ? (p + 2) % 3 : (p + 1) % 3;
}
__device__ __forceinline__ int old_buf(int p, int stage) {
  return stage == 0 ? (p + 2) % 3 : p;
}

template <typename R>
__device__ __forceinline__ R4<R> ld4(const R4<R> *p) { return *p; }

// Bulk prefetch of [p, p + bytes) into L2 (cp.async.bulk.prefetch, no
// completion to wait for).  The range is shrunk to 16-byte boundaries
// inside the given one, so nothing outside it is touched.
__device__ __forceinline__ void prefetch_l2(const void *p, size_t bytes) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(p);
  const uintptr_t b = (a + 15) & ~uintptr_t(15);
  const uintptr_t e = (a + bytes) & ~uintptr_t(15);
  if (e <= b) return;
  uintptr_t n = e - b;
  // the size operand is 32-bit; split very long ranges
  while (n > 0) {
    const uint32_t chunk = n > (1u << 20) ? (1u << 20) : (uint32_t)n;
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(b + (e - b - n)), "r"(chunk)
                 : "memory");
    n -= chunk;
  }
}

// The next block this CTA will process (persistent loop), for prefetching.
// The blocks a launch covers: the whole work list (part 0) or part k, which
// ends at nwork[k] and starts where part k-1 ends (parts end at mesh
// boundaries).
template <typename R>
__device__ __forceinline__ void work_range(const ArenaPtrs<R> &A, int &w0, int &w1) {
  if (A.wpart == 0) {
    w0 = 0;
    w1 = A.nwork[0];
  } else {
    w0 = A.wpart == 1 ? 0 : A.nwork[A.wpart - 1];
    w1 = A.nwork[A.wpart];
  }
}

// Block w of the work list: its copy in work-list order (one load, not an
// index load followed by the block's; the host refreshes the copies with
// the work list)
template <typename R>
__device__ __forceinline__ const BlockInfo &work_block(const ArenaPtrs<R> &A, int w) {
  return A.wblocks[w];
}

template <typename R>
__device__ __forceinline__ const BlockInfo *next_block(const ArenaPtrs<R> &A, int w, int nwork) {
  const int nw = w + gridDim.x;
  return nw < nwork ? &work_block(A, nw) : nullptr;
}

// ---------------------------------------------------------------------------
// Viscosity (viscosity.f:2-55) and, at stage 1, the viscous time step
// (time_step.f:13-20) from the previous mu.  One thread per vertex.
// ---------------------------------------------------------------------------
// mbarrier and bulk-copy primitives (sm_90+ PTX) for staging a block's
// contiguous ranges in shared memory.
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
// global -> shared bulk copy; addresses 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// waits for the phase with the given parity; false after about a second
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > (1LL << 31)) return false;
  return true;
}
// orders this thread's generic-proxy shared-memory accesses before later
// async-proxy (bulk copy) writes to the same bytes
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Threads of the per-mesh monitor CTA (a power of two; the fixed-order
// reduction trees depend on it).  Wider CTAs measured no faster.
constexpr int kMonitorMaxThreads = 256;
template <typename R>
constexpr int monitor_threads() { return 256; }

// Per-vertex geometry in the kernel's precision (FP32 copies for R = float).
template <typename R>
__device__ __forceinline__ R v_ais(const ArenaPtrs<R> &A, int v) {
  if constexpr (sizeof(R) == 4) return A.ais32[v];
  else return A.ais[v];
}
template <typename R>
__device__ __forceinline__ R v_cvarea(const ArenaPtrs<R> &A, int v) {
  if constexpr (sizeof(R) == 4) return A.cvarea32[v];
  else return A.cvarea[v];
}
template <typename R>
__device__ __forceinline__ R v_wd(const ArenaPtrs<R> &A, int v) {
  if constexpr (sizeof(R) == 4) return A.wd32[v];
  else return A.wd[v];
}
template <typename R>
__device__ __forceinline__ R v_drmin(const ArenaPtrs<R> &A, int v) {
  if constexpr (sizeof(R) == 4) return A.drmin32[v];
  else return A.drmin[v];
}

// viscosity.f for the state a stage has just produced, which the next stage
// of the iteration starts from (what k_visc would compute at that stage)
template <typename R>
__device__ __forceinline__ void next_viscosity(const ArenaPtrs<R> &A, const MeshConst &mc,
                                               const MeshCtl &ctl, int v, const R4<R> &pn) {
  const R mul = sutherland_viscosity<R>(mc, pn.x, pn.w);
  A.mul[v] = mul;
  A.mu[v] = mc.iflow == 2 ? mul : mul + mu_turb<R>(mc, mul, pn.x, A.nut[ctl.nphase][v]);
}

template <typename R>
__global__ void __launch_bounds__(kBlockVerts) k_visc(ArenaPtrs<R> A, int stage, int do_dt,
                                                      int routine) {
  int w0, nwork;
  work_range(A, w0, nwork);
  for (int w = w0 + blockIdx.x; w < nwork; w += gridDim.x) {
    const BlockInfo bi = work_block(A, w);
    const MeshCtl &ctl = A.ctl[bi.mesh];
    if (!routine && !ctl.active) continue;
    const MeshConst &mc = A.mc[bi.mesh];
    if (mc.iflow == 1 || threadIdx.x >= bi.nv) continue;   // inviscid: mu stays 0
    const int v = bi.v0 + threadIdx.x;
    const R4<R> P = A.st[cur_buf(ctl.phase, stage)][v];
    if (do_dt) A.dt[v] = time_step<R>(mc, P, A.mu[v], v_drmin(A, v));
    R mul = sutherland_viscosity<R>(mc, P.x, P.w);
    A.mul[v] = mul;
    if (mc.iflow == 2) {
      A.mu[v] = mul;
    } else {
      R mut = mu_turb<R>(mc, mul, P.x, A.nut[ctl.nphase][v]);
      A.mu[v] = mul + mut;
    }
  }
}

// ---------------------------------------------------------------------------
// Gradient pass: green_gauss_euler / green_gauss_visc (green_gauss.f:2-92)
// with tri_gg and tri_visc; at stage 1 of an inviscid iteration also the
// local time step (time_step.f:22-27).
// ---------------------------------------------------------------------------
template <typename R>
struct TriSmem {
  R dxt[4];
  R dyt[4];
};

// a + b rounded as written (never fused with a product that forms b)
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }

// Green-Gauss terms of one triangle (green_gauss.f:100-127): dbxx/dbyy of
// its vertices and the sums dxt/dyt of the four primitive variables.
template <typename R>
__device__ __forceinline__ void tri_geom(const ArenaPtrs<R> &A, const int4 &t, int entry,
                                         R dbxx[3], R dbyy[3]) {
  if constexpr (sizeof(R) == 4) {
    const TriGeo32 tg = A.tri_g32[entry];
    for (int j = 0; j < 3; j++) {
      dbxx[j] = tg.dbxx[j];
      dbyy[j] = tg.dbyy[j];
    }
  } else {
    const double2 c1 = A.coord[t.x], c2 = A.coord[t.y], c3 = A.coord[t.z];
    dbxx[0] = c2.y - c3.y;
    dbxx[1] = c3.y - c1.y;
    dbxx[2] = c1.y - c2.y;
    dbyy[0] = c3.x - c2.x;
    dbyy[1] = c1.x - c3.x;
    dbyy[2] = c2.x - c1.x;
  }
}

template <typename R>
__device__ __forceinline__ void tri_sums(const R4<R> &p1, const R4<R> &p2, const R4<R> &p3,
                                         const R dbxx[3], const R dbyy[3], TriSmem<R> &ts) {
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const R a1 = comp(p1, q), a2 = comp(p2, q), a3 = comp(p3, q);
    ts.dxt[q] = a1 * dbxx[0] + a2 * dbxx[1] + a3 * dbxx[2];
    ts.dyt[q] = a1 * dbyy[0] + a2 * dbyy[1] + a3 * dbyy[2];
  }
}

// tri_visc (green_gauss.f:132-194): stresses and heat flux of one triangle;
// the contribution to its vertex at position j is
// ((txx, txy, efx) . dbxx[j] + (txy, tyy, efy) . dbyy[j]) * areat.
template <typename R>
struct TriVisc {
  R txx, txy, tyy, efx, efy, areat;
};

template <typename R>
__device__ __forceinline__ R tri_areat(const ArenaPtrs<R> &A, const int4 &t, int entry) {
  if constexpr (sizeof(R) == 4) return A.tri_g32[entry].areat;
  else return 0.25 / A.elarea[t.w];   // green_gauss.f:180
}

template <typename R>
__device__ __forceinline__ TriVisc<R> tri_visc(const ArenaPtrs<R> &A, const MeshConst &mc,
                                               int nbuf, const int4 &t, R areat,
                                               const R4<R> &p1, const R4<R> &p2,
                                               const R4<R> &p3, const R dbxx[3],
                                               const R dbyy[3], const TriSmem<R> &ts) {
  const R n2b3 = R(2) / R(3);
  const R en1 = mdiv(p1.w, p1.x), en2 = mdiv(p2.w, p2.x), en3 = mdiv(p3.w, p3.x);
  const R ext = en1 * dbxx[0] + en2 * dbxx[1] + en3 * dbxx[2];
  const R eyt = en1 * dbyy[0] + en2 * dbyy[1] + en3 * dbyy[2];
  const R um = mdiv(p1.y + p2.y + p3.y, R(3));
  const R vm = mdiv(p1.z + p2.z + p3.z, R(3));
  const R mult = mdiv(A.mul[t.x] + A.mul[t.y] + A.mul[t.z], R(3));
  // laminar meshes: mu = mul and nu~ = 0 exactly (viscosity.f, initialize.f),
  // so the turbulent heat-flux term is exactly zero and mu, nu~ need no loads
  R mut = mult, tterm = R(0);
  if (mc.iflow == 3) {
    mut = (A.mu[t.x] + A.mu[t.y] + A.mu[t.z]) / R(3);
    const R prim5t = (A.nut[nbuf][t.x] + A.nut[nbuf][t.y] + A.nut[nbuf][t.z]) / R(3);
    const R rhot = (p1.x + p2.x + p3.x) / R(3);
    const R chi = prim5t * rhot / mult;
    const R chi3 = cube(chi);
    const R fv1 = chi3 / (chi3 + MCR(R, cv11));
    tterm = rhot * prim5t * fv1 / MCR(R, prandtl_turb);
  }
  TriVisc<R> o;
  o.txx = n2b3 * mut * (R(2) * ts.dxt[1] - ts.dyt[2]);
  o.txy = mut * (ts.dyt[1] + ts.dxt[2]);
  o.tyy = n2b3 * mut * (R(2) * ts.dyt[2] - ts.dxt[1]);
  const R gpr = mdiv(MCR(R, gamma) * (mdiv(mult, MCR(R, prandtl)) + tterm), MCR(R, gamma1));
  o.efx = o.txx * um + o.txy * vm + gpr * ext;
  o.efy = o.txy * um + o.tyy * vm + gpr * eyt;
  o.areat = areat;
  return o;
}

template <typename R>
__device__ __forceinline__ void tri_visc_term(const TriVisc<R> &tv, R dbx, R dby, R out[3]) {
  out[0] = (tv.txx * dbx + tv.txy * dby) * tv.areat;
  out[1] = (tv.txy * dbx + tv.tyy * dby) * tv.areat;
  out[2] = (tv.efx * dbx + tv.efy * dby) * tv.areat;
}

// Sums of one vertex's triangle terms in the order of its incidence list
// (green_gauss.f:23-39 visits triangles in ascending order): entries
// [j0, j1) of `vtl`, each a triangle slot and the vertex's position in it.
// The slots and terms of up to B triangles are loaded before they are
// added, so the shared-memory latency is paid once per B triangles; the
// additions stay in list order (same bits as one triangle at a time).
// vis = nullptr: inviscid (rv is zero).
template <typename R, int B>
__device__ __forceinline__ void grad_vertex_sums(const uint16_t *vtl, int j0, int j1,
                                                 const TriSmem<R> *tri, const R *vis, R qx[4],
                                                 R qy[4], R rv[3]) {
#pragma unroll
  for (int q = 0; q < 4; q++) qx[q] = qy[q] = R(0);
  rv[0] = rv[1] = rv[2] = R(0);
  for (int j = j0; j < j1; j += B) {
    const int n = j1 - j;
    uint16_t e[B];
#pragma unroll
    for (int u = 0; u < B; u++) e[u] = u < n ? vtl[j + u] : uint16_t(0);
    TriSmem<R> ts[B];
#pragma unroll
    for (int u = 0; u < B; u++)
      if (u < n) ts[u] = tri[e[u] & 0x3fff];
#pragma unroll
    for (int u = 0; u < B; u++) {
      if (u < n) {
#pragma unroll
        for (int q = 0; q < 4; q++) {
          qx[q] = qx[q] + ts[u].dxt[q];
          qy[q] = qy[q] + ts[u].dyt[q];
        }
        if (vis) {
          const R *sv = vis + 9 * (e[u] & 0x3fff) + 3 * (e[u] >> kTriPosShift);
          rv[0] = rv[0] + sv[0];
          rv[1] = rv[1] + sv[1];
          rv[2] = rv[2] + sv[2];
        }
      }
    }
  }
}

template <typename R>
__global__ void __launch_bounds__(kBlockVerts, sizeof(R) == 4 ? FVM_GRAD_MINB32 : 1)
    k_grad(ArenaPtrs<R> A, int stage, int do_dt,
                                                      int routine, int max_tri, int skip_inviscid) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  TriSmem<R> *s_tri = reinterpret_cast<TriSmem<R> *>(smem_raw);
  R *s_vis = reinterpret_cast<R *>(s_tri + max_tri);   // [max_tri][3 pos][3 comp]
  int w0, nwork;
  work_range(A, w0, nwork);
  for (int w = w0 + blockIdx.x; w < nwork; w += gridDim.x) {
    const BlockInfo bi = work_block(A, w);
    const MeshCtl &ctl = A.ctl[bi.mesh];
    if (!routine && !ctl.active) continue;
    const MeshConst &mc = A.mc[bi.mesh];
    if (skip_inviscid && mc.iflow == 1) continue;   // the stencil pass's meshes
    const bool visc = mc.iflow != 1;
    const R4<R> *P = A.st[cur_buf(ctl.phase, stage)];
    if (threadIdx.x == 0) {
      const BlockInfo *nb = next_block(A, w, nwork);
      if (nb) {
        const BlockInfo n = *nb;
        prefetch_l2(A.bt_nodes + n.t0, sizeof(int4) * n.nt);
        if (sizeof(R) == 4) prefetch_l2(A.tri_g32 + n.t0, sizeof(TriGeo32) * n.nt);
        prefetch_l2(P + n.v0, sizeof(R4<R>) * n.nv);
        if (sizeof(R) == 8) prefetch_l2(A.coord + n.v0, sizeof(double2) * n.nv);
        prefetch_l2(A.vt_rng + n.v0, sizeof(int2) * n.nv);
        prefetch_l2(sizeof(R) == 4 ? (const void *)(A.ais32 + n.v0) : (const void *)(A.ais + n.v0), sizeof(R) * n.nv);
      }
    }
    // phase 1: one thread per triangle touching the block
    for (int k = threadIdx.x; k < bi.nt; k += blockDim.x) {
      const int4 t = A.bt_nodes[bi.t0 + k];
      const R4<R> p1 = P[t.x], p2 = P[t.y], p3 = P[t.z];
      R dbxx[3], dbyy[3];
      tri_geom<R>(A, t, bi.t0 + k, dbxx, dbyy);
      TriSmem<R> ts;
      tri_sums<R>(p1, p2, p3, dbxx, dbyy, ts);
      s_tri[k] = ts;
      if (visc) {
        const TriVisc<R> tv = tri_visc<R>(A, mc, ctl.nphase, t, tri_areat<R>(A, t, bi.t0 + k), p1, p2, p3, dbxx, dbyy, ts);
        R *sv = s_vis + 9 * k;
#pragma unroll
        for (int j = 0; j < 3; j++) tri_visc_term<R>(tv, dbxx[j], dbyy[j], sv + 3 * j);
      }
    }
    __syncthreads();
    // phase 2: one thread per vertex, triangles in original order
    if (threadIdx.x < bi.nv) {
      const int v = bi.v0 + threadIdx.x;
      R qx[4], qy[4], rv[3];
      const int2 jr = A.vt_rng[v];
      // (FP32: one triangle at a time, the 48 registers of five CTAs per SM)
      grad_vertex_sums<R, sizeof(R) == 8 ? 2 : 1>(A.vt_list, jr.x, jr.y, s_tri,
                                                  visc ? s_vis : nullptr, qx, qy, rv);
      const R ais = v_ais(A, v);
      Grad<R> g;
#pragma unroll
      for (int q = 0; q < 4; q++) {
        g.qx[q] = qx[q] * ais;
        g.qy[q] = qy[q] * ais;
      }
      A.grad[v] = g;
      if (visc) {
        R4<R> r;
        r.x = R(0);
        r.y = rv[0];
        r.z = rv[1];
        r.w = rv[2];
        A.resv[v] = r;
      } else if (do_dt) {
        A.dt[v] = time_step<R>(mc, P[v], R(0), v_drmin(A, v));
      }
    }
    __syncthreads();
  }
}

// Gradient pass with the block's contiguous inputs staged by bulk copies
// (FP32): one thread issues cp.async.bulk copies of the triangle entries,
// their geometry, the vertices' incidence ranges and the incidence list
// into shared memory (a few tens of KB in flight per CTA, tracked by one
// mbarrier); the threads then only gather the three states of each
// triangle.  Same arithmetic and order as k_grad.  Wait on the copies is
// bounded: after about a second the mesh gets FVM_ERR_TIMEOUT and the CTA
// returns.
template <typename R>
__global__ void __launch_bounds__(kBlockVerts, sizeof(R) == 4 ? FVM_GRAD_MINB32 : 1)
    k_grad_bulk(ArenaPtrs<R> A, int stage, int do_dt, int routine, int max_tri, int max_halo,
                int viscous, int skip_inviscid) {
  if constexpr (sizeof(R) == 4) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    const GradBulkLayout lay = grad_bulk_layout(max_tri, max_halo, viscous != 0);
    int *s_halo = reinterpret_cast<int *>(smem_raw + lay.halo);
    const TriGeo32 *s_geo = reinterpret_cast<const TriGeo32 *>(smem_raw + lay.geo);
    TriSmem<R> *s_tri = reinterpret_cast<TriSmem<R> *>(smem_raw + lay.geo);   // in place
    R *s_vis = reinterpret_cast<R *>(smem_raw + lay.vis);
    int2 *s_vtr = reinterpret_cast<int2 *>(smem_raw + lay.vtr);
    uint16_t *s_vtl = reinterpret_cast<uint16_t *>(smem_raw + lay.vtl);
    R4<R> *s_pv = reinterpret_cast<R4<R> *>(smem_raw + lay.pv);
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    uint32_t parity = 0;
    int w0, nwork;
  work_range(A, w0, nwork);
    for (int w = w0 + blockIdx.x; w < nwork; w += gridDim.x) {
      const BlockInfo bi = work_block(A, w);
      const MeshCtl &ctl = A.ctl[bi.mesh];
      if (!routine && !ctl.active) continue;
      const MeshConst &mc = A.mc[bi.mesh];
      if (skip_inviscid && mc.iflow == 1) continue;   // the stencil pass's meshes
      const bool visc = mc.iflow != 1;
      const R4<R> *P = A.st[cur_buf(ctl.phase, stage)];
      const int vt_a = bi.vt0 & ~7;                       // 16-byte units of uint16
      const int vt_b = (bi.vt0 + bi.nvt + 7) & ~7;
      // the halo vertices' ids, for the records' local slots (plain loads,
      // in flight during the copies)
      for (int h = threadIdx.x; h < bi.nh; h += blockDim.x) s_halo[h] = A.halo_ids[bi.h0 + h];
      if (threadIdx.x == 0) {
        const uint32_t ngeo = 32u * bi.nt;
        const uint32_t nvtr = 8u * ((bi.nv + 1) & ~1), nvtl = 2u * (vt_b - vt_a);
        const uint32_t npv = 16u * bi.nv;
        mbar_expect_tx(&bar, ngeo + nvtr + nvtl + npv);
        if (ngeo) bulk_g2s((void *)s_geo, A.tri_g32 + bi.t0, ngeo, &bar);
        bulk_g2s(s_vtr, A.vt_rng + bi.v0, nvtr, &bar);
        if (nvtl) bulk_g2s(s_vtl, A.vt_list + vt_a, nvtl, &bar);
        bulk_g2s(s_pv, P + bi.v0, npv, &bar);
        const BlockInfo *nb = next_block(A, w, nwork);
        if (nb) {
          const BlockInfo n = *nb;
          prefetch_l2(A.tri_g32 + n.t0, sizeof(TriGeo32) * n.nt);
          prefetch_l2(P + n.v0, sizeof(R4<R>) * n.nv);
          prefetch_l2(A.vt_rng + n.v0, sizeof(int2) * n.nv);
          prefetch_l2(A.vt_list + n.vt0, sizeof(uint16_t) * n.nvt);
          prefetch_l2(A.ais32 + n.v0, sizeof(float) * n.nv);
          prefetch_l2(A.halo_ids + n.h0, sizeof(int) * n.nh);
        }
      }
      const bool late = !mbar_wait_bounded(&bar, parity);
      parity ^= 1u;
      if (__syncthreads_or(late)) {
        if (threadIdx.x == 0) atomicCAS(&A.ctl[bi.mesh].err, 0, 6 /* FVM_ERR_TIMEOUT */);
        return;
      }
      // phase 1: one thread per triangle touching the block; its ends by
      // local slot: own vertices' states from shared memory, the halo's
      // from global memory
      auto state = [&](uint32_t l) {
        return l < (uint32_t)bi.nv ? s_pv[l] : P[s_halo[l - bi.nv]];
      };
      auto vertex = [&](uint32_t l) {
        return l < (uint32_t)bi.nv ? bi.v0 + (int)l : s_halo[l - bi.nv];
      };
      for (int k = threadIdx.x; k < bi.nt; k += blockDim.x) {
        const TriGeo32 tg = s_geo[k];
        constexpr uint32_t lm = (uint32_t)(kTriLocMax - 1);
        const uint32_t l1 = tg.loc & lm, l2 = (tg.loc >> kTriLocBits) & lm,
                       l3 = (tg.loc >> (2 * kTriLocBits)) & lm;
        const R4<R> p1 = state(l1), p2 = state(l2), p3 = state(l3);
        R dbxx[3], dbyy[3];
#pragma unroll
        for (int j = 0; j < 3; j++) {
          dbxx[j] = tg.dbxx[j];
          dbyy[j] = tg.dbyy[j];
        }
        TriSmem<R> ts;
        tri_sums<R>(p1, p2, p3, dbxx, dbyy, ts);
        if (visc) {
          const int4 t = make_int4(vertex(l1), vertex(l2), vertex(l3), 0);
          const TriVisc<R> tv = tri_visc<R>(A, mc, ctl.nphase, t, tg.areat, p1, p2, p3, dbxx, dbyy, ts);
          R *sv = s_vis + 9 * k;
#pragma unroll
          for (int j = 0; j < 3; j++) tri_visc_term<R>(tv, dbxx[j], dbyy[j], sv + 3 * j);
        }
        s_tri[k] = ts;   // over this thread's own geometry entry
      }
      __syncthreads();
      // phase 2: one thread per vertex, triangles in original order
      if (threadIdx.x < bi.nv) {
        const int v = bi.v0 + threadIdx.x;
        R qx[4], qy[4], rv[3];
        const int2 jr = s_vtr[threadIdx.x];
        // one triangle at a time: batched loads spill at 48 registers
        grad_vertex_sums<R, 1>(s_vtl, jr.x - vt_a, jr.y - vt_a, s_tri, visc ? s_vis : nullptr, qx,
                               qy, rv);
        const R ais = v_ais(A, v);
        Grad<R> g;
#pragma unroll
        for (int q = 0; q < 4; q++) {
          g.qx[q] = qx[q] * ais;
          g.qy[q] = qy[q] * ais;
        }
        A.grad[v] = g;
        if (visc) {
          R4<R> r;
          r.x = R(0);
          r.y = rv[0];
          r.z = rv[1];
          r.w = rv[2];
          A.resv[v] = r;
        } else if (do_dt) {
          A.dt[v] = time_step<R>(mc, s_pv[threadIdx.x], R(0), v_drmin(A, v));
        }
      }
      fence_proxy_async_smem();   // before the next block's copies land here
      __syncthreads();
    }
  }
}

// Gradient pass, vertex-stencil form (FP32, inviscid meshes): green_gauss.f
// (2-42) as precomputed per-vertex weights over the vertex's edges,
//   qx, qy (v) = sum over edges (v,u) of W(v,u) * (prim_u - prim_v),
// W formed on the host in FP64 from the triangles around the edge and
// rounded once (fvm_batch_prepare).  Equal to the triangle sums in exact
// arithmetic; in FP32 it rounds differently (and maps a uniform state to
// zero exactly).  One thread per vertex, no shared memory and no barrier;
// the weights and neighbour states of FVM_STENCIL_BATCH edges are in flight
// at once.  At stage 1 also time_step.f:22-27.
template <typename R>
__global__ void __launch_bounds__(kBlockVerts, FVM_STENCIL_MINB)
    k_grad_stencil(ArenaPtrs<R> A, int stage, int do_dt, int routine) {
  constexpr int B = FVM_STENCIL_BATCH;
  if constexpr (sizeof(R) == 4) {
    int w0, nwork;
    work_range(A, w0, nwork);
    for (int w = w0 + blockIdx.x; w < nwork; w += gridDim.x) {
      const BlockInfo bi = work_block(A, w);
      const MeshCtl &ctl = A.ctl[bi.mesh];
      if (!routine && !ctl.active) continue;
      const MeshConst &mc = A.mc[bi.mesh];
      if (mc.iflow != 1 || threadIdx.x >= bi.nv) continue;
      const int v = bi.v0 + threadIdx.x;
      const R4<R> *P = A.st[cur_buf(ctl.phase, stage)];
      const R4<R> pv = P[v];
      const int2 r = A.va_rng[v];
      R qx[4] = {R(0), R(0), R(0), R(0)}, qy[4] = {R(0), R(0), R(0), R(0)};
#if FVM_STENCIL_PIPE
      // the next trip's neighbour ids are loaded while this trip's states
      // are in flight: one dependent load latency per trip instead of two
      int un[B];
#pragma unroll
      for (int k = 0; k < B; k++)
        un[k] = k < r.y - r.x ? (A.va_list[r.x + k] & 0x7fffffff) : v;
#endif
      for (int j = r.x; j < r.y; j += B) {
        const int n = r.y - j;
        int u[B];
        float2 wt[B];
#pragma unroll
        for (int k = 0; k < B; k++) {
#if FVM_STENCIL_PIPE
          u[k] = un[k];
#else
          u[k] = k < n ? (A.va_list[j + k] & 0x7fffffff) : v;
#endif
          wt[k] = k < n ? A.va_w[j + k] : make_float2(0.f, 0.f);
        }
        R4<R> pu[B];
#pragma unroll
        for (int k = 0; k < B; k++) pu[k] = k < n ? P[u[k]] : pv;
#if FVM_STENCIL_PIPE
#pragma unroll
        for (int k = 0; k < B; k++)
          un[k] = k < n - B ? (A.va_list[j + B + k] & 0x7fffffff) : v;
#endif
#pragma unroll
        for (int k = 0; k < B; k++) {
          if (k < n) {
#pragma unroll
            for (int q = 0; q < 4; q++) {
              const R d = comp(pu[k], q) - comp(pv, q);
              qx[q] = fmaf(wt[k].x, d, qx[q]);
              qy[q] = fmaf(wt[k].y, d, qy[q]);
            }
          }
        }
      }
      Grad<R> g;
#pragma unroll
      for (int q = 0; q < 4; q++) {
        g.qx[q] = qx[q];
        g.qy[q] = qy[q];
      }
      A.grad[v] = g;
      if (do_dt) A.dt[v] = time_step<R>(mc, pv, R(0), v_drmin(A, v));
    }
  }
}

// Gradient pass, per-vertex form: each thread walks its vertex's triangles
// (ascending, as green_gauss.f visits them) and computes each triangle's
// terms itself, straight from the triangle entries; no shared memory and no
// barrier, at the price of computing every triangle once per vertex.  The
// arithmetic of each term is that of k_grad, so both give the same sums.
template <typename R>
__global__ void __launch_bounds__(kBlockVerts, sizeof(R) == 4 ? FVM_GRADV_MINB32 : 1)
    k_grad_v(ArenaPtrs<R> A, int stage, int do_dt, int routine, int skip_inviscid) {
  int w0, nwork;
  work_range(A, w0, nwork);
  for (int w = w0 + blockIdx.x; w < nwork; w += gridDim.x) {
    const BlockInfo bi = work_block(A, w);
    const MeshCtl &ctl = A.ctl[bi.mesh];
    if (!routine && !ctl.active) continue;
    const MeshConst &mc = A.mc[bi.mesh];
    if (skip_inviscid && mc.iflow == 1) continue;   // the stencil pass's meshes
    const bool visc = mc.iflow != 1;
    const R4<R> *P = A.st[cur_buf(ctl.phase, stage)];
    if (threadIdx.x == 0) {
      const BlockInfo *nb = next_block(A, w, nwork);
      if (nb) {
        const BlockInfo n = *nb;
        prefetch_l2(A.bt_nodes + n.t0, sizeof(int4) * n.nt);
        if (sizeof(R) == 4) prefetch_l2(A.tri_g32 + n.t0, sizeof(TriGeo32) * n.nt);
        prefetch_l2(P + n.v0, sizeof(R4<R>) * n.nv);
        if (sizeof(R) == 8) prefetch_l2(A.coord + n.v0, sizeof(double2) * n.nv);
        prefetch_l2(A.vt_rng + n.v0, sizeof(int2) * n.nv);
        prefetch_l2(sizeof(R) == 4 ? (const void *)(A.ais32 + n.v0) : (const void *)(A.ais + n.v0), sizeof(R) * n.nv);
      }
    }
    if (threadIdx.x >= bi.nv) continue;   // no barrier follows
    const int v = bi.v0 + threadIdx.x;
    R qx[4] = {R(0), R(0), R(0), R(0)}, qy[4] = {R(0), R(0), R(0), R(0)};
    R rv[3] = {R(0), R(0), R(0)};
    const int2 jr = A.vt_rng[v];
    for (int j = jr.x; j < jr.y; j++) {
      const uint16_t e = A.vt_list[j];
      const int entry = bi.t0 + (e & 0x3fff);
      const int4 t = A.bt_nodes[entry];
      const R4<R> p1 = P[t.x], p2 = P[t.y], p3 = P[t.z];
      R dbxx[3], dbyy[3];
      tri_geom<R>(A, t, entry, dbxx, dbyy);
      TriSmem<R> ts;
      tri_sums<R>(p1, p2, p3, dbxx, dbyy, ts);
      // plain (uncontracted) adds: each term is rounded before it is
      // summed, as when k_grad reads it back from shared memory
#pragma unroll
      for (int q = 0; q < 4; q++) {
        qx[q] = add_rn(qx[q], ts.dxt[q]);
        qy[q] = add_rn(qy[q], ts.dyt[q]);
      }
      if (visc) {
        const int pos = e >> kTriPosShift;
        const TriVisc<R> tv = tri_visc<R>(A, mc, ctl.nphase, t, tri_areat<R>(A, t, entry), p1, p2, p3, dbxx, dbyy, ts);
        R sv[3];
        tri_visc_term<R>(tv, pos == 0 ? dbxx[0] : pos == 1 ? dbxx[1] : dbxx[2],
                         pos == 0 ? dbyy[0] : pos == 1 ? dbyy[1] : dbyy[2], sv);
        rv[0] = add_rn(rv[0], sv[0]);
        rv[1] = add_rn(rv[1], sv[1]);
        rv[2] = add_rn(rv[2], sv[2]);
      }
    }
    const R ais = v_ais(A, v);
    Grad<R> g;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      g.qx[q] = qx[q] * ais;
      g.qy[q] = qy[q] * ais;
    }
    A.grad[v] = g;
    if (visc) {
      R4<R> r;
      r.x = R(0);
      r.y = rv[0];
      r.z = rv[1];
      r.w = rv[2];
      A.resv[v] = r;
    } else if (do_dt) {
      A.dt[v] = time_step<R>(mc, P[v], R(0), v_drmin(A, v));
    }
  }
}

// ---------------------------------------------------------------------------
// conres.f:14-22 partials of one block: sum of gra^2 and max |gra| (first
// driver index on ties), gra = rho_new - rho_old.  Called by every thread
// of the CTA (contains barriers).  FP64 states: FP64 arithmetic as before.
// FP32 states: gra is formed exactly as a pair of floats (TwoSum), its
// square as a pair (FMA residual), and the warp and block sums are pair
// sums, converted to FP64 once per block.  The FP64 pipe of this GPU is
// slow, and this keeps it out of the reduction: the sum carries ~2^-47
// relative error instead of 2^-53; max |gra| is exact.
// ---------------------------------------------------------------------------
struct DFloat {
  float hi, lo;
};
__device__ __forceinline__ DFloat two_sum(float a, float b) {   // a + b = hi + lo exactly
  const float s = __fadd_rn(a, b);
  const float z = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, z)), __fsub_rn(b, z));
  return {s, e};
}
__device__ __forceinline__ DFloat df_add(DFloat x, DFloat y) {
  const DFloat s = two_sum(x.hi, y.hi);
  const float e = __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo));
  const float hi = __fadd_rn(s.hi, e);
  return {hi, __fsub_rn(e, __fsub_rn(hi, s.hi))};
}
__device__ __forceinline__ bool df_greater(DFloat x, DFloat y) {   // normalized pairs
  return x.hi > y.hi || (x.hi == y.hi && x.lo > y.lo);
}

template <typename R>
__device__ __forceinline__ void block_conres_partial(bool have, R rho_new, R rho_old, int orig,
                                                     double *s_red, double *s_max, int *s_arg,
                                                     BlockPartial *out) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int darg = INT_MAX;
  if constexpr (sizeof(R) == 8) {
    double d2 = 0.0, dabs = 0.0;
    if (have) {
      const double gra = double(rho_new) - double(rho_old);
      d2 = gra * gra;
      dabs = fabs(gra);
      // conres.f:17-21 keeps a point only when |gra| > fresi, which a NaN
      // never is: a NaN poisons the sum of squares, not the maximum
      if (dabs > 0.0) darg = orig;
      else dabs = 0.0;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const double o2 = __shfl_down_sync(0xffffffffu, d2, off);
      const double om = __shfl_down_sync(0xffffffffu, dabs, off);
      const int oa = __shfl_down_sync(0xffffffffu, darg, off);
      d2 += o2;
      if (om > dabs || (om == dabs && oa < darg)) {
        dabs = om;
        darg = oa;
      }
    }
    if (lane == 0) {
      s_red[wid] = d2;
      s_max[wid] = dabs;
      s_arg[wid] = darg;
    }
  } else {
    DFloat sq2 = {0.f, 0.f}, mx = {0.f, 0.f};
    if (have) {
      const DFloat g = two_sum(float(rho_new), -float(rho_old));
      const float h2 = __fmul_rn(g.hi, g.hi);
      const float l2 = __fadd_rn(__fmaf_rn(g.hi, g.hi, -h2), __fmul_rn(__fmul_rn(2.f, g.hi), g.lo));
      sq2 = two_sum(h2, l2);
      mx = g.hi >= 0.f ? g : DFloat{-g.hi, -g.lo};
      if (mx.hi > 0.f) darg = orig;
      else mx = DFloat{0.f, 0.f};   // NaN or no change (see the FP64 branch)
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const DFloat o2 = {__shfl_down_sync(0xffffffffu, sq2.hi, off),
                         __shfl_down_sync(0xffffffffu, sq2.lo, off)};
      const DFloat om = {__shfl_down_sync(0xffffffffu, mx.hi, off),
                         __shfl_down_sync(0xffffffffu, mx.lo, off)};
      const int oa = __shfl_down_sync(0xffffffffu, darg, off);
      sq2 = df_add(sq2, o2);
      if (df_greater(om, mx) || (om.hi == mx.hi && om.lo == mx.lo && oa < darg)) {
        mx = om;
        darg = oa;
      }
    }
    // warps' pairs summed by thread 0, still as pairs; one conversion to FP64
    __shared__ DFloat s_sq[kFluxThreads / 32], s_mx[kFluxThreads / 32];
    if (lane == 0) {
      s_sq[wid] = sq2;
      s_mx[wid] = mx;
      s_arg[wid] = darg;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      DFloat t = s_sq[0], m = s_mx[0];
      int a = s_arg[0];
      for (int i = 1; i < (int)(blockDim.x >> 5); i++) {
        t = df_add(t, s_sq[i]);
        if (df_greater(s_mx[i], m) || (s_mx[i].hi == m.hi && s_mx[i].lo == m.lo && s_arg[i] < a)) {
          m = s_mx[i];
          a = s_arg[i];
        }
      }
      BlockPartial bp;
      bp.sumsq = double(t.hi) + double(t.lo);
      bp.maxabs = double(m.hi) + double(m.lo);   // exact
      bp.argmax = a;
      bp.pad = 0;
      *out = bp;
    }
    return;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double sacc = 0.0, m = 0.0;
    int a = INT_MAX;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) {
      sacc += s_red[i];
      if (s_max[i] > m || (s_max[i] == m && s_arg[i] < a)) {
        m = s_max[i];
        a = s_arg[i];
      }
    }
    BlockPartial bp;
    bp.sumsq = sacc;
    bp.maxabs = m;
    bp.argmax = a;
    bp.pad = 0;
    *out = bp;
  }
}

// ---------------------------------------------------------------------------
// Flux pass: residu.f:37-88 (recon + roe/kfvs/hllc over iedge, solid_flux,
// farfield_flux) gathered per vertex in Fortran order, then either the
// residual is written (MODE_RESIDUAL) or the RK stage of update.f:17-35 is
// applied (MODE_UPDATE).  At stage 3 of an iteration it also produces the
// conres.f partials and the density/pressure positivity check.
// ---------------------------------------------------------------------------
// Mesh constants of the flux pass in the state precision, loaded once per
// block (keeps conversions out of the edge loop).
template <typename R>
struct FluxConst {
  R a11, a12, a21, a22, eps, gamma, gamma1, pi;
  int ilimit, iflux, rotate_back;
};

template <typename R>
__device__ __forceinline__ FluxConst<R> flux_const(const MeshConst &mc) {
  FluxConst<R> c;
  c.a11 = MCR(R, albada11);
  c.a12 = MCR(R, albada12);
  c.a21 = MCR(R, albada21);
  c.a22 = MCR(R, albada22);
  c.eps = MCR(R, epsilon);
  c.gamma = MCR(R, gamma);
  c.gamma1 = MCR(R, gamma1);
  c.pi = MCR(R, pi);
  c.ilimit = mc.ilimit;
  c.iflux = mc.iflux;
  c.rotate_back = mc.bugcompat ? 0 : 1;
  return c;
}

// The same constants when every resident mesh has math.f:8-40's values
// (fvm_params_init; the host checks): compile-time values, each the FP32
// rounding of the double the driver computes, so the edge loop keeps none
// of them in registers.
__device__ __forceinline__ FluxConst<float> flux_const_std(const MeshConst &mc) {
  FluxConst<float> c;
  c.a11 = (float)(2.0 / 3.0);
  c.a12 = (float)(1.0 - 2.0 / 3.0);
  c.a21 = (float)(4.0 / 3.0);
  c.a22 = (float)(1.0 - 4.0 / 3.0);
  c.eps = (float)1.0e-16;
  c.gamma = (float)1.4;
  c.gamma1 = (float)(1.4 - 1.0);
  c.pi = (float)3.141592653589793;
  c.ilimit = mc.ilimit;
  c.iflux = mc.iflux;
  c.rotate_back = mc.bugcompat ? 0 : 1;
  return c;
}

// Flux-pass template code: the Riemann solver (1/2/3; 0 dispatches on the
// mesh's iflux) plus kFluxStd when the FP32 constants are the standard ones.
constexpr int kFluxStd = 4;

// FP32: the edge's unit normal and length from its ds (flux.f:10-13) with
// one reciprocal square root.
__device__ __forceinline__ void edge_normal_f32(float dsx, float dsy, float &ct, float &st,
                                                float &len) {
  const float d2 = fmaf(dsx, dsx, dsy * dsy);
  const float il = rsqrtf(d2);
  ct = dsx * il;
  st = dsy * il;
  len = d2 * il;
}

// FP32: recon.f:4-50 for the four variables of an edge.  With the limiter,
// albada21 scales the edge vector once per edge instead of each projected
// gradient, and albada22 * dq serves both sides; the same values as recon1
// up to FP32 rounding.
__device__ __forceinline__ void recon_edge_f32(const R4<float> &p1, const R4<float> &p2,
                                               const Grad<float> &g1, const Grad<float> &g2,
                                               float dx, float dy, const FluxConst<float> &fc,
                                               float pl[4], float pr[4]) {
  if (fc.ilimit == 1) {
    const float dxa = fc.a21 * dx, dya = fc.a21 * dy;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const float a = comp(p1, q), b = comp(p2, q);
      const float dqp = b - a;
      const float c = fc.a22 * dqp;
      const float dql = fmaf(dxa, g1.qx[q], fmaf(dya, g1.qy[q], c));
      const float dqr = fmaf(dxa, g2.qx[q], fmaf(dya, g2.qy[q], c));
      pl[q] = fmaf(0.5f, limit_albada<float>(dql, dqp, fc.eps), a);
      pr[q] = fmaf(-0.5f, limit_albada<float>(dqr, dqp, fc.eps), b);
    }
  } else {
#pragma unroll
    for (int q = 0; q < 4; q++)
      recon1<float>(comp(p1, q), comp(p2, q), g1.qx[q], g1.qy[q], g2.qx[q], g2.qy[q], dx, dy,
                    fc.ilimit, fc.a11, fc.a12, fc.a21, fc.a22, fc.eps, pl[q], pr[q]);
  }
}

// FLUX = 1/2/3 compiles one Riemann solver only (every resident mesh uses
// it); FLUX = 0 dispatches on the mesh's iflux.
// nn_in: the entry's ends when the caller has loaded them (FP32 edge loop),
// else nullptr
template <typename R, int FLUX>
__device__ __forceinline__ void edge_flux(const ArenaPtrs<R> &A, const FluxConst<R> &fc,
                                          const R4<R> *P, int e, R f[4], int &err,
                                          const int2 *nn_in = nullptr) {
  int2 nn;
  R dx, dy, ct, st, len;
  float dsx = 0.f, dsy = 0.f;
  if constexpr (sizeof(R) == 4) {
    // ends, edge vector and ds (24 bytes per entry); ds/|ds| and |ds| are
    // formed after the reconstruction
    nn = nn_in ? *nn_in : A.be_nodes[e];
    const float4 h = A.be_g32[e].v;
    dx = h.x;
    dy = h.y;
    dsx = h.z;
    dsy = h.w;
  } else {
    nn = A.be_nodes[e];
    const double2 c1 = A.coord[nn.x], c2 = A.coord[nn.y];
    dx = c2.x - c1.x;
    dy = c2.y - c1.y;
  }
  const R4<R> p1 = P[nn.x], p2 = P[nn.y];
  const Grad<R> g1 = A.grad[nn.x], g2 = A.grad[nn.y];
  R pl[4], pr[4];
  if constexpr (sizeof(R) == 4) {
    recon_edge_f32(p1, p2, g1, g2, dx, dy, fc, pl, pr);
  } else {
#pragma unroll
    for (int q = 0; q < 4; q++)
      recon1<R>(comp(p1, q), comp(p2, q), g1.qx[q], g1.qy[q], g2.qx[q], g2.qy[q], dx, dy,
                fc.ilimit, fc.a11, fc.a12, fc.a21, fc.a22, fc.eps, pl[q], pr[q]);
  }
  if constexpr (sizeof(R) == 4) {
    edge_normal_f32(dsx, dsy, ct, st, len);
  } else {
    const D4 csl = A.be_csl[e];
    ct = R(csl.x);
    st = R(csl.y);
    len = R(csl.z);
  }
  constexpr int FL = FLUX & 3;
  const int which = FL ? FL : fc.iflux;
  if (which == 1) {
    if (!roe_flux<R>(ct, st, len, pl, pr, fc.gamma, fc.gamma1, f)) err = 1;
  } else if (which == 2) {
    kfvs_flux<R>(ct, st, len, pl, pr, fc.gamma1, fc.pi, f);
  } else {
    hllc_flux<R>(ct, st, len, pl, pr, fc.gamma, fc.gamma1, fc.rotate_back, f);
  }
}

// Phase 1b of the flux pass: boundary edges, two slots each (contribution
// to n1, to n2) after the block's ne interior slots.
template <typename R>
__device__ __forceinline__ void flux_boundary(const ArenaPtrs<R> &A, const MeshConst &mc,
                                              const MeshCtl &ctl, const BlockInfo &bi,
                                              const R4<R> *P, R4<R> *s_flux) {
  for (int k = threadIdx.x; k < bi.nb; k += blockDim.x) {
    const int4 b = A.bb_nodes[bi.b0 + k];
    const double2 x1 = A.coord[b.x], x2 = A.coord[b.y];
    const R4<R> p1 = P[b.x], p2 = P[b.y];
    R4<R> o1, o2;
    if (b.z == 1) {
      // solid_flux.f:10-17
      const R sx = R(0.5) * R(x2.y - x1.y);
      const R sy = -R(0.5) * R(x2.x - x1.x);
      const R pp1 = R(0.75) * p1.w + R(0.25) * p2.w;
      const R pp2 = R(0.25) * p1.w + R(0.75) * p2.w;
      o1.x = R(0);
      o1.y = pp1 * sx;
      o1.z = pp1 * sy;
      o1.w = R(0);
      o2.x = R(0);
      o2.y = pp2 * sx;
      o2.z = pp2 * sy;
      o2.w = R(0);
    } else {
      R f1[4], f2[4];
      farfield_flux<R>(mc, ctl.cl, x1, x2, p1, p2, f1, f2);
      o1.x = f1[0];
      o1.y = f1[1];
      o1.z = f1[2];
      o1.w = f1[3];
      o2.x = f2[0];
      o2.y = f2[1];
      o2.z = f2[2];
      o2.w = f2[3];
    }
    s_flux[bi.ne + 2 * k] = o1;
    s_flux[bi.ne + 2 * k + 1] = o2;
  }
}

// Phase 2 of the flux pass: one thread per vertex sums its edge slots in
// Fortran order, then writes the residual (MODE_RESIDUAL) or applies the RK
// stage (MODE_UPDATE); at stage 3 the block's conres partial follows.
template <typename R>
__device__ __forceinline__ void flux_gather(const ArenaPtrs<R> &A, const MeshConst &mc,
                                            MeshCtl &ctl, const BlockInfo &bi, const R4<R> *P,
                                            const R4<R> *s_flux, int p, int stage, int mode,
                                            int irk, int routine, double *s_red, double *s_max,
                                            int *s_arg) {
  bool have = false;
  R rho_new = R(0), rho_old = R(0);
  int org = 0;
  if (threadIdx.x < bi.nv) {
    const int v = bi.v0 + threadIdx.x;
    R acc[4];
    if (mc.iflow != 1) {
      const R4<R> rv = A.resv[v];
      acc[0] = R(0);
      acc[1] = rv.y;
      acc[2] = rv.z;
      acc[3] = rv.w;
    } else {
      acc[0] = acc[1] = acc[2] = acc[3] = R(0);
    }
    const int2 jr = A.ve_rng[v];
    // FVM_GATHER_BATCH incidences' slots and fluxes loaded together, then
    // added in list order
    constexpr int GB = sizeof(R) == 4 ? FVM_GATHER_BATCH : 1;
    for (int j = jr.x; j < jr.y; j += GB) {
      uint16_t es[GB];
      R4<R> fs[GB];
#pragma unroll
      for (int u = 0; u < GB; u++) es[u] = j + u < jr.y ? A.ve_list[j + u] : uint16_t(0);
#pragma unroll
      for (int u = 0; u < GB; u++)
        if (j + u < jr.y) fs[u] = s_flux[es[u] & kSlotMask];
#pragma unroll
      for (int u = 0; u < GB; u++) {
        if (j + u >= jr.y) break;
        const uint16_t e = es[u];
        const R4<R> f = fs[u];
        if (e & kSolidBit) {
          acc[1] = acc[1] + f.y;
          acc[2] = acc[2] + f.z;
        } else if (e & kNegBit) {
          acc[0] = acc[0] - f.x;
          acc[1] = acc[1] - f.y;
          acc[2] = acc[2] - f.z;
          acc[3] = acc[3] - f.w;
        } else {
          acc[0] = acc[0] + f.x;
          acc[1] = acc[1] + f.y;
          acc[2] = acc[2] + f.z;
          acc[3] = acc[3] + f.w;
        }
      }
    }
    if (mode == MODE_RESIDUAL) {
      R4<R> r;
      r.x = acc[0];
      r.y = acc[1];
      r.z = acc[2];
      r.w = acc[3];
      A.res[v] = r;
    } else {
      const R4<R> po = A.st[old_buf(p, stage)][v];
      const R4<R> pc = P[v];
      const bool noslip = (mc.iflow != 1) && (A.vflag[v] & kVtxSolid);
      const R4<R> pn = rk_update<R>(mc, irk, po, pc, A.dt[v], v_cvarea(A, v), acc, noslip);
      A.st[out_buf(p, stage)][v] = pn;
      // iterate mode: stages 2 and 3 start from the viscosity computed here
      if (!routine && stage < 3 && mc.iflow != 1) next_viscosity<R>(A, mc, ctl, v, pn);
      if (stage == 3) {
        // conres.f:14-22 partials and check_positivity.f:13-14 (rho, p)
        have = true;
        rho_new = pn.x;
        rho_old = po.x;
        org = A.orig[v];
        if (pn.x <= R(0) || pn.w <= R(0)) atomicMin(&ctl.err_point, org);
      }
    }
  }
  if (mode == MODE_UPDATE && stage == 3)
    block_conres_partial<R>(have, rho_new, rho_old, org, s_red, s_max, s_arg, A.part + bi.part);
}

template <typename R, int FLUX>
__global__ void __launch_bounds__(sizeof(R) == 4 ? kFluxThreads : kBlockVerts,
                                  sizeof(R) == 4 ? FVM_FLUX_MINB32 : 2)
    k_flux(ArenaPtrs<R> A, int stage, int mode, int irk, int routine) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  R4<R> *s_flux = reinterpret_cast<R4<R> *>(smem_raw);
  __shared__ double s_red[kFluxThreads / 32];
  __shared__ double s_max[kFluxThreads / 32];
  __shared__ int s_arg[kFluxThreads / 32];
  int w0, nwork;
  work_range(A, w0, nwork);
  for (int w = w0 + blockIdx.x; w < nwork; w += gridDim.x) {
    const BlockInfo bi = work_block(A, w);
    MeshCtl &ctl = A.ctl[bi.mesh];
    if (!routine && !ctl.active) continue;
    const MeshConst &mc = A.mc[bi.mesh];
    const int p = ctl.phase;
    const R4<R> *P = A.st[cur_buf(p, stage)];
    // FP64: the next block's inputs into L2.  Not in FP32, where the same
    // prefetches made the pass slower (0.206 -> 0.216 ms on 8 meshes of
    // 1024 x 384 timed alone; whole iterations 1.025 -> 1.040 ms).
    if (sizeof(R) == 8 && threadIdx.x == 0) {
      const BlockInfo *nb = next_block(A, w, nwork);
      if (nb) {
        const BlockInfo n = *nb;
        prefetch_l2(A.be_nodes + n.e0, sizeof(int2) * n.ne);
        prefetch_l2(A.be_csl + n.e0, sizeof(D4) * n.ne);
        prefetch_l2(P + n.v0, sizeof(R4<R>) * n.nv);
        prefetch_l2(A.grad + n.v0, sizeof(Grad<R>) * n.nv);
        prefetch_l2(A.coord + n.v0, sizeof(double2) * n.nv);
        prefetch_l2(A.ve_rng + n.v0, sizeof(int2) * n.nv);
        if (mode == MODE_UPDATE) {
          prefetch_l2(A.st[old_buf(p, stage)] + n.v0, sizeof(R4<R>) * n.nv);
          prefetch_l2(A.dt + n.v0, sizeof(R) * n.nv);
          prefetch_l2(A.cvarea + n.v0, sizeof(R) * n.nv);
        }
      }
    }
    int err = 0;
    FluxConst<R> fc;
    if constexpr (sizeof(R) == 4 && (FLUX & kFluxStd) != 0) fc = flux_const_std(mc);
    else fc = flux_const<R>(mc);
    // phase 1a: interior edges.  FP32: the next entry's ends are loaded
    // while this entry's states and gradients are in flight
#if FVM_FLUX_PIPE
    int2 nn_next = make_int2(0, 0);
    if (sizeof(R) == 4 && threadIdx.x < bi.ne) nn_next = A.be_nodes[bi.e0 + threadIdx.x];
#endif
    for (int k = threadIdx.x; k < bi.ne; k += blockDim.x) {
      R f[4];
#if FVM_FLUX_PIPE
      if constexpr (sizeof(R) == 4) {
        const int2 nn = nn_next;
        if (k + (int)blockDim.x < bi.ne) nn_next = A.be_nodes[bi.e0 + k + blockDim.x];
        edge_flux<R, FLUX>(A, fc, P, bi.e0 + k, f, err, &nn);
      } else {
        edge_flux<R, FLUX>(A, fc, P, bi.e0 + k, f, err);
      }
#else
      edge_flux<R, FLUX>(A, fc, P, bi.e0 + k, f, err);
#endif
      R4<R> o;
      o.x = f[0];
      o.y = f[1];
      o.z = f[2];
      o.w = f[3];
      s_flux[k] = o;
    }
    // phase 1b: boundary edges
    flux_boundary<R>(A, mc, ctl, bi, P, s_flux);
    if (err) atomicCAS(&ctl.err, 0, 4 /* FVM_ERR_ROE_SONIC */);
    __syncthreads();
    // phase 2: gather per vertex in Fortran order
    flux_gather<R>(A, mc, ctl, bi, P, s_flux, p, stage, mode, irk, routine, s_red, s_max, s_arg);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Fused stage: gradients, fluxes and the RK stage of one block in one pass
// (iterate mode).  Phase A computes dxt/dyt of every triangle touching the
// block or its halo (and the tri_visc terms of the block's own triangles);
// phase B sums them into the Green-Gauss gradients of the block's own and
// halo vertices, each in ascending triangle order exactly as the owner
// block would, so the halo gradients equal the owner's bit for bit; phase C
// computes the edge fluxes from those gradients; phase D gathers and
// updates.  Replaces k_grad + k_flux: the gradients never leave shared
// memory except the own ones, written for the stage-3 consumers (clcd, SA).
// ---------------------------------------------------------------------------
// Shared memory: region 1 = max(max_tri2 triangle records [+ viscous terms of
// max_tri], max_slots fluxes) (fluxes reuse the triangle area after phase B);
// region 2 = max_loc gradients.
template <typename R, int FLUX>
__global__ void __launch_bounds__(kBlockVerts, sizeof(R) == 4 ? FVM_FLUX_MINB32 : 2)
    k_step(ArenaPtrs<R> A, int stage, int max_tri, int max_tri2, int max_slots, int max_loc,
           int viscous) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const size_t tri_bytes = size_t(max_tri2) * sizeof(TriSmem<R>) + (viscous ? size_t(max_tri) * 9 * sizeof(R) : 0);
  const size_t flux_bytes = size_t(max_slots) * sizeof(R4<R>);
  const size_t r1 = ((tri_bytes > flux_bytes ? tri_bytes : flux_bytes) + 63) & ~size_t(63);
  TriSmem<R> *s_tri = reinterpret_cast<TriSmem<R> *>(smem_raw);
  R *s_vis = reinterpret_cast<R *>(s_tri + max_tri2);
  R4<R> *s_flux = reinterpret_cast<R4<R> *>(smem_raw);
  Grad<R> *s_grad = reinterpret_cast<Grad<R> *>(smem_raw + r1);
  __shared__ double s_red[kBlockVerts / 32];
  __shared__ double s_max[kBlockVerts / 32];
  __shared__ int s_arg[kBlockVerts / 32];
  int w0, nwork;
  work_range(A, w0, nwork);
  for (int w = w0 + blockIdx.x; w < nwork; w += gridDim.x) {
    const BlockInfo bi = work_block(A, w);
    MeshCtl &ctl = A.ctl[bi.mesh];
    if (!ctl.active) continue;
    const MeshConst &mc = A.mc[bi.mesh];
    const bool visc = mc.iflow != 1;
    const int p = ctl.phase;
    const R4<R> *P = A.st[cur_buf(p, stage)];
    if (threadIdx.x == 0) {
      const BlockInfo *nb = next_block(A, w, nwork);
      if (nb) {
        const BlockInfo n = *nb;
        prefetch_l2(A.bt_nodes + n.t0, sizeof(int4) * n.nt2);
        if (sizeof(R) == 4) {
          prefetch_l2(A.tri_g32 + n.t0, sizeof(TriGeo32) * n.nt2);
          prefetch_l2(A.be_g32 + n.e0, sizeof(EdgeGeo32) * n.ne);
          prefetch_l2(A.be_nodes + n.e0, sizeof(int2) * n.ne);
        } else {
          prefetch_l2(A.coord + n.v0, sizeof(double2) * n.nv);
          prefetch_l2(A.be_csl + n.e0, sizeof(D4) * n.ne);
          prefetch_l2(A.be_nodes + n.e0, sizeof(int2) * n.ne);
          prefetch_l2(A.be_loc + n.e0, sizeof(uint32_t) * n.ne);
        }
        prefetch_l2(P + n.v0, sizeof(R4<R>) * n.nv);
        prefetch_l2(A.vt_rng + n.v0, sizeof(int2) * n.nv);
        prefetch_l2(A.ve_rng + n.v0, sizeof(int2) * n.nv);
        prefetch_l2(sizeof(R) == 4 ? (const void *)(A.ais32 + n.v0) : (const void *)(A.ais + n.v0), sizeof(R) * n.nv);
        prefetch_l2(A.st[old_buf(p, stage)] + n.v0, sizeof(R4<R>) * n.nv);
        prefetch_l2(sizeof(R) == 4 ? (const void *)(A.cvarea32 + n.v0) : (const void *)(A.cvarea + n.v0), sizeof(R) * n.nv);
      }
    }
    // phase A: triangles of the block and of its halo
    for (int k = threadIdx.x; k < bi.nt2; k += blockDim.x) {
      const int4 t = A.bt_nodes[bi.t0 + k];
      const R4<R> p1 = P[t.x], p2 = P[t.y], p3 = P[t.z];
      R dbxx[3], dbyy[3];
      tri_geom<R>(A, t, bi.t0 + k, dbxx, dbyy);
      TriSmem<R> ts;
      tri_sums<R>(p1, p2, p3, dbxx, dbyy, ts);
      s_tri[k] = ts;
      if (visc && k < bi.nt) {
        const TriVisc<R> tv = tri_visc<R>(A, mc, ctl.nphase, t, tri_areat<R>(A, t, bi.t0 + k), p1, p2, p3, dbxx, dbyy, ts);
        R *sv = s_vis + 9 * k;
#pragma unroll
        for (int j = 0; j < 3; j++) tri_visc_term<R>(tv, dbxx[j], dbyy[j], sv + 3 * j);
      }
    }
    __syncthreads();
    // phase B: gradients of own vertices (thread t = own vertex t, which
    // keeps its viscous residual part and time step in registers) and of
    // the halo vertices
    R rv[3] = {R(0), R(0), R(0)};
    R dtv = R(0);
    const int t = threadIdx.x;
    if (t < bi.nv) {
      const int v = bi.v0 + t;
      R qx[4] = {R(0), R(0), R(0), R(0)}, qy[4] = {R(0), R(0), R(0), R(0)};
      const int2 jr = A.vt_rng[v];
      for (int j = jr.x; j < jr.y; j++) {
        const uint16_t e = A.vt_list[j];
        const int slot = e & 0x3fff;
        const TriSmem<R> ts = s_tri[slot];
#pragma unroll
        for (int q = 0; q < 4; q++) {
          qx[q] = qx[q] + ts.dxt[q];
          qy[q] = qy[q] + ts.dyt[q];
        }
        if (visc) {
          const R *sv = s_vis + 9 * slot + 3 * (e >> kTriPosShift);
          rv[0] = rv[0] + sv[0];
          rv[1] = rv[1] + sv[1];
          rv[2] = rv[2] + sv[2];
        }
      }
      const R ais = v_ais(A, v);
      Grad<R> g;
#pragma unroll
      for (int q = 0; q < 4; q++) {
        g.qx[q] = qx[q] * ais;
        g.qy[q] = qy[q] * ais;
      }
      s_grad[t] = g;
      A.grad[v] = g;
      if (visc) dtv = A.dt[v];
      else if (stage == 1) {
        dtv = time_step<R>(mc, P[v], R(0), v_drmin(A, v));
        A.dt[v] = dtv;
      } else {
        dtv = A.dt[v];
      }
    }
    for (int h = t; h < bi.nh; h += blockDim.x) {
      const int g0 = A.hl_ptr[bi.hp0 + h], g1 = A.hl_ptr[bi.hp0 + h + 1];
      R qx[4] = {R(0), R(0), R(0), R(0)}, qy[4] = {R(0), R(0), R(0), R(0)};
      for (int j = g0; j < g1; j++) {
        const TriSmem<R> ts = s_tri[A.hl_list[j] & 0x3fff];
#pragma unroll
        for (int q = 0; q < 4; q++) {
          qx[q] = qx[q] + ts.dxt[q];
          qy[q] = qy[q] + ts.dyt[q];
        }
      }
      const R ais = v_ais(A, A.halo_ids[bi.h0 + h]);
      Grad<R> g;
#pragma unroll
      for (int q = 0; q < 4; q++) {
        g.qx[q] = qx[q] * ais;
        g.qy[q] = qy[q] * ais;
      }
      s_grad[bi.nv + h] = g;
    }
    __syncthreads();
    // phase C: interior edge fluxes from the shared gradients
    int err = 0;
    const FluxConst<R> fc = flux_const<R>(mc);
    for (int k = threadIdx.x; k < bi.ne; k += blockDim.x) {
      const int e = bi.e0 + k;
      int2 nn;
      uint32_t ll;
      R dx, dy, ct, st, len;
      if constexpr (sizeof(R) == 4) {
        const float4 g = A.be_g32[e].v;
        nn = A.be_nodes[e];
        ll = A.be_loc[e];
        dx = g.x;
        dy = g.y;
        edge_normal_f32(g.z, g.w, ct, st, len);
      } else {
        nn = A.be_nodes[e];
        ll = A.be_loc[e];
        const double2 c1 = A.coord[nn.x], c2 = A.coord[nn.y];
        dx = c2.x - c1.x;
        dy = c2.y - c1.y;
        const D4 csl = A.be_csl[e];
        ct = R(csl.x);
        st = R(csl.y);
        len = R(csl.z);
      }
      const R4<R> p1 = P[nn.x], p2 = P[nn.y];
      const Grad<R> g1 = s_grad[ll & 0xffff], g2 = s_grad[ll >> 16];
      R pl[4], pr[4];
#pragma unroll
      for (int q = 0; q < 4; q++)
        recon1<R>(comp(p1, q), comp(p2, q), g1.qx[q], g1.qy[q], g2.qx[q], g2.qy[q], dx, dy,
                  fc.ilimit, fc.a11, fc.a12, fc.a21, fc.a22, fc.eps, pl[q], pr[q]);
      R f[4];
      const int which = FLUX ? FLUX : fc.iflux;
      if (which == 1) {
        if (!roe_flux<R>(ct, st, len, pl, pr, fc.gamma, fc.gamma1, f)) err = 1;
      } else if (which == 2) {
        kfvs_flux<R>(ct, st, len, pl, pr, fc.gamma1, fc.pi, f);
      } else {
        hllc_flux<R>(ct, st, len, pl, pr, fc.gamma, fc.gamma1, fc.rotate_back, f);
      }
      R4<R> o;
      o.x = f[0];
      o.y = f[1];
      o.z = f[2];
      o.w = f[3];
      s_flux[k] = o;
    }
    // boundary edges, two slots each (contribution to n1, to n2)
    for (int k = threadIdx.x; k < bi.nb; k += blockDim.x) {
      const int4 b = A.bb_nodes[bi.b0 + k];
      const double2 x1 = A.coord[b.x], x2 = A.coord[b.y];
      const R4<R> p1 = P[b.x], p2 = P[b.y];
      R4<R> o1, o2;
      if (b.z == 1) {
        // solid_flux.f:10-17
        const R sx = R(0.5) * R(x2.y - x1.y);
        const R sy = -R(0.5) * R(x2.x - x1.x);
        const R pp1 = R(0.75) * p1.w + R(0.25) * p2.w;
        const R pp2 = R(0.25) * p1.w + R(0.75) * p2.w;
        o1.x = R(0);
        o1.y = pp1 * sx;
        o1.z = pp1 * sy;
        o1.w = R(0);
        o2.x = R(0);
        o2.y = pp2 * sx;
        o2.z = pp2 * sy;
        o2.w = R(0);
      } else {
        R f1[4], f2[4];
        farfield_flux<R>(mc, ctl.cl, x1, x2, p1, p2, f1, f2);
        o1.x = f1[0];
        o1.y = f1[1];
        o1.z = f1[2];
        o1.w = f1[3];
        o2.x = f2[0];
        o2.y = f2[1];
        o2.z = f2[2];
        o2.w = f2[3];
      }
      s_flux[bi.ne + 2 * k] = o1;
      s_flux[bi.ne + 2 * k + 1] = o2;
    }
    if (err) atomicCAS(&ctl.err, 0, 4 /* FVM_ERR_ROE_SONIC */);
    __syncthreads();
    // phase D: gather per own vertex in Fortran order, RK stage
    bool have = false;
    R rho_new = R(0), rho_old = R(0);
    int org = 0;
    if (t < bi.nv) {
      const int v = bi.v0 + t;
      R acc[4];
      acc[0] = R(0);
      acc[1] = rv[0];
      acc[2] = rv[1];
      acc[3] = rv[2];
      const int2 jr = A.ve_rng[v];
      for (int j = jr.x; j < jr.y; j++) {
        const uint16_t e = A.ve_list[j];
        const R4<R> f = s_flux[e & kSlotMask];
        if (e & kSolidBit) {
          acc[1] = acc[1] + f.y;
          acc[2] = acc[2] + f.z;
        } else if (e & kNegBit) {
          acc[0] = acc[0] - f.x;
          acc[1] = acc[1] - f.y;
          acc[2] = acc[2] - f.z;
          acc[3] = acc[3] - f.w;
        } else {
          acc[0] = acc[0] + f.x;
          acc[1] = acc[1] + f.y;
          acc[2] = acc[2] + f.z;
          acc[3] = acc[3] + f.w;
        }
      }
      const R4<R> po = A.st[old_buf(p, stage)][v];
      const R4<R> pc = P[v];
      const bool noslip = visc && (A.vflag[v] & kVtxSolid);
      const R4<R> pn = rk_update<R>(mc, stage, po, pc, dtv, v_cvarea(A, v), acc, noslip);
      A.st[out_buf(p, stage)][v] = pn;
      if (stage == 3) {
        have = true;
        rho_new = pn.x;
        rho_old = po.x;
        org = A.orig[v];
        if (pn.x <= R(0) || pn.w <= R(0)) atomicMin(&ctl.err_point, org);
      }
    }
    if (stage == 3)
      block_conres_partial<R>(have, rho_new, rho_old, org, s_red, s_max, s_arg, A.part + bi.part);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Spalart-Allmaras step (sa_model.f:3-201): viscous_sa over triangles,
// divergence_sa over iedge, outer_flux_sa over farfield edges, then
// update_sa; nu~ is zero at solid points.  Reads nut[nphase], writes
// nut[1-nphase].  Uses the state buffer that holds the new solution.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(kBlockVerts) k_sa(ArenaPtrs<R> A, int stage, int routine,
                                                    int max_tri) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  R *s_t = reinterpret_cast<R *>(smem_raw);   // [max_tri][3]
  R *s_e = s_t + 3 * max_tri;                  // [slots]
  int w0, nwork;
  work_range(A, w0, nwork);
  for (int w = w0 + blockIdx.x; w < nwork; w += gridDim.x) {
    const BlockInfo bi = work_block(A, w);
    MeshCtl &ctl = A.ctl[bi.mesh];
    if (!routine && !ctl.active) continue;
    const MeshConst &mc = A.mc[bi.mesh];
    if (mc.iflow != 3) continue;
    // the solution after the RK stages: out of stage 3, or the state itself
    const int p = ctl.phase;
    const R4<R> *P = A.st[stage == 3 ? out_buf(p, 3) : p];
    const R *nut = A.nut[ctl.nphase];
    R *nut_new = A.nut[1 - ctl.nphase];
    for (int k = threadIdx.x; k < bi.nt; k += blockDim.x) {
      const int4 t = A.bt_nodes[bi.t0 + k];
      R areat, dbxx[3], dbyy[3];
      if constexpr (sizeof(R) == 4) {   // FP32 copies rounded once
        const TriGeo32 tg = A.tri_g32[bi.t0 + k];
        areat = tg.areat;
        for (int j = 0; j < 3; j++) {
          dbxx[j] = tg.dbxx[j];
          dbyy[j] = tg.dbyy[j];
        }
      } else {
        const double2 c1 = A.coord[t.x], c2 = A.coord[t.y], c3 = A.coord[t.z];
        areat = R(0.25 / A.elarea[t.w]);
        dbxx[0] = R(c2.y - c3.y);
        dbxx[1] = R(c3.y - c1.y);
        dbxx[2] = R(c1.y - c2.y);
        dbyy[0] = R(c3.x - c2.x);
        dbyy[1] = R(c1.x - c3.x);
        dbyy[2] = R(c2.x - c1.x);
      }
      int a1 = t.x, a2 = t.y, a3 = t.z;
      if (mc.bugcompat) {
        a1 = mc.orig123[0];
        a2 = mc.orig123[1];
        a3 = mc.orig123[2];
      }
      const R nux = nut[a1] * dbxx[0] + nut[a2] * dbxx[1] + nut[a3] * dbxx[2];
      const R nuy = nut[a1] * dbyy[0] + nut[a2] * dbyy[1] + nut[a3] * dbyy[2];
      const R mul1 = A.mul[t.x], mul2 = A.mul[t.y], mul3 = A.mul[t.z];
      const R n1 = nut[t.x], n2 = nut[t.y], n3 = nut[t.z];
      const R r1 = P[t.x].x, r2 = P[t.y].x, r3 = P[t.z].x;
      const R mult = mdiv(mul1 + mul2 + mul3, R(3));
      const R prim5t = mdiv(n1 + n2 + n3, R(3));
      const R rhot = mdiv(r1 + r2 + r3, R(3));
      const R mutb = mdiv(mult, rhot) + prim5t;
      const R cs1 = MCR(R, cb2sig1), cs2 = MCR(R, cb2sig2);
      s_t[3 * k + 0] = (cs1 * mutb - cs2 * (mdiv(mul1, r1) + n1)) * (nux * dbxx[0] + nuy * dbyy[0]) * areat;
      s_t[3 * k + 1] = (cs1 * mutb - cs2 * (mdiv(mul2, r2) + n2)) * (nux * dbxx[1] + nuy * dbyy[1]) * areat;
      s_t[3 * k + 2] = (cs1 * mutb - cs2 * (mdiv(mul3, r3) + n3)) * (nux * dbxx[2] + nuy * dbyy[2]) * areat;
    }
    for (int k = threadIdx.x; k < bi.ne; k += blockDim.x) {
      const int e = bi.e0 + k;
      int2 nn;
      R d1, d2;
      if constexpr (sizeof(R) == 4) {   // ds from the FP32 record
        const float4 g = A.be_g32[e].v;
        nn = A.be_nodes[e];
        d1 = g.z;
        d2 = g.w;
      } else {
        nn = A.be_nodes[e];
        const double2 ds = A.be_ds[e];
        d1 = R(ds.x);
        d2 = R(ds.y);
      }
      const R4<R> p1 = P[nn.x], p2 = P[nn.y];
      const R unl = p1.y * d1 + p1.z * d2;
      const R unr = p2.y * d1 + p2.z * d2;
      const R una = R(0.5) * (unl + unr);
      s_e[k] = (una > R(0)) ? una * nut[nn.x] : una * nut[nn.y];
    }
    for (int k = threadIdx.x; k < bi.nb; k += blockDim.x) {
      const int4 b = A.bb_nodes[bi.b0 + k];
      R f1 = R(0), f2 = R(0);
      if (b.z == 2) {
        const double2 x1 = A.coord[b.x], x2 = A.coord[b.y];
        const R dx = R(x2.x - x1.x), dy = R(x2.y - x1.y);
        const R sx = dy, sy = -dx;
        const R4<R> p1 = P[b.x], p2 = P[b.y];
        const R u = R(0.5) * (p1.y + p2.y);
        const R vv = R(0.5) * (p1.z + p2.z);
        const R un = u * sx + vv * sy;
        if (un > R(0)) {
          f1 = un * nut[b.x];
          f2 = un * nut[b.y];
        } else {
          f1 = un * MCR(R, nut_inf);
          f2 = un * MCR(R, nut_inf);
        }
        f1 = R(0.5) * f1;
        f2 = R(0.5) * f2;
      }
      s_e[bi.ne + 2 * k] = f1;
      s_e[bi.ne + 2 * k + 1] = f2;
    }
    __syncthreads();
    if (threadIdx.x < bi.nv) {
      const int v = bi.v0 + threadIdx.x;
      R divf = R(0);
      const int2 tr = A.vt_rng[v];
      for (int j = tr.x; j < tr.y; j++) {
        const uint16_t e = A.vt_list[j];
        divf = divf + s_t[3 * (e & 0x3fff) + (e >> kTriPosShift)];
      }
      const int2 er = A.ve_rng[v];
      for (int j = er.x; j < er.y; j++) {
        const uint16_t e = A.ve_list[j];
        if (e & kSolidBit) continue;
        const R f = s_e[e & kSlotMask];
        divf = (e & kNegBit) ? divf - f : divf + f;
      }
      R nn;
      if (A.vflag[v] & kVtxSolid) {
        nn = R(0);
      } else {
        const Grad<R> g = A.grad[v];
        const R omega = g.qy[1] - g.qx[2];
        nn = update_sa<R>(mc, nut[v], P[v].x, A.mul[v], v_wd(A, v), A.dt[v], v_cvarea(A, v), divf,
                          omega);
      }
      nut_new[v] = nn;
      if (nn < R(0)) atomicMin(&ctl.err_point, A.orig[v]);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// End-of-iteration monitor, one CTA per mesh: conres.f (from the block
// partials), clcd.f, the positivity verdict, RES.DAT history row and the
// stop test of main.f:42.  FP64 arithmetic; the clcd sum is the serial
// Fortran chain when serial_clcd is set.
// ---------------------------------------------------------------------------
// One solid edge's pressure and viscous force (clcd.f:20-40), added to
// (xf, yf).  FP32 states: the terms from the FP32 values (the edge vector
// an FP64 difference rounded once), accumulated in FP64.
template <typename R>
__device__ __forceinline__ void wall_force(double2 c1, double2 c2, R mu1, R mu2, const Grad<R> &g1,
                                           const Grad<R> &g2, R p1, R p2, double &xf,
                                           double &yf) {
  if constexpr (sizeof(R) == 4) {
    const float sx = float(c2.y - c1.y), sy = -float(c2.x - c1.x);
    const float n2b3 = 2.0f / 3.0f;
    const float txx = 0.5f * (n2b3 * mu1 * (2.0f * g1.qx[1] - g1.qy[2]) +
                              n2b3 * mu2 * (2.0f * g2.qx[1] - g2.qy[2]));
    const float txy = 0.5f * (mu1 * (g1.qy[1] + g1.qx[2]) + mu2 * (g2.qy[1] + g2.qx[2]));
    const float tyy = 0.5f * (n2b3 * mu1 * (2.0f * g1.qy[2] - g1.qx[1]) +
                              n2b3 * mu2 * (2.0f * g2.qy[2] - g2.qx[1]));
    const float pp = 0.5f * (p1 + p2);
    xf += double(pp * sx - txx * sx - txy * sy);
    yf += double(pp * sy - txy * sx - tyy * sy);
  } else {
    const double dx = c2.x - c1.x, dy = c2.y - c1.y;
    const double sx = dy, sy = -dx;
    const double txx = 0.5 * (2.0 / 3.0 * mu1 * (2.0 * double(g1.qx[1]) - double(g1.qy[2])) +
                              2.0 / 3.0 * mu2 * (2.0 * double(g2.qx[1]) - double(g2.qy[2])));
    const double txy = 0.5 * (mu1 * (double(g1.qy[1]) + double(g1.qx[2])) +
                              mu2 * (double(g2.qy[1]) + double(g2.qx[2])));
    const double tyy = 0.5 * (2.0 / 3.0 * mu1 * (2.0 * double(g1.qy[2]) - double(g1.qx[1])) +
                              2.0 / 3.0 * mu2 * (2.0 * double(g2.qy[2]) - double(g2.qx[1])));
    const double pp = 0.5 * (double(p1) + double(p2));
    xf += pp * sx - txx * sx - txy * sy;
    yf += pp * sy - txy * sx - tyy * sy;
  }
}

template <typename R>
__device__ void clcd_block(const ArenaPtrs<R> &A, const MeshConst &mc, int mesh_phase,
                           int serial, double &cl, double &cd) {
  __shared__ double s_x[kMonitorMaxThreads], s_y[kMonitorMaxThreads];
  const R4<R> *P = A.st[mesh_phase];
  double xf = 0.0, yf = 0.0;
  if (serial) {
    if (threadIdx.x == 0) {
      for (int i = 0; i < mc.nsw; i++) {
        const int2 nn = A.sw_nodes[mc.sw0 + i];
        const double2 c1 = A.coord[nn.x], c2 = A.coord[nn.y];
        const double dx = c2.x - c1.x, dy = c2.y - c1.y;
        const double sx = dy, sy = -dx;
        const double mu1 = double(A.mu[nn.x]), mu2 = double(A.mu[nn.y]);
        const Grad<R> g1 = A.grad[nn.x], g2 = A.grad[nn.y];
        const double p1 = double(P[nn.x].w), p2 = double(P[nn.y].w);
        const double txx1 = 2.0 / 3.0 * mu1 * (2.0 * double(g1.qx[1]) - double(g1.qy[2]));
        const double txy1 = mu1 * (double(g1.qy[1]) + double(g1.qx[2]));
        const double tyy1 = 2.0 / 3.0 * mu1 * (2.0 * double(g1.qy[2]) - double(g1.qx[1]));
        const double txx2 = 2.0 / 3.0 * mu2 * (2.0 * double(g2.qx[1]) - double(g2.qy[2]));
        const double txy2 = mu2 * (double(g2.qy[1]) + double(g2.qx[2]));
        const double tyy2 = 2.0 / 3.0 * mu2 * (2.0 * double(g2.qy[2]) - double(g2.qx[1]));
        const double pp = 0.5 * (p1 + p2);
        const double txx = 0.5 * (txx1 + txx2);
        const double txy = 0.5 * (txy1 + txy2);
        const double tyy = 0.5 * (tyy1 + tyy2);
        xf = xf + pp * sx - txx * sx - txy * sy;
        yf = yf + pp * sy - txy * sx - tyy * sy;
      }
    }
  } else {
    // each thread's edges i, i + blockDim, ... summed in that order, with
    // the loads of four edges issued together per trip
    constexpr int kU = 4;
    const int nt = (int)blockDim.x;
    for (int i0 = threadIdx.x; i0 < mc.nsw; i0 += kU * nt) {
      int2 nn[kU];
#pragma unroll
      for (int u = 0; u < kU; u++)
        nn[u] = (i0 + u * nt < mc.nsw) ? A.sw_nodes[mc.sw0 + i0 + u * nt] : make_int2(0, 0);
      double2 c1[kU], c2[kU];
      R mu1[kU], mu2[kU], p1[kU], p2[kU];
      Grad<R> g1[kU], g2[kU];
#pragma unroll
      for (int u = 0; u < kU; u++) {
        c1[u] = A.coord[nn[u].x];
        c2[u] = A.coord[nn[u].y];
        mu1[u] = A.mu[nn[u].x];
        mu2[u] = A.mu[nn[u].y];
        g1[u] = A.grad[nn[u].x];
        g2[u] = A.grad[nn[u].y];
        p1[u] = P[nn[u].x].w;
        p2[u] = P[nn[u].y].w;
      }
#pragma unroll
      for (int u = 0; u < kU; u++) {
        if (i0 + u * nt >= mc.nsw) break;
        wall_force<R>(c1[u], c2[u], mu1[u], mu2[u], g1[u], g2[u], p1[u], p2[u], xf, yf);
      }
    }
    s_x[threadIdx.x] = xf;
    s_y[threadIdx.x] = yf;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) {
        s_x[threadIdx.x] += s_x[threadIdx.x + s];
        s_y[threadIdx.x] += s_y[threadIdx.x + s];
      }
      __syncthreads();
    }
    xf = s_x[0];
    yf = s_y[0];
  }
  const double q = 0.5 * mc.r_inf * (mc.q_inf * mc.q_inf);
  cl = (-mc.sin_aoa * xf + mc.cos_aoa * yf) / q;
  cd = (mc.cos_aoa * xf + mc.sin_aoa * yf) / q;
}

template <typename R>
__device__ void conres_block(const ArenaPtrs<R> &A, const MeshConst &mc, double &sum,
                             double &mx, int &arg) {
  __shared__ double s_s[kMonitorMaxThreads], s_m[kMonitorMaxThreads];
  __shared__ int s_a[kMonitorMaxThreads];
  double s = 0.0, m = 0.0;
  int a = INT_MAX;
  // the mesh's partials are contiguous (block k's record is blk0 + k);
  // eight loads in flight per thread (a 2048-block mesh in one trip),
  // folded in index order
  constexpr int kU = 8;
  for (int i0 = threadIdx.x; i0 < mc.nblk; i0 += kU * blockDim.x) {
    BlockPartial bp[kU];
#pragma unroll
    for (int u = 0; u < kU; u++) {
      const int i = i0 + u * (int)blockDim.x;
      if (i < mc.nblk) bp[u] = A.part[mc.blk0 + i];
    }
#pragma unroll
    for (int u = 0; u < kU; u++) {
      if (i0 + u * (int)blockDim.x >= mc.nblk) break;
      s += bp[u].sumsq;
      if (bp[u].maxabs > m || (bp[u].maxabs == m && bp[u].argmax < a)) {
        m = bp[u].maxabs;
        a = bp[u].argmax;
      }
    }
  }
  s_s[threadIdx.x] = s;
  s_m[threadIdx.x] = m;
  s_a[threadIdx.x] = a;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) {
      s_s[threadIdx.x] += s_s[threadIdx.x + st];
      const double om = s_m[threadIdx.x + st];
      const int oa = s_a[threadIdx.x + st];
      if (om > s_m[threadIdx.x] || (om == s_m[threadIdx.x] && oa < s_a[threadIdx.x])) {
        s_m[threadIdx.x] = om;
        s_a[threadIdx.x] = oa;
      }
    }
    __syncthreads();
  }
  sum = s_s[0];
  mx = s_m[0];
  arg = s_a[0];
}

// One CTA (256 threads) per mesh slot listed in mesh_list.
template <typename R>
__global__ void __launch_bounds__(kMonitorMaxThreads) k_monitor(ArenaPtrs<R> A, int serial_clcd) {
  const int m = blockIdx.x;
  MeshCtl &ctl = A.ctl[m];
  if (!ctl.active) return;
  if (A.wpart > 0 && A.mesh_part[m] != A.wpart) return;   // another chain's mesh
  const MeshConst &mc = A.mc[m];
  double sum, mx;
  int arg;
  conres_block<R>(A, mc, sum, mx, arg);
  const int newp = (ctl.phase + 1) % 3;
  double cl, cd;
  clcd_block<R>(A, mc, newp, serial_clcd, cl, cd);
  __syncthreads();
  if (threadIdx.x != 0) return;
  ctl.phase = newp;
  if (mc.iflow == 3) ctl.nphase = 1 - ctl.nphase;
  if (ctl.err) {                            // roe_flux.f stop, inside residu
    ctl.active = 0;
    return;
  }
  if (ctl.err_point != INT_MAX) {          // check_positivity.f stop
    ctl.err = 3;
    ctl.active = 0;
    return;
  }
  ctl.cl = cl;
  ctl.cd = cd;
  double fres = sqrt(sum / double(mc.nv));
  ctl.fresi = mx;
  ctl.iresi = (mx > 0.0) ? arg : 0;
  if (ctl.iter == ctl.iterlast) {
    ctl.fres1 = fres;
    if (fres == 0.0) {
      ctl.fres = fres;
      ctl.err = 5;
      ctl.active = 0;
      return;
    }
  }
  fres = fres / ctl.fres1;
  ctl.fres = fres;
  {
    const int row = ctl.hist_off + ctl.n_done % ctl.hist_cap;
    A.h_fres[row] = fres;
    A.h_iresi[row] = ctl.iresi;
    A.h_fresi[row] = ctl.fresi;
    A.h_cl[row] = cl;
    A.h_cd[row] = cd;
  }
  ctl.iter += 1;
  ctl.n_done += 1;
  if (fres <= ctl.minres || ctl.n_done >= ctl.n_max) ctl.active = 0;
}

// ---------------------------------------------------------------------------
// Per-routine kernels (routine mode: state = buffer p, prim_old = p+2).
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(kBlockVerts) k_update(ArenaPtrs<R> A, int irk) {
  int w0, nwork;
  work_range(A, w0, nwork);
  for (int w = w0 + blockIdx.x; w < nwork; w += gridDim.x) {
    const BlockInfo bi = work_block(A, w);
    if (threadIdx.x >= bi.nv) continue;
    const MeshCtl &ctl = A.ctl[bi.mesh];
    const MeshConst &mc = A.mc[bi.mesh];
    const int v = bi.v0 + threadIdx.x;
    const int p = ctl.phase;
    const R4<R> r4 = A.res[v];
    const R res[4] = {r4.x, r4.y, r4.z, r4.w};
    const bool noslip = (mc.iflow != 1) && (A.vflag[v] & kVtxSolid);
    A.st[p][v] = rk_update<R>(mc, irk, A.st[(p + 2) % 3][v], A.st[p][v], A.dt[v], v_cvarea(A, v),
                              res, noslip);
  }
}

template <typename R>
__global__ void __launch_bounds__(kBlockVerts) k_time_step(ArenaPtrs<R> A) {
  int w0, nwork;
  work_range(A, w0, nwork);
  for (int w = w0 + blockIdx.x; w < nwork; w += gridDim.x) {
    const BlockInfo bi = work_block(A, w);
    if (threadIdx.x >= bi.nv) continue;
    const MeshCtl &ctl = A.ctl[bi.mesh];
    const int v = bi.v0 + threadIdx.x;
    A.dt[v] = time_step<R>(A.mc[bi.mesh], A.st[ctl.phase][v], A.mu[v], v_drmin(A, v));
  }
}

template <typename R>
__global__ void __launch_bounds__(kBlockVerts) k_positivity(ArenaPtrs<R> A) {
  int w0, nwork;
  work_range(A, w0, nwork);
  for (int w = w0 + blockIdx.x; w < nwork; w += gridDim.x) {
    const BlockInfo bi = work_block(A, w);
    if (threadIdx.x >= bi.nv) continue;
    MeshCtl &ctl = A.ctl[bi.mesh];
    const int v = bi.v0 + threadIdx.x;
    const R4<R> P = A.st[ctl.phase][v];
    if (P.x <= R(0) || P.w <= R(0) || A.nut[ctl.nphase][v] < R(0))
      atomicMin(&ctl.err_point, A.orig[v]);
  }
}

// conres.f:14-22 partials between buffer p and prim_old = p+2
template <typename R>
__global__ void __launch_bounds__(kBlockVerts) k_conres_part(ArenaPtrs<R> A) {
  __shared__ double s_red[kBlockVerts / 32], s_max[kBlockVerts / 32];
  __shared__ int s_arg[kBlockVerts / 32];
  int w0, nwork;
  work_range(A, w0, nwork);
  for (int w = w0 + blockIdx.x; w < nwork; w += gridDim.x) {
    const BlockInfo bi = work_block(A, w);
    const MeshCtl &ctl = A.ctl[bi.mesh];
    double d2 = 0.0, dabs = 0.0;
    int darg = INT_MAX;
    if (threadIdx.x < bi.nv) {
      const int v = bi.v0 + threadIdx.x;
      const double gra = double(A.st[ctl.phase][v].x) - double(A.st[(ctl.phase + 2) % 3][v].x);
      d2 = gra * gra;
      dabs = fabs(gra);
      if (dabs > 0.0) darg = A.orig[v];
      else dabs = 0.0;   // a NaN never becomes the maximum (conres.f:17-21)
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const double o2 = __shfl_down_sync(0xffffffffu, d2, off);
      const double om = __shfl_down_sync(0xffffffffu, dabs, off);
      const int oa = __shfl_down_sync(0xffffffffu, darg, off);
      d2 += o2;
      if (om > dabs || (om == dabs && oa < darg)) {
        dabs = om;
        darg = oa;
      }
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
      s_red[wid] = d2;
      s_max[wid] = dabs;
      s_arg[wid] = darg;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0, m = 0.0;
      int a = INT_MAX;
      for (int i = 0; i < (int)(blockDim.x >> 5); i++) {
        s += s_red[i];
        if (s_max[i] > m || (s_max[i] == m && s_arg[i] < a)) {
          m = s_max[i];
          a = s_arg[i];
        }
      }
      BlockPartial bp;
      bp.sumsq = s;
      bp.maxabs = m;
      bp.argmax = a;
      bp.pad = 0;
      A.part[bi.part] = bp;
    }
    __syncthreads();
  }
}

// conres (first: set fres1) or clcd for one mesh, routine mode.
template <typename R>
__global__ void __launch_bounds__(256) k_routine_monitor(ArenaPtrs<R> A, int mesh, int what,
                                                         int first, int serial_clcd) {
  MeshCtl &ctl = A.ctl[mesh];
  const MeshConst &mc = A.mc[mesh];
  if (what == 0) {
    double sum, mx;
    int arg;
    conres_block<R>(A, mc, sum, mx, arg);
    if (threadIdx.x != 0) return;
    double fres = sqrt(sum / double(mc.nv));
    ctl.fresi = mx;
    ctl.iresi = (mx > 0.0) ? arg : 0;
    if (first) {
      ctl.fres1 = fres;
      if (fres == 0.0) {
        ctl.fres = fres;
        ctl.err = 5;
        return;
      }
    }
    ctl.fres = fres / ctl.fres1;
  } else {
    double cl, cd;
    clcd_block<R>(A, mc, ctl.phase, serial_clcd, cl, cd);
    if (threadIdx.x != 0) return;
    ctl.cl = cl;
    ctl.cd = cd;
  }
}

// limitgrad.f:14-75 on the current gradients, one thread per vertex over
// all of its edges in edge order.
// ---------------------------------------------------------------------------
// gradient.f:1-63 (never called by the reference: main.f:29 comments it
// out), routine mode: edge-based Green-Gauss over the dual cells.  Each
// interior edge contributes +-(qa*ds) with qa the mean of its ends' states;
// each boundary edge contributes (5 p1 + p2)/6 and (p1 + 5 p2)/6 times half
// its rotated edge vector to its two ends; each vertex sums its interior
// edges in iedge order, then its boundary edges in beindx order (the flux
// pass's incidence lists), and divides by its dual-cell area.  The
// reference's print of every vertex (gradient.f:60) is left out.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(kBlockVerts) k_gradient_edge(ArenaPtrs<R> A) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  Grad<R> *s_g = reinterpret_cast<Grad<R> *>(smem_raw);   // [max_slots]
  int w0, nwork;
  work_range(A, w0, nwork);
  for (int w = w0 + blockIdx.x; w < nwork; w += gridDim.x) {
    const BlockInfo bi = work_block(A, w);
    const MeshCtl &ctl = A.ctl[bi.mesh];
    const R4<R> *P = A.st[ctl.phase];
    for (int k = threadIdx.x; k < bi.ne; k += blockDim.x) {
      const int2 nn = A.be_nodes[bi.e0 + k];
      const double2 ds = A.be_ds[bi.e0 + k];
      const R4<R> p1 = P[nn.x], p2 = P[nn.y];
      Grad<R> g;
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const R qa = R(0.5) * (comp(p1, q) + comp(p2, q));
        g.qx[q] = qa * R(ds.x);
        g.qy[q] = qa * R(ds.y);
      }
      s_g[k] = g;
    }
    for (int k = threadIdx.x; k < bi.nb; k += blockDim.x) {
      const int4 b = A.bb_nodes[bi.b0 + k];
      const double2 x1 = A.coord[b.x], x2 = A.coord[b.y];
      const R dx = R(x2.x - x1.x), dy = R(x2.y - x1.y);
      const R nx = R(0.5) * dy, ny = -R(0.5) * dx;
      const R4<R> p1 = P[b.x], p2 = P[b.y];
      Grad<R> g1, g2;
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const R qa1 = (R(5) * comp(p1, q) + comp(p2, q)) / R(6);
        const R qa2 = (comp(p1, q) + R(5) * comp(p2, q)) / R(6);
        g1.qx[q] = qa1 * nx;
        g1.qy[q] = qa1 * ny;
        g2.qx[q] = qa2 * nx;
        g2.qy[q] = qa2 * ny;
      }
      s_g[bi.ne + 2 * k] = g1;
      s_g[bi.ne + 2 * k + 1] = g2;
    }
    __syncthreads();
    if (threadIdx.x < bi.nv) {
      const int v = bi.v0 + threadIdx.x;
      R qx[4] = {R(0), R(0), R(0), R(0)}, qy[4] = {R(0), R(0), R(0), R(0)};
      const int2 jr = A.ve_rng[v];
      for (int j = jr.x; j < jr.y; j++) {
        const uint16_t e = A.ve_list[j];
        const Grad<R> g = s_g[e & kSlotMask];
        if (e & kNegBit) {      // n2 of an interior edge
#pragma unroll
          for (int q = 0; q < 4; q++) {
            qx[q] = qx[q] - g.qx[q];
            qy[q] = qy[q] - g.qy[q];
          }
        } else {
#pragma unroll
          for (int q = 0; q < 4; q++) {
            qx[q] = qx[q] + g.qx[q];
            qy[q] = qy[q] + g.qy[q];
          }
        }
      }
      const R ai = R(1) / v_cvarea(A, v);
      Grad<R> g;
#pragma unroll
      for (int q = 0; q < 4; q++) {
        g.qx[q] = ai * qx[q];
        g.qy[q] = ai * qy[q];
      }
      A.grad[v] = g;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// shockind.f:1-52 (never called by the reference), routine mode: the
// density-jump indicator of every vertex from all its edges (edge order),
// ind/drmin/cvarea**0.75; the gradients of vertices where it exceeds 1 are
// set to zero.  One thread per vertex; each edge's term is formed by both
// of its ends with the same operations, so both add the same value.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(kBlockVerts) k_shockind(ArenaPtrs<R> A) {
  int w0, nwork;
  work_range(A, w0, nwork);
  for (int w = w0 + blockIdx.x; w < nwork; w += gridDim.x) {
    const BlockInfo bi = work_block(A, w);
    if (threadIdx.x >= bi.nv) continue;
    const MeshCtl &ctl = A.ctl[bi.mesh];
    const MeshConst &mc = A.mc[bi.mesh];
    const int v = bi.v0 + threadIdx.x;
    const R4<R> *P = A.st[ctl.phase];
    const R a11 = MCR(R, albada11), a12 = MCR(R, albada12);
    R ind = R(0);
    const int2 r = A.va_rng[v];
    for (int j = r.x; j < r.y; j++) {
      const int raw = A.va_list[j];
      const int o = raw & 0x7fffffff;
      const bool is_n2 = raw < 0;
      const int n1 = is_n2 ? o : v, n2 = is_n2 ? v : o;
      const double2 c1 = A.coord[n1], c2 = A.coord[n2];
      const R dx = R(c2.x - c1.x), dy = R(c2.y - c1.y);
      const R r1 = P[n1].x, r2 = P[n2].x;
      const Grad<R> g1 = A.grad[n1], g2 = A.grad[n2];
      const R dvc = r2 - r1;
      R dvt = dx * g1.qx[0] + dy * g1.qy[0];
      const R dvl = a11 * dvt + a12 * dvc;
      const R vl = r1 + dvl;
      dvt = dx * g2.qx[0] + dy * g2.qy[0];
      const R dvr = a11 * dvt + a12 * dvc;
      const R vr = r2 - dvr;
      const R li = sq(vr - vl) * R(A.va_dsl[j]);
      ind = ind + li;
    }
    ind = ind / v_drmin(A, v) / mpow(v_cvarea(A, v), R(0.75));
    if (ind > R(1)) {
      Grad<R> z;
#pragma unroll
      for (int q = 0; q < 4; q++) z.qx[q] = z.qy[q] = R(0);
      A.grad[v] = z;
    }
  }
}

template <typename R>
__global__ void __launch_bounds__(kBlockVerts) k_limitgrad(ArenaPtrs<R> A) {
  int w0, nwork;
  work_range(A, w0, nwork);
  for (int w = w0 + blockIdx.x; w < nwork; w += gridDim.x) {
    const BlockInfo bi = work_block(A, w);
    if (threadIdx.x >= bi.nv) continue;
    const MeshCtl &ctl = A.ctl[bi.mesh];
    const MeshConst &mc = A.mc[bi.mesh];
    const int v = bi.v0 + threadIdx.x;
    const R4<R> *P = A.st[ctl.phase];
    const R4<R> pv = P[v];
    const double2 cv = A.coord[v];
    Grad<R> g = A.grad[v];
    R qmin[4], qmax[4], phi[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      qmin[q] = R(1.0e10);
      qmax[q] = R(-1.0e10);
      phi[q] = R(1);
    }
    const int2 ar = A.va_rng[v];
    const int j0 = ar.x, j1 = ar.y;
    for (int j = j0; j < j1; j++) {
      const int o = A.va_list[j] & 0x7fffffff;
      const R4<R> po = P[o];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        if (!mc.bugcompat) {
          qmin[q] = dmin1(qmin[q], comp(pv, q));
          qmax[q] = dmax1(qmax[q], comp(pv, q));
          qmin[q] = dmin1(qmin[q], comp(po, q));
          qmax[q] = dmax1(qmax[q], comp(po, q));
        } else {
          qmin[q] = dmin1(qmin[q], comp(pv, q));
          qmax[q] = dmax1(qmax[q], comp(pv, q));
        }
      }
    }
    for (int j = j0; j < j1; j++) {
      const int raw = A.va_list[j];
      const int o = raw & 0x7fffffff;
      const bool is_n2 = raw < 0;
      const double2 co = A.coord[o];
      // dx, dy always from edge(1) to edge(2)
      const R dx = is_n2 ? R(cv.x - co.x) : R(co.x - cv.x);
      const R dy = is_n2 ? R(cv.y - co.y) : R(co.y - cv.y);
#pragma unroll
      for (int q = 0; q < 4; q++) {
        R dq = g.qx[q] * dx + g.qy[q] * dy;
        if (is_n2) dq = -dq;
        const R dqmax = qmax[q] - comp(pv, q);
        const R dqmin = qmin[q] - comp(pv, q);
        if (dq != R(0)) {
          const R ppp = (dq > R(0)) ? dqmax / dq : dqmin / dq;
          phi[q] = dmin1(phi[q], ppp);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      g.qx[q] = phi[q] * g.qx[q];
      g.qy[q] = phi[q] * g.qy[q];
    }
    A.grad[v] = g;
  }
}

}  // namespace fvm

#include "fvm_pipe.cuh"
