// fvm_pipe.cuh -- warp-specialised, mbarrier-pipelined forms of the FP32
// block kernels.  Included by fvm_kernels.cuh.
//
// A CTA is one producer warp and NG consumer groups of kBlockVerts threads.
// Its blocks (the persistent grid-stride sequence over the work list,
// inactive meshes skipped) become jobs 0, 1, 2, ...; job j lives in stage
// j % nstages of a ring in shared memory and is processed by consumer group
// j % NG.  Two mbarriers per stage:
//   full[s]   armed by the producer (arrive + expected bytes); completes when
//             the stage's bulk copies have landed;
//   empty[s]  one arrival by the consumer group when it has finished with
//             the stage; the producer waits for it before refilling.
// The producer runs up to nstages jobs ahead of the consumers, so the copies
// of the next blocks stream from HBM while the groups compute, instead of
// each CTA alternating between waiting for its inputs and computing.
//
// Every wait is bounded (a clock64 budget, about a second in normal
// launches).  A wait that runs out sets FVM_ERR_TIMEOUT on the job's mesh
// and raises the CTA's abort flag; the other waits give up when they see the
// flag.  Consumers then leave at once.  Each consumer group signals a
// `done` mbarrier when it leaves, by any path; the producer waits for all
// groups (bounded), then for the copies of the jobs it issued last (one per
// stage at most) to have landed, and only then exits: no copy is in flight
// into the CTA's shared memory when the CTA ends.  Within a consumer group
// only its first thread waits on a barrier and the group follows its
// verdict through a named barrier, so every thread of the group reaches the
// same barriers.
#pragma once

namespace fvm {

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// barrier `id` (1..15) of `n` threads (a multiple of 32)
__device__ __forceinline__ void named_sync(int id, int n) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}

// Waits for the phase of the given parity.  false when the budget (clock64
// cycles) runs out or, if abort is given, when *abort is set.
__device__ __forceinline__ bool mbar_wait_budget(uint64_t *bar, uint32_t parity,
                                                 long long budget, const volatile int *abort) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (abort && *abort) return false;
    if (clock64() - t0 > budget) return false;
  }
  return true;
}

// Wait budget of the pipelined kernels in normal launches (about a second
// at 2 GHz).
constexpr long long kPipeBudget = 1LL << 31;

// What a consumer group needs to know of its job besides the staged data:
// the block and its mesh's state buffer, nu~ buffer and flow type (copied
// by the producer, so the consumers' first loads do not wait on them).
struct PipeJob {
  BlockInfo bi;
  int phase, nphase, iflow, pad;
};
static_assert(sizeof(BlockInfo) == 16 * sizeof(int), "BlockInfo is 16 ints");

__device__ __forceinline__ BlockInfo shfl_block(const BlockInfo &b, int src) {
  BlockInfo o;
  const int *pi = reinterpret_cast<const int *>(&b);
  int *po = reinterpret_cast<int *>(&o);
#pragma unroll
  for (int k = 0; k < 16; k++) po[k] = __shfl_sync(0xffffffffu, pi[k], src);
  return o;
}

// The producer warp's look-ahead: lane i loads the block of the CTA's
// sequence at position `first + i` (its block record, its mesh's control
// and flow type), so the dependent loads of 32 jobs are paid at once.
template <typename R>
struct PipeLook {
  BlockInfo bi;
  int ok, phase, nphase, iflow;
};
template <typename R>
__device__ __forceinline__ PipeLook<R> pipe_look(const ArenaPtrs<R> &A, int w, int nwork,
                                                 int routine, int skip_inviscid) {
  PipeLook<R> c;
  int *z = reinterpret_cast<int *>(&c.bi);
#pragma unroll
  for (int k = 0; k < 16; k++) z[k] = 0;
  c.ok = c.phase = c.nphase = c.iflow = 0;
  if (w < nwork) {
    c.bi = work_block(A, w);
    const MeshCtl &ctl = A.ctl[c.bi.mesh];
    c.phase = ctl.phase;
    c.nphase = ctl.nphase;
    c.iflow = A.mc[c.bi.mesh].iflow;
    c.ok = ((routine || ctl.active) && !(skip_inviscid && c.iflow == 1)) ? 1 : 0;
  }
  return c;
}

// Records a timed-out wait: FVM_ERR_TIMEOUT on `mesh` (or, when the stage
// never held a block, on the mesh of the CTA's first block) and the abort
// flag.
template <typename R>
__device__ __forceinline__ void pipe_timeout(const ArenaPtrs<R> &A, int mesh, int w_first,
                                             int nwork, volatile int *abort) {
  if (mesh < 0 && w_first < nwork) mesh = work_block(A, w_first).mesh;
  if (mesh >= 0) atomicCAS(&A.ctl[mesh].err, 0, 6 /* FVM_ERR_TIMEOUT */);
  *abort = 1;
  __threadfence_block();
}

// ---------------------------------------------------------------------------
// Pipelined gradient pass (FP32): green_gauss_euler / green_gauss_visc
// (green_gauss.f:2-92) with tri_gg and tri_visc, and at stage 1 of an
// inviscid iteration time_step.f:22-27.  The arithmetic and summation order
// are those of k_grad / k_grad_bulk (same bits).
//
// Per job the producer copies the block's triangle records (geometry and
// the ends' local slots), the vertex-triangle ranges and list, the own
// states, the halo ids, the own (1/6)/mcarea and (stage-1 time step) drmin.
// The consumer group first gathers the halo states into the stage (one
// round of loads), then computes every triangle's sums from shared memory
// only, then each vertex's gradient.
//
// inject != 0 (tests of the bounded wait only): the first job of each CTA
// is armed with its byte count but its copies are never issued, so its
// consumer's wait runs out after `budget` cycles with nothing in flight.
// ---------------------------------------------------------------------------
template <typename R, int NG>
__global__ void __launch_bounds__(32 + NG * kBlockVerts, 1)
    k_grad_pipe(ArenaPtrs<R> A, int stage, int do_dt, int routine, int max_tri, int max_halo,
                int viscous, int nstages, long long budget, int inject, int skip_inviscid) {
  if constexpr (sizeof(R) == 4) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full[kPipeMaxStages], empty[kPipeMaxStages], done;
    __shared__ PipeJob s_job[kPipeMaxStages];
    __shared__ int s_ok[NG];
    __shared__ volatile int s_abort;
    const GradPipeLayout lay = grad_pipe_layout(max_tri, max_halo, viscous != 0);
    int w0, nwork;
    work_range(A, w0, nwork);
    const int w_first = w0 + blockIdx.x;
    if (threadIdx.x == 0) {
      for (int s = 0; s < nstages; s++) {
        mbar_init(&full[s], 1);
        mbar_init(&empty[s], 1);
        s_job[s].bi.mesh = -1;
      }
      mbar_init(&done, NG);
      s_abort = 0;
    }
    __syncthreads();

    if (threadIdx.x < 32) {
      // ---------------- producer warp (lane 0 issues) ----------------
      const int lane = threadIdx.x;
      int j = 0;
      bool aborted = false;
      for (int wb = w_first; wb < nwork && !aborted; wb += 32 * gridDim.x) {
        const PipeLook<R> look =
            pipe_look(A, wb + lane * (int)gridDim.x, nwork, routine, skip_inviscid);
        unsigned todo = __ballot_sync(0xffffffffu, look.ok);
        while (todo) {
          const int src = __ffs(todo) - 1;
          todo &= todo - 1;
          const BlockInfo bi = shfl_block(look.bi, src);
          const int phase = __shfl_sync(0xffffffffu, look.phase, src);
          const int nphase = __shfl_sync(0xffffffffu, look.nphase, src);
          const int iflow = __shfl_sync(0xffffffffu, look.iflow, src);
          const int s = j % nstages;
          int ok = 1;
          if (lane == 0 && j >= nstages) {
            ok = mbar_wait_budget(&empty[s], ((j / nstages) & 1) ^ 1, budget, &s_abort);
            if (!ok && !s_abort) pipe_timeout(A, bi.mesh, w_first, nwork, &s_abort);
          }
          if (lane == 0 && s_abort) ok = 0;
          ok = __shfl_sync(0xffffffffu, ok, 0);
          if (!ok) {
            aborted = true;
            break;
          }
          if (lane == 0) {
            s_job[s].bi = bi;
            s_job[s].phase = phase;
            s_job[s].nphase = nphase;
            s_job[s].iflow = iflow;
            const R4<R> *P = A.st[cur_buf(phase, stage)];
            const bool dt_here = do_dt && iflow == 1;
            unsigned char *sb = smem_raw + (size_t)s * lay.stage;
            const int vt_a = bi.vt0 & ~7, vt_b = (bi.vt0 + bi.nvt + 7) & ~7;
            const int h_a = bi.h0 & ~3, h_b = (bi.h0 + bi.nh + 3) & ~3;
            const uint32_t ngeo = 32u * bi.nt;
            const uint32_t nvtr = 8u * ((bi.nv + 1) & ~1), nvtl = 2u * (vt_b - vt_a);
            const uint32_t npv = 16u * bi.nv, nhid = 4u * (h_b - h_a);
            const uint32_t nais = 4u * ((bi.nv + 3) & ~3), ndrm = dt_here ? nais : 0u;
            mbar_expect_tx(&full[s], ngeo + nvtr + nvtl + npv + nhid + nais + ndrm);
            if (!(inject && j == 0)) {
              if (ngeo) bulk_g2s(sb + lay.geo, A.tri_g32 + bi.t0, ngeo, &full[s]);
              bulk_g2s(sb + lay.vtr, A.vt_rng + bi.v0, nvtr, &full[s]);
              if (nvtl) bulk_g2s(sb + lay.vtl, A.vt_list + vt_a, nvtl, &full[s]);
              bulk_g2s(sb + lay.pv, P + bi.v0, npv, &full[s]);
              if (nhid) bulk_g2s(sb + lay.hid, A.halo_ids + h_a, nhid, &full[s]);
              bulk_g2s(sb + lay.ais, A.ais32 + bi.v0, nais, &full[s]);
              if (ndrm) bulk_g2s(sb + lay.drm, A.drmin32 + bi.v0, ndrm, &full[s]);
            }
          }
          j++;
        }
      }
      // one end marker per consumer group
      for (int k = 0; k < NG && !aborted; k++, j++) {
        const int s = j % nstages;
        int ok = 1;
        if (lane == 0 && j >= nstages) {
          ok = mbar_wait_budget(&empty[s], ((j / nstages) & 1) ^ 1, budget, &s_abort);
          if (!ok && !s_abort) pipe_timeout(A, -1, w_first, nwork, &s_abort);
        }
        if (lane == 0 && s_abort) ok = 0;
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) {
          aborted = true;
          break;
        }
        if (lane == 0) {
          s_job[s].bi.nv = -1;
          s_job[s].bi.mesh = -1;
          mbar_arrive(&full[s]);
        }
      }
      (void)aborted;
      if (lane == 0) {
        // every consumer group has left, and the copies of the jobs issued
        // last (one per stage at most) have landed, before the CTA may end
        (void)mbar_wait_budget(&done, 0, budget, nullptr);
        for (int jj = j > nstages ? j - nstages : 0; jj < j; jj++)
          (void)mbar_wait_budget(&full[jj % nstages], (jj / nstages) & 1, budget, nullptr);
      }
      __syncwarp();
      return;
    }

    // ---------------- consumer groups ----------------
    const int g = (threadIdx.x - 32) / kBlockVerts;
    const int t = (threadIdx.x - 32) % kBlockVerts;
    for (int j = g;; j += NG) {
      const int s = j % nstages;
      const uint32_t par = (j / nstages) & 1;
      if (t == 0) {
        int ok = mbar_wait_budget(&full[s], par, budget, &s_abort);
        if (!ok && !s_abort) pipe_timeout(A, s_job[s].bi.mesh, w_first, nwork, &s_abort);
        s_ok[g] = ok;
      }
      named_sync(1 + g, kBlockVerts);
      if (!s_ok[g]) {
        if (t == 0) mbar_arrive(&done);
        return;
      }
      // the phase has completed: this returns at once and gives every
      // thread the copies' data
      (void)mbar_wait_budget(&full[s], par, budget, nullptr);
      const BlockInfo bi = s_job[s].bi;
      const int phase = s_job[s].phase, nphase = s_job[s].nphase;
      const bool visc = s_job[s].iflow != 1;
      if (bi.nv < 0) {   // end marker
        if (t == 0) mbar_arrive(&done);
        return;
      }
      unsigned char *sb = smem_raw + (size_t)s * lay.stage;
      const TriGeo32 *s_geo = reinterpret_cast<const TriGeo32 *>(sb + lay.geo);
      TriSmem<R> *s_tri = reinterpret_cast<TriSmem<R> *>(sb + lay.geo);   // in place
      R *s_vis = reinterpret_cast<R *>(sb + lay.vis);
      const int2 *s_vtr = reinterpret_cast<const int2 *>(sb + lay.vtr);
      const uint16_t *s_vtl = reinterpret_cast<const uint16_t *>(sb + lay.vtl);
      const R4<R> *s_pv = reinterpret_cast<const R4<R> *>(sb + lay.pv);
      R4<R> *s_hst = reinterpret_cast<R4<R> *>(sb + lay.hst);
      const int *s_hid = reinterpret_cast<const int *>(sb + lay.hid) + (bi.h0 & 3);
      const float *s_ais = reinterpret_cast<const float *>(sb + lay.ais);
      const float *s_drm = reinterpret_cast<const float *>(sb + lay.drm);
      const MeshConst &mc = A.mc[bi.mesh];
      const R4<R> *P = A.st[cur_buf(phase, stage)];
      // halo states: this thread's first halo vertex is loaded into a
      // register now and stored after the interior triangles, so the load's
      // latency hides under them (any further halo vertices, a block of
      // more than kBlockVerts halo vertices, are loaded after)
      R4<R> h0 = {R(0), R(0), R(0), R(0)};
      if (t < bi.nh) h0 = P[s_hid[t]];
      auto state = [&](uint32_t l) { return l < (uint32_t)bi.nv ? s_pv[l] : s_hst[l - bi.nv]; };
      auto vertex = [&](uint32_t l) { return l < (uint32_t)bi.nv ? bi.v0 + (int)l : s_hid[l - bi.nv]; };
      auto triangle = [&](int k, const TriGeo32 &tg, uint32_t l1, uint32_t l2, uint32_t l3) {
        const R4<R> p1 = state(l1), p2 = state(l2), p3 = state(l3);
        R dbxx[3], dbyy[3];
#pragma unroll
        for (int q = 0; q < 3; q++) {
          dbxx[q] = tg.dbxx[q];
          dbyy[q] = tg.dbyy[q];
        }
        TriSmem<R> ts;
        tri_sums<R>(p1, p2, p3, dbxx, dbyy, ts);
        if (visc) {
          const int4 tv4 = make_int4(vertex(l1), vertex(l2), vertex(l3), 0);
          const TriVisc<R> tv = tri_visc<R>(A, mc, nphase, tv4, tg.areat, p1, p2, p3, dbxx,
                                            dbyy, ts);
          R *sv = s_vis + 9 * k;
#pragma unroll
          for (int q = 0; q < 3; q++) tri_visc_term<R>(tv, dbxx[q], dbyy[q], sv + 3 * q);
        }
        s_tri[k] = ts;   // over this thread's own record
      };
      constexpr uint32_t lm = (uint32_t)(kTriLocMax - 1);
      // phase 1a: the triangles whose three ends are the block's own
      // (listed first); those touching the halo wait for its states
      const int rounds = bi.nt > t ? (bi.nt - t + kBlockVerts - 1) / kBlockVerts : 0;
      uint32_t deferred = 0;
#pragma unroll 2
      for (int r = 0; r < rounds && r < 32; r++) {
        const int k = t + r * kBlockVerts;
        const TriGeo32 tg = s_geo[k];
        const uint32_t l1 = tg.loc & lm, l2 = (tg.loc >> kTriLocBits) & lm,
                       l3 = (tg.loc >> (2 * kTriLocBits)) & lm;
        if (max(l1, max(l2, l3)) >= (uint32_t)bi.nv) {
          deferred |= 1u << r;
          continue;
        }
        triangle(k, tg, l1, l2, l3);
      }
      if (t < bi.nh) s_hst[t] = h0;
      for (int h = t + kBlockVerts; h < bi.nh; h += kBlockVerts) s_hst[h] = P[s_hid[h]];
      named_sync(1 + g, kBlockVerts);
      // phase 1b: the triangles touching the halo
      for (int r = 0; r < rounds; r++) {
        if (r < 32 && !((deferred >> r) & 1u)) continue;
        const int k = t + r * kBlockVerts;
        const TriGeo32 tg = s_geo[k];
        const uint32_t l1 = tg.loc & lm, l2 = (tg.loc >> kTriLocBits) & lm,
                       l3 = (tg.loc >> (2 * kTriLocBits)) & lm;
        triangle(k, tg, l1, l2, l3);
      }
      named_sync(1 + g, kBlockVerts);
      // phase 2: one thread per vertex, its triangles in original order
      if (t < bi.nv) {
        const int v = bi.v0 + t;
        const int vt_a = bi.vt0 & ~7;
        R qx[4], qy[4], rv[3];
        const int2 jr = s_vtr[t];
        grad_vertex_sums<R, 4>(s_vtl, jr.x - vt_a, jr.y - vt_a, s_tri, visc ? s_vis : nullptr, qx,
                               qy, rv);
        const R ais = s_ais[t];
        Grad<R> gr;
#pragma unroll
        for (int q = 0; q < 4; q++) {
          gr.qx[q] = qx[q] * ais;
          gr.qy[q] = qy[q] * ais;
        }
        A.grad[v] = gr;
        if (visc) {
          R4<R> rr;
          rr.x = R(0);
          rr.y = rv[0];
          rr.z = rv[1];
          rr.w = rv[2];
          A.resv[v] = rr;
        } else if (do_dt) {
          A.dt[v] = time_step<R>(mc, s_pv[t], R(0), s_drm[t]);
        }
      }
      // the stage may be refilled by bulk copies once every thread of the
      // group is done with it
      fence_proxy_async_smem();
      named_sync(1 + g, kBlockVerts);
      if (t == 0) mbar_arrive(&empty[s]);
    }
  }
}

}  // namespace fvm
