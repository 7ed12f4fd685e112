// fvm_batch.cpp -- host runtime of include/fvm_gpu.h.
//
// A Batch owns one device arena: every array of the hot path sized for a
// capacity of vertices, block entries, incidence entries and mesh slots,
// sub-allocated per mesh by first-fit range allocators.  Meshes are
// admitted (fvm_batch_add) and retired (fvm_batch_remove) between steps;
// the block work list lives in device memory, so the captured iteration
// graph never changes.  The single-mesh fvm_gpu_* entry points are a batch
// of one sized exactly for its mesh.
#include <algorithm>
#include <climits>
#include <cstddef>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/fvm_gpu.h"
#include "fvm_internal.h"
#include "fvm_launch.h"
#include "fvm_layout.h"

using namespace fvm;

namespace {

constexpr int kHistRows = 512;    // history ring per slot (RES.DAT rows)
#ifndef FVM_GRAPH_ITERS
#define FVM_GRAPH_ITERS 10
#endif
constexpr int kGraphIters = FVM_GRAPH_ITERS;   // iterations per graph launch (untimed steps)

// first-fit allocator of index ranges [0, cap)
class RangeAlloc {
 public:
  void init(int64_t cap) {
    cap_ = cap;
    free_.clear();
    if (cap > 0) free_[0] = cap;
  }
  int64_t alloc(int64_t n) {   // -1 when no room; n == 0 gives 0
    if (n <= 0) return 0;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= n) {
        const int64_t off = it->first, len = it->second;
        free_.erase(it);
        if (len > n) free_[off + n] = len - n;
        return off;
      }
    }
    return -1;
  }
  void release(int64_t off, int64_t n) {
    if (n <= 0) return;
    auto it = free_.emplace(off, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  int64_t cap() const { return cap_; }

 private:
  int64_t cap_ = 0;
  std::map<int64_t, int64_t> free_;
};

enum Pool { P_V, P_BLK, P_BE, P_BB, P_BT, P_TRI, P_VE, P_VT, P_VA, P_SW, P_HALO, P_HP, P_HL, P_COUNT };

struct Slot {
  bool used = false;
  bool staged = false;        // uploaded on the side stream, not yet in the work list
  fvm_params par{};
  MeshLayout L;
  int64_t off[P_COUNT] = {0};
  int64_t len[P_COUNT] = {0};
};

// math.f:8-40's values of the constants the flux pass uses (as
// fvm_params_init sets them; pi compared with its correctly rounded double)
bool standard_constants(const fvm_params &p) {
  return p.gamma == 1.4 && p.gamma1 == 1.4 - 1.0 && p.albada11 == 2.0 / 3.0 &&
         p.albada12 == 1.0 - 2.0 / 3.0 && p.albada21 == 4.0 / 3.0 &&
         p.albada22 == 1.0 - 4.0 / 3.0 && p.epsilon == 1.0e-16 && p.pi == 3.141592653589793;
}

const char *kKernelNames[] = {"visc", "grad", "flux", "sa", "monitor", "step"};
enum { K_VISC, K_GRAD, K_FLUX, K_SA, K_MON, K_STEP, K_COUNT };

}  // namespace

struct fvm_batch {
  int prec = FVM_PREC_FP64;
  size_t rsz = 8;
  fvm_batch_caps caps{};
  int64_t cap[P_COUNT] = {0};
  RangeAlloc pool[P_COUNT];
  std::vector<Slot> slots;
  cudaStream_t stream = nullptr;
  // further chains of the overlapped iteration (chain 0 runs on `stream`)
  cudaStream_t chain_stream[kMaxChains] = {};
  cudaEvent_t ev_fork[kMaxChains] = {}, ev_join[kMaxChains] = {};
  int chains = 1;                          // chains of kernels over parts of the meshes
  std::vector<void *> owned;
  // device arrays
  void *st[3] = {nullptr, nullptr, nullptr};
  void *grad = nullptr, *resv = nullptr, *res = nullptr;
  void *dt = nullptr, *mu = nullptr, *mul = nullptr, *nut[2] = {nullptr, nullptr};
  double2 *coord = nullptr;
  double *ais = nullptr, *cvarea = nullptr, *drmin = nullptr, *wd = nullptr;
  float *ais32 = nullptr, *cvarea32 = nullptr, *drmin32 = nullptr, *wd32 = nullptr;   // FP32
  int *orig = nullptr;
  uint8_t *vflag = nullptr;
  int2 *ve_rng = nullptr, *vt_rng = nullptr, *va_rng = nullptr;
  uint16_t *ve_list = nullptr, *vt_list = nullptr;
  int *va_list = nullptr;
  float2 *va_w = nullptr;   // FP32: Green-Gauss stencil weights per va_list entry
  double *va_dsl = nullptr; // |ds| of each va_list entry's edge
  BlockInfo *blocks = nullptr;
  BlockInfo *wblocks = nullptr;   // blocks[work[w]], refreshed with the work list
  int2 *be_nodes = nullptr, *sw_nodes = nullptr;
  double2 *be_ds = nullptr;
  D4 *be_csl = nullptr;
  int4 *bb_nodes = nullptr, *bt_nodes = nullptr;
  double *elarea = nullptr;
  EdgeGeo32 *be_g32 = nullptr;
  TriGeo32 *tri_g32 = nullptr;
  uint32_t *be_loc = nullptr;
  int *halo_ids = nullptr, *hl_ptr = nullptr;
  uint16_t *hl_list = nullptr;
  bool fused = false;          // the fused pass runs (wanted and fits)
  bool fused_wanted = false;   // asked for by the caps or chosen by the tuner
  bool fused_fits = true;      // resident halo tiles within max_tri2 / max_loc
  bool run_sa = false;         // a turbulent mesh is resident
  MeshConst *mc = nullptr;
  MeshCtl *ctl = nullptr;
  BlockPartial *part = nullptr;
  double *h_fres = nullptr, *h_fresi = nullptr, *h_cl = nullptr, *h_cd = nullptr;
  int *h_iresi = nullptr;
  int *work = nullptr, *nwork = nullptr;
  int *mesh_part = nullptr;                // per slot: the part (chain) holding its blocks
  std::vector<int> mesh_part_h;
  LaunchCfg cfg{};
  bool any_turbulent_ok = true;
  cudaGraphExec_t graph = nullptr;         // one iteration
  cudaGraphExec_t graph_multi = nullptr;   // kGraphIters iterations
  // timing
  bool timing = false;
  std::vector<cudaEvent_t> ev;    // pairs around each kernel of an iteration
  std::vector<int> ev_kind;
  double t_ms[K_COUNT] = {0};
  int64_t t_launch[K_COUNT] = {0};
  int64_t launches = 0;           // kernels launched since creation
  int kernels_per_iter = 0;
  cudaStream_t upload = nullptr;      // side stream of deferred admissions
  bool pending = false;               // staged slots wait for batch_commit
  double *dstage = nullptr;           // device staging of driver-order state transfers
  size_t dstage_size = 0;
  // autotuner: each candidate form's last measured ms per iteration, calls
  double tune_last[16] = {};
  int tune_calls = 0;
  std::string last_error;
};

namespace {

template <typename T>
cudaError_t dalloc(std::vector<void *> &owned, T **p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  void *q = nullptr;
  cudaError_t e = cudaMalloc(&q, n * sizeof(T));
  if (e != cudaSuccess) return e;
  owned.push_back(q);
  *p = static_cast<T *>(q);
  return cudaSuccess;
}

int32_t cuda_status(fvm_batch *b, cudaError_t e) {
  if (e == cudaSuccess) return FVM_OK;
  if (b) b->last_error = cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return FVM_ERR_NOMEM;
  return FVM_ERR_CUDA;
}

#define FVM_TRY(b, expr)                              \
  do {                                                \
    cudaError_t _e = (expr);                          \
    if (_e != cudaSuccess) return cuda_status(b, _e); \
  } while (0)

template <typename R>
ArenaPtrs<R> ptrs(const fvm_batch *b) {
  ArenaPtrs<R> A;
  std::memset(&A, 0, sizeof(A));
  for (int i = 0; i < 3; i++) A.st[i] = static_cast<R4<R> *>(b->st[i]);
  A.grad = static_cast<Grad<R> *>(b->grad);
  A.resv = static_cast<R4<R> *>(b->resv);
  A.res = static_cast<R4<R> *>(b->res);
  A.dt = static_cast<R *>(b->dt);
  A.mu = static_cast<R *>(b->mu);
  A.mul = static_cast<R *>(b->mul);
  A.nut[0] = static_cast<R *>(b->nut[0]);
  A.nut[1] = static_cast<R *>(b->nut[1]);
  A.coord = b->coord;
  A.ais = b->ais;
  A.cvarea = b->cvarea;
  A.drmin = b->drmin;
  A.ais32 = b->ais32;
  A.cvarea32 = b->cvarea32;
  A.drmin32 = b->drmin32;
  A.wd32 = b->wd32;
  A.wd = b->wd;
  A.orig = b->orig;
  A.vflag = b->vflag;
  A.ve_rng = b->ve_rng;
  A.ve_list = b->ve_list;
  A.vt_rng = b->vt_rng;
  A.vt_list = b->vt_list;
  A.blocks = b->blocks;
  A.wblocks = b->wblocks;
  A.be_nodes = b->be_nodes;
  A.be_ds = b->be_ds;
  A.be_csl = b->be_csl;
  A.bb_nodes = b->bb_nodes;
  A.bt_nodes = b->bt_nodes;
  A.elarea = b->elarea;
  A.be_g32 = b->be_g32;
  A.tri_g32 = b->tri_g32;
  A.be_loc = b->be_loc;
  A.halo_ids = b->halo_ids;
  A.hl_ptr = b->hl_ptr;
  A.hl_list = b->hl_list;
  A.sw_nodes = b->sw_nodes;
  A.va_rng = b->va_rng;
  A.va_list = b->va_list;
  A.va_w = b->va_w;
  A.va_dsl = b->va_dsl;
  A.mc = b->mc;
  A.ctl = b->ctl;
  A.part = b->part;
  A.h_fres = b->h_fres;
  A.h_fresi = b->h_fresi;
  A.h_cl = b->h_cl;
  A.h_cd = b->h_cd;
  A.h_iresi = b->h_iresi;
  A.work = b->work;
  A.nwork = b->nwork;
  A.mesh_part = b->mesh_part;
  A.wpart = 0;
  A.nslots = (int)b->slots.size();
  return A;
}

MeshConst make_const(const fvm_params &p) {
  MeshConst c;
  std::memset(&c, 0, sizeof(c));
  c.iflow = p.iflow;
  c.iflux = p.iflux;
  c.ilimit = p.ilimit;
  c.vortex = p.vortex;
  c.bugcompat = p.bugcompat;
  c.precision = p.precision;
  c.gamma = p.gamma;
  c.gamma1 = p.gamma1;
  c.gas_const = p.gas_const;
  c.pi = p.pi;
  c.prandtl = p.prandtl;
  c.prandtl_turb = p.prandtl_turb;
  c.albada11 = p.albada11;
  c.albada12 = p.albada12;
  c.albada21 = p.albada21;
  c.albada22 = p.albada22;
  c.epsilon = p.epsilon;
  c.cb1 = p.cb1;
  c.cb2 = p.cb2;
  c.sigma_sa = p.sigma_sa;
  c.kolm = p.kolm;
  c.cw1 = p.cw1;
  c.cw2 = p.cw2;
  c.cw3 = p.cw3;
  c.cv1 = p.cv1;
  c.cv2 = p.cv2;
  c.cv11 = p.cv11;
  c.cw31 = p.cw31;
  c.cw32 = p.cw32;
  c.kolm2 = p.kolm2;
  c.cb2sig1 = p.cb2sig1;
  c.cb2sig2 = p.cb2sig2;
  c.mach_inf = p.mach_inf;
  c.aoa = p.aoa;
  c.rey = p.rey;
  c.cfl = p.cfl;
  c.q_inf = p.q_inf;
  c.r_inf = p.r_inf;
  c.p_inf = p.p_inf;
  c.t_inf = p.t_inf;
  c.u_inf = p.u_inf;
  c.v_inf = p.v_inf;
  c.a_inf = p.a_inf;
  c.sconst = p.sconst;
  c.nut_inf = p.nut_inf;
  c.xref = p.xref;
  c.yref = p.yref;
  for (int k = 0; k < 3; k++) {
    c.airk[k] = p.airk[k];
    c.birk[k] = p.birk[k];
  }
  c.sin_aoa = std::sin(p.aoa);
  c.cos_aoa = std::cos(p.aoa);
  MeshConstF &f = c.f;
#define F32(x) f.x = (float)c.x
  F32(gamma); F32(gamma1); F32(gas_const); F32(pi); F32(prandtl); F32(prandtl_turb);
  F32(albada11); F32(albada12); F32(albada21); F32(albada22); F32(epsilon);
  F32(cb1); F32(cb2); F32(sigma_sa); F32(kolm); F32(cw1); F32(cw2); F32(cw3); F32(cv1); F32(cv2);
  F32(cv11); F32(cw31); F32(cw32); F32(kolm2); F32(cb2sig1); F32(cb2sig2);
  F32(mach_inf); F32(aoa); F32(rey); F32(cfl);
  F32(q_inf); F32(r_inf); F32(p_inf); F32(t_inf); F32(u_inf); F32(v_inf); F32(a_inf);
  F32(sconst); F32(nut_inf);
  for (int k = 0; k < 3; k++) {
    F32(airk[k]);
    F32(birk[k]);
  }
#undef F32
  return c;
}

// device staging buffer of at least n bytes
double *dstaging(fvm_batch *b, size_t n, cudaError_t &e) {
  e = cudaSuccess;
  if (b->dstage_size < n) {
    if (b->dstage) cudaFree(b->dstage);
    b->dstage = nullptr;
    b->dstage_size = 0;
    void *p = nullptr;
    e = cudaMalloc(&p, n);
    if (e != cudaSuccess) return nullptr;
    b->dstage = static_cast<double *>(p);
    b->dstage_size = n;
  }
  return b->dstage;
}

int32_t get_ctl(fvm_batch *b, int slot, MeshCtl &c) {
  FVM_TRY(b, cudaMemcpyAsync(&c, b->ctl + slot, sizeof(MeshCtl), cudaMemcpyDeviceToHost, b->stream));
  FVM_TRY(b, cudaStreamSynchronize(b->stream));
  return FVM_OK;
}

int32_t put_ctl(fvm_batch *b, int slot, const MeshCtl &c) {
  FVM_TRY(b, cudaMemcpyAsync(b->ctl + slot, &c, sizeof(MeshCtl), cudaMemcpyHostToDevice, b->stream));
  FVM_TRY(b, cudaStreamSynchronize(b->stream));
  return FVM_OK;
}

// device [np][stride] of the slot, values c0..c0+k-1 -> host double [np][k]
// in driver order (permuted and widened on the device); queued on the batch
// stream, complete after the caller's synchronisation
int32_t get_vertex(fvm_batch *b, const Slot &s, double *dst, const void *src_base, int k,
                   size_t stride, int c0 = 0) {
  const int np = s.L.np;
  const size_t n = (size_t)np * k * sizeof(double);
  cudaError_t e;
  double *stage = dstaging(b, n, e);
  FVM_TRY(b, e);
  const unsigned char *src = static_cast<const unsigned char *>(src_base) + (size_t)s.off[P_V] * stride;
  FVM_TRY(b, launch_get_vertex(b->rsz, stage, src, stride, b->orig + s.off[P_V], np, k, c0, b->stream));
  FVM_TRY(b, cudaMemcpyAsync(dst, stage, n, cudaMemcpyDeviceToHost, b->stream));
  return FVM_OK;
}

int32_t sync_stream(fvm_batch *b) {
  FVM_TRY(b, cudaStreamSynchronize(b->stream));
  return FVM_OK;
}

// The same transfers for a slot's state arrays whose buffer rotates with the
// mesh (state: ctl.phase of 3, nu~: ctl.nphase of 2) or not (one buffer):
// the device picks the buffer from the control block, so no host read of
// it is needed.  Queued on the batch stream.
enum class Rot { None, Phase, NutPhase };
struct RotBufs {
  unsigned char *b[3];
  const int *sel;
};
RotBufs rot_bufs(fvm_batch *b, int32_t slot, Rot rot, void *single) {
  RotBufs r;
  const char *ctl = reinterpret_cast<const char *>(b->ctl + slot);
  r.sel = reinterpret_cast<const int *>(ctl + (rot == Rot::NutPhase ? offsetof(MeshCtl, nphase)
                                                                     : offsetof(MeshCtl, phase)));
  if (rot == Rot::Phase) {
    for (int i = 0; i < 3; i++) r.b[i] = static_cast<unsigned char *>(b->st[i]);
  } else if (rot == Rot::NutPhase) {
    r.b[0] = static_cast<unsigned char *>(b->nut[0]);
    r.b[1] = r.b[2] = static_cast<unsigned char *>(b->nut[1]);
  } else {
    r.b[0] = r.b[1] = r.b[2] = static_cast<unsigned char *>(single);
  }
  return r;
}

int32_t put_vertex_rot(fvm_batch *b, int32_t slot, const Slot &s, Rot rot, void *single,
                       const double *src, int k, size_t stride) {
  const int np = s.L.np;
  const size_t n = (size_t)np * k * sizeof(double);
  cudaError_t e;
  double *stage = dstaging(b, n, e);
  FVM_TRY(b, e);
  const RotBufs rb = rot_bufs(b, slot, rot, single);
  FVM_TRY(b, cudaMemcpyAsync(stage, src, n, cudaMemcpyHostToDevice, b->stream));
  FVM_TRY(b, launch_put_vertex_sel(b->rsz, rb.b, rb.sel, (size_t)s.off[P_V] * stride, stride,
                                   stage, b->orig + s.off[P_V], np, k, b->stream));
  return FVM_OK;
}

int32_t get_vertex_rot(fvm_batch *b, int32_t slot, const Slot &s, Rot rot, void *single,
                       double *dst, int k, size_t stride, int c0 = 0) {
  const int np = s.L.np;
  const size_t n = (size_t)np * k * sizeof(double);
  cudaError_t e;
  double *stage = dstaging(b, n, e);
  FVM_TRY(b, e);
  const RotBufs rb = rot_bufs(b, slot, rot, single);
  FVM_TRY(b, launch_get_vertex_sel(b->rsz, stage, rb.b, rb.sel, (size_t)s.off[P_V] * stride,
                                   stride, b->orig + s.off[P_V], np, k, c0, b->stream));
  FVM_TRY(b, cudaMemcpyAsync(dst, stage, n, cudaMemcpyDeviceToHost, b->stream));
  return FVM_OK;
}

template <typename T>
cudaError_t put_range(fvm_batch *b, T *base, int64_t off, const std::vector<T> &h,
                      cudaStream_t s = nullptr) {
  if (h.empty()) return cudaSuccess;
  return cudaMemcpyAsync(base + off, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice,
                         s ? s : b->stream);
}

void drop_graphs(fvm_batch *b);

int32_t update_work(fvm_batch *b) {
  std::vector<int> work, mesh_first;
  int flux = -1;
  for (const Slot &s : b->slots)
    if (s.used && !s.staged) {
      mesh_first.push_back((int)work.size());
      for (int k = 0; k < s.L.nblk; k++) work.push_back((int)(s.off[P_BLK] + k));
      flux = (flux == -1 || flux == s.par.iflux) ? s.par.iflux : 0;
    }
  if (flux < 0) flux = b->cfg.flux;   // empty batch: keep the current kernels
  // Shared-memory tiles sized for the resident meshes (rounded up to 8, so
  // small changes of the mix keep the graph), never above the arena's
  // capacities: smaller tiles let more CTAs share an SM.
  int tile[4] = {0, 0, 0, 0};
  int max_halo = 0;
  bool any_visc = false, any_turb = false, any_inv = false, tri_loc = true, std_const = true;
  for (const Slot &s : b->slots)
    if (s.used && !s.staged) {
      std_const &= standard_constants(s.par);
      any_visc |= s.par.iflow != FVM_INVISCID;
      any_inv |= s.par.iflow == FVM_INVISCID;
      any_turb |= s.par.iflow == FVM_TURBULENT;
      tile[0] = std::max(tile[0], s.L.max_tri);
      tile[1] = std::max(tile[1], s.L.max_slots);
      tile[2] = std::max(tile[2], s.L.max_tri2);
      tile[3] = std::max(tile[3], s.L.max_loc);
      max_halo = std::max(max_halo, s.L.max_halo);
      tri_loc &= s.L.max_loc <= kTriLocMax;
    }
  // the bulk gradient pass's halo ids (rounded up to 8 like the tiles; a
  // block of more than kTriLocMax own + halo vertices sends the pass to its
  // per-thread form while its mesh is resident)
  max_halo = std::min((max_halo + 7) & ~7, kTriLocMax);
  bool changed_halo = max_halo != b->cfg.max_halo || tri_loc != b->cfg.tri_loc;
  b->cfg.max_halo = max_halo;
  b->cfg.tri_loc = tri_loc;
  const int cap[4] = {b->caps.max_tri, b->caps.max_slots, b->caps.max_tri2, b->caps.max_loc};
  int *cur[4] = {&b->cfg.max_tri, &b->cfg.max_slots, &b->cfg.max_tri2, &b->cfg.max_loc};
  bool changed = flux != b->cfg.flux || changed_halo || std_const != b->cfg.std_const;
  b->cfg.std_const = std_const;
  b->cfg.flux = flux;
  for (int i = 0; i < 4; i++) {
    if (!tile[i]) continue;             // empty batch: keep the current tiles
    const int t = std::min(cap[i], (tile[i] + 7) & ~7);
    changed |= t != *cur[i];
    *cur[i] = t;
  }
  // kernels for viscous terms and the SA model only while such meshes are
  // resident (the shared memory of viscous terms likewise)
  const bool visc_now = b->caps.viscous != 0 && any_visc;
  changed |= visc_now != b->cfg.viscous || any_turb != b->run_sa || any_inv != b->cfg.any_inviscid;
  b->cfg.viscous = visc_now;
  b->cfg.any_inviscid = any_inv;
  b->run_sa = any_turb;
  // the fused pass needs every resident block's halo within its tiles
  b->fused_fits = tile[2] <= cap[2] && tile[3] <= cap[3];
  const bool use_fused = b->fused_wanted && b->fused_fits;
  changed |= use_fused != b->fused;
  b->fused = use_fused;
  if (changed) drop_graphs(b);          // different kernels or tiles: re-capture
  const int n = (int)work.size();
  // the work list in kMaxChains parts at mesh boundaries: part k ends at
  // the boundary nearest (k+1)/chains of the list (the last parts are empty
  // when fewer chains run)
  int head[1 + kMaxChains];
  head[0] = n;
  int prev = 0;
  for (int k = 1; k <= kMaxChains; k++) {
    int end = n;
    if (k < b->chains) {
      const long target = (long)k * n / b->chains;
      end = prev;
      for (int x : mesh_first)
        if (x >= prev && std::labs(x - target) < std::labs(end - target)) end = x;
    }
    head[k] = end;
    prev = end;
  }
  // the part (chain) of every resident mesh, for the per-chain monitors
  std::vector<int> part(b->slots.size(), 0);
  {
    size_t m = 0;
    for (size_t i = 0; i < b->slots.size(); i++)
      if (b->slots[i].used && !b->slots[i].staged) {
        const int first = mesh_first[m++];
        int k = 1;
        while (k < kMaxChains && first >= head[k]) k++;
        part[i] = k;
      }
  }
  b->mesh_part_h = part;
  if (n) FVM_TRY(b, cudaMemcpyAsync(b->work, work.data(), n * sizeof(int), cudaMemcpyHostToDevice, b->stream));
  FVM_TRY(b, launch_gather_blocks(b->work, b->blocks, b->wblocks, n, b->stream));
  FVM_TRY(b, cudaMemcpyAsync(b->nwork, head, sizeof(head), cudaMemcpyHostToDevice, b->stream));
  FVM_TRY(b, cudaMemcpyAsync(b->mesh_part, b->mesh_part_h.data(), part.size() * sizeof(int),
                             cudaMemcpyHostToDevice, b->stream));
  FVM_TRY(b, cudaStreamSynchronize(b->stream));
  return FVM_OK;
}

// Deferred admissions join the work list once their uploads have finished.
int32_t batch_commit(fvm_batch *b) {
  if (!b->pending) return FVM_OK;
  FVM_TRY(b, cudaStreamSynchronize(b->upload));
  for (Slot &s : b->slots) s.staged = false;
  b->pending = false;
  return update_work(b);
}

// kernels of `iters` iterations, in order; optional timing events around
// each (one iteration only)
template <typename R>
int32_t enqueue_iteration(fvm_batch *b, bool with_events, int iters) {
  const ArenaPtrs<R> A = ptrs<R>(b);
  const LaunchCfg &c = b->cfg;
  const bool visc = c.viscous;   // a viscous mesh is resident
  int k = 0;
  // per-kernel timing events, recorded on the kernel's own stream
  auto mark = [&](int kind, cudaStream_t st) -> cudaError_t {
    if (!with_events) return cudaSuccess;
    if ((size_t)(2 * k + 1) >= b->ev.size()) return cudaErrorInvalidValue;
    b->ev_kind[k] = kind;
    return cudaEventRecordWithFlags(b->ev[2 * k], st, cudaEventRecordExternal);
  };
  auto done = [&](cudaStream_t st) -> cudaError_t {
    if (!with_events) {
      k++;
      return cudaSuccess;
    }
    cudaError_t e = cudaEventRecordWithFlags(b->ev[2 * k + 1], st, cudaEventRecordExternal);
    k++;
    return e;
  };
  // the three RK stages of the blocks of one part of the work list; with
  // fork set, an event after the first gradient pass lets the other part
  // start then, so the parts' passes overlap on the device
  auto stages = [&](const ArenaPtrs<R> &Ap, const LaunchCfg &cp, cudaEvent_t fork) -> int32_t {
    cudaStream_t st = cp.stream;
    for (int s = 1; s <= 3; s++) {
      // viscosity (and at stage 1 the viscous time step); with separate
      // passes, stages 2 and 3 take the viscosity the previous flux pass
      // computed from its output (the fused pass reads halo viscosities
      // while other CTAs update theirs, so it keeps the viscosity pass)
      if (visc && (s == 1 || b->fused)) {
        FVM_TRY(b, mark(K_VISC, st));
        FVM_TRY(b, launch_visc(Ap, cp, s, s == 1, 0));
        FVM_TRY(b, done(st));
      }
      if (b->fused) {
        // one pass: gradients (own + halo), fluxes, RK stage; inviscid
        // meshes take their time step in the stage-1 pass
        FVM_TRY(b, mark(K_STEP, st));
        FVM_TRY(b, launch_step(Ap, cp, s));
        FVM_TRY(b, done(st));
      } else {
        FVM_TRY(b, mark(K_GRAD, st));
        // inviscid meshes take their time step in the stage-1 gradient pass
        FVM_TRY(b, launch_grad(Ap, cp, s, s == 1 ? 1 : 0, 0));
        FVM_TRY(b, done(st));
        if (s == 1 && fork) FVM_TRY(b, cudaEventRecord(fork, st));
        FVM_TRY(b, mark(K_FLUX, st));
        FVM_TRY(b, launch_flux(Ap, cp, s, 1 /*MODE_UPDATE*/, s, 0));
        FVM_TRY(b, done(st));
      }
      if (s == 1 && fork && b->fused) FVM_TRY(b, cudaEventRecord(fork, st));
    }
    return FVM_OK;
  };
  // the end of an iteration for the meshes of one part: SA step, then the
  // monitor of those meshes (conres, clcd, stop test)
  auto finish_iteration = [&](const ArenaPtrs<R> &Ap, const LaunchCfg &cp) -> int32_t {
    cudaStream_t st = cp.stream;
    if (b->run_sa) {
      FVM_TRY(b, mark(K_SA, st));
      FVM_TRY(b, launch_sa(Ap, cp, 3, 0));
      FVM_TRY(b, done(st));
    }
    FVM_TRY(b, mark(K_MON, st));
    FVM_TRY(b, launch_monitor(Ap, cp, b->prec == FVM_PREC_FP64 ? 1 : 0));
    FVM_TRY(b, done(st));
    return FVM_OK;
  };
  if (b->chains > 1) {
    // independent chains over the parts of the work list, each running
    // `iters` whole iterations of its meshes; chain k starts after chain
    // k-1's first pass, then all join the first stream
    for (int k = 0; k < b->chains; k++) {
      ArenaPtrs<R> Ak = A;
      Ak.wpart = k + 1;
      LaunchCfg ck = c;
      ck.stream = k ? b->chain_stream[k] : b->stream;
      if (k) FVM_TRY(b, cudaStreamWaitEvent(ck.stream, b->ev_fork[k - 1], 0));
      for (int it = 0; it < iters; it++) {
        int32_t st = stages(Ak, ck, (it == 0 && k + 1 < b->chains) ? b->ev_fork[k] : nullptr);
        if (!st) st = finish_iteration(Ak, ck);
        if (st) return st;
      }
    }
    for (int k = 1; k < b->chains; k++) {
      FVM_TRY(b, cudaEventRecord(b->ev_join[k], b->chain_stream[k]));
      FVM_TRY(b, cudaStreamWaitEvent(b->stream, b->ev_join[k], 0));
    }
  } else {
    for (int it = 0; it < iters; it++) {
      int32_t st = stages(A, c, nullptr);
      if (!st) st = finish_iteration(A, c);
      if (st) return st;
    }
  }
  b->kernels_per_iter = k / iters;
  return FVM_OK;
}

// The graph of one iteration (iters = 1, per-kernel events when timing) or
// of kGraphIters iterations (fewer launches, and with several chains each
// chain runs on into its next iteration without waiting for the others).
int32_t build_graph(fvm_batch *b, int iters) {
  cudaGraphExec_t &out = iters > 1 ? b->graph_multi : b->graph;
  if (out) return FVM_OK;
  cudaGraph_t g = nullptr;
  FVM_TRY(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  const bool ev = b->timing && iters == 1;
  int32_t st = b->prec == FVM_PREC_FP64 ? enqueue_iteration<double>(b, ev, iters)
                                        : enqueue_iteration<float>(b, ev, iters);
  cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  if (st != FVM_OK) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  FVM_TRY(b, e);
  e = cudaGraphInstantiate(&out, g, 0);
  cudaGraphDestroy(g);
  FVM_TRY(b, e);
  return FVM_OK;
}

void drop_graphs(fvm_batch *b) {
  if ((b->graph || b->graph_multi) && b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  if (b->graph_multi) cudaGraphExecDestroy(b->graph_multi);
  b->graph = b->graph_multi = nullptr;
}

Slot *slot_of(fvm_batch *b, int32_t slot) {
  if (!b || slot < 0 || slot >= (int32_t)b->slots.size() || !b->slots[slot].used) return nullptr;
  return &b->slots[slot];
}

void default_caps(fvm_batch_caps &c) {
  const int64_t V = std::max<int64_t>(c.vertices, 1024);
  const int64_t M = std::max<int32_t>(c.meshes, 1);
  if (!c.blocks) c.blocks = V / 128 + 4 * M + 16;
  if (!c.edge_entries) c.edge_entries = 4 * V + 4096 * M;
  if (!c.boundary_entries) c.boundary_entries = V / 8 + 256 * M;
  if (!c.tri_entries) c.tri_entries = 3 * V + 4096 * M;
  if (!c.triangles) c.triangles = 2 * V + 64 * M;
  if (!c.edge_incidence) c.edge_incidence = 7 * V + 1024 * M;
  if (!c.tri_incidence) c.tri_incidence = 7 * V + 1024 * M;
  if (!c.all_incidence) c.all_incidence = 7 * V + 1024 * M;
  if (!c.solid_edges) c.solid_edges = V / 8 + 256 * M;
  if (!c.max_slots) c.max_slots = 1280;
  if (!c.max_tri) c.max_tri = 1024;
  if (!c.max_tri2) c.max_tri2 = 1280;
  if (!c.max_loc) c.max_loc = 576;
  if (!c.halo_entries) c.halo_entries = V / 2 + 1024 * M;
  if (!c.halo_incidence) c.halo_incidence = 4 * V + 4096 * M;
}

}  // namespace

// ---------------------------------------------------------------------------
// batch API
// ---------------------------------------------------------------------------
extern "C" int32_t fvm_batch_history_depth(void) { return kHistRows; }

extern "C" int32_t fvm_batch_create(int32_t precision, const fvm_batch_caps *caps_in,
                                    fvm_batch **out) {
  if (!caps_in || !out) return FVM_ERR_ARG;
  if (precision != FVM_PREC_FP64 && precision != FVM_PREC_FP32) return FVM_ERR_ARG;
  if (caps_in->vertices <= 0 || caps_in->meshes <= 0 || caps_in->meshes > kMaxMeshes)
    return FVM_ERR_ARG;
  *out = nullptr;
  fvm_batch *b = new (std::nothrow) fvm_batch();
  if (!b) return FVM_ERR_NOMEM;
  b->prec = precision;
  b->rsz = precision == FVM_PREC_FP64 ? 8 : 4;
  b->caps = *caps_in;
  default_caps(b->caps);
  const fvm_batch_caps &c = b->caps;
  if (c.max_slots > (int)kSlotMask || c.max_tri > 0x3fff || c.max_tri2 > 0x3fff ||
      c.max_loc > (int)kBlockVerts * 8 || c.vertices > INT_MAX / 8) {
    delete b;
    return FVM_ERR_ARG;
  }
  // vertex ranges are rounded up to kVertAlign per mesh
  const int64_t vcap = (c.vertices + kVertAlign - 1) / kVertAlign * kVertAlign +
                       (int64_t)kVertAlign * c.meshes;
  const int64_t caps[P_COUNT] = {vcap, c.blocks, c.edge_entries, c.boundary_entries,
                                 c.tri_entries, c.triangles, c.edge_incidence,
                                 c.tri_incidence, c.all_incidence, c.solid_edges,
                                 c.halo_entries, c.halo_entries + c.blocks,
                                 c.halo_incidence};
  for (int i = 0; i < P_COUNT; i++) {
    if (caps[i] > INT_MAX) {
      delete b;
      return FVM_ERR_ARG;
    }
    b->cap[i] = caps[i];
    b->pool[i].init(caps[i]);
  }
  b->slots.resize(c.meshes);
  auto fail = [&](int32_t st) {
    fvm_batch_destroy(b);
    return st;
  };
#define TRYB(expr)                                           \
  do {                                                       \
    cudaError_t _e = (expr);                                 \
    if (_e != cudaSuccess) return fail(cuda_status(b, _e));  \
  } while (0)
  TRYB(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  TRYB(cudaStreamCreateWithFlags(&b->upload, cudaStreamNonBlocking));
  for (int k = 0; k < kMaxChains; k++) {
    if (k) TRYB(cudaStreamCreateWithFlags(&b->chain_stream[k], cudaStreamNonBlocking));
    TRYB(cudaEventCreateWithFlags(&b->ev_fork[k], cudaEventDisableTiming));
    TRYB(cudaEventCreateWithFlags(&b->ev_join[k], cudaEventDisableTiming));
  }
  auto &O = b->owned;
  const size_t V = (size_t)b->cap[P_V] + kVertAlign, r = b->rsz;   // with slack
  for (int i = 0; i < 3; i++) TRYB(dalloc(O, (unsigned char **)&b->st[i], 4 * r * V));
  TRYB(dalloc(O, (unsigned char **)&b->grad, 8 * r * V));
  TRYB(dalloc(O, (unsigned char **)&b->resv, 4 * r * V));
  TRYB(dalloc(O, (unsigned char **)&b->res, 4 * r * V));
  TRYB(dalloc(O, (unsigned char **)&b->dt, r * V));
  TRYB(dalloc(O, (unsigned char **)&b->mu, r * V));
  TRYB(dalloc(O, (unsigned char **)&b->mul, r * V));
  TRYB(dalloc(O, (unsigned char **)&b->nut[0], r * V));
  TRYB(dalloc(O, (unsigned char **)&b->nut[1], r * V));
  TRYB(dalloc(O, &b->coord, V));
  TRYB(dalloc(O, &b->ais, V));
  TRYB(dalloc(O, &b->cvarea, V));
  TRYB(dalloc(O, &b->drmin, V));
  TRYB(dalloc(O, &b->wd, V));
  TRYB(dalloc(O, &b->orig, V));
  TRYB(dalloc(O, &b->vflag, V));
  TRYB(dalloc(O, &b->ve_rng, V));
  TRYB(dalloc(O, &b->vt_rng, V));
  TRYB(dalloc(O, &b->va_rng, V));
  TRYB(dalloc(O, &b->ve_list, (size_t)c.edge_incidence));
  TRYB(dalloc(O, &b->vt_list, (size_t)c.tri_incidence + 16));   // slack: 16-byte copies
  TRYB(dalloc(O, &b->va_list, (size_t)c.all_incidence));
  TRYB(dalloc(O, &b->va_dsl, (size_t)c.all_incidence));
  TRYB(dalloc(O, &b->blocks, (size_t)c.blocks));
  TRYB(dalloc(O, &b->wblocks, (size_t)c.blocks));
  TRYB(dalloc(O, &b->part, (size_t)c.blocks));
  TRYB(dalloc(O, &b->work, (size_t)c.blocks));
  TRYB(dalloc(O, &b->nwork, 1 + kMaxChains));
  TRYB(dalloc(O, &b->mesh_part, (size_t)c.meshes));
  TRYB(dalloc(O, &b->be_nodes, (size_t)c.edge_entries));
  TRYB(dalloc(O, &b->be_loc, (size_t)c.edge_entries));
  TRYB(dalloc(O, &b->halo_ids, (size_t)b->cap[P_HALO] + 4));   // slack: 16-byte copies
  TRYB(dalloc(O, &b->hl_ptr, (size_t)b->cap[P_HP]));
  TRYB(dalloc(O, &b->hl_list, (size_t)b->cap[P_HL]));
  TRYB(dalloc(O, &b->be_ds, (size_t)c.edge_entries));
  if (precision == FVM_PREC_FP64) TRYB(dalloc(O, &b->be_csl, (size_t)c.edge_entries));
  TRYB(dalloc(O, &b->bb_nodes, (size_t)c.boundary_entries));
  TRYB(dalloc(O, &b->bt_nodes, (size_t)c.tri_entries));
  TRYB(dalloc(O, &b->elarea, (size_t)c.triangles));
  if (precision == FVM_PREC_FP32) {
    TRYB(dalloc(O, &b->be_g32, (size_t)c.edge_entries));
    TRYB(dalloc(O, &b->va_w, (size_t)c.all_incidence));
    TRYB(dalloc(O, &b->ais32, V));
    TRYB(dalloc(O, &b->cvarea32, V));
    TRYB(dalloc(O, &b->drmin32, V));
    TRYB(dalloc(O, &b->wd32, V));
    TRYB(dalloc(O, &b->tri_g32, (size_t)c.tri_entries));
  }
  TRYB(dalloc(O, &b->sw_nodes, (size_t)c.solid_edges));
  TRYB(dalloc(O, &b->mc, (size_t)c.meshes));
  TRYB(dalloc(O, &b->ctl, (size_t)c.meshes));
  const size_t H = (size_t)c.meshes * kHistRows;
  TRYB(dalloc(O, &b->h_fres, H));
  TRYB(dalloc(O, &b->h_fresi, H));
  TRYB(dalloc(O, &b->h_cl, H));
  TRYB(dalloc(O, &b->h_cd, H));
  TRYB(dalloc(O, &b->h_iresi, H));
  TRYB(cudaMemsetAsync(b->ctl, 0, sizeof(MeshCtl) * c.meshes, b->stream));
  TRYB(cudaMemsetAsync(b->nwork, 0, (1 + kMaxChains) * sizeof(int), b->stream));
  TRYB(cudaMemsetAsync(b->grad, 0, 8 * r * V, b->stream));
  TRYB(cudaMemsetAsync(b->resv, 0, 4 * r * V, b->stream));
  TRYB(cudaStreamSynchronize(b->stream));
#undef TRYB
  b->cfg.max_slots = c.max_slots;
  b->cfg.max_tri = c.max_tri;
  b->cfg.max_tri2 = c.max_tri2;
  b->cfg.max_loc = c.max_loc;
  b->cfg.max_halo = 0;
  b->cfg.tri_loc = true;
  // the fused pass computes triangle-form gradients: FP64 only (FP32
  // inviscid meshes take the vertex-stencil gradient)
  if (c.fused > 0 && precision != FVM_PREC_FP64) return fail(FVM_ERR_ARG);
  b->fused = b->fused_wanted = c.fused > 0;
  b->cfg.stencil = precision == FVM_PREC_FP32;
  b->cfg.any_inviscid = false;
  b->chains = std::min(std::max(c.overlap, 1), kMaxChains);
  // gradient pass (the triangle form, of viscous meshes in FP32): the
  // bulk-copy form by default in FP32 (the pipelined form measured 1-4%
  // slower on laminar and RANS batches and is a tuner candidate),
  // per-thread loads in FP64
  const bool bulk_fits = grad_bulk_layout(c.max_tri, kTriLocMax, c.viscous != 0).total <= kMaxSmem;
  if (c.pipe_groups < 0 || c.pipe_groups > 2 || c.pipe_stages < 0 || c.pipe_stages > kPipeMaxStages)
    return fail(FVM_ERR_ARG);
  b->cfg.pipe_groups = c.pipe_groups == 1 ? 1 : 2;
  b->cfg.pipe_stages = c.pipe_stages;
  b->cfg.grad_mode = c.grad_mode > 0 ? c.grad_mode
                                      : (precision == FVM_PREC_FP32 && bulk_fits ? 3 : 1);
  if (b->cfg.grad_mode < 1 || b->cfg.grad_mode > 4 ||
      (b->cfg.grad_mode >= 3 && (precision != FVM_PREC_FP32 || !bulk_fits)))
    return fail(FVM_ERR_ARG);
  b->cfg.viscous = c.viscous != 0;
  b->cfg.std_const = false;   // set when meshes are admitted
  b->cfg.stream = b->stream;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms <= 0) sms = 152;
  b->cfg.sms = sms;
  b->cfg.fit = c.grid <= 0;            // an explicit grid is taken as given
  b->cfg.grid = c.grid > 0 ? c.grid : std::max<int>(1, std::min<int64_t>(c.blocks, 8LL * sms));
  cudaError_t e = precision == FVM_PREC_FP64 ? prepare_attributes(b->cfg, (double *)nullptr)
                                             : prepare_attributes(b->cfg, (float *)nullptr);
  if (e != cudaSuccess) return fail(cuda_status(b, e));
  *out = b;
  return FVM_OK;
}

extern "C" int32_t fvm_batch_destroy(fvm_batch *b) {
  if (!b) return FVM_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graphs(b);
  for (cudaEvent_t e : b->ev) cudaEventDestroy(e);
  for (void *p : b->owned) cudaFree(p);
  if (b->upload) cudaStreamSynchronize(b->upload);
  if (b->dstage) cudaFree(b->dstage);
  if (b->upload) cudaStreamDestroy(b->upload);
  if (b->stream) cudaStreamDestroy(b->stream);
  for (int k = 0; k < kMaxChains; k++) {
    if (b->chain_stream[k]) cudaStreamDestroy(b->chain_stream[k]);
    if (b->ev_fork[k]) cudaEventDestroy(b->ev_fork[k]);
    if (b->ev_join[k]) cudaEventDestroy(b->ev_join[k]);
  }
  delete b;
  return FVM_OK;
}

// A mesh ready to upload: block layout plus every host array the device
// needs, in renumbered order with mesh-relative indices.
struct fvm_prepared {
  fvm_params par{};
  MeshLayout L;
  std::vector<double2> coord;
  std::vector<double> ais, cvarea, drmin, wd, elarea;
  std::vector<int> orig;
  std::vector<double2> be_ds;
  std::vector<EdgeGeo32> be_g32;   // FP32 batches
  std::vector<float2> va_w;        // FP32 batches: Green-Gauss weights per va_list entry
  std::vector<double> va_dsl;      // |ds| of each va_list entry's edge (shockind.f:36)
  std::vector<TriGeo32> tri_g32;   // FP32 batches
};

extern "C" int32_t fvm_batch_prepare(const fvm_params *par, const fvm_mesh *m, fvm_prepared **out) {
  if (!par || !m || !out) return FVM_ERR_ARG;
  *out = nullptr;
  if (m->np < 3 || m->nt < 1 || m->netot < 1 || m->ne < 1 || !m->coord || !m->elem ||
      !m->ptype || !m->edge || !m->iedge || !m->ds || !m->elarea || !m->cvarea ||
      !m->mcarea || !m->drmin)
    return FVM_ERR_ARG;
  if (par->iflow == FVM_TURBULENT && !m->wd) return FVM_ERR_ARG;
  if (m->nbe > 0 && !m->beindx) return FVM_ERR_ARG;
  fvm_prepared *P = new (std::nothrow) fvm_prepared();
  if (!P) return FVM_ERR_NOMEM;
  P->par = *par;
  int32_t st = build_layout(*m, kBlockVerts, P->L);
  if (st != FVM_OK) {
    delete P;
    return st;
  }
  const MeshLayout &L = P->L;
  const int np = L.np;
  P->coord.resize(np);
  P->ais.resize(np);
  P->cvarea.resize(np);
  P->drmin.resize(np);
  P->wd.assign(np, 1.0);
  P->orig.resize(np);
  const double n1b6 = 1.0 / 6.0;
  for (int v = 0; v < np; v++) {
    const int o = L.perm[v];
    P->coord[v] = make_double2(m->coord[2 * o], m->coord[2 * o + 1]);
    P->ais[v] = n1b6 / m->mcarea[o];   // green_gauss.f:34
    P->cvarea[v] = m->cvarea[o];
    P->drmin[v] = m->drmin[o];
    if (m->wd) P->wd[v] = m->wd[o];
    P->orig[v] = o + 1;
  }
  P->elarea.assign(m->elarea, m->elarea + L.nt);
  P->be_ds.resize(L.be_edge.size());
  P->be_g32.resize(L.be_edge.size());
  for (size_t k = 0; k < L.be_edge.size(); k++) {
    const int e = L.be_edge[k];
    const double dsx = m->ds[2 * e], dsy = m->ds[2 * e + 1];
    P->be_ds[k] = make_double2(dsx, dsy);
    // FP32 copies of FP64 quantities, rounded once
    const int n1 = m->edge[2 * e] - 1, n2 = m->edge[2 * e + 1] - 1;
    EdgeGeo32 g;
    g.v = make_float4((float)(m->coord[2 * n2] - m->coord[2 * n1]),
                      (float)(m->coord[2 * n2 + 1] - m->coord[2 * n1 + 1]), (float)dsx,
                      (float)dsy);
    P->be_g32[k] = g;
  }
  // Green-Gauss as a vertex stencil (FP32 batches).  green_gauss.f:23-39
  // sums, for each triangle t around v, (1/6 mcarea_v) * sum_j prim_j *
  // (dbxx_j, dbyy_j)(t) over t's three vertices j.  The three coefficients
  // of a triangle sum to zero, so the same sum is
  //   sum over v's neighbours u of W(v,u) * (prim_u - prim_v),
  //   W(v,u) = (1/6 mcarea_v) * sum over the triangles t holding v and u of
  //            (dbxx, dbyy) at u's position in t,
  // which a uniform state maps to zero exactly.  W is formed in FP64 and
  // rounded once, one entry per va_list entry of v (its edges, in edge
  // order).
  if (par->precision == FVM_PREC_FP32) {
    P->va_w.assign(L.va_list.size(), make_float2(0.f, 0.f));
    std::vector<double> wx(L.va_list.size(), 0.0), wy(L.va_list.size(), 0.0);
    auto slot = [&](int v, int u) -> int {
      for (int j = L.va_ptr[v]; j < L.va_ptr[v + 1]; j++)
        if ((L.va_list[j] & 0x7fffffff) == u) return j;
      return -1;
    };
    bool ok = true;
    for (int t = 0; t < L.nt && ok; t++) {
      int a[3];
      double x[3], y[3];
      for (int i = 0; i < 3; i++) {
        const int o = m->elem[3 * t + i] - 1;
        a[i] = L.iperm[o];
        x[i] = m->coord[2 * o];
        y[i] = m->coord[2 * o + 1];
      }
      const double bx[3] = {y[1] - y[2], y[2] - y[0], y[0] - y[1]};
      const double by[3] = {x[2] - x[1], x[0] - x[2], x[1] - x[0]};
      for (int i = 0; i < 3 && ok; i++)
        for (int jj = 0; jj < 3; jj++) {
          if (jj == i) continue;
          const int k = slot(a[i], a[jj]);
          if (k < 0) {
            ok = false;
            break;
          }
          wx[k] += bx[jj];
          wy[k] += by[jj];
        }
    }
    if (!ok) {
      delete P;
      return FVM_ERR_GEOMETRY;   // a triangle side that is not an edge
    }
    for (int v = 0; v < np; v++)
      for (int j = L.va_ptr[v]; j < L.va_ptr[v + 1]; j++)
        P->va_w[j] = make_float2((float)(P->ais[v] * wx[j]), (float)(P->ais[v] * wy[j]));
  }
  // |ds| per all-edge incidence entry, in the order build_layout lists them
  // (edge order, both ends of each edge); dsqrt(ds(1)**2 + ds(2)**2)
  P->va_dsl.resize(L.va_list.size());
  {
    std::vector<int> cur(L.va_ptr.begin(), L.va_ptr.end() - 1);
    for (int e = 0; e < m->netot; e++) {
      const int a = L.iperm[m->edge[2 * e] - 1], c = L.iperm[m->edge[2 * e + 1] - 1];
      const double dsx = m->ds[2 * e], dsy = m->ds[2 * e + 1];
      const double dl = std::sqrt(dsx * dsx + dsy * dsy);
      P->va_dsl[cur[a]++] = dl;
      P->va_dsl[cur[c]++] = dl;
    }
  }
  P->tri_g32.resize(L.bt_nodes.size());
  for (size_t k = 0; k < L.bt_nodes.size(); k++) {
    const int t = L.bt_nodes[k].w;   // driver triangle of this block entry
    const int a = m->elem[3 * t] - 1, c2 = m->elem[3 * t + 1] - 1, c3 = m->elem[3 * t + 2] - 1;
    const double x1 = m->coord[2 * a], y1 = m->coord[2 * a + 1];
    const double x2 = m->coord[2 * c2], y2 = m->coord[2 * c2 + 1];
    const double x3 = m->coord[2 * c3], y3 = m->coord[2 * c3 + 1];
    TriGeo32 g;
    g.dbxx[0] = (float)(y2 - y3);
    g.dbxx[1] = (float)(y3 - y1);
    g.dbxx[2] = (float)(y1 - y2);
    g.dbyy[0] = (float)(x3 - x2);
    g.dbyy[1] = (float)(x1 - x3);
    g.dbyy[2] = (float)(x2 - x1);
    g.areat = (float)(0.25 / m->elarea[t]);
    g.loc = L.bt_loc[k];
    P->tri_g32[k] = g;
  }
  *out = P;
  return FVM_OK;
}

extern "C" int32_t fvm_prepared_free(fvm_prepared *prep) {
  delete prep;
  return FVM_OK;
}

extern "C" int64_t fvm_prepared_bytes(const fvm_prepared *prep, int32_t precision) {
  if (!prep) return -1;
  const MeshLayout &L = prep->L;
  const int64_t r = precision == FVM_PREC_FP64 ? 8 : 4;
  const int64_t V = L.np;
  int64_t bytes = V * (3 * 4 * r + 8 * r + 4 * r + 4 * r + 5 * r + 16 + 4 * 8 + 4 + 1 + 3 * 8);
  bytes += (int64_t)L.be_nodes.size() * (8 + 16 + (r == 4 ? 16 : 32));
  bytes += (int64_t)L.bb_nodes.size() * 16 + (int64_t)L.bt_nodes.size() * (16 + (r == 4 ? 32 : 0));
  bytes += (int64_t)L.nt * 8 + (int64_t)L.ve_list.size() * 2 + (int64_t)L.vt_list.size() * 2;
  bytes += (int64_t)L.va_list.size() * (12 + (r == 4 ? 8 : 0)) + (int64_t)L.sw_nodes.size() * 8;
  bytes += (int64_t)L.nblk * (sizeof(BlockInfo) + sizeof(BlockPartial) + 4);
  bytes += (int64_t)L.be_loc.size() * 4 + (int64_t)L.halo_ids.size() * 4;
  bytes += (int64_t)L.hl_ptr.size() * 4 + (int64_t)L.hl_list.size() * 2;
  return bytes;
}

// Admits a prepared mesh.  Deferred: every upload goes to the side stream
// (it may run beside kernels on the batch's stream: the mesh's ranges are
// free) and the mesh joins the work list at batch_commit.
static int32_t add_prepared(fvm_batch *b, fvm_prepared *prep, int32_t *slot_out, bool deferred) {
  if (!b || !prep || !slot_out) return FVM_ERR_ARG;
  *slot_out = -1;
  const fvm_params *par = &prep->par;
  if (par->precision != b->prec) return FVM_ERR_ARG;
  if (par->iflow != FVM_INVISCID && !b->caps.viscous) return FVM_ERR_ARG;
  int sid = -1;
  for (size_t i = 0; i < b->slots.size(); i++)
    if (!b->slots[i].used) {
      sid = (int)i;
      break;
    }
  if (sid < 0) return FVM_ERR_CAPACITY;
  const MeshLayout &Lp = prep->L;
  // (a mesh whose halo tiles exceed max_tri2 / max_loc is admitted; the
  // fused pass is then off while it is resident)
  if (Lp.max_slots > b->caps.max_slots || Lp.max_tri > b->caps.max_tri) return FVM_ERR_CAPACITY;
  const int64_t need[P_COUNT] = {(Lp.np + kVertAlign - 1) / kVertAlign * kVertAlign, Lp.nblk, (int64_t)Lp.be_nodes.size(), (int64_t)Lp.bb_nodes.size(),
                                 (int64_t)Lp.bt_nodes.size(), Lp.nt, (int64_t)Lp.ve_list.size(),
                                 (int64_t)Lp.vt_list.size(), (int64_t)Lp.va_list.size(),
                                 (int64_t)Lp.sw_nodes.size(), (int64_t)Lp.halo_ids.size(),
                                 (int64_t)Lp.hl_ptr.size(), (int64_t)Lp.hl_list.size()};
  int64_t off[P_COUNT];
  for (int i = 0; i < P_COUNT; i++) {
    off[i] = b->pool[i].alloc(need[i]);
    if (off[i] < 0) {
      for (int j = 0; j < i; j++) b->pool[j].release(off[j], need[j]);
      return FVM_ERR_CAPACITY;
    }
  }
  Slot &S = b->slots[sid];
  S = Slot();
  S.par = *par;
  S.L = prep->L;
  for (int i = 0; i < P_COUNT; i++) {
    S.off[i] = off[i];
    S.len[i] = need[i];
  }
  const MeshLayout &L = S.L;
  const int np = L.np;
  const int v0 = (int)S.off[P_V];
  std::vector<int2> ve(np), vt(np), va(np);
  for (int v = 0; v < np; v++) {
    ve[v] = make_int2((int)(S.off[P_VE] + L.ve_ptr[v]), (int)(S.off[P_VE] + L.ve_ptr[v + 1]));
    vt[v] = make_int2((int)(S.off[P_VT] + L.vt_ptr[v]), (int)(S.off[P_VT] + L.vt_ptr[v + 1]));
    va[v] = make_int2((int)(S.off[P_VA] + L.va_ptr[v]), (int)(S.off[P_VA] + L.va_ptr[v + 1]));
  }
  std::vector<BlockInfo> blocks = L.blocks;
  for (int k = 0; k < L.nblk; k++) {
    BlockInfo &bi = blocks[k];
    bi.mesh = sid;
    bi.v0 += v0;
    bi.e0 += (int)S.off[P_BE];
    bi.b0 += (int)S.off[P_BB];
    bi.t0 += (int)S.off[P_BT];
    bi.vt0 += (int)S.off[P_VT];
    bi.h0 += (int)S.off[P_HALO];
    bi.hp0 += (int)S.off[P_HP];
    bi.part = (int)S.off[P_BLK] + k;
  }
  std::vector<int> halo(L.halo_ids);
  for (int &x : halo) x += v0;
  std::vector<int> hlp(L.hl_ptr);
  for (int &x : hlp) x += (int)S.off[P_HL];
  std::vector<int2> be(L.be_nodes);
  for (int2 &q : be) {
    q.x += v0;
    q.y += v0;
  }
  std::vector<int4> bb(L.bb_nodes);
  for (int4 &q : bb) {
    q.x += v0;
    q.y += v0;
  }
  std::vector<int4> bt(L.bt_nodes);
  for (int4 &q : bt) {
    q.x += v0;
    q.y += v0;
    q.z += v0;
    q.w += (int)S.off[P_TRI];
  }
  std::vector<int> valist(L.va_list);
  for (int &x : valist) {
    const unsigned u = (unsigned)x;
    x = (int)((u & 0x80000000u) | ((u & 0x7fffffffu) + (unsigned)v0));
  }
  std::vector<int2> sw(L.sw_nodes);
  for (int2 &q : sw) {
    q.x += v0;
    q.y += v0;
  }
  MeshConst mc = make_const(*par);
  mc.v0 = v0;
  mc.nv = np;
  mc.blk0 = (int)S.off[P_BLK];
  mc.nblk = L.nblk;
  mc.sw0 = (int)S.off[P_SW];
  mc.nsw = (int)L.sw_nodes.size();
  for (int k = 0; k < 3; k++) mc.orig123[k] = v0 + L.iperm[k];
  MeshCtl ctl;
  std::memset(&ctl, 0, sizeof(ctl));
  ctl.err_point = INT_MAX;
  ctl.hist_off = sid * kHistRows;
  ctl.hist_cap = kHistRows;
  auto err = [&](cudaError_t e) -> int32_t {
    fvm_batch_remove(b, sid);
    return cuda_status(b, e);
  };
  S.used = true;
  S.staged = deferred;
  const cudaStream_t us = deferred ? b->upload : b->stream;
  cudaError_t e = cudaSuccess;
#define PUT(expr)                  \
  if ((e = (expr)) != cudaSuccess) \
    return err(e);
  PUT(put_range(b, b->coord, v0, prep->coord, us));
  PUT(put_range(b, b->ais, v0, prep->ais, us));
  PUT(put_range(b, b->cvarea, v0, prep->cvarea, us));
  PUT(put_range(b, b->drmin, v0, prep->drmin, us));
  if (b->ais32) {
    std::vector<float> f(prep->ais.size());
    for (size_t i = 0; i < f.size(); i++) f[i] = (float)prep->ais[i];
    PUT(put_range(b, b->ais32, v0, f, us));
    for (size_t i = 0; i < f.size(); i++) f[i] = (float)prep->cvarea[i];
    PUT(put_range(b, b->cvarea32, v0, f, us));
    for (size_t i = 0; i < f.size(); i++) f[i] = (float)prep->drmin[i];
    PUT(put_range(b, b->drmin32, v0, f, us));
    for (size_t i = 0; i < f.size(); i++) f[i] = (float)prep->wd[i];
    PUT(put_range(b, b->wd32, v0, f, us));
  }
  PUT(put_range(b, b->wd, v0, prep->wd, us));
  PUT(put_range(b, b->orig, v0, prep->orig, us));
  PUT(put_range(b, b->vflag, v0, L.vflag, us));
  PUT(put_range(b, b->ve_rng, v0, ve, us));
  PUT(put_range(b, b->vt_rng, v0, vt, us));
  PUT(put_range(b, b->va_rng, v0, va, us));
  PUT(put_range(b, b->ve_list, S.off[P_VE], L.ve_list, us));
  PUT(put_range(b, b->vt_list, S.off[P_VT], L.vt_list, us));
  PUT(put_range(b, b->va_list, S.off[P_VA], valist, us));
  PUT(put_range(b, b->blocks, S.off[P_BLK], blocks, us));
  PUT(put_range(b, b->be_nodes, S.off[P_BE], be, us));
  PUT(put_range(b, b->be_loc, S.off[P_BE], L.be_loc, us));
  PUT(put_range(b, b->halo_ids, S.off[P_HALO], halo, us));
  PUT(put_range(b, b->hl_ptr, S.off[P_HP], hlp, us));
  PUT(put_range(b, b->hl_list, S.off[P_HL], L.hl_list, us));
  PUT(put_range(b, b->be_ds, S.off[P_BE], prep->be_ds, us));
  if (b->be_csl)
    PUT(launch_edge_csl(b->be_ds + S.off[P_BE], b->be_csl + S.off[P_BE], (int)be.size(), us));
  PUT(put_range(b, b->bb_nodes, S.off[P_BB], bb, us));
  PUT(put_range(b, b->bt_nodes, S.off[P_BT], bt, us));
  PUT(put_range(b, b->elarea, S.off[P_TRI], prep->elarea, us));
  if (b->be_g32) PUT(put_range(b, b->be_g32, S.off[P_BE], prep->be_g32, us));
  if (b->tri_g32) PUT(put_range(b, b->tri_g32, S.off[P_BT], prep->tri_g32, us));
  if (b->va_w) PUT(put_range(b, b->va_w, S.off[P_VA], prep->va_w, us));
  PUT(put_range(b, b->va_dsl, S.off[P_VA], prep->va_dsl, us));
  PUT(put_range(b, b->sw_nodes, S.off[P_SW], sw, us));
  PUT(cudaMemcpyAsync(b->mc + sid, &mc, sizeof(mc), cudaMemcpyHostToDevice, us));
  PUT(cudaMemcpyAsync(b->ctl + sid, &ctl, sizeof(ctl), cudaMemcpyHostToDevice, us));
  const size_t r = b->rsz;
  PUT(cudaMemsetAsync(static_cast<unsigned char *>(b->grad) + (size_t)v0 * 8 * r, 0, 8 * r * np, us));
  PUT(cudaMemsetAsync(static_cast<unsigned char *>(b->resv) + (size_t)v0 * 4 * r, 0, 4 * r * np, us));
#undef PUT
  // freestream state (initialize.f:60-89): the same values at every
  // vertex, written on the device into the phase-0 buffers of the control
  // record uploaded above (iteration 0, nothing active)
  int32_t st;
  {
    double nut0 = 0.0, mul0 = 0.0, mu0 = 0.0;
    if (par->iflow != FVM_INVISCID) {
      const double temp = par->p_inf / par->r_inf / par->gas_const;
      mul0 = std::pow(temp / par->t_inf, 1.5) *
             ((par->t_inf + par->sconst) / (temp + par->sconst)) / par->rey;
      mu0 = mul0;
      if (par->iflow == FVM_TURBULENT) {
        nut0 = par->nut_inf;
        const double chi = nut0 * par->r_inf / mul0;
        const double chi3 = (chi * chi) * chi;
        mu0 = mul0 + par->r_inf * nut0 * (chi3 / (chi3 + par->cv11));
      }
    }
    const double prim0[4] = {par->r_inf, par->u_inf, par->v_inf, par->p_inf};
    auto at = [&](void *base, size_t stride) {
      return static_cast<unsigned char *>(base) + (size_t)v0 * stride;
    };
    cudaError_t fe = launch_fill_vertex((int)r, at(b->st[0], 4 * r), 4 * r, np, 4, prim0, us);
    if (fe == cudaSuccess) fe = launch_fill_vertex((int)r, at(b->nut[0], r), r, np, 1, &nut0, us);
    if (fe == cudaSuccess) fe = launch_fill_vertex((int)r, at(b->mul, r), r, np, 1, &mul0, us);
    if (fe == cudaSuccess) fe = launch_fill_vertex((int)r, at(b->mu, r), r, np, 1, &mu0, us);
    if (fe == cudaSuccess && !deferred) fe = cudaStreamSynchronize(us);
    if (fe != cudaSuccess) return err(fe);
  }
  if (deferred) {
    b->pending = true;
  } else if ((st = update_work(b))) {
    fvm_batch_remove(b, sid);
    return st;
  }
  delete prep;   // consumed on success only
  *slot_out = sid;
  return FVM_OK;
}

extern "C" int32_t fvm_batch_add_prepared(fvm_batch *b, fvm_prepared *prep, int32_t *slot_out) {
  if (!b) return FVM_ERR_ARG;
  int32_t st = batch_commit(b);
  if (st) return st;
  return add_prepared(b, prep, slot_out, false);
}

namespace fvm {
int32_t batch_add_prepared_deferred(fvm_batch *b, fvm_prepared *prep, int32_t *slot_out) {
  if (!b) return FVM_ERR_ARG;
  return add_prepared(b, prep, slot_out, true);
}
int32_t batch_commit_admissions(fvm_batch *b) {
  if (!b) return FVM_ERR_ARG;
  return batch_commit(b);
}
}  // namespace fvm

extern "C" int32_t fvm_batch_add(fvm_batch *b, const fvm_params *par, const fvm_mesh *m,
                                 int32_t *slot_out) {
  if (!b || !par || !m || !slot_out) return FVM_ERR_ARG;
  *slot_out = -1;
  if (par->precision != b->prec) return FVM_ERR_ARG;
  if (par->iflow != FVM_INVISCID && !b->caps.viscous) return FVM_ERR_ARG;
  fvm_prepared *prep = nullptr;
  int32_t st = fvm_batch_prepare(par, m, &prep);
  if (st) return st;
  st = fvm_batch_add_prepared(b, prep, slot_out);
  if (st) delete prep;
  return st;
}

extern "C" int32_t fvm_batch_remove(fvm_batch *b, int32_t slot) {
  if (b && b->pending) {   // deferred admissions first
    const int32_t cst = batch_commit(b);
    if (cst) return cst;
  }
  Slot *S = slot_of(b, slot);
  if (!S) return FVM_ERR_ARG;
  MeshCtl z;
  std::memset(&z, 0, sizeof(z));
  int32_t st = put_ctl(b, slot, z);
  for (int i = 0; i < P_COUNT; i++) b->pool[i].release(S->off[i], S->len[i]);
  *S = Slot();
  int32_t st2 = update_work(b);
  return st ? st : st2;
}

extern "C" int32_t fvm_batch_set_state(fvm_batch *b, int32_t slot, const double *prim,
                                       const double *nut, const double *mul, const double *mu,
                                       int32_t iterlast) {
  if (b && b->pending) {   // deferred admissions first
    const int32_t cst = batch_commit(b);
    if (cst) return cst;
  }
  Slot *S = slot_of(b, slot);
  if (!S || !prim || iterlast < 0) return FVM_ERR_ARG;
  const size_t r = b->rsz;
  int32_t st;
  if ((st = put_vertex_rot(b, slot, *S, Rot::Phase, nullptr, prim, 4, 4 * r))) return st;
  if (nut && (st = put_vertex_rot(b, slot, *S, Rot::NutPhase, nullptr, nut, 1, r))) return st;
  if (mul && (st = put_vertex_rot(b, slot, *S, Rot::None, b->mul, mul, 1, r))) return st;
  if (mu && (st = put_vertex_rot(b, slot, *S, Rot::None, b->mu, mu, 1, r))) return st;
  FVM_TRY(b, launch_ctl_update(b->ctl + slot, 0, iterlast, 0.0, b->stream));
  // the caller's arrays have been read when the call returns
  return sync_stream(b);
}

extern "C" int32_t fvm_batch_get_state(fvm_batch *b, int32_t slot, double *prim, double *nut,
                                       double *mul, double *mu, double *qx, double *qy) {
  if (b && b->pending) {   // deferred admissions first
    const int32_t cst = batch_commit(b);
    if (cst) return cst;
  }
  Slot *S = slot_of(b, slot);
  if (!S) return FVM_ERR_ARG;
  const size_t r = b->rsz;
  int32_t st;
  if (prim && (st = get_vertex_rot(b, slot, *S, Rot::Phase, nullptr, prim, 4, 4 * r))) return st;
  if (nut && (st = get_vertex_rot(b, slot, *S, Rot::NutPhase, nullptr, nut, 1, r))) return st;
  if (mul && (st = get_vertex_rot(b, slot, *S, Rot::None, b->mul, mul, 1, r))) return st;
  if (mu && (st = get_vertex_rot(b, slot, *S, Rot::None, b->mu, mu, 1, r))) return st;
  if (qx && (st = get_vertex_rot(b, slot, *S, Rot::None, b->grad, qx, 4, 8 * r, 0))) return st;
  if (qy && (st = get_vertex_rot(b, slot, *S, Rot::None, b->grad, qy, 4, 8 * r, 4))) return st;
  return sync_stream(b);
}

extern "C" int32_t fvm_batch_start(fvm_batch *b, int32_t slot, int32_t nmax, double minres) {
  if (b && b->pending) {   // deferred admissions first
    const int32_t cst = batch_commit(b);
    if (cst) return cst;
  }
  Slot *S = slot_of(b, slot);
  if (!S || nmax < 0) return FVM_ERR_ARG;
  // on the device, in stream order before the next step (no host wait)
  FVM_TRY(b, launch_ctl_update(b->ctl + slot, 1, nmax, minres, b->stream));
  return FVM_OK;
}

extern "C" int32_t fvm_batch_step(fvm_batch *b, int32_t niter) {
  if (b && b->pending) {   // deferred admissions first
    const int32_t cst = batch_commit(b);
    if (cst) return cst;
  }
  if (!b || niter < 0) return FVM_ERR_ARG;
  int32_t st;
  if (!b->timing && niter >= kGraphIters) {
    if ((st = build_graph(b, kGraphIters))) return st;
    for (; niter >= kGraphIters; niter -= kGraphIters) {
      FVM_TRY(b, cudaGraphLaunch(b->graph_multi, b->stream));
      b->launches += (int64_t)b->kernels_per_iter * kGraphIters;
    }
  }
  if (niter == 0) return FVM_OK;
  if ((st = build_graph(b, 1))) return st;
  for (int i = 0; i < niter; i++) {
    FVM_TRY(b, cudaGraphLaunch(b->graph, b->stream));
    b->launches += b->kernels_per_iter;
    if (b->timing) {
      FVM_TRY(b, cudaStreamSynchronize(b->stream));
      for (int k = 0; k < b->kernels_per_iter; k++) {
        float ms = 0.f;
        FVM_TRY(b, cudaEventElapsedTime(&ms, b->ev[2 * k], b->ev[2 * k + 1]));
        b->t_ms[b->ev_kind[k]] += ms;
        b->t_launch[b->ev_kind[k]] += 1;
      }
    }
  }
  return FVM_OK;
}

// Forms of the iteration the tuner chooses from (fvm_batch_tune codes).
struct Form {
  bool fused;
  int grad;
  int chains;
};
constexpr int kForms = 11;

static Form form_of(const fvm_batch *b, int i) {
  const bool bulk = b->prec == FVM_PREC_FP32 &&
                    grad_bulk_layout(b->caps.max_tri, kTriLocMax, b->caps.viscous != 0).total <= kMaxSmem;
  const int g = bulk ? 3 : 1;
  const int gp = 4;   // the pipelined forms exist in FP32 only
  const Form f[kForms] = {{false, 3, 1}, {false, 1, 1}, {false, 2, 1}, {true, 1, 1},
                          {false, g, 2}, {true, 1, 2},  {false, g, 4}, {false, g, 8},
                          {false, gp, 1}, {false, gp, 2}, {false, gp, 4}};
  return f[i];
}

static bool form_fits(const fvm_batch *b, const Form &f) {
  const bool fp32 = b->prec == FVM_PREC_FP32;
  if (f.grad >= 3 && !(fp32 && grad_bulk_layout(b->caps.max_tri, kTriLocMax, b->caps.viscous != 0).total <= kMaxSmem))
    return false;
  if (f.fused) {
    if (fp32) return false;   // FP64 only (the FP32 stencil gradient)
    const size_t sm = fp32 ? smem_step(b->cfg, (float *)nullptr) : smem_step(b->cfg, (double *)nullptr);
    if (sm > kMaxSmem || !b->fused_fits) return false;
  }
  return true;
}

static int32_t apply_form(fvm_batch *b, const Form &f) {
  b->fused = b->fused_wanted = f.fused;
  b->cfg.grad_mode = f.grad;
  const bool rechain = f.chains != b->chains;
  b->chains = f.chains;
  drop_graphs(b);
  return rechain ? update_work(b) : FVM_OK;   // the parts of the work list
}

extern "C" int32_t fvm_batch_set_form(fvm_batch *b, int32_t form) {
  if (b && b->pending) {   // deferred admissions first
    const int32_t cst = batch_commit(b);
    if (cst) return cst;
  }
  if (!b || form < 0 || form >= kForms) return FVM_ERR_ARG;
  const Form f = form_of(b, form);
  if (!form_fits(b, f)) return FVM_ERR_ARG;
  return apply_form(b, f);
}

extern "C" int32_t fvm_batch_tune(fvm_batch *b, int32_t iters, int32_t max, double *ms_per_iter,
                                  int32_t *choice) {
  if (b && b->pending) {   // deferred admissions first
    const int32_t cst = batch_commit(b);
    if (cst) return cst;
  }
  if (!b || iters < 1 || max < 0 || (max > 0 && !ms_per_iter)) return FVM_ERR_ARG;
  // whole multi-iteration graphs when the steps are untimed
  const int timed = b->timing ? iters : (iters + kGraphIters - 1) / kGraphIters * kGraphIters;
  for (int i = 0; i < max; i++) ms_per_iter[i] = 0.0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  FVM_TRY(b, cudaEventCreate(&e0));
  cudaError_t ce = cudaEventCreate(&e1);
  if (ce != cudaSuccess) {
    cudaEventDestroy(e0);
    FVM_TRY(b, ce);
  }
  int best = -1;
  double best_ms = 0.0;
  int32_t st = FVM_OK;
  // every fourth call times every candidate; in between, a candidate more
  // than kTuneSkip times slower than the best of its last timing is not
  // re-timed (its last time is reported)
  static_assert(kForms <= 16, "tune_last holds 16 forms");
  constexpr double kTuneSkip = 1.25;
  double prev_best = 0.0;
  for (int i = 0; i < kForms; i++)
    if (b->tune_last[i] > 0.0 && (prev_best == 0.0 || b->tune_last[i] < prev_best))
      prev_best = b->tune_last[i];
  const bool full = b->tune_calls % 4 == 0 || prev_best == 0.0;
  b->tune_calls++;
  for (int i = 0; i < kForms && st == FVM_OK; i++) {
    const Form f = form_of(b, i);
    // FP32: the per-thread-load and per-vertex triangle passes are not
    // timed (they only serve viscous meshes there and were never fastest);
    // set_form still accepts them
    if (!form_fits(b, f) || (b->prec == FVM_PREC_FP32 && (f.grad == 1 || f.grad == 2))) {
      b->tune_last[i] = 0.0;
      continue;
    }
    if (!full && b->tune_last[i] > kTuneSkip * prev_best) {
      if (i < max) ms_per_iter[i] = b->tune_last[i];
      continue;
    }
    if ((st = apply_form(b, f))) break;
    // timed as the steps will run: whole multi-iteration graphs (captured
    // before the timing), so each form is timed over at least one
    if (!b->timing && (st = build_graph(b, kGraphIters))) break;
    if ((st = fvm_batch_step(b, 1))) break;   // one untimed iteration
    cudaError_t e = cudaEventRecord(e0, b->stream);
    if (e == cudaSuccess) st = fvm_batch_step(b, timed);
    if (e == cudaSuccess && st == FVM_OK) e = cudaEventRecord(e1, b->stream);
    if (e == cudaSuccess && st == FVM_OK) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess && st == FVM_OK) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e != cudaSuccess) st = cuda_status(b, e);
    if (st) break;
    const double per = (double)ms / timed;
    b->tune_last[i] = per;
    if (i < max) ms_per_iter[i] = per;
    if (best < 0 || per < best_ms) {
      best = i;
      best_ms = per;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (best < 0) best = form_fits(b, form_of(b, 0)) ? 0 : 1;
  const int32_t st2 = apply_form(b, form_of(b, best));
  if (choice) *choice = best;
  return st ? st : st2;
}

extern "C" int32_t fvm_batch_sync(fvm_batch *b) {
  if (!b) return FVM_ERR_ARG;
  FVM_TRY(b, cudaStreamSynchronize(b->stream));
  return FVM_OK;
}

extern "C" int32_t fvm_batch_poll(fvm_batch *b, int32_t slot, int32_t *active, int32_t *niter,
                                  double *fres, double *cl, double *cd, int32_t *status,
                                  int32_t *bad_point) {
  if (b && b->pending) {   // deferred admissions first
    const int32_t cst = batch_commit(b);
    if (cst) return cst;
  }
  if (!slot_of(b, slot)) return FVM_ERR_ARG;
  MeshCtl c;
  int32_t st = get_ctl(b, slot, c);
  if (st) return st;
  if (active) *active = c.active;
  if (niter) *niter = c.n_done;
  if (fres) *fres = c.fres;
  if (cl) *cl = c.cl;
  if (cd) *cd = c.cd;
  if (status) *status = c.err;
  if (bad_point) *bad_point = (c.err == FVM_ERR_NONPOSITIVE) ? c.err_point : 0;
  return FVM_OK;
}

extern "C" int32_t fvm_batch_history(fvm_batch *b, int32_t slot, int32_t first, int32_t count,
                                     double *fres, int32_t *iresi, double *fresi, double *cl,
                                     double *cd) {
  if (b && b->pending) {   // deferred admissions first
    const int32_t cst = batch_commit(b);
    if (cst) return cst;
  }
  if (!slot_of(b, slot) || first < 0 || count < 0) return FVM_ERR_ARG;
  MeshCtl c;
  int32_t st = get_ctl(b, slot, c);
  if (st) return st;
  if (first + count > c.n_done || c.n_done - first > kHistRows) return FVM_ERR_ARG;
  std::vector<double> f(count), fi(count), l(count), d(count);
  std::vector<int> ir(count);
  // the rows form at most two contiguous runs of the slot's ring
  int done = 0;
  while (done < count) {
    const int r0 = (first + done) % kHistRows;
    const int run = std::min(count - done, kHistRows - r0);
    const size_t row = (size_t)c.hist_off + r0;
    FVM_TRY(b, cudaMemcpyAsync(&f[done], b->h_fres + row, 8 * run, cudaMemcpyDeviceToHost, b->stream));
    FVM_TRY(b, cudaMemcpyAsync(&fi[done], b->h_fresi + row, 8 * run, cudaMemcpyDeviceToHost, b->stream));
    FVM_TRY(b, cudaMemcpyAsync(&l[done], b->h_cl + row, 8 * run, cudaMemcpyDeviceToHost, b->stream));
    FVM_TRY(b, cudaMemcpyAsync(&d[done], b->h_cd + row, 8 * run, cudaMemcpyDeviceToHost, b->stream));
    FVM_TRY(b, cudaMemcpyAsync(&ir[done], b->h_iresi + row, 4 * run, cudaMemcpyDeviceToHost, b->stream));
    done += run;
  }
  FVM_TRY(b, cudaStreamSynchronize(b->stream));
  for (int i = 0; i < count; i++) {
    if (fres) fres[i] = f[i];
    if (fresi) fresi[i] = fi[i];
    if (cl) cl[i] = l[i];
    if (cd) cd[i] = d[i];
    if (iresi) iresi[i] = ir[i];
  }
  return FVM_OK;
}

extern "C" void *fvm_batch_stream(fvm_batch *b) { return b ? (void *)b->stream : nullptr; }

extern "C" int32_t fvm_batch_timing(fvm_batch *b, int32_t on) {
  if (b && b->pending) {   // deferred admissions first
    const int32_t cst = batch_commit(b);
    if (cst) return cst;
  }
  if (!b) return FVM_ERR_ARG;
  const bool want = on != 0;
  for (int k = 0; k < K_COUNT; k++) {
    b->t_ms[k] = 0.0;
    b->t_launch[k] = 0;
  }
  if (want == b->timing) return FVM_OK;
  FVM_TRY(b, cudaStreamSynchronize(b->stream));
  if (want && b->ev.empty()) {
    const int pairs = 128;
    b->ev.resize(2 * pairs);
    b->ev_kind.assign(pairs, 0);
    for (auto &e : b->ev) FVM_TRY(b, cudaEventCreate(&e));
  }
  b->timing = want;
  drop_graphs(b);
  return FVM_OK;
}

extern "C" int32_t fvm_batch_timing_read(fvm_batch *b, int32_t max, char *names, double *ms,
                                         int64_t *launches, int32_t *n) {
  if (!b || max < 0) return FVM_ERR_ARG;
  const int cnt = std::min<int>(max, K_COUNT);
  for (int k = 0; k < cnt; k++) {
    if (names) std::snprintf(names + 32 * k, 32, "%s", kKernelNames[k]);
    if (ms) ms[k] = b->t_ms[k];
    if (launches) launches[k] = b->t_launch[k];
  }
  if (n) *n = cnt;
  return FVM_OK;
}

extern "C" int64_t fvm_batch_launch_count(fvm_batch *b) { return b ? b->launches : -1; }

extern "C" int32_t fvm_batch_test_wait_timeout(fvm_batch *b, int64_t budget_cycles) {
  if (b && b->pending) {   // deferred admissions first
    const int32_t cst = batch_commit(b);
    if (cst) return cst;
  }
  if (!b || budget_cycles <= 0 || b->prec != FVM_PREC_FP32) return FVM_ERR_ARG;
  // one stage-1 gradient pass over every resident mesh (routine mode), each
  // CTA's first block armed but never copied
  const cudaError_t e = launch_grad_pipe(ptrs<float>(b), b->cfg, 1, 0, 1, budget_cycles, 1, 0);
  if (e == cudaErrorNotSupported) return FVM_ERR_STATE;
  FVM_TRY(b, e);
  FVM_TRY(b, cudaStreamSynchronize(b->stream));
  return FVM_OK;
}

extern "C" int32_t fvm_layout_stats(const fvm_mesh *m, int64_t *out) {
  if (!m || !out) return FVM_ERR_ARG;
  MeshLayout L;
  int32_t st = build_layout(*m, kBlockVerts, L);
  if (st) return st;
  out[0] = L.nblk;
  out[1] = (int64_t)L.be_nodes.size();
  out[2] = (int64_t)L.bt_nodes.size();
  out[3] = L.max_slots;
  out[4] = L.max_tri;
  out[5] = (int64_t)L.bb_nodes.size();
  out[6] = L.max_tri2;
  out[7] = L.max_loc;
  out[8] = (int64_t)L.halo_ids.size();
  out[9] = verify_layout(L);
  return FVM_OK;
}

// ---------------------------------------------------------------------------
// single-mesh API: a batch of one
// ---------------------------------------------------------------------------
struct fvm_handle {
  fvm_batch *b = nullptr;
  int slot = 0;
  int np = 0;
  int iflow = 1;
};

namespace {

Slot &hslot(fvm_handle *h) { return h->b->slots[h->slot]; }

template <typename R>
int32_t residu_impl(fvm_handle *h) {
  fvm_batch *b = h->b;
  const ArenaPtrs<R> A = ptrs<R>(b);
  if (h->iflow != FVM_INVISCID) FVM_TRY(b, launch_visc(A, b->cfg, 0, 0, 1));
  FVM_TRY(b, launch_grad(A, b->cfg, 0, 0, 1));
  FVM_TRY(b, launch_flux(A, b->cfg, 0, 0 /*MODE_RESIDUAL*/, 0, 1));
  b->launches += (h->iflow != FVM_INVISCID) ? 3 : 2;
  FVM_TRY(b, cudaStreamSynchronize(b->stream));
  return FVM_OK;
}

}  // namespace

extern "C" void fvm_abi_sizes(int64_t out[4]) {
  out[0] = (int64_t)sizeof(fvm_params);
  out[1] = (int64_t)sizeof(fvm_mesh);
  out[2] = (int64_t)sizeof(fvm_geom);
  out[3] = (int64_t)sizeof(fvm_batch_caps);
}

extern "C" const char *fvm_gpu_strerror(int32_t s) {
  switch (s) {
    case FVM_OK: return "ok";
    case FVM_ERR_ARG: return "invalid argument";
    case FVM_ERR_CUDA: return "CUDA runtime error";
    case FVM_ERR_NONPOSITIVE: return "Density/pressure is negative at point";
    case FVM_ERR_ROE_SONIC: return "Sonic speed is negative";
    case FVM_ERR_ZERO_FIRST_RES: return "Residue in first iteration is zero";
    case FVM_ERR_TIMEOUT: return "device wait timed out";
    case FVM_ERR_NOMEM: return "device memory allocation failed";
    case FVM_ERR_STATE: return "call out of order";
    case FVM_ERR_GEOMETRY: return "degenerate or inconsistent geometry";
    case FVM_ERR_CAPACITY: return "capacity exceeded";
    case FVM_CHECKPOINTED: return "stopped at a checkpoint";
    default: return "unknown status";
  }
}

extern "C" int32_t fvm_gpu_create(const fvm_params *par, const fvm_mesh *m, fvm_handle **out) {
  if (!par || !m || !out) return FVM_ERR_ARG;
  *out = nullptr;
  if (m->np < 3 || m->nt < 1) return FVM_ERR_ARG;
  // size the arena exactly for this mesh
  MeshLayout L;
  if (!m->edge || !m->iedge || !m->elem || !m->ptype || (m->nbe > 0 && !m->beindx))
    return FVM_ERR_ARG;
  int32_t st = build_layout(*m, kBlockVerts, L);
  if (st) return st;
  fvm_batch_caps c;
  std::memset(&c, 0, sizeof(c));
  c.vertices = L.np;
  c.meshes = 1;
  c.viscous = par->iflow != FVM_INVISCID;
  c.blocks = L.nblk;
  c.edge_entries = std::max<int64_t>(1, L.be_nodes.size());
  c.boundary_entries = std::max<int64_t>(1, L.bb_nodes.size());
  c.tri_entries = std::max<int64_t>(1, L.bt_nodes.size());
  c.triangles = L.nt;
  c.edge_incidence = std::max<int64_t>(1, L.ve_list.size());
  c.tri_incidence = std::max<int64_t>(1, L.vt_list.size());
  c.all_incidence = std::max<int64_t>(1, L.va_list.size());
  c.solid_edges = std::max<int64_t>(1, L.sw_nodes.size());
  c.max_slots = std::max(1, L.max_slots);
  c.max_tri = std::max(1, L.max_tri);
  c.max_tri2 = std::max(1, L.max_tri2);
  c.max_loc = std::max(1, L.max_loc);
  c.halo_entries = std::max<int64_t>(1, L.halo_ids.size());
  c.halo_incidence = std::max<int64_t>(1, L.hl_list.size());
  c.grid = L.nblk;
  fvm_handle *h = new (std::nothrow) fvm_handle();
  if (!h) return FVM_ERR_NOMEM;
  if ((st = fvm_batch_create(par->precision, &c, &h->b))) {
    delete h;
    return st;
  }
  if ((st = fvm_batch_add(h->b, par, m, &h->slot))) {
    fvm_batch_destroy(h->b);
    delete h;
    return st;
  }
  h->np = m->np;
  h->iflow = par->iflow;
  *out = h;
  return FVM_OK;
}

extern "C" int32_t fvm_gpu_destroy(fvm_handle *h) {
  if (!h) return FVM_OK;
  fvm_batch_destroy(h->b);
  delete h;
  return FVM_OK;
}

extern "C" int32_t fvm_gpu_set_state(fvm_handle *h, const double *prim, const double *nut,
                                     const double *mul, const double *mu, int32_t iterlast) {
  if (!h) return FVM_ERR_ARG;
  return fvm_batch_set_state(h->b, h->slot, prim, nut, mul, mu, iterlast);
}

extern "C" int32_t fvm_gpu_get_state(fvm_handle *h, double *prim, double *nut, double *mul,
                                     double *mu, double *qx, double *qy) {
  if (!h) return FVM_ERR_ARG;
  return fvm_batch_get_state(h->b, h->slot, prim, nut, mul, mu, qx, qy);
}

extern "C" int32_t fvm_gpu_get_residual(fvm_handle *h, double *res) {
  if (!h || !res) return FVM_ERR_ARG;
  const int32_t st = get_vertex(h->b, hslot(h), res, h->b->res, 4, 4 * h->b->rsz);
  return st ? st : sync_stream(h->b);
}

extern "C" int32_t fvm_gpu_get_dt(fvm_handle *h, double *dt) {
  if (!h || !dt) return FVM_ERR_ARG;
  const int32_t st = get_vertex(h->b, hslot(h), dt, h->b->dt, 1, h->b->rsz);
  return st ? st : sync_stream(h->b);
}

extern "C" int32_t fvm_gpu_get_prim_old(fvm_handle *h, double *prim_old) {
  if (!h || !prim_old) return FVM_ERR_ARG;
  MeshCtl c;
  int32_t st = get_ctl(h->b, h->slot, c);
  if (st) return st;
  st = get_vertex(h->b, hslot(h), prim_old, h->b->st[(c.phase + 2) % 3], 4, 4 * h->b->rsz);
  return st ? st : sync_stream(h->b);
}

extern "C" int32_t fvm_gpu_save_old(fvm_handle *h) {
  if (!h) return FVM_ERR_ARG;
  fvm_batch *b = h->b;
  MeshCtl c;
  int32_t st = get_ctl(b, h->slot, c);
  if (st) return st;
  const size_t rec = 4 * b->rsz, off = (size_t)hslot(h).off[P_V] * rec;
  FVM_TRY(b, cudaMemcpyAsync(static_cast<unsigned char *>(b->st[(c.phase + 2) % 3]) + off,
                             static_cast<unsigned char *>(b->st[c.phase]) + off, rec * h->np,
                             cudaMemcpyDeviceToDevice, b->stream));
  FVM_TRY(b, cudaStreamSynchronize(b->stream));
  return FVM_OK;
}

extern "C" int32_t fvm_gpu_time_step(fvm_handle *h) {
  if (!h) return FVM_ERR_ARG;
  fvm_batch *b = h->b;
  if (b->prec == FVM_PREC_FP64) FVM_TRY(b, launch_time_step(ptrs<double>(b), b->cfg));
  else FVM_TRY(b, launch_time_step(ptrs<float>(b), b->cfg));
  b->launches++;
  FVM_TRY(b, cudaStreamSynchronize(b->stream));
  return FVM_OK;
}

extern "C" int32_t fvm_gpu_residu(fvm_handle *h) {
  if (!h) return FVM_ERR_ARG;
  MeshCtl c;
  int32_t st = get_ctl(h->b, h->slot, c);
  if (st) return st;
  c.err = 0;
  if ((st = put_ctl(h->b, h->slot, c))) return st;
  st = h->b->prec == FVM_PREC_FP64 ? residu_impl<double>(h) : residu_impl<float>(h);
  if (st) return st;
  if ((st = get_ctl(h->b, h->slot, c))) return st;
  return c.err ? c.err : FVM_OK;
}

extern "C" int32_t fvm_gpu_update(fvm_handle *h, int32_t irk) {
  if (!h || irk < 1 || irk > 3) return FVM_ERR_ARG;
  fvm_batch *b = h->b;
  if (b->prec == FVM_PREC_FP64) FVM_TRY(b, launch_update(ptrs<double>(b), b->cfg, irk));
  else FVM_TRY(b, launch_update(ptrs<float>(b), b->cfg, irk));
  b->launches++;
  FVM_TRY(b, cudaStreamSynchronize(b->stream));
  return FVM_OK;
}

extern "C" int32_t fvm_gpu_sa_model(fvm_handle *h) {
  if (!h) return FVM_ERR_ARG;
  if (h->iflow != FVM_TURBULENT) return FVM_OK;
  fvm_batch *b = h->b;
  if (b->prec == FVM_PREC_FP64) FVM_TRY(b, launch_sa(ptrs<double>(b), b->cfg, 0, 1));
  else FVM_TRY(b, launch_sa(ptrs<float>(b), b->cfg, 0, 1));
  b->launches++;
  MeshCtl c;
  int32_t st = get_ctl(b, h->slot, c);
  if (st) return st;
  c.nphase = 1 - c.nphase;
  return put_ctl(b, h->slot, c);
}

extern "C" int32_t fvm_gpu_limitgrad(fvm_handle *h) {
  if (!h) return FVM_ERR_ARG;
  fvm_batch *b = h->b;
  if (b->prec == FVM_PREC_FP64) FVM_TRY(b, launch_limitgrad(ptrs<double>(b), b->cfg));
  else FVM_TRY(b, launch_limitgrad(ptrs<float>(b), b->cfg));
  b->launches++;
  FVM_TRY(b, cudaStreamSynchronize(b->stream));
  return FVM_OK;
}

extern "C" int32_t fvm_gpu_gradient(fvm_handle *h) {
  if (!h) return FVM_ERR_ARG;
  fvm_batch *b = h->b;
  if (b->prec == FVM_PREC_FP64) FVM_TRY(b, launch_gradient_edge(ptrs<double>(b), b->cfg));
  else FVM_TRY(b, launch_gradient_edge(ptrs<float>(b), b->cfg));
  b->launches++;
  FVM_TRY(b, cudaStreamSynchronize(b->stream));
  return FVM_OK;
}

extern "C" int32_t fvm_gpu_shockind(fvm_handle *h) {
  if (!h) return FVM_ERR_ARG;
  fvm_batch *b = h->b;
  if (b->prec == FVM_PREC_FP64) FVM_TRY(b, launch_shockind(ptrs<double>(b), b->cfg));
  else FVM_TRY(b, launch_shockind(ptrs<float>(b), b->cfg));
  b->launches++;
  FVM_TRY(b, cudaStreamSynchronize(b->stream));
  return FVM_OK;
}

extern "C" int32_t fvm_gpu_check_positivity(fvm_handle *h, int32_t *bad_point) {
  if (!h) return FVM_ERR_ARG;
  fvm_batch *b = h->b;
  MeshCtl c;
  int32_t st = get_ctl(b, h->slot, c);
  if (st) return st;
  c.err_point = INT_MAX;
  if ((st = put_ctl(b, h->slot, c))) return st;
  if (b->prec == FVM_PREC_FP64) FVM_TRY(b, launch_positivity(ptrs<double>(b), b->cfg));
  else FVM_TRY(b, launch_positivity(ptrs<float>(b), b->cfg));
  b->launches++;
  if ((st = get_ctl(b, h->slot, c))) return st;
  const int bad = c.err_point == INT_MAX ? 0 : c.err_point;
  if (bad_point) *bad_point = bad;
  return bad ? FVM_ERR_NONPOSITIVE : FVM_OK;
}

extern "C" int32_t fvm_gpu_clcd(fvm_handle *h, double *cl, double *cd) {
  if (!h) return FVM_ERR_ARG;
  fvm_batch *b = h->b;
  const int serial = b->prec == FVM_PREC_FP64;
  if (b->prec == FVM_PREC_FP64) FVM_TRY(b, launch_clcd(ptrs<double>(b), b->cfg, h->slot, serial));
  else FVM_TRY(b, launch_clcd(ptrs<float>(b), b->cfg, h->slot, serial));
  b->launches++;
  MeshCtl c;
  int32_t st = get_ctl(b, h->slot, c);
  if (st) return st;
  if (cl) *cl = c.cl;
  if (cd) *cd = c.cd;
  return FVM_OK;
}

extern "C" int32_t fvm_gpu_conres(fvm_handle *h, int32_t first, double *fres, double *fresi,
                                  int32_t *iresi) {
  if (!h) return FVM_ERR_ARG;
  fvm_batch *b = h->b;
  MeshCtl c;
  int32_t st = get_ctl(b, h->slot, c);
  if (st) return st;
  c.err = 0;
  if ((st = put_ctl(b, h->slot, c))) return st;
  if (b->prec == FVM_PREC_FP64) FVM_TRY(b, launch_conres(ptrs<double>(b), b->cfg, h->slot, first));
  else FVM_TRY(b, launch_conres(ptrs<float>(b), b->cfg, h->slot, first));
  b->launches += 2;
  if ((st = get_ctl(b, h->slot, c))) return st;
  if (fres) *fres = c.fres;
  if (fresi) *fresi = c.fresi;
  if (iresi) *iresi = c.iresi;
  return c.err ? c.err : FVM_OK;
}

extern "C" int32_t fvm_gpu_iterate(fvm_handle *h, int32_t nmax, double minres, int32_t *niter,
                                   double *hist_fres, int32_t *hist_iresi, double *hist_fresi,
                                   double *hist_cl, double *hist_cd, int32_t *bad_point) {
  if (!h || nmax < 0) return FVM_ERR_ARG;
  if (niter) *niter = 0;
  if (bad_point) *bad_point = 0;
  if (nmax == 0) return FVM_OK;
  fvm_batch *b = h->b;
  int32_t st = fvm_batch_start(b, h->slot, nmax, minres);
  if (st) return st;
  int consumed = 0, active = 1, done = 0, status = 0, bad = 0;
  while (true) {
    const int k = std::min(kHistRows, nmax - consumed);
    if ((st = fvm_batch_step(b, k))) return st;
    if ((st = fvm_batch_poll(b, h->slot, &active, &done, nullptr, nullptr, nullptr, &status, &bad)))
      return st;
    const int rows = done - consumed;
    if (rows > 0) {
      auto off_d = [&](double *p) { return p ? p + consumed : nullptr; };
      if ((st = fvm_batch_history(b, h->slot, consumed, rows, off_d(hist_fres),
                                  hist_iresi ? hist_iresi + consumed : nullptr, off_d(hist_fresi),
                                  off_d(hist_cl), off_d(hist_cd))))
        return st;
    }
    consumed = done;
    if (!active || consumed >= nmax) break;
  }
  if (niter) *niter = consumed;
  if (bad_point) *bad_point = bad;
  return status ? status : FVM_OK;
}

// ---- stand-alone set-up kernels -----------------------------------------
extern "C" int32_t fvm_gpu_dtlength(int32_t np, int32_t nt, const double *coord,
                                    const int32_t *elem, const double *elarea, double *drmin) {
  if (np < 1 || nt < 1 || !coord || !elem || !elarea || !drmin) return FVM_ERR_ARG;
  for (int64_t k = 0; k < 3 * (int64_t)nt; k++)
    if (elem[k] < 1 || elem[k] > np) return FVM_ERR_ARG;
  std::vector<void *> O;
  double2 *dc = nullptr;
  int *de = nullptr;
  double *da = nullptr, *dr = nullptr;
  cudaError_t e = cudaSuccess;
  if ((e = dalloc(O, &dc, np)) == cudaSuccess && (e = dalloc(O, &de, 3 * (size_t)nt)) == cudaSuccess &&
      (e = dalloc(O, &da, nt)) == cudaSuccess && (e = dalloc(O, &dr, np)) == cudaSuccess &&
      (e = cudaMemcpy(dc, coord, 16 * (size_t)np, cudaMemcpyHostToDevice)) == cudaSuccess &&
      (e = cudaMemcpy(de, elem, 12 * (size_t)nt, cudaMemcpyHostToDevice)) == cudaSuccess &&
      (e = cudaMemcpy(da, elarea, 8 * (size_t)nt, cudaMemcpyHostToDevice)) == cudaSuccess &&
      (e = launch_dtlength(np, nt, dc, de, da, dr, 0)) == cudaSuccess)
    e = cudaMemcpy(drmin, dr, 8 * (size_t)np, cudaMemcpyDeviceToHost);
  for (void *p : O) cudaFree(p);
  return cuda_status(nullptr, e);
}

extern "C" int32_t fvm_gpu_wall_dist(int32_t np, int32_t ne, const double *coord,
                                     const int32_t *edge, const int32_t *ptype, int32_t bugcompat,
                                     double *wd) {
  if (np < 1 || ne < 0 || !coord || !edge || !ptype || !wd) return FVM_ERR_ARG;
  std::vector<int2> sedge;   // wall_dist.f:17-25
  for (int i = 0; i < ne; i++) {
    const int a = edge[2 * i] - 1, c = edge[2 * i + 1] - 1;
    if (a < 0 || a >= np || c < 0 || c >= np) return FVM_ERR_ARG;
    if (ptype[a] == FVM_PT_SOLID && ptype[c] == FVM_PT_SOLID) sedge.push_back(make_int2(a, c));
  }
  std::vector<void *> O;
  double2 *dc = nullptr;
  int2 *ds = nullptr;
  int *dp = nullptr;
  double *dw = nullptr;
  cudaError_t e = cudaSuccess;
  if ((e = dalloc(O, &dc, np)) == cudaSuccess && (e = dalloc(O, &ds, sedge.size())) == cudaSuccess &&
      (e = dalloc(O, &dp, np)) == cudaSuccess && (e = dalloc(O, &dw, np)) == cudaSuccess &&
      (e = cudaMemcpy(dc, coord, 16 * (size_t)np, cudaMemcpyHostToDevice)) == cudaSuccess &&
      (sedge.empty() ||
       (e = cudaMemcpy(ds, sedge.data(), 8 * sedge.size(), cudaMemcpyHostToDevice)) == cudaSuccess) &&
      (e = cudaMemcpy(dp, ptype, 4 * (size_t)np, cudaMemcpyHostToDevice)) == cudaSuccess &&
      (e = launch_wall_dist(np, (int)sedge.size(), dc, ds, dp, bugcompat, dw, 0)) == cudaSuccess)
    e = cudaMemcpy(wd, dw, 8 * (size_t)np, cudaMemcpyDeviceToHost);
  for (void *p : O) cudaFree(p);
  return cuda_status(nullptr, e);
}
