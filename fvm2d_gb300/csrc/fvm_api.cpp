// fvm_api.cpp -- the C ABI of include/fvm_gpu.h: handle, device arena of one
// mesh, per-routine entry points and the graph-captured iteration loop.
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
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

constexpr int kHistChunk = 512;   // iterations per host round trip

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

template <typename T>
cudaError_t upload(std::vector<void *> &owned, T **p, const std::vector<T> &h, cudaStream_t s) {
  cudaError_t e = dalloc(owned, p, h.size());
  if (e != cudaSuccess || h.empty()) return e;
  return cudaMemcpyAsync(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s);
}

}  // namespace

struct fvm_handle {
  fvm_params par{};
  int prec = 0;          // FVM_PREC_*
  size_t rsz = 8;        // bytes of one state scalar
  MeshLayout L;
  cudaStream_t stream = nullptr;
  std::vector<void *> owned;
  // vertex arrays
  void *st[3] = {nullptr, nullptr, nullptr};
  void *grad = nullptr, *resv = nullptr, *res = nullptr;
  void *dt = nullptr, *mu = nullptr, *mul = nullptr, *nut[2] = {nullptr, nullptr};
  double2 *coord = nullptr;
  double *ais = nullptr, *cvarea = nullptr, *drmin = nullptr, *wd = nullptr;
  int *orig = nullptr;
  uint8_t *vflag = nullptr;
  int *ve_ptr = nullptr, *vt_ptr = nullptr, *va_ptr = nullptr, *va_list = nullptr;
  uint16_t *ve_list = nullptr, *vt_list = nullptr;
  BlockInfo *blocks = nullptr;
  int2 *be_nodes = nullptr, *sw_nodes = nullptr;
  double2 *be_ds = nullptr;
  D4 *be_csl = nullptr;
  int4 *bb_nodes = nullptr, *bt_nodes = nullptr;
  double *elarea = nullptr;
  MeshConst *mc = nullptr;
  MeshCtl *ctl = nullptr;
  BlockPartial *part = nullptr;
  double *h_fres = nullptr, *h_fresi = nullptr, *h_cl = nullptr, *h_cd = nullptr;
  int *h_iresi = nullptr;
  int *work = nullptr, *nwork = nullptr, *mesh_list = nullptr;
  LaunchCfg cfg{};
  cudaGraphExec_t graph = nullptr;
  bool state_set = false;
  std::string last_error;
};

namespace {

template <typename R>
ArenaPtrs<R> ptrs(fvm_handle *h) {
  ArenaPtrs<R> A;
  std::memset(&A, 0, sizeof(A));
  for (int i = 0; i < 3; i++) A.st[i] = static_cast<R4<R> *>(h->st[i]);
  A.grad = static_cast<Grad<R> *>(h->grad);
  A.resv = static_cast<R4<R> *>(h->resv);
  A.res = static_cast<R4<R> *>(h->res);
  A.dt = static_cast<R *>(h->dt);
  A.mu = static_cast<R *>(h->mu);
  A.mul = static_cast<R *>(h->mul);
  A.nut[0] = static_cast<R *>(h->nut[0]);
  A.nut[1] = static_cast<R *>(h->nut[1]);
  A.coord = h->coord;
  A.ais = h->ais;
  A.cvarea = h->cvarea;
  A.drmin = h->drmin;
  A.wd = h->wd;
  A.orig = h->orig;
  A.vflag = h->vflag;
  A.ve_ptr = h->ve_ptr;
  A.ve_list = h->ve_list;
  A.vt_ptr = h->vt_ptr;
  A.vt_list = h->vt_list;
  A.blocks = h->blocks;
  A.be_nodes = h->be_nodes;
  A.be_ds = h->be_ds;
  A.be_csl = h->be_csl;
  A.bb_nodes = h->bb_nodes;
  A.bt_nodes = h->bt_nodes;
  A.elarea = h->elarea;
  A.sw_nodes = h->sw_nodes;
  A.va_ptr = h->va_ptr;
  A.va_list = h->va_list;
  A.mc = h->mc;
  A.ctl = h->ctl;
  A.part = h->part;
  A.h_fres = h->h_fres;
  A.h_fresi = h->h_fresi;
  A.h_cl = h->h_cl;
  A.h_cd = h->h_cd;
  A.h_iresi = h->h_iresi;
  A.work = h->work;
  A.nwork = h->nwork;
  return A;
}

int32_t cuda_status(fvm_handle *h, cudaError_t e) {
  if (e == cudaSuccess) return FVM_OK;
  if (h) h->last_error = cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return FVM_ERR_NOMEM;
  return FVM_ERR_CUDA;
}

#define FVM_TRY(h, expr)                               \
  do {                                                 \
    cudaError_t _e = (expr);                           \
    if (_e != cudaSuccess) return cuda_status(h, _e);  \
  } while (0)

MeshConst make_const(const fvm_params &p, const MeshLayout &L) {
  MeshConst c;
  std::memset(&c, 0, sizeof(c));
  c.iflow = p.iflow;
  c.iflux = p.iflux;
  c.ilimit = p.ilimit;
  c.vortex = p.vortex;
  c.bugcompat = p.bugcompat;
  c.precision = p.precision;
  c.v0 = 0;
  c.nv = L.np;
  c.blk0 = 0;
  c.nblk = L.nblk;
  c.sw0 = 0;
  c.nsw = (int)L.sw_nodes.size();
  for (int k = 0; k < 3; k++) c.orig123[k] = L.np > k ? L.iperm[k] : 0;
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
  return c;
}

int32_t get_ctl(fvm_handle *h, MeshCtl &c) {
  FVM_TRY(h, cudaMemcpyAsync(&c, h->ctl, sizeof(MeshCtl), cudaMemcpyDeviceToHost, h->stream));
  FVM_TRY(h, cudaStreamSynchronize(h->stream));
  return FVM_OK;
}

int32_t put_ctl(fvm_handle *h, const MeshCtl &c) {
  FVM_TRY(h, cudaMemcpyAsync(h->ctl, &c, sizeof(MeshCtl), cudaMemcpyHostToDevice, h->stream));
  FVM_TRY(h, cudaStreamSynchronize(h->stream));
  return FVM_OK;
}

// host double [np][k] (driver order) -> device R [np][k] (renumbered)
int32_t put_vertex(fvm_handle *h, void *dst, const double *src, int k, size_t dst_stride) {
  const int np = h->L.np;
  std::vector<unsigned char> buf((size_t)np * dst_stride, 0);
  for (int v = 0; v < np; v++) {
    const double *s = src + (size_t)h->L.perm[v] * k;
    unsigned char *d = buf.data() + (size_t)v * dst_stride;
    for (int q = 0; q < k; q++) {
      if (h->rsz == 8) {
        const double x = s[q];
        std::memcpy(d + 8 * q, &x, 8);
      } else {
        const float x = (float)s[q];
        std::memcpy(d + 4 * q, &x, 4);
      }
    }
  }
  FVM_TRY(h, cudaMemcpyAsync(dst, buf.data(), buf.size(), cudaMemcpyHostToDevice, h->stream));
  FVM_TRY(h, cudaStreamSynchronize(h->stream));
  return FVM_OK;
}

// device R [np][stride] -> host double [np][k] (driver order), components
// [c0, c0+k) of each record
int32_t get_vertex(fvm_handle *h, double *dst, const void *src, int k, size_t src_stride,
                   int c0 = 0) {
  const int np = h->L.np;
  std::vector<unsigned char> buf((size_t)np * src_stride);
  FVM_TRY(h, cudaMemcpyAsync(buf.data(), src, buf.size(), cudaMemcpyDeviceToHost, h->stream));
  FVM_TRY(h, cudaStreamSynchronize(h->stream));
  for (int v = 0; v < np; v++) {
    double *d = dst + (size_t)h->L.perm[v] * k;
    const unsigned char *s = buf.data() + (size_t)v * src_stride;
    for (int q = 0; q < k; q++) {
      if (h->rsz == 8) {
        double x;
        std::memcpy(&x, s + 8 * (c0 + q), 8);
        d[q] = x;
      } else {
        float x;
        std::memcpy(&x, s + 4 * (c0 + q), 4);
        d[q] = x;
      }
    }
  }
  return FVM_OK;
}

template <typename R>
int32_t record_iteration(fvm_handle *h) {
  const ArenaPtrs<R> A = ptrs<R>(h);
  const LaunchCfg &c = h->cfg;
  const int iflow = h->par.iflow;
  for (int s = 1; s <= 3; s++) {
    if (iflow != FVM_INVISCID) FVM_TRY(h, launch_visc(A, c, s, s == 1, 0));
    FVM_TRY(h, launch_grad(A, c, s, (s == 1 && iflow == FVM_INVISCID) ? 1 : 0, 0));
    FVM_TRY(h, launch_flux(A, c, s, 1 /*MODE_UPDATE*/, s, 0));
  }
  if (iflow == FVM_TURBULENT) FVM_TRY(h, launch_sa(A, c, 3, 0));
  FVM_TRY(h, launch_monitor(A, c, h->mesh_list, 1, h->prec == FVM_PREC_FP64 ? 1 : 0));
  return FVM_OK;
}

int32_t build_graph(fvm_handle *h) {
  if (h->graph) return FVM_OK;
  cudaGraph_t g = nullptr;
  FVM_TRY(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  int32_t st = h->prec == FVM_PREC_FP64 ? record_iteration<double>(h) : record_iteration<float>(h);
  cudaError_t e = cudaStreamEndCapture(h->stream, &g);
  if (st != FVM_OK) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  FVM_TRY(h, e);
  e = cudaGraphInstantiate(&h->graph, g, 0);
  cudaGraphDestroy(g);
  FVM_TRY(h, e);
  return FVM_OK;
}

template <typename R>
int32_t prepare_kernels(fvm_handle *h) {
  // dynamic shared-memory limits, set once outside any stream capture
  FVM_TRY(h, prepare_attributes(h->cfg, (R *)nullptr));
  return FVM_OK;
}

int32_t check_handle(fvm_handle *h) {
  if (!h) return FVM_ERR_ARG;
  return FVM_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
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
    default: return "unknown status";
  }
}

extern "C" int32_t fvm_gpu_create(const fvm_params *par, const fvm_mesh *m, fvm_handle **out) {
  if (!par || !m || !out) return FVM_ERR_ARG;
  *out = nullptr;
  if (m->np < 3 || m->nt < 1 || m->netot < 1 || !m->coord || !m->elem || !m->ptype || !m->edge ||
      !m->iedge || !m->ds || !m->elarea || !m->cvarea || !m->mcarea || !m->drmin)
    return FVM_ERR_ARG;
  if (par->iflow == FVM_TURBULENT && !m->wd) return FVM_ERR_ARG;
  if (m->nbe > 0 && !m->beindx) return FVM_ERR_ARG;
  if (par->precision != FVM_PREC_FP64 && par->precision != FVM_PREC_FP32) return FVM_ERR_ARG;
  fvm_handle *h = new (std::nothrow) fvm_handle();
  if (!h) return FVM_ERR_NOMEM;
  h->par = *par;
  h->prec = par->precision;
  h->rsz = h->prec == FVM_PREC_FP64 ? 8 : 4;
  int32_t st = build_layout(*m, kBlockVerts, h->L);
  if (st != FVM_OK) {
    delete h;
    return st;
  }
  auto fail = [&](int32_t s) {
    fvm_gpu_destroy(h);
    return s;
  };
  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return fail(cuda_status(h, e));
  const MeshLayout &L = h->L;
  const int np = L.np, nt = L.nt, nblk = L.nblk;
  const size_t r = h->rsz;
  auto &O = h->owned;
  cudaStream_t s = h->stream;
#define TRYA(expr)                                     \
  do {                                                 \
    cudaError_t _e = (expr);                           \
    if (_e != cudaSuccess) return fail(cuda_status(h, _e)); \
  } while (0)
  // state and work arrays
  for (int i = 0; i < 3; i++) TRYA(dalloc(O, (unsigned char **)&h->st[i], 4 * r * np));
  TRYA(dalloc(O, (unsigned char **)&h->grad, 8 * r * np));
  TRYA(dalloc(O, (unsigned char **)&h->resv, 4 * r * np));
  TRYA(dalloc(O, (unsigned char **)&h->res, 4 * r * np));
  TRYA(dalloc(O, (unsigned char **)&h->dt, r * np));
  TRYA(dalloc(O, (unsigned char **)&h->mu, r * np));
  TRYA(dalloc(O, (unsigned char **)&h->mul, r * np));
  TRYA(dalloc(O, (unsigned char **)&h->nut[0], r * np));
  TRYA(dalloc(O, (unsigned char **)&h->nut[1], r * np));
  TRYA(cudaMemsetAsync(h->resv, 0, 4 * r * np, s));
  TRYA(cudaMemsetAsync(h->grad, 0, 8 * r * np, s));
  // geometry, renumbered
  std::vector<double2> coord(np);
  std::vector<double> ais(np), cvarea(np), drmin(np), wd(np, 1.0);
  std::vector<int> orig(np);
  const double n1b6 = 1.0 / 6.0;
  for (int v = 0; v < np; v++) {
    const int o = L.perm[v];
    coord[v] = make_double2(m->coord[2 * o], m->coord[2 * o + 1]);
    ais[v] = n1b6 / m->mcarea[o];            // green_gauss.f:34
    cvarea[v] = m->cvarea[o];
    drmin[v] = m->drmin[o];
    if (m->wd) wd[v] = m->wd[o];
    orig[v] = o + 1;
  }
  TRYA(upload(O, &h->coord, coord, s));
  TRYA(upload(O, &h->ais, ais, s));
  TRYA(upload(O, &h->cvarea, cvarea, s));
  TRYA(upload(O, &h->drmin, drmin, s));
  TRYA(upload(O, &h->wd, wd, s));
  TRYA(upload(O, &h->orig, orig, s));
  TRYA(upload(O, &h->vflag, L.vflag, s));
  TRYA(upload(O, &h->ve_ptr, L.ve_ptr, s));
  TRYA(upload(O, &h->ve_list, L.ve_list, s));
  TRYA(upload(O, &h->vt_ptr, L.vt_ptr, s));
  TRYA(upload(O, &h->vt_list, L.vt_list, s));
  TRYA(upload(O, &h->va_ptr, L.va_ptr, s));
  TRYA(upload(O, &h->va_list, L.va_list, s));
  std::vector<BlockInfo> blocks = L.blocks;
  for (int b = 0; b < nblk; b++) {
    blocks[b].mesh = 0;
    blocks[b].part = b;
  }
  TRYA(upload(O, &h->blocks, blocks, s));
  TRYA(upload(O, &h->be_nodes, L.be_nodes, s));
  std::vector<double2> be_ds(L.be_edge.size());
  for (size_t k = 0; k < L.be_edge.size(); k++) {
    const int e = L.be_edge[k];
    be_ds[k] = make_double2(m->ds[2 * e], m->ds[2 * e + 1]);
  }
  TRYA(upload(O, &h->be_ds, be_ds, s));
  TRYA(dalloc(O, &h->be_csl, be_ds.size()));
  TRYA(launch_edge_csl(h->be_ds, h->be_csl, (int)be_ds.size(), s));
  TRYA(upload(O, &h->bb_nodes, L.bb_nodes, s));
  std::vector<int4> bt = L.bt_nodes;   // .w = driver triangle = index into elarea
  TRYA(upload(O, &h->bt_nodes, bt, s));
  std::vector<double> elarea(m->elarea, m->elarea + nt);
  TRYA(upload(O, &h->elarea, elarea, s));
  TRYA(upload(O, &h->sw_nodes, L.sw_nodes, s));
  std::vector<MeshConst> mc(1, make_const(*par, L));
  TRYA(upload(O, &h->mc, mc, s));
  TRYA(dalloc(O, &h->ctl, 1));
  TRYA(dalloc(O, &h->part, nblk));
  TRYA(dalloc(O, &h->h_fres, kHistChunk));
  TRYA(dalloc(O, &h->h_fresi, kHistChunk));
  TRYA(dalloc(O, &h->h_cl, kHistChunk));
  TRYA(dalloc(O, &h->h_cd, kHistChunk));
  TRYA(dalloc(O, &h->h_iresi, kHistChunk));
  std::vector<int> work(nblk);
  for (int b = 0; b < nblk; b++) work[b] = b;
  TRYA(upload(O, &h->work, work, s));
  std::vector<int> nwork(1, nblk), mesh_list(1, 0);
  TRYA(upload(O, &h->nwork, nwork, s));
  TRYA(upload(O, &h->mesh_list, mesh_list, s));
#undef TRYA
  h->cfg.grid = nblk;
  h->cfg.max_tri = L.max_tri;
  h->cfg.max_slots = L.max_slots;
  h->cfg.viscous = par->iflow != FVM_INVISCID;
  h->cfg.stream = s;
  MeshCtl ctl;
  std::memset(&ctl, 0, sizeof(ctl));
  ctl.err_point = INT_MAX;
  if ((st = put_ctl(h, ctl))) return fail(st);
  // freestream state (initialize.f:60-89)
  {
    std::vector<double> prim(4 * (size_t)np), nut(np, 0.0), mul(np, 0.0), mu(np, 0.0);
    for (int v = 0; v < np; v++) {
      prim[4 * v] = par->r_inf;
      prim[4 * v + 1] = par->u_inf;
      prim[4 * v + 2] = par->v_inf;
      prim[4 * v + 3] = par->p_inf;
    }
    if (par->iflow != FVM_INVISCID) {
      const double temp = par->p_inf / par->r_inf / par->gas_const;
      const double mul0 = std::pow(temp / par->t_inf, 1.5) *
                          ((par->t_inf + par->sconst) / (temp + par->sconst)) / par->rey;
      for (int v = 0; v < np; v++) {
        mul[v] = mul0;
        if (par->iflow == FVM_TURBULENT) {
          nut[v] = par->nut_inf;
          const double chi = nut[v] * par->r_inf / mul0;
          const double chi3 = (chi * chi) * chi;
          mu[v] = mul0 + par->r_inf * nut[v] * (chi3 / (chi3 + par->cv11));
        } else {
          mu[v] = mul0;
        }
      }
    }
    if ((st = fvm_gpu_set_state(h, prim.data(), nut.data(), mul.data(), mu.data(), 0)))
      return fail(st);
    h->state_set = true;
  }
  st = h->prec == FVM_PREC_FP64 ? prepare_kernels<double>(h) : prepare_kernels<float>(h);
  if (st) return fail(st);
  *out = h;
  return FVM_OK;
}

extern "C" int32_t fvm_gpu_destroy(fvm_handle *h) {
  if (!h) return FVM_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->graph) cudaGraphExecDestroy(h->graph);
  for (void *p : h->owned) cudaFree(p);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return FVM_OK;
}

extern "C" int32_t fvm_gpu_set_state(fvm_handle *h, const double *prim, const double *nut,
                                     const double *mul, const double *mu, int32_t iterlast) {
  if (check_handle(h) || !prim) return FVM_ERR_ARG;
  MeshCtl c;
  int32_t st = get_ctl(h, c);
  if (st) return st;
  const size_t r = h->rsz;
  if ((st = put_vertex(h, h->st[c.phase], prim, 4, 4 * r))) return st;
  if (nut && (st = put_vertex(h, h->nut[c.nphase], nut, 1, r))) return st;
  if (mul && (st = put_vertex(h, h->mul, mul, 1, r))) return st;
  if (mu && (st = put_vertex(h, h->mu, mu, 1, r))) return st;
  c.iter = iterlast;
  c.iterlast = iterlast;
  c.fres1 = 0.0;
  c.err = 0;
  c.err_point = INT_MAX;
  h->state_set = true;
  return put_ctl(h, c);
}

extern "C" int32_t fvm_gpu_get_state(fvm_handle *h, double *prim, double *nut, double *mul,
                                     double *mu, double *qx, double *qy) {
  if (check_handle(h)) return FVM_ERR_ARG;
  MeshCtl c;
  int32_t st = get_ctl(h, c);
  if (st) return st;
  const size_t r = h->rsz;
  if (prim && (st = get_vertex(h, prim, h->st[c.phase], 4, 4 * r))) return st;
  if (nut && (st = get_vertex(h, nut, h->nut[c.nphase], 1, r))) return st;
  if (mul && (st = get_vertex(h, mul, h->mul, 1, r))) return st;
  if (mu && (st = get_vertex(h, mu, h->mu, 1, r))) return st;
  if (qx && (st = get_vertex(h, qx, h->grad, 4, 8 * r, 0))) return st;
  if (qy && (st = get_vertex(h, qy, h->grad, 4, 8 * r, 4))) return st;
  return FVM_OK;
}

extern "C" int32_t fvm_gpu_get_residual(fvm_handle *h, double *res) {
  if (check_handle(h) || !res) return FVM_ERR_ARG;
  return get_vertex(h, res, h->res, 4, 4 * h->rsz);
}

extern "C" int32_t fvm_gpu_get_dt(fvm_handle *h, double *dt) {
  if (check_handle(h) || !dt) return FVM_ERR_ARG;
  return get_vertex(h, dt, h->dt, 1, h->rsz);
}

extern "C" int32_t fvm_gpu_get_prim_old(fvm_handle *h, double *prim_old) {
  if (check_handle(h) || !prim_old) return FVM_ERR_ARG;
  MeshCtl c;
  int32_t st = get_ctl(h, c);
  if (st) return st;
  return get_vertex(h, prim_old, h->st[(c.phase + 2) % 3], 4, 4 * h->rsz);
}

// ---- per-routine entry points -------------------------------------------
extern "C" int32_t fvm_gpu_save_old(fvm_handle *h) {
  if (check_handle(h)) return FVM_ERR_ARG;
  MeshCtl c;
  int32_t st = get_ctl(h, c);
  if (st) return st;
  FVM_TRY(h, cudaMemcpyAsync(h->st[(c.phase + 2) % 3], h->st[c.phase], 4 * h->rsz * h->L.np,
                             cudaMemcpyDeviceToDevice, h->stream));
  FVM_TRY(h, cudaStreamSynchronize(h->stream));
  return FVM_OK;
}

extern "C" int32_t fvm_gpu_time_step(fvm_handle *h) {
  if (check_handle(h)) return FVM_ERR_ARG;
  if (h->prec == FVM_PREC_FP64) FVM_TRY(h, launch_time_step(ptrs<double>(h), h->cfg));
  else FVM_TRY(h, launch_time_step(ptrs<float>(h), h->cfg));
  FVM_TRY(h, cudaStreamSynchronize(h->stream));
  return FVM_OK;
}

template <typename R>
static int32_t residu_impl(fvm_handle *h) {
  const ArenaPtrs<R> A = ptrs<R>(h);
  if (h->par.iflow != FVM_INVISCID) FVM_TRY(h, launch_visc(A, h->cfg, 0, 0, 1));
  FVM_TRY(h, launch_grad(A, h->cfg, 0, 0, 1));
  FVM_TRY(h, launch_flux(A, h->cfg, 0, 0 /*MODE_RESIDUAL*/, 0, 1));
  FVM_TRY(h, cudaStreamSynchronize(h->stream));
  return FVM_OK;
}

extern "C" int32_t fvm_gpu_residu(fvm_handle *h) {
  if (check_handle(h)) return FVM_ERR_ARG;
  MeshCtl c;
  int32_t st = get_ctl(h, c);
  if (st) return st;
  c.err = 0;
  if ((st = put_ctl(h, c))) return st;
  st = h->prec == FVM_PREC_FP64 ? residu_impl<double>(h) : residu_impl<float>(h);
  if (st) return st;
  if ((st = get_ctl(h, c))) return st;
  return c.err ? c.err : FVM_OK;
}

extern "C" int32_t fvm_gpu_update(fvm_handle *h, int32_t irk) {
  if (check_handle(h) || irk < 1 || irk > 3) return FVM_ERR_ARG;
  if (h->prec == FVM_PREC_FP64) FVM_TRY(h, launch_update(ptrs<double>(h), h->cfg, irk));
  else FVM_TRY(h, launch_update(ptrs<float>(h), h->cfg, irk));
  FVM_TRY(h, cudaStreamSynchronize(h->stream));
  return FVM_OK;
}

extern "C" int32_t fvm_gpu_sa_model(fvm_handle *h) {
  if (check_handle(h)) return FVM_ERR_ARG;
  if (h->par.iflow != FVM_TURBULENT) return FVM_OK;
  if (h->prec == FVM_PREC_FP64) FVM_TRY(h, launch_sa(ptrs<double>(h), h->cfg, 0, 1));
  else FVM_TRY(h, launch_sa(ptrs<float>(h), h->cfg, 0, 1));
  MeshCtl c;
  int32_t st = get_ctl(h, c);
  if (st) return st;
  c.nphase = 1 - c.nphase;
  return put_ctl(h, c);
}

extern "C" int32_t fvm_gpu_limitgrad(fvm_handle *h) {
  if (check_handle(h)) return FVM_ERR_ARG;
  if (h->prec == FVM_PREC_FP64) FVM_TRY(h, launch_limitgrad(ptrs<double>(h), h->cfg));
  else FVM_TRY(h, launch_limitgrad(ptrs<float>(h), h->cfg));
  FVM_TRY(h, cudaStreamSynchronize(h->stream));
  return FVM_OK;
}

extern "C" int32_t fvm_gpu_check_positivity(fvm_handle *h, int32_t *bad_point) {
  if (check_handle(h)) return FVM_ERR_ARG;
  MeshCtl c;
  int32_t st = get_ctl(h, c);
  if (st) return st;
  c.err_point = INT_MAX;
  if ((st = put_ctl(h, c))) return st;
  if (h->prec == FVM_PREC_FP64) FVM_TRY(h, launch_positivity(ptrs<double>(h), h->cfg));
  else FVM_TRY(h, launch_positivity(ptrs<float>(h), h->cfg));
  if ((st = get_ctl(h, c))) return st;
  const int bad = c.err_point == INT_MAX ? 0 : c.err_point;
  if (bad_point) *bad_point = bad;
  return bad ? FVM_ERR_NONPOSITIVE : FVM_OK;
}

extern "C" int32_t fvm_gpu_clcd(fvm_handle *h, double *cl, double *cd) {
  if (check_handle(h)) return FVM_ERR_ARG;
  const int serial = h->prec == FVM_PREC_FP64;
  if (h->prec == FVM_PREC_FP64) FVM_TRY(h, launch_clcd(ptrs<double>(h), h->cfg, 0, serial));
  else FVM_TRY(h, launch_clcd(ptrs<float>(h), h->cfg, 0, serial));
  MeshCtl c;
  int32_t st = get_ctl(h, c);
  if (st) return st;
  if (cl) *cl = c.cl;
  if (cd) *cd = c.cd;
  return FVM_OK;
}

extern "C" int32_t fvm_gpu_conres(fvm_handle *h, int32_t first, double *fres, double *fresi,
                                  int32_t *iresi) {
  if (check_handle(h)) return FVM_ERR_ARG;
  MeshCtl c;
  int32_t st = get_ctl(h, c);
  if (st) return st;
  c.err = 0;
  if ((st = put_ctl(h, c))) return st;
  if (h->prec == FVM_PREC_FP64) FVM_TRY(h, launch_conres(ptrs<double>(h), h->cfg, 0, first));
  else FVM_TRY(h, launch_conres(ptrs<float>(h), h->cfg, 0, first));
  if ((st = get_ctl(h, c))) return st;
  if (fres) *fres = c.fres;
  if (fresi) *fresi = c.fresi;
  if (iresi) *iresi = c.iresi;
  return c.err ? c.err : FVM_OK;
}

// ---- the iteration loop --------------------------------------------------
extern "C" int32_t fvm_gpu_iterate(fvm_handle *h, int32_t nmax, double minres, int32_t *niter,
                                   double *hist_fres, int32_t *hist_iresi, double *hist_fresi,
                                   double *hist_cl, double *hist_cd, int32_t *bad_point) {
  if (check_handle(h) || nmax < 0) return FVM_ERR_ARG;
  if (niter) *niter = 0;
  if (bad_point) *bad_point = 0;
  if (nmax == 0) return FVM_OK;
  int32_t st = build_graph(h);
  if (st) return st;
  MeshCtl c;
  if ((st = get_ctl(h, c))) return st;
  c.active = 1;
  c.n_done = 0;
  c.n_max = nmax;
  c.minres = minres;
  c.err = 0;
  c.err_point = INT_MAX;
  c.hist_off = 0;
  c.hist_cap = kHistChunk;
  if ((st = put_ctl(h, c))) return st;
  int consumed = 0;
  std::vector<double> f(kHistChunk), fi(kHistChunk), cl(kHistChunk), cd(kHistChunk);
  std::vector<int> ir(kHistChunk);
  while (true) {
    const int k = std::min(kHistChunk, nmax - consumed);
    for (int i = 0; i < k; i++) FVM_TRY(h, cudaGraphLaunch(h->graph, h->stream));
    if ((st = get_ctl(h, c))) return st;
    const int rows = c.n_done - consumed;
    if (rows > 0) {
      FVM_TRY(h, cudaMemcpyAsync(f.data(), h->h_fres, rows * 8, cudaMemcpyDeviceToHost, h->stream));
      FVM_TRY(h, cudaMemcpyAsync(fi.data(), h->h_fresi, rows * 8, cudaMemcpyDeviceToHost, h->stream));
      FVM_TRY(h, cudaMemcpyAsync(cl.data(), h->h_cl, rows * 8, cudaMemcpyDeviceToHost, h->stream));
      FVM_TRY(h, cudaMemcpyAsync(cd.data(), h->h_cd, rows * 8, cudaMemcpyDeviceToHost, h->stream));
      FVM_TRY(h, cudaMemcpyAsync(ir.data(), h->h_iresi, rows * 4, cudaMemcpyDeviceToHost, h->stream));
      FVM_TRY(h, cudaStreamSynchronize(h->stream));
      for (int i = 0; i < rows; i++) {
        if (hist_fres) hist_fres[consumed + i] = f[i];
        if (hist_fresi) hist_fresi[consumed + i] = fi[i];
        if (hist_cl) hist_cl[consumed + i] = cl[i];
        if (hist_cd) hist_cd[consumed + i] = cd[i];
        if (hist_iresi) hist_iresi[consumed + i] = ir[i];
      }
    }
    consumed = c.n_done;
    if (!c.active || consumed >= nmax) break;
    // next chunk writes its rows from the start of the history buffers
    c.hist_off = -consumed;
    c.hist_cap = consumed + kHistChunk;
    MeshCtl cur;
    if ((st = get_ctl(h, cur))) return st;
    cur.hist_off = c.hist_off;
    cur.hist_cap = c.hist_cap;
    if ((st = put_ctl(h, cur))) return st;
  }
  if (niter) *niter = consumed;
  if (c.err == FVM_ERR_NONPOSITIVE && bad_point) *bad_point = c.err_point;
  return c.err ? c.err : FVM_OK;
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
  int32_t st = FVM_OK;
  cudaError_t e = cudaSuccess;
  if ((e = dalloc(O, &dc, np)) == cudaSuccess && (e = dalloc(O, &de, 3 * (size_t)nt)) == cudaSuccess &&
      (e = dalloc(O, &da, nt)) == cudaSuccess && (e = dalloc(O, &dr, np)) == cudaSuccess &&
      (e = cudaMemcpy(dc, coord, 16 * (size_t)np, cudaMemcpyHostToDevice)) == cudaSuccess &&
      (e = cudaMemcpy(de, elem, 12 * (size_t)nt, cudaMemcpyHostToDevice)) == cudaSuccess &&
      (e = cudaMemcpy(da, elarea, 8 * (size_t)nt, cudaMemcpyHostToDevice)) == cudaSuccess &&
      (e = launch_dtlength(np, nt, dc, de, da, dr, 0)) == cudaSuccess)
    e = cudaMemcpy(drmin, dr, 8 * (size_t)np, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) st = cuda_status(nullptr, e);
  for (void *p : O) cudaFree(p);
  return st;
}

extern "C" int32_t fvm_gpu_wall_dist(int32_t np, int32_t ne, const double *coord,
                                     const int32_t *edge, const int32_t *ptype, int32_t bugcompat,
                                     double *wd) {
  if (np < 1 || ne < 0 || !coord || !edge || !ptype || !wd) return FVM_ERR_ARG;
  std::vector<int2> sedge;   // wall_dist.f:17-25
  for (int i = 0; i < ne; i++) {
    const int a = edge[2 * i] - 1, b = edge[2 * i + 1] - 1;
    if (a < 0 || a >= np || b < 0 || b >= np) return FVM_ERR_ARG;
    if (ptype[a] == FVM_PT_SOLID && ptype[b] == FVM_PT_SOLID) sedge.push_back(make_int2(a, b));
  }
  std::vector<void *> O;
  double2 *dc = nullptr;
  int2 *ds = nullptr;
  int *dp = nullptr;
  double *dw = nullptr;
  int32_t st = FVM_OK;
  cudaError_t e = cudaSuccess;
  if ((e = dalloc(O, &dc, np)) == cudaSuccess && (e = dalloc(O, &ds, sedge.size())) == cudaSuccess &&
      (e = dalloc(O, &dp, np)) == cudaSuccess && (e = dalloc(O, &dw, np)) == cudaSuccess &&
      (e = cudaMemcpy(dc, coord, 16 * (size_t)np, cudaMemcpyHostToDevice)) == cudaSuccess &&
      (sedge.empty() ||
       (e = cudaMemcpy(ds, sedge.data(), 8 * sedge.size(), cudaMemcpyHostToDevice)) == cudaSuccess) &&
      (e = cudaMemcpy(dp, ptype, 4 * (size_t)np, cudaMemcpyHostToDevice)) == cudaSuccess &&
      (e = launch_wall_dist(np, (int)sedge.size(), dc, ds, dp, bugcompat, dw, 0)) == cudaSuccess)
    e = cudaMemcpy(wd, dw, 8 * (size_t)np, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) st = cuda_status(nullptr, e);
  for (void *p : O) cudaFree(p);
  return st;
}
