// fvm_geometry.cpp -- host-side driver geometry and the constants of the
// COMMON blocks, for callers without the Fortran driver.
//
// fvm_geom_build restates the chain of src/geometric.f:15-60 with 0-based
// containers: tri_orient.f:15-41, el_surr_point.f:12-40 (elements around a
// point, Lohner's two-pass CSR), pt_surr_pt.f:13-33 (points around a point
// in first-seen order), create_edge.f:9-18, el_surr_edge.f:9-33,
// tri_coord.f (centroid / circumcentre), areas.f, flength.f:13-61,
// reorder_edges (flength.f:71-107), make_bdedges.f:9-44 and the checks of
// geom_stat.f:10-37.  The edge numbering, orientation and every floating
// point operation follow those files, so the arrays are identical to the
// driver's.  Compiled with -ffp-contract=off.
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <new>
#include <utility>
#include <vector>

#include "../../include/fvm_gpu.h"
#include "fvm_geom_gpu.h"

namespace {

inline double sqr(double x) { return x * x; }
inline double maxd(double a, double b) { return b > a ? b : a; }

// flength.f:52 and make_bdedges.f:12 test edneigh(1,i)*edneigh(2,i) .eq. 0:
// the 32-bit product, formed here in unsigned arithmetic (defined wrap-around)
inline int boundary_edge(const int32_t *edneigh, int i) {
  return (uint32_t)edneigh[2 * i] * (uint32_t)edneigh[2 * i + 1] == 0u;
}

template <typename T>
T *dup(const std::vector<T> &v) {
  T *p = static_cast<T *>(std::malloc(sizeof(T) * (v.empty() ? 1 : v.size())));
  if (p && !v.empty()) std::memcpy(p, v.data(), sizeof(T) * v.size());
  return p;
}

}  // namespace

extern "C" int32_t fvm_params_init(fvm_params *p, int32_t iflow, double mach_inf, double aoa_deg,
                                   double rey, double cfl, int32_t iflux, int32_t ilimit,
                                   int32_t vortex, double xref, double yref, int32_t cell_type,
                                   double nut_ratio, int32_t precision, int32_t bugcompat) {
  if (!p) return FVM_ERR_ARG;
  if (iflow < 1 || iflow > 3 || iflux < 1 || iflux > 3 || (ilimit != 0 && ilimit != 1) ||
      (vortex != 0 && vortex != 1) || (cell_type != 1 && cell_type != 2) ||
      (precision != FVM_PREC_FP64 && precision != FVM_PREC_FP32) || !(mach_inf > 0.0))
    return FVM_ERR_ARG;  // read_input.f:72-110
  std::memset(p, 0, sizeof(*p));
  p->iflow = iflow;
  p->iflux = iflux;
  p->ilimit = ilimit;
  p->vortex = vortex;
  p->cell_type = cell_type;
  p->precision = precision;
  p->bugcompat = bugcompat ? 1 : 0;
  // math.f:8-40
  p->gamma = 1.4;
  p->gamma1 = p->gamma - 1.0;
  p->gas_const = 1.0;
  p->pi = 4.0 * std::atan2(1.0, 1.0);
  p->prandtl = 0.72;
  p->prandtl_turb = 0.9;
  p->albada11 = 2.0 / 3.0;
  p->albada12 = 1.0 - p->albada11;
  p->albada21 = 4.0 / 3.0;
  p->albada22 = 1.0 - p->albada21;
  p->epsilon = 1.0e-16;  // param.h:105
  p->cb1 = 0.1355;
  p->cb2 = 0.622;
  p->sigma_sa = 2.0 / 3.0;
  p->kolm = 0.41;
  p->cw1 = p->cb1 / sqr(p->kolm) + (1.0 + p->cb2) / p->sigma_sa;
  p->cw2 = 0.3;
  p->cw3 = 2.0;
  p->cv1 = 7.1;
  p->cv2 = 5.0;
  p->cv11 = (p->cv1 * p->cv1) * p->cv1;
  const double cw3_3 = (p->cw3 * p->cw3) * p->cw3;
  p->cw31 = 1.0 + cw3_3 * cw3_3;
  p->cw32 = cw3_3 * cw3_3;
  p->kolm2 = sqr(p->kolm);
  p->cb2sig1 = (1.0 + p->cb2) / p->sigma_sa;
  p->cb2sig2 = p->cb2 / p->sigma_sa;
  // read_input.f / initialize.f:14-34
  p->mach_inf = mach_inf;
  p->aoa_deg = aoa_deg;
  p->rey = rey;
  p->cfl = cfl;
  p->xref = xref;
  p->yref = yref;
  p->q_inf = 1.0;
  p->r_inf = 1.0;
  p->p_inf = 1.0 / (p->gamma * sqr(mach_inf));
  p->t_inf = p->p_inf / (p->r_inf * p->gas_const);
  p->aoa = aoa_deg * p->pi / 180.0;
  p->u_inf = p->q_inf * std::cos(p->aoa);
  p->v_inf = p->q_inf * std::sin(p->aoa);
  p->a_inf = std::sqrt(p->gamma * p->p_inf / p->r_inf);
  p->sconst = 110.4 * p->t_inf / 300.0;
  p->nut_inf = 0.0;
  if (iflow == FVM_TURBULENT) {
    // initialize.f:69-74: nut = 0.1*mul/rho at the freestream; nut_inf = nut(1)
    const double temp = p->p_inf / p->r_inf / p->gas_const;
    const double num = p->t_inf + p->sconst;
    const double den = temp + p->sconst;
    const double mul = std::pow(temp / p->t_inf, 1.5) * (num / den) / p->rey;
    p->nut_inf = nut_ratio * mul / p->r_inf;
  }
  // initialize.f:52-58
  p->airk[0] = 0.0;
  p->airk[1] = 3.0 / 4.0;
  p->airk[2] = 1.0 / 3.0;
  p->birk[0] = 1.0;
  p->birk[1] = 1.0 / 4.0;
  p->birk[2] = 2.0 / 3.0;
  return FVM_OK;
}

struct GeomOwned {
  fvm_geom g;
  std::vector<int32_t> edge, edneigh, iedge, beindx, spts;
  std::vector<double> ds, dsb, elarea, cvarea, mcarea, drmin, wd;
};

// Points the fvm_geom struct (and its fvm_mesh) at G's arrays.
static fvm_geom *publish(GeomOwned *G, int32_t np, int32_t nt, int nswe, const double *coord,
                         int32_t *elem, const int32_t *ptype) {
  fvm_geom &g = G->g;
  g.edge = G->edge.data();
  g.edneigh = G->edneigh.data();
  g.iedge = G->iedge.data();
  g.beindx = G->beindx.data();
  g.spts = G->spts.data();
  g.ds = G->ds.data();
  g.dsb = G->dsb.data();
  g.elarea = G->elarea.data();
  g.cvarea = G->cvarea.data();
  g.mcarea = G->mcarea.data();
  g.drmin = G->drmin.data();
  g.wd = G->wd.data();
  fvm_mesh &m = g.mesh;
  m.np = np;
  m.nt = nt;
  m.ne = (int)G->iedge.size();
  m.netot = (int)(G->edge.size() / 2);
  m.nsp = (int)G->spts.size();
  m.nbe = (int)G->beindx.size();
  m.nswe1 = 1;
  m.nswe2 = nswe;
  m.nffe1 = nswe + 1;
  m.nffe2 = m.nbe;
  m.coord = coord;
  m.elem = elem;
  m.ptype = ptype;
  m.spts = g.spts;
  m.edge = g.edge;
  m.iedge = g.iedge;
  m.beindx = g.beindx;
  m.ds = g.ds;
  m.elarea = g.elarea;
  m.cvarea = g.cvarea;
  m.mcarea = g.mcarea;
  m.drmin = g.drmin;
  m.wd = g.wd;
  return &G->g;
}

extern "C" int32_t fvm_geom_build(int32_t np, int32_t nt, const double *coord, int32_t *elem,
                                  const int32_t *ptype, int32_t cell_type, fvm_geom **out) {
  if (!out || np < 3 || nt < 1 || !coord || !elem || !ptype) return FVM_ERR_ARG;
  if (cell_type != FVM_CELL_MEDIAN && cell_type != FVM_CELL_BARTH) return FVM_ERR_ARG;
  *out = nullptr;
  for (int64_t k = 0; k < 3 * (int64_t)nt; k++)
    if (elem[k] < 1 || elem[k] > np) return FVM_ERR_ARG;
  auto X = [&](int n) { return coord[2 * n]; };      // n 0-based
  auto Y = [&](int n) { return coord[2 * n + 1]; };
  auto E = [&](int t, int k) -> int32_t & { return elem[3 * t + k]; };  // 1-based values

  // tri_orient.f:15-41
  for (int t = 0; t < nt; t++) {
    const int p1 = E(t, 0) - 1, p2 = E(t, 1) - 1, p3 = E(t, 2) - 1;
    const double dx1 = X(p2) - X(p1), dy1 = Y(p2) - Y(p1);
    const double dx2 = X(p3) - X(p2), dy2 = Y(p3) - Y(p2);
    const double cross = dx1 * dy2 - dx2 * dy1;
    if (cross == 0.0) return FVM_ERR_GEOMETRY;
    if (cross < 0.0) {
      const int32_t tmp = E(t, 1);
      E(t, 1) = E(t, 2);
      E(t, 2) = tmp;
    }
  }
  // el_surr_point.f: esup_ptr[p]..esup_ptr[p+1] lists the elements around p
  std::vector<int> esup_ptr(np + 1, 0), esup(3 * (size_t)nt);
  for (int t = 0; t < nt; t++)
    for (int k = 0; k < 3; k++) esup_ptr[E(t, k)]++;
  for (int p = 0; p < np; p++) esup_ptr[p + 1] += esup_ptr[p];
  {
    std::vector<int> fill(esup_ptr.begin(), esup_ptr.end() - 1);
    for (int t = 0; t < nt; t++)
      for (int k = 0; k < 3; k++) esup[fill[E(t, k) - 1]++] = t;
  }
  // pt_surr_pt.f: neighbours in first-seen order over the elements of p
  std::vector<int> psup_ptr(np + 1, 0), psup;
  psup.reserve(6 * (size_t)np);
  {
    std::vector<int> last(np, -1);
    for (int p = 0; p < np; p++) {
      for (int j = esup_ptr[p]; j < esup_ptr[p + 1]; j++) {
        const int t = esup[j];
        for (int k = 0; k < 3; k++) {
          const int q = E(t, k) - 1;
          if (q != p && last[q] != p) {
            psup.push_back(q);
            last[q] = p;
          }
        }
      }
      psup_ptr[p + 1] = (int)psup.size();
    }
  }
  GeomOwned *G = new (std::nothrow) GeomOwned();
  if (!G) return FVM_ERR_NOMEM;
  // create_edge.f:9-18
  for (int p = 0; p < np; p++)
    for (int j = psup_ptr[p]; j < psup_ptr[p + 1]; j++)
      if (psup[j] > p) {
        G->edge.push_back(p + 1);
        G->edge.push_back(psup[j] + 1);
      }
  const int ne_all = (int)(G->edge.size() / 2);
  // el_surr_edge.f:9-33: left triangle first; boundary edges oriented so
  // that their single triangle is on the left
  G->edneigh.assign(2 * (size_t)ne_all, 0);
  for (int i = 0; i < ne_all; i++) {
    const int n1 = G->edge[2 * i], n2 = G->edge[2 * i + 1];
    int left = 0, right = 0;
    for (int j = esup_ptr[n1 - 1]; j < esup_ptr[n1]; j++) {
      const int t = esup[j];
      const int a = E(t, 0), b = E(t, 1), c = E(t, 2);
      if ((n1 == a && n2 == b) || (n1 == b && n2 == c) || (n1 == c && n2 == a)) left = t + 1;
      if ((n2 == a && n1 == b) || (n2 == b && n1 == c) || (n2 == c && n1 == a)) right = t + 1;
    }
    if (left == 0) {
      left = right;
      right = 0;
      G->edge[2 * i] = n2;
      G->edge[2 * i + 1] = n1;
    }
    G->edneigh[2 * i] = left;
    G->edneigh[2 * i + 1] = right;
  }
  // tri_coord.f: centroid (median) or circumcentre (Barth)
  std::vector<double> tc(2 * (size_t)nt);
  for (int t = 0; t < nt; t++) {
    const int n1 = E(t, 0) - 1, n2 = E(t, 1) - 1, n3 = E(t, 2) - 1;
    if (cell_type == FVM_CELL_MEDIAN) {
      tc[2 * t] = (X(n1) + X(n2) + X(n3)) / 3.0;
      tc[2 * t + 1] = (Y(n1) + Y(n2) + Y(n3)) / 3.0;
      continue;
    }
    const double x1 = X(n1), y1 = Y(n1), x2 = X(n2), y2 = Y(n2), x3 = X(n3), y3 = Y(n3);
    const double l1 = sqr(x2 - x3) + sqr(y2 - y3);
    const double l2 = sqr(x3 - x1) + sqr(y3 - y1);
    const double l3 = sqr(x1 - x2) + sqr(y1 - y2);
    const double beta1 = maxd(0.0, l2 + l3 - l1);
    const double beta2 = maxd(0.0, l3 + l1 - l2);
    const double beta3 = maxd(0.0, l1 + l2 - l3);
    const double det = (x2 - x1) * (y3 - y1) - (x3 - x1) * (y2 - y1);
    const double b1 = 0.5 * ((x2 - x1) * (x2 + x1) + (y2 - y1) * (y2 + y1));
    const double b2 = 0.5 * ((x3 - x1) * (x3 + x1) + (y3 - y1) * (y3 + y1));
    const double xc = ((y3 - y1) * b1 - (y2 - y1) * b2) / det;
    const double yc = (-(x3 - x1) * b1 + (x2 - x1) * b2) / det;
    if (beta1 == 0.0) {
      tc[2 * t] = 0.5 * (x2 + x3);
      tc[2 * t + 1] = 0.5 * (y2 + y3);
    } else if (beta2 == 0.0) {
      tc[2 * t] = 0.5 * (x3 + x1);
      tc[2 * t + 1] = 0.5 * (y3 + y1);
    } else if (beta3 == 0.0) {
      tc[2 * t] = 0.5 * (x1 + x2);
      tc[2 * t + 1] = 0.5 * (y1 + y2);
    } else {
      tc[2 * t] = xc;
      tc[2 * t + 1] = yc;
    }
  }
  // areas.f: tri_area, mc_area, cvareas_mc / cvareas_bc
  G->elarea.resize(nt);
  G->mcarea.assign(np, 0.0);
  for (int t = 0; t < nt; t++) {
    const int n1 = E(t, 0) - 1, n2 = E(t, 1) - 1, n3 = E(t, 2) - 1;
    const double dx1 = X(n2) - X(n1), dy1 = Y(n2) - Y(n1);
    const double dx2 = X(n3) - X(n1), dy2 = Y(n3) - Y(n1);
    G->elarea[t] = 0.5 * (dx1 * dy2 - dx2 * dy1);
  }
  for (int t = 0; t < nt; t++) {
    const double a3 = G->elarea[t] / 3.0;
    for (int k = 0; k < 3; k++) G->mcarea[E(t, k) - 1] += a3;
  }
  if (cell_type == FVM_CELL_MEDIAN) {
    G->cvarea = G->mcarea;
  } else {
    G->cvarea.assign(np, 0.0);
    for (int t = 0; t < nt; t++)
      for (int j = 0; j < 3; j++) {
        const int n1 = E(t, j) - 1;
        const int n2 = E(t, (j + 2) % 3) - 1;   // previous vertex
        const int n3 = E(t, (j + 1) % 3) - 1;   // next vertex
        const double x[5] = {X(n1), 0.5 * (X(n1) + X(n3)), tc[2 * t], 0.5 * (X(n1) + X(n2)), X(n1)};
        const double y[5] = {Y(n1), 0.5 * (Y(n1) + Y(n3)), tc[2 * t + 1], 0.5 * (Y(n1) + Y(n2)), Y(n1)};
        double area = 0.0;
        for (int k = 0; k < 4; k++) area = area + x[k] * y[k + 1] - x[k + 1] * y[k];
        if (area < 0.0) {
          delete G;
          return FVM_ERR_GEOMETRY;  // areas.f:145-150
        }
        G->cvarea[n1] += 0.5 * area;
      }
  }
  // flength.f:13-61
  G->ds.resize(2 * (size_t)ne_all);
  G->dsb.assign(2 * (size_t)np, 0.0);
  for (int i = 0; i < ne_all; i++) {
    const int n1 = G->edge[2 * i] - 1, n2 = G->edge[2 * i + 1] - 1;
    const int p1 = G->edneigh[2 * i], p2 = G->edneigh[2 * i + 1];
    if (p1 == 0) {
      delete G;
      return FVM_ERR_GEOMETRY;
    }
    const double x1 = tc[2 * (p1 - 1)], y1 = tc[2 * (p1 - 1) + 1];
    double x2, y2;
    if (p2 != 0) {
      x2 = tc[2 * (p2 - 1)];
      y2 = tc[2 * (p2 - 1) + 1];
    } else {
      x2 = 0.5 * (X(n1) + X(n2));
      y2 = 0.5 * (Y(n1) + Y(n2));
    }
    G->ds[2 * i] = -(y2 - y1);
    G->ds[2 * i + 1] = (x2 - x1);
  }
  for (int i = 0; i < ne_all; i++) {
    if (boundary_edge(G->edneigh.data(), i) == 0) continue;
    const int n1 = G->edge[2 * i] - 1, n2 = G->edge[2 * i + 1] - 1;
    const double nx = Y(n2) - Y(n1);
    const double ny = -(X(n2) - X(n1));
    G->dsb[2 * n1] += 0.5 * nx;
    G->dsb[2 * n1 + 1] += 0.5 * ny;
    G->dsb[2 * n2] += 0.5 * nx;
    G->dsb[2 * n2 + 1] += 0.5 * ny;
  }
  // reorder_edges (flength.f:82-105)
  for (int i = 0; i < ne_all; i++) {
    if (cell_type == FVM_CELL_BARTH) {
      const double length = std::sqrt(sqr(G->ds[2 * i]) + sqr(G->ds[2 * i + 1]));
      if (length == 0.0) continue;
    }
    G->iedge.push_back(i + 1);
  }
  // make_bdedges.f:9-44: solid edges, then farfield edges
  std::vector<int32_t> ff;
  for (int i = 0; i < ne_all; i++) {
    if (boundary_edge(G->edneigh.data(), i) == 0) continue;
    const int t1 = ptype[G->edge[2 * i] - 1], t2 = ptype[G->edge[2 * i + 1] - 1];
    if (t1 == FVM_PT_SOLID && t2 == FVM_PT_SOLID) G->beindx.push_back(i + 1);
    if (t1 == FVM_PT_FARFIELD && t2 == FVM_PT_FARFIELD) ff.push_back(i + 1);
  }
  const int nswe = (int)G->beindx.size();
  G->beindx.insert(G->beindx.end(), ff.begin(), ff.end());
  // geom_stat.f:10-37
  double minel = 1.0e8, mincv = 1.0e8;
  for (int t = 0; t < nt; t++) minel = G->elarea[t] < minel ? G->elarea[t] : minel;
  for (int p = 0; p < np; p++) mincv = G->cvarea[p] < mincv ? G->cvarea[p] : mincv;
  if (minel <= 0.0 || mincv <= 0.0) {
    delete G;
    return FVM_ERR_GEOMETRY;
  }
  for (int p = 0; p < np; p++)
    if (ptype[p] == FVM_PT_SOLID) G->spts.push_back(p + 1);
  G->drmin.assign(np, 0.0);
  G->wd.assign(np, 0.0);

  *out = publish(G, np, nt, nswe, coord, elem, ptype);
  return FVM_OK;
}

// The same chain on the GPU (fvm_geom_gpu.cu): identical arrays, and drmin
// (dtlength.f) from the same device arrays.
extern "C" int32_t fvm_gpu_geom_build(int32_t np, int32_t nt, const double *coord,
                                      int32_t *elem, const int32_t *ptype, int32_t cell_type,
                                      fvm_geom **out) {
  if (!out || np < 3 || nt < 1 || !coord || !elem || !ptype) return FVM_ERR_ARG;
  if (cell_type != FVM_CELL_MEDIAN && cell_type != FVM_CELL_BARTH) return FVM_ERR_ARG;
  *out = nullptr;
  for (int64_t k = 0; k < 3 * (int64_t)nt; k++)
    if (elem[k] < 1 || elem[k] > np) return FVM_ERR_ARG;
  fvm::GeomChainOut R;
  const int32_t st = fvm::geom_chain_gpu(np, nt, coord, elem, ptype, cell_type, R);
  if (st != FVM_OK) return st;
  GeomOwned *G = new (std::nothrow) GeomOwned();
  if (!G) return FVM_ERR_NOMEM;
  std::memcpy(elem, R.elem.data(), sizeof(int32_t) * 3 * (size_t)nt);
  G->edge = std::move(R.edge);
  G->edneigh = std::move(R.edneigh);
  G->iedge = std::move(R.iedge);
  G->beindx = std::move(R.beindx);
  G->spts = std::move(R.spts);
  G->ds = std::move(R.ds);
  G->dsb = std::move(R.dsb);
  G->elarea = std::move(R.elarea);
  G->cvarea = std::move(R.cvarea);
  G->mcarea = std::move(R.mcarea);
  G->drmin = std::move(R.drmin);
  G->wd.assign(np, 0.0);
  *out = publish(G, np, nt, R.nswe, coord, elem, ptype);
  return FVM_OK;
}

extern "C" int32_t fvm_geom_free(fvm_geom *g) {
  if (!g) return FVM_OK;
  // g is the first member of the GeomOwned that fvm_geom_build allocated
  delete reinterpret_cast<GeomOwned *>(g);
  return FVM_OK;
}
