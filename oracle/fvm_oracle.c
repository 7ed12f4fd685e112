/*
 * fvm_oracle.c -- CPU oracle (test infrastructure, see fvm_oracle.h).
 *
 * Serial FP64 restatement of the fvm2d Fortran sources, loop by loop.
 * Arrays keep the Fortran layout; the macros below index them 1-based so
 * each statement reads like the line it restates.  Compile with
 * -ffp-contract=off.
 */
#include "fvm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define NVAR 4
#define INVISCID 1
#define LAMINAR 2
#define TURBULENT 3
#define IROE 1
#define IKFVS 2
#define IHLLC 3
#define MEDIAN 1
#define BARTH 2
#define SOLID 3
#define FARFIELD 5
#define EPSILON 1.0e-16

struct orc {
  orc_input in;
  orc_scalars s;
  /* grid */
  double *coord;   /* coord(2,np)  */
  int32_t *elem;   /* elem(3,nt)   */
  int32_t *ptype, *spts, *fpts;
  /* connectivity */
  int32_t *esup1, *esup2, *psup1, *psup2;
  int32_t *edge, *edneigh, *iedge, *beindx;
  /* geometry */
  double *tcoord, *elarea, *cvarea, *mcarea, *ds, *dsb, *drmin, *wd, *wd1;
  /* state */
  double *prim, *prim_old, *qx, *qy, *res, *dt, *mu, *mul, *nut, *divf;
  double *con_new;
  int64_t len_esup1, len_psup1, len_edge;
};

#define COORD(k, i)   o->coord[2 * ((i) - 1) + (k) - 1]
#define TCOORD(k, i)  o->tcoord[2 * ((i) - 1) + (k) - 1]
#define ELEM(k, i)    o->elem[3 * ((i) - 1) + (k) - 1]
#define EDGE(k, i)    o->edge[2 * ((i) - 1) + (k) - 1]
#define EDNEIGH(k, i) o->edneigh[2 * ((i) - 1) + (k) - 1]
#define DS(k, i)      o->ds[2 * ((i) - 1) + (k) - 1]
#define DSB(k, i)     o->dsb[2 * ((i) - 1) + (k) - 1]
#define PRIM(k, i)    o->prim[NVAR * ((i) - 1) + (k) - 1]
#define PRIMO(k, i)   o->prim_old[NVAR * ((i) - 1) + (k) - 1]
#define QX(k, i)      o->qx[NVAR * ((i) - 1) + (k) - 1]
#define QY(k, i)      o->qy[NVAR * ((i) - 1) + (k) - 1]
#define RES(k, i)     o->res[NVAR * ((i) - 1) + (k) - 1]
#define CONNEW(k, i)  o->con_new[NVAR * ((i) - 1) + (k) - 1]
#define V1(a, i)      (a)[(i) - 1]

static double dmin1(double a, double b) { return b < a ? b : a; }
static double dmax1(double a, double b) { return b > a ? b : a; }
static double sq(double x) { return x * x; }
static double cube(double x) { return (x * x) * x; }
static double pow6(double x) { double x3 = (x * x) * x; return x3 * x3; }

/* ------------------------------------------------------------------ */
/* math.f:4-43                                                         */
/* ------------------------------------------------------------------ */
static void math_consts(orc_scalars *s) {
  s->gamma = 1.4;
  s->gamma1 = s->gamma - 1.0;
  s->gas_const = 1.0;
  s->pi = 4.0 * atan2(1.0, 1.0);
  s->prandtl = 0.72;
  s->prandtl_turb = 0.9;
  s->albada11 = 2.0 / 3.0;
  s->albada12 = 1.0 - s->albada11;
  s->albada21 = 4.0 / 3.0;
  s->albada22 = 1.0 - s->albada21;
  s->cb1 = 0.1355;
  s->cb2 = 0.622;
  s->sigma_sa = 2.0 / 3.0;
  s->kolm = 0.41;
  s->cw1 = s->cb1 / sq(s->kolm) + (1.0 + s->cb2) / s->sigma_sa;
  s->cw2 = 0.3;
  s->cw3 = 2.0;
  s->cv1 = 7.1;
  s->cv2 = 5.0;
  s->cv11 = cube(s->cv1);
  s->cw31 = 1.0 + pow6(s->cw3);
  s->cw32 = pow6(s->cw3);
  s->kolm2 = sq(s->kolm);
  s->cb2sig1 = (1.0 + s->cb2) / s->sigma_sa;
  s->cb2sig2 = s->cb2 / s->sigma_sa;
}

/* ------------------------------------------------------------------ */
/* viscosity.f                                                          */
/* ------------------------------------------------------------------ */
static double sutherland_viscosity(const orc_t *o, double density, double pressure) {
  const orc_scalars *s = &o->s;
  double temp = pressure / density / s->gas_const;
  double num = s->t_inf + s->sconst;
  double den = temp + s->sconst;
  return pow(temp / s->t_inf, 1.5) * (num / den) / s->rey;
}

static double mu_turb(const orc_t *o, double mu_lam, double density, double nu_tilde) {
  double chi = nu_tilde * density / mu_lam;
  double chi3 = cube(chi);
  double fv1 = chi3 / (chi3 + o->s.cv11);
  return density * nu_tilde * fv1;
}

static void sutherland(orc_t *o) {
  for (int i = 1; i <= o->s.np; i++)
    V1(o->mul, i) = sutherland_viscosity(o, PRIM(1, i), PRIM(4, i));
}

static void viscosity(orc_t *o) {
  if (o->in.iflow == LAMINAR) {
    for (int i = 1; i <= o->s.np; i++) V1(o->mu, i) = V1(o->mul, i);
  } else if (o->in.iflow == TURBULENT) {
    for (int i = 1; i <= o->s.np; i++) {
      double mut = mu_turb(o, V1(o->mul, i), PRIM(1, i), V1(o->nut, i));
      V1(o->mu, i) = V1(o->mul, i) + mut;
    }
  }
}

/* ------------------------------------------------------------------ */
/* geometry: tri_orient.f, el_surr_point.f, pt_surr_pt.f, create_edge.f,*/
/* el_surr_edge.f, tri_coord.f, areas.f, flength.f, dtlength.f,        */
/* make_bdedges.f, wall_dist.f, geom_stat.f                            */
/* ------------------------------------------------------------------ */
static int tri_orient(orc_t *o) {
  for (int i = 1; i <= o->s.nt; i++) {
    int p1 = ELEM(1, i), p2 = ELEM(2, i), p3 = ELEM(3, i);
    double dx1 = COORD(1, p2) - COORD(1, p1);
    double dy1 = COORD(2, p2) - COORD(2, p1);
    double dx2 = COORD(1, p3) - COORD(1, p2);
    double dy2 = COORD(2, p3) - COORD(2, p2);
    double cross = dx1 * dy2 - dx2 * dy1;
    if (cross == 0.0) return ORC_ERR_GEOMETRY;
    if (cross < 0.0) {
      int tmp = ELEM(2, i);
      ELEM(2, i) = ELEM(3, i);
      ELEM(3, i) = tmp;
    }
  }
  return ORC_OK;
}

static void el_surr_point(orc_t *o) {
  int np = o->s.np, nt = o->s.nt;
  int32_t *esup2 = o->esup2; /* esup2(1..np+1) stored at [0..np] */
  for (int i = 1; i <= np + 1; i++) esup2[i - 1] = 0;
  for (int ie = 1; ie <= nt; ie++)
    for (int in = 1; in <= 3; in++) {
      int ipoi1 = ELEM(in, ie) + 1;
      esup2[ipoi1 - 1] += 1;
    }
  for (int ip = 2; ip <= np + 1; ip++) esup2[ip - 1] += esup2[ip - 2];
  for (int ie = 1; ie <= nt; ie++)
    for (int in = 1; in <= 3; in++) {
      int ipoin = ELEM(in, ie);
      int istor = esup2[ipoin - 1] + 1;
      esup2[ipoin - 1] = istor;
      o->esup1[istor - 1] = ie;
    }
  for (int ip = np + 1; ip >= 2; ip--) esup2[ip - 1] = esup2[ip - 2];
  esup2[0] = 0;
}

static void pt_surr_pt(orc_t *o) {
  int np = o->s.np;
  int32_t *lpoin = (int32_t *)calloc((size_t)np + 1, sizeof(int32_t));
  o->psup2[0] = 0;
  int istor = 0;
  for (int ipoin = 1; ipoin <= np; ipoin++) {
    for (int iesup = o->esup2[ipoin - 1] + 1; iesup <= o->esup2[ipoin]; iesup++) {
      int ie = o->esup1[iesup - 1];
      for (int in = 1; in <= 3; in++) {
        int jpoin = ELEM(in, ie);
        if (jpoin != ipoin && lpoin[jpoin - 1] != ipoin) {
          istor++;
          o->psup1[istor - 1] = jpoin;
          lpoin[jpoin - 1] = ipoin;
        }
      }
    }
    o->psup2[ipoin] = istor;
  }
  free(lpoin);
}

static void create_edge(orc_t *o) {
  int ne = 0;
  for (int ipoin = 1; ipoin <= o->s.np; ipoin++)
    for (int ip = o->psup2[ipoin - 1] + 1; ip <= o->psup2[ipoin]; ip++) {
      int neigh = o->psup1[ip - 1];
      if (neigh > ipoin) {
        ne++;
        EDGE(1, ne) = ipoin;
        EDGE(2, ne) = neigh;
      }
    }
  o->s.ne = ne;
}

static void el_surr_edge(orc_t *o) {
  for (int i = 1; i <= o->s.ne; i++) {
    EDNEIGH(1, i) = 0;
    EDNEIGH(2, i) = 0;
    int n1 = EDGE(1, i), n2 = EDGE(2, i);
    for (int jt = o->esup2[n1 - 1] + 1; jt <= o->esup2[n1]; jt++) {
      int el = o->esup1[jt - 1];
      if ((n1 == ELEM(1, el) && n2 == ELEM(2, el)) ||
          (n1 == ELEM(2, el) && n2 == ELEM(3, el)) ||
          (n1 == ELEM(3, el) && n2 == ELEM(1, el)))
        EDNEIGH(1, i) = el;
      if ((n2 == ELEM(1, el) && n1 == ELEM(2, el)) ||
          (n2 == ELEM(2, el) && n1 == ELEM(3, el)) ||
          (n2 == ELEM(3, el) && n1 == ELEM(1, el)))
        EDNEIGH(2, i) = el;
    }
    if (EDNEIGH(1, i) == 0) {
      EDNEIGH(1, i) = EDNEIGH(2, i);
      EDNEIGH(2, i) = 0;
      int tmp = EDGE(1, i);
      EDGE(1, i) = EDGE(2, i);
      EDGE(2, i) = tmp;
    }
  }
}

static void circumcenter(orc_t *o, int el) {
  int n1 = ELEM(1, el), n2 = ELEM(2, el), n3 = ELEM(3, el);
  double x1 = COORD(1, n1), y1 = COORD(2, n1);
  double x2 = COORD(1, n2), y2 = COORD(2, n2);
  double x3 = COORD(1, n3), y3 = COORD(2, n3);
  double dx1 = x2 - x3, dy1 = y2 - y3, l1 = sq(dx1) + sq(dy1);
  double dx2 = x3 - x1, dy2 = y3 - y1, l2 = sq(dx2) + sq(dy2);
  double dx3 = x1 - x2, dy3 = y1 - y2, l3 = sq(dx3) + sq(dy3);
  double beta1 = dmax1(0.0, l2 + l3 - l1);
  double beta2 = dmax1(0.0, l3 + l1 - l2);
  double beta3 = dmax1(0.0, l1 + l2 - l3);
  double det = (x2 - x1) * (y3 - y1) - (x3 - x1) * (y2 - y1);
  double b1 = 0.5 * ((x2 - x1) * (x2 + x1) + (y2 - y1) * (y2 + y1));
  double b2 = 0.5 * ((x3 - x1) * (x3 + x1) + (y3 - y1) * (y3 + y1));
  double xc = ((y3 - y1) * b1 - (y2 - y1) * b2) / det;
  double yc = (-(x3 - x1) * b1 + (x2 - x1) * b2) / det;
  if (beta1 == 0.0) {
    TCOORD(1, el) = 0.5 * (x2 + x3);
    TCOORD(2, el) = 0.5 * (y2 + y3);
  } else if (beta2 == 0.0) {
    TCOORD(1, el) = 0.5 * (x3 + x1);
    TCOORD(2, el) = 0.5 * (y3 + y1);
  } else if (beta3 == 0.0) {
    TCOORD(1, el) = 0.5 * (x1 + x2);
    TCOORD(2, el) = 0.5 * (y1 + y2);
  } else {
    TCOORD(1, el) = xc;
    TCOORD(2, el) = yc;
  }
}

static void tri_coord(orc_t *o) {
  for (int i = 1; i <= o->s.nt; i++) {
    if (o->in.cell_type == MEDIAN) {
      int n1 = ELEM(1, i), n2 = ELEM(2, i), n3 = ELEM(3, i);
      TCOORD(1, i) = (COORD(1, n1) + COORD(1, n2) + COORD(1, n3)) / 3.0;
      TCOORD(2, i) = (COORD(2, n1) + COORD(2, n2) + COORD(2, n3)) / 3.0;
    } else {
      circumcenter(o, i);
    }
  }
}

static int areas(orc_t *o) {
  int np = o->s.np, nt = o->s.nt;
  for (int i = 1; i <= nt; i++) {           /* tri_area */
    int n1 = ELEM(1, i), n2 = ELEM(2, i), n3 = ELEM(3, i);
    double dx1 = COORD(1, n2) - COORD(1, n1);
    double dy1 = COORD(2, n2) - COORD(2, n1);
    double dx2 = COORD(1, n3) - COORD(1, n1);
    double dy2 = COORD(2, n3) - COORD(2, n1);
    V1(o->elarea, i) = 0.5 * (dx1 * dy2 - dx2 * dy1);
  }
  for (int i = 1; i <= np; i++) V1(o->mcarea, i) = 0.0;
  for (int i = 1; i <= nt; i++) {           /* mc_area */
    double area3 = V1(o->elarea, i) / 3.0;
    V1(o->mcarea, ELEM(1, i)) += area3;
    V1(o->mcarea, ELEM(2, i)) += area3;
    V1(o->mcarea, ELEM(3, i)) += area3;
  }
  if (o->in.cell_type == MEDIAN) {
    for (int i = 1; i <= np; i++) V1(o->cvarea, i) = V1(o->mcarea, i);
    return ORC_OK;
  }
  for (int i = 1; i <= np; i++) V1(o->cvarea, i) = 0.0;   /* cvareas_bc */
  for (int i = 1; i <= nt; i++) {
    for (int j = 1; j <= 3; j++) {
      int n1 = ELEM(j, i);
      int n2 = (j == 1) ? ELEM(3, i) : ELEM(j - 1, i);
      int n3 = (j == 3) ? ELEM(1, i) : ELEM(j + 1, i);
      double x[5], y[5];
      x[0] = COORD(1, n1);
      y[0] = COORD(2, n1);
      x[1] = 0.5 * (COORD(1, n1) + COORD(1, n3));
      y[1] = 0.5 * (COORD(2, n1) + COORD(2, n3));
      x[2] = TCOORD(1, i);
      y[2] = TCOORD(2, i);
      x[3] = 0.5 * (COORD(1, n1) + COORD(1, n2));
      y[3] = 0.5 * (COORD(2, n1) + COORD(2, n2));
      x[4] = x[0];
      y[4] = y[0];
      double area = 0.0;
      for (int k = 0; k < 4; k++) area = area + x[k] * y[k + 1] - x[k + 1] * y[k];
      if (area < 0.0) return ORC_ERR_GEOMETRY;
      area = 0.5 * area;
      V1(o->cvarea, n1) += area;
    }
  }
  return ORC_OK;
}

static void wall_dist_core(int np, int ne, const double *coord, const int32_t *edge,
                           const int32_t *ptype, int bugcompat, double *wd) {
  /* wall_dist.f:16-61 */
  int nbe = 0;
  int32_t *sedge = (int32_t *)malloc(sizeof(int32_t) * (size_t)(ne > 0 ? ne : 1));
  for (int i = 1; i <= ne; i++) {
    int n1 = edge[2 * (i - 1)], n2 = edge[2 * (i - 1) + 1];
    if (ptype[n1 - 1] == SOLID && ptype[n2 - 1] == SOLID) sedge[nbe++] = i;
  }
#define C_(k, i) coord[2 * ((i) - 1) + (k) - 1]
  for (int i = 1; i <= np; i++) {
    double w = 1.0e10;
    for (int j = 0; j < nbe; j++) {
      int je = sedge[j];
      int n1 = edge[2 * (je - 1)], n2 = edge[2 * (je - 1) + 1];
      double dx1 = C_(1, n1) - C_(1, i);
      double dy1 = C_(2, n1) - C_(2, i);
      double ds1 = sqrt(sq(dx1) + sq(dy1));
      w = dmin1(w, ds1);
      double dx2 = C_(1, n2) - C_(1, i);
      double dy2 = C_(2, n2) - C_(2, i);
      double ds2 = sqrt(sq(dx2) + sq(dy2));
      w = dmin1(w, ds2);
      double dx3 = C_(1, n2) - C_(1, n1);
      double dy3 = bugcompat ? (C_(1, n2) - C_(1, n1)) : (C_(2, n2) - C_(2, n1));
      double dl2 = sq(dx3) + sq(dy3);
      double xi = -(dx1 * dx3 + dy1 * dy3) / dl2;
      if (xi >= 0.0 && xi <= 1.0) {
        double xp = C_(1, n1) + xi * dx3;
        double yp = C_(2, n1) + xi * dy3;
        double dsperp = sqrt(sq(C_(1, i) - xp) + sq(C_(2, i) - yp));
        w = dmin1(w, dsperp);
      }
    }
    if (ptype[i - 1] == SOLID) w = 0.0;
    wd[i - 1] = w;
  }
  /* wall_dist.f:90-92 */
  for (int i = 1; i <= np; i++)
    if (ptype[i - 1] == SOLID) wd[i - 1] = 1.0;
#undef C_
  free(sedge);
}

static void wall_dist(orc_t *o) {
  wall_dist_core(o->s.np, o->s.ne, o->coord, o->edge, o->ptype, o->in.bugcompat, o->wd);
  /* wall_dist.f:63-73: wd1 uses wd before the solid points are reset to 1;
   * those neighbours are non-solid, so the final wd serves as well. */
  for (int i = 1; i <= o->s.nsp; i++) {
    int n1 = V1(o->spts, i);
    double w = 1.0e10;
    for (int j = o->psup2[n1 - 1] + 1; j <= o->psup2[n1]; j++) {
      int n2 = o->psup1[j - 1];
      if (V1(o->ptype, n2) != SOLID) w = dmin1(w, V1(o->wd, n2));
    }
    V1(o->wd1, i) = w;
  }
}

static int flength(orc_t *o) {
  for (int i = 1; i <= o->s.ne; i++) {
    int n1 = EDGE(1, i), n2 = EDGE(2, i);
    int p1 = EDNEIGH(1, i), p2 = EDNEIGH(2, i);
    double x1, y1, x2, y2;
    if (p1 != 0) {
      x1 = TCOORD(1, p1);
      y1 = TCOORD(2, p1);
    } else {
      return ORC_ERR_GEOMETRY;
    }
    if (p2 != 0) {
      x2 = TCOORD(1, p2);
      y2 = TCOORD(2, p2);
    } else {
      x2 = 0.5 * (COORD(1, n1) + COORD(1, n2));
      y2 = 0.5 * (COORD(2, n1) + COORD(2, n2));
    }
    DS(1, i) = -(y2 - y1);
    DS(2, i) = (x2 - x1);
  }
  for (int i = 1; i <= o->s.np; i++) {
    DSB(1, i) = 0.0;
    DSB(2, i) = 0.0;
  }
  for (int i = 1; i <= o->s.ne; i++) {
    int n1 = EDGE(1, i), n2 = EDGE(2, i);
    if (EDNEIGH(1, i) * EDNEIGH(2, i) == 0) {
      double nx = COORD(2, n2) - COORD(2, n1);
      double ny = -(COORD(1, n2) - COORD(1, n1));
      DSB(1, n1) += 0.5 * nx;
      DSB(2, n1) += 0.5 * ny;
      DSB(1, n2) += 0.5 * nx;
      DSB(2, n2) += 0.5 * ny;
    }
  }
  return ORC_OK;
}

static void reorder_edges(orc_t *o) {
  o->s.netot = o->s.ne;
  if (o->in.cell_type == BARTH) {
    int ecount = 0;
    for (int i = 1; i <= o->s.ne; i++) {
      double length = sqrt(sq(DS(1, i)) + sq(DS(2, i)));
      if (length != 0.0) V1(o->iedge, ++ecount) = i;
    }
    o->s.ne = ecount;
  } else {
    for (int i = 1; i <= o->s.ne; i++) V1(o->iedge, i) = i;
  }
}

void orc_dtlength(int32_t np, int32_t nt, const double *coord, const int32_t *elem,
                  const double *elarea, double *drmin) {
#define C_(k, i) coord[2 * ((i) - 1) + (k) - 1]
  for (int ip = 1; ip <= np; ip++) drmin[ip - 1] = 1.0e15;
  for (int it = 1; it <= nt; it++) {
    int n1 = elem[3 * (it - 1)], n2 = elem[3 * (it - 1) + 1], n3 = elem[3 * (it - 1) + 2];
    double ea = elarea[it - 1];
    double dx1 = C_(1, n2) - C_(1, n3), dy1 = C_(2, n2) - C_(2, n3);
    double dr1 = sqrt(sq(dx1) + sq(dy1)), h1 = 2.0 * ea / dr1;
    double dx2 = C_(1, n3) - C_(1, n1), dy2 = C_(2, n3) - C_(2, n1);
    double dr2 = sqrt(sq(dx2) + sq(dy2)), h2 = 2.0 * ea / dr2;
    double dx3 = C_(1, n1) - C_(1, n2), dy3 = C_(2, n1) - C_(2, n2);
    double dr3 = sqrt(sq(dx3) + sq(dy3)), h3 = 2.0 * ea / dr3;
    drmin[n1 - 1] = dmin1(h1, drmin[n1 - 1]);
    drmin[n2 - 1] = dmin1(h2, drmin[n2 - 1]);
    drmin[n3 - 1] = dmin1(h3, drmin[n3 - 1]);
  }
#undef C_
}

void orc_wall_dist(int32_t np, int32_t ne, const double *coord, const int32_t *edge,
                   const int32_t *ptype, int32_t bugcompat, double *wd) {
  wall_dist_core(np, ne, coord, edge, ptype, bugcompat, wd);
}

static void make_bdedges(orc_t *o) {
  int nswe = 0, nffe = 0, netot = o->s.netot;
  int32_t *swedge = (int32_t *)malloc(sizeof(int32_t) * (size_t)netot);
  int32_t *ffedge = (int32_t *)malloc(sizeof(int32_t) * (size_t)netot);
  for (int i = 1; i <= netot; i++) {
    if (EDNEIGH(1, i) * EDNEIGH(2, i) != 0) continue;
    int n1 = EDGE(1, i), n2 = EDGE(2, i);
    if (V1(o->ptype, n1) == SOLID && V1(o->ptype, n2) == SOLID) swedge[nswe++] = i;
    if (V1(o->ptype, n1) == FARFIELD && V1(o->ptype, n2) == FARFIELD) ffedge[nffe++] = i;
  }
  int ec = 0;
  o->s.nswe1 = 1;
  for (int i = 0; i < nswe; i++) V1(o->beindx, ++ec) = swedge[i];
  o->s.nswe2 = ec;
  o->s.nffe1 = ec + 1;
  for (int i = 0; i < nffe; i++) V1(o->beindx, ++ec) = ffedge[i];
  o->s.nffe2 = ec;
  o->s.nbe = ec;
  free(swedge);
  free(ffedge);
}

static int geom_stat(orc_t *o) {
  double minel = 1.0e8, mincv = 1.0e8;
  for (int i = 1; i <= o->s.nt; i++) minel = dmin1(minel, V1(o->elarea, i));
  if (minel <= 0.0) return ORC_ERR_GEOMETRY;
  for (int i = 1; i <= o->s.np; i++) mincv = dmin1(mincv, V1(o->cvarea, i));
  if (mincv <= 0.0) return ORC_ERR_GEOMETRY;
  return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* gradients: green_gauss.f                                             */
/* ------------------------------------------------------------------ */
static void tri_gg(orc_t *o, int n1, int n2, int n3, double dbxx[3], double dbyy[3],
                   double dxt[4], double dyt[4]) {
  dbxx[0] = COORD(2, n2) - COORD(2, n3);
  dbxx[1] = COORD(2, n3) - COORD(2, n1);
  dbxx[2] = COORD(2, n1) - COORD(2, n2);
  dbyy[0] = COORD(1, n3) - COORD(1, n2);
  dbyy[1] = COORD(1, n1) - COORD(1, n3);
  dbyy[2] = COORD(1, n2) - COORD(1, n1);
  for (int k = 1; k <= NVAR; k++) {
    dxt[k - 1] = PRIM(k, n1) * dbxx[0] + PRIM(k, n2) * dbxx[1] + PRIM(k, n3) * dbxx[2];
    dyt[k - 1] = PRIM(k, n1) * dbyy[0] + PRIM(k, n2) * dbyy[1] + PRIM(k, n3) * dbyy[2];
    QX(k, n1) = QX(k, n1) + dxt[k - 1];
    QX(k, n2) = QX(k, n2) + dxt[k - 1];
    QX(k, n3) = QX(k, n3) + dxt[k - 1];
    QY(k, n1) = QY(k, n1) + dyt[k - 1];
    QY(k, n2) = QY(k, n2) + dyt[k - 1];
    QY(k, n3) = QY(k, n3) + dyt[k - 1];
  }
}

static void tri_visc(orc_t *o, int jt, int n1, int n2, int n3, const double dbxx[3],
                     const double dbyy[3], const double dxt[4], const double dyt[4]) {
  const orc_scalars *s = &o->s;
  double n2b3 = 2.0 / 3.0;
  double en1 = PRIM(4, n1) / PRIM(1, n1);
  double en2 = PRIM(4, n2) / PRIM(1, n2);
  double en3 = PRIM(4, n3) / PRIM(1, n3);
  double ext = en1 * dbxx[0] + en2 * dbxx[1] + en3 * dbxx[2];
  double eyt = en1 * dbyy[0] + en2 * dbyy[1] + en3 * dbyy[2];
  double um = (PRIM(2, n1) + PRIM(2, n2) + PRIM(2, n3)) / 3.0;
  double vm = (PRIM(3, n1) + PRIM(3, n2) + PRIM(3, n3)) / 3.0;
  double mut = (V1(o->mu, n1) + V1(o->mu, n2) + V1(o->mu, n3)) / 3.0;
  double mult = (V1(o->mul, n1) + V1(o->mul, n2) + V1(o->mul, n3)) / 3.0;
  double prim5t = (V1(o->nut, n1) + V1(o->nut, n2) + V1(o->nut, n3)) / 3.0;
  double rhot = (PRIM(1, n1) + PRIM(1, n2) + PRIM(1, n3)) / 3.0;
  double chi = prim5t * rhot / mult;
  double chi3 = cube(chi);
  double fv1 = chi3 / (chi3 + s->cv11);
  double txx = n2b3 * mut * (2.0 * dxt[1] - dyt[2]);
  double txy = mut * (dyt[1] + dxt[2]);
  double tyy = n2b3 * mut * (2.0 * dyt[2] - dxt[1]);
  double gpr = s->gamma * (mult / s->prandtl + rhot * prim5t * fv1 / s->prandtl_turb) / s->gamma1;
  double efx = txx * um + txy * vm + gpr * ext;
  double efy = txy * um + tyy * vm + gpr * eyt;
  double areat = 0.25 / V1(o->elarea, jt);
  int nn[3] = {n1, n2, n3};
  for (int j = 0; j < 3; j++) {
    int n = nn[j];
    RES(2, n) = RES(2, n) + (txx * dbxx[j] + txy * dbyy[j]) * areat;
    RES(3, n) = RES(3, n) + (txy * dbxx[j] + tyy * dbyy[j]) * areat;
    RES(4, n) = RES(4, n) + (efx * dbxx[j] + efy * dbyy[j]) * areat;
  }
}

static void green_gauss(orc_t *o, int visc) {
  double n1b6 = 1.0 / 6.0;
  for (int is = 1; is <= o->s.np; is++)
    for (int iv = 1; iv <= NVAR; iv++) {
      QX(iv, is) = 0.0;
      QY(iv, is) = 0.0;
    }
  for (int jt = 1; jt <= o->s.nt; jt++) {
    int n1 = ELEM(1, jt), n2 = ELEM(2, jt), n3 = ELEM(3, jt);
    double dbxx[3], dbyy[3], dxt[4], dyt[4];
    tri_gg(o, n1, n2, n3, dbxx, dbyy, dxt, dyt);
    if (visc) tri_visc(o, jt, n1, n2, n3, dbxx, dbyy, dxt, dyt);
  }
  for (int is = 1; is <= o->s.np; is++) {
    double ais = n1b6 / V1(o->mcarea, is);
    for (int k = 1; k <= NVAR; k++) {
      QX(k, is) = QX(k, is) * ais;
      QY(k, is) = QY(k, is) * ais;
    }
  }
}

/* ------------------------------------------------------------------ */
/* recon.f                                                              */
/* ------------------------------------------------------------------ */
static double limit_albada(double ul, double ur) {
  if (ul * ur <= 0.0) return 0.0;
  double top = (sq(ul) + EPSILON) * ur + (sq(ur) + EPSILON) * ul;
  double bot = sq(ul) + sq(ur) + 2.0 * EPSILON;
  return top / bot;
}

static void recon(const orc_t *o, int e1, int e2, double priml[4], double primr[4]) {
  const orc_scalars *s = &o->s;
  double dx = COORD(1, e2) - COORD(1, e1);
  double dy = COORD(2, e2) - COORD(2, e1);
  for (int i = 1; i <= NVAR; i++) {
    double dqp = PRIM(i, e2) - PRIM(i, e1);
    if (o->in.ilimit == 1) {
      double dql = s->albada21 * (dx * QX(i, e1) + dy * QY(i, e1)) + s->albada22 * dqp;
      double si = limit_albada(dql, dqp);
      priml[i - 1] = PRIM(i, e1) + 0.5 * si;
      double dqr = s->albada21 * (dx * QX(i, e2) + dy * QY(i, e2)) + s->albada22 * dqp;
      double sj = limit_albada(dqr, dqp);
      primr[i - 1] = PRIM(i, e2) - 0.5 * sj;
    } else {
      double dql = dx * QX(i, e1) + dy * QY(i, e1);
      double si = s->albada11 * dql + s->albada12 * dqp;
      priml[i - 1] = PRIM(i, e1) + 0.5 * si;
      double dqr = dx * QX(i, e2) + dy * QY(i, e2);
      double sj = s->albada11 * dqr + s->albada12 * dqp;
      primr[i - 1] = PRIM(i, e2) - 0.5 * sj;
    }
  }
}

/* ------------------------------------------------------------------ */
/* interior fluxes: roe_flux.f, kfvs_flux.f, hllc_flux.f                */
/* ------------------------------------------------------------------ */
static void roe_flux(orc_t *o, const double ds[2], const double priml[4],
                     const double primr[4], double flux[4]) {
  const double GAMMA = o->s.gamma, GAMMA1 = o->s.gamma1;
  double length = sqrt(sq(ds[0]) + sq(ds[1]));
  double ct = ds[0] / length, st = ds[1] / length;
  double rl = priml[0], ul = priml[1], vl = priml[2], pl = priml[3];
  double al2 = GAMMA * pl / rl;
  double ql2 = sq(ul) + sq(vl);
  double hl = al2 / GAMMA1 + 0.5 * ql2;
  double rr = primr[0], ur = primr[1], vr = primr[2], pr = primr[3];
  double ar2 = GAMMA * pr / rr;
  double qr2 = sq(ur) + sq(vr);
  double hr = ar2 / GAMMA1 + 0.5 * qr2;
  double unl = ul * ct + vl * st;
  double Fc[4];
  Fc[0] = rl * unl;
  Fc[1] = pl * ct + rl * ul * unl;
  Fc[2] = pl * st + rl * vl * unl;
  Fc[3] = rl * hl * unl;
  double rl12 = sqrt(rl), rr12 = sqrt(rr);
  double rd = 1.0 / (rl12 + rr12);
  double ua = (ul * rl12 + ur * rr12) * rd;
  double va = (vl * rl12 + vr * rr12) * rd;
  double ha = (hl * rl12 + hr * rr12) * rd;
  double qa2 = sq(ua) + sq(va);
  double aa2 = GAMMA1 * (ha - 0.5 * qa2);
  double aa;
  if (aa2 > 0.0) {
    aa = sqrt(aa2);
  } else {
    if (!o->s.err) o->s.err = ORC_ERR_ROE_SONIC;
    aa = sqrt(aa2);
  }
  double una = ua * ct + va * st;
  double vna = -ua * st + va * ct;
  double l1 = dmin1(una - aa, 0.0);
  double l2 = dmin1(una, 0.0);
  double l3 = l2;
  double l4 = dmin1(una + aa, 0.0);
  double du1 = rr - rl;
  double du2 = rr * ur - rl * ul;
  double du3 = rr * vr - rl * vl;
  double du4 = (pr - pl) / GAMMA1 + 0.5 * (rr * qr2 - rl * ql2);
  double m1 = (ct * du2 + st * du3 - una * du1) / aa;
  double m2 = GAMMA1 * (du4 - ua * du2 - va * du3 + qa2 * du1) / sq(aa);
  double a4 = 0.5 * (m1 + m2);
  double a1 = 0.5 * (m2 - m1);
  double a3 = du1 - a1 - a4;
  double a2 = (st * du2 - ct * du3 + vna * du1) / aa;
  double a1l1 = a1 * l1, a2l2 = a2 * l2, a3l3 = a3 * l3, a4l4 = a4 * l4;
  double aact = aa * ct, aast = aa * st;
  double Fd[4];
  Fd[0] = a1l1 + a3l3 + a4l4;
  Fd[1] = a1l1 * (ua - aact) + a2l2 * aa * st + a3l3 * ua + a4l4 * (ua + aact);
  Fd[2] = a1l1 * (va - aast) - a2l2 * aa * ct + a3l3 * va + a4l4 * (va + aast);
  Fd[3] = a1l1 * (ha - una * aa) + a2l2 * aa * vna + a3l3 * 0.5 * qa2 + a4l4 * (ha + una * aa);
  for (int i = 0; i < 4; i++) flux[i] = (Fc[i] + Fd[i]) * length;
}

static void kfvs_flux(orc_t *o, const double ds[2], const double priml[4],
                      const double primr[4], double flux[4]) {
  const double GAMMA1 = o->s.gamma1, M_PI_ = o->s.pi;
  double length = sqrt(sq(ds[0]) + sq(ds[1]));
  double ct = ds[0] / length, st = ds[1] / length;
  double rl = priml[0], ul = priml[1], vl = priml[2], pl = priml[3];
  double ql2 = sq(ul) + sq(vl);
  double el = pl / GAMMA1 + 0.5 * rl * ql2;
  double rr = primr[0], ur = primr[1], vr = primr[2], pr = primr[3];
  double qr2 = sq(ur) + sq(vr);
  double er = pr / GAMMA1 + 0.5 * rr * qr2;
  double unl = ul * ct + vl * st;
  double unr = ur * ct + vr * st;
  double vnl = -ul * st + vl * ct;
  double vnr = -ur * st + vr * ct;
  double betal = 0.5 * rl / pl;
  double sl = unl * sqrt(betal);
  double Al = 0.5 * (1.0 + erf(sl));
  double Bl = 0.5 * exp(-sq(sl)) / sqrt(M_PI_ * betal);
  double Fp[4], Fm[4], Ff[4];
  Fp[0] = rl * (unl * Al + Bl);
  Fp[1] = (pl + rl * sq(unl)) * Al + rl * unl * Bl;
  Fp[2] = rl * (unl * Al + Bl) * vnl;
  Fp[3] = (el + pl) * unl * Al + (el + 0.5 * pl) * Bl;
  double betar = 0.5 * rr / pr;
  double sr = unr * sqrt(betar);
  double Ar = 0.5 * (1.0 - erf(sr));
  double Br = 0.5 * exp(-sq(sr)) / sqrt(M_PI_ * betar);
  Fm[0] = rr * (unr * Ar - Br);
  Fm[1] = (pr + rr * sq(unr)) * Ar - rr * unr * Br;
  Fm[2] = rr * (unr * Ar - Br) * vnr;
  Fm[3] = (er + pr) * unr * Ar - (er + 0.5 * pr) * Br;
  for (int i = 0; i < 4; i++) Ff[i] = Fp[i] + Fm[i];
  flux[0] = Ff[0] * length;
  flux[1] = (ct * Ff[1] - st * Ff[2]) * length;
  flux[2] = (st * Ff[1] + ct * Ff[2]) * length;
  flux[3] = Ff[3] * length;
}

static void hllc_flux(orc_t *o, const double ds[2], const double priml[4],
                      const double primr[4], double flux[4]) {
  const double gamma = o->s.gamma, GAMMA1 = o->s.gamma1;
  double length = sqrt(sq(ds[0]) + sq(ds[1]));
  double ct = ds[0] / length, st = ds[1] / length;
  double rl = priml[0];
  double ul = priml[1] * ct + priml[2] * st;
  double vl = -priml[1] * st + priml[2] * ct;
  double pl = priml[3];
  double al = sqrt(gamma * pl / rl);
  double El = pl / GAMMA1 + 0.5 * rl * (sq(ul) + sq(vl));
  double rr = primr[0];
  double ur = primr[1] * ct + primr[2] * st;
  double vr = -primr[1] * st + primr[2] * ct;
  double pr = primr[3];
  double ar = sqrt(gamma * pr / rr);
  double Er = pr / GAMMA1 + 0.5 * rr * (sq(ur) + sq(vr));
  double rbar = 0.5 * (rl + rr);
  double abar = 0.5 * (al + ar);
  double Ppv = 0.5 * (pl + pr - (ur - ul) * rbar * abar);
  double Upv = 0.5 * (ul + ur - (pr - pl) / (rbar * abar));
  double prmax, prmin;
  if (pl > pr) {
    prmax = pl;
    prmin = pr;
  } else {
    prmax = pr;
    prmin = pl;
  }
  double Q = prmax / prmin;
  double pstar, ustar;
  if (Q < 2.0 && prmin < Ppv && Ppv < prmax) {
    pstar = Ppv;
    ustar = Upv;
  } else if (Ppv < prmin) {
    double z = 0.5 * (gamma - 1.0) / gamma;
    double a1 = al + ar - 0.5 * (gamma - 1.0) * (ur - ul);
    double a2 = al / pow(pl, z) + ar / pow(pr, z);
    pstar = pow(a1 / a2, 1.0 / z);
    double Plr = pow(pl / pr, z);
    double b1 = Plr * ul / al + ur / ar + 2.0 * (Plr - 1.0) / (gamma - 1.0);
    double b2 = Plr / al + 1.0 / ar;
    ustar = b1 / b2;
  } else {
    double po = dmax1(0.0, Ppv);
    double Ml = 2.0 / (gamma + 1.0) / rl;
    double Nl = (gamma - 1.0) * pl / (gamma + 1.0);
    double gl = sqrt(Ml / (po + Nl));
    double Mr = 2.0 / (gamma + 1.0) / rr;
    double Nr = (gamma - 1.0) * pr / (gamma + 1.0);
    double gr = sqrt(Mr / (po + Nr));
    double a1 = gl * pl + gr * pr - (ur - ul);
    double a2 = gl + gr;
    pstar = a1 / a2;
    ustar = 0.5 * (ul + ur + (pstar - pr) * gr - (pstar - pl) * gl);
  }
  double ql, qr;
  if (pstar <= pl) ql = 1.0;
  else ql = sqrt(1.0 + 0.5 * (gamma + 1.0) * (pstar / pl - 1.0) / gamma);
  if (pstar <= pr) qr = 1.0;
  else qr = sqrt(1.0 + 0.5 * (gamma + 1.0) * (pstar / pr - 1.0) / gamma);
  double Sl = ul - al * ql;
  double Ss = ustar;
  double Sr = ur + ar * qr;
  if (0.0 <= Sl) {
    flux[0] = rl * ul;
    flux[1] = pl + rl * sq(ul);
    flux[2] = rl * ul * vl;
    flux[3] = (El + pl) * ul;
  } else if (Sl <= 0.0 && 0.0 <= Ss) {
    double fl[4], du[4];
    fl[0] = rl * ul;
    fl[1] = pl + rl * sq(ul);
    fl[2] = rl * ul * vl;
    fl[3] = (El + pl) * ul;
    double fact = rl * (Sl - ul) / (Sl - Ss);
    du[0] = fact - rl;
    du[1] = fact * Ss - rl * ul;
    du[2] = fact * vl - rl * vl;
    double t1 = El / rl + (Ss - ul) * (Ss + pl / rl / (Sl - ul));
    du[3] = fact * t1 - El;
    for (int i = 0; i < 4; i++) flux[i] = fl[i] + Sl * du[i];
  } else if (Ss <= 0.0 && 0.0 <= Sr) {
    double fr[4], du[4];
    fr[0] = rr * ur;
    fr[1] = pr + rr * sq(ur);
    fr[2] = rr * ur * vr;
    fr[3] = (Er + pr) * ur;
    double fact = rr * (Sr - ur) / (Sr - Ss);
    du[0] = fact - rr;
    du[1] = fact * Ss - rr * ur;
    du[2] = fact * vr - rr * vr;
    double t1 = Er / rr + (Ss - ur) * (Ss + pr / rr / (Sr - ur));
    du[3] = fact * t1 - Er;
    for (int i = 0; i < 4; i++) flux[i] = fr[i] + Sr * du[i];
  } else {
    flux[0] = rr * ur;
    flux[1] = pr + rr * sq(ur);
    flux[2] = rr * ur * vr;
    flux[3] = (Er + pr) * ur;
  }
  if (!o->in.bugcompat) {
    /* hllc_flux.f:149-154 adds the (normal, tangential) momentum flux as if
     * it were (x, y); the corrected form rotates it back as kfvs_flux.f:71-72 */
    double fn = flux[1], ft = flux[2];
    flux[1] = ct * fn - st * ft;
    flux[2] = st * fn + ct * ft;
  }
  for (int i = 0; i < 4; i++) flux[i] = flux[i] * length;
}

/* ------------------------------------------------------------------ */
/* boundary fluxes: solid_flux.f, farfield_flux.f                       */
/* ------------------------------------------------------------------ */
static void solid_flux(orc_t *o, int n1, int n2) {
  double sx = 0.5 * (COORD(2, n2) - COORD(2, n1));
  double sy = -0.5 * (COORD(1, n2) - COORD(1, n1));
  double p1 = 0.75 * PRIM(4, n1) + 0.25 * PRIM(4, n2);
  double p2 = 0.25 * PRIM(4, n1) + 0.75 * PRIM(4, n2);
  RES(2, n1) = RES(2, n1) + p1 * sx;
  RES(3, n1) = RES(3, n1) + p1 * sy;
  RES(2, n2) = RES(2, n2) + p2 * sx;
  RES(3, n2) = RES(3, n2) + p2 * sy;
}

static void farfield_flux(orc_t *o, int n1, int n2) {
  const orc_scalars *s = &o->s;
  const double GAMMA = s->gamma, gamma1 = s->gamma1;
  double x1[2] = {COORD(1, n1), COORD(2, n1)}, x2[2] = {COORD(1, n2), COORD(2, n2)};
  double uinf, vinf, q2inf, pinf, rinf;
  if (s->mach_inf < 1.0 && o->in.vortex == 1) {
    double dx = 0.5 * (x1[0] + x2[0]) - s->xref;
    double dy = 0.5 * (x1[1] + x2[1]) - s->yref;
    double dref = sqrt(sq(dx) + sq(dy));
    double theta = atan2(dy, dx);
    double circ = 0.5 * s->q_inf * s->cl;
    double fact1 = circ * sqrt(1.0 - sq(s->mach_inf));
    double fact2 = 2.0 * s->pi * dref;
    double fact3 = 1.0 - sq(s->mach_inf * sin(theta - s->aoa));
    double fact = fact1 / (fact2 * fact3);
    uinf = s->u_inf + fact * sin(theta);
    vinf = s->v_inf - fact * cos(theta);
    q2inf = sq(uinf) + sq(vinf);
    double fact4 = 1.0 + 0.5 * gamma1 * (sq(s->q_inf) - q2inf) / sq(s->a_inf);
    rinf = s->r_inf * pow(fact4, 1.0 / gamma1);
    pinf = s->p_inf * pow(rinf / s->r_inf, GAMMA);
  } else {
    uinf = s->u_inf;
    vinf = s->v_inf;
    q2inf = sq(uinf) + sq(vinf);
    pinf = s->p_inf;
    rinf = s->r_inf;
  }
  double Uout[4] = {rinf, rinf * uinf, rinf * vinf, pinf / gamma1 + 0.5 * rinf * q2inf};
  double ra = 0.5 * (PRIM(1, n1) + PRIM(1, n2));
  double ua = 0.5 * (PRIM(2, n1) + PRIM(2, n2));
  double va = 0.5 * (PRIM(3, n1) + PRIM(3, n2));
  double pa = 0.5 * (PRIM(4, n1) + PRIM(4, n2));
  double qa2 = sq(ua) + sq(va);
  double aa2 = GAMMA * pa / ra;
  double aa = sqrt(GAMMA * pa / ra);
  double ha = aa2 / gamma1 + 0.5 * qa2;
  double Uin1[4], Uin2[4];
  Uin1[0] = PRIM(1, n1);
  Uin1[1] = PRIM(1, n1) * PRIM(2, n1);
  Uin1[2] = PRIM(1, n1) * PRIM(3, n1);
  Uin1[3] = PRIM(4, n1) / gamma1 + 0.5 * PRIM(1, n1) * (sq(PRIM(2, n1)) + sq(PRIM(3, n1)));
  Uin2[0] = PRIM(1, n2);
  Uin2[1] = PRIM(1, n2) * PRIM(2, n2);
  Uin2[2] = PRIM(1, n2) * PRIM(3, n2);
  Uin2[3] = PRIM(4, n2) / gamma1 + 0.5 * PRIM(1, n2) * (sq(PRIM(2, n2)) + sq(PRIM(3, n2)));
  double ct = (x2[1] - x1[1]);
  double st = -(x2[0] - x1[0]);
  double lent = sqrt(sq(ct) + sq(st));
  ct = ct / lent;
  st = st / lent;
  double una = ua * ct + va * st;
  double vna = -ua * st + va * ct;
  double l1 = una, l2 = una, l3 = una + aa, l4 = una - aa;
  double lp1 = dmax1(l1, 0.0), lp2 = lp1, lp3 = dmax1(l3, 0.0), lp4 = dmax1(l4, 0.0);
  double lm1 = l1 - lp1, lm2 = l2 - lp2, lm3 = l3 - lp3, lm4 = l4 - lp4;
  double T[4][4], S[4][4], Tp[4][4], Tm[4][4], jacp[4][4], jacm[4][4];
  double t1 = 0.5 * ra / aa;
  double m2 = qa2 / aa2;
  T[0][0] = 1.0;      T[1][0] = ua;       T[2][0] = va;       T[3][0] = 0.5 * qa2;
  T[0][1] = 0.0;      T[1][1] = ra * st;  T[2][1] = -ra * ct; T[3][1] = -ra * vna;
  T[0][2] = t1;       T[1][2] = t1 * (ua + aa * ct);
  T[2][2] = t1 * (va + aa * st);          T[3][2] = t1 * (ha + aa * una);
  T[0][3] = t1;       T[1][3] = t1 * (ua - aa * ct);
  T[2][3] = t1 * (va - aa * st);          T[3][3] = t1 * (ha - aa * una);
  t1 = 0.5 * gamma1 * m2 * aa / ra;
  double t2 = una / ra, t3 = gamma1 * ua / aa, t4 = gamma1 * va / aa, t5 = gamma1 / (ra * aa);
  S[0][0] = 1.0 - 0.5 * gamma1 * m2;
  S[1][0] = vna / ra;
  S[2][0] = t1 - t2;
  S[3][0] = t1 + t2;
  S[0][1] = t3 / aa;
  S[1][1] = st / ra;
  S[2][1] = (ct - t3) / ra;
  S[3][1] = -(ct + t3) / ra;
  S[0][2] = t4 / aa;
  S[1][2] = -ct / ra;
  S[2][2] = (st - t4) / ra;
  S[3][2] = -(st + t4) / ra;
  S[0][3] = -gamma1 / aa2;
  S[1][3] = 0.0;
  S[2][3] = t5;
  S[3][3] = t5;
  for (int i = 0; i < 4; i++) {
    Tp[i][0] = lp1 * T[i][0];
    Tp[i][1] = lp2 * T[i][1];
    Tp[i][2] = lp3 * T[i][2];
    Tp[i][3] = lp4 * T[i][3];
    Tm[i][0] = lm1 * T[i][0];
    Tm[i][1] = lm2 * T[i][1];
    Tm[i][2] = lm3 * T[i][2];
    Tm[i][3] = lm4 * T[i][3];
  }
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) {
      jacp[i][j] = 0.0;
      jacm[i][j] = 0.0;
      for (int k = 0; k < 4; k++) {
        jacp[i][j] = jacp[i][j] + Tp[i][k] * S[k][j];
        jacm[i][j] = jacm[i][j] + Tm[i][k] * S[k][j];
      }
    }
  for (int i = 0; i < 4; i++) {
    double f1 = 0.0, f2 = 0.0;
    for (int j = 0; j < 4; j++) {
      f1 = f1 + jacp[i][j] * Uin1[j] + jacm[i][j] * Uout[j];
      f2 = f2 + jacp[i][j] * Uin2[j] + jacm[i][j] * Uout[j];
    }
    f1 = 0.5 * lent * f1;
    f2 = 0.5 * lent * f2;
    RES(i + 1, n1) = RES(i + 1, n1) + f1;
    RES(i + 1, n2) = RES(i + 1, n2) + f2;
  }
}

/* ------------------------------------------------------------------ */
/* residu.f                                                             */
/* ------------------------------------------------------------------ */
void orc_residu(orc_t *o) {
  int np = o->s.np;
  for (int ip = 1; ip <= np; ip++)
    for (int iv = 1; iv <= NVAR; iv++) RES(iv, ip) = 0.0;
  if (o->in.iflow != INVISCID) {
    sutherland(o);
    viscosity(o);
  }
  green_gauss(o, o->in.iflow != INVISCID);
  for (int i = 1; i <= o->s.ne; i++) {
    int ie = V1(o->iedge, i);
    int e1 = EDGE(1, ie), e2 = EDGE(2, ie);
    double priml[4], primr[4], flux[4], ds[2] = {DS(1, ie), DS(2, ie)};
    recon(o, e1, e2, priml, primr);
    if (o->in.iflux == IROE) roe_flux(o, ds, priml, primr, flux);
    else if (o->in.iflux == IKFVS) kfvs_flux(o, ds, priml, primr, flux);
    else hllc_flux(o, ds, priml, primr, flux);
    for (int k = 1; k <= NVAR; k++) {
      RES(k, e1) = RES(k, e1) + flux[k - 1];
      RES(k, e2) = RES(k, e2) - flux[k - 1];
    }
  }
  for (int i = o->s.nswe1; i <= o->s.nswe2; i++) {
    int ie = V1(o->beindx, i);
    solid_flux(o, EDGE(1, ie), EDGE(2, ie));
  }
  for (int i = o->s.nffe1; i <= o->s.nffe2; i++) {
    int ie = V1(o->beindx, i);
    farfield_flux(o, EDGE(1, ie), EDGE(2, ie));
  }
}

/* ------------------------------------------------------------------ */
/* time stepping: save_old.f, time_step.f, update.f, convert.f          */
/* ------------------------------------------------------------------ */
void orc_save_old(orc_t *o) {
  memcpy(o->prim_old, o->prim, sizeof(double) * NVAR * (size_t)o->s.np);
}

void orc_time_step(orc_t *o) {
  const orc_scalars *s = &o->s;
  for (int i = 1; i <= s->np; i++) {
    double q = sqrt(sq(PRIM(2, i)) + sq(PRIM(3, i)));
    double a = sqrt(s->gamma * PRIM(4, i) / PRIM(1, i));
    double dr = V1(o->drmin, i);
    if (o->in.iflow != INVISCID) {
      double dtv = 2.0 * s->gamma * V1(o->mu, i) / (PRIM(1, i) * s->prandtl);
      V1(o->dt, i) = s->cfl * sq(dr) / (dr * (q + a) + dtv);
    } else {
      V1(o->dt, i) = s->cfl * dr / (q + a);
    }
  }
  double dtg = 1.0e10;
  for (int i = 1; i <= s->np; i++) dtg = dmin1(dtg, V1(o->dt, i));
  o->s.dtglobal = dtg;
}

static void prim2con(const orc_t *o, const double *prim, double con[4]) {
  con[0] = prim[0];
  con[1] = prim[0] * prim[1];
  con[2] = prim[0] * prim[2];
  con[3] = prim[3] / o->s.gamma1 + 0.5 * prim[0] * (sq(prim[1]) + sq(prim[2]));
}

void orc_update(orc_t *o, int32_t irk) {
  const orc_scalars *s = &o->s;
  double a = s->airk[irk - 1], b = s->birk[irk - 1];
  for (int i = 1; i <= s->np; i++) {
    double c0[4], c1[4];
    prim2con(o, &PRIMO(1, i), c0);
    prim2con(o, &PRIM(1, i), c1);
    for (int j = 1; j <= NVAR; j++)
      CONNEW(j, i) = a * c0[j - 1] + b * (c1[j - 1] - (V1(o->dt, i) / V1(o->cvarea, i)) * RES(j, i));
  }
  if (o->in.iflow != INVISCID) {
    for (int i = 1; i <= s->nsp; i++) {
      int j = V1(o->spts, i);
      CONNEW(2, j) = 0.0;
      CONNEW(3, j) = 0.0;
    }
  }
  for (int pt = 1; pt <= s->np; pt++) {           /* con_to_prim */
    PRIM(1, pt) = CONNEW(1, pt);
    PRIM(2, pt) = CONNEW(2, pt) / CONNEW(1, pt);
    PRIM(3, pt) = CONNEW(3, pt) / CONNEW(1, pt);
    PRIM(4, pt) = s->gamma1 * (CONNEW(4, pt) - 0.5 * (sq(CONNEW(2, pt)) + sq(CONNEW(3, pt))) / CONNEW(1, pt));
  }
}

/* ------------------------------------------------------------------ */
/* sa_model.f                                                           */
/* ------------------------------------------------------------------ */
void orc_sa_model(orc_t *o) {
  const orc_scalars *s = &o->s;
  int np = s->np;
  double *divf = o->divf;
  /* viscous_sa, sa_model.f:39-83 */
  for (int is = 1; is <= np; is++) V1(divf, is) = 0.0;
  for (int jt = 1; jt <= s->nt; jt++) {
    double areat = 0.25 / V1(o->elarea, jt);
    int n1 = ELEM(1, jt), n2 = ELEM(2, jt), n3 = ELEM(3, jt);
    double dbxx[3], dbyy[3];
    dbxx[0] = COORD(2, n2) - COORD(2, n3);
    dbxx[1] = COORD(2, n3) - COORD(2, n1);
    dbxx[2] = COORD(2, n1) - COORD(2, n2);
    dbyy[0] = COORD(1, n3) - COORD(1, n2);
    dbyy[1] = COORD(1, n1) - COORD(1, n3);
    dbyy[2] = COORD(1, n2) - COORD(1, n1);
    int a1 = o->in.bugcompat ? 1 : n1;
    int a2 = o->in.bugcompat ? 2 : n2;
    int a3 = o->in.bugcompat ? 3 : n3;
    double nux = V1(o->nut, a1) * dbxx[0] + V1(o->nut, a2) * dbxx[1] + V1(o->nut, a3) * dbxx[2];
    double nuy = V1(o->nut, a1) * dbyy[0] + V1(o->nut, a2) * dbyy[1] + V1(o->nut, a3) * dbyy[2];
    double mult = (V1(o->mul, n1) + V1(o->mul, n2) + V1(o->mul, n3)) / 3.0;
    double prim5t = (V1(o->nut, n1) + V1(o->nut, n2) + V1(o->nut, n3)) / 3.0;
    double rhot = (PRIM(1, n1) + PRIM(1, n2) + PRIM(1, n3)) / 3.0;
    double mutb = mult / rhot + prim5t;
    int nn[3] = {n1, n2, n3};
    double dv[3];
    for (int j = 0; j < 3; j++) {
      int n = nn[j];
      dv[j] = (s->cb2sig1 * mutb - s->cb2sig2 * (V1(o->mul, n) / PRIM(1, n) + V1(o->nut, n))) *
              (nux * dbxx[j] + nuy * dbyy[j]) * areat;
    }
    V1(divf, n1) = V1(divf, n1) + dv[0];
    V1(divf, n2) = V1(divf, n2) + dv[1];
    V1(divf, n3) = V1(divf, n3) + dv[2];
  }
  /* divergence_sa, sa_model.f:98-115 */
  for (int ii = 1; ii <= s->ne; ii++) {
    int i = V1(o->iedge, ii);
    int n1 = EDGE(1, i), n2 = EDGE(2, i);
    double unl = PRIM(2, n1) * DS(1, i) + PRIM(3, n1) * DS(2, i);
    double unr = PRIM(2, n2) * DS(1, i) + PRIM(3, n2) * DS(2, i);
    double una = 0.5 * (unl + unr);
    double flux = (una > 0.0) ? una * V1(o->nut, n1) : una * V1(o->nut, n2);
    V1(divf, n1) = V1(divf, n1) + flux;
    V1(divf, n2) = V1(divf, n2) - flux;
  }
  /* outer_flux_sa, sa_model.f:134-155 */
  for (int i = s->nffe1; i <= s->nffe2; i++) {
    int ie = V1(o->beindx, i);
    int n1 = EDGE(1, ie), n2 = EDGE(2, ie);
    double dx = COORD(1, n2) - COORD(1, n1);
    double dy = COORD(2, n2) - COORD(2, n1);
    double sx = dy, sy = -dx;
    double u = 0.5 * (PRIM(2, n1) + PRIM(2, n2));
    double v = 0.5 * (PRIM(3, n1) + PRIM(3, n2));
    double un = u * sx + v * sy;
    double flux1, flux2;
    if (un > 0.0) {
      flux1 = un * V1(o->nut, n1);
      flux2 = un * V1(o->nut, n2);
    } else {
      flux1 = un * s->nut_inf;
      flux2 = un * s->nut_inf;
    }
    V1(divf, n1) = V1(divf, n1) + 0.5 * flux1;
    V1(divf, n2) = V1(divf, n2) + 0.5 * flux2;
  }
  /* update_sa, sa_model.f:175-198 */
  double n1b6 = 1.0 / 6.0;
  for (int i = 1; i <= np; i++) {
    double nut = V1(o->nut, i), rho = PRIM(1, i), mul = V1(o->mul, i), wd = V1(o->wd, i);
    double dt = V1(o->dt, i);
    double chi = nut * rho / mul;
    double chi3 = cube(chi);
    double fv1 = chi3 / (chi3 + s->cv11);
    double fv2 = 1.0 / cube(1.0 + chi / s->cv2);
    double r = nut / wd / (wd * s->kolm2);
    double Omega = QY(2, i) - QX(3, i);
    double fv3 = (1.0 + chi * fv1) * (1.0 - fv2) / dmax1(chi, 0.001);
    double S = fv3 * fabs(Omega) + r * fv2;
    r = r / S;
    r = dmin1(r, 2.0);
    double g = r + s->cw2 * (pow6(r) - r);
    double fw = g * pow(s->cw31 / (pow6(g) + s->cw32), n1b6);
    double source = s->cb1 * S * nut;
    double fact = 1.0 + s->cw1 * fw * (nut / wd) * (dt / wd);
    V1(o->nut, i) = (nut - (dt / V1(o->cvarea, i)) * V1(divf, i) + dt * source) / fact;
  }
  for (int i = 1; i <= s->nsp; i++) V1(o->nut, V1(o->spts, i)) = 0.0;
}

/* ------------------------------------------------------------------ */
/* limitgrad.f (never called by the reference; kept for the kernel)     */
/* ------------------------------------------------------------------ */
void orc_limitgrad(orc_t *o) {
  int np = o->s.np, netot = o->s.netot;
  double *qmin = (double *)malloc(sizeof(double) * NVAR * (size_t)np);
  double *qmax = (double *)malloc(sizeof(double) * NVAR * (size_t)np);
  double *phi = (double *)malloc(sizeof(double) * NVAR * (size_t)np);
#define A4(a, j, i) (a)[NVAR * ((i) - 1) + (j) - 1]
  for (int i = 1; i <= np; i++)
    for (int j = 1; j <= NVAR; j++) {
      A4(qmin, j, i) = 1.0e10;
      A4(qmax, j, i) = -1.0e10;
      A4(phi, j, i) = 1.0;
    }
  for (int i = 1; i <= netot; i++) {
    int n1 = EDGE(1, i), n2 = EDGE(2, i);
    /* bugcompat: each end's bounds see only its own value (lines 26-29) */
    int m1 = o->in.bugcompat ? n1 : n2;
    int m2 = o->in.bugcompat ? n2 : n1;
    for (int j = 1; j <= NVAR; j++) {
      if (!o->in.bugcompat) {
        A4(qmin, j, n1) = dmin1(A4(qmin, j, n1), PRIM(j, n1));
        A4(qmax, j, n1) = dmax1(A4(qmax, j, n1), PRIM(j, n1));
        A4(qmin, j, n2) = dmin1(A4(qmin, j, n2), PRIM(j, n2));
        A4(qmax, j, n2) = dmax1(A4(qmax, j, n2), PRIM(j, n2));
      }
      A4(qmin, j, n1) = dmin1(A4(qmin, j, n1), PRIM(j, m1));
      A4(qmax, j, n1) = dmax1(A4(qmax, j, n1), PRIM(j, m1));
      A4(qmin, j, n2) = dmin1(A4(qmin, j, n2), PRIM(j, m2));
      A4(qmax, j, n2) = dmax1(A4(qmax, j, n2), PRIM(j, m2));
    }
  }
  for (int i = 1; i <= netot; i++) {
    int n1 = EDGE(1, i), n2 = EDGE(2, i);
    double dx = COORD(1, n2) - COORD(1, n1);
    double dy = COORD(2, n2) - COORD(2, n1);
    for (int j = 1; j <= NVAR; j++) {
      double dq1 = QX(j, n1) * dx + QY(j, n1) * dy;
      double dqmax1 = A4(qmax, j, n1) - PRIM(j, n1);
      double dqmin1 = A4(qmin, j, n1) - PRIM(j, n1);
      if (dq1 != 0.0) {
        double ppp = (dq1 > 0.0) ? dqmax1 / dq1 : dqmin1 / dq1;
        A4(phi, j, n1) = dmin1(A4(phi, j, n1), ppp);
      }
      double dq2 = -(QX(j, n2) * dx + QY(j, n2) * dy);
      double dqmax2 = A4(qmax, j, n2) - PRIM(j, n2);
      double dqmin2 = A4(qmin, j, n2) - PRIM(j, n2);
      if (dq2 != 0.0) {
        double ppp = (dq2 > 0.0) ? dqmax2 / dq2 : dqmin2 / dq2;
        A4(phi, j, n2) = dmin1(A4(phi, j, n2), ppp);
      }
    }
  }
  for (int i = 1; i <= np; i++)
    for (int j = 1; j <= NVAR; j++) {
      QX(j, i) = A4(phi, j, i) * QX(j, i);
      QY(j, i) = A4(phi, j, i) * QY(j, i);
    }
#undef A4
  free(qmin);
  free(qmax);
  free(phi);
}

/* ------------------------------------------------------------------ */
/* gradient.f:1-63 (never called by the reference: main.f:29 comments   */
/* it out).  The print of every vertex (gradient.f:60) is left out.     */
/* ------------------------------------------------------------------ */
void orc_gradient(orc_t *o) {
  int np = o->s.np;
  for (int i = 1; i <= np; i++)
    for (int j = 1; j <= NVAR; j++) {
      QX(j, i) = 0.0;
      QY(j, i) = 0.0;
    }
  for (int i = 1; i <= o->s.ne; i++) {            /* interior non-zero edges */
    int ie = V1(o->iedge, i);
    int n1 = EDGE(1, ie), n2 = EDGE(2, ie);
    for (int j = 1; j <= NVAR; j++) {
      double qa = 0.5 * (PRIM(j, n1) + PRIM(j, n2));
      double tmpx = qa * DS(1, ie);
      double tmpy = qa * DS(2, ie);
      QX(j, n1) = QX(j, n1) + tmpx;
      QY(j, n1) = QY(j, n1) + tmpy;
      QX(j, n2) = QX(j, n2) - tmpx;
      QY(j, n2) = QY(j, n2) - tmpy;
    }
  }
  for (int i = 1; i <= o->s.nbe; i++) {           /* all boundary edges */
    int ie = V1(o->beindx, i);
    int n1 = EDGE(1, ie), n2 = EDGE(2, ie);
    double dx = COORD(1, n2) - COORD(1, n1);
    double dy = COORD(2, n2) - COORD(2, n1);
    double nx = 0.5 * dy;
    double ny = -0.5 * dx;
    for (int j = 1; j <= NVAR; j++) {
      double qa1 = (5.0 * PRIM(j, n1) + PRIM(j, n2)) / 6.0;
      double qa2 = (PRIM(j, n1) + 5.0 * PRIM(j, n2)) / 6.0;
      QX(j, n1) = QX(j, n1) + qa1 * nx;
      QY(j, n1) = QY(j, n1) + qa1 * ny;
      QX(j, n2) = QX(j, n2) + qa2 * nx;
      QY(j, n2) = QY(j, n2) + qa2 * ny;
    }
  }
  for (int i = 1; i <= np; i++) {                 /* divide by area */
    double ai = 1.0 / V1(o->cvarea, i);
    for (int j = 1; j <= NVAR; j++) {
      QX(j, i) = ai * QX(j, i);
      QY(j, i) = ai * QY(j, i);
    }
  }
}

/* ------------------------------------------------------------------ */
/* shockind.f:1-52 (never called by the reference)                      */
/* ------------------------------------------------------------------ */
void orc_shockind(orc_t *o, double *ind_out) {
  int np = o->s.np;
  double *ind = (double *)malloc(sizeof(double) * (size_t)np);
  for (int i = 1; i <= np; i++) V1(ind, i) = 0.0;
  for (int i = 1; i <= o->s.netot; i++) {
    int n1 = EDGE(1, i), n2 = EDGE(2, i);
    double dx = COORD(1, n2) - COORD(1, n1);
    double dy = COORD(2, n2) - COORD(2, n1);
    double dvc = PRIM(1, n2) - PRIM(1, n1);
    double dvt = dx * QX(1, n1) + dy * QY(1, n1);
    double dvl = o->s.albada11 * dvt + o->s.albada12 * dvc;
    double vl = PRIM(1, n1) + dvl;
    dvt = dx * QX(1, n2) + dy * QY(1, n2);
    double dvr = o->s.albada11 * dvt + o->s.albada12 * dvc;
    double vr = PRIM(1, n2) - dvr;
    double ln = sqrt(sq(DS(1, i)) + sq(DS(2, i)));
    double li = sq(vr - vl) * ln;
    V1(ind, n1) = V1(ind, n1) + li;
    V1(ind, n2) = V1(ind, n2) + li;
  }
  for (int i = 1; i <= np; i++) {
    V1(ind, i) = V1(ind, i) / V1(o->drmin, i) / pow(V1(o->cvarea, i), 0.75);
    if (V1(ind, i) > 1.0)
      for (int j = 1; j <= NVAR; j++) {
        QX(j, i) = 0.0;
        QY(j, i) = 0.0;
      }
  }
  if (ind_out) memcpy(ind_out, ind, sizeof(double) * (size_t)np);
  free(ind);
}

/* ------------------------------------------------------------------ */
/* monitors: check_positivity.f, clcd.f, conres.f                       */
/* ------------------------------------------------------------------ */
int32_t orc_check_positivity(orc_t *o) {
  for (int pt = 1; pt <= o->s.np; pt++)
    if (PRIM(1, pt) <= 0.0 || PRIM(4, pt) <= 0.0 || V1(o->nut, pt) < 0.0) return pt;
  return 0;
}

void orc_clcd(orc_t *o) {
  orc_scalars *s = &o->s;
  double xf = 0.0, yf = 0.0;
  for (int i = s->nswe1; i <= s->nswe2; i++) {
    int ie = V1(o->beindx, i);
    int ip1 = EDGE(1, ie), ip2 = EDGE(2, ie);
    double dx = COORD(1, ip2) - COORD(1, ip1);
    double dy = COORD(2, ip2) - COORD(2, ip1);
    double sx = dy, sy = -dx;
    double mu1 = V1(o->mu, ip1), mu2 = V1(o->mu, ip2);
    double p1 = PRIM(4, ip1);
    double txx1 = 2.0 / 3.0 * mu1 * (2.0 * QX(2, ip1) - QY(3, ip1));
    double txy1 = mu1 * (QY(2, ip1) + QX(3, ip1));
    double tyy1 = 2.0 / 3.0 * mu1 * (2.0 * QY(3, ip1) - QX(2, ip1));
    double p2 = PRIM(4, ip2);
    double txx2 = 2.0 / 3.0 * mu2 * (2.0 * QX(2, ip2) - QY(3, ip2));
    double txy2 = mu2 * (QY(2, ip2) + QX(3, ip2));
    double tyy2 = 2.0 / 3.0 * mu2 * (2.0 * QY(3, ip2) - QX(2, ip2));
    double p = 0.5 * (p1 + p2);
    double txx = 0.5 * (txx1 + txx2);
    double txy = 0.5 * (txy1 + txy2);
    double tyy = 0.5 * (tyy1 + tyy2);
    xf = xf + p * sx - txx * sx - txy * sy;
    yf = yf + p * sy - txy * sx - tyy * sy;
  }
  s->cl = (-sin(s->aoa) * xf + cos(s->aoa) * yf) / (0.5 * s->r_inf * sq(s->q_inf));
  s->cd = (cos(s->aoa) * xf + sin(s->aoa) * yf) / (0.5 * s->r_inf * sq(s->q_inf));
}

int32_t orc_conres(orc_t *o) {
  orc_scalars *s = &o->s;
  double fres = 0.0, fresi = 0.0;
  int iresi = 0;
  for (int i = 1; i <= s->np; i++) {
    double gra = PRIM(1, i) - PRIMO(1, i);
    fres = fres + sq(gra);
    double dif = fabs(gra);
    if (dif > fresi) {
      fresi = dif;
      iresi = i;
    }
  }
  fres = sqrt(fres / s->np);
  s->fresi = fresi;
  s->iresi = iresi;
  if (s->iter == s->iterlast) {
    s->fres1 = fres;
    if (s->fres1 == 0.0) {
      s->fres = fres;
      return ORC_ERR_ZERO_FIRST_RES;
    }
  }
  s->fres = fres / s->fres1;
  return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* main.f:42-76                                                         */
/* ------------------------------------------------------------------ */
int32_t orc_iterate(orc_t *o, int32_t nmax, double minres, int32_t *niter, double *hist_fres,
                    int32_t *hist_iresi, double *hist_fresi, double *hist_cl, double *hist_cd) {
  int n = 0;
  int32_t st = ORC_OK;
  o->s.err = 0;
  while (n < nmax) {
    orc_save_old(o);
    orc_time_step(o);
    for (int irk = 1; irk <= 3; irk++) {
      orc_residu(o);
      if (o->s.err) {
        st = o->s.err;
        goto done;
      }
      orc_update(o, irk);
    }
    if (o->in.iflow == TURBULENT) orc_sa_model(o);
    int bad = orc_check_positivity(o);
    if (bad) {
      o->s.err_point = bad;
      st = ORC_ERR_NONPOSITIVE;
      goto done;
    }
    orc_clcd(o);
    st = orc_conres(o);
    if (st) goto done;
    if (hist_fres) hist_fres[n] = o->s.fres;
    if (hist_iresi) hist_iresi[n] = o->s.iresi;
    if (hist_fresi) hist_fresi[n] = o->s.fresi;
    if (hist_cl) hist_cl[n] = o->s.cl;
    if (hist_cd) hist_cd[n] = o->s.cd;
    o->s.iter++;
    n++;
    if (o->s.fres <= minres) break;
  }
done:
  if (niter) *niter = n;
  return st;
}

/* ------------------------------------------------------------------ */
/* start-up                                                             */
/* ------------------------------------------------------------------ */
static void *xcalloc(size_t n, size_t sz) { return calloc(n ? n : 1, sz); }

orc_t *orc_create(const orc_input *in, int32_t np, int32_t nt, const double *coord,
                  const int32_t *elem, const int32_t *ptype, int32_t *status) {
  orc_t *o = (orc_t *)calloc(1, sizeof(orc_t));
  o->in = *in;
  orc_scalars *s = &o->s;
  s->np = np;
  s->nt = nt;
  math_consts(s);
  s->mach_inf = in->mach_inf;
  s->aoa_deg = in->aoa_deg;
  s->rey = in->rey;
  s->cfl = in->cfl;
  s->xref = in->xref;
  s->yref = in->yref;
  s->iterlast = in->iterlast;
  s->iter = in->iterlast;
  size_t P = (size_t)np, T = (size_t)nt;
  o->coord = (double *)xcalloc(2 * P, sizeof(double));
  memcpy(o->coord, coord, sizeof(double) * 2 * P);
  o->elem = (int32_t *)xcalloc(3 * T, sizeof(int32_t));
  memcpy(o->elem, elem, sizeof(int32_t) * 3 * T);
  o->ptype = (int32_t *)xcalloc(P, sizeof(int32_t));
  memcpy(o->ptype, ptype, sizeof(int32_t) * P);
  /* read_grid.f:62-84 */
  o->spts = (int32_t *)xcalloc(P, sizeof(int32_t));
  o->fpts = (int32_t *)xcalloc(P, sizeof(int32_t));
  for (int ip = 1; ip <= np; ip++) {
    if (V1(o->ptype, ip) == SOLID) V1(o->spts, ++s->nsp) = ip;
    if (V1(o->ptype, ip) == FARFIELD) V1(o->fpts, ++s->nfp) = ip;
  }
  /* geometric.f:15-60 */
  int32_t st = tri_orient(o);
  if (st) goto fail;
  o->esup2 = (int32_t *)xcalloc(P + 1, sizeof(int32_t));
  o->len_esup1 = 3 * (int64_t)T;
  o->esup1 = (int32_t *)xcalloc((size_t)o->len_esup1, sizeof(int32_t));
  el_surr_point(o);
  o->psup2 = (int32_t *)xcalloc(P + 1, sizeof(int32_t));
  o->psup1 = (int32_t *)xcalloc(6 * T + 1, sizeof(int32_t));
  pt_surr_pt(o);
  o->len_psup1 = o->psup2[np];
  o->len_edge = o->len_psup1 / 2 + 1;
  o->edge = (int32_t *)xcalloc(2 * (size_t)o->len_edge, sizeof(int32_t));
  create_edge(o);
  o->edneigh = (int32_t *)xcalloc(2 * (size_t)s->ne, sizeof(int32_t));
  el_surr_edge(o);
  o->tcoord = (double *)xcalloc(2 * T, sizeof(double));
  tri_coord(o);
  o->elarea = (double *)xcalloc(T, sizeof(double));
  o->mcarea = (double *)xcalloc(P, sizeof(double));
  o->cvarea = (double *)xcalloc(P, sizeof(double));
  st = areas(o);
  if (st) goto fail;
  o->wd = (double *)xcalloc(P, sizeof(double));
  o->wd1 = (double *)xcalloc((size_t)s->nsp, sizeof(double));
  if (in->iflow == TURBULENT) wall_dist(o);
  o->ds = (double *)xcalloc(2 * (size_t)s->ne, sizeof(double));
  o->dsb = (double *)xcalloc(2 * P, sizeof(double));
  st = flength(o);
  if (st) goto fail;
  o->iedge = (int32_t *)xcalloc((size_t)s->ne, sizeof(int32_t));
  reorder_edges(o);
  o->drmin = (double *)xcalloc(P, sizeof(double));
  orc_dtlength(np, nt, o->coord, o->elem, o->elarea, o->drmin);
  o->beindx = (int32_t *)xcalloc((size_t)s->netot, sizeof(int32_t));
  make_bdedges(o);
  st = geom_stat(o);
  if (st) goto fail;
  /* initialize.f:14-89 */
  s->q_inf = 1.0;
  s->r_inf = 1.0;
  s->p_inf = 1.0 / (s->gamma * sq(s->mach_inf));
  s->t_inf = s->p_inf / (s->r_inf * s->gas_const);
  s->aoa = s->aoa_deg * s->pi / 180.0;
  s->u_inf = s->q_inf * cos(s->aoa);
  s->v_inf = s->q_inf * sin(s->aoa);
  s->a_inf = sqrt(s->gamma * s->p_inf / s->r_inf);
  s->sconst = 110.4 * s->t_inf / 300.0;
  s->airk[0] = 0.0;
  s->airk[1] = 3.0 / 4.0;
  s->airk[2] = 1.0 / 3.0;
  s->birk[0] = 1.0;
  s->birk[1] = 1.0 / 4.0;
  s->birk[2] = 2.0 / 3.0;
  o->prim = (double *)xcalloc(NVAR * P, sizeof(double));
  o->prim_old = (double *)xcalloc(NVAR * P, sizeof(double));
  o->qx = (double *)xcalloc(NVAR * P, sizeof(double));
  o->qy = (double *)xcalloc(NVAR * P, sizeof(double));
  o->res = (double *)xcalloc(NVAR * P, sizeof(double));
  o->con_new = (double *)xcalloc(NVAR * P, sizeof(double));
  o->dt = (double *)xcalloc(P, sizeof(double));
  o->mu = (double *)xcalloc(P, sizeof(double));
  o->mul = (double *)xcalloc(P, sizeof(double));
  o->nut = (double *)xcalloc(P, sizeof(double));
  o->divf = (double *)xcalloc(P, sizeof(double));
  for (int j = 1; j <= np; j++) {
    PRIM(1, j) = s->r_inf;
    PRIM(2, j) = s->u_inf;
    PRIM(3, j) = s->v_inf;
    PRIM(4, j) = s->p_inf;
  }
  s->nut_inf = 0.0;
  if (in->iflow == TURBULENT) {
    sutherland(o);
    for (int i = 1; i <= np; i++) V1(o->nut, i) = in->nut_ratio * V1(o->mul, i) / PRIM(1, i);
    viscosity(o);
    s->nut_inf = V1(o->nut, 1);
  } else if (in->iflow == LAMINAR) {
    sutherland(o);
    viscosity(o);
  }
  s->fres = in->minres + 1.0;
  s->fres1 = 0.0;
  if (status) *status = ORC_OK;
  return o;
fail:
  if (status) *status = st;
  orc_destroy(o);
  return NULL;
}

void orc_destroy(orc_t *o) {
  if (!o) return;
  void *ptrs[] = {o->coord, o->elem, o->ptype, o->spts, o->fpts, o->esup1, o->esup2,
                  o->psup1, o->psup2, o->edge, o->edneigh, o->iedge, o->beindx,
                  o->tcoord, o->elarea, o->cvarea, o->mcarea, o->ds, o->dsb, o->drmin,
                  o->wd, o->wd1, o->prim, o->prim_old, o->qx, o->qy, o->res, o->dt,
                  o->mu, o->mul, o->nut, o->divf, o->con_new};
  for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); i++) free(ptrs[i]);
  free(o);
}

void orc_get_scalars(const orc_t *o, orc_scalars *s) { *s = o->s; }
void orc_set_cl(orc_t *o, double cl) { o->s.cl = cl; }

double *orc_darray(orc_t *o, const char *name, int64_t *len) {
  int64_t P = o->s.np, T = o->s.nt;
  struct { const char *n; double *p; int64_t l; } tab[] = {
      {"coord", o->coord, 2 * P},   {"prim", o->prim, 4 * P},     {"prim_old", o->prim_old, 4 * P},
      {"qx", o->qx, 4 * P},         {"qy", o->qy, 4 * P},         {"res", o->res, 4 * P},
      {"dt", o->dt, P},             {"mu", o->mu, P},             {"mul", o->mul, P},
      {"nut", o->nut, P},           {"ds", o->ds, 2 * (int64_t)o->s.netot},
      {"dsb", o->dsb, 2 * P},       {"elarea", o->elarea, T},     {"cvarea", o->cvarea, P},
      {"mcarea", o->mcarea, P},     {"drmin", o->drmin, P},       {"wd", o->wd, P},
      {"wd1", o->wd1, o->s.nsp},    {"tcoord", o->tcoord, 2 * T}, {"divf", o->divf, P}};
  for (size_t i = 0; i < sizeof(tab) / sizeof(tab[0]); i++)
    if (!strcmp(tab[i].n, name)) {
      if (len) *len = tab[i].l;
      return tab[i].p;
    }
  if (len) *len = 0;
  return NULL;
}

int32_t *orc_iarray(orc_t *o, const char *name, int64_t *len) {
  int64_t P = o->s.np, T = o->s.nt;
  struct { const char *n; int32_t *p; int64_t l; } tab[] = {
      {"elem", o->elem, 3 * T},         {"edge", o->edge, 2 * (int64_t)o->s.netot},
      {"edneigh", o->edneigh, 2 * (int64_t)o->s.netot},
      {"iedge", o->iedge, o->s.ne},     {"beindx", o->beindx, o->s.nbe},
      {"spts", o->spts, o->s.nsp},      {"ptype", o->ptype, P},
      {"esup1", o->esup1, 3 * T},       {"esup2", o->esup2, P + 1},
      {"psup1", o->psup1, o->len_psup1}, {"psup2", o->psup2, P + 1}};
  for (size_t i = 0; i < sizeof(tab) / sizeof(tab[0]); i++)
    if (!strcmp(tab[i].n, name)) {
      if (len) *len = tab[i].l;
      return tab[i].p;
    }
  if (len) *len = 0;
  return NULL;
}

/* ------------------------------------------------------------------ */
/* Test hooks: one interior flux or one limiter value in isolation.     */
/* ------------------------------------------------------------------ */
int32_t orc_eval_flux(orc_t *o, int32_t iflux, const double *ds, const double *priml,
                      const double *primr, double *flux) {
  int32_t err0 = o->s.err;
  o->s.err = 0;
  if (iflux == IROE) roe_flux(o, ds, priml, primr, flux);
  else if (iflux == IKFVS) kfvs_flux(o, ds, priml, primr, flux);
  else hllc_flux(o, ds, priml, primr, flux);
  int32_t e = o->s.err;
  o->s.err = err0;
  return e;
}

double orc_limit_albada(double ul, double ur) { return limit_albada(ul, ur); }
