/*
 * fvm_oracle.h -- CPU oracle for the fvm2d hot path.  TEST INFRASTRUCTURE:
 * only the tests, the smoke check and the benchmark's CPU-baseline leg use
 * it, as the checker; no product code links it.
 *
 * A serial FP64 restatement, in the reference's loop order, of fvm2d's
 * Fortran sources (src/ *.f): the start-up sequence of main.f:20-27 (math,
 * read_grid's point lists, geometric, initialize) and the iteration loop of
 * main.f:42-76 with every routine it calls.  Built with -O3
 * -ffp-contract=off so every floating-point operation is rounded as
 * written.  Integer powers are multiplication chains: x**2 = x*x,
 * x**3 = (x*x)*x, x**6 = ((x*x)*x)*((x*x)*x).  libgfortran intrinsics map to
 * glibc: dsqrt->sqrt, dexp->exp, derf->erf, **(real)->pow, datan2->atan2.
 *
 * Parity is unpinned by the reference: it ships no tests, golden vectors or
 * grids, and no Fortran compiler exists to run it.  The oracle is pinned by
 * equation-derived known answers instead (freestream preservation, flux
 * consistency, conservation, exact gradients of linear fields).
 */
#ifndef FVM_ORACLE_H
#define FVM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* The fvm.inp inputs (read_input.f:20-66) plus two switches. */
typedef struct orc_input {
  int32_t iflow;
  double mach_inf, aoa_deg, rey, cfl;
  int32_t iterlast, maxiter;
  double minres;
  int32_t iflux, ilimit, vortex;
  double xref, yref;
  int32_t cell_type;
  double nut_ratio;   /* initialize.f:71 uses 0.1                        */
  int32_t bugcompat;  /* sa_model.f:57-62, wall_dist.f:46, limitgrad.f:26-29,
                         hllc_flux.f:149-154 (no rotation back)          */
} orc_input;

/* Scalars of the COMMON blocks (read-only view). */
typedef struct orc_scalars {
  int32_t np, nt, ne, netot, nsp, nfp, nbe, nswe1, nswe2, nffe1, nffe2;
  int32_t iter, iterlast, iresi, err, err_point;
  double fres, fres1, fresi, cl, cd, dtglobal;
  double gamma, gamma1, gas_const, pi, prandtl, prandtl_turb;
  double albada11, albada12, albada21, albada22;
  double cb1, cb2, sigma_sa, kolm, cw1, cw2, cw3, cv1, cv2, cv11, cw31, cw32;
  double kolm2, cb2sig1, cb2sig2;
  double mach_inf, aoa_deg, aoa, rey, cfl, q_inf, r_inf, p_inf, t_inf;
  double u_inf, v_inf, a_inf, sconst, nut_inf, xref, yref;
  double airk[3], birk[3];
} orc_scalars;

#define ORC_OK 0
#define ORC_ERR_GEOMETRY 9
#define ORC_ERR_NONPOSITIVE 3
#define ORC_ERR_ROE_SONIC 4
#define ORC_ERR_ZERO_FIRST_RES 5

typedef struct orc orc_t;

/* Start-up: math, point lists (read_grid.f:62-94), geometric, initialize
 * (scratch start).  elem is copied; returns NULL with *status set on a
 * geometry stop. */
orc_t *orc_create(const orc_input *in, int32_t np, int32_t nt,
                  const double *coord, const int32_t *elem,
                  const int32_t *ptype, int32_t *status);
void orc_destroy(orc_t *o);
void orc_get_scalars(const orc_t *o, orc_scalars *s);
void orc_set_cl(orc_t *o, double cl);

/* Raw access to the arrays (Fortran layout, 0-based C pointers).
 * Names: coord prim prim_old qx qy res dt mu mul nut ds dsb elarea cvarea
 * mcarea drmin wd wd1 tcoord (double); elem edge edneigh iedge beindx spts
 * ptype esup1 esup2 psup1 psup2 (int32).  *len is the element count. */
double *orc_darray(orc_t *o, const char *name, int64_t *len);
int32_t *orc_iarray(orc_t *o, const char *name, int64_t *len);

/* The routines of the loop body. */
void orc_save_old(orc_t *o);
void orc_time_step(orc_t *o);
void orc_residu(orc_t *o);
void orc_update(orc_t *o, int32_t irk);
void orc_sa_model(orc_t *o);
void orc_limitgrad(orc_t *o);
/* gradient.f and shockind.f (both uncalled by the reference): edge-based
 * Green-Gauss gradients with the boundary closure into qx, qy; the shock
 * indicator, zeroing the gradients where it exceeds 1 (ind, length np,
 * may be NULL). */
void orc_gradient(orc_t *o);
void orc_shockind(orc_t *o, double *ind);
int32_t orc_check_positivity(orc_t *o);      /* first bad point or 0 */
void orc_clcd(orc_t *o);
int32_t orc_conres(orc_t *o);                /* ORC_OK or ZERO_FIRST_RES */

/* main.f:42-76: up to nmax iterations, stopping once fres <= minres.
 * hist_* (length >= nmax, may be NULL) receive the RES.DAT columns.
 * Returns ORC_OK or an error; *niter = iterations completed. */
int32_t orc_iterate(orc_t *o, int32_t nmax, double minres, int32_t *niter,
                    double *hist_fres, int32_t *hist_iresi,
                    double *hist_fresi, double *hist_cl, double *hist_cd);

/* Stand-alone set-up passes on caller arrays (1-based connectivity). */
void orc_dtlength(int32_t np, int32_t nt, const double *coord,
                  const int32_t *elem, const double *elarea, double *drmin);
void orc_wall_dist(int32_t np, int32_t ne, const double *coord,
                   const int32_t *edge, const int32_t *ptype,
                   int32_t bugcompat, double *wd);

/* Test hooks: the interior flux of one face (roe/kfvs/hllc_flux.f) with
 * this instance's constants and bugcompat switch; the van Albada limiter
 * (recon.f:55-71). */
int32_t orc_eval_flux(orc_t *o, int32_t iflux, const double *ds, const double *priml,
                      const double *primr, double *flux);
double orc_limit_albada(double ul, double ur);

#ifdef __cplusplus
}
#endif
#endif
