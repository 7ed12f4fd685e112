/*
 * fvm_gpu.h -- C ABI of the GB300 implementation of fvm2d's per-iteration
 * hot path (cell-vertex, edge-based finite volumes on triangles).
 *
 * The reference is one serial Fortran 77 program.  Its hot path is the body
 * of the iteration loop in src/main.f:44-62:
 *
 *     save_old -> time_step -> 3 x { residu -> update } -> [sa_model]
 *              -> check_positivity -> clcd -> conres
 *
 * The routines take arrays by reference and read scalars from COMMON blocks
 * (src/param.h:36-142, src/gdata.h:1-6).  This header is the drop-in
 * boundary for that loop: a Fortran driver binds every function below with
 * ISO_C_BINDING (`bind(C, name="...")`), keeps its own input, grid, geometry
 * and output path, and calls these entry points in place of the loop body.
 *
 * Conventions
 *   - All functions return int32 status: FVM_OK (0) or an FVM_ERR_* code.
 *   - Arrays are the Fortran ones, column-major: prim(4,np) is the C array
 *     double[np][4]; coord(2,np) is double[np][2]; ds(2,netot) is
 *     double[netot][2]; elem(3,nt), edge(2,netot), edneigh(2,netot) are
 *     int32[..][3|2].  Connectivity values are 1-based as in Fortran.
 *   - Host arrays stay owned by the caller and are only read (or written,
 *     for outputs) during the call.  The library owns all device memory.
 *   - One handle per host thread; calls are synchronous from the caller's
 *     point of view; each handle has its own CUDA stream.
 *   - Errors mirror the reference's `stop` sites; the driver prints and
 *     stops as before.  fvm_gpu_strerror() gives the text.
 */
#ifndef FVM_GPU_H
#define FVM_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- codes, as in src/param.h:97-142 ---------------------------------- */
#define FVM_INVISCID   1
#define FVM_LAMINAR    2
#define FVM_TURBULENT  3

#define FVM_FLUX_ROE   1
#define FVM_FLUX_KFVS  2
#define FVM_FLUX_HLLC  3

#define FVM_CELL_MEDIAN 1
#define FVM_CELL_BARTH  2

#define FVM_PT_INTERIOR 0
#define FVM_PT_SOLID    3
#define FVM_PT_OUTFLOW  4
#define FVM_PT_FARFIELD 5

/* arithmetic of the state, reconstruction, fluxes and RK stages */
#define FVM_PREC_FP64  0   /* plain method, FP64 throughout               */
#define FVM_PREC_FP32  1   /* FP32 state/flux, FP64 geometry and monitors */

/* ---- status codes ------------------------------------------------------ */
#define FVM_OK                  0
#define FVM_ERR_ARG             1  /* bad argument / size                       */
#define FVM_ERR_CUDA            2  /* CUDA runtime error                        */
#define FVM_ERR_NONPOSITIVE     3  /* check_positivity.f:13-24                  */
#define FVM_ERR_ROE_SONIC       4  /* roe_flux.f:60-65 (Roe-average a^2 <= 0)   */
#define FVM_ERR_ZERO_FIRST_RES  5  /* conres.f:28                               */
#define FVM_ERR_TIMEOUT         6  /* a bounded device wait ran out             */
#define FVM_ERR_NOMEM           7  /* device allocation failed                  */
#define FVM_ERR_STATE           8  /* call out of order (e.g. no state set)     */
#define FVM_ERR_GEOMETRY        9  /* tri_orient.f:28-31, geom_stat.f:18-37,
                                      flength.f:20-27, areas.f:145-150          */
#define FVM_ERR_CAPACITY       10  /* a batch arena has no room                 */
#define FVM_CHECKPOINTED       11  /* a served solve stopped on request with its
                                      state kept (fvm_serve_checkpoint)        */

/*
 * Scalars of the COMMON blocks that the hot path reads.  Fill with
 * fvm_params_init() (which restates src/math.f:8-40 and
 * src/initialize.f:14-34,52-58) or copy from the driver's COMMON blocks.
 */
typedef struct fvm_params {
  /* switches: /flowtype/ /fluxtype/ /lim/ /farfieldbc/ /celltypes/ */
  int32_t iflow;        /* FVM_INVISCID | FVM_LAMINAR | FVM_TURBULENT     */
  int32_t iflux;        /* FVM_FLUX_ROE | FVM_FLUX_KFVS | FVM_FLUX_HLLC   */
  int32_t ilimit;       /* 0 = unlimited MUSCL, 1 = van Albada limiter    */
  int32_t vortex;       /* farfield point-vortex correction 0/1           */
  int32_t cell_type;    /* FVM_CELL_MEDIAN | FVM_CELL_BARTH               */
  int32_t precision;    /* FVM_PREC_FP64 | FVM_PREC_FP32                  */
  int32_t bugcompat;    /* 1: reproduce sa_model.f:57-62 (nut(1..3)),
                           wall_dist.f:46 (dy3 from x) and the
                           limitgrad.f:26-29 bounds; 0: corrected forms    */
  int32_t reserved;
  /* /const/ /viscparam/ (math.f:8-14) */
  double gamma, gamma1, gas_const, pi;
  double prandtl, prandtl_turb;
  /* /lim/ (math.f:16-20), EPSILON (param.h:105) */
  double albada11, albada12, albada21, albada22, epsilon;
  /* /samodel/ (math.f:25-40) */
  double cb1, cb2, sigma_sa, kolm, cw1, cw2, cw3, cv1, cv2;
  double cv11, cw31, cw32, kolm2, cb2sig1, cb2sig2;
  /* /itparam/ /inf/ (read_input.f:20-66, initialize.f:14-34) */
  double mach_inf, aoa_deg, aoa, rey, cfl;
  double q_inf, r_inf, p_inf, t_inf, u_inf, v_inf, a_inf, sconst, nut_inf;
  double xref, yref;
  /* /timeintegration/ (initialize.f:52-58) */
  double airk[3], birk[3];
} fvm_params;

/*
 * Mesh arrays produced by the driver's geometric() (src/geometric.f:15-60).
 * ne <= netot: the interior-flux loop runs over iedge(1..ne)
 * (flength.f:84-98 drops zero-length Barth faces).  beindx(nswe1..nswe2)
 * are the solid edges and beindx(nffe1..nffe2) the farfield edges
 * (make_bdedges.f:29-44), all 1-based positions.
 */
typedef struct fvm_mesh {
  int32_t np, nt, ne, netot, nsp, nbe;
  int32_t nswe1, nswe2, nffe1, nffe2;
  const double  *coord;    /* [np][2]                                     */
  const int32_t *elem;     /* [nt][3]   counter-clockwise (tri_orient.f)  */
  const int32_t *ptype;    /* [np]                                        */
  const int32_t *spts;     /* [nsp]     solid points, ascending           */
  const int32_t *edge;     /* [netot][2]                                  */
  const int32_t *iedge;    /* [ne]                                        */
  const int32_t *beindx;   /* [nbe]                                       */
  const double  *ds;       /* [netot][2] dual-face normal (flength.f)     */
  const double  *elarea;   /* [nt]                                        */
  const double  *cvarea;   /* [np]      control-volume area               */
  const double  *mcarea;   /* [np]      median-cell area (gradients)      */
  const double  *drmin;    /* [np]      dtlength.f                        */
  const double  *wd;       /* [np]      wall distance (turbulent only;
                                        may be NULL otherwise)            */
} fvm_mesh;

typedef struct fvm_handle fvm_handle;

/* ---- set-up ------------------------------------------------------------ */

/* Restates math.f:8-40 and initialize.f:14-34,52-58: fills every constant
 * and freestream value of `p` from the fvm.inp inputs (read_input.f:20-66).
 * nut_ratio is the freestream nu~/nu of a turbulent start: nut_inf =
 * nut_ratio*mul_inf/r_inf (initialize.f:69-74 hard-codes 0.1). */
int32_t fvm_params_init(fvm_params *p, int32_t iflow, double mach_inf,
                        double aoa_deg, double rey, double cfl,
                        int32_t iflux, int32_t ilimit, int32_t vortex,
                        double xref, double yref, int32_t cell_type,
                        double nut_ratio, int32_t precision,
                        int32_t bugcompat);

/* Copies params and mesh to the device, reorders vertices for locality,
 * builds the gather structures and allocates all device state.  Replaces
 * nothing in the reference (it is the device-side half of geometric.f).
 * The state is the freestream until fvm_gpu_set_state() is called. */
int32_t fvm_gpu_create(const fvm_params *params, const fvm_mesh *mesh,
                       fvm_handle **out);
int32_t fvm_gpu_destroy(fvm_handle *h);
const char *fvm_gpu_strerror(int32_t status);
/* sizeof of the ABI structs, for bindings to check their mirrors:
 * out[0] fvm_params, [1] fvm_mesh, [2] fvm_geom, [3] fvm_batch_caps. */
void fvm_abi_sizes(int64_t out[4]);

/* State transfer in the driver's vertex order (initialize.f / finalize.f
 * arrays).  iterlast is the iteration counter of the first iteration to run
 * (main.f:32); the residual is normalised by the first iteration after a
 * set_state (conres.f:25-31).  Any pointer except prim may be NULL. */
int32_t fvm_gpu_set_state(fvm_handle *h, const double *prim,
                          const double *nut, const double *mul,
                          const double *mu, int32_t iterlast);
int32_t fvm_gpu_get_state(fvm_handle *h, double *prim, double *nut,
                          double *mul, double *mu, double *qx, double *qy);

/* ---- whole iterations: replaces main.f:44-62 ---------------------------- */

/* Runs up to nmax iterations of the loop body, stopping after the first
 * iteration whose normalised residual is <= minres (main.f:42).  Writes the
 * RES.DAT columns of every iteration run (main.f:63) to the hist_* arrays
 * (each of length >= nmax; any may be NULL) and the count to *niter.  On a
 * positivity failure returns FVM_ERR_NONPOSITIVE with *bad_point set to the
 * first offending vertex (1-based, check_positivity.f:11-24). */
int32_t fvm_gpu_iterate(fvm_handle *h, int32_t nmax, double minres,
                        int32_t *niter, double *hist_fres,
                        int32_t *hist_iresi, double *hist_fresi,
                        double *hist_cl, double *hist_cd,
                        int32_t *bad_point);

/* ---- per-routine entry points (incremental adoption, parity) ----------- */
int32_t fvm_gpu_save_old(fvm_handle *h);                 /* save_old.f:4-18   */
int32_t fvm_gpu_time_step(fvm_handle *h);                /* time_step.f:4-37  */
int32_t fvm_gpu_residu(fvm_handle *h);                   /* residu.f:2-91     */
int32_t fvm_gpu_update(fvm_handle *h, int32_t irk);      /* update.f:5-38     */
int32_t fvm_gpu_sa_model(fvm_handle *h);                 /* sa_model.f:3-25   */
int32_t fvm_gpu_limitgrad(fvm_handle *h);                /* limitgrad.f:1-78  */
/* gradient.f:1-63, never called by the reference (main.f:29 comments it
 * out): edge-based Green-Gauss gradients over the dual cells (interior edges
 * in iedge order, then boundary edges in beindx order with the 5/6, 1/6
 * closure), divided by cvarea; they replace the handle's gradients (read
 * them with fvm_gpu_get_state).  Boundary edges other than solid and
 * farfield are not represented (the reference's grids have none). */
int32_t fvm_gpu_gradient(fvm_handle *h);
/* shockind.f:1-52, never called by the reference: the density-jump
 * indicator over all edges from the handle's current gradients; the
 * gradients of vertices where it exceeds 1 are set to zero. */
int32_t fvm_gpu_shockind(fvm_handle *h);
int32_t fvm_gpu_check_positivity(fvm_handle *h,
                                 int32_t *bad_point);    /* check_positivity.f */
int32_t fvm_gpu_clcd(fvm_handle *h, double *cl, double *cd);   /* clcd.f:4-49 */
/* conres.f:3-34; first != 0 sets fres1 from this call (iter == iterlast). */
int32_t fvm_gpu_conres(fvm_handle *h, int32_t first, double *fres,
                       double *fresi, int32_t *iresi);
/* Arrays the per-routine calls produce, in the driver's vertex order. */
int32_t fvm_gpu_get_residual(fvm_handle *h, double *res);     /* res(4,np) */
int32_t fvm_gpu_get_dt(fvm_handle *h, double *dt);            /* dt(np)    */
int32_t fvm_gpu_get_prim_old(fvm_handle *h, double *prim_old);

/* ---- set-up kernels (FP64), each a whole-array pass ---------------------- */
/* dtlength.f:6-47: drmin(np) = min altitude of the triangles around each
 * point.  elem is 1-based and counter-clockwise; elarea from tri_area. */
int32_t fvm_gpu_dtlength(int32_t np, int32_t nt, const double *coord,
                         const int32_t *elem, const double *elarea,
                         double *drmin);
/* wall_dist.f:3-95 (the wd part, lines 16-61 and 87-92): distance from
 * every point to the nearest solid edge (edges with both ends solid among
 * edge(1..ne)); wd = 1 at solid points.  bugcompat reproduces line 46. */
int32_t fvm_gpu_wall_dist(int32_t np, int32_t ne, const double *coord,
                          const int32_t *edge, const int32_t *ptype,
                          int32_t bugcompat, double *wd);

/* Driver-side geometry on the host: restates the chain of
 * src/geometric.f:15-60 (tri_orient, el_surr_point, pt_surr_pt,
 * create_edge, el_surr_edge, tri_coord, areas, flength, reorder_edges,
 * make_bdedges, geom_stat) for callers that have no Fortran geometric().
 * elem is modified in place (orientation, tri_orient.f:33-37).  drmin and
 * wd are left zero: fill them with fvm_gpu_dtlength / fvm_gpu_wall_dist.
 * Output arrays are owned by the library; release with fvm_geom_free().
 * Runs on the host only (no GPU needed). */
typedef struct fvm_geom {
  fvm_mesh mesh;            /* points into the arrays below               */
  int32_t *edge, *edneigh, *iedge, *beindx, *spts;
  double *ds, *dsb, *elarea, *cvarea, *mcarea, *drmin, *wd;
} fvm_geom;
int32_t fvm_geom_build(int32_t np, int32_t nt, const double *coord,
                       int32_t *elem, const int32_t *ptype,
                       int32_t cell_type, fvm_geom **out);
int32_t fvm_geom_free(fvm_geom *g);
/* The same chain on the GPU, for callers that build many grids (the
 * serving path's request preparation): every array equal to
 * fvm_geom_build's, bit for bit (same numbering, same floating-point
 * operations in the same order), and drmin filled as fvm_gpu_dtlength
 * fills it.  elem is oriented in place on success and left untouched on
 * error.  Release with fvm_geom_free(). */
int32_t fvm_gpu_geom_build(int32_t np, int32_t nt, const double *coord,
                           int32_t *elem, const int32_t *ptype,
                           int32_t cell_type, fvm_geom **out);

/* ---- allocation-free entry point ----------------------------------------- */
/* No counterpart in the reference.  conres.f:11-31 (RMS and first argmax of
 * the density change, normalised by the first iteration's value) for
 * callers that cannot allocate device memory: drivers whose device memory
 * is owned by an OpenACC / CUDA Fortran data region or by another
 * framework's pool, where a library cudaMalloc (which also synchronises the
 * device and may fail mid-run) is not allowed.  prim and prim_old are the
 * caller's DEVICE arrays prim(4,np) in driver order; the results go to host
 * memory.  first != 0 sets *fres1 from this call (and returns
 * FVM_ERR_ZERO_FIRST_RES when it is zero); otherwise *fres1 is the
 * normaliser.  Scratch is a fixed static device array sized for
 * FVM_NOALLOC_MAX_POINTS points, held by every GPU that loads the library
 * until exit; larger np is refused with FVM_ERR_ARG.  Nothing is allocated.
 * The first call on a device looks up the scratch address on that device,
 * so make it before any stream capture.  All calls share the scratch and
 * run on the default stream, synchronously: calls that overlap on the GPU
 * (from several host threads) race.  The legacy default stream is not
 * ordered against non-blocking streams or async queues, so finish the
 * writes of prim and prim_old first (`!$acc wait`, cudaStreamSynchronize
 * on the writing stream).  A NaN density change makes fres NaN but, as in
 * conres.f, never becomes fresi/iresi. */
#define FVM_NOALLOC_MAX_POINTS (1 << 20)
int32_t fvm_gpu_conres_noalloc(const double *prim, const double *prim_old,
                               int32_t np, int32_t first, double *fres1,
                               double *fres, double *fresi, int32_t *iresi);

/* ---- batches: many meshes of uneven size in one launch per kernel ------- */
/*
 * No counterpart in the reference (which solves one grid per process).  A
 * batch is a device arena holding many meshes at once; every kernel of an
 * iteration runs once for all of them (a persistent grid-stride loop over
 * the blocks of every armed mesh), and one CUDA graph holds the whole
 * iteration.  Meshes are admitted and retired between steps without
 * re-capturing the graph: the kernels read the work list from device
 * memory.  The single-mesh fvm_gpu_* calls above are a batch of one.
 */
typedef struct fvm_batch fvm_batch;

typedef struct fvm_batch_caps {
  int64_t vertices;          /* total vertices of all resident meshes         */
  int32_t meshes;            /* resident meshes at a time                     */
  int32_t viscous;           /* 1 if laminar/turbulent meshes may be admitted */
  /* optional overrides; 0 = derived from vertices and meshes */
  int64_t blocks, edge_entries, boundary_entries, tri_entries, triangles;
  int64_t edge_incidence, tri_incidence, all_incidence, solid_edges;
  int32_t max_slots, max_tri;   /* per-block shared-memory sizing           */
  int32_t grid;                 /* CTAs of the block kernels (0 = occupancy) */
  int32_t max_tri2;             /* triangles of a block and of its halo      */
  int32_t max_loc;              /* own + halo vertices of a block            */
  int32_t fused;                /* 1: one fused gradient+flux pass per stage
                                   (recomputes halo gradients in shared
                                   memory) while every resident mesh's halo
                                   tiles fit max_tri2 / max_loc; 0
                                   (default): separate passes               */
  int64_t halo_entries, halo_incidence;
  int32_t grad_mode;            /* gradient pass: 1 per-thread loads of the
                                   block's triangles; 2 each vertex walks its
                                   triangles itself (no shared memory); 3 the
                                   block's triangles and incidence staged by
                                   bulk copies (FP32 only); 4 the same inputs
                                   streamed through a ring of shared-memory
                                   stages by a producer warp for consumer
                                   groups (FP32 only); 0 (default): 3 in
                                   FP32, 1 in FP64.  In FP32 this is the
                                   pass of viscous meshes: inviscid meshes
                                   take the vertex-stencil gradient        */
  int32_t overlap;              /* 2..8: the meshes run in that many chains
                                   of kernels on their own streams (parts of
                                   the work list split at mesh boundaries),
                                   so one part's gradient pass overlaps
                                   another's flux pass; 0 or 1 (default):
                                   one chain                                */
  int32_t pipe_groups;          /* consumer groups per CTA of the pipelined
                                   kernels: 1 or 2 (0 = default, 2)         */
  int32_t pipe_stages;          /* stages of their ring (0 = as many as fit
                                   the shared memory, at most 8)            */
} fvm_batch_caps;

int32_t fvm_batch_create(int32_t precision, const fvm_batch_caps *caps,
                         fvm_batch **out);
int32_t fvm_batch_destroy(fvm_batch *b);
/* Admits a mesh (geometry upload, block tables, freestream state) and
 * returns its slot; FVM_ERR_CAPACITY when the arena has no room. */
int32_t fvm_batch_add(fvm_batch *b, const fvm_params *p, const fvm_mesh *m,
                      int32_t *slot);
int32_t fvm_batch_remove(fvm_batch *b, int32_t slot);
/* fvm_batch_add in two halves, so the host work can overlap the GPU:
 * fvm_batch_prepare builds the block layout on the host (thread safe, no
 * device work; the mesh arrays are copied), fvm_batch_add_prepared uploads
 * it.  On success the batch takes the prepared object; on any error
 * (FVM_ERR_CAPACITY included) it stays with the caller, who may retry it
 * later or release it with fvm_prepared_free. */
typedef struct fvm_prepared fvm_prepared;
int32_t fvm_batch_prepare(const fvm_params *p, const fvm_mesh *m,
                          fvm_prepared **out);
int32_t fvm_batch_add_prepared(fvm_batch *b, fvm_prepared *prep,
                               int32_t *slot);
int32_t fvm_prepared_free(fvm_prepared *prep);
/* Device bytes a prepared mesh occupies in a batch of this precision. */
int64_t fvm_prepared_bytes(const fvm_prepared *prep, int32_t precision);
/* A slot's state in the driver's vertex order and FP64 (prim(4,np),
 * nut, mul, mu(np), qx, qy(4,np)); the arrays cross as they are and are
 * permuted and converted on the device.  set: prim is required, a NULL
 * nut/mul/mu is left as it is; get: a NULL array is not read back. */
int32_t fvm_batch_set_state(fvm_batch *b, int32_t slot, const double *prim,
                            const double *nut, const double *mul,
                            const double *mu, int32_t iterlast);
int32_t fvm_batch_get_state(fvm_batch *b, int32_t slot, double *prim,
                            double *nut, double *mul, double *mu, double *qx,
                            double *qy);
/* Arms a solve of up to nmax iterations that stops after the first
 * iteration with fres <= minres (main.f:42). */
int32_t fvm_batch_start(fvm_batch *b, int32_t slot, int32_t nmax,
                        double minres);
/* Enqueues niter iterations of every armed mesh; asynchronous. */
int32_t fvm_batch_step(fvm_batch *b, int32_t niter);
int32_t fvm_batch_sync(fvm_batch *b);
/* Waits for the stream and reports one slot: *active (still iterating),
 * *niter (iterations since start), the last fres, cl, cd, and the status
 * (FVM_OK or the stop that ended it, with *bad_point for positivity). */
int32_t fvm_batch_poll(fvm_batch *b, int32_t slot, int32_t *active,
                       int32_t *niter, double *fres, double *cl, double *cd,
                       int32_t *status, int32_t *bad_point);
/* Copies RES.DAT rows [first, first+count) of the current solve (the
 * device keeps the last fvm_batch_history_depth() rows). */
int32_t fvm_batch_history(fvm_batch *b, int32_t slot, int32_t first,
                          int32_t count, double *fres, int32_t *iresi,
                          double *fresi, double *cl, double *cd);
int32_t fvm_batch_history_depth(void);
/* The batch's CUDA stream (cudaStream_t), for callers that order their own
 * work or events after the batch's. */
void *fvm_batch_stream(fvm_batch *b);
/* Per-kernel device time: when on, CUDA events are recorded around every
 * kernel of each iteration and accumulated by kernel name. */
int32_t fvm_batch_timing(fvm_batch *b, int32_t on);
int32_t fvm_batch_timing_read(fvm_batch *b, int32_t max, char *names,
                              double *ms, int64_t *launches, int32_t *n);
/* Launches of this library's kernels since the batch was created. */
int64_t fvm_batch_launch_count(fvm_batch *b);
/* Test of the bounded device waits (no counterpart in the reference): one
 * stage-1 gradient pass of the pipelined kernel (FP32 batches) in which the
 * first block of every CTA is armed for its copies but the copies are never
 * issued.  Its consumers give up after budget_cycles clock cycles with
 * nothing in flight, and that block's mesh then reports FVM_ERR_TIMEOUT
 * through fvm_batch_poll; the context stays usable.  Gradients of the other
 * blocks are recomputed by the next iteration.  FVM_ERR_STATE when the
 * pipelined kernel does not fit the resident meshes. */
int32_t fvm_batch_test_wait_timeout(fvm_batch *b, int64_t budget_cycles);

/* Autotuner (no counterpart in the reference): runs `iters` timed
 * iterations (rounded up to whole graphs of 10 iterations, which is how
 * untimed steps run) of the resident solves under each form of the
 * iteration (the
 * gradient pass staged by bulk copies, by per-thread loads or walked per
 * vertex; or the fused gradient+flux pass; in one chain of kernels or
 * two overlapped ones) and keeps the fastest.  Every
 * form gives the same bits, so the tuning iterations are ordinary
 * iterations of the solves (they count toward each solve's iterations).
 * The first call and every fourth call after it time every candidate; the
 * calls in between skip a candidate whose last time was more than 1.25x
 * the best last time, and report that last time for it.
 * ms_per_iter[i] (i < max) receives candidate i's device time per
 * iteration (0 for a candidate that does not fit), *choice the candidate
 * kept: 0 bulk, 1 loads, 2 per vertex, 3 fused, 4 bulk (FP32) or loads
 * (FP64) in two overlapped chains, 5 fused in two chains, 6 and 7 as 4 in
 * four and eight chains. */
int32_t fvm_batch_tune(fvm_batch *b, int32_t iters, int32_t max, double *ms_per_iter,
                       int32_t *choice);
/* Sets the form of the iteration to a candidate of fvm_batch_tune (the
 * same codes); FVM_ERR_ARG for a form that does not fit this batch. */
int32_t fvm_batch_set_form(fvm_batch *b, int32_t form);

/* ------------------------------------------------------------------------
 * Serving (no counterpart in the reference, whose driver runs one solve per
 * process, main.f:42-76): a continuous-batching service on one GPU.  One
 * service thread owns a batch arena; solves submitted from any thread are
 * admitted in arrival order while the arena has room (their uploads run
 * beside the current step, and they join the batch when it ends), advanced
 * together `chunk` iterations at a time, and retired at their residual
 * drop or iteration cap, freeing room for the next.  With tune_every > 0 the
 * autotuner re-picks the form of the iteration every tune_every steps.
 * ---------------------------------------------------------------------- */
typedef struct fvm_server fvm_server;
int32_t fvm_serve_create(int32_t precision, const fvm_batch_caps *caps,
                         int32_t chunk, int32_t tune_every, fvm_server **out);
/* Queues a solve of up to nmax iterations stopping at fres <= minres.  The
 * block layout is built on the calling thread (submit from several threads
 * to prepare in parallel); the mesh arrays are copied.  keep_state = 1
 * keeps the final state for fvm_serve_state. */
int32_t fvm_serve_submit(fvm_server *s, const fvm_params *p,
                         const fvm_mesh *m, int32_t nmax, double minres,
                         int32_t keep_state, int64_t *ticket);
/* *state: 0 queued, 1 running, 2 done. */
int32_t fvm_serve_poll(fvm_server *s, int64_t ticket, int32_t *state);
/* Waits until the ticket is done or timeout_s seconds pass (<= 0: do not
 * wait; >= 1e9 or +inf: wait until done; NaN: FVM_ERR_ARG). */
int32_t fvm_serve_wait(fvm_server *s, int64_t ticket, double timeout_s,
                       int32_t *state);
/* Results of a done solve: status (FVM_OK, a stop of the method, or
 * FVM_ERR_CAPACITY for a solve larger than the empty arena), iterations,
 * last fres, cl, cd; tail[2] = mean cl, cd over the last 256 iterations;
 * times[3] = seconds queued, resident, in total. */
int32_t fvm_serve_result(fvm_server *s, int64_t ticket, int32_t *status,
                         int32_t *niter, double *fres, double *cl, double *cd,
                         double *tail, double *times);
/* Final state (prim(4,np), nut(np), driver order) of a done solve submitted
 * with keep_state. */
int32_t fvm_serve_state(fvm_server *s, int64_t ticket, double *prim,
                        double *nut);
/* Forgets a done solve. */
int32_t fvm_serve_release(fvm_server *s, int64_t ticket);
/* Checkpoint and restart of resident solves (the SOL file of
 * finalize.f:14-24 and the restart of initialize.f:91-103, for solves that
 * live in the service).  fvm_serve_checkpoint asks the service to stop a
 * running solve at the end of the current step: its ticket then finishes
 * with status FVM_CHECKPOINTED and keeps the solution, nu~, laminar and
 * total viscosity (what the next iteration starts from) and its iteration
 * count.  FVM_ERR_STATE when the ticket is queued or done.
 * fvm_serve_checkpoint_read copies them out (driver order; prim(4,np),
 * nut/mul/mu(np); any output may be NULL); results.write_sol writes
 * the SOL text from prim and nut.  fvm_serve_resume queues a solve that
 * starts from such a state at iteration iterlast: as in the reference's
 * restart, its first iteration sets the residual normaliser
 * (conres.f:25-29), and its state then evolves exactly as the
 * uninterrupted solve's. */
int32_t fvm_serve_checkpoint(fvm_server *s, int64_t ticket);
int32_t fvm_serve_checkpoint_read(fvm_server *s, int64_t ticket, double *prim,
                                  double *nut, double *mul, double *mu,
                                  int32_t *iter);
int32_t fvm_serve_resume(fvm_server *s, const fvm_params *p,
                         const fvm_mesh *m, int32_t nmax, double minres,
                         const double *prim, const double *nut,
                         const double *mul, const double *mu,
                         int32_t iterlast, int32_t keep_state,
                         int64_t *ticket);
/* out[6]: submitted, done, queued, running, steps, service status. */
int32_t fvm_serve_stats(fvm_server *s, int64_t *out);
/* out[5]: seconds the service thread spent admitting (between steps),
 * tuning, stepping (launching and waiting for the GPU; this includes
 * out[4]), retiring, and admitting beside a running step. */
int32_t fvm_serve_times(fvm_server *s, double *out);
/* Stops the service thread after its current step and frees everything.
 * Solves not yet done end with FVM_ERR_STATE, so threads blocked in
 * fvm_serve_wait wake up; destroy returns only after every fvm_serve_* call
 * already in progress on other threads has returned.  No fvm_serve_* call
 * on this server may start once destroy has been called. */
int32_t fvm_serve_destroy(fvm_server *s);

/* Layout statistics of a mesh after renumbering (no GPU needed):
 * out[0] blocks, [1] interior edge entries (cut edges counted in both
 * blocks), [2] triangle entries (block and halo), [3] max slots of a
 * block, [4] max triangles of a block, [5] boundary edge entries, [6] max
 * triangles of a block and its halo, [7] max own + halo vertices, [8] halo
 * vertices, [9] violations of the layout's invariants (0 for a valid
 * layout).  out has 10 elements. */
int32_t fvm_layout_stats(const fvm_mesh *m, int64_t *out);

#ifdef __cplusplus
}
#endif

#endif /* FVM_GPU_H */
