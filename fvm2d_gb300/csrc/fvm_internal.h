// fvm_internal.h -- device data layout shared by the host runtime and the
// kernels of the GB300 fvm2d hot path.
//
// Layout in HBM ("arena"): every mesh of a batch owns contiguous ranges of
// the vertex, block, block-edge, block-boundary, block-triangle and
// incidence arrays.  Vertices are renumbered so that each block of at most
// kBlockVerts consecutive vertices is a compact patch of the mesh graph
// (recursive BFS bisection).  One CTA processes one block:
//
//   gradient pass (green_gauss.f:23-39, tri_visc :132-194):
//     phase 1  each triangle touching the block -> dxt,dyt (+ viscous terms)
//              into shared memory, computed once per block
//     phase 2  each vertex sums its triangles in original triangle order
//   flux pass (residu.f:37-88 + update.f:17-35):
//     phase 1  each edge touching the block -> recon + Riemann flux into
//              shared memory (edges cut by the block boundary are computed
//              by both blocks: no atomics, no global flux buffer)
//     phase 2  each vertex sums its edge fluxes in original iedge order,
//              then solid and farfield contributions in beindx order, then
//              applies the RK stage and writes the next state buffer.
//
// Summation order per vertex equals the Fortran serial order, so the FP64
// build (no FMA contraction) reproduces the reference arithmetic exactly.
#pragma once

#include <stdint.h>

namespace fvm {

constexpr int kBlockVerts = 256;      // vertices (and threads) per block
constexpr int kMaxMeshes = 4096;

// incidence-list entry bits (uint16)
constexpr uint16_t kSlotMask = 0x1fff;     // slot in the block's list
constexpr uint16_t kNegBit = 0x8000;       // edge entry: subtract (vertex is n2)
constexpr uint16_t kSolidBit = 0x4000;     // boundary entry: components 2,3 only
constexpr uint16_t kFarBit = 0x2000;       // boundary entry: farfield
constexpr int kTriPosShift = 14;           // triangle entry: vertex position 0..2

// per-vertex flag bits
constexpr uint8_t kVtxSolid = 1;
constexpr uint8_t kVtxFarfield = 2;

struct BlockInfo {          // 16 ints, one per CTA
  int mesh;                 // mesh slot
  int v0, nv;               // arena vertex range (local slots [0, nv))
  int e0, ne;               // interior edge entries (be_* arrays)
  int b0, nb;               // boundary edges (bb_* arrays); 2 slots each
  int t0, nt;               // triangles touching the block (bt_* arrays)
  int part;                 // index of this block's partial-sum record
  int nt2;                  // nt + triangles touching only the halo (bt_* from t0)
  int h0, nh;               // halo vertices (halo_ids): local slots [nv, nv+nh)
  int hp0;                  // halo incidence pointers (hl_ptr, nh+1 entries)
  int vt0, nvt;             // the block's vertex-triangle incidence (vt_list range)
};

// Vertex ranges of meshes start on multiples of kVertAlign, so per-vertex
// arrays of 2- to 16-byte elements can be copied block by block in 16-byte
// units (bulk copies); every per-vertex array has kVertAlign entries of
// slack at its end for the rounded-up copies.
constexpr int kVertAlign = 8;

// Most chains of kernels an iteration runs side by side (parts of the
// work list split at mesh boundaries).
constexpr int kMaxChains = 8;

#ifdef __CUDACC__
#define FVM_HD __host__ __device__
#else
#define FVM_HD
#endif

// Shared memory of the bulk-copy gradient pass (FP32): the block's triangle
// records (geometry and the ends' local slots, 32 B, overwritten in place
// by the triangle sums), the viscous terms (9 values), the vertices'
// incidence ranges and the incidence list (both copied in 16-byte units),
// the states of the block's own vertices and the ids of its halo vertices.
struct GradBulkLayout {
  uint32_t geo, vis, vtr, vtl, pv, halo, total;
};
FVM_HD inline uint32_t fvm_up16(uint32_t x) { return (x + 15u) & ~15u; }
FVM_HD inline GradBulkLayout grad_bulk_layout(int max_tri, int max_halo, bool viscous) {
  GradBulkLayout l;
  const uint32_t mt = (uint32_t)max_tri;
  l.geo = 0;
  l.vis = fvm_up16(mt * 32u);
  l.vtr = l.vis + (viscous ? fvm_up16(mt * 36u) : 0u);
  l.vtl = l.vtr + fvm_up16((uint32_t)(kBlockVerts + kVertAlign) * 8u);
  l.pv = l.vtl + fvm_up16((3u * mt + 16u) * 2u);
  l.halo = l.pv + (uint32_t)kBlockVerts * 16u;
  l.total = l.halo + fvm_up16((uint32_t)max_halo * 4u);
  return l;
}

// One stage of the pipelined gradient pass (FP32): everything a consumer
// group needs for one block, filled by the producer warp's bulk copies
// (triangle records, incidence ranges and list, own states, halo ids, the
// own vertices' (1/6)/mcarea and drmin) plus the halo states the consumers
// gather themselves.  Stages are 128-byte aligned.
struct GradPipeLayout {
  uint32_t geo, vis, vtr, vtl, pv, hst, hid, ais, drm, stage;
};
FVM_HD inline GradPipeLayout grad_pipe_layout(int max_tri, int max_halo, bool viscous) {
  GradPipeLayout l;
  const uint32_t mt = (uint32_t)max_tri, mh = (uint32_t)max_halo;
  const uint32_t nvr = (uint32_t)(kBlockVerts + kVertAlign);
  l.geo = 0;
  l.vis = fvm_up16(mt * 32u);
  l.vtr = l.vis + (viscous ? fvm_up16(mt * 36u) : 0u);
  l.vtl = l.vtr + fvm_up16(nvr * 8u);
  l.pv = l.vtl + fvm_up16((3u * mt + 16u) * 2u);
  l.hst = l.pv + (uint32_t)kBlockVerts * 16u;
  l.hid = l.hst + fvm_up16(mh * 16u);
  l.ais = l.hid + fvm_up16((mh + 8u) * 4u);   // copied from a 16-byte boundary
  l.drm = l.ais + fvm_up16(nvr * 4u);
  l.stage = (l.drm + fvm_up16(nvr * 4u) + 127u) & ~127u;
  return l;
}
constexpr int kPipeMaxStages = 8;
// Shared memory of a pipelined kernel's CTA besides its stages (barriers,
// stage headers, flags)
constexpr uint32_t kPipeStaticSmem = 2048;

// Per-mesh constants (read-only during a solve).  Mirrors fvm_params plus
// arena placement.
// FP32 copies of a mesh's constants (each the FP64 value rounded once, as a
// conversion in the kernel would give), so the FP32 kernels convert nothing.
struct MeshConstF {
  float gamma, gamma1, gas_const, pi, prandtl, prandtl_turb;
  float albada11, albada12, albada21, albada22, epsilon;
  float cb1, cb2, sigma_sa, kolm, cw1, cw2, cw3, cv1, cv2;
  float cv11, cw31, cw32, kolm2, cb2sig1, cb2sig2;
  float mach_inf, aoa, rey, cfl;
  float q_inf, r_inf, p_inf, t_inf, u_inf, v_inf, a_inf, sconst, nut_inf;
  float airk[3], birk[3];
};

struct MeshConst {
  int iflow, iflux, ilimit, vortex, bugcompat, precision;
  int v0, nv;                       // vertex range
  int blk0, nblk;                   // range in the block table
  int sw0, nsw;                     // solid edges (sw_nodes)
  int orig123[3];                   // arena ids of driver vertices 1,2,3
  int pad0;
  double gamma, gamma1, gas_const, pi, prandtl, prandtl_turb;
  double albada11, albada12, albada21, albada22, epsilon;
  double cb1, cb2, sigma_sa, kolm, cw1, cw2, cw3, cv1, cv2;
  double cv11, cw31, cw32, kolm2, cb2sig1, cb2sig2;
  double mach_inf, aoa, rey, cfl;
  double q_inf, r_inf, p_inf, t_inf, u_inf, v_inf, a_inf, sconst, nut_inf;
  double xref, yref;
  double airk[3], birk[3];
  double sin_aoa, cos_aoa;          // host libm values (clcd.f:45-46)
  MeshConstF f;
};

// A mesh constant in the kernel's precision: the FP32 copy for R = float.
#define MCR(R, name) (sizeof(R) == 4 ? R(mc.f.name) : R(mc.name))

// Per-mesh mutable control block.
struct MeshCtl {
  int active;        // 1 while iterating
  int phase;         // state buffer holding the current solution (0..2)
  int nphase;        // nut buffer holding the current nu~ (0..1)
  int iter;          // iteration counter (main.f iter)
  int iterlast;      // iteration whose residual sets fres1
  int n_done;        // iterations completed in this iterate call
  int n_max;         // iterations allowed in this iterate call
  int err;           // FVM_ERR_* (0 = none)
  int err_point;     // min driver index (1-based) of a non-positive point
  int hist_off;      // first history row of this slot
  int hist_cap;      // rows of the slot's history ring
  int pad;
  double minres, fres1, fres, fresi, cl, cd;
  int iresi, pad2;
};

struct BlockPartial {       // conres.f:14-22 partials of one block
  double sumsq;
  double maxabs;
  int argmax;               // driver index (1-based); INT_MAX if none
  int pad;
};

template <typename R>
struct alignas(4 * sizeof(R)) R4 {
  R x, y, z, w;
};
template <typename R>
struct alignas(8 * sizeof(R) > 32 ? 32 : 8 * sizeof(R)) Grad {
  R qx[4];
  R qy[4];
};
struct alignas(32) D4 {
  double x, y, z, w;
};
// FP32 copies of FP64 geometric differences, rounded once (used by the FP32
// kernels so their hot loops execute no FP64 instruction)
struct alignas(16) TriGeo32 {
  float dbxx[3], dbyy[3];   // green_gauss.f:108-113: y2-y3, y3-y1, y1-y2 / x3-x2, x1-x3, x2-x1
  float areat;              // 0.25/elarea (green_gauss.f:180)
  uint32_t loc;             // the three ends' block-local slots (kTriLocBits each), or kTriNoLoc
};
// Block-local slot of a vertex: own vertices 0..nv-1, then the block's halo
// vertices (halo_ids order).  Three slots of kTriLocBits bits fit one word
// when the block has at most kTriLocMax own + halo vertices.
constexpr int kTriLocBits = 10;
constexpr int kTriLocMax = 1 << kTriLocBits;
constexpr uint32_t kTriNoLoc = 0xffffffffu;

// One interior edge entry of a block for the FP32 kernels (its ends are
// be_nodes): the FP64 edge vector and dual-face normal ds rounded once to
// FP32; 16 bytes, one load.  The flux pass forms ct, st, len from ds
// (flux.f:10-13) itself.
struct alignas(16) EdgeGeo32 {
  float4 v;            // x(n2)-x(n1), y(n2)-y(n1), ds (flength.f:38-39)
};

// Device pointers of an arena (all arena-global indices).
template <typename R>
struct ArenaPtrs {
  // vertices
  R4<R> *st[3];          // state buffers (rho, u, v, p)
  Grad<R> *grad;         // qx, qy of the last gradient pass
  R4<R> *resv;           // viscous residual part (components 1..3 = res 2..4)
  R4<R> *res;            // residual (per-routine calls)
  R *dt, *mu, *mul;
  R *nut[2];
  const double2 *coord;
  const double *ais;     // (1/6)/mcarea
  const double *cvarea, *drmin, *wd;
  const int *orig;       // driver index (1-based) of each vertex
  const uint8_t *vflag;
  // incidence: per vertex {begin, end} into the list arrays
  const int2 *ve_rng;
  const uint16_t *ve_list;
  const int2 *vt_rng;
  const uint16_t *vt_list;
  // block entries
  const BlockInfo *blocks;
  const BlockInfo *wblocks;  // blocks[work[w]] for each w (copies in work-list order)
  const int2 *be_nodes;   // interior edge entries (n1, n2)
  const double2 *be_ds;   // ds of the edge (flength.f:38-39)
  const D4 *be_csl;       // (ct, st, length) precomputed in FP64
  const int4 *bb_nodes;   // boundary entries (n1, n2, type, -)
  const int4 *bt_nodes;   // triangle entries (n1, n2, n3, arena triangle)
  const double *elarea;   // per arena triangle
  const EdgeGeo32 *be_g32; // FP32 path: edge vector and ds of each edge entry (ends: be_nodes)
  const float *ais32, *cvarea32, *drmin32, *wd32;   // FP32 path: per-vertex copies
  const TriGeo32 *tri_g32; // FP32 path: per triangle entry of the blocks (bt_* order)
  // solid edges per mesh for clcd (n1, n2) in beindx order
  const int2 *sw_nodes;
  // fused gradient+flux pass: local slots of edge ends, halo vertices and
  // their triangle incidence (slot | pos << 14 in the block's bt list)
  const uint32_t *be_loc;
  const int *halo_ids;
  const int *hl_ptr;      // per block, nh+1 absolute offsets into hl_list
  const uint16_t *hl_list;
  // all-edge incidence (limitgrad.f loops over netot edges)
  const int2 *va_rng;
  const int *va_list;     // other vertex | (is n2) << 31
  const float2 *va_w;     // FP32: Green-Gauss stencil weight of each va_list entry
  const double *va_dsl;   // |ds| of the edge of each va_list entry (shockind.f:36)
  // per mesh
  const MeshConst *mc;
  MeshCtl *ctl;
  BlockPartial *part;
  // history rows
  double *h_fres, *h_fresi, *h_cl, *h_cd;
  int *h_iresi;
  // block work list (indices into blocks[]) and its length
  const int *work;
  const int *nwork;    // [0] blocks in the work list, [k] end of part k (k = 1..kMaxChains)
  int wpart;           // 0 the whole list, k part k
  const int *mesh_part;  // per slot: the part holding the mesh's blocks
  int nslots;             // mesh slots (monitor grid)
};

}  // namespace fvm
