// fvm_setup.cu -- FP64 set-up kernels, run once per mesh.  Compiled with
// --fmad=false so the results equal the serial FP64 arithmetic.
#include <climits>
#include <cstddef>

#include <cuda_runtime.h>

#include "fvm_launch.h"

namespace fvm {

// (ct, st, length) of every edge face from ds, as roe_flux.f:18-20 /
// kfvs_flux.f:16-18 / hllc_flux.f:18-20 compute them on every call.
__global__ void k_edge_csl(const double2 *__restrict__ ds, D4 *__restrict__ csl, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 d = ds[i];
  const double length = sqrt(d.x * d.x + d.y * d.y);
  D4 o;
  o.x = d.x / length;
  o.y = d.y / length;
  o.z = length;
  o.w = 0.0;
  csl[i] = o;
}

// dtlength.f:21-44: per triangle altitudes, min-scattered to its vertices.
// drmin holds positive doubles, whose bit patterns order like integers.
__global__ void k_dtlength(int nt, const double2 *__restrict__ coord, const int *__restrict__ elem,
                           const double *__restrict__ elarea, unsigned long long *drmin) {
  const int it = blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= nt) return;
  const int n1 = elem[3 * it] - 1, n2 = elem[3 * it + 1] - 1, n3 = elem[3 * it + 2] - 1;
  const double2 c1 = coord[n1], c2 = coord[n2], c3 = coord[n3];
  const double ea = elarea[it];
  const double dx1 = c2.x - c3.x, dy1 = c2.y - c3.y;
  const double h1 = 2.0 * ea / sqrt(dx1 * dx1 + dy1 * dy1);
  const double dx2 = c3.x - c1.x, dy2 = c3.y - c1.y;
  const double h2 = 2.0 * ea / sqrt(dx2 * dx2 + dy2 * dy2);
  const double dx3 = c1.x - c2.x, dy3 = c1.y - c2.y;
  const double h3 = 2.0 * ea / sqrt(dx3 * dx3 + dy3 * dy3);
  atomicMin(drmin + n1, (unsigned long long)__double_as_longlong(h1));
  atomicMin(drmin + n2, (unsigned long long)__double_as_longlong(h2));
  atomicMin(drmin + n3, (unsigned long long)__double_as_longlong(h3));
}

__global__ void k_fill(double *a, double v, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = v;
}

// wall_dist.f:28-61 and 87-92: each thread one point, the solid edges
// staged through shared memory in tiles.  The result is a minimum, which
// does not depend on the order the candidates are visited.
constexpr int kWallTile = 256;
__global__ void __launch_bounds__(256) k_wall_dist(int np, int nsedge, const double2 *__restrict__ coord,
                                                   const int2 *__restrict__ sedge,
                                                   const int *__restrict__ ptype, int bugcompat,
                                                   double *__restrict__ wd) {
  __shared__ double2 s_a[kWallTile], s_b[kWallTile];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const double2 ci = (i < np) ? coord[i] : make_double2(0.0, 0.0);
  double w = 1.0e10;
  for (int t0 = 0; t0 < nsedge; t0 += kWallTile) {
    __syncthreads();
    for (int k = threadIdx.x; k < kWallTile && t0 + k < nsedge; k += blockDim.x) {
      const int2 e = sedge[t0 + k];
      s_a[k] = coord[e.x];
      s_b[k] = coord[e.y];
    }
    __syncthreads();
    const int nk = min(kWallTile, nsedge - t0);
    for (int k = 0; k < nk; k++) {
      const double2 a = s_a[k], b = s_b[k];
      const double dx1 = a.x - ci.x, dy1 = a.y - ci.y;
      const double ds1 = sqrt(dx1 * dx1 + dy1 * dy1);
      w = (ds1 < w) ? ds1 : w;
      const double dx2 = b.x - ci.x, dy2 = b.y - ci.y;
      const double ds2 = sqrt(dx2 * dx2 + dy2 * dy2);
      w = (ds2 < w) ? ds2 : w;
      const double dx3 = b.x - a.x;
      const double dy3 = bugcompat ? (b.x - a.x) : (b.y - a.y);
      const double dl2 = dx3 * dx3 + dy3 * dy3;
      const double xi = -(dx1 * dx3 + dy1 * dy3) / dl2;
      if (xi >= 0.0 && xi <= 1.0) {
        const double xp = a.x + xi * dx3;
        const double yp = a.y + xi * dy3;
        const double ex = ci.x - xp, ey = ci.y - yp;
        const double dsperp = sqrt(ex * ex + ey * ey);
        w = (dsperp < w) ? dsperp : w;
      }
    }
  }
  if (i < np) wd[i] = (ptype[i] == 3) ? 1.0 : w;
}

cudaError_t launch_edge_csl(const double2 *ds, D4 *csl, int n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_edge_csl<<<(n + 255) / 256, 256, 0, s>>>(ds, csl, n);
  return cudaGetLastError();
}

cudaError_t launch_dtlength(int np, int nt, const double2 *coord, const int *elem,
                            const double *elarea, double *drmin, cudaStream_t s) {
  if (np <= 0) return cudaSuccess;
  k_fill<<<(np + 255) / 256, 256, 0, s>>>(drmin, 1.0e15, np);
  if (nt > 0)
    k_dtlength<<<(nt + 255) / 256, 256, 0, s>>>(nt, coord, elem, elarea,
                                               reinterpret_cast<unsigned long long *>(drmin));
  return cudaGetLastError();
}

cudaError_t launch_wall_dist(int np, int nsedge, const double2 *coord, const int2 *sedge,
                             const int *ptype, int bugcompat, double *wd, cudaStream_t s) {
  if (np <= 0) return cudaSuccess;
  k_wall_dist<<<(np + 255) / 256, 256, 0, s>>>(np, nsedge, coord, sedge, ptype, bugcompat, wd);
  return cudaGetLastError();
}

// Driver-order FP64 arrays (k values per vertex) to and from a mesh's
// per-vertex arrays in arena order (rows of `stride` bytes, values of type R
// from column c0): orig holds each arena vertex's driver index (1-based).
// Conversions round to nearest, as the host's would (this unit does not
// flush subnormals).
template <typename R>
__global__ void k_get_vertex(double *dst, const unsigned char *src, size_t stride,
                             const int *__restrict__ orig, int np, int k, int c0) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < np; v += gridDim.x * blockDim.x) {
    const R *q = reinterpret_cast<const R *>(src + (size_t)v * stride) + c0;
    double *d = dst + (size_t)(orig[v] - 1) * k;
    for (int c = 0; c < k; c++) d[c] = (double)q[c];
  }
}

// The same transfers into / out of one of three buffers chosen on the
// device by *sel (a mesh's state phase or nu~ phase in its control block),
// so the host need not read the control block first.  off: the mesh's
// first row, in bytes.
template <typename R>
__global__ void k_put_vertex_sel(unsigned char *b0, unsigned char *b1, unsigned char *b2,
                                 const int *sel, size_t off, size_t stride,
                                 const double *__restrict__ src, const int *__restrict__ orig,
                                 int np, int k) {
  const int i = *sel;
  unsigned char *dst = (i == 0 ? b0 : i == 1 ? b1 : b2) + off;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < np; v += gridDim.x * blockDim.x) {
    const double *q = src + (size_t)(orig[v] - 1) * k;
    R *d = reinterpret_cast<R *>(dst + (size_t)v * stride);
    for (int c = 0; c < k; c++) d[c] = (R)q[c];
  }
}

template <typename R>
__global__ void k_get_vertex_sel(double *dst, const unsigned char *b0, const unsigned char *b1,
                                 const unsigned char *b2, const int *sel, size_t off,
                                 size_t stride, const int *__restrict__ orig, int np, int k,
                                 int c0) {
  const int i = *sel;
  const unsigned char *src = (i == 0 ? b0 : i == 1 ? b1 : b2) + off;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < np; v += gridDim.x * blockDim.x) {
    const R *q = reinterpret_cast<const R *>(src + (size_t)v * stride) + c0;
    double *d = dst + (size_t)(orig[v] - 1) * k;
    for (int c = 0; c < k; c++) d[c] = (double)q[c];
  }
}

// A mesh's control block set for a new state (what 0: iteration and
// iterlast = n, residual normaliser cleared, inactive) or for a start
// (what 1: up to n iterations stopping at fres <= minres), on the device.
__global__ void k_ctl_update(MeshCtl *c, int what, int n, double minres) {
  if (what == 0) {
    c->iter = n;
    c->iterlast = n;
    c->fres1 = 0.0;
    c->active = 0;
  } else {
    c->active = n > 0 ? 1 : 0;
    c->n_done = 0;
    c->n_max = n;
    c->minres = minres;
  }
  c->err = 0;
  c->err_point = INT_MAX;
}

cudaError_t launch_put_vertex_sel(int rsz, unsigned char *const b[3], const int *sel, size_t off,
                                  size_t stride, const double *src, const int *orig, int np,
                                  int k, cudaStream_t s) {
  if (np <= 0) return cudaSuccess;
  const int g = (np + 255) / 256;
  if (rsz == 8)
    k_put_vertex_sel<double><<<g, 256, 0, s>>>(b[0], b[1], b[2], sel, off, stride, src, orig, np, k);
  else
    k_put_vertex_sel<float><<<g, 256, 0, s>>>(b[0], b[1], b[2], sel, off, stride, src, orig, np, k);
  return cudaGetLastError();
}

cudaError_t launch_get_vertex_sel(int rsz, double *dst, unsigned char *const b[3], const int *sel,
                                  size_t off, size_t stride, const int *orig, int np, int k,
                                  int c0, cudaStream_t s) {
  if (np <= 0) return cudaSuccess;
  const int g = (np + 255) / 256;
  if (rsz == 8)
    k_get_vertex_sel<double><<<g, 256, 0, s>>>(dst, b[0], b[1], b[2], sel, off, stride, orig, np, k, c0);
  else
    k_get_vertex_sel<float><<<g, 256, 0, s>>>(dst, b[0], b[1], b[2], sel, off, stride, orig, np, k, c0);
  return cudaGetLastError();
}

cudaError_t launch_ctl_update(MeshCtl *c, int what, int n, double minres, cudaStream_t s) {
  k_ctl_update<<<1, 1, 0, s>>>(c, what, n, minres);
  return cudaGetLastError();
}

// every row of a mesh's per-vertex array set to the same k values
template <typename R>
__global__ void k_fill_vertex(unsigned char *dst, size_t stride, int np, int k, double a0,
                              double a1, double a2, double a3) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < np; v += gridDim.x * blockDim.x) {
    R *d = reinterpret_cast<R *>(dst + (size_t)v * stride);
    const double a[4] = {a0, a1, a2, a3};
    for (int c = 0; c < k; c++) d[c] = (R)a[c];
  }
}

cudaError_t launch_fill_vertex(int rsz, unsigned char *dst, size_t stride, int np, int k,
                               const double *values, cudaStream_t s) {
  if (np <= 0) return cudaSuccess;
  if (k < 1 || k > 4) return cudaErrorInvalidValue;
  double a[4] = {0.0, 0.0, 0.0, 0.0};
  for (int c = 0; c < k; c++) a[c] = values[c];
  const int g = (np + 255) / 256;
  if (rsz == 8) k_fill_vertex<double><<<g, 256, 0, s>>>(dst, stride, np, k, a[0], a[1], a[2], a[3]);
  else k_fill_vertex<float><<<g, 256, 0, s>>>(dst, stride, np, k, a[0], a[1], a[2], a[3]);
  return cudaGetLastError();
}

cudaError_t launch_get_vertex(int rsz, double *dst, const unsigned char *src, size_t stride,
                              const int *orig, int np, int k, int c0, cudaStream_t s) {
  if (np <= 0) return cudaSuccess;
  const int g = (np + 255) / 256;
  if (rsz == 8) k_get_vertex<double><<<g, 256, 0, s>>>(dst, src, stride, orig, np, k, c0);
  else k_get_vertex<float><<<g, 256, 0, s>>>(dst, src, stride, orig, np, k, c0);
  return cudaGetLastError();
}

// The work list's blocks copied in work-list order (the per-block kernels
// then read a block with one load instead of an index load and the block's).
__global__ void k_gather_blocks(const int *__restrict__ work, const BlockInfo *__restrict__ blocks,
                                BlockInfo *__restrict__ out, int n) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w < n) out[w] = blocks[work[w]];
}

cudaError_t launch_gather_blocks(const int *work, const BlockInfo *blocks, BlockInfo *out, int n,
                                 cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_gather_blocks<<<(n + 255) / 256, 256, 0, s>>>(work, blocks, out, n);
  return cudaGetLastError();
}

}  // namespace fvm
