// fvm_geom_gpu.cu -- the driver geometry chain of src/geometric.f:15-60 on
// the GPU, equal to the host restatement (fvm_geometry.cpp) array for array
// and bit for bit.  Compiled with --fmad=false: every floating point
// operation is the IEEE operation the host performs, in the same order.
//
// Orders that define the driver's numbering are kept by construction, not
// by atomics: each point's element list is sorted ascending (the order of
// el_surr_point.f's fill loop); each point walks its elements in that order
// to find its neighbours in first-seen order (pt_surr_pt.f) and to number
// its edges (create_edge.f: point by point, edge ids from an exclusive
// scan of the per-point counts); per-point sums (areas.f) run over the
// point's elements in ascending order, as the host's element loop adds
// them; order-preserving compactions (exclusive scans of flags) build
// iedge, beindx and spts; dsb (flength.f:51-60) sums over the boundary
// edges in edge order in one thread.
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "../../include/fvm_gpu.h"
#include "fvm_geom_gpu.h"
#include "fvm_launch.h"

namespace fvm {
namespace {

constexpr int kT = 256;          // threads per CTA of the per-item kernels
constexpr int kScanItems = 1024; // items per CTA of the scan (4 per thread)

inline int nblocks(int64_t n) { return (int)((n + kT - 1) / kT); }

enum : int { kErrDegenerate = 1, kErrNoLeft = 2, kErrNegArea = 4, kErrNonPositive = 8 };

// ---- exclusive scan (out[0..n], out[n] = total) ---------------------------
__global__ void k_scan_blocks(const int *__restrict__ in, int *__restrict__ out, int n,
                              int *__restrict__ bsum) {
  __shared__ int wsum[kT / 32];
  const int base = blockIdx.x * kScanItems + threadIdx.x * 4;
  int v[4], s = 0;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    v[i] = base + i < n ? in[base + i] : 0;
    s += v[i];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int w = lane < kT / 32 ? wsum[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kT / 32) wsum[lane] = w;
  }
  __syncthreads();
  int excl = x - s + (warp ? wsum[warp - 1] : 0);
#pragma unroll
  for (int i = 0; i < 4; i++) {
    if (base + i < n) out[base + i] = excl;
    excl += v[i];
  }
  if (threadIdx.x == kT - 1) bsum[blockIdx.x] = excl;
}

__global__ void k_scan_add(int *__restrict__ out, int n, const int *__restrict__ boff) {
  const int base = blockIdx.x * kScanItems + threadIdx.x * 4;
  const int add = boff[blockIdx.x];
#pragma unroll
  for (int i = 0; i < 4; i++)
    if (base + i < n) out[base + i] += add;
}

__global__ void k_scan_total(const int *__restrict__ in, int *__restrict__ out, int n) {
  out[n] = n > 0 ? out[n - 1] + in[n - 1] : 0;
}

// ---- per-triangle and per-point passes -----------------------------------
// tri_orient.f:15-41
__global__ void k_orient(int nt, const double2 *__restrict__ c, int *__restrict__ e, int *err) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const int p1 = e[3 * t] - 1, p2 = e[3 * t + 1] - 1, p3 = e[3 * t + 2] - 1;
  const double dx1 = c[p2].x - c[p1].x, dy1 = c[p2].y - c[p1].y;
  const double dx2 = c[p3].x - c[p2].x, dy2 = c[p3].y - c[p2].y;
  const double cross = dx1 * dy2 - dx2 * dy1;
  if (cross == 0.0) atomicOr(err, kErrDegenerate);
  if (cross < 0.0) {
    const int tmp = e[3 * t + 1];
    e[3 * t + 1] = e[3 * t + 2];
    e[3 * t + 2] = tmp;
  }
}

__global__ void k_count_corners(int nt, const int *__restrict__ e, int *cnt) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
#pragma unroll
  for (int k = 0; k < 3; k++) atomicAdd(cnt + e[3 * t + k] - 1, 1);
}

__global__ void k_fill_corners(int nt, const int *__restrict__ e, const int *__restrict__ ptr,
                               int *fill, int *__restrict__ esup) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const int p = e[3 * t + k] - 1;
    esup[ptr[p] + atomicAdd(fill + p, 1)] = t;
  }
}

// el_surr_point.f fills each point's list in ascending element order
__global__ void k_sort_lists(int np, const int *__restrict__ ptr, int *__restrict__ a) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  const int j0 = ptr[p], j1 = ptr[p + 1];
  for (int j = j0 + 1; j < j1; j++) {
    const int x = a[j];
    int i = j - 1;
    while (i >= j0 && a[i] > x) {
      a[i + 1] = a[i];
      i--;
    }
    a[i + 1] = x;
  }
}

// pt_surr_pt.f:13-33 and create_edge.f:9-18: point p walks its elements in
// ascending order, each element's corners in order; a corner q != p not met
// before in the walk is p's next neighbour, and q > p numbers the next edge
// of p.  FILL = 0 counts the edges, FILL = 1 writes them from eptr[p].
template <int FILL>
__global__ void k_point_edges(int np, const int *__restrict__ ptr, const int *__restrict__ esup,
                              const int *__restrict__ e, int *__restrict__ ecnt,
                              const int *__restrict__ eptr, int *__restrict__ edge) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  const int j0 = ptr[p], j1 = ptr[p + 1];
  int ne = 0, out = FILL ? eptr[p] : 0;
  for (int j = j0; j < j1; j++) {
    const int t = esup[j];
    for (int k = 0; k < 3; k++) {
      const int q = e[3 * t + k] - 1;
      if (q == p) continue;
      bool seen = false;
      for (int jj = j0; jj <= j && !seen; jj++) {
        const int tt = esup[jj];
        const int kend = jj < j ? 3 : k;
        for (int kk = 0; kk < kend; kk++)
          if (e[3 * tt + kk] - 1 == q) seen = true;
      }
      if (seen || q < p) continue;
      if (FILL) {
        edge[2 * out] = p + 1;
        edge[2 * out + 1] = q + 1;
        out++;
      }
      ne++;
    }
  }
  if (!FILL) ecnt[p] = ne;
}

// el_surr_edge.f:9-33: the triangle holding (n1, n2) counter-clockwise is
// the left one (the last match over n1's elements in ascending order); a
// boundary edge is turned so that its triangle is on the left
__global__ void k_edge_neighbours(int ne, const int *__restrict__ ptr, const int *__restrict__ esup,
                                  const int *__restrict__ e, int *__restrict__ edge,
                                  int *__restrict__ edneigh) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ne) return;
  const int n1 = edge[2 * i], n2 = edge[2 * i + 1];
  int left = 0, right = 0;
  for (int j = ptr[n1 - 1]; j < ptr[n1]; j++) {
    const int t = esup[j];
    const int a = e[3 * t], b = e[3 * t + 1], c = e[3 * t + 2];
    if ((n1 == a && n2 == b) || (n1 == b && n2 == c) || (n1 == c && n2 == a)) left = t + 1;
    if ((n2 == a && n1 == b) || (n2 == b && n1 == c) || (n2 == c && n1 == a)) right = t + 1;
  }
  if (left == 0) {
    left = right;
    right = 0;
    edge[2 * i] = n2;
    edge[2 * i + 1] = n1;
  }
  edneigh[2 * i] = left;
  edneigh[2 * i + 1] = right;
}

__device__ __forceinline__ double dmax(double a, double b) { return b > a ? b : a; }

// tri_coord.f (centroid or circumcentre) and areas.f's triangle areas
__global__ void k_triangles(int nt, int cell_type, const double2 *__restrict__ c,
                            const int *__restrict__ e, double2 *__restrict__ tc,
                            double *__restrict__ elarea) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const int n1 = e[3 * t] - 1, n2 = e[3 * t + 1] - 1, n3 = e[3 * t + 2] - 1;
  const double x1 = c[n1].x, y1 = c[n1].y, x2 = c[n2].x, y2 = c[n2].y, x3 = c[n3].x,
               y3 = c[n3].y;
  double2 o;
  if (cell_type == FVM_CELL_MEDIAN) {
    o.x = (x1 + x2 + x3) / 3.0;
    o.y = (y1 + y2 + y3) / 3.0;
  } else {
    const double l1 = (x2 - x3) * (x2 - x3) + (y2 - y3) * (y2 - y3);
    const double l2 = (x3 - x1) * (x3 - x1) + (y3 - y1) * (y3 - y1);
    const double l3 = (x1 - x2) * (x1 - x2) + (y1 - y2) * (y1 - y2);
    const double beta1 = dmax(0.0, l2 + l3 - l1);
    const double beta2 = dmax(0.0, l3 + l1 - l2);
    const double beta3 = dmax(0.0, l1 + l2 - l3);
    const double det = (x2 - x1) * (y3 - y1) - (x3 - x1) * (y2 - y1);
    const double b1 = 0.5 * ((x2 - x1) * (x2 + x1) + (y2 - y1) * (y2 + y1));
    const double b2 = 0.5 * ((x3 - x1) * (x3 + x1) + (y3 - y1) * (y3 + y1));
    const double xc = ((y3 - y1) * b1 - (y2 - y1) * b2) / det;
    const double yc = (-(x3 - x1) * b1 + (x2 - x1) * b2) / det;
    if (beta1 == 0.0) {
      o.x = 0.5 * (x2 + x3);
      o.y = 0.5 * (y2 + y3);
    } else if (beta2 == 0.0) {
      o.x = 0.5 * (x3 + x1);
      o.y = 0.5 * (y3 + y1);
    } else if (beta3 == 0.0) {
      o.x = 0.5 * (x1 + x2);
      o.y = 0.5 * (y1 + y2);
    } else {
      o.x = xc;
      o.y = yc;
    }
  }
  tc[t] = o;
  const double dx1 = x2 - x1, dy1 = y2 - y1;
  const double dx2 = x3 - x1, dy2 = y3 - y1;
  elarea[t] = 0.5 * (dx1 * dy2 - dx2 * dy1);
}

// areas.f: mcarea (a third of each triangle) and, for Barth cells, the
// polygon of the point's corner in each triangle, summed over the point's
// triangles in ascending order
__global__ void k_point_areas(int np, int cell_type, const int *__restrict__ ptr,
                              const int *__restrict__ esup, const int *__restrict__ e,
                              const double2 *__restrict__ c, const double2 *__restrict__ tc,
                              const double *__restrict__ elarea, double *__restrict__ mcarea,
                              double *__restrict__ cvarea, int *err) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  double m = 0.0, cv = 0.0;
  for (int j = ptr[p]; j < ptr[p + 1]; j++) {
    const int t = esup[j];
    const double a3 = elarea[t] / 3.0;
    m = m + a3;
    if (cell_type == FVM_CELL_BARTH) {
      int jj = 0;
      while (jj < 2 && e[3 * t + jj] - 1 != p) jj++;
      const int n1 = p;
      const int n2 = e[3 * t + (jj + 2) % 3] - 1;   // previous vertex
      const int n3 = e[3 * t + (jj + 1) % 3] - 1;   // next vertex
      const double x[5] = {c[n1].x, 0.5 * (c[n1].x + c[n3].x), tc[t].x, 0.5 * (c[n1].x + c[n2].x),
                           c[n1].x};
      const double y[5] = {c[n1].y, 0.5 * (c[n1].y + c[n3].y), tc[t].y, 0.5 * (c[n1].y + c[n2].y),
                           c[n1].y};
      double area = 0.0;
      for (int k = 0; k < 4; k++) area = area + x[k] * y[k + 1] - x[k + 1] * y[k];
      if (area < 0.0) atomicOr(err, kErrNegArea);
      cv = cv + 0.5 * area;
    }
  }
  mcarea[p] = m;
  cvarea[p] = cell_type == FVM_CELL_MEDIAN ? m : cv;
}

// flength.f:13-49 (ds of each edge) and the flags of the order-preserving
// compactions: boundary edges (flength.f:52, make_bdedges.f:12, the
// product of the neighbours as the 32-bit product the driver forms), kept
// edges (reorder_edges, flength.f:82-105)
__global__ void k_edges(int ne, int cell_type, const double2 *__restrict__ c,
                        const double2 *__restrict__ tc, const int *__restrict__ edge,
                        const int *__restrict__ edneigh, double *__restrict__ ds,
                        int *__restrict__ fbnd, int *__restrict__ fkeep, int *err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ne) return;
  const int n1 = edge[2 * i] - 1, n2 = edge[2 * i + 1] - 1;
  const int p1 = edneigh[2 * i], p2 = edneigh[2 * i + 1];
  double dsx = 0.0, dsy = 0.0;
  if (p1 == 0) {
    atomicOr(err, kErrNoLeft);
  } else {
    const double x1 = tc[p1 - 1].x, y1 = tc[p1 - 1].y;
    double x2, y2;
    if (p2 != 0) {
      x2 = tc[p2 - 1].x;
      y2 = tc[p2 - 1].y;
    } else {
      x2 = 0.5 * (c[n1].x + c[n2].x);
      y2 = 0.5 * (c[n1].y + c[n2].y);
    }
    dsx = -(y2 - y1);
    dsy = x2 - x1;
  }
  ds[2 * i] = dsx;
  ds[2 * i + 1] = dsy;
  fbnd[i] = (uint32_t)p1 * (uint32_t)p2 == 0u ? 1 : 0;
  int keep = 1;
  if (cell_type == FVM_CELL_BARTH) keep = sqrt(dsx * dsx + dsy * dsy) != 0.0;
  fkeep[i] = keep;
}

// writes i + 1 (a 1-based id) at pos[i] for every flagged i
__global__ void k_compact(int n, const int *__restrict__ flag, const int *__restrict__ pos,
                          int *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && flag[i]) out[pos[i]] = i + 1;
}

// make_bdedges.f:9-44 over the boundary edges in edge order: solid flags,
// farfield flags
__global__ void k_bd_flags(int nb, const int *__restrict__ bidx, const int *__restrict__ edge,
                           const int *__restrict__ ptype, int *__restrict__ fsol,
                           int *__restrict__ fff) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  const int i = bidx[k] - 1;
  const int t1 = ptype[edge[2 * i] - 1], t2 = ptype[edge[2 * i + 1] - 1];
  fsol[k] = t1 == FVM_PT_SOLID && t2 == FVM_PT_SOLID;
  fff[k] = t1 == FVM_PT_FARFIELD && t2 == FVM_PT_FARFIELD;
}

// compaction of boundary-edge ids through their positions
__global__ void k_compact_ids(int n, const int *__restrict__ flag, const int *__restrict__ pos,
                              const int *__restrict__ ids, int *__restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n && flag[k]) out[pos[k]] = ids[k];
}

// flength.f:51-60: the boundary edges' half normals, added to both ends in
// edge order (one thread: the host's order of additions)
__global__ void k_dsb(int nb, const int *__restrict__ bidx, const int *__restrict__ edge,
                      const double2 *__restrict__ c, double *__restrict__ dsb) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  for (int k = 0; k < nb; k++) {
    const int i = bidx[k] - 1;
    const int n1 = edge[2 * i] - 1, n2 = edge[2 * i + 1] - 1;
    const double nx = c[n2].y - c[n1].y;
    const double ny = -(c[n2].x - c[n1].x);
    dsb[2 * n1] += 0.5 * nx;
    dsb[2 * n1 + 1] += 0.5 * ny;
    dsb[2 * n2] += 0.5 * nx;
    dsb[2 * n2 + 1] += 0.5 * ny;
  }
}

// geom_stat.f:18-37: any non-positive triangle or control-volume area
__global__ void k_positive(int n, const double *__restrict__ a, int *err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && !(a[i] > 0.0)) atomicOr(err, kErrNonPositive);
}

__global__ void k_flag_solid(int np, const int *__restrict__ ptype, int *__restrict__ f) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < np) f[p] = ptype[p] == FVM_PT_SOLID;
}

// ---- host side -------------------------------------------------------------
struct Dev {
  std::vector<void *> owned;
  ~Dev() {
    for (void *p : owned) cudaFree(p);
  }
  template <typename T>
  cudaError_t alloc(T **p, size_t n) {
    void *q = nullptr;
    const cudaError_t e = cudaMalloc(&q, sizeof(T) * (n ? n : 1));
    if (e == cudaSuccess) owned.push_back(q);
    *p = static_cast<T *>(q);
    return e;
  }
};

// exclusive scan of in[0..n) into out[0..n] (out[n] = total)
cudaError_t scan(Dev &D, const int *in, int *out, int n) {
  const int nb = (n + kScanItems - 1) / kScanItems;
  if (nb == 0) {
    k_scan_total<<<1, 1>>>(in, out, 0);
    return cudaGetLastError();
  }
  int *bsum = nullptr, *boff = nullptr;
  cudaError_t e = D.alloc(&bsum, (size_t)nb);
  if (e == cudaSuccess) e = D.alloc(&boff, (size_t)nb + 1);
  if (e != cudaSuccess) return e;
  k_scan_blocks<<<nb, kT>>>(in, out, n, bsum);
  if (nb > 1) {
    if ((e = scan(D, bsum, boff, nb)) != cudaSuccess) return e;
    k_scan_add<<<nb, kT>>>(out, n, boff);
  }
  k_scan_total<<<1, 1>>>(in, out, n);
  return cudaGetLastError();
}

template <typename T>
cudaError_t to_host(std::vector<T> &h, const T *d, size_t n) {
  h.resize(n);
  return n ? cudaMemcpy(h.data(), d, sizeof(T) * n, cudaMemcpyDeviceToHost) : cudaSuccess;
}

int read_int(const int *d, cudaError_t &e) {
  int v = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&v, d, sizeof(int), cudaMemcpyDeviceToHost);
  return v;
}

}  // namespace

int32_t geom_chain_gpu(int32_t np, int32_t nt, const double *coord, const int32_t *elem,
                       const int32_t *ptype, int32_t cell_type, GeomChainOut &out) {
  Dev D;
  double2 *c = nullptr, *tc = nullptr;
  int *e = nullptr, *pt = nullptr, *err = nullptr, *cnt = nullptr, *ptr = nullptr,
      *fill = nullptr, *esup = nullptr, *ecnt = nullptr, *eptr = nullptr;
  double *elarea = nullptr, *mcarea = nullptr, *cvarea = nullptr, *drmin = nullptr;
  cudaError_t ce = cudaSuccess;
#define GTRY(x)                                   \
  do {                                            \
    if ((ce = (x)) != cudaSuccess) goto cuda_fail; \
  } while (0)
  {
    GTRY(D.alloc(&c, (size_t)np));
    GTRY(D.alloc(&e, 3 * (size_t)nt));
    GTRY(D.alloc(&pt, (size_t)np));
    GTRY(D.alloc(&err, 1));
    GTRY(D.alloc(&cnt, (size_t)np));
    GTRY(D.alloc(&fill, (size_t)np));
    GTRY(D.alloc(&ptr, (size_t)np + 1));
    GTRY(D.alloc(&esup, 3 * (size_t)nt));
    GTRY(D.alloc(&ecnt, (size_t)np));
    GTRY(D.alloc(&eptr, (size_t)np + 1));
    GTRY(D.alloc(&tc, (size_t)nt));
    GTRY(D.alloc(&elarea, (size_t)nt));
    GTRY(D.alloc(&mcarea, (size_t)np));
    GTRY(D.alloc(&cvarea, (size_t)np));
    GTRY(D.alloc(&drmin, (size_t)np));
    GTRY(cudaMemcpy(c, coord, 16 * (size_t)np, cudaMemcpyHostToDevice));
    GTRY(cudaMemcpy(e, elem, 12 * (size_t)nt, cudaMemcpyHostToDevice));
    GTRY(cudaMemcpy(pt, ptype, 4 * (size_t)np, cudaMemcpyHostToDevice));
    GTRY(cudaMemset(err, 0, sizeof(int)));
    GTRY(cudaMemset(cnt, 0, 4 * (size_t)np));
    GTRY(cudaMemset(fill, 0, 4 * (size_t)np));
    k_orient<<<nblocks(nt), kT>>>(nt, c, e, err);
    GTRY(cudaGetLastError());
    if (read_int(err, ce)) return FVM_ERR_GEOMETRY;
    GTRY(ce);
    // el_surr_point.f
    k_count_corners<<<nblocks(nt), kT>>>(nt, e, cnt);
    GTRY(cudaGetLastError());
    GTRY(scan(D, cnt, ptr, np));
    k_fill_corners<<<nblocks(nt), kT>>>(nt, e, ptr, fill, esup);
    k_sort_lists<<<nblocks(np), kT>>>(np, ptr, esup);
    // pt_surr_pt.f + create_edge.f
    k_point_edges<0><<<nblocks(np), kT>>>(np, ptr, esup, e, ecnt, nullptr, nullptr);
    GTRY(cudaGetLastError());
    GTRY(scan(D, ecnt, eptr, np));
    const int ne = read_int(eptr + np, ce);
    GTRY(ce);
    int *edge = nullptr, *edneigh = nullptr, *fbnd = nullptr, *fkeep = nullptr, *pbnd = nullptr,
        *pkeep = nullptr, *iedge = nullptr, *bidx = nullptr;
    double *ds = nullptr, *dsb = nullptr;
    GTRY(D.alloc(&edge, 2 * (size_t)ne));
    GTRY(D.alloc(&edneigh, 2 * (size_t)ne));
    GTRY(D.alloc(&ds, 2 * (size_t)ne));
    GTRY(D.alloc(&fbnd, (size_t)ne));
    GTRY(D.alloc(&fkeep, (size_t)ne));
    GTRY(D.alloc(&pbnd, (size_t)ne + 1));
    GTRY(D.alloc(&pkeep, (size_t)ne + 1));
    GTRY(D.alloc(&dsb, 2 * (size_t)np));
    k_point_edges<1><<<nblocks(np), kT>>>(np, ptr, esup, e, nullptr, eptr, edge);
    // el_surr_edge.f
    k_edge_neighbours<<<nblocks(ne), kT>>>(ne, ptr, esup, e, edge, edneigh);
    // tri_coord.f, areas.f
    k_triangles<<<nblocks(nt), kT>>>(nt, cell_type, c, e, tc, elarea);
    k_point_areas<<<nblocks(np), kT>>>(np, cell_type, ptr, esup, e, c, tc, elarea, mcarea,
                                       cvarea, err);
    // flength.f, reorder_edges
    k_edges<<<nblocks(ne), kT>>>(ne, cell_type, c, tc, edge, edneigh, ds, fbnd, fkeep, err);
    GTRY(cudaGetLastError());
    if (read_int(err, ce)) return FVM_ERR_GEOMETRY;
    GTRY(ce);
    GTRY(scan(D, fbnd, pbnd, ne));
    GTRY(scan(D, fkeep, pkeep, ne));
    const int nb = read_int(pbnd + ne, ce);
    const int nkeep = read_int(pkeep + ne, ce);
    GTRY(ce);
    GTRY(D.alloc(&iedge, (size_t)nkeep));
    GTRY(D.alloc(&bidx, (size_t)nb));
    k_compact<<<nblocks(ne), kT>>>(ne, fbnd, pbnd, bidx);
    k_compact<<<nblocks(ne), kT>>>(ne, fkeep, pkeep, iedge);
    GTRY(cudaMemset(dsb, 0, 16 * (size_t)np));
    k_dsb<<<1, 32>>>(nb, bidx, edge, c, dsb);
    // make_bdedges.f: solid edges, then farfield edges
    int *fsol = nullptr, *fff = nullptr, *psol = nullptr, *pff = nullptr, *beindx = nullptr;
    GTRY(D.alloc(&fsol, (size_t)nb));
    GTRY(D.alloc(&fff, (size_t)nb));
    GTRY(D.alloc(&psol, (size_t)nb + 1));
    GTRY(D.alloc(&pff, (size_t)nb + 1));
    if (nb > 0) k_bd_flags<<<nblocks(nb), kT>>>(nb, bidx, edge, pt, fsol, fff);
    GTRY(cudaGetLastError());
    GTRY(scan(D, fsol, psol, nb));
    GTRY(scan(D, fff, pff, nb));
    const int nswe = read_int(psol + nb, ce);
    const int nffe = read_int(pff + nb, ce);
    GTRY(ce);
    GTRY(D.alloc(&beindx, (size_t)(nswe + nffe)));
    if (nb > 0) {
      k_compact_ids<<<nblocks(nb), kT>>>(nb, fsol, psol, bidx, beindx);
      k_compact_ids<<<nblocks(nb), kT>>>(nb, fff, pff, bidx, beindx + nswe);
    }
    // geom_stat.f:18-37
    k_positive<<<nblocks(nt), kT>>>(nt, elarea, err);
    k_positive<<<nblocks(np), kT>>>(np, cvarea, err);
    GTRY(cudaGetLastError());
    if (read_int(err, ce)) return FVM_ERR_GEOMETRY;
    GTRY(ce);
    // solid points; dtlength.f on the resident arrays
    int *fsp = nullptr, *psp = nullptr, *spts = nullptr;
    GTRY(D.alloc(&fsp, (size_t)np));
    GTRY(D.alloc(&psp, (size_t)np + 1));
    k_flag_solid<<<nblocks(np), kT>>>(np, pt, fsp);
    GTRY(cudaGetLastError());
    GTRY(scan(D, fsp, psp, np));
    const int nsp = read_int(psp + np, ce);
    GTRY(ce);
    GTRY(D.alloc(&spts, (size_t)nsp));
    k_compact<<<nblocks(np), kT>>>(np, fsp, psp, spts);
    GTRY(launch_dtlength(np, nt, c, e, elarea, drmin, 0));
    GTRY(to_host(out.elem, e, 3 * (size_t)nt));
    GTRY(to_host(out.edge, edge, 2 * (size_t)ne));
    GTRY(to_host(out.edneigh, edneigh, 2 * (size_t)ne));
    GTRY(to_host(out.iedge, iedge, (size_t)nkeep));
    GTRY(to_host(out.beindx, beindx, (size_t)(nswe + nffe)));
    GTRY(to_host(out.spts, spts, (size_t)nsp));
    GTRY(to_host(out.ds, ds, 2 * (size_t)ne));
    GTRY(to_host(out.dsb, dsb, 2 * (size_t)np));
    GTRY(to_host(out.elarea, elarea, (size_t)nt));
    GTRY(to_host(out.cvarea, cvarea, (size_t)np));
    GTRY(to_host(out.mcarea, mcarea, (size_t)np));
    GTRY(to_host(out.drmin, drmin, (size_t)np));
    out.nswe = nswe;
    return FVM_OK;
  }
cuda_fail:
  return ce == cudaErrorMemoryAllocation ? FVM_ERR_NOMEM : FVM_ERR_CUDA;
#undef GTRY
}

}  // namespace fvm
