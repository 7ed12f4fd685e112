// fvm_geom_gpu.h -- the driver geometry chain on the GPU (fvm_geom_gpu.cu),
// for fvm_gpu_geom_build in fvm_geometry.cpp.
#pragma once

#include <cstdint>
#include <vector>

namespace fvm {

// Arrays of the chain of src/geometric.f:15-60, as fvm_geom_build fills
// them (1-based ids where the driver's are 1-based), plus drmin
// (dtlength.f) from the same device arrays.
struct GeomChainOut {
  std::vector<int32_t> elem;      // oriented (tri_orient.f:33-37)
  std::vector<int32_t> edge, edneigh, iedge, beindx, spts;
  std::vector<double> ds, dsb, elarea, cvarea, mcarea, drmin;
  int nswe = 0;                   // solid edges at the head of beindx
};

// FVM_OK, FVM_ERR_GEOMETRY (tri_orient.f:28-31, a triangle without a left
// neighbour edge, areas.f:145-150, geom_stat.f:18-37), FVM_ERR_NOMEM or
// FVM_ERR_CUDA.  elem is read, not modified; the oriented copy is returned.
int32_t geom_chain_gpu(int32_t np, int32_t nt, const double *coord, const int32_t *elem,
                       const int32_t *ptype, int32_t cell_type, GeomChainOut &out);

}  // namespace fvm
