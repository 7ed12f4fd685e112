// fvm_layout.h -- host construction of the block layout of one mesh.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "../../include/fvm_gpu.h"
#include "fvm_internal.h"

namespace fvm {

// Everything the device needs for one mesh, in mesh-local indices (vertex
// ids are the renumbered ones, 0-based; offsets start at 0).  Upload adds
// the arena offsets.
struct MeshLayout {
  int np = 0, nt = 0, nblk = 0;
  std::vector<int> perm;          // new vertex -> driver vertex (0-based)
  std::vector<int> iperm;         // driver vertex -> new vertex
  std::vector<BlockInfo> blocks;  // v0,e0,b0,t0 relative; mesh/part filled at upload
  std::vector<int2> be_nodes;     // interior edge entries (new ids)
  std::vector<int> be_edge;       // driver edge index (0-based) of each entry
  std::vector<int4> bb_nodes;     // boundary entries (n1, n2, 1 solid | 2 farfield, -)
  std::vector<int4> bt_nodes;     // triangle entries (n1, n2, n3, driver triangle)
  std::vector<uint32_t> bt_loc;   // per triangle entry: the ends' local slots (kTriLoc*)
  std::vector<int> ve_ptr;        // [np+1]
  std::vector<uint16_t> ve_list;
  std::vector<int> vt_ptr;        // [np+1]
  std::vector<uint16_t> vt_list;
  std::vector<int> va_ptr;        // [np+1] all netot edges, edge order
  std::vector<int> va_list;
  std::vector<int2> sw_nodes;     // solid edges in beindx order (new ids)
  std::vector<uint8_t> vflag;     // kVtxSolid / kVtxFarfield
  // fused gradient+flux pass
  std::vector<uint32_t> be_loc;   // local slots of each edge entry's ends
  std::vector<int> halo_ids;      // per block: halo vertices (new ids), ascending
  std::vector<int> hl_ptr;        // per block: nh+1 offsets (relative) into hl_list
  std::vector<uint16_t> hl_list;  // halo vertex triangles: slot | pos << 14
  int max_tri = 0, max_slots = 0, max_tri2 = 0, max_loc = 0;
  int max_halo = 0;               // max halo vertices of a block
};

// Builds the layout; returns FVM_OK or FVM_ERR_ARG (bad connectivity) /
// FVM_ERR_CAPACITY (a block needs more slots than the incidence entries can
// address).
int32_t build_layout(const fvm_mesh &m, int block_verts, MeshLayout &L);

// Checks the fused-pass invariants of a built layout (local slots decode to
// the edge ends, halo triangle lists equal the owners' lists in order,
// every index inside its block's tiles); returns the number of violations.
int64_t verify_layout(const MeshLayout &L);

// Vertex order only (exposed for tests of the partitioner).
void order_vertices(int np, const std::vector<int> &adj_ptr, const std::vector<int> &adj,
                    int block_verts, std::vector<int> &perm, std::vector<int> &block_start);

}  // namespace fvm
