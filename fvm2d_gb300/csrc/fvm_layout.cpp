// fvm_layout.cpp -- vertex renumbering and block tables of one mesh.
//
// Renumbering: recursive bisection of the vertex graph.  A part is split by
// a breadth-first sweep from a pseudo-peripheral vertex (the last vertex
// reached by a sweep from an arbitrary one); the first ceil(k/2) blocks'
// worth of vertices in sweep order form one half.  Splits alternate
// direction by themselves, so the leaves (blocks of <= block_verts
// vertices, consecutive in the new numbering) are compact patches and few
// edges cross block boundaries.
//
// Block tables: the interior edges of iedge (residu.f:38-66) touching a
// block, in iedge order; the solid then farfield edges of beindx
// (residu.f:73-88) touching it; the triangles touching it in triangle
// order (green_gauss.f:23-31).  Each vertex lists its slots in exactly the
// order the Fortran loops visit them, so gathering the per-slot values in
// list order reproduces the serial sums.
#include "fvm_layout.h"

#include <algorithm>
#include <cstring>
#include <unordered_map>

namespace fvm {

namespace {

struct Bfs {
  std::vector<int> seen;   // stamp of the last sweep that reached a vertex
  std::vector<int> inset;  // stamp of the part a vertex belongs to
  int stamp = 0;
};

// Breadth-first sweep over the vertices of the current part (inset ==
// part_stamp) starting at root; visits every component.  Returns order.
void sweep(const std::vector<int> &adj_ptr, const std::vector<int> &adj,
           const std::vector<int> &verts, int root, int part_stamp, Bfs &B,
           std::vector<int> &order) {
  const int s = ++B.stamp;
  order.clear();
  order.reserve(verts.size());
  size_t head = 0;
  auto visit_from = [&](int r) {
    B.seen[r] = s;
    order.push_back(r);
    while (head < order.size()) {
      const int v = order[head++];
      for (int j = adj_ptr[v]; j < adj_ptr[v + 1]; j++) {
        const int w = adj[j];
        if (B.inset[w] == part_stamp && B.seen[w] != s) {
          B.seen[w] = s;
          order.push_back(w);
        }
      }
    }
  };
  visit_from(root);
  if (order.size() < verts.size())
    for (int v : verts)
      if (B.seen[v] != s) visit_from(v);
}

void bisect(const std::vector<int> &adj_ptr, const std::vector<int> &adj, std::vector<int> verts,
            int bv, Bfs &B, std::vector<int> &perm, std::vector<int> &block_start) {
  // explicit stack to bound recursion depth
  std::vector<std::vector<int>> stack;
  stack.push_back(std::move(verts));
  std::vector<int> order;
  while (!stack.empty()) {
    std::vector<int> part = std::move(stack.back());
    stack.pop_back();
    const int part_stamp = ++B.stamp;
    for (int v : part) B.inset[v] = part_stamp;
    sweep(adj_ptr, adj, part, part[part.size() / 2], part_stamp, B, order);
    const int root = order.back();
    sweep(adj_ptr, adj, part, root, part_stamp, B, order);
    if ((int)part.size() <= bv) {
      block_start.push_back((int)perm.size());
      perm.insert(perm.end(), order.begin(), order.end());
      continue;
    }
    const int nblocks = ((int)part.size() + bv - 1) / bv;
    const size_t nleft = size_t((nblocks + 1) / 2) * bv;
    std::vector<int> left(order.begin(), order.begin() + nleft);
    std::vector<int> right(order.begin() + nleft, order.end());
    // right is processed after left: push right first
    stack.push_back(std::move(right));
    stack.push_back(std::move(left));
  }
}

}  // namespace

void order_vertices(int np, const std::vector<int> &adj_ptr, const std::vector<int> &adj,
                    int block_verts, std::vector<int> &perm, std::vector<int> &block_start) {
  perm.clear();
  block_start.clear();
  if (np <= 0) return;
  Bfs B;
  B.seen.assign(np, 0);
  B.inset.assign(np, 0);
  std::vector<int> all(np);
  for (int i = 0; i < np; i++) all[i] = i;
  bisect(adj_ptr, adj, std::move(all), block_verts, B, perm, block_start);
}

int32_t build_layout(const fvm_mesh &m, int bv, MeshLayout &L) {
  const int np = m.np, nt = m.nt, netot = m.netot;
  if (np < 3 || nt < 1 || m.ne < 1 || m.ne > netot) return FVM_ERR_ARG;
  L = MeshLayout();
  L.np = np;
  L.nt = nt;
  // adjacency over all edges
  std::vector<int> deg(np + 1, 0);
  for (int e = 0; e < netot; e++) {
    const int a = m.edge[2 * e] - 1, b = m.edge[2 * e + 1] - 1;
    if (a < 0 || a >= np || b < 0 || b >= np || a == b) return FVM_ERR_ARG;
    deg[a + 1]++;
    deg[b + 1]++;
  }
  for (int i = 0; i < np; i++) deg[i + 1] += deg[i];
  std::vector<int> adj(deg[np]);
  {
    std::vector<int> fill(deg.begin(), deg.end() - 1);
    for (int e = 0; e < netot; e++) {
      const int a = m.edge[2 * e] - 1, b = m.edge[2 * e + 1] - 1;
      adj[fill[a]++] = b;
      adj[fill[b]++] = a;
    }
  }
  std::vector<int> block_start;
  order_vertices(np, deg, adj, bv, L.perm, block_start);
  L.iperm.assign(np, -1);
  for (int i = 0; i < np; i++) L.iperm[L.perm[i]] = i;
  const int nblk = (int)block_start.size();
  L.nblk = nblk;
  std::vector<int> blk_of(np);
  L.blocks.assign(nblk, BlockInfo());
  for (int b = 0; b < nblk; b++) {
    const int v0 = block_start[b];
    const int v1 = (b + 1 < nblk) ? block_start[b + 1] : np;
    std::memset(&L.blocks[b], 0, sizeof(BlockInfo));
    L.blocks[b].v0 = v0;
    L.blocks[b].nv = v1 - v0;
    for (int v = v0; v < v1; v++) blk_of[v] = b;
  }
  L.vflag.assign(np, 0);
  for (int i = 0; i < np; i++) {
    const int t = m.ptype[i];
    if (t == FVM_PT_SOLID) L.vflag[L.iperm[i]] |= kVtxSolid;
    if (t == FVM_PT_FARFIELD) L.vflag[L.iperm[i]] |= kVtxFarfield;
  }
  // interior edges, iedge order, per block
  std::vector<std::vector<int>> bedges(nblk);
  for (int i = 0; i < m.ne; i++) {
    const int e = m.iedge[i] - 1;
    if (e < 0 || e >= netot) return FVM_ERR_ARG;
    const int a = L.iperm[m.edge[2 * e] - 1], b = L.iperm[m.edge[2 * e + 1] - 1];
    const int ba = blk_of[a], bb = blk_of[b];
    bedges[ba].push_back(e);
    if (bb != ba) bedges[bb].push_back(e);
  }
  // boundary edges, beindx order (solid, then farfield)
  std::vector<std::vector<int4>> bbnd(nblk);
  auto add_bnd = [&](int pos1, int pos2, int type) -> int32_t {
    for (int i = pos1; i <= pos2; i++) {
      const int e = m.beindx[i - 1] - 1;
      if (e < 0 || e >= netot) return FVM_ERR_ARG;
      const int a = L.iperm[m.edge[2 * e] - 1], b = L.iperm[m.edge[2 * e + 1] - 1];
      const int ba = blk_of[a], bb = blk_of[b];
      bbnd[ba].push_back(make_int4(a, b, type, 0));
      if (bb != ba) bbnd[bb].push_back(make_int4(a, b, type, 0));
      if (type == 1) L.sw_nodes.push_back(make_int2(a, b));
    }
    return FVM_OK;
  };
  if (m.nswe2 >= m.nswe1)
    if (add_bnd(m.nswe1, m.nswe2, 1)) return FVM_ERR_ARG;
  if (m.nffe2 >= m.nffe1)
    if (add_bnd(m.nffe1, m.nffe2, 2)) return FVM_ERR_ARG;
  // triangles, triangle order, per block
  std::vector<std::vector<int>> btris(nblk);
  for (int t = 0; t < nt; t++) {
    int bl[3];
    for (int k = 0; k < 3; k++) {
      const int n = m.elem[3 * t + k] - 1;
      if (n < 0 || n >= np) return FVM_ERR_ARG;
      bl[k] = blk_of[L.iperm[n]];
    }
    btris[bl[0]].push_back(t);
    if (bl[1] != bl[0]) btris[bl[1]].push_back(t);
    if (bl[2] != bl[0] && bl[2] != bl[1]) btris[bl[2]].push_back(t);
  }
  // vertex -> triangles (ascending), for the halo's triangles
  std::vector<int> vt_cnt(np + 1, 0);
  for (int t = 0; t < nt; t++)
    for (int k = 0; k < 3; k++) vt_cnt[L.iperm[m.elem[3 * t + k] - 1] + 1]++;
  for (int v = 0; v < np; v++) vt_cnt[v + 1] += vt_cnt[v];
  std::vector<int> vt_adj(vt_cnt[np]);
  {
    std::vector<int> fill(vt_cnt.begin(), vt_cnt.end() - 1);
    for (int t = 0; t < nt; t++)
      for (int k = 0; k < 3; k++) vt_adj[fill[L.iperm[m.elem[3 * t + k] - 1]]++] = t;
  }
  // halo of each block (vertices outside it sharing an edge or a triangle
  // with it) and the triangles touching the halo but not the block, which
  // follow the block's own triangles in its bt list
  std::vector<int> loc(np, -1);
  std::vector<std::vector<int>> btris_extra(nblk);
  for (int b = 0; b < nblk; b++) {
    const int v0 = L.blocks[b].v0, v1 = v0 + L.blocks[b].nv;
    auto inblk = [&](int v) { return v >= v0 && v < v1; };
    std::vector<int> halo;
    auto want = [&](int v) {
      if (!inblk(v) && loc[v] == -1) {
        loc[v] = -2;
        halo.push_back(v);
      }
    };
    for (int t : btris[b])
      for (int q = 0; q < 3; q++) want(L.iperm[m.elem[3 * t + q] - 1]);
    for (int e : bedges[b]) {
      want(L.iperm[m.edge[2 * e] - 1]);
      want(L.iperm[m.edge[2 * e + 1] - 1]);
    }
    for (const int4 &q : bbnd[b]) {
      want(q.x);
      want(q.y);
    }
    std::sort(halo.begin(), halo.end());
    for (int v : halo) loc[v] = -1;
    BlockInfo &bi = L.blocks[b];
    bi.h0 = (int)L.halo_ids.size();
    bi.nh = (int)halo.size();
    L.max_halo = std::max(L.max_halo, bi.nh);
    L.halo_ids.insert(L.halo_ids.end(), halo.begin(), halo.end());
    const int nloc = bi.nv + bi.nh;
    if (nloc > 0xffff) return FVM_ERR_CAPACITY;
    L.max_loc = std::max(L.max_loc, nloc);
    // triangles of halo vertices not already in the block's list
    std::vector<int> extra;
    for (int v : halo)
      for (int j = vt_cnt[v]; j < vt_cnt[v + 1]; j++) {
        const int t = vt_adj[j];
        bool touches_block = false;
        for (int q = 0; q < 3; q++) touches_block |= inblk(L.iperm[m.elem[3 * t + q] - 1]);
        if (!touches_block) extra.push_back(t);
      }
    std::sort(extra.begin(), extra.end());
    extra.erase(std::unique(extra.begin(), extra.end()), extra.end());
    btris_extra[b] = std::move(extra);
  }
  // per-vertex lists
  std::vector<std::vector<uint16_t>> vint(np), vbnd(np), vtri(np);
  for (int b = 0; b < nblk; b++) {
    BlockInfo &bi = L.blocks[b];
    const int v0 = bi.v0, v1 = bi.v0 + bi.nv;
    auto inblk = [&](int v) { return v >= v0 && v < v1; };
    bi.e0 = (int)L.be_nodes.size();
    bi.ne = (int)bedges[b].size();
    const int *hbeg = L.halo_ids.data() + bi.h0, *hend = hbeg + bi.nh;
    auto local = [&](int v) -> uint32_t {
      if (inblk(v)) return (uint32_t)(v - v0);
      return (uint32_t)(bi.nv + (std::lower_bound(hbeg, hend, v) - hbeg));
    };
    for (int k = 0; k < bi.ne; k++) {
      const int e = bedges[b][k];
      const int a = L.iperm[m.edge[2 * e] - 1], c = L.iperm[m.edge[2 * e + 1] - 1];
      L.be_nodes.push_back(make_int2(a, c));
      L.be_loc.push_back(local(a) | (local(c) << 16));
      L.be_edge.push_back(e);
      if (inblk(a)) vint[a].push_back((uint16_t)k);
      if (inblk(c)) vint[c].push_back((uint16_t)(k | kNegBit));
    }
    bi.b0 = (int)L.bb_nodes.size();
    bi.nb = (int)bbnd[b].size();
    for (int k = 0; k < bi.nb; k++) {
      const int4 q = bbnd[b][k];
      L.bb_nodes.push_back(q);
      const uint16_t flag = (q.z == 1) ? kSolidBit : kFarBit;
      if (inblk(q.x)) vbnd[q.x].push_back((uint16_t)((bi.ne + 2 * k) | flag));
      if (inblk(q.y)) vbnd[q.y].push_back((uint16_t)((bi.ne + 2 * k + 1) | flag));
    }
    const int slots = bi.ne + 2 * bi.nb;
    if (slots > kSlotMask) return FVM_ERR_CAPACITY;
    L.max_slots = std::max(L.max_slots, slots);
    bi.t0 = (int)L.bt_nodes.size();
    bi.nt = (int)btris[b].size();
    if (bi.nt > 0x3fff) return FVM_ERR_CAPACITY;
    L.max_tri = std::max(L.max_tri, bi.nt);
    // the block's interior triangles (all three vertices its own) first,
    // then those touching the halo, each group ascending: the gradient
    // passes' first trips over the entries then read only the block's own
    // (staged) states.  Sums follow the per-vertex lists, which are put
    // back in ascending triangle order below, so the order here changes
    // no result.
    std::stable_partition(btris[b].begin(), btris[b].end(), [&](int t) {
      for (int q = 0; q < 3; q++)
        if (!inblk(L.iperm[m.elem[3 * t + q] - 1])) return false;
      return true;
    });
    for (int k = 0; k < bi.nt; k++) {
      const int t = btris[b][k];
      int n[3];
      for (int q = 0; q < 3; q++) n[q] = L.iperm[m.elem[3 * t + q] - 1];
      L.bt_nodes.push_back(make_int4(n[0], n[1], n[2], t));
      uint32_t lc = 0;
      bool packs = true;
      for (int q = 0; q < 3; q++) {
        const uint32_t l = local(n[q]);
        packs &= l < (uint32_t)kTriLocMax;
        lc |= (l & (uint32_t)(kTriLocMax - 1)) << (kTriLocBits * q);
      }
      L.bt_loc.push_back(packs ? lc : kTriNoLoc);
      for (int q = 0; q < 3; q++)
        if (inblk(n[q])) vtri[n[q]].push_back((uint16_t)(k | (q << kTriPosShift)));
    }
    for (int v = v0; v < v1; v++)   // green_gauss.f visits triangles ascending
      std::sort(vtri[v].begin(), vtri[v].end(), [&](uint16_t x, uint16_t y) {
        return btris[b][x & 0x3fff] < btris[b][y & 0x3fff];
      });
    // the halo's other triangles follow, then each halo vertex lists its
    // triangles (ascending triangle number: the order green_gauss.f visits)
    const std::vector<int> &extra = btris_extra[b];
    bi.nt2 = bi.nt + (int)extra.size();
    if (bi.nt2 > 0x3fff) return FVM_ERR_CAPACITY;
    L.max_tri2 = std::max(L.max_tri2, bi.nt2);
    for (int t : extra) {
      int n[3];
      for (int q = 0; q < 3; q++) n[q] = L.iperm[m.elem[3 * t + q] - 1];
      L.bt_nodes.push_back(make_int4(n[0], n[1], n[2], t));
      L.bt_loc.push_back(kTriNoLoc);   // halo-only triangle: no slots of its own block
    }
    {
      std::unordered_map<int, int> slot_of;
      slot_of.reserve(2 * bi.nt2);
      for (int k = 0; k < bi.nt; k++) slot_of[btris[b][k]] = k;
      for (size_t k = 0; k < extra.size(); k++) slot_of[extra[k]] = bi.nt + (int)k;
      bi.hp0 = (int)L.hl_ptr.size();
      for (int h = 0; h < bi.nh; h++) {
        const int v = hbeg[h];
        L.hl_ptr.push_back((int)L.hl_list.size());
        for (int j = vt_cnt[v]; j < vt_cnt[v + 1]; j++) {
          const int t = vt_adj[j];
          int pos = 0;
          for (int q = 0; q < 3; q++)
            if (L.iperm[m.elem[3 * t + q] - 1] == v) pos = q;
          L.hl_list.push_back((uint16_t)(slot_of.at(t) | (pos << kTriPosShift)));
        }
      }
      L.hl_ptr.push_back((int)L.hl_list.size());
    }
  }
  L.ve_ptr.assign(np + 1, 0);
  L.vt_ptr.assign(np + 1, 0);
  for (int v = 0; v < np; v++) {
    L.ve_ptr[v + 1] = L.ve_ptr[v] + (int)(vint[v].size() + vbnd[v].size());
    L.vt_ptr[v + 1] = L.vt_ptr[v] + (int)vtri[v].size();
  }
  for (BlockInfo &bi : L.blocks) {
    bi.vt0 = L.vt_ptr[bi.v0];
    bi.nvt = L.vt_ptr[bi.v0 + bi.nv] - bi.vt0;
  }
  L.ve_list.reserve(L.ve_ptr[np]);
  L.vt_list.reserve(L.vt_ptr[np]);
  for (int v = 0; v < np; v++) {
    L.ve_list.insert(L.ve_list.end(), vint[v].begin(), vint[v].end());
    L.ve_list.insert(L.ve_list.end(), vbnd[v].begin(), vbnd[v].end());
    L.vt_list.insert(L.vt_list.end(), vtri[v].begin(), vtri[v].end());
  }
  // all-edge incidence in edge order (limitgrad.f:22-68)
  std::vector<std::vector<int>> vall(np);
  for (int e = 0; e < netot; e++) {
    const int a = L.iperm[m.edge[2 * e] - 1], b = L.iperm[m.edge[2 * e + 1] - 1];
    vall[a].push_back(b);
    vall[b].push_back(int(uint32_t(a) | 0x80000000u));
  }
  L.va_ptr.assign(np + 1, 0);
  for (int v = 0; v < np; v++) L.va_ptr[v + 1] = L.va_ptr[v] + (int)vall[v].size();
  L.va_list.reserve(L.va_ptr[np]);
  for (int v = 0; v < np; v++) L.va_list.insert(L.va_list.end(), vall[v].begin(), vall[v].end());
  return FVM_OK;
}

int64_t verify_layout(const MeshLayout &L) {
  int64_t bad = 0;
  auto has = [](const int4 &t, int v, int pos) {
    return (pos == 0 ? t.x : pos == 1 ? t.y : t.z) == v;
  };
  for (const BlockInfo &bi : L.blocks) {
    const int nloc = bi.nv + bi.nh, nslot = bi.ne + 2 * bi.nb;
    if (bi.nv > kBlockVerts || nloc > L.max_loc || bi.nt > L.max_tri || bi.nt2 > L.max_tri2 ||
        bi.nt2 < bi.nt || nslot > L.max_slots) {
      bad++;
      continue;
    }
    auto vert_of = [&](uint32_t l) {
      return (int)l < bi.nv ? bi.v0 + (int)l : L.halo_ids[bi.h0 + (int)l - bi.nv];
    };
    if (bi.nh > L.max_halo || L.bt_loc.size() != L.bt_nodes.size()) bad++;
    // triangle records: the packed local slots name the entry's ends
    for (int k = 0; k < bi.nt2 && L.bt_loc.size() == L.bt_nodes.size(); k++) {
      const uint32_t lc = L.bt_loc[bi.t0 + k];
      if (lc == kTriNoLoc) {
        if (k < bi.nt && nloc <= kTriLocMax) bad++;
        continue;
      }
      const int4 &t = L.bt_nodes[bi.t0 + k];
      for (int q = 0; q < 3; q++) {
        const uint32_t l = (lc >> (kTriLocBits * q)) & (uint32_t)(kTriLocMax - 1);
        if ((int)l >= nloc || !has(t, vert_of(l), q)) bad++;
      }
    }
    for (int k = 0; k < bi.ne; k++) {
      const uint32_t ll = L.be_loc[bi.e0 + k];
      const int2 nn = L.be_nodes[bi.e0 + k];
      if ((int)(ll & 0xffff) >= nloc || (int)(ll >> 16) >= nloc ||
          vert_of(ll & 0xffff) != nn.x || vert_of(ll >> 16) != nn.y)
        bad++;
    }
    for (int h = 1; h < bi.nh; h++)
      if (L.halo_ids[bi.h0 + h] <= L.halo_ids[bi.h0 + h - 1]) bad++;
    // the bulk-copy gradient pass stages [vt0, vt0 + nvt) in a tile of
    // 3 * max_tri + 16 entries and the block's vertex ranges from v0
    if (bi.vt0 != L.vt_ptr[bi.v0] || bi.nvt != L.vt_ptr[bi.v0 + bi.nv] - bi.vt0 ||
        bi.nvt > 3 * bi.nt || bi.v0 % kBlockVerts != 0)
      bad++;
    // own vertices: triangles among the block's own, ascending
    for (int v = bi.v0; v < bi.v0 + bi.nv; v++) {
      int last = -1;
      for (int j = L.vt_ptr[v]; j < L.vt_ptr[v + 1]; j++) {
        const int slot = L.vt_list[j] & 0x3fff, pos = L.vt_list[j] >> kTriPosShift;
        if (slot >= bi.nt || pos > 2 || !has(L.bt_nodes[bi.t0 + slot], v, pos) ||
            L.bt_nodes[bi.t0 + slot].w <= last) {
          bad++;
          break;
        }
        last = L.bt_nodes[bi.t0 + slot].w;
      }
      for (int j = L.ve_ptr[v]; j < L.ve_ptr[v + 1]; j++)
        if ((L.ve_list[j] & kSlotMask) >= nslot) bad++;
    }
    // halo vertices: the owner's triangles, in the owner's order
    for (int h = 0; h < bi.nh; h++) {
      const int v = L.halo_ids[bi.h0 + h];
      const int g0 = L.hl_ptr[bi.hp0 + h], g1 = L.hl_ptr[bi.hp0 + h + 1];
      const int o0 = L.vt_ptr[v], o1 = L.vt_ptr[v + 1];
      if (g1 - g0 != o1 - o0) {
        bad++;
        continue;
      }
      for (int j = 0; j < g1 - g0; j++) {
        const int slot = L.hl_list[g0 + j] & 0x3fff, pos = L.hl_list[g0 + j] >> kTriPosShift;
        if (slot >= bi.nt2 || pos > 2 || !has(L.bt_nodes[bi.t0 + slot], v, pos)) {
          bad++;
          break;
        }
      }
    }
  }
  // halo triangle order equals the owner's: compare driver triangle ids
  std::vector<int> owner(L.np, -1);
  for (int b = 0; b < L.nblk; b++)
    for (int v = L.blocks[b].v0; v < L.blocks[b].v0 + L.blocks[b].nv; v++) owner[v] = b;
  for (const BlockInfo &bi : L.blocks)
    for (int h = 0; h < bi.nh; h++) {
      const int v = L.halo_ids[bi.h0 + h];
      if (v < 0 || v >= L.np || owner[v] < 0) {
        bad++;
        continue;
      }
      const BlockInfo &ob = L.blocks[owner[v]];
      const int g0 = L.hl_ptr[bi.hp0 + h], o0 = L.vt_ptr[v], n = L.vt_ptr[v + 1] - o0;
      if (L.hl_ptr[bi.hp0 + h + 1] - g0 != n) continue;   // counted above
      for (int j = 0; j < n; j++)
        if (L.bt_nodes[bi.t0 + (L.hl_list[g0 + j] & 0x3fff)].w !=
            L.bt_nodes[ob.t0 + (L.vt_list[o0 + j] & 0x3fff)].w) {
          bad++;
          break;
        }
    }
  return bad;
}

}  // namespace fvm
