// HEX8 -> TET4 split (all_tri) and TET4 -> TET10 (all_second_order), plus the
// C-ABI entry points for the host mesh mirror.
#include <algorithm>
#include <array>
#include <map>
#include <new>

#include "lmg_internal.h"

namespace lmg {

static const int HEX8_SIDES_T[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5},
                                       {2, 3, 7, 6}, {3, 0, 4, 7}, {4, 5, 6, 7}};
static const int TET4_SIDES_T[4][3] = {{0, 2, 1}, {0, 1, 3}, {1, 2, 3}, {2, 0, 3}};

// Tables of the hex split (src/mesh/mesh_modification.C:90-91, 633-650).
static const int OPPOSING_NODE[8] = {6, 7, 4, 5, 2, 3, 0, 1};
static const int OPPOSING_NODES[8][3] = {{2, 5, 7}, {3, 4, 6}, {0, 5, 7}, {1, 4, 6},
                                         {1, 3, 6}, {0, 2, 7}, {1, 3, 4}, {0, 2, 5}};
static const int SIDES_OPPOSING_HIGHEST[8][3] = {{2, 3, 5}, {3, 4, 5}, {1, 4, 5}, {1, 2, 5},
                                                 {0, 2, 3}, {0, 3, 4}, {0, 1, 4}, {0, 1, 2}};
static const int NODES_NEIGHBORING_HIGHEST[8][3] = {{1, 3, 4}, {0, 2, 5}, {1, 3, 6}, {0, 2, 7},
                                                    {0, 5, 7}, {1, 4, 6}, {2, 5, 7}, {3, 4, 6}};

namespace {

struct Tet { int v[4]; };  // hex-local vertex numbers

// The diagonal of a hex face through its highest-id node
// (split_diagonal, mesh_modification.C:96-123).
std::pair<int, int> split_diagonal(const int32_t *ids, const int *side) {
  int hn = side[0];
  int32_t hid = ids[side[0]];
  for (int s = 0; s < 4; ++s)
    if (ids[side[s]] > hid) { hn = side[s]; hid = ids[side[s]]; }
  for (int s = 0; s < 4; ++s)
    for (int o = 0; o < 3; ++o)
      if (OPPOSING_NODES[hn][o] == side[s]) return {hn, side[s]};
  return {-1, -1};
}

bool in3(const int *a, int x) { return a[0] == x || a[1] == x || a[2] == x; }

// Elem::orient -> Tet::is_flipped (cell_tet.C:242) then Tet4::flip swaps nodes 0 and 2.
void orient(Tet &t, const double *xyz, const int32_t *ids) {
  const double *p0 = xyz + 3 * (int64_t)ids[t.v[0]], *p1 = xyz + 3 * (int64_t)ids[t.v[1]];
  const double *p2 = xyz + 3 * (int64_t)ids[t.v[2]], *p3 = xyz + 3 * (int64_t)ids[t.v[3]];
  double a[3], b[3], c[3];
  for (int d = 0; d < 3; ++d) { a[d] = p1[d] - p0[d]; b[d] = p2[d] - p0[d]; c[d] = p3[d] - p0[d]; }
  const double tp = a[0] * (b[1] * c[2] - b[2] * c[1]) - a[1] * (b[0] * c[2] - b[2] * c[0]) +
                    a[2] * (b[0] * c[1] - b[1] * c[0]);
  if (tp < 0) std::swap(t.v[0], t.v[2]);
}

// The HEX8 case of all_tri (mesh_modification.C:622-785).  Returns the number
// of tets written (5 or 6).
int split_hex(const int32_t *ids, const double *xyz, Tet *out) {
  int hn = 0;
  int32_t hid = ids[0];
  for (int n = 1; n < 8; ++n)
    if (ids[n] > hid) { hn = n; hid = ids[n]; }
  const int *nbr = NODES_NEIGHBORING_HIGHEST[hn];
  int nt = 0;
  bool made_null = false;
  for (int si = 0; si < 3; ++si) {
    const int *side = HEX8_SIDES_T[SIDES_OPPOSING_HIGHEST[hn][si]];
    auto [dn, dn2] = split_diagonal(ids, side);
    const bool split_on_neighbor = in3(nbr, dn) || in3(nbr, dn2);
    if (split_on_neighbor) {
      Tet t{{hn, dn, dn2, -1}};
      for (int s = 0; s < 4; ++s)
        if (side[s] != dn && side[s] != dn2) { t.v[3] = side[s]; break; }
      orient(t, xyz, ids);
      out[nt++] = t;
      Tet u{{hn, dn, dn2, -1}};
      for (int s = 3; s >= 0; --s)
        if (side[s] != dn && side[s] != dn2) { u.v[3] = side[s]; break; }
      orient(u, xyz, ids);
      out[nt++] = u;
    } else {
      Tet t{{hn, dn, dn2, -1}};
      for (int s = 0; s < 4 && t.v[3] < 0; ++s)
        if (in3(nbr, side[s])) t.v[3] = side[s];
      orient(t, xyz, ids);
      out[nt++] = t;
    }
  }
  if (nt == 3) {
    const int *on = OPPOSING_NODES[hn];
    Tet t{{on[0], on[1], on[2], OPPOSING_NODE[hn]}};
    orient(t, xyz, ids);
    out[nt++] = t;
    Tet u{{on[0], on[1], on[2], hn}};
    orient(u, xyz, ids);
    out[nt++] = u;
    made_null = true;  // the sixth sub-element is reset
  }
  if (nt == 4 || nt == 5) {
    for (int si = 0; si < 3; ++si) {
      const int *side = HEX8_SIDES_T[SIDES_OPPOSING_HIGHEST[hn][si]];
      auto [dn, dn2] = split_diagonal(ids, side);
      const bool split_on_neighbor = in3(nbr, dn) || in3(nbr, dn2);
      if (!split_on_neighbor) {
        Tet t{{hn, dn, dn2, OPPOSING_NODE[hn]}};
        orient(t, xyz, ids);
        out[nt++] = t;
      }
    }
  }
  (void)made_null;
  return nt;
}

}  // namespace

std::string all_tri_hex8(HostMesh &m) {
  if (m.elem_type != LMG_HEX8) return "all_tri: mesh is not HEX8";
  const int64_t E = m.n_elem();
  HostMesh t;
  t.elem_type = LMG_TET4;
  t.npe = 4;
  t.nsides = 4;
  t.xyz = m.xyz;
  t.conn.reserve((size_t)E * 24);
  t.side_bid.reserve((size_t)E * 24);
  Tet sub[6];
  for (int64_t e = 0; e < E; ++e) {
    const int32_t *ids = &m.conn[(size_t)(e * 8)];
    const int nt = split_hex(ids, m.xyz.data(), sub);
    if (nt < 5) return "all_tri: hex split failed";
    for (int s = 0; s < nt; ++s) {
      for (int a = 0; a < 4; ++a) t.conn.push_back(ids[sub[s].v[a]]);
      int8_t bid[4] = {-1, -1, -1, -1};
      // Boundary transfer (mesh_modification.C:1097-1155): a tet side inherits
      // the hex side's id when its vertices are a subset of that side's nodes.
      for (int hs = 0; hs < 6; ++hs) {
        const int8_t b = m.side_bid[(size_t)(e * 6 + hs)];
        if (b < 0) continue;
        std::array<int32_t, 4> hsn;
        for (int i = 0; i < 4; ++i) hsn[i] = ids[HEX8_SIDES_T[hs][i]];
        std::sort(hsn.begin(), hsn.end());
        for (int ts = 0; ts < 4; ++ts) {
          std::array<int32_t, 3> tsn;
          for (int i = 0; i < 3; ++i) tsn[i] = ids[sub[s].v[TET4_SIDES_T[ts][i]]];
          std::sort(tsn.begin(), tsn.end());
          if (std::includes(hsn.begin(), hsn.end(), tsn.begin(), tsn.end())) bid[ts] = b;
        }
      }
      for (int ts = 0; ts < 4; ++ts) t.side_bid.push_back(bid[ts]);
    }
  }
  renumber_nodes_first_touch(t);
  m = std::move(t);
  return "";
}

std::string all_second_order_tet4(HostMesh &m) {
  if (m.elem_type != LMG_TET4) return "all_second_order: mesh is not TET4";
  static const int EV[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
  const int64_t E = m.n_elem();
  int64_t next = m.n_nodes();
  std::map<std::pair<int32_t, int32_t>, int32_t> edge_node;
  std::vector<int32_t> conn((size_t)E * 10);
  std::vector<double> xyz = m.xyz;
  for (int64_t e = 0; e < E; ++e) {
    const int32_t *c4 = &m.conn[(size_t)(e * 4)];
    int32_t *c10 = &conn[(size_t)(e * 10)];
    for (int a = 0; a < 4; ++a) c10[a] = c4[a];
    for (int k = 0; k < 6; ++k) {
      int32_t lo = c4[EV[k][0]], hi = c4[EV[k][1]];
      if (lo > hi) std::swap(lo, hi);
      auto it = edge_node.find({lo, hi});
      if (it == edge_node.end()) {
        // New node at the average of the sorted adjacent vertices
        // (unstructured_mesh.C:128-136): ((0 + p_lo) + p_hi) / 2.
        for (int d = 0; d < 3; ++d) {
          double v = 0.0;
          v += xyz[(size_t)(3 * lo + d)];
          v += xyz[(size_t)(3 * hi + d)];
          v /= 2.0;
          xyz.push_back(v);
        }
        it = edge_node.emplace(std::make_pair(lo, hi), (int32_t)next++).first;
      }
      c10[4 + k] = it->second;
    }
  }
  m.elem_type = LMG_TET10;
  m.npe = 10;
  m.conn.swap(conn);
  m.xyz.swap(xyz);
  renumber_nodes_first_touch(m);
  return "";
}

// TET4 -> TET14 (MeshBase::all_complete_order, unstructured_mesh.C:60-170):
// per element in order, the new nodes 4..13 in local order, each keyed by its
// sorted adjacent vertices (Tet14 _second_order_adjacent_vertices: the edge's
// two vertices for 4..9, the face's three for 10..13) and placed, when first
// seen, at ((0 + p_a) + p_b [+ p_c]) / k over the sorted vertex ids.
std::string all_complete_order_tet4(HostMesh &m) {
  if (m.elem_type != LMG_TET4) return "all_complete_order: mesh is not TET4";
  static const int ADJ[10][3] = {{0, 1, -1}, {1, 2, -1}, {0, 2, -1}, {0, 3, -1}, {1, 3, -1},
                                 {2, 3, -1}, {0, 1, 2},  {0, 1, 3},  {1, 2, 3},  {0, 2, 3}};
  const int64_t E = m.n_elem();
  int64_t next = m.n_nodes();
  std::map<std::array<int32_t, 3>, int32_t> ho_node;
  std::vector<int32_t> conn((size_t)E * 14);
  std::vector<double> xyz = m.xyz;
  for (int64_t e = 0; e < E; ++e) {
    const int32_t *c4 = &m.conn[(size_t)(e * 4)];
    int32_t *c14 = &conn[(size_t)(e * 14)];
    for (int a = 0; a < 4; ++a) c14[a] = c4[a];
    for (int k = 0; k < 10; ++k) {
      const int nv = ADJ[k][2] < 0 ? 2 : 3;
      std::array<int32_t, 3> key = {c4[ADJ[k][0]], c4[ADJ[k][1]], nv == 3 ? c4[ADJ[k][2]] : -1};
      std::sort(key.begin(), key.begin() + nv);
      auto it = ho_node.find(key);
      if (it == ho_node.end()) {
        for (int d = 0; d < 3; ++d) {
          double v = 0.0;
          for (int t = 0; t < nv; ++t) v += xyz[(size_t)(3 * key[t] + d)];
          v /= (double)nv;
          xyz.push_back(v);
        }
        it = ho_node.emplace(key, (int32_t)next++).first;
      }
      c14[4 + k] = it->second;
    }
  }
  m.elem_type = LMG_TET14;
  m.npe = 14;
  m.conn.swap(conn);
  m.xyz.swap(xyz);
  renumber_nodes_first_touch(m);
  return "";
}

}  // namespace lmg

extern "C" {

lmg_status lmg_mesh_cube(int32_t nx, int32_t ny, int32_t nz, int32_t elem_type, double jitter,
                         uint64_t seed, lmg_mesh **out) {
  if (!out) return LMG_ERR_ARG;
  *out = nullptr;
  if (jitter < 0.0 || jitter >= 0.5) return LMG_ERR_ARG;
  lmg_mesh *mesh = new (std::nothrow) lmg_mesh;
  if (!mesh) return LMG_ERR_OOM;
  try {
    const bool tets = (elem_type == LMG_TET4 || elem_type == LMG_TET10 || elem_type == LMG_TET14);
    const int base = tets ? LMG_HEX8 : elem_type;
    std::string err = lmg::build_cube_hex(mesh->m, nx, ny, nz, base);
    const bool prism_hi = elem_type == LMG_PRISM18 || elem_type == LMG_PRISM21;
    if (err.empty() && prism_hi && jitter != 0.0) err = "build_cube: PRISM18 / PRISM21 meshes are not jittered";
    if (err.empty()) lmg::jitter_interior(mesh->m, jitter, nx, ny, nz, seed);
    if (err.empty() && !tets && elem_type != LMG_PRISM6 && !prism_hi && jitter == 0.0) {  // unjittered hex cube: lattice for refinement
      mesh->m.cube[0] = nx;
      mesh->m.cube[1] = ny;
      mesh->m.cube[2] = nz;
    }
    if (err.empty() && tets) err = lmg::all_tri_hex8(mesh->m);
    if (err.empty() && elem_type == LMG_TET10) err = lmg::all_second_order_tet4(mesh->m);
    if (err.empty() && elem_type == LMG_TET14) err = lmg::all_complete_order_tet4(mesh->m);
    if (!err.empty()) {
      delete mesh;
      return (elem_type == LMG_HEX8 || elem_type == LMG_HEX27 || elem_type == LMG_PRISM6 || prism_hi || tets)
                 ? LMG_ERR_ARG
                 : LMG_ERR_UNSUPPORTED;
    }
  } catch (const std::bad_alloc &) {
    delete mesh;
    return LMG_ERR_OOM;
  }
  *out = mesh;
  return LMG_OK;
}

lmg_status lmg_mesh_info(const lmg_mesh *m, int64_t *n_nodes, int64_t *n_elem, int32_t *elem_type,
                         int32_t *nodes_per_elem, int32_t *sides_per_elem) {
  if (!m) return LMG_ERR_ARG;
  if (n_nodes) *n_nodes = m->m.n_nodes();
  if (n_elem) *n_elem = m->m.n_elem();
  if (elem_type) *elem_type = m->m.elem_type;
  if (nodes_per_elem) *nodes_per_elem = m->m.npe;
  if (sides_per_elem) *sides_per_elem = m->m.nsides;
  return LMG_OK;
}

lmg_status lmg_mesh_copy(const lmg_mesh *m, double *xyz, int32_t *conn, int8_t *side_bid) {
  if (!m) return LMG_ERR_ARG;
  if (xyz) std::copy(m->m.xyz.begin(), m->m.xyz.end(), xyz);
  if (conn) std::copy(m->m.conn.begin(), m->m.conn.end(), conn);
  if (side_bid) std::copy(m->m.side_bid.begin(), m->m.side_bid.end(), side_bid);
  return LMG_OK;
}

lmg_status lmg_mesh_free(lmg_mesh *m) {
  delete m;
  return LMG_OK;
}

}  // extern "C"
