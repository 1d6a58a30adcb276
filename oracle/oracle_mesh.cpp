// CPU oracle — test infrastructure only (tests/, the smoke check and the CPU
// legs of bench.py use it as the checker; the product never links it).
//
// Restatement of libMesh's structured mesh generation for the benchmark
// meshes, written from the reference sources step by step:
//   MeshTools::Generation::build_cube (HEX8 / HEX27 / PRISM18 / PRISM21 node
//     grids and element loops, boundary ids) src/mesh/mesh_generation.C:1281-1377, 1398-1430, 1569-1604,
//                                            1634-1745, 1776-1786
//   MeshBase::prepare_for_use -> ReplicatedMesh::renumber_nodes_and_elements
//     (elements compacted in id order, nodes renumbered by the swap walk)
//                                            src/mesh/replicated_mesh.C:700-800
//   MeshTools::Modification::all_tri, HEX8 case (highest vertex, split
//     diagonals, 5- or 6-tet split, Elem::orient, new ids
//     max_orig_id + 6 id + i, boundary sides by vertex inclusion)
//                                            src/mesh/mesh_modification.C:88-123, 615-790, 1097-1200
//   Tet::is_flipped / Tet4::flip             src/geom/cell_tet.C:242-247, src/geom/cell_tet4.C:613-622
//   MeshBase::all_second_order (TET4 -> TET10: new node per sorted adjacent
//     vertex set, placed at their average, appended)
//                                            src/mesh/unstructured_mesh.C:60-200, 1732-1790
// The interior-vertex jitter is the synthetic-input rule of the benchmark
// meshes (not a libMesh operation): after build_cube, every node with no
// coordinate equal to 0 or 1, in node id order, moves by (2u - 1) amp h per
// coordinate, u from a splitmix64 stream (53-bit uniforms).
#include <algorithm>
#include <array>
#include <cstdint>
#include <map>
#include <memory>
#include <vector>

namespace {

struct OMesh {
  int type = 0;   // libMesh ElemType value: 10 HEX8, 12 HEX27, 8 TET4, 9 TET10
  int npe = 0, nsides = 0;
  std::vector<std::array<double, 3>> nodes;
  // element slots indexed by id (null slots are deleted or unused ids)
  std::vector<std::unique_ptr<std::vector<int64_t>>> elems;
  std::vector<std::unique_ptr<std::vector<int>>> bids;  // per element, per side (-1 none)
};

// ReplicatedMesh::renumber_nodes_and_elements: compact the element slots in
// id order; walk the elements' nodes, and whenever a node id exceeds the next
// free id, swap the two node slots (the node moved out of the way keeps its
// place in line for a later swap).
void renumber(OMesh &m) {
  std::vector<std::unique_ptr<std::vector<int64_t>>> el;
  std::vector<std::unique_ptr<std::vector<int>>> bd;
  for (size_t i = 0; i < m.elems.size(); ++i)
    if (m.elems[i]) {
      el.push_back(std::move(m.elems[i]));
      bd.push_back(std::move(m.bids[i]));
    }
  m.elems.swap(el);
  m.bids.swap(bd);
  const int64_t n = (int64_t)m.nodes.size();
  std::vector<int64_t> slot_of(n), node_at(n);  // current slot of original node / node in a slot
  for (int64_t i = 0; i < n; ++i) slot_of[i] = node_at[i] = i;
  int64_t next_free = 0;
  for (auto &e : m.elems)
    for (int64_t orig : *e) {
      const int64_t id = slot_of[orig];
      if (id == next_free) {
        ++next_free;
      } else if (id > next_free) {
        const int64_t dst = next_free++;
        const int64_t other = node_at[dst];
        node_at[dst] = orig;
        slot_of[orig] = dst;
        node_at[id] = other;
        slot_of[other] = id;
      }
    }
  std::vector<std::array<double, 3>> nodes(n);
  for (int64_t s = 0; s < n; ++s) nodes[s] = m.nodes[node_at[s]];
  m.nodes.swap(nodes);
  for (auto &e : m.elems)
    for (auto &v : *e) v = slot_of[v];
}

uint64_t splitmix(uint64_t &s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// build_cube(nx, ny, nz, 0..1 x3, HEX8 | HEX27) + prepare_for_use
void build_cube(OMesh &m, int nx, int ny, int nz, int type) {
  const bool q = (type == 12);
  const int f = q ? 2 : 1;
  const int64_t gx = (int64_t)f * nx + 1, gy = (int64_t)f * ny + 1, gz = (int64_t)f * nz + 1;
  auto idx = [&](int64_t i, int64_t j, int64_t k) { return i + gx * (j + gy * k); };
  m.type = type;
  m.npe = q ? 27 : 8;
  m.nsides = 6;
  m.nodes.clear();
  for (int64_t k = 0; k < gz; ++k)
    for (int64_t j = 0; j < gy; ++j)
      for (int64_t i = 0; i < gx; ++i) {
        std::array<double, 3> p = {(double)i / (double)(f * nx), (double)j / (double)(f * ny),
                                   (double)k / (double)(f * nz)};
        for (int d = 0; d < 3; ++d) p[d] = p[d] * (1.0 - 0.0) + 0.0;
        m.nodes.push_back(p);
      }
  // HEX27 node offsets on the doubled grid, libMesh local order
  static const int H27[27][3] = {{0, 0, 0}, {2, 0, 0}, {2, 2, 0}, {0, 2, 0}, {0, 0, 2}, {2, 0, 2}, {2, 2, 2},
                                 {0, 2, 2}, {1, 0, 0}, {2, 1, 0}, {1, 2, 0}, {0, 1, 0}, {0, 0, 1}, {2, 0, 1},
                                 {2, 2, 1}, {0, 2, 1}, {1, 0, 2}, {2, 1, 2}, {1, 2, 2}, {0, 1, 2}, {1, 1, 0},
                                 {1, 0, 1}, {2, 1, 1}, {1, 2, 1}, {0, 1, 1}, {1, 1, 2}, {1, 1, 1}};
  static const int H8[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                               {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
  m.elems.clear();
  m.bids.clear();
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        auto e = std::make_unique<std::vector<int64_t>>();
        for (int a = 0; a < m.npe; ++a) {
          const int *o = q ? H27[a] : H8[a];
          e->push_back(idx((int64_t)f * i + o[0], (int64_t)f * j + o[1], (int64_t)f * k + o[2]));
        }
        auto b = std::make_unique<std::vector<int>>(6, -1);
        if (k == 0) (*b)[0] = 0;
        if (k == nz - 1) (*b)[5] = 5;
        if (j == 0) (*b)[1] = 1;
        if (j == ny - 1) (*b)[3] = 3;
        if (i == 0) (*b)[4] = 4;
        if (i == nx - 1) (*b)[2] = 2;
        m.elems.push_back(std::move(e));
        m.bids.push_back(std::move(b));
      }
  renumber(m);
}

// build_cube(nx, ny, nz, 0..1 x3, PRISM18 | PRISM21) + prepare_for_use
// (mesh_generation.C:1324-1377 nodes, 1634-1745 elements): the (2n+1)^3 node
// grid in k, j, i order, for PRISM21 then two nodes per (k, j, i) with k over
// all 2 nz + 1 grid levels and (j, i) over the cells; two prisms per cell.
void build_cube_prism(OMesh &m, int nx, int ny, int nz, int type) {
  const bool p21 = type == 36;
  const int64_t gx = 2 * (int64_t)nx + 1, gy = 2 * (int64_t)ny + 1, gz = 2 * (int64_t)nz + 1;
  auto idx = [&](int64_t i, int64_t j, int64_t k) { return i + gx * (j + gy * k); };
  m.type = type;
  m.npe = p21 ? 21 : 18;
  m.nsides = 5;
  m.nodes.clear();
  for (int64_t k = 0; k <= 2 * nz; ++k)
    for (int64_t j = 0; j <= 2 * ny; ++j)
      for (int64_t i = 0; i <= 2 * nx; ++i)
        m.nodes.push_back({(double)i / (double)(2 * nx), (double)j / (double)(2 * ny), (double)k / (double)(2 * nz)});
  if (p21) {
    const int64_t kmax = 2 * (int64_t)nz;
    for (int64_t k = 0; k <= kmax; k++)
      for (int64_t j = 0; j < ny; j++)
        for (int64_t i = 0; i < nx; i++) {
          m.nodes.push_back({((double)i + 1 / 3.0) / (double)nx, ((double)j + 1 / 3.0) / (double)ny,
                             (double)k / (double)kmax});
          m.nodes.push_back({((double)i + 2 / 3.0) / (double)nx, ((double)j + 2 / 3.0) / (double)ny,
                             (double)k / (double)kmax});
        }
  }
  for (auto &p : m.nodes)
    for (int d = 0; d < 3; ++d) p[d] = p[d] * (1.0 - 0.0) + 0.0;
  const int64_t base = gx * gy * gz;
  m.elems.clear();
  m.bids.clear();
  for (int64_t k = 0; k < 2 * nz; k += 2)
    for (int64_t j = 0; j < 2 * ny; j += 2)
      for (int64_t i = 0; i < 2 * nx; i += 2) {
        // first prism
        auto e = std::make_unique<std::vector<int64_t>>(std::vector<int64_t>{
            idx(i, j, k), idx(i + 2, j, k), idx(i, j + 2, k), idx(i, j, k + 2), idx(i + 2, j, k + 2),
            idx(i, j + 2, k + 2), idx(i + 1, j, k), idx(i + 1, j + 1, k), idx(i, j + 1, k), idx(i, j, k + 1),
            idx(i + 2, j, k + 1), idx(i, j + 2, k + 1), idx(i + 1, j, k + 2), idx(i + 1, j + 1, k + 2),
            idx(i, j + 1, k + 2), idx(i + 1, j, k + 1), idx(i + 1, j + 1, k + 1), idx(i, j + 1, k + 1)});
        if (p21) {
          e->push_back(base + (k * (nx * ny) + j / 2 * nx + i / 2) * 2);
          e->push_back(base + ((k + 2) * (nx * ny) + j / 2 * nx + i / 2) * 2);
          e->push_back(base + ((k + 1) * (nx * ny) + j / 2 * nx + i / 2) * 2);
        }
        auto b = std::make_unique<std::vector<int>>(5, -1);
        if (i == 0) (*b)[3] = 4;
        if (j == 0) (*b)[1] = 1;
        if (k == 0) (*b)[0] = 0;
        if (k == 2 * (nz - 1)) (*b)[4] = 5;
        m.elems.push_back(std::move(e));
        m.bids.push_back(std::move(b));
        // second prism
        e = std::make_unique<std::vector<int64_t>>(std::vector<int64_t>{
            idx(i + 2, j, k), idx(i + 2, j + 2, k), idx(i, j + 2, k), idx(i + 2, j, k + 2), idx(i + 2, j + 2, k + 2),
            idx(i, j + 2, k + 2), idx(i + 2, j + 1, k), idx(i + 1, j + 2, k), idx(i + 1, j + 1, k),
            idx(i + 2, j, k + 1), idx(i + 2, j + 2, k + 1), idx(i, j + 2, k + 1), idx(i + 2, j + 1, k + 2),
            idx(i + 1, j + 2, k + 2), idx(i + 1, j + 1, k + 2), idx(i + 2, j + 1, k + 1), idx(i + 1, j + 2, k + 1),
            idx(i + 1, j + 1, k + 1)});
        if (p21) {
          e->push_back(base + (k * (nx * ny) + j / 2 * nx + i / 2) * 2 + 1);
          e->push_back(base + ((k + 2) * (nx * ny) + j / 2 * nx + i / 2) * 2 + 1);
          e->push_back(base + ((k + 1) * (nx * ny) + j / 2 * nx + i / 2) * 2 + 1);
        }
        b = std::make_unique<std::vector<int>>(5, -1);
        if (i == 2 * (nx - 1)) (*b)[1] = 2;
        if (j == 2 * (ny - 1)) (*b)[2] = 3;
        if (k == 0) (*b)[0] = 0;
        if (k == 2 * (nz - 1)) (*b)[4] = 5;
        m.elems.push_back(std::move(e));
        m.bids.push_back(std::move(b));
      }
  renumber(m);
}

void jitter(OMesh &m, double amp, int nx, int ny, int nz, uint64_t seed) {
  if (amp == 0.0) return;
  uint64_t s = seed;
  const double h[3] = {1.0 / nx, 1.0 / ny, 1.0 / nz};
  for (auto &p : m.nodes) {
    if (p[0] == 0.0 || p[0] == 1.0 || p[1] == 0.0 || p[1] == 1.0 || p[2] == 0.0 || p[2] == 1.0) continue;
    for (int d = 0; d < 3; ++d) {
      const double u = (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
      p[d] += (2.0 * u - 1.0) * amp * h[d];
    }
  }
}

const int HEX_SIDE[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}, {4, 5, 6, 7}};
const int TET_SIDE[4][3] = {{0, 2, 1}, {0, 1, 3}, {1, 2, 3}, {2, 0, 3}};
const unsigned OPP_NODES[8][3] = {{2, 5, 7}, {3, 4, 6}, {0, 5, 7}, {1, 4, 6}, {1, 3, 6}, {0, 2, 7}, {1, 3, 4}, {0, 2, 5}};
const unsigned OPP_NODE[8] = {6, 7, 4, 5, 2, 3, 0, 1};
const unsigned SIDES_OPP_HIGHEST[8][3] = {{2, 3, 5}, {3, 4, 5}, {1, 4, 5}, {1, 2, 5},
                                          {0, 2, 3}, {0, 3, 4}, {0, 1, 4}, {0, 1, 2}};
const unsigned NODES_NBR_HIGHEST[8][3] = {{1, 3, 4}, {0, 2, 5}, {1, 3, 6}, {0, 2, 7},
                                          {0, 5, 7}, {1, 4, 6}, {2, 5, 7}, {3, 4, 6}};

// all_tri on a HEX8 mesh + prepare_for_use
void all_tri(OMesh &m) {
  const int64_t max_orig_id = (int64_t)m.elems.size();  // ids are 0..n-1 after prepare_for_use
  std::vector<std::unique_ptr<std::vector<int64_t>>> out((size_t)(max_orig_id + 6 * max_orig_id));
  std::vector<std::unique_ptr<std::vector<int>>> outb(out.size());
  for (int64_t id = 0; id < max_orig_id; ++id) {
    const std::vector<int64_t> &h = *m.elems[id];
    unsigned hn = 0;  // highest_vertex_on: first vertex with the largest node id
    for (unsigned n = 1; n < 8; ++n)
      if (h[n] > h[hn]) hn = n;
    auto diag = [&](const int *side) {  // split_diagonal
      unsigned hs = side[0];
      for (int s = 0; s < 4; ++s)
        if (h[side[s]] > h[hs]) hs = side[s];
      for (int s = 0; s < 4; ++s)
        for (unsigned o : OPP_NODES[hs])
          if ((int)o == side[s]) return std::make_pair(hs, o);
      return std::make_pair(99u, 99u);
    };
    auto nbr = [&](unsigned n) {
      for (unsigned x : NODES_NBR_HIGHEST[hn])
        if (x == n) return true;
      return false;
    };
    std::vector<std::array<unsigned, 4>> sub;
    std::vector<bool> present;
    for (unsigned side : SIDES_OPP_HIGHEST[hn]) {
      const int *sn = HEX_SIDE[side];
      auto [dn, dn2] = diag(sn);
      const bool on_nbr = nbr(dn) || nbr(dn2);
      if (on_nbr) {
        std::array<unsigned, 4> t = {hn, dn, dn2, 99};
        for (int s = 0; s < 4; ++s)
          if ((unsigned)sn[s] != dn && (unsigned)sn[s] != dn2) { t[3] = sn[s]; break; }
        sub.push_back(t);
        std::array<unsigned, 4> u = {hn, dn, dn2, 99};
        for (int s = 3; s >= 0; --s)
          if ((unsigned)sn[s] != dn && (unsigned)sn[s] != dn2) { u[3] = sn[s]; break; }
        sub.push_back(u);
      } else {
        std::array<unsigned, 4> t = {hn, dn, dn2, 99};
        for (int s = 0; s < 4 && t[3] == 99; ++s)
          if (nbr(sn[s])) t[3] = sn[s];
        sub.push_back(t);
      }
    }
    present.assign(sub.size(), true);
    if (sub.size() == 3) {
      const unsigned *on = OPP_NODES[hn];
      sub.push_back({on[0], on[1], on[2], OPP_NODE[hn]});
      sub.push_back({on[0], on[1], on[2], hn});
      sub.push_back({0, 0, 0, 0});  // the sixth sub-element is reset
      present.assign(6, true);
      present[5] = false;
    }
    if (sub.size() == 4 || sub.size() == 5) {
      for (unsigned side : SIDES_OPP_HIGHEST[hn]) {
        auto [dn, dn2] = diag(HEX_SIDE[side]);
        if (!(nbr(dn) || nbr(dn2))) sub.push_back({hn, dn, dn2, OPP_NODE[hn]});
      }
      present.assign(sub.size(), true);
    }
    for (size_t i = 0; i < sub.size(); ++i) {
      if (!present[i]) continue;
      std::vector<int64_t> t = {h[sub[i][0]], h[sub[i][1]], h[sub[i][2]], h[sub[i][3]]};
      // Elem::orient: Tet::is_flipped (triple product < 0) -> Tet4::flip swaps nodes 0 and 2
      const auto &p0 = m.nodes[t[0]], &p1 = m.nodes[t[1]], &p2 = m.nodes[t[2]], &p3 = m.nodes[t[3]];
      const double a[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
      const double b[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
      const double c[3] = {p3[0] - p0[0], p3[1] - p0[1], p3[2] - p0[2]};
      const double tp = a[0] * (b[1] * c[2] - b[2] * c[1]) - a[1] * (b[0] * c[2] - b[2] * c[0]) +
                        a[2] * (b[0] * c[1] - b[1] * c[0]);
      if (tp < 0) std::swap(t[0], t[2]);
      // boundary sides: a tet side whose vertices all lie on a hex side with an id
      auto bd = std::make_unique<std::vector<int>>(4, -1);
      for (int hs = 0; hs < 6; ++hs) {
        const int bid = (*m.bids[id])[hs];
        if (bid < 0) continue;
        std::vector<int64_t> hsn;
        for (int s = 0; s < 4; ++s) hsn.push_back(h[HEX_SIDE[hs][s]]);
        std::sort(hsn.begin(), hsn.end());
        for (int ts = 0; ts < 4; ++ts) {
          std::vector<int64_t> tsn;
          for (int s = 0; s < 3; ++s) tsn.push_back(t[TET_SIDE[ts][s]]);
          std::sort(tsn.begin(), tsn.end());
          if (std::includes(hsn.begin(), hsn.end(), tsn.begin(), tsn.end())) (*bd)[ts] = bid;
        }
      }
      const int64_t nid = max_orig_id + 6 * id + (int64_t)i;
      out[nid] = std::make_unique<std::vector<int64_t>>(t);
      outb[nid] = std::move(bd);
    }
  }
  m.elems.swap(out);
  m.bids.swap(outb);
  m.type = 8;
  m.npe = 4;
  m.nsides = 4;
  renumber(m);
}

// all_second_order on a TET4 mesh + prepare_for_use
void second_order(OMesh &m) {
  static const int ADJ[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
  std::map<std::vector<int64_t>, int64_t> ho;
  for (auto &e : m.elems) {
    std::vector<int64_t> &t = *e;
    for (int k = 0; k < 6; ++k) {
      std::vector<int64_t> key = {t[ADJ[k][0]], t[ADJ[k][1]]};
      std::sort(key.begin(), key.end());
      auto it = ho.find(key);
      if (it == ho.end()) {
        std::array<double, 3> p = {0.0, 0.0, 0.0};
        for (int64_t v : key)
          for (int d = 0; d < 3; ++d) p[d] += m.nodes[v][d];
        for (int d = 0; d < 3; ++d) p[d] /= (double)key.size();
        m.nodes.push_back(p);
        it = ho.emplace(key, (int64_t)m.nodes.size() - 1).first;
      }
      t.push_back(it->second);
    }
  }
  m.type = 9;
  m.npe = 10;
  renumber(m);
}

}  // namespace

extern "C" {

// The benchmark meshes: elem_type 10 HEX8 / 12 HEX27 (build_cube, jitter),
// 8 TET4 / 9 TET10 (build_cube HEX8, jitter, all_tri [, all_second_order]),
// 15 PRISM18 / 36 PRISM21 (build_cube, no jitter).
// Returns a handle (null on a bad argument).
void *orc_mesh_cube(int nx, int ny, int nz, int elem_type, double amp, uint64_t seed) {
  if (nx <= 0 || ny <= 0 || nz <= 0) return nullptr;
  if (elem_type != 10 && elem_type != 12 && elem_type != 8 && elem_type != 9 && elem_type != 15 && elem_type != 36)
    return nullptr;
  auto *m = new OMesh;
  if (elem_type == 15 || elem_type == 36) {  // unjittered prisms of order 2 / 3
    if (amp != 0.0) {
      delete m;
      return nullptr;
    }
    build_cube_prism(*m, nx, ny, nz, elem_type);
    return m;
  }
  const bool tets = elem_type == 8 || elem_type == 9;
  build_cube(*m, nx, ny, nz, tets ? 10 : elem_type);
  jitter(*m, amp, nx, ny, nz, seed);
  if (tets) all_tri(*m);
  if (elem_type == 9) second_order(*m);
  return m;
}

void orc_mesh_info(void *h, int64_t *n_nodes, int64_t *n_elem, int32_t *npe, int32_t *nsides) {
  const OMesh &m = *static_cast<OMesh *>(h);
  *n_nodes = (int64_t)m.nodes.size();
  *n_elem = (int64_t)m.elems.size();
  *npe = m.npe;
  *nsides = m.nsides;
}

void orc_mesh_copy(void *h, double *xyz, int32_t *conn, int8_t *side_bid) {
  const OMesh &m = *static_cast<OMesh *>(h);
  for (size_t i = 0; i < m.nodes.size(); ++i)
    for (int d = 0; d < 3; ++d) xyz[3 * i + d] = m.nodes[i][d];
  for (size_t e = 0; e < m.elems.size(); ++e) {
    for (int a = 0; a < m.npe; ++a) conn[e * m.npe + a] = (int32_t)(*m.elems[e])[a];
    for (int s = 0; s < m.nsides; ++s) side_bid[e * m.nsides + s] = (int8_t)(*m.bids[e])[s];
  }
}

void orc_mesh_free(void *h) { delete static_cast<OMesh *>(h); }

}  // extern "C"
