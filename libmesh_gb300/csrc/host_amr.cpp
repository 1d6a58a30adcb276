// Host mirror of libMesh's h-refinement and hanging-node constraints for
// structured hex cubes (the inputs of the constrained assembly path).
//
//   MeshRefinement::refine_and_coarsen_elements   src/mesh/mesh_refinement.C:482-786
//     level-one rule across faces (make_refinement_compatible, face mismatch 1)
//   Elem::refine / MeshRefinement::add_node        src/geom/elem_refinement.C:87-150;
//                                                  src/mesh/mesh_refinement.C:141-205
//     children appended after all existing elements, child c at parent vertex c;
//     a new node is sum_n embedding(c, node, n) * parent point n (n ascending,
//     zero weights skipped, src/geom/cell_hex27.C:794 embedding matrices =
//     tensor products of the 1-D Lagrange shapes at the child node)
//   ReplicatedMesh::renumber_nodes_and_elements    src/mesh/replicated_mesh.C:700-860
//     node ids in first-touch order over every element (parents included)
//   lagrange_compute_constraints                   src/fe/fe_lagrange.C:867-1063
//   DofMap::process_constraints                    src/base/dof_map_constraints.C:4341-4490
//   AddPrimalConstraint (Dirichlet rows only for dofs still free)
//                                                  src/base/dof_map_constraints.C:216-228
//
// Nodes and element corners sit on an integer lattice (level-0 edge AMR_S0),
// so a node shared by several parents is found by its lattice position, the
// same node libMesh finds through its bracketing-node map.  The parent-side
// coordinates of a hanging node are exact lattice ratios (what FEMap::inverse_map
// converges to on these affine faces).
#include <algorithm>
#include <cmath>
#include <map>
#include <new>
#include <set>
#include <unordered_map>

#include "lmg_internal.h"

namespace lmg {

namespace {

// Hex vertex c sits at lattice offset HEX_VBITS[c] * size (cell_hex8.C node order).
const int HEX_VBITS[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                             {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
// HEX27 node offsets in half edges (build_cube's doubled-grid stencil).
const int HEX27_OFF[27][3] = {
    {0, 0, 0}, {2, 0, 0}, {2, 2, 0}, {0, 2, 0}, {0, 0, 2}, {2, 0, 2}, {2, 2, 2}, {0, 2, 2}, {1, 0, 0},
    {2, 1, 0}, {1, 2, 0}, {0, 1, 0}, {0, 0, 1}, {2, 0, 1}, {2, 2, 1}, {0, 2, 1}, {1, 0, 2}, {2, 1, 2},
    {1, 2, 2}, {0, 1, 2}, {1, 1, 0}, {1, 0, 1}, {2, 1, 1}, {1, 2, 1}, {0, 1, 1}, {1, 1, 2}, {1, 1, 1}};
// Outward normal axis and sign of hex side s (side 0: z-, 1: y-, 2: x+, 3: y+, 4: x-, 5: z+).
const int SIDE_AXIS[6] = {2, 1, 0, 1, 0, 2};
const int SIDE_SIGN[6] = {-1, -1, 1, 1, -1, 1};

// node offset of local node a in units of (element size / 2)
inline void node_offset(int npe, int a, int o[3]) {
  for (int d = 0; d < 3; ++d) o[d] = (npe == 27) ? HEX27_OFF[a][d] : 2 * HEX_VBITS[a][d];
}

// 1-D Lagrange shapes on [-1,1]: linear (index 0 at -1, 1 at +1) and quadratic
// (0 at -1, 1 at +1, 2 at 0), include/fe/fe_lagrange_shape_1D.h.
inline double shape1d(int order, int i, double xi) {
  if (order == 1) return i == 0 ? .5 * (1. - xi) : .5 * (1. + xi);
  switch (i) {
    case 0: return .5 * xi * (xi - 1.);
    case 1: return .5 * xi * (xi + 1.);
    default: return (1. - xi) * (1. + xi);
  }
}
// 1-D index of a node offset (0, 1, 2 half edges) in the quadratic basis
inline int quad_index(int off) { return off == 0 ? 0 : (off == 2 ? 1 : 2); }

struct LatKey {
  int64_t x, y, z;
  bool operator==(const LatKey &o) const { return x == o.x && y == o.y && z == o.z; }
};
// Node lookup by lattice point: open addressing over the packed point
// (21 bits per coordinate; init_tree bounds the grid so that every lattice
// coordinate fits), linear probing, power-of-two capacity kept under half full.
class LatMap {
 public:
  explicit LatMap(size_t expect) {
    size_t cap = 16;
    while (cap < 2 * expect + 16) cap <<= 1;
    keys_.assign(cap, EMPTY);
    vals_.assign(cap, -1);
  }
  // id of point k, or -1
  int32_t find(const LatKey &k) const {
    const uint64_t key = pack(k);
    for (size_t i = slot(key);; i = (i + 1) & (keys_.size() - 1)) {
      if (keys_[i] == key) return vals_[i];
      if (keys_[i] == EMPTY) return -1;
    }
  }
  void insert(const LatKey &k, int32_t id) {
    if (2 * (n_ + 1) > keys_.size()) grow();
    place(pack(k), id);
  }

 private:
  static constexpr uint64_t EMPTY = ~0ull;
  static uint64_t pack(const LatKey &k) {
    return (uint64_t)k.x | ((uint64_t)k.y << 21) | ((uint64_t)k.z << 42);
  }
  size_t slot(uint64_t key) const {  // splitmix64 finaliser
    uint64_t h = key + 0x9E3779B97F4A7C15ull;
    h = (h ^ (h >> 30)) * 0xBF58476D1CE4E5B9ull;
    h = (h ^ (h >> 27)) * 0x94D049BB133111EBull;
    return (size_t)(h ^ (h >> 31)) & (keys_.size() - 1);
  }
  void place(uint64_t key, int32_t id) {
    size_t i = slot(key);
    while (keys_[i] != EMPTY && keys_[i] != key) i = (i + 1) & (keys_.size() - 1);
    if (keys_[i] == EMPTY) ++n_;
    keys_[i] = key;
    vals_[i] = id;
  }
  void grow() {
    std::vector<uint64_t> k;
    std::vector<int32_t> v;
    k.swap(keys_);
    v.swap(vals_);
    keys_.assign(k.size() * 2, EMPTY);
    vals_.assign(k.size() * 2, -1);
    n_ = 0;
    for (size_t i = 0; i < k.size(); ++i)
      if (k[i] != EMPTY) place(k[i], v[i]);
  }
  std::vector<uint64_t> keys_;
  std::vector<int32_t> vals_;
  size_t n_ = 0;
};

int64_t elem_size(const AmrTree &t, int32_t e) { return AMR_S0 >> t.level[(size_t)e]; }

// Active element containing lattice point p (strictly inside a cell), -1 outside the cube.
int32_t locate(const AmrTree &t, const int64_t p[3]) {
  const int64_t n[3] = {t.nx, t.ny, t.nz};
  int64_t c[3];
  for (int d = 0; d < 3; ++d) {
    if (p[d] <= 0 || p[d] >= n[d] * AMR_S0) return -1;
    c[d] = p[d] / AMR_S0;
  }
  int32_t e = (int32_t)(c[0] + t.nx * (c[1] + t.ny * c[2]));
  while (t.first_child[(size_t)e] >= 0) {
    const int64_t h = elem_size(t, e) / 2;
    int b[3];
    for (int d = 0; d < 3; ++d) b[d] = (p[d] - t.origin[3 * (size_t)e + d]) >= h ? 1 : 0;
    int child = 0;
    for (int v = 0; v < 8; ++v)
      if (HEX_VBITS[v][0] == b[0] && HEX_VBITS[v][1] == b[1] && HEX_VBITS[v][2] == b[2]) child = v;
    e = t.first_child[(size_t)e] + child;
  }
  return e;
}

// Active element across side s of e (the neighbor libMesh links: same level
// or coarser; finer regions report one of their elements), -1 on the boundary.
int32_t across(const AmrTree &t, int32_t e, int s) {
  const int64_t S = elem_size(t, e);
  int64_t p[3];
  for (int d = 0; d < 3; ++d) p[d] = t.origin[3 * (size_t)e + d] + S / 2;
  const int ax = SIDE_AXIS[s];
  p[ax] = t.origin[3 * (size_t)e + ax] + (SIDE_SIGN[s] > 0 ? S + 1 : -1);
  return locate(t, p);
}

bool child_on_side(int c, int s) {
  int sn[9];
  side_nodes(LMG_HEX8, s, sn);
  for (int i = 0; i < 4; ++i)
    if (sn[i] == c) return true;
  return false;
}

std::string init_tree(HostMesh &m) {
  AmrTree &t = m.amr;
  if (m.elem_type != LMG_HEX8 && m.elem_type != LMG_HEX27) return "refine: HEX8 or HEX27 cube required";
  if (m.cube[0] <= 0) return "refine: only unjittered build_cube meshes carry the lattice";
  t.nx = m.cube[0];
  t.ny = m.cube[1];
  t.nz = m.cube[2];
  if (t.nx > 2000 || t.ny > 2000 || t.nz > 2000) return "refine: grid too large for the lattice";
  const int64_t E = m.n_elem();
  t.conn = m.conn;
  t.parent.assign((size_t)E, -1);
  t.first_child.assign((size_t)E, -1);
  t.level.assign((size_t)E, 0);
  t.side_bid = m.side_bid;
  t.origin.resize((size_t)E * 3);
  int64_t e = 0;
  for (int k = 0; k < t.nz; ++k)
    for (int j = 0; j < t.ny; ++j)
      for (int i = 0; i < t.nx; ++i, ++e) {
        t.origin[3 * e + 0] = (int64_t)i * AMR_S0;
        t.origin[3 * e + 1] = (int64_t)j * AMR_S0;
        t.origin[3 * e + 2] = (int64_t)k * AMR_S0;
      }
  t.node_lat.assign((size_t)m.n_nodes() * 3, -1);
  for (e = 0; e < E; ++e)
    for (int a = 0; a < m.npe; ++a) {
      int o[3];
      node_offset(m.npe, a, o);
      const int32_t nd = t.conn[(size_t)(e * m.npe + a)];
      for (int d = 0; d < 3; ++d) t.node_lat[3 * (size_t)nd + d] = t.origin[3 * e + d] + o[d] * (AMR_S0 / 2);
    }
  t.active.resize((size_t)E);
  for (e = 0; e < E; ++e) t.active[(size_t)e] = (int32_t)e;
  t.on = true;
  return "";
}

// Node ids in first-touch order over every element in id order; HostMesh then
// holds the active elements.
void finish(HostMesh &m) {
  AmrTree &t = m.amr;
  const int64_t N = m.n_nodes();
  std::vector<int32_t> newid((size_t)N, -1);
  int32_t next = 0;
  for (int32_t &c : t.conn) {
    int32_t &slot = newid[(size_t)c];
    if (slot < 0) slot = next++;
  }
  for (int64_t n = 0; n < N; ++n)
    if (newid[(size_t)n] < 0) newid[(size_t)n] = next++;
  std::vector<double> xyz((size_t)N * 3);
  std::vector<int64_t> lat((size_t)N * 3);
  for (int64_t n = 0; n < N; ++n)
    for (int d = 0; d < 3; ++d) {
      xyz[3 * (size_t)newid[(size_t)n] + d] = m.xyz[3 * (size_t)n + d];
      lat[3 * (size_t)newid[(size_t)n] + d] = t.node_lat[3 * (size_t)n + d];
    }
  m.xyz.swap(xyz);
  t.node_lat.swap(lat);
  for (int32_t &c : t.conn) c = newid[(size_t)c];
  t.active.clear();
  for (int64_t e = 0; e < t.n_all(); ++e)
    if (t.first_child[(size_t)e] < 0) t.active.push_back((int32_t)e);
  const int npe = m.npe;
  m.conn.resize(t.active.size() * (size_t)npe);
  m.side_bid.resize(t.active.size() * 6);
  for (size_t a = 0; a < t.active.size(); ++a) {
    const int32_t e = t.active[a];
    std::copy(&t.conn[(size_t)e * npe], &t.conn[(size_t)e * npe] + npe, &m.conn[a * npe]);
    std::copy(&t.side_bid[(size_t)e * 6], &t.side_bid[(size_t)e * 6] + 6, &m.side_bid[a * 6]);
  }
}

void refine_elem(HostMesh &m, int32_t e, LatMap &nodes) {
  AmrTree &t = m.amr;
  const int npe = m.npe, order = (npe == 27) ? 2 : 1;
  const int64_t S = elem_size(t, e), Sc = S / 2;
  const int32_t first = (int32_t)t.n_all();
  t.first_child[(size_t)e] = first;
  double X[27][3];
  for (int n = 0; n < npe; ++n)
    for (int d = 0; d < 3; ++d) X[n][d] = m.xyz[3 * (size_t)t.conn[(size_t)e * npe + n] + d];
  for (int c = 0; c < 8; ++c) {
    int64_t oc[3];
    for (int d = 0; d < 3; ++d) oc[d] = t.origin[3 * (size_t)e + d] + HEX_VBITS[c][d] * Sc;
    t.parent.push_back(e);
    t.first_child.push_back(-1);
    t.level.push_back((int8_t)(t.level[(size_t)e] + 1));
    for (int d = 0; d < 3; ++d) t.origin.push_back(oc[d]);
    for (int s = 0; s < 6; ++s) t.side_bid.push_back(child_on_side(c, s) ? t.side_bid[(size_t)e * 6 + s] : -1);
    for (int a = 0; a < npe; ++a) {
      int o[3];
      node_offset(npe, a, o);
      LatKey k{oc[0] + o[0] * (Sc / 2), oc[1] + o[1] * (Sc / 2), oc[2] + o[2] * (Sc / 2)};
      int32_t id = nodes.find(k);
      if (id < 0) {
        // embedding weights: tensor product of 1-D shapes at the child node's
        // parent-reference coordinates, summed over parent nodes in order
        const int64_t L[3] = {k.x, k.y, k.z};
        double xi[3];
        for (int d = 0; d < 3; ++d)
          xi[d] = -1. + 2. * (double)(L[d] - t.origin[3 * (size_t)e + d]) / (double)S;
        double p[3] = {0., 0., 0.};
        for (int n = 0; n < npe; ++n) {
          int on[3];
          node_offset(npe, n, on);
          double w = 1.;
          for (int d = 0; d < 3; ++d)
            w *= (order == 2) ? shape1d(2, quad_index(on[d]), xi[d]) : shape1d(1, on[d] / 2, xi[d]);
          if (w != 0.)
            for (int d = 0; d < 3; ++d) p[d] += w * X[n][d];
        }
        id = (int32_t)m.n_nodes();
        for (int d = 0; d < 3; ++d) m.xyz.push_back(p[d]);
        t.node_lat.push_back(k.x);
        t.node_lat.push_back(k.y);
        t.node_lat.push_back(k.z);
        nodes.insert(k, id);
      }
      t.conn.push_back(id);
    }
  }
}

}  // namespace

std::string amr_refine(HostMesh &m, int cycles, double fraction, uint64_t seed) {
  if (cycles < 0 || !(fraction >= 0.0 && fraction <= 1.0)) return "refine: bad cycles or fraction";
  if (!m.amr.on) {
    std::string err = init_tree(m);
    if (!err.empty()) return err;
  }
  AmrTree &t = m.amr;
  SplitMix64 rng(seed);
  for (int cyc = 0; cyc < cycles; ++cyc) {
    const std::vector<int32_t> act = t.active;
    const int64_t n_act = (int64_t)act.size();
    const int64_t n_flag = (int64_t)std::floor(fraction * (double)n_act);
    std::vector<uint8_t> flag((size_t)t.n_all(), 0);
    std::vector<int32_t> perm = act;
    for (int64_t i = 0; i < n_flag; ++i) {  // partial Fisher-Yates draw without replacement
      const int64_t j = i + (int64_t)(rng.next() % (uint64_t)(n_act - i));
      std::swap(perm[(size_t)i], perm[(size_t)j]);
      flag[(size_t)perm[(size_t)i]] = 1;
    }
    // level-one rule: a flagged element's coarser face neighbors are refined too
    for (bool changed = true; changed;) {
      changed = false;
      for (int32_t e : act) {
        if (!flag[(size_t)e]) continue;
        for (int s = 0; s < 6; ++s) {
          const int32_t nb = across(t, e, s);
          if (nb >= 0 && t.level[(size_t)nb] < t.level[(size_t)e] && !flag[(size_t)nb]) {
            flag[(size_t)nb] = 1;
            changed = true;
          }
        }
      }
    }
    for (int32_t e : act)
      if (flag[(size_t)e] && t.level[(size_t)e] >= AMR_MAX_LEVEL) return "refine: maximum level reached";
    LatMap nodes((size_t)m.n_nodes() * 2);
    for (int64_t n = 0; n < m.n_nodes(); ++n)
      nodes.insert(LatKey{t.node_lat[3 * n], t.node_lat[3 * n + 1], t.node_lat[3 * n + 2]}, (int32_t)n);
    for (int32_t e : act)
      if (flag[(size_t)e]) refine_elem(m, e, nodes);
    finish(m);
  }
  return "";
}

namespace {

// LAGRANGE shapes of the QUAD9 / QUAD4 side (fe_lagrange_shape_2D.C: tensor of
// the 1-D shapes with the node index tables below).
const int QUAD_I0[9] = {0, 1, 1, 0, 2, 1, 2, 0, 2};
const int QUAD_I1[9] = {0, 0, 1, 1, 0, 2, 1, 2, 2};
inline double side_shape(int ns, int j, double xi, double eta) {
  const int order = (ns == 9) ? 2 : 1;
  return shape1d(order, QUAD_I0[j], xi) * shape1d(order, QUAD_I1[j], eta);
}

typedef std::map<int32_t, double> Row;

}  // namespace

// Rows keyed by dof in a dense table: the same ascending order and lookups as
// the reference's std::map<dof_id_type, DofConstraintRow>, without the tree.
struct RowTable {
  std::vector<Row> row;
  std::vector<uint8_t> has;
  explicit RowTable(int64_t n) : row((size_t)n), has((size_t)n, 0) {}
  bool count(int32_t d) const { return d >= 0 && (size_t)d < has.size() && has[(size_t)d]; }
  Row &operator[](int32_t d) {
    has[(size_t)d] = 1;
    return row[(size_t)d];
  }
};

std::string finish_constraint_rows(RowTable &rows, int64_t n_dofs, const uint8_t *dirichlet, ConstraintRows &out);

// The same rows from hanging-node rows formed on the device: dof d's row has
// cnt[d] entries (-1: no row) at col / val[d * width ..], in ascending column
// order.  Dirichlet rows are added for the dofs still free.  process_constraints
// only changes rows that refer to another constrained dof; the sweep below
// visits exactly those (ascending, repeated until none changes) and reads every
// other row from the raw arrays, which gives the same substitutions in the same
// order as a sweep over all rows (an unchanged row leaves the set at its first
// visit without touching any other row).
std::string constraint_rows_from_raw(int64_t n_dofs, const int32_t *cnt, const int32_t *col, const double *val,
                                     int width, const uint8_t *dirichlet, ConstraintRows &out) {
  std::vector<int32_t> len(cnt, cnt + n_dofs);
  if (dirichlet)
    for (int64_t d = 0; d < n_dofs; ++d)
      if (dirichlet[d] && len[(size_t)d] < 0) len[(size_t)d] = 0;
  auto has = [&](int32_t d) { return d >= 0 && d < n_dofs && len[(size_t)d] >= 0; };
  std::map<int32_t, Row> chg;  // rows that refer to constrained dofs
  for (int64_t d = 0; d < n_dofs; ++d)
    for (int k = 0; k < std::max(len[(size_t)d], 0); ++k)
      if (col[d * width + k] != (int32_t)d && has(col[d * width + k])) {
        Row &row = chg[(int32_t)d];
        for (int j = 0; j < len[(size_t)d]; ++j) row.emplace(col[d * width + j], val[d * width + j]);
        break;
      }
  std::set<int32_t> unexpanded;
  for (const auto &r : chg) unexpanded.insert(unexpanded.end(), r.first);
  auto other = [&](int32_t x, std::vector<std::pair<int32_t, double>> &sub) {
    sub.clear();
    auto it = chg.find(x);
    if (it != chg.end()) {
      for (const auto &item : it->second) sub.push_back(item);
    } else {
      for (int j = 0; j < len[(size_t)x]; ++j) sub.emplace_back(col[(int64_t)x * width + j], val[(int64_t)x * width + j]);
    }
  };
  std::vector<std::pair<int32_t, double>> sub;
  while (!unexpanded.empty())
    for (auto i = unexpanded.begin(); i != unexpanded.end();) {
      auto it = chg.find(*i);
      if (it == chg.end()) {  // a row that never changes
        i = unexpanded.erase(i);
        continue;
      }
      Row &row = it->second;
      std::vector<int32_t> expand;
      for (const auto &item : row)
        if (item.first != *i && has(item.first)) {
          unexpanded.insert(item.first);
          expand.push_back(item.first);
        }
      for (int32_t x : expand) {
        const double coef = row[x];
        other(x, sub);
        for (const auto &e : sub) row[e.first] += e.second * coef;
        row.erase(x);
      }
      if (expand.empty()) i = unexpanded.erase(i);
      else ++i;
    }
  out.dofs.clear();
  out.ptr.assign(1, 0);
  out.col.clear();
  out.val.clear();
  for (int64_t d = 0; d < n_dofs; ++d) {
    if (len[(size_t)d] < 0) continue;
    out.dofs.push_back((int32_t)d);
    auto it = chg.find((int32_t)d);
    if (it != chg.end()) {
      for (const auto &item : it->second) {
        out.col.push_back(item.first);
        out.val.push_back(item.second);
      }
    } else {
      for (int j = 0; j < len[(size_t)d]; ++j) {
        out.col.push_back(col[d * width + j]);
        out.val.push_back(val[d * width + j]);
      }
    }
    out.ptr.push_back((int64_t)out.col.size());
  }
  return "";
}

std::string amr_constraint_rows(const HostMesh &m, int n_vars, const int32_t *elem_dofs, int64_t n_dofs,
                                const uint8_t *dirichlet, ConstraintRows &out) {
  RowTable rows(n_dofs);
  const int npe = m.npe, nl = npe * n_vars;
  const int64_t E = m.n_elem();
  if (m.amr.on) {
    const AmrTree &t = m.amr;
    // dof of (node, variable) from the active elements' dof lists
    std::vector<int32_t> node_dof((size_t)m.n_nodes() * n_vars, -1);
    for (int64_t a = 0; a < E; ++a)
      for (int v = 0; v < n_vars; ++v)
        for (int k = 0; k < npe; ++k)
          node_dof[(size_t)m.conn[(size_t)(a * npe + k)] * n_vars + v] = elem_dofs[a * nl + v * npe + k];
    for (int v = 0; v < n_vars; ++v)
      for (int64_t a = 0; a < E; ++a) {
        const int32_t e = t.active[(size_t)a];
        const int32_t P = t.parent[(size_t)e];
        if (P < 0) continue;
        const int c = e - t.first_child[(size_t)P];
        for (int s = 0; s < 6; ++s) {
          if (!child_on_side(c, s)) continue;  // faces inside the parent meet siblings
          const int32_t nb = across(t, e, s);
          if (nb < 0 || t.level[(size_t)nb] >= t.level[(size_t)e]) continue;
          int sn[9];
          const int ns = side_nodes(m.elem_type, s, sn);
          int32_t pn[9], pd[9];
          for (int j = 0; j < ns; ++j) {
            pn[j] = t.conn[(size_t)P * npe + sn[j]];
            pd[j] = node_dof[(size_t)pn[j] * n_vars + v];
          }
          // parent side frame: node 0 at (-1,-1), node 1 at (1,-1), node 3 at (-1,1)
          const int64_t *L0 = &t.node_lat[3 * (size_t)pn[0]], *L1 = &t.node_lat[3 * (size_t)pn[1]],
                        *L3 = &t.node_lat[3 * (size_t)pn[3]];
          int64_t u[3], w[3], uu = 0, ww = 0;
          for (int d = 0; d < 3; ++d) {
            u[d] = L1[d] - L0[d];
            w[d] = L3[d] - L0[d];
            uu += u[d] * u[d];
            ww += w[d] * w[d];
          }
          for (int k = 0; k < ns; ++k) {
            const int32_t my_node = t.conn[(size_t)e * npe + sn[k]];
            const int32_t my_dof = node_dof[(size_t)my_node * n_vars + v];
            bool self = false;
            for (int j = 0; j < ns; ++j) self |= (pd[j] == my_dof);
            if (self || rows.count(my_dof)) continue;
            if (my_dof < 0 || my_dof >= n_dofs) return "constraints: dof out of range";
            const int64_t *Lp = &t.node_lat[3 * (size_t)my_node];
            int64_t pu = 0, pw = 0;
            for (int d = 0; d < 3; ++d) {
              pu += (Lp[d] - L0[d]) * u[d];
              pw += (Lp[d] - L0[d]) * w[d];
            }
            const double xi = -1. + 2. * (double)pu / (double)uu, eta = -1. + 2. * (double)pw / (double)ww;
            Row &row = rows[my_dof];
            for (int j = 0; j < ns; ++j) {
              const double val = side_shape(ns, j, xi, eta);
              if (std::abs(val) > 1.e-5 && std::abs(val) < .999) row.emplace(pd[j], val);
            }
          }
        }
      }
  }
  return finish_constraint_rows(rows, n_dofs, dirichlet, out);
}

// Dirichlet rows for the dofs still free, process_constraints, and the
// output in ascending dof order.
std::string finish_constraint_rows(RowTable &rows, int64_t n_dofs, const uint8_t *dirichlet, ConstraintRows &out) {
  if (dirichlet)
    for (int64_t d = 0; d < n_dofs; ++d)
      if (dirichlet[d] && !rows.count((int32_t)d)) rows[(int32_t)d];
  // process_constraints: substitute constrained dofs inside rows until every
  // row refers to free dofs only (sweeps over the ascending set of unexpanded rows)
  std::set<int32_t> unexpanded;
  for (int64_t d = 0; d < n_dofs; ++d)
    if (rows.has[(size_t)d]) unexpanded.insert(unexpanded.end(), (int32_t)d);
  while (!unexpanded.empty())
    for (auto i = unexpanded.begin(); i != unexpanded.end();) {
      Row &row = rows[*i];
      std::vector<int32_t> expand;
      for (const auto &item : row)
        if (item.first != *i && rows.count(item.first)) {
          unexpanded.insert(item.first);
          expand.push_back(item.first);
        }
      for (int32_t x : expand) {
        const double coef = row[x];
        for (const auto &sub : rows[x]) row[sub.first] += sub.second * coef;
        row.erase(x);
      }
      if (expand.empty()) i = unexpanded.erase(i);
      else ++i;
    }
  out.dofs.clear();
  out.ptr.assign(1, 0);
  out.col.clear();
  out.val.clear();
  for (int64_t d = 0; d < n_dofs; ++d) {
    if (!rows.has[(size_t)d]) continue;
    out.dofs.push_back((int32_t)d);
    for (const auto &item : rows.row[(size_t)d]) {
      out.col.push_back(item.first);
      out.val.push_back(item.second);
    }
    out.ptr.push_back((int64_t)out.col.size());
  }
  return "";
}

}  // namespace lmg

extern "C" {

lmg_status lmg_mesh_refine(lmg_mesh *mesh, int32_t cycles, double fraction, uint64_t seed) {
  if (!mesh) return LMG_ERR_ARG;
  mesh->rows_valid = false;
  try {
    const std::string err = lmg::amr_refine(mesh->m, cycles, fraction, seed);
    return err.empty() ? LMG_OK : LMG_ERR_ARG;
  } catch (const std::bad_alloc &) {
    return LMG_ERR_OOM;
  }
}

lmg_status lmg_mesh_tree(const lmg_mesh *mesh, int64_t *n_all, int32_t *all_conn, int32_t *parent,
                         int8_t *level, int32_t *active_ids) {
  if (!mesh || !n_all) return LMG_ERR_ARG;
  const lmg::HostMesh &m = mesh->m;
  if (!m.amr.on) {  // an unrefined mesh is its own level 0
    *n_all = m.n_elem();
    if (all_conn) std::copy(m.conn.begin(), m.conn.end(), all_conn);
    for (int64_t e = 0; e < m.n_elem(); ++e) {
      if (parent) parent[e] = -1;
      if (level) level[e] = 0;
      if (active_ids) active_ids[e] = (int32_t)e;
    }
    return LMG_OK;
  }
  const lmg::AmrTree &t = m.amr;
  *n_all = t.n_all();
  if (all_conn) std::copy(t.conn.begin(), t.conn.end(), all_conn);
  if (parent) std::copy(t.parent.begin(), t.parent.end(), parent);
  if (level) std::copy(t.level.begin(), t.level.end(), level);
  if (active_ids) std::copy(t.active.begin(), t.active.end(), active_ids);
  return LMG_OK;
}

}  // extern "C"

namespace {

// lmg_constraint_rows with the hanging-node rows formed on the host
// (device < 0) or on the given device.
lmg_status constraint_rows(const lmg_mesh *mesh, int32_t device, int32_t n_vars, const int32_t *elem_dofs,
                           int64_t n_dofs, const uint8_t *dirichlet, uint8_t *constrained, int64_t *cons_ptr,
                           int32_t *cons_col, double *cons_val, int64_t cap) {
  if (!mesh || n_vars <= 0 || !elem_dofs || n_dofs <= 0 || !cons_ptr) return LMG_ERR_ARG;
  try {
    // The count call and the fill call of a caller see the same inputs: keep
    // the rows of the last call, keyed by a checksum of the inputs.
    uint64_t key = 1469598103934665603ull;
    auto mix = [&](uint64_t x) { key = (key ^ x) * 1099511628211ull; };
    mix((uint64_t)n_vars);
    mix((uint64_t)n_dofs);
    mix((uint64_t)(int64_t)device);
    const int64_t nl = (int64_t)mesh->m.npe * n_vars;
    for (int64_t i = 0; i < mesh->m.n_elem() * nl; ++i) mix((uint64_t)(uint32_t)elem_dofs[i]);
    for (int64_t d = 0; d < n_dofs; ++d) mix(dirichlet ? dirichlet[d] : 0);
    lmg_mesh *mm = const_cast<lmg_mesh *>(mesh);
    if (!mm->rows_valid || mm->rows_key != key) {
      mm->rows_valid = false;
      std::string err;
      if (device < 0) {
        err = lmg::amr_constraint_rows(mesh->m, n_vars, elem_dofs, n_dofs, dirichlet, mm->rows);
      } else {
        std::vector<int32_t> cnt, col;
        std::vector<double> val;
        err = lmg::amr_raw_rows_device(mesh->m, device, n_vars, elem_dofs, n_dofs, cnt, col, val);
        if (err.rfind("device rows", 0) == 0) return LMG_ERR_CUDA;
        if (err.empty())
          err = lmg::constraint_rows_from_raw(n_dofs, cnt.data(), col.data(), val.data(), lmg::AMR_ROW_WIDTH,
                                              dirichlet, mm->rows);
      }
      if (!err.empty()) return LMG_ERR_BOUNDS;
      mm->rows_key = key;
      mm->rows_valid = true;
    }
    const lmg::ConstraintRows &r = mm->rows;
    std::vector<int64_t> len((size_t)n_dofs, 0);
    for (size_t i = 0; i < r.dofs.size(); ++i) len[(size_t)r.dofs[i]] = r.ptr[i + 1] - r.ptr[i];
    cons_ptr[0] = 0;
    for (int64_t d = 0; d < n_dofs; ++d) cons_ptr[d + 1] = cons_ptr[d] + len[(size_t)d];
    if (constrained) {
      std::fill(constrained, constrained + n_dofs, (uint8_t)0);
      for (int32_t d : r.dofs) constrained[d] = 1;
    }
    if (cons_col && cons_val) {
      if (cap < (int64_t)r.col.size()) return LMG_ERR_ARG;
      for (size_t i = 0; i < r.dofs.size(); ++i) {
        const int64_t o = cons_ptr[r.dofs[i]];
        for (int64_t k = r.ptr[i]; k < r.ptr[i + 1]; ++k) {
          cons_col[o + k - r.ptr[i]] = r.col[(size_t)k];
          cons_val[o + k - r.ptr[i]] = r.val[(size_t)k];
        }
      }
    }
    return LMG_OK;
  } catch (const std::bad_alloc &) {
    return LMG_ERR_OOM;
  }
}

}  // namespace

extern "C" {

lmg_status lmg_constraint_rows(const lmg_mesh *mesh, int32_t n_vars, const int32_t *elem_dofs, int64_t n_dofs,
                               const uint8_t *dirichlet, uint8_t *constrained, int64_t *cons_ptr,
                               int32_t *cons_col, double *cons_val, int64_t cap) {
  return constraint_rows(mesh, -1, n_vars, elem_dofs, n_dofs, dirichlet, constrained, cons_ptr, cons_col, cons_val,
                         cap);
}

lmg_status lmg_constraint_rows_device(const lmg_mesh *mesh, int32_t device, int32_t n_vars,
                                      const int32_t *elem_dofs, int64_t n_dofs, const uint8_t *dirichlet,
                                      uint8_t *constrained, int64_t *cons_ptr, int32_t *cons_col, double *cons_val,
                                      int64_t cap) {
  if (device < 0) return LMG_ERR_ARG;
  return constraint_rows(mesh, device, n_vars, elem_dofs, n_dofs, dirichlet, constrained, cons_ptr, cons_col,
                         cons_val, cap);
}

}  // extern "C"
