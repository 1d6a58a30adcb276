// CPU oracle: constraint rows and constrained sparsity.
//
// TEST INFRASTRUCTURE ONLY (see oracle.cpp).  Restates, from libMesh:
//   lagrange_compute_constraints      src/fe/fe_lagrange.C:867-1063
//   FEMap::inverse_map (dim 2)        src/fe/fe_map.C:1512-1700
//   LAGRANGE QUAD4/QUAD9 shapes       src/fe/fe_lagrange_shape_2D.C (tensor of 1-D shapes)
//   AddPrimalConstraint               src/base/dof_map_constraints.C:216-228
//   DofMap::process_constraints       src/base/dof_map_constraints.C:4341-4490
//   DofMap::find_connected_dofs       src/base/dof_map.C:2915-2970
//   SparsityPattern::Build            src/base/sparsity_pattern.C:152-363
// The neighbor across a side is found geometrically (the active element that
// contains a point just outside the side's centroid); libMesh links the same
// element through Elem::neighbor_ptr.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <map>
#include <set>
#include <vector>

namespace {

const int HEX8 = 10, HEX27 = 12;
const int H8_SIDES[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}, {4, 5, 6, 7}};
const int H27_SIDES[6][9] = {{0, 3, 2, 1, 11, 10, 9, 8, 20}, {0, 1, 5, 4, 8, 13, 16, 12, 21},
                             {1, 2, 6, 5, 9, 14, 17, 13, 22}, {2, 3, 7, 6, 10, 15, 18, 14, 23},
                             {3, 0, 4, 7, 11, 12, 19, 15, 24}, {4, 5, 6, 7, 16, 17, 18, 19, 25}};

// include/fe/fe_lagrange_shape_1D.h
double lag1(int order, int i, double x) {
  if (order == 1) return i == 0 ? .5 * (1. - x) : .5 * (1. + x);
  switch (i) {
    case 0: return .5 * x * (x - 1.);
    case 1: return .5 * x * (x + 1.);
    default: return (1. - x) * (1. + x);
  }
}
double lag1d(int order, int i, double x) {
  if (order == 1) return i == 0 ? -.5 : .5;
  switch (i) {
    case 0: return x - .5;
    case 1: return x + .5;
    default: return -2. * x;
  }
}
// fe_lagrange_shape_2D.C, QUAD4 / QUAD9 index tables
const int Q_I0[9] = {0, 1, 1, 0, 2, 1, 2, 0, 2};
const int Q_I1[9] = {0, 0, 1, 1, 0, 2, 1, 2, 2};
double quad_shape(int ns, int i, double xi, double eta) {
  const int o = ns == 9 ? 2 : 1;
  return lag1(o, Q_I0[i], xi) * lag1(o, Q_I1[i], eta);
}
double quad_deriv(int ns, int i, int j, double xi, double eta) {
  const int o = ns == 9 ? 2 : 1;
  return j == 0 ? lag1d(o, Q_I0[i], xi) * lag1(o, Q_I1[i], eta) : lag1(o, Q_I0[i], xi) * lag1d(o, Q_I1[i], eta);
}

struct P3 {
  double v[3];
};
double dot3(const P3 &a, const P3 &b) { return a.v[0] * b.v[0] + a.v[1] * b.v[1] + a.v[2] * b.v[2]; }

// FEMap::inverse_map for a 2-D side element in 3-D space (tolerance TOLERANCE = 1e-6).
void inverse_map_2d(int ns, const std::vector<P3> &X, const P3 &phys, double &xi, double &eta) {
  double p[2] = {0., 0.};
  double err = 0.;
  int cnt = 0;
  do {
    P3 guess = {{0, 0, 0}}, dxi = {{0, 0, 0}}, deta = {{0, 0, 0}};
    for (int i = 0; i < ns; ++i) {
      const double s = quad_shape(ns, i, p[0], p[1]);
      const double d0 = quad_deriv(ns, i, 0, p[0], p[1]), d1 = quad_deriv(ns, i, 1, p[0], p[1]);
      for (int c = 0; c < 3; ++c) {
        guess.v[c] += X[i].v[c] * s;
        dxi.v[c] += X[i].v[c] * d0;
        deta.v[c] += X[i].v[c] * d1;
      }
    }
    P3 delta;
    for (int c = 0; c < 3; ++c) delta.v[c] = phys.v[c] - guess.v[c];
    const double G11 = dot3(dxi, dxi), G12 = dot3(dxi, deta), G21 = dot3(dxi, deta), G22 = dot3(deta, deta);
    const double det = (G11 * G22 - G12 * G21);
    const double inv_det = 1. / det;
    const double Ginv11 = G22 * inv_det, Ginv12 = -G12 * inv_det, Ginv21 = -G21 * inv_det, Ginv22 = G11 * inv_det;
    const double dxidelta = dot3(dxi, delta), detadelta = dot3(deta, delta);
    const double dp0 = (Ginv11 * dxidelta + Ginv12 * detadelta);
    const double dp1 = (Ginv21 * dxidelta + Ginv22 * detadelta);
    err = std::sqrt(dp0 * dp0 + dp1 * dp1);
    p[0] += dp0;
    p[1] += dp1;
    cnt++;
  } while (err > 1e-6 && cnt <= 20);
  xi = p[0];
  eta = p[1];
}

typedef std::map<int32_t, double> Row;

}  // namespace

extern "C" {

// Constraint rows of a refined hex mesh.
//   tree: all_conn [n_all][npe], parent [n_all], level [n_all]; active_ids [n_active];
//   elem_dofs [n_active][n_vars*npe] (dof_indices of the active elements).
// Output as CSR over all dofs (see lmg_constraint_rows); returns the number of
// entries, or -1 if cap is too small.
int64_t orc_constraint_rows(int elem_type, int64_t n_nodes, const double *xyz, int64_t n_all,
                            const int32_t *all_conn, const int32_t *parent, const int8_t *level,
                            int64_t n_active, const int32_t *active_ids, int n_vars, const int32_t *elem_dofs,
                            int64_t n_dofs, const uint8_t *dirichlet, uint8_t *constrained, int64_t *cons_ptr,
                            int32_t *cons_col, double *cons_val, int64_t cap) {
  const int npe = elem_type == HEX27 ? 27 : 8, ns = elem_type == HEX27 ? 9 : 4, nl = npe * n_vars;
  (void)n_nodes;
  (void)n_all;
  // bounding boxes of the active elements for point location
  std::vector<double> box((size_t)n_active * 6);
  for (int64_t a = 0; a < n_active; ++a) {
    const int32_t *c = all_conn + (int64_t)active_ids[a] * npe;
    for (int d = 0; d < 3; ++d) {
      double lo = 1e300, hi = -1e300;
      for (int k = 0; k < 8; ++k) {
        lo = std::min(lo, xyz[3 * (int64_t)c[k] + d]);
        hi = std::max(hi, xyz[3 * (int64_t)c[k] + d]);
      }
      box[6 * a + d] = lo;
      box[6 * a + 3 + d] = hi;
    }
  }
  // bucket grid over the domain
  double glo[3] = {1e300, 1e300, 1e300}, ghi[3] = {-1e300, -1e300, -1e300};
  for (int64_t a = 0; a < n_active; ++a)
    for (int d = 0; d < 3; ++d) {
      glo[d] = std::min(glo[d], box[6 * a + d]);
      ghi[d] = std::max(ghi[d], box[6 * a + 3 + d]);
    }
  const int G = std::max(1, (int)std::cbrt((double)n_active / 2.0));
  auto cell = [&](double x, int d) {
    int i = (int)((x - glo[d]) / (ghi[d] - glo[d]) * G);
    return std::min(G - 1, std::max(0, i));
  };
  std::vector<std::vector<int32_t>> bucket((size_t)G * G * G);
  for (int64_t a = 0; a < n_active; ++a) {
    int lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
      lo[d] = cell(box[6 * a + d], d);
      hi[d] = cell(box[6 * a + 3 + d], d);
    }
    for (int k = lo[2]; k <= hi[2]; ++k)
      for (int j = lo[1]; j <= hi[1]; ++j)
        for (int i = lo[0]; i <= hi[0]; ++i) bucket[(size_t)(i + G * (j + G * k))].push_back((int32_t)a);
  }
  auto find_active = [&](const P3 &p) -> int64_t {
    for (int d = 0; d < 3; ++d)
      if (p.v[d] < glo[d] || p.v[d] > ghi[d]) return -1;
    const auto &b = bucket[(size_t)(cell(p.v[0], 0) + G * (cell(p.v[1], 1) + G * cell(p.v[2], 2)))];
    for (int32_t a : b) {
      bool in = true;
      for (int d = 0; d < 3; ++d) in = in && p.v[d] > box[6 * a + d] && p.v[d] < box[6 * a + 3 + d];
      if (in) return a;
    }
    return -1;
  };
  auto side_list = [&](int s, int k) { return elem_type == HEX27 ? H27_SIDES[s][k] : H8_SIDES[s][k]; };
  // dof of (node, variable)
  std::map<int64_t, int32_t> node_dof;
  for (int64_t a = 0; a < n_active; ++a)
    for (int v = 0; v < n_vars; ++v)
      for (int k = 0; k < npe; ++k)
        node_dof[(int64_t)all_conn[(int64_t)active_ids[a] * npe + k] * n_vars + v] = elem_dofs[a * nl + v * npe + k];
  std::map<int32_t, Row> constraints;
  for (int v = 0; v < n_vars; ++v)
    for (int64_t a = 0; a < n_active; ++a) {
      const int32_t e = active_ids[a];
      const int32_t *ce = all_conn + (int64_t)e * npe;
      for (int s = 0; s < 6; ++s) {
        // outward point just past the side centroid
        P3 cen = {{0, 0, 0}}, ecen = {{0, 0, 0}};
        for (int k = 0; k < 4; ++k)
          for (int d = 0; d < 3; ++d) cen.v[d] += 0.25 * xyz[3 * (int64_t)ce[side_list(s, k)] + d];
        for (int k = 0; k < 8; ++k)
          for (int d = 0; d < 3; ++d) ecen.v[d] += 0.125 * xyz[3 * (int64_t)ce[k] + d];
        P3 q;
        for (int d = 0; d < 3; ++d) q.v[d] = cen.v[d] + 1e-3 * (cen.v[d] - ecen.v[d]);
        const int64_t nb = find_active(q);
        if (nb < 0) continue;
        const int32_t ne = active_ids[nb];
        if (!(level[ne] < level[e])) continue;
        const int32_t P = parent[e];
        const int32_t *cp = all_conn + (int64_t)P * npe;
        std::vector<int32_t> my_dofs(ns), parent_dofs(ns);
        std::vector<P3> Xp(ns);
        for (int k = 0; k < ns; ++k) {
          my_dofs[k] = node_dof[(int64_t)ce[side_list(s, k)] * n_vars + v];
          parent_dofs[k] = node_dof[(int64_t)cp[side_list(s, k)] * n_vars + v];
          for (int d = 0; d < 3; ++d) Xp[k].v[d] = xyz[3 * (int64_t)cp[side_list(s, k)] + d];
        }
        for (int my = 0; my != ns; my++) {
          const int32_t my_dof_g = my_dofs[my];
          bool self_constraint = false;
          for (int their = 0; their != ns; their++)
            if (parent_dofs[their] == my_dof_g) {
              self_constraint = true;
              break;
            }
          if (self_constraint) continue;
          if (constraints.count(my_dof_g)) continue;
          Row &constraint_row = constraints[my_dof_g];
          P3 support;
          for (int d = 0; d < 3; ++d) support.v[d] = xyz[3 * (int64_t)ce[side_list(s, my)] + d];
          double xi, eta;
          inverse_map_2d(ns, Xp, support, xi, eta);
          for (int their = 0; their != ns; their++) {
            const double val = quad_shape(ns, their, xi, eta);
            if ((std::abs(val) > 1.e-5) && (std::abs(val) < .999)) constraint_row.emplace(parent_dofs[their], val);
          }
        }
      }
    }
  // ConstrainDirichlet through AddPrimalConstraint: only dofs still free
  if (dirichlet)
    for (int64_t d = 0; d < n_dofs; ++d)
      if (dirichlet[d] && !constraints.count((int32_t)d)) constraints[(int32_t)d];
  // process_constraints
  std::set<int32_t> unexpanded_set;
  for (const auto &i : constraints) unexpanded_set.insert(i.first);
  while (!unexpanded_set.empty())
    for (auto i = unexpanded_set.begin(); i != unexpanded_set.end();) {
      Row &constraint_row = constraints[*i];
      std::vector<int32_t> constraints_to_expand;
      for (const auto &item : constraint_row)
        if (item.first != *i && constraints.count(item.first)) {
          unexpanded_set.insert(item.first);
          constraints_to_expand.push_back(item.first);
        }
      for (const auto &expandable : constraints_to_expand) {
        const double this_coef = constraint_row[expandable];
        const Row &subconstraint_row = constraints[expandable];
        for (const auto &item : subconstraint_row) constraint_row[item.first] += item.second * this_coef;
        constraint_row.erase(expandable);
      }
      if (constraints_to_expand.empty()) i = unexpanded_set.erase(i);
      else ++i;
    }
  int64_t total = 0;
  for (const auto &r : constraints) total += (int64_t)r.second.size();
  if (cons_col && cap < total) return -1;
  std::fill(constrained, constrained + n_dofs, (uint8_t)0);
  int64_t o = 0;
  auto it = constraints.begin();
  for (int64_t d = 0; d < n_dofs; ++d) {
    cons_ptr[d] = o;
    if (it != constraints.end() && it->first == d) {
      constrained[d] = 1;
      for (const auto &item : it->second) {
        if (cons_col) {
          cons_col[o] = item.first;
          cons_val[o] = item.second;
        }
        ++o;
      }
      ++it;
    }
  }
  cons_ptr[n_dofs] = o;
  return total;
}

// DofMap::compute_sparsity with find_connected_dofs.  Call with row_ptr/col NULL for nnz.
int orc_sparsity_constrained(int64_t n_dofs, int64_t n_elem, int nl, const int32_t *elem_dofs,
                             const int64_t *cons_ptr, const int32_t *cons_col, int64_t *nnz, int32_t *row_ptr,
                             int32_t *col) {
  std::vector<std::vector<int32_t>> rows(n_dofs);
  for (int64_t e = 0; e < n_elem; ++e) {
    std::vector<int32_t> elem_dofs_e(elem_dofs + e * nl, elem_dofs + (e + 1) * nl);
    // find_connected_dofs, recursive form
    for (;;) {
      std::set<int32_t> dof_set(elem_dofs_e.begin(), elem_dofs_e.end());
      bool done = true;
      for (const auto &dof : elem_dofs_e)
        for (int64_t k = cons_ptr[dof]; k < cons_ptr[dof + 1]; ++k)
          if (!dof_set.count(cons_col[k])) {
            dof_set.insert(cons_col[k]);
            done = false;
          }
      elem_dofs_e.assign(dof_set.begin(), dof_set.end());  // sorted_connected_dofs
      if (done) break;
    }
    for (int32_t r : elem_dofs_e) {
      std::vector<int32_t> out;
      std::set_union(rows[r].begin(), rows[r].end(), elem_dofs_e.begin(), elem_dofs_e.end(),
                     std::back_inserter(out));
      rows[r].swap(out);
    }
  }
  int64_t total = 0;
  for (auto &r : rows) total += (int64_t)r.size();
  *nnz = total;
  if (row_ptr && col) {
    int64_t o = 0;
    for (int64_t r = 0; r < n_dofs; ++r) {
      row_ptr[r] = (int32_t)o;
      for (int32_t c : rows[r]) col[o++] = c;
    }
    row_ptr[n_dofs] = (int32_t)o;
  }
  return 0;
}

}  // extern "C"
