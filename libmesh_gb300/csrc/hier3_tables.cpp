// Tables of the cubic HIERARCHIC hex (FEType{THIRD, HIERARCHIC} on HEX27).
//
// libMesh evaluates shape i of an element as
//   phi_i(xi) = h(i0, c0) * h(i1, c1) * h(i2, c2),  c_s = +-xi_{src(s)}
// where cube_indices (src/fe/fe_hierarchic_shape_3D.C:166-760) picks the 1-D
// indices (i0, i1, i2) and, from the element's edge and face orientation,
// which reference coordinate feeds each slot and with which sign; the
// derivatives are central differences with eps = 1e-6 (fe_fdm_deriv,
// src/fe/fe.C:794-811, 929-944).  Every element thus uses shapes drawn from
// a small set of "variants" (i0, i1, i2, slot sources, slot signs).  The
// host finds each element's 64 variants, tabulates every variant that occurs
// -- evaluated in the same order, so the difference quotients are the
// reference's bit for bit -- and the affine reference tensors over variant
// pairs,
//   D_k[v][w] = sum_q w_q dphi_v^m(q) dphi_w^n(q)   (k = the six m <= n pairs,
//                                                     off-diagonal pairs summed)
//   M[v][g]   = sum_q w_q phi_v(q) phi^geo_g(q)     (load through the HEX27 map basis)
// so that the device forms K_ij = sum_k A_k D_k[var_i][var_j] per element.
#include <algorithm>
#include <cmath>
#include <map>
#include <unordered_map>

#include "lmg_internal.h"

namespace lmg {

namespace {

bool pt_less(const double *a, const double *b) {  // TypeVector::operator<
  for (int i = 0; i < 3; i++) {
    if (a[i] < b[i]) return true;
    if (a[i] > b[i]) return false;
  }
  return false;
}
bool pt_eq(const double *a, const double *b) { return a[0] == b[0] && a[1] == b[1] && a[2] == b[2]; }

const int EDGE[12][2] = {{0, 1}, {1, 2}, {2, 3}, {0, 3}, {0, 4}, {1, 5}, {2, 6}, {3, 7}, {4, 5}, {5, 6}, {6, 7}, {4, 7}};
const int SIDE4[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}, {4, 5, 6, 7}};

// Signature of one shape: 1-D indices per slot, source coordinate per slot,
// negation per slot.
struct Sig {
  int idx[3];
  int src[3];
  int neg[3];
  uint32_t key() const {
    uint32_t k = 0;
    for (int s = 0; s < 3; ++s) k |= (uint32_t)idx[s] << (2 * s) | (uint32_t)src[s] << (6 + 2 * s) |
                                     (uint32_t)neg[s] << (12 + s);
    return k;
  }
};

// cube_indices at totalorder e + 1 (e = 1 or 2 dofs per edge) for the element
// with vertex coordinates X[8][3].
Sig cube_sig(const double (*X)[3], int i, int e = 2) {
  Sig g = {{0, 0, 0}, {0, 1, 2}, {0, 0, 0}};
  static const int V[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
  if (i < 8) {
    for (int s = 0; s < 3; ++s) g.idx[s] = V[i][s];
    return g;
  }
  if (i < 8 + 12 * e) {  // e dofs per edge; the edge's own coordinate flips by orientation
    static const int DIR[12] = {0, 1, 0, 1, 2, 2, 2, 2, 0, 1, 0, 1};
    static const int FIX[12][2] = {{0, 0}, {1, 0}, {1, 0}, {0, 0}, {0, 0}, {1, 0},
                                   {1, 1}, {0, 1}, {0, 1}, {1, 1}, {1, 1}, {0, 1}};
    const int ed = (i - 8) / e, k = i - e * ed - 6, d = DIR[ed];
    const bool pos = pt_less(X[EDGE[ed][1]], X[EDGE[ed][0]]);  // Elem::positive_edge_orientation
    const bool flip = (ed == 2 || ed == 10) ? !pos : pos;
    for (int s = 0, f = 0; s < 3; ++s) g.idx[s] = (s == d) ? k : FIX[ed][f++];
    g.neg[d] = flip ? 1 : 0;
    return g;
  }
  if (i < 8 + 12 * e + 6 * e * e) {  // e^2 dofs per face: in-face coordinates swapped / reflected by the face case
    static const int SQ_ROW[4] = {0, 1, 1, 0}, SQ_COL[4] = {0, 0, 1, 1};
    static const int AX[6][2] = {{0, 1}, {0, 2}, {1, 2}, {0, 2}, {1, 2}, {0, 1}};  // slots A, B
    static const int FIXED[6][2] = {{2, 0}, {1, 0}, {0, 1}, {1, 1}, {0, 0}, {2, 1}};  // slot, index
    static const int TESTV[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5}, {3, 7, 6, 2}, {0, 4, 7, 3}, {4, 5, 6, 7}};
    static const int GMP[6][4] = {{1, 2, 0, 3}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}, {4, 5, 6, 7}};
    static const bool NEG[6] = {false, true, true, false, false, true};
    // (A source, A negated, B source, B negated) with 0 = A, 1 = B
    enum { ID, SW, TA, TB, NG, NS, TC, TD };
    static const int MAP[8][4] = {{0, 0, 1, 0}, {1, 0, 0, 0}, {1, 1, 0, 0}, {0, 0, 1, 1},
                                  {0, 1, 1, 1}, {1, 1, 0, 1}, {1, 0, 0, 1}, {0, 1, 1, 0}};
    static const int CASE[6][4][2] = {{{ID, SW}, {TA, TB}, {NG, NS}, {TC, TD}},
                                      {{ID, SW}, {TC, TD}, {NG, NS}, {TD, TB}},
                                      {{ID, SW}, {TC, TD}, {NG, NS}, {TA, TB}},
                                      {{ID, SW}, {TA, TB}, {NG, NS}, {TC, TD}},
                                      {{ID, SW}, {TA, TB}, {NG, NS}, {TC, TD}},
                                      {{ID, SW}, {TC, TD}, {NG, NS}, {TA, ID}}};
    const int f = (i - 8 - 12 * e) / (e * e), b = i - 8 - 12 * e - e * e * f;
    const int sa = AX[f][0], sb = AX[f][1];
    g.idx[sa] = SQ_ROW[b] + 2;
    g.idx[sb] = SQ_COL[b] + 2;
    g.idx[FIXED[f][0]] = FIXED[f][1];
    // get_min_point and positive_face_orientation (elem.C:3642-3661)
    const double *m = X[GMP[f][0]];
    for (int t = 1; t < 4; ++t)
      if (pt_less(X[GMP[f][t]], m)) m = X[GMP[f][t]];
    int v = 0;
    for (int t = 1; t < 4; ++t)
      if (pt_less(X[SIDE4[f][t]], X[SIDE4[f][v]])) v = t;
    const bool pos = pt_less(X[SIDE4[f][(v + 3) % 4]], X[SIDE4[f][(v + 1) % 4]]);
    const bool o = NEG[f] ? !pos : pos;
    for (int t = 0; t < 4; ++t) {
      if (!pt_eq(X[TESTV[f][t]], m)) continue;
      const int *mp = MAP[CASE[f][t][o ? 0 : 1]];
      const int slot[2] = {sa, sb};
      g.src[sa] = slot[mp[0]];
      g.neg[sa] = mp[1];
      g.src[sb] = slot[mp[2]];
      g.neg[sb] = mp[3];
      break;
    }
    return g;
  }
  static const int CB_COL[8] = {0, 0, 1, 1, 0, 1, 1, 0}, CB_ROW[8] = {0, 1, 1, 0, 1, 1, 0, 0},
                   CB_PAGE[8] = {0, 0, 0, 0, 1, 1, 1, 1};
  const int b = i - 8 - 12 * e - 6 * e * e;
  g.idx[0] = CB_COL[b] + 2;
  g.idx[1] = CB_ROW[b] + 2;
  g.idx[2] = CB_PAGE[b] + 2;
  return g;
}

// fe_hierarchic_1D_shape for i <= 3 (src/fe/fe_hierarchic_shape_1D.C:430-498).
double h1(int i, double x) {
  switch (i) {
    case 0: return .5 * (1. - x);
    case 1: return .5 * (1. + x);
    case 2: return (x * x - 1.) / 2.;
    default: return (x * x * x - x) / 6.;
  }
}

double sig_value(const Sig &g, const double *p) {
  double c[3];
  for (int s = 0; s < 3; ++s) c[s] = g.neg[s] ? -p[g.src[s]] : p[g.src[s]];
  return h1(g.idx[0], c[0]) * h1(g.idx[1], c[1]) * h1(g.idx[2], c[2]);
}

}  // namespace

// HIERARCHIC SECOND on HEX27: the per-shape signature of an element (from its
// vertex coordinates X[8][3]) and the evaluation of shape a at p in the
// reference's order (s0 s1) s2 at the remapped coordinates.  The face swaps
// of cube_indices change the rounding of the face shapes and, through the
// central differences, their derivatives; elements of one mesh that share a
// signature share their reference tables.
uint64_t hex27_p2_pattern(const double (*X)[3]) {
  uint64_t k = 0;
  for (int i = 20; i < 26; ++i) {  // only the face shapes' signatures vary at this order
    const Sig g = cube_sig(X, i, 1);
    k = k * 64 + (uint64_t)(g.src[0] * 16 + g.src[1] * 4 + g.src[2]);
  }
  return k;
}

double hex27_p2_shape(const double (*X)[3], int a, const double *p) { return sig_value(cube_sig(X, a, 1), p); }

std::string build_hier3_tables(Hier3Tables &h, int q_order, int64_t n_elem, const double *xyz, const int32_t *conn) {
  h = Hier3Tables();
  FETables geo;
  std::string err = build_fe_tables(geo, LMG_HEX27, 2, q_order, 0);  // QGauss and the HEX27 map basis
  if (!err.empty()) return err;
  h.q = geo.q;
  h.gd0.assign(geo.gdphi.begin(), geo.gdphi.begin() + 27 * 3);
  std::unordered_map<uint32_t, int> id;
  std::vector<Sig> vars;
  h.var.resize((size_t)n_elem * 64);
  double X[8][3];
  for (int64_t e = 0; e < n_elem; ++e) {
    for (int a = 0; a < 8; ++a)
      for (int d = 0; d < 3; ++d) X[a][d] = xyz[3 * (int64_t)conn[e * 27 + a] + d];
    for (int i = 0; i < 64; ++i) {
      const Sig g = cube_sig(X, i);
      auto it = id.find(g.key());
      int v;
      if (it == id.end()) {
        v = (int)vars.size();
        id.emplace(g.key(), v);
        vars.push_back(g);
      } else {
        v = it->second;
      }
      h.var[(size_t)e * 64 + i] = (uint16_t)v;
    }
  }
  const int V = (int)vars.size(), Q = geo.q;
  if (V > 65535) return "too many shape variants";
  h.V = V;
  // variant values and difference-quotient derivatives at the quadrature points
  std::vector<double> phi((size_t)V * Q), dphi((size_t)V * Q * 3);
  const double eps = 1.e-6;
  for (int v = 0; v < V; ++v)
    for (int q = 0; q < Q; ++q) {
      const double *p = &geo.qp[3 * (size_t)q];
      phi[(size_t)v * Q + q] = sig_value(vars[(size_t)v], p);
      for (int j = 0; j < 3; ++j) {
        double pp[3] = {p[0], p[1], p[2]}, pm[3] = {p[0], p[1], p[2]};
        pp[j] += eps;
        pm[j] -= eps;
        dphi[((size_t)v * Q + q) * 3 + j] =
            (sig_value(vars[(size_t)v], pp) - sig_value(vars[(size_t)v], pm)) / 2. / eps;
      }
    }
  const int pm[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
  h.D.assign((size_t)V * V * 6, 0.0);
  for (int v = 0; v < V; ++v)
    for (int w = 0; w < V; ++w) {
      double S[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
      for (int q = 0; q < Q; ++q) {
        const double *a = &dphi[((size_t)v * Q + q) * 3], *b = &dphi[((size_t)w * Q + q) * 3];
        for (int m = 0; m < 3; ++m)
          for (int n = 0; n < 3; ++n) S[m][n] += geo.qw[(size_t)q] * a[m] * b[n];
      }
      double *o = &h.D[((size_t)v * V + w) * 6];
      for (int k = 0; k < 6; ++k) {
        const int m0 = pm[k][0], m1 = pm[k][1];
        o[k] = (m0 == m1) ? S[m0][m0] : S[m0][m1] + S[m1][m0];
      }
    }
  h.M.assign((size_t)V * 27, 0.0);
  for (int v = 0; v < V; ++v)
    for (int g = 0; g < 27; ++g) {
      double s = 0.0;
      for (int q = 0; q < Q; ++q) s += geo.qw[(size_t)q] * phi[(size_t)v * Q + q] * geo.gphi[(size_t)q * 27 + g];
      h.M[(size_t)v * 27 + g] = s;
    }
  // patterns: distinct 64-variant vectors (one on build_cube meshes, where
  // every element has the same orientation)
  std::map<std::vector<uint16_t>, int> pat;
  std::vector<int32_t> pid((size_t)n_elem);
  std::vector<const uint16_t *> first;
  for (int64_t e = 0; e < n_elem; ++e) {
    std::vector<uint16_t> key(h.var.begin() + e * 64, h.var.begin() + (e + 1) * 64);
    auto it = pat.find(key);
    if (it == pat.end()) {
      it = pat.emplace(std::move(key), (int)first.size()).first;
      first.push_back(&h.var[(size_t)e * 64]);
    }
    pid[(size_t)e] = it->second;
  }
  h.P = (int)first.size();
  if ((size_t)h.P * 6 * 4096 * sizeof(double) > ((size_t)2 << 30)) return "too many orientation patterns";
  h.Dp.resize((size_t)h.P * 6 * 4096);
  h.Mp.resize((size_t)h.P * 64 * 27);
  for (int p = 0; p < h.P; ++p) {
    const uint16_t *vr = first[(size_t)p];
    for (int k = 0; k < 6; ++k)
      for (int i = 0; i < 64; ++i)
        for (int j = 0; j < 64; ++j)
          h.Dp[((size_t)p * 6 + k) * 4096 + i * 64 + j] = h.D[((size_t)vr[i] * V + vr[j]) * 6 + k];
    for (int i = 0; i < 64; ++i)
      for (int g = 0; g < 27; ++g) h.Mp[((size_t)p * 64 + i) * 27 + g] = h.M[(size_t)vr[i] * 27 + g];
  }
  h.order.resize((size_t)n_elem);
  for (int64_t e = 0; e < n_elem; ++e) h.order[(size_t)e] = (int32_t)e;
  std::stable_sort(h.order.begin(), h.order.end(), [&](int32_t a, int32_t b) { return pid[(size_t)a] < pid[(size_t)b]; });
  for (int64_t i = 0; i < n_elem;) {
    const int p = pid[(size_t)h.order[(size_t)i]];
    int64_t j = i;
    while (j < n_elem && j - i < 8 && pid[(size_t)h.order[(size_t)j]] == p) ++j;
    h.batch.push_back(p);
    h.batch.push_back((int32_t)i);
    h.batch.push_back((int32_t)(j - i));
    i = j;
  }
  return "";
}

// Cubic HIERARCHIC tets on TET14: a pattern is the element's orientation
// (edge flips and sorted face vertices, tet_orient); per pattern the shapes are
// evaluated at the quadrature points as the reference evaluates them for such
// an element, and tabulated as for the hexahedra: D_k (the affine reference
// tensors S^00, S^11, S^22, S^01+S^10, S^02+S^20, S^12+S^21), M (shape x TET14
// map basis) and the TET14 map derivatives at qp 0.
std::string build_tet3_tables(Hier3Tables &h, int q_order, int64_t n_elem, const double *xyz, const int32_t *conn) {
  h = Hier3Tables();
  h.N = 20;
  h.G = 14;
  FETables geo;
  std::string err = build_fe_tables(geo, LMG_TET14, 1, q_order, 0);  // QGauss and the TET14 map basis
  if (!err.empty()) return err;
  if (geo.n_geo != 14) return "TET14 map basis";
  h.q = geo.q;
  h.gd0.assign(geo.gdphi.begin(), geo.gdphi.begin() + 14 * 3);
  std::unordered_map<uint32_t, int> id;
  std::vector<TetOrient> pats;
  std::vector<int> pid((size_t)n_elem);
  double X[12];
  for (int64_t e = 0; e < n_elem; ++e) {
    for (int a = 0; a < 4; ++a)
      for (int d = 0; d < 3; ++d) X[3 * a + d] = xyz[3 * (int64_t)conn[e * 14 + a] + d];
    const TetOrient o = tet_orient(X);
    auto it = id.find(o.key());
    if (it == id.end()) {
      it = id.emplace(o.key(), (int)pats.size()).first;
      pats.push_back(o);
    }
    pid[(size_t)e] = it->second;
  }
  const int N = 20, G = 14, Q = geo.q;
  h.P = (int)pats.size();
  h.Dp.assign((size_t)h.P * 6 * N * N, 0.0);
  h.Mp.assign((size_t)h.P * N * G, 0.0);
  std::vector<double> v((size_t)Q * N), g((size_t)Q * N * 3);
  for (int p = 0; p < h.P; ++p) {
    for (int q = 0; q < Q; ++q) hier_tet3_shapes(pats[(size_t)p], &geo.qp[3 * q], &v[(size_t)q * N], &g[(size_t)q * N * 3]);
    double *D = &h.Dp[(size_t)p * 6 * N * N];
    double *M = &h.Mp[(size_t)p * N * G];
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) {
        double S[3][3] = {};
        for (int q = 0; q < Q; ++q)
          for (int m = 0; m < 3; ++m)
            for (int n = 0; n < 3; ++n)
              S[m][n] += geo.qw[q] * g[((size_t)q * N + i) * 3 + m] * g[((size_t)q * N + j) * 3 + n];
        const double d6[6] = {S[0][0], S[1][1], S[2][2], S[0][1] + S[1][0], S[0][2] + S[2][0], S[1][2] + S[2][1]};
        for (int k = 0; k < 6; ++k) D[(size_t)k * N * N + i * N + j] = d6[k];
      }
    for (int i = 0; i < N; ++i)
      for (int gg = 0; gg < G; ++gg) {
        double m = 0.0;
        for (int q = 0; q < Q; ++q) m += geo.qw[q] * v[(size_t)q * N + i] * geo.gphi[(size_t)q * G + gg];
        M[i * G + gg] = m;
      }
  }
  h.order.resize((size_t)n_elem);
  for (int64_t e = 0; e < n_elem; ++e) h.order[(size_t)e] = (int32_t)e;
  std::stable_sort(h.order.begin(), h.order.end(), [&](int32_t a, int32_t b) { return pid[(size_t)a] < pid[(size_t)b]; });
  for (int64_t i = 0; i < n_elem;) {
    const int p = pid[(size_t)h.order[(size_t)i]];
    int64_t j = i;
    while (j < n_elem && j - i < 8 && pid[(size_t)h.order[(size_t)j]] == p) ++j;
    h.batch.push_back(p);
    h.batch.push_back((int32_t)i);
    h.batch.push_back((int32_t)(j - i));
    i = j;
  }
  return "";
}

// ------------------------------------------------------------------ prisms
// HIERARCHIC of order 2 on PRISM18 and order 3 on PRISM21.  libMesh forms
// shape i of a prism (fe_hierarchic_shape_3D.C:2290-2345, prism_indices
// :764-1150) as a 2-D HIERARCHIC triangle shape of (xi, eta) times a 1-D
// HIERARCHIC shape of zeta, after moving the coordinates of the quadrilateral
// faces' bases by the face's orientation, and negates odd triangle-edge bases
// on the bottom and top triangles by the edge's direction.  An element's
// orientation record holds every decision that evaluation makes; the shapes
// of a record are tabulated once (value and central-difference gradient,
// eps = 1e-6, evaluated operation for operation as the reference does so the
// difference quotients are its bits) and shared by the elements that have it.
namespace {

struct PrismOrient {
  uint8_t zflip[3] = {};     // vertical edge 3 + v: its 1-D bases take -zeta (positive_edge_orientation)
  uint8_t fcase[3] = {};     // quad face 1 + f: 2 * (rank of its minimum vertex in the test order) + positive
  uint8_t tflip[2][3] = {};  // bottom / top triangle edge t: odd bases negated
  uint32_t key() const {
    uint32_t k = 0;
    for (int v = 0; v < 3; ++v) k = (k << 1) | zflip[v];
    for (int f = 0; f < 3; ++f) k = (k << 3) | fcase[f];
    for (int b = 0; b < 2; ++b)
      for (int t = 0; t < 3; ++t) k = (k << 1) | tflip[b][t];
    return k;
  }
};

// Prism6 side and edge maps (cell_prism6.C:113-142) for the faces and edges used.
const int PR_QUAD[3][4] = {{0, 1, 4, 3}, {1, 2, 5, 4}, {2, 0, 3, 5}};
const int PR_MINTEST[3][4] = {{0, 3, 1, 4}, {1, 4, 2, 5}, {2, 5, 0, 3}};  // order of the == min_point tests
const int PR_SQ_ROW[4] = {0, 1, 1, 0}, PR_SQ_COL[4] = {0, 0, 1, 1};     // square_number_row / _column
const int PR_INT_PAGE[2] = {0, 1};                                       // prism_number_page (triangle index 0)

PrismOrient prism_orient(const double (*X)[3]) {
  PrismOrient o;
  for (int v = 0; v < 3; ++v) o.zflip[v] = pt_less(X[v + 3], X[v]);  // edge (v, v + 3): first vertex greater
  for (int f = 0; f < 3; ++f) {
    const int *q = PR_QUAD[f];
    // std::min(std::min(a, b), std::min(c, d)) over the face's vertices in get_min_point's argument order
    auto mn = [&](const double *a, const double *b) { return pt_less(b, a) ? b : a; };
    const int *t = PR_MINTEST[f];
    const double *m = mn(mn(X[q[0]], X[q[1]]), mn(X[q[3]], X[q[2]]));
    int v = 0;
    for (int k = 1; k < 4; ++k)
      if (pt_less(X[q[k]], X[q[v]])) v = k;
    const bool pos = pt_less(X[q[(v + 3) % 4]], X[q[(v + 1) % 4]]);
    int rank = 0;
    while (rank < 4 && !pt_eq(X[t[rank]], m)) ++rank;
    o.fcase[f] = (uint8_t)(2 * rank + (pos ? 1 : 0));
  }
  for (int b = 0; b < 2; ++b)
    for (int k = 0; k < 3; ++k) o.tflip[b][k] = pt_less(X[3 * b + (k + 1) % 3], X[3 * b + k]);
  return o;
}

// HIERARCHIC triangle shape i01 at (x, y); edge bases of odd order negated
// when `flip` has the edge's bit (fe_hierarchic_shape_2D.C:915-1026).
double prism_tri(int order, int i01, double x, double y, const uint8_t *flip) {
  const double zeta1 = x, zeta2 = y, zeta0 = 1. - zeta1 - zeta2;
  if (i01 == 0) return zeta0;
  if (i01 == 1) return zeta1;
  if (i01 == 2) return zeta2;
  double num, cross;
  int bo, t;
  if (i01 < order + 2) {
    bo = i01 - 1; t = 0; num = zeta1 - zeta0; cross = zeta0 + zeta1;
  } else if (i01 < 2 * order + 1) {
    bo = i01 - order; t = 1; num = zeta2 - zeta1; cross = zeta2 + zeta1;
  } else if (i01 < 3 * order) {
    bo = i01 - 2 * order + 1; t = 2; num = zeta0 - zeta2; cross = zeta0 + zeta2;
  } else {  // the first interior basis: zeta0 zeta1 zeta2
    double r = 1;
    r *= zeta0;
    r *= zeta1;
    r *= zeta2;
    return r;
  }
  if (cross == 0.) {
    unsigned fact = 1;
    for (int n = 2; n <= bo; ++n) fact *= (unsigned)n;
    return std::pow(num, bo) / fact;
  }
  const double sgn = (bo % 2 && flip && flip[t]) ? -1. : 1.;
  return sgn * std::pow(cross, bo) * h1(bo, num / cross);
}

// Shape i of a prism with record o at reference point p.
double prism_shape(const PrismOrient &o, int order, int i, const double *p) {
  const int e = order - 1;
  double xi = p[0], eta = p[1], zeta = p[2];
  const double xs = xi, es = eta, zs = zeta;
  int i01, i2;
  const uint8_t *flip = nullptr;  // triangle-edge flips apply to the bottom and top triangles' bases only
  if (i < 6) {
    i01 = i % 3;
    i2 = i / 3;
  } else if (i < 6 + 3 * e) {
    i01 = i - 3;
    i2 = 0;
  } else if (i < 6 + 6 * e) {
    i01 = (i - 6 - 3 * e) / e;
    i2 = (i - 6 - 3 * e) % e + 2;
    if (o.zflip[i01]) zeta = -zeta;
  } else if (i < 6 + 9 * e) {
    i01 = i - 3 - 6 * e;
    i2 = 1;
  } else if (i < 6 + 9 * e + 3 * e * e) {
    const int f = (i - 6 - 9 * e) / (e * e), b = (i - 6 - 9 * e) % (e * e);
    const int s0 = PR_SQ_ROW[b] + 2, s1 = PR_SQ_COL[b] + 2, c = o.fcase[f];
    const bool swap = c == 1 || c == 2 || c == 4 || c == 7;
    // triangle edge f numbering; face 2's first case takes index s0 + 1 + 3 as the reference does
    const int off = f == 0 ? 0 : (f == 1 ? (c == 0 ? 3 : e) : 2 * e);
    i01 = (swap ? s1 : s0) + 1 + off;
    i2 = swap ? s0 : s1;
    double xsc, xf;
    if (f == 0) {
      xsc = 1 - es;
      xf = (xsc == 0) ? 0 : xs / xsc;
    } else if (f == 1) {
      xsc = xs + es;
      xf = (xsc == 0) ? 0 : xs / xsc;
    } else {
      xsc = 1 - xs;
      xf = (xsc == 0) ? 0 : (xsc - es) / xsc;
    }
    // the in-face coordinate that runs along the triangle edge, set from v
    auto along = [&](double v) {
      if (f == 1) {
        eta = v * xsc;
        xi = xsc - eta;
      } else {
        eta = xsc - v * xsc;
      }
    };
    switch (c) {
      case 1:
        zeta = 2 * xf - 1;
        if (f == 0) xi = (zs + 1) * xsc / 2; else along((zs + 1) / 2);
        break;
      case 2:
        zeta = 1 - 2 * xf;
        if (f == 0) xi = (zs + 1) * xsc / 2; else along((zs + 1) / 2);
        break;
      case 3:
        zeta = -zs;
        break;
      case 4:
        zeta = 2 * xf - 1;
        if (f == 0) xi = (1 - zs) * xsc / 2; else along((1 - zs) / 2);
        break;
      case 5:
        if (f == 0) xi = (1 - xf) * xsc; else along(1 - xf);
        break;
      case 6:
        zeta = -zs;
        if (f == 0) xi = (1 - xf) * xsc; else along(1 - xf);
        break;
      case 7:
        zeta = 1 - 2 * xf;
        if (f == 0) xi = (1 - zs) * xsc / 2; else along((1 - zs) / 2);
        break;
      default: break;
    }
  } else if (i < 6 + 9 * e + 3 * e * e + e * (e - 1) / 2) {
    i01 = i - 3 - 6 * e - 3 * e * e;
    i2 = 0;
  } else if (i < 6 + 9 * e + 3 * e * e + e * (e - 1)) {
    i01 = i - 3 - 6 * e - 3 * e * e - e * (e - 1) / 2;
    i2 = 1;
  } else {
    const int b = i - 6 - 9 * e - 3 * e * e - e * (e - 1);
    i01 = 3 + 3 * e;  // prism_number_triangle = 0 for the first bases
    i2 = PR_INT_PAGE[b] + 2;
  }
  if (i2 < 2) flip = o.tflip[i2];
  return prism_tri(order, i01, xi, eta, flip) * h1(i2, zeta);
}

}  // namespace

// HIERARCHIC prisms (order 2 on PRISM18, 3 on PRISM21), affine elements:
// patterns are the elements' orientation records; per pattern the shapes at
// the quadrature points, D_k and M as for the cubic tets.  The map and the
// nodal load use the six vertices with the PRISM6 LAGRANGE basis (the same
// affine map as the elements' own 18- / 21-node bases, up to rounding).
std::string build_prism_tables(Hier3Tables &h, int order, int q_order, int64_t n_elem, const double *xyz,
                               const int32_t *conn, int npe) {
  if (order != 2 && order != 3) return "HIERARCHIC prisms are built for orders 2 and 3";
  h = Hier3Tables();
  const int N = (order + 1) * (order + 1) * (order + 2) / 2, G = 6;
  h.N = N;
  h.G = G;
  FETables geo;
  std::string err = build_fe_tables(geo, LMG_PRISM6, 1, q_order, 0);  // QGauss and the PRISM6 map basis
  if (!err.empty()) return err;
  if (geo.n_geo != G) return "PRISM6 map basis";
  const int Q = geo.q;
  h.q = Q;
  h.gd0.assign(geo.gdphi.begin(), geo.gdphi.begin() + G * 3);
  std::unordered_map<uint32_t, int> id;
  std::vector<PrismOrient> pats;
  std::vector<int> pid((size_t)n_elem);
  double X[6][3];
  for (int64_t e = 0; e < n_elem; ++e) {
    for (int a = 0; a < 6; ++a)
      for (int d = 0; d < 3; ++d) X[a][d] = xyz[3 * (int64_t)conn[e * npe + a] + d];
    const PrismOrient o = prism_orient(X);
    auto it = id.find(o.key());
    if (it == id.end()) {
      it = id.emplace(o.key(), (int)pats.size()).first;
      pats.push_back(o);
    }
    pid[(size_t)e] = it->second;
  }
  h.P = (int)pats.size();
  h.Dp.assign((size_t)h.P * 6 * N * N, 0.0);
  h.Mp.assign((size_t)h.P * N * G, 0.0);
  std::vector<double> v((size_t)Q * N), g((size_t)Q * N * 3);
  const double eps = 1.e-6;
  for (int pp = 0; pp < h.P; ++pp) {
    const PrismOrient &o = pats[(size_t)pp];
    for (int q = 0; q < Q; ++q)
      for (int i = 0; i < N; ++i) {
        const double *x = &geo.qp[3 * q];
        v[(size_t)q * N + i] = prism_shape(o, order, i, x);
        for (int j = 0; j < 3; ++j) {
          double xp[3] = {x[0], x[1], x[2]}, xm[3] = {x[0], x[1], x[2]};
          xp[j] += eps;
          xm[j] -= eps;
          g[((size_t)q * N + i) * 3 + j] = (prism_shape(o, order, i, xp) - prism_shape(o, order, i, xm)) / 2. / eps;
        }
      }
    double *D = &h.Dp[(size_t)pp * 6 * N * N];
    double *M = &h.Mp[(size_t)pp * N * G];
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) {
        double S[3][3] = {};
        for (int q = 0; q < Q; ++q)
          for (int m = 0; m < 3; ++m)
            for (int n = 0; n < 3; ++n)
              S[m][n] += geo.qw[q] * g[((size_t)q * N + i) * 3 + m] * g[((size_t)q * N + j) * 3 + n];
        const double d6[6] = {S[0][0], S[1][1], S[2][2], S[0][1] + S[1][0], S[0][2] + S[2][0], S[1][2] + S[2][1]};
        for (int k = 0; k < 6; ++k) D[(size_t)k * N * N + i * N + j] = d6[k];
      }
    for (int i = 0; i < N; ++i)
      for (int gg = 0; gg < G; ++gg) {
        double m = 0.0;
        for (int q = 0; q < Q; ++q) m += geo.qw[q] * v[(size_t)q * N + i] * geo.gphi[(size_t)q * G + gg];
        M[i * G + gg] = m;
      }
  }
  h.order.resize((size_t)n_elem);
  for (int64_t e = 0; e < n_elem; ++e) h.order[(size_t)e] = (int32_t)e;
  std::stable_sort(h.order.begin(), h.order.end(), [&](int32_t a, int32_t b) { return pid[(size_t)a] < pid[(size_t)b]; });
  for (int64_t i = 0; i < n_elem;) {
    const int p = pid[(size_t)h.order[(size_t)i]];
    int64_t j = i;
    while (j < n_elem && j - i < 8 && pid[(size_t)h.order[(size_t)j]] == p) ++j;
    h.batch.push_back(p);
    h.batch.push_back((int32_t)i);
    h.batch.push_back((int32_t)(j - i));
    i = j;
  }
  return "";
}

}  // namespace lmg
