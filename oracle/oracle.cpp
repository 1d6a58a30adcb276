// CPU oracle for the libMesh finite-element assembly path.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, operation by operation and in
// plain scalar C++, what libMesh does on the assembly path, so that the GPU
// product can be checked against it.  Only tests/, __graft_entry__.smoke() and
// the cpu_baseline / reference legs of bench.py may load it; the product
// (libmesh_gb300) never links or calls it.
//
// The reference cannot be compiled here (its TIMPI / MetaPhysicL submodules are
// empty and there is no MPI or PETSc), so this restatement is the oracle.  It
// is pinned by the reference's own known-answer tests as far as they reach:
// QGauss monomial exactness (tests/quadrature/quadrature_test.C), exact
// reproduction of linear / quadratic fields and gradients by LAGRANGE shapes
// (tests/fe/fe_test.h), build_cube counts (tests/mesh/mesh_generation_test.C)
// and element volumes (tests/geom/volume_test.C).  No reference test or file
// holds assembled K / F values.
//
// Build: oracle/build.py compiles it with -O2 -ffp-contract=off so that no
// multiply-add is fused, as in libMesh's x86-64 default build.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <thread>
#include <vector>

namespace {

enum { TET4 = 8, TET10 = 9, HEX8 = 10, HEX27 = 12, PRISM6 = 13, PRISM18 = 15, TET14 = 34, PRISM21 = 36 };
enum { POISSON = 0, ELASTICITY = 1 };

// libMesh's _R literal: a long double literal narrowed to Real
// (include/base/libmesh.h:283-286).
#define R_(x) ((double)(x##L))

struct Pt { double v[3]; };

// ------------------------------------------------------------------ QGauss
// QGauss::init_1D, src/quadrature/quadrature_gauss_1D.C:30-120.
void qgauss_1d(int order, std::vector<double> &x, std::vector<double> &w) {
  x.clear(); w.clear();
  switch (order) {
    case 0: case 1:
      x = {0.}; w = {2.}; return;
    case 2: case 3: {
      double p0 = -std::sqrt(3.0) / 3;
      x = {p0, -p0}; w = {1., 1.}; return;
    }
    case 4: case 5: {
      double p0 = R_(-7.7459666924148337703585307995648e-01);
      x = {p0, 0., -p0};
      double w0 = 5.0 / 9, w1 = 8.0 / 9;
      w = {w0, w1, w0}; return;
    }
    case 6: case 7: {
      double p0 = R_(-8.6113631159405257522394648889281e-01), p1 = R_(-3.3998104358485626480266575910324e-01);
      x = {p0, p1, -p1, -p0};
      double w0 = R_(3.4785484513745385737306394922200e-01), w1 = R_(6.5214515486254614262693605077800e-01);
      w = {w0, w1, w1, w0}; return;
    }
    default: {  // EIGHTH / NINTH
      double p0 = R_(-9.0617984593866399279762687829939e-01), p1 = R_(-5.3846931010568309103631442070021e-01);
      x = {p0, p1, 0., -p1, -p0};
      double w0 = R_(2.3692688505618908751426404071992e-01), w1 = R_(4.7862867049936646804129151483564e-01),
             w2 = R_(5.6888888888888888888888888888889e-01);
      w = {w0, w1, w2, w1, w0}; return;
    }
  }
}

// QGauss::keast_rule, src/quadrature/quadrature_gauss.C:43-190.
void keast_rule(const double rule[][4], int n_pts, std::vector<Pt> &P, std::vector<double> &W) {
  for (int p = 0; p < n_pts; ++p) {
    int type = 1;
    if (rule[p][1] != 0.0) type = (rule[p][2] != 0.0) ? 12 : 4;
    else if (rule[p][2] != 0.0) type = 6;
    const double a = rule[p][0], wt = rule[p][3];
    if (type == 1) { P.push_back({{a, a, a}}); W.push_back(wt); }
    else if (type == 4) {
      const double b = rule[p][1];
      P.push_back({{a, b, b}}); P.push_back({{b, a, b}}); P.push_back({{b, b, a}}); P.push_back({{b, b, b}});
      for (int j = 0; j < 4; ++j) W.push_back(wt);
    } else if (type == 6) {
      const double b = rule[p][2];
      P.push_back({{a, a, b}}); P.push_back({{a, b, b}}); P.push_back({{b, b, a}});
      P.push_back({{b, a, b}}); P.push_back({{b, a, a}}); P.push_back({{a, b, a}});
      for (int j = 0; j < 6; ++j) W.push_back(wt);
    } else {  // 12-permutation (quadrature_gauss.C:154-175), slots 0..11 in order
      const double b = rule[p][1], c = rule[p][2];
      const Pt o[12] = {{{a, a, b}}, {{a, a, c}}, {{b, a, a}}, {{c, a, a}}, {{a, b, a}}, {{a, c, a}},
                        {{a, b, c}}, {{a, c, b}}, {{b, a, c}}, {{b, c, a}}, {{c, a, b}}, {{c, b, a}}};
      for (int j = 0; j < 12; ++j) { P.push_back(o[j]); W.push_back(wt); }
    }
  }
}

// QGauss::init_3D, src/quadrature/quadrature_gauss_3D.C:30-226, and
// QBase::tensor_product_hex, src/quadrature/quadrature.C:283-305.
// QGauss::init_2D for TRI3, orders CONSTANT-FIFTH (src/quadrature/quadrature_gauss_2D.C:73-262),
// with dunavant_rule2's orbit expansion (src/quadrature/quadrature_gauss.C:195-260):
// a 3-orbit of a gives (a, a), (a, 1-2a), (1-2a, a).
void qgauss_tri(int order, std::vector<double> &x, std::vector<double> &y, std::vector<double> &w) {
  x.clear(); y.clear(); w.clear();
  auto pt = [&](double a, double b, double wt) { x.push_back(a); y.push_back(b); w.push_back(wt); };
  auto orbit3 = [&](double a, double wt) { pt(a, a, wt); pt(a, 1 - 2 * a, wt); pt(1 - 2 * a, a, wt); };
  switch (order) {
    case 0: case 1:
      pt(1.0 / 3, 1.0 / 3, 0.5); return;
    case 2:
      pt(2.0 / 3, 1.0 / 6, 1.0 / 6); pt(1.0 / 6, 2.0 / 3, 1.0 / 6); pt(1.0 / 6, 1.0 / 6, 1.0 / 6); return;
    case 3:
      pt(R_(1.5505102572168219018027159252941e-01), R_(1.7855872826361642311703513337422e-01),
         R_(1.5902069087198858469718450103758e-01));
      pt(R_(6.4494897427831780981972840747059e-01), R_(7.5031110222608118177475598324603e-02),
         R_(9.0979309128011415302815498962418e-02));
      pt(R_(1.5505102572168219018027159252941e-01), R_(6.6639024601470138670269327409637e-01),
         R_(1.5902069087198858469718450103758e-01));
      pt(R_(6.4494897427831780981972840747059e-01), R_(2.8001991549907407200279599420481e-01),
         R_(9.0979309128011415302815498962418e-02));
      return;
    case 4:
      orbit3(R_(4.4594849091596488631832925388305199e-01), R_(1.1169079483900573284750350421656140e-01));
      orbit3(R_(9.1576213509770743459571463402201508e-02), R_(5.4975871827660933819163162450105264e-02));
      return;
    default:  // FIFTH
      pt(1.0 / 3, 1.0 / 3, 9.0 / 80);
      orbit3(2.0 / 7 + std::sqrt(15.0) / 21, 31.0 / 480 + std::sqrt(15.0) / 2400);
      orbit3(2.0 / 7 - std::sqrt(15.0) / 21, 31.0 / 480 - std::sqrt(15.0) / 2400);
      return;
  }
}

bool qgauss_3d(int type, int order, std::vector<Pt> &P, std::vector<double> &W) {
  P.clear(); W.clear();
  if (type == PRISM6 || type == PRISM18 || type == PRISM21) {  // quadrature_gauss_3D.C:507-525, tensor_product_prism (quadrature.C:310-331)
    if (order > 5) return false;
    std::vector<double> z, wz, tx, ty, tw;
    qgauss_1d(order, z, wz);
    qgauss_tri(order, tx, ty, tw);
    for (size_t j = 0; j < z.size(); j++)
      for (size_t i = 0; i < tw.size(); i++) {
        P.push_back({{tx[i], ty[i], z[j]}});
        W.push_back(tw[i] * wz[j]);
      }
    return true;
  }
  if (type == HEX8 || type == HEX27) {
    std::vector<double> x, w;
    qgauss_1d(order, x, w);
    const int np = (int)x.size();
    for (int k = 0; k < np; k++)
      for (int j = 0; j < np; j++)
        for (int i = 0; i < np; i++) {
          P.push_back({{x[i], x[j], x[k]}});
          W.push_back(w[i] * w[j] * w[k]);
        }
    return true;
  }
  if (type != TET4 && type != TET10 && type != TET14) return false;
  switch (order) {
    case 0: case 1:
      P.push_back({{.25, .25, .25}}); W.push_back(1.0 / 6); return true;
    case 2: {
      const double b = 0.25 * (1 - std::sqrt(5.0) / 5);
      const double a = 1 - 3 * b;
      P = {{{a, b, b}}, {{b, a, b}}, {{b, b, a}}, {{b, b, b}}};
      const double w0 = 1.0 / 24;
      W = {w0, w0, w0, w0}; return true;
    }
    case 3: {  // allow_rules_with_negative_weights defaults to true (quadrature.C:29)
      P = {{{.25, .25, .25}}, {{.5, 1.0 / 6, 1.0 / 6}}, {{1.0 / 6, .5, 1.0 / 6}},
           {{1.0 / 6, 1.0 / 6, .5}}, {{1.0 / 6, 1.0 / 6, 1.0 / 6}}};
      W = {-2.0 / 15, .075, .075, .075, .075}; return true;
    }
    case 4: {
      const double rule[3][4] = {
          {R_(0.250000000000000000e+00), 0., 0., R_(-0.131555555555555556e-01)},
          {R_(0.785714285714285714e+00), R_(0.714285714285714285e-01), 0., R_(0.762222222222222222e-02)},
          {R_(0.399403576166799219e+00), 0., R_(0.100596423833200785e+00), R_(0.248888888888888889e-01)}};
      keast_rule(rule, 3, P, W);
      return true;
    }
    case 5: {  // quadrature_gauss_3D.C:231-287
      const double a[3] = {R_(0.31088591926330060980), R_(0.092735250310891226402), R_(0.045503704125649649492)};
      const double wt[3] = {R_(0.018781320953002641800), R_(0.012248840519393658257),
                            R_(0.0070910034628469110730)};
      for (int i = 0; i < 2; ++i) {
        const double b = 1. - 3. * a[i];
        P.push_back({{a[i], a[i], a[i]}}); P.push_back({{a[i], b, a[i]}});
        P.push_back({{b, a[i], a[i]}}); P.push_back({{a[i], a[i], b}});
        for (int j = 0; j < 4; ++j) W.push_back(wt[i]);
      }
      const double b = 0.5 * (1. - 2. * a[2]);
      P.push_back({{b, b, a[2]}}); P.push_back({{b, a[2], a[2]}}); P.push_back({{a[2], a[2], b}});
      P.push_back({{a[2], b, a[2]}}); P.push_back({{b, a[2], b}}); P.push_back({{a[2], b, b}});
      for (int j = 0; j < 6; ++j) W.push_back(wt[2]);
      return true;
    }
    case 6: {  // quadrature_gauss_3D.C:401-420
      const double rule[4][4] = {
          {R_(0.356191386222544953e+00), R_(0.214602871259151684e+00), 0., R_(0.00665379170969464506e+00)},
          {R_(0.877978124396165982e+00), R_(0.0406739585346113397e+00), 0., R_(0.00167953517588677620e+00)},
          {R_(0.0329863295731730594e+00), R_(0.322337890142275646e+00), 0., R_(0.00922619692394239843e+00)},
          {R_(0.0636610018750175299e+00), R_(0.269672331458315867e+00), R_(0.603005664791649076e+00),
           R_(0.00803571428571428248e+00)}};
      keast_rule(rule, 4, P, W);
      return true;
    }
    default:
      return false;
  }
}

// ------------------------------------------------------------------ shapes
// include/fe/fe_lagrange_shape_1D.h
double l1(int i, double xi) { return i == 0 ? .5 * (1. - xi) : .5 * (1. + xi); }
double l1d(int i) { return i == 0 ? -.5 : .5; }
double q1(int i, double xi) {
  if (i == 0) return .5 * xi * (xi - 1.);
  if (i == 1) return .5 * xi * (xi + 1);
  return (1. - xi * xi);
}
double q1d(int i, double xi) {
  if (i == 0) return xi - .5;
  if (i == 1) return xi + .5;
  return -2. * xi;
}

const unsigned H8_I0[] = {0, 1, 1, 0, 0, 1, 1, 0};
const unsigned H8_I1[] = {0, 0, 1, 1, 0, 0, 1, 1};
const unsigned H8_I2[] = {0, 0, 0, 0, 1, 1, 1, 1};
const unsigned H27_I0[] = {0, 1, 1, 0, 0, 1, 1, 0, 2, 1, 2, 0, 0, 1, 1, 0, 2, 1, 2, 0, 2, 2, 1, 2, 0, 2, 2};
const unsigned H27_I1[] = {0, 0, 1, 1, 0, 0, 1, 1, 0, 2, 1, 2, 0, 0, 1, 1, 0, 2, 1, 2, 2, 0, 2, 1, 2, 2, 2};
const unsigned H27_I2[] = {0, 0, 0, 0, 1, 1, 1, 1, 0, 0, 0, 0, 2, 2, 2, 2, 1, 1, 1, 1, 0, 2, 2, 2, 2, 1, 2};

// Number of LAGRANGE shapes of `order` on `type` (isoparametric cases only).
int n_shapes(int type, int order) {
  if (type == PRISM6) return order == 1 ? 6 : 0;
  if (type == HEX8 || type == HEX27) return order == 1 ? 8 : (type == HEX27 ? 27 : 0);
  if (type == TET4 || type == TET10) return order == 1 ? 4 : (type == TET10 ? 10 : 0);
  if (type == TET14) return order == 1 ? 4 : 14;
  return 0;
}

// TET14 (fe_lagrange_shape_3D.C:1402-1460): quadratic shapes plus multiples
// of the face bubbles; derivatives as written at :2931-3260.
double tet14_shape(int i, const Pt &p) {
  const double zeta1 = p.v[0], zeta2 = p.v[1], zeta3 = p.v[2];
  const double zeta0 = 1. - zeta1 - zeta2 - zeta3;
  const double bubble_012 = zeta0 * zeta1 * zeta2, bubble_013 = zeta0 * zeta1 * zeta3,
               bubble_123 = zeta1 * zeta2 * zeta3, bubble_023 = zeta0 * zeta2 * zeta3;
  switch (i) {
    case 0: return zeta0 * (2. * zeta0 - 1.) + 3. * (bubble_012 + bubble_013 + bubble_023);
    case 1: return zeta1 * (2. * zeta1 - 1.) + 3. * (bubble_012 + bubble_013 + bubble_123);
    case 2: return zeta2 * (2. * zeta2 - 1.) + 3. * (bubble_012 + bubble_023 + bubble_123);
    case 3: return zeta3 * (2. * zeta3 - 1.) + 3. * (bubble_013 + bubble_023 + bubble_123);
    case 4: return 4. * zeta0 * zeta1 - 12. * (bubble_012 + bubble_013);
    case 5: return 4. * zeta1 * zeta2 - 12. * (bubble_012 + bubble_123);
    case 6: return 4. * zeta2 * zeta0 - 12. * (bubble_012 + bubble_023);
    case 7: return 4. * zeta0 * zeta3 - 12. * (bubble_013 + bubble_023);
    case 8: return 4. * zeta1 * zeta3 - 12. * (bubble_013 + bubble_123);
    case 9: return 4. * zeta2 * zeta3 - 12. * (bubble_023 + bubble_123);
    case 10: return 27. * bubble_012;
    case 11: return 27. * bubble_013;
    case 12: return 27. * bubble_123;
    default: return 27. * bubble_023;
  }
}
double tet14_deriv(int i, int j, const Pt &p) {
  const double zeta1 = p.v[0], zeta2 = p.v[1], zeta3 = p.v[2];
  const double zeta0 = 1. - zeta1 - zeta2 - zeta3;
  const double dz[3][4] = {{-1., 1., 0., 0.}, {-1., 0., 1., 0.}, {-1., 0., 0., 1.}};
  double b012, b013, b123, b023;
  if (j == 0) { b012 = (zeta0 - zeta1) * zeta2; b013 = (zeta0 - zeta1) * zeta3; b123 = zeta2 * zeta3; b023 = -zeta2 * zeta3; }
  else if (j == 1) { b012 = (zeta0 - zeta2) * zeta1; b013 = -zeta1 * zeta3; b123 = zeta1 * zeta3; b023 = (zeta0 - zeta2) * zeta3; }
  else { b012 = -zeta1 * zeta2; b013 = (zeta0 - zeta3) * zeta1; b123 = zeta1 * zeta2; b023 = (zeta0 - zeta3) * zeta2; }
  const double *d = dz[j];
  switch (i) {
    case 0: return (4. * zeta0 - 1.) * d[0] + 3. * (b012 + b013 + b023);
    case 1: return (4. * zeta1 - 1.) * d[1] + 3. * (b012 + b013 + b123);
    case 2: return (4. * zeta2 - 1.) * d[2] + 3. * (b012 + b023 + b123);
    case 3: return (4. * zeta3 - 1.) * d[3] + 3. * (b013 + b023 + b123);
    case 4: return 4. * (zeta0 * d[1] + d[0] * zeta1) - 12. * (b012 + b013);
    case 5: return 4. * (zeta1 * d[2] + d[1] * zeta2) - 12. * (b012 + b123);
    case 6: return 4. * (zeta0 * d[2] + d[0] * zeta2) - 12. * (b012 + b023);
    case 7: return 4. * (zeta0 * d[3] + d[0] * zeta3) - 12. * (b013 + b023);
    case 8: return 4. * (zeta1 * d[3] + d[1] * zeta3) - 12. * (b013 + b123);
    case 9: return 4. * (zeta2 * d[3] + d[2] * zeta3) - 12. * (b023 + b123);
    case 10: return 27. * b012;
    case 11: return 27. * b013;
    case 12: return 27. * b123;
    default: return 27. * b023;
  }
}

// fe_lagrange_3D_shape for TET4/TET10 (src/fe/fe_lagrange_shape_3D.C:710-740, 957-1010).
double tet_shape(int order, int i, const Pt &p) {
  const double zeta1 = p.v[0], zeta2 = p.v[1], zeta3 = p.v[2];
  const double zeta0 = 1. - zeta1 - zeta2 - zeta3;
  if (order == 1) {
    const double z[4] = {zeta0, zeta1, zeta2, zeta3};
    return z[i];
  }
  if (order == 3) return tet14_shape(i, p);
  switch (i) {
    case 0: return zeta0 * (2. * zeta0 - 1.);
    case 1: return zeta1 * (2. * zeta1 - 1.);
    case 2: return zeta2 * (2. * zeta2 - 1.);
    case 3: return zeta3 * (2. * zeta3 - 1.);
    case 4: return 4. * zeta0 * zeta1;
    case 5: return 4. * zeta1 * zeta2;
    case 6: return 4. * zeta2 * zeta0;
    case 7: return 4. * zeta0 * zeta3;
    case 8: return 4. * zeta1 * zeta3;
    default: return 4. * zeta2 * zeta3;
  }
}

// fe_lagrange_3D_shape_deriv for TET4/TET10 (src/fe/fe_lagrange_shape_3D.C:1543-1638, 2175-2330).
double tet_shape_deriv(int order, int i, int j, const Pt &p) {
  const double dz[4][3] = {{-1., -1., -1.}, {1., 0., 0.}, {0., 1., 0.}, {0., 0., 1.}};
  if (order == 1) return dz[i][j];
  if (order == 3) return tet14_deriv(i, j, p);
  const double zeta1 = p.v[0], zeta2 = p.v[1], zeta3 = p.v[2];
  const double zeta0 = 1. - zeta1 - zeta2 - zeta3;
  const double z[4] = {zeta0, zeta1, zeta2, zeta3};
  if (i < 4) return (4. * z[i] - 1.) * dz[i][j];
  static const int E[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
  const int a = E[i - 4][0], b = E[i - 4][1];
  return 4. * (z[a] * dz[b][j] + dz[a][j] * z[b]);
}

// fe_lagrange_3D_shape(_deriv) for PRISM6 (fe_lagrange_shape_3D.C:742-762, 1639-1676):
// FE<2,LAGRANGE>::shape(TRI3, FIRST) = (1 - xi - eta, xi, eta) times the 1-D
// linear shape in zeta, i0 = {0,0,0,1,1,1}, i1 = {0,1,2,0,1,2}.
double tri3_shape(int i, double xi, double eta) {
  return i == 0 ? 1. - xi - eta : (i == 1 ? xi : eta);
}
double tri3_deriv(int i, int j) {
  static const double d[3][2] = {{-1., -1.}, {1., 0.}, {0., 1.}};
  return d[i][j];
}
double prism6_shape(int i, const Pt &p) {
  static const int i0[] = {0, 0, 0, 1, 1, 1}, i1[] = {0, 1, 2, 0, 1, 2};
  return tri3_shape(i1[i], p.v[0], p.v[1]) * l1(i0[i], p.v[2]);
}
double prism6_deriv(int i, int j, const Pt &p) {
  static const int i0[] = {0, 0, 0, 1, 1, 1}, i1[] = {0, 1, 2, 0, 1, 2};
  if (j < 2) return tri3_deriv(i1[i], j) * l1(i0[i], p.v[2]);
  return tri3_shape(i1[i], p.v[0], p.v[1]) * l1d(i0[i]);
}

// FE<3,LAGRANGE>::all_shapes / all_shape_derivs at a list of points
// (hex tensor fast path, fe_lagrange_shape_3D.C:72-416; tets by scalar calls).
// phi[i][p], d[c][i][p].
void all_shapes(int type, int order, const std::vector<Pt> &pts, std::vector<std::vector<double>> &phi,
                std::vector<std::vector<double>> d[3]) {
  const int n = n_shapes(type, order), np = (int)pts.size();
  phi.assign(n, std::vector<double>(np));
  for (int c = 0; c < 3; ++c) d[c].assign(n, std::vector<double>(np));
  const bool hex = (type == HEX8 || type == HEX27);
  for (int q = 0; q < np; ++q) {
    if (hex) {
      const double xi = pts[q].v[0], eta = pts[q].v[1], zeta = pts[q].v[2];
      const unsigned *i0 = order == 1 ? H8_I0 : H27_I0, *i1 = order == 1 ? H8_I1 : H27_I1,
                     *i2 = order == 1 ? H8_I2 : H27_I2;
      double s[3][3], ds[3][3];
      for (int k = 0; k < (order == 1 ? 2 : 3); ++k) {
        const double c3[3] = {xi, eta, zeta};
        for (int m = 0; m < 3; ++m) {
          s[m][k] = order == 1 ? l1(k, c3[m]) : q1(k, c3[m]);
          ds[m][k] = order == 1 ? l1d(k) : q1d(k, c3[m]);
        }
      }
      for (int i = 0; i < n; ++i) {
        phi[i][q] = s[0][i0[i]] * s[1][i1[i]] * s[2][i2[i]];
        d[0][i][q] = ds[0][i0[i]] * s[1][i1[i]] * s[2][i2[i]];
        d[1][i][q] = s[0][i0[i]] * ds[1][i1[i]] * s[2][i2[i]];
        d[2][i][q] = s[0][i0[i]] * s[1][i1[i]] * ds[2][i2[i]];
      }
    } else if (type == PRISM6) {
      for (int i = 0; i < n; ++i) {
        phi[i][q] = prism6_shape(i, pts[q]);
        for (int c = 0; c < 3; ++c) d[c][i][q] = prism6_deriv(i, c, pts[q]);
      }
    } else {
      for (int i = 0; i < n; ++i) {
        phi[i][q] = tet_shape(order, i, pts[q]);
        for (int c = 0; c < 3; ++c) d[c][i][q] = tet_shape_deriv(order, i, c, pts[q]);
      }
    }
  }
}

// ------------------------------------------------------------------ HIERARCHIC
// fe_hierarchic_1D_shape (src/fe/fe_hierarchic_shape_1D.C:430-498).
double hier_1d(unsigned i, double xi) {
  double returnval = 1.;
  switch (i) {
    case 0: returnval = .5 * (1. - xi); break;
    case 1: returnval = .5 * (1. + xi); break;
    case 2: returnval = (xi * xi - 1.) / 2.; break;
    case 3: returnval = (xi * xi * xi - xi) / 6.; break;
    default: {
      double denominator = 1.;
      for (unsigned n = 1; n <= i; ++n) {
        returnval *= xi;
        denominator *= n;
      }
      returnval = (i % 2) ? (returnval - xi) / denominator : (returnval - 1.) / denominator;
    }
  }
  return returnval;
}

// cube_indices (fe_hierarchic_shape_3D.C:166-760) for totalorder <= 2: vertex
// dofs 0-7, edge dofs 8-19 (e = 1 per edge), face dofs 20-25, interior 26.
// The edge / face flips it applies negate or swap arguments of even 1-D
// functions at this order, which leaves every value unchanged, so they are
// not restated.
void cube_indices_p2(unsigned i, unsigned &i0, unsigned &i1, unsigned &i2) {
  static const unsigned V[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                   {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
  static const unsigned EF[19][3] = {  // i = 8 .. 26
      {2, 0, 0}, {1, 2, 0}, {2, 1, 0}, {0, 2, 0}, {0, 0, 2}, {1, 0, 2}, {1, 1, 2}, {0, 1, 2}, {2, 0, 1},
      {1, 2, 1}, {2, 1, 1}, {0, 2, 1}, {2, 2, 0}, {2, 0, 2}, {1, 2, 2}, {2, 1, 2}, {0, 2, 2}, {2, 2, 1},
      {2, 2, 2}};
  const unsigned *t = i < 8 ? V[i] : EF[i - 8];
  i0 = t[0];
  i1 = t[1];
  i2 = t[2];
}

// FE<3,HIERARCHIC>::shape on a hex: (s0 * s1) * s2.
double hier_hex_shape(unsigned i, const Pt &p) {
  unsigned i0, i1, i2;
  cube_indices_p2(i, i0, i1, i2);
  return hier_1d(i0, p.v[0]) * hier_1d(i1, p.v[1]) * hier_1d(i2, p.v[2]);
}

// ---------------------------------------------------------- HIERARCHIC p = 3
// cube_indices for totalorder 3 on a HEX27 (fe_hierarchic_shape_3D.C:166-760):
// e = 2 dofs per edge, e^2 = 4 per face, e^3 = 8 interior.  Edge dofs reflect
// their coordinate when Elem::positive_edge_orientation (elem.C:3634-3640,
// lexicographic Point >) says so; face dofs swap / reflect the two in-face
// coordinates by the face's minimum vertex (get_min_point) and
// Elem::positive_face_orientation (elem.C:3642-3661).  Interior dofs use
// cube_number_column / row / page; face dofs square_number_row / column
// (number_lookups.C), restated for the entries this order reaches.
bool pt_less(const Pt &a, const Pt &b) {  // TypeVector::operator< (type_vector.C:66-76)
  for (int i = 0; i < 3; i++) {
    if (a.v[i] < b.v[i]) return true;
    if (a.v[i] > b.v[i]) return false;
  }
  return false;
}
bool pt_eq(const Pt &a, const Pt &b) { return a.v[0] == b.v[0] && a.v[1] == b.v[1] && a.v[2] == b.v[2]; }

const unsigned HEX_EDGE[12][2] = {{0, 1}, {1, 2}, {2, 3}, {0, 3}, {0, 4}, {1, 5},
                                  {2, 6}, {3, 7}, {4, 5}, {5, 6}, {6, 7}, {4, 7}};
const unsigned HEX_SIDE4[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}, {4, 5, 6, 7}};

bool positive_edge_orientation(const std::vector<Pt> &X, unsigned i) {
  return pt_less(X[HEX_EDGE[i][1]], X[HEX_EDGE[i][0]]);
}
bool positive_face_orientation(const std::vector<Pt> &X, unsigned i) {
  const unsigned *nodes = HEX_SIDE4[i];
  const unsigned N = 4;
  unsigned v = 0;
  for (unsigned k = 1; k < N; ++k)
    if (pt_less(X[nodes[k]], X[nodes[v]])) v = k;  // std::min_element: first minimum
  return pt_less(X[nodes[(v - 1 + N) % N]], X[nodes[(v + 1) % N]]);
}
Pt min_point(const std::vector<Pt> &X, unsigned a, unsigned b, unsigned c, unsigned d) {
  auto mn = [](const Pt &p, const Pt &q) { return pt_less(q, p) ? q : p; };  // std::min
  return mn(mn(X[a], X[b]), mn(X[c], X[d]));
}

// e = totalorder - 1 dofs per edge (e <= 2: totalorder 2 or 3).  At
// totalorder 2 the edge flips and face reflections negate arguments of even
// 1-D functions (no change), but the face swaps move coordinates between the
// product's factors, which changes its rounding -- and, through the central
// differences, the derivatives by ~1e-11 -- so the remap is applied there too.
void cube_indices_hex(const std::vector<Pt> &X, unsigned e, unsigned i, double &xi, double &eta, double &zeta,
                      unsigned &i0, unsigned &i1, unsigned &i2) {
  static const unsigned SQ_ROW[4] = {0, 1, 1, 0}, SQ_COL[4] = {0, 0, 1, 1};
  static const unsigned CB_COL[8] = {0, 0, 1, 1, 0, 1, 1, 0}, CB_ROW[8] = {0, 1, 1, 0, 1, 1, 0, 0},
                        CB_PAGE[8] = {0, 0, 0, 0, 1, 1, 1, 1};
  static const unsigned V[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                   {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
  const double xs = xi, es = eta, zs = zeta;
  if (i < 8) {
    i0 = V[i][0]; i1 = V[i][1]; i2 = V[i][2];
    return;
  }
  if (i < 8 + 12 * e) {  // edges: the varying index and its direction, then the flip rule
    const unsigned ed = (i - 8) / e, k = i - ed * e - 6;
    static const int DIR[12] = {0, 1, 0, 1, 2, 2, 2, 2, 0, 1, 0, 1};
    static const unsigned FIX[12][2] = {{0, 0}, {1, 0}, {1, 0}, {0, 0}, {0, 0}, {1, 0},
                                        {1, 1}, {0, 1}, {0, 1}, {1, 1}, {1, 1}, {0, 1}};
    const bool pos = positive_edge_orientation(X, ed);
    const bool flip = (ed == 2 || ed == 10) ? !pos : pos;
    const int d = DIR[ed];
    if (d == 0) { i0 = k; i1 = FIX[ed][0]; i2 = FIX[ed][1]; if (flip) xi = -xs; }
    else if (d == 1) { i0 = FIX[ed][0]; i1 = k; i2 = FIX[ed][1]; if (flip) eta = -es; }
    else { i0 = FIX[ed][0]; i1 = FIX[ed][1]; i2 = k; if (flip) zeta = -zs; }
    return;
  }
  if (i < 8 + 12 * e + 6 * e * e) {
    const unsigned f = (i - 8 - 12 * e) / (e * e), basisnum = i - 8 - 12 * e - f * e * e;
    const unsigned r = SQ_ROW[basisnum] + 2, c = SQ_COL[basisnum] + 2;
    // Per face: its in-face coordinates (A, B), the vertices the cases test
    // against get_min_point in their order, whether the orientation test is
    // negated, and the remap of each case (o = orientation test true / false):
    // ID (A, B), SW (B, A), TA (-B, A), TB (A, -B), NG (-A, -B), NS (-B, -A),
    // TC (B, -A), TD (-A, B) -- the eight cases of every face as written there.
    enum { ID, SW, TA, TB, NG, NS, TC, TD };
    static const unsigned TESTV[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5},
                                         {3, 7, 6, 2}, {0, 4, 7, 3}, {4, 5, 6, 7}};
    static const unsigned GMP[6][4] = {{1, 2, 0, 3}, {0, 1, 5, 4}, {1, 2, 6, 5},
                                       {2, 3, 7, 6}, {3, 0, 4, 7}, {4, 5, 6, 7}};
    static const bool NEG[6] = {false, true, true, false, false, true};
    static const int CASE[6][4][2] = {{{ID, SW}, {TA, TB}, {NG, NS}, {TC, TD}},
                                      {{ID, SW}, {TC, TD}, {NG, NS}, {TD, TB}},
                                      {{ID, SW}, {TC, TD}, {NG, NS}, {TA, TB}},
                                      {{ID, SW}, {TA, TB}, {NG, NS}, {TC, TD}},
                                      {{ID, SW}, {TA, TB}, {NG, NS}, {TC, TD}},
                                      {{ID, SW}, {TC, TD}, {NG, NS}, {TA, ID}}};
    double *A, *B;
    double As, Bs;
    switch (f) {
      case 0: i0 = r; i1 = c; i2 = 0; A = &xi; B = &eta; As = xs; Bs = es; break;
      case 1: i0 = r; i1 = 0; i2 = c; A = &xi; B = &zeta; As = xs; Bs = zs; break;
      case 2: i0 = 1; i1 = r; i2 = c; A = &eta; B = &zeta; As = es; Bs = zs; break;
      case 3: i0 = r; i1 = 1; i2 = c; A = &xi; B = &zeta; As = xs; Bs = zs; break;
      case 4: i0 = 0; i1 = r; i2 = c; A = &eta; B = &zeta; As = es; Bs = zs; break;
      default: i0 = r; i1 = c; i2 = 1; A = &xi; B = &eta; As = xs; Bs = es; break;
    }
    const Pt m = min_point(X, GMP[f][0], GMP[f][1], GMP[f][2], GMP[f][3]);
    const bool o = NEG[f] ? !positive_face_orientation(X, f) : positive_face_orientation(X, f);
    for (int t = 0; t < 4; ++t) {
      if (!pt_eq(X[TESTV[f][t]], m)) continue;
      switch (CASE[f][t][o ? 0 : 1]) {
        case ID: *A = As; *B = Bs; break;
        case SW: *A = Bs; *B = As; break;
        case TA: *A = -Bs; *B = As; break;
        case TB: *A = As; *B = -Bs; break;
        case NG: *A = -As; *B = -Bs; break;
        case NS: *A = -Bs; *B = -As; break;
        case TC: *A = Bs; *B = -As; break;
        default: *A = -As; *B = Bs; break;
      }
      break;
    }
    return;
  }
  const unsigned basisnum = i - 8 - 12 * e - 6 * e * e;
  i0 = CB_COL[basisnum] + 2;
  i1 = CB_ROW[basisnum] + 2;
  i2 = CB_PAGE[basisnum] + 2;
}

// FE<3,HIERARCHIC>::shape at totalorder 3 on one element: cube_indices, then
// (s0 * s1) * s2 at the remapped coordinates.
double hier_hexo_shape(const std::vector<Pt> &X, unsigned order, unsigned i, const Pt &p) {
  double xi = p.v[0], eta = p.v[1], zeta = p.v[2];
  unsigned i0, i1, i2;
  cube_indices_hex(X, order - 1, i, xi, eta, zeta, i0, i1, i2);
  return hier_1d(i0, xi) * hier_1d(i1, eta) * hier_1d(i2, zeta);
}
double hier_hexo_deriv(const std::vector<Pt> &X, unsigned order, unsigned i, unsigned j, const Pt &p) {
  const double eps = 1.e-6;
  Pt pp = p, pm = p;
  pp.v[j] += eps;
  pm.v[j] -= eps;
  return (hier_hexo_shape(X, order, i, pp) - hier_hexo_shape(X, order, i, pm)) / 2. / eps;
}
double hier_hex3_shape(const std::vector<Pt> &X, unsigned i, const Pt &p) { return hier_hexo_shape(X, 3, i, p); }
double hier_hex3_deriv(const std::vector<Pt> &X, unsigned i, unsigned j, const Pt &p) {
  return hier_hexo_deriv(X, 3, i, j, p);
}

// fe_fdm_deriv (src/fe/fe.C:794-811, 929-944): central difference, eps = 1e-6.
double hier_hex_deriv(unsigned i, unsigned j, const Pt &p) {
  const double eps = 1.e-6;
  Pt pp = p, pm = p;
  pp.v[j] += eps;
  pm.v[j] -= eps;
  return (hier_hex_shape(i, pp) - hier_hex_shape(i, pm)) / 2. / eps;
}

// FE<3,HIERARCHIC>::shape on a tet, totalorder <= 2 (fe_hierarchic_shape_3D.C,
// TET4/TET10/TET14 branch): vertex dofs are the barycentric coordinates; edge
// dof of edge k (Tet4::edge_nodes_map, cell_tet4.C:46-54) is
// crossval^2 * hier_1d(2, (z1 - z0) / crossval) with crossval = z0 + z1, or
// (z1 - z0)^2 / 2 when crossval is exactly 0.  The odd-order edge flip does
// not arise at this order.
double hier_tet_shape(unsigned i, const Pt &p) {
  const double zeta[4] = {1 - p.v[0] - p.v[1] - p.v[2], p.v[0], p.v[1], p.v[2]};
  if (i < 4) return zeta[i];
  static const unsigned EN[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
  const unsigned edge_num = i - 4, basisorder = 2;
  const double crossval = zeta[EN[edge_num][0]] + zeta[EN[edge_num][1]];
  const double edgenumerator = zeta[EN[edge_num][1]] - zeta[EN[edge_num][0]];
  if (crossval == 0.) {
    unsigned basisfactorial = 1;
    for (unsigned n = 2; n <= basisorder; ++n) basisfactorial *= n;
    return std::pow(edgenumerator, basisorder) / basisfactorial;
  }
  const double edgeval = edgenumerator / crossval;
  const double crossfunc = std::pow(crossval, basisorder);
  const double flip = 1;
  return flip * crossfunc * hier_1d(basisorder, edgeval);
}

// FE<3,HIERARCHIC>::shape on a TET14 at totalorder 3
// (fe_hierarchic_shape_3D.C:2361-2440).  Edge e of Tet4::edge_nodes_map has
// the bases of order 2 and 3; the odd one is negated when
// Elem::positive_edge_orientation(e) holds, i.e. the edge's first vertex is
// greater in TypeVector's lexicographic order (elem.C:3634-3640,
// type_vector.C:95-105).  Face f's one basis is the triangular monomial with
// exponents (1, 1) times the third coordinate, over the face's vertices
// sorted by orient_triangle (fe_hierarchic_shape_3D.C:2193-2243).
bool pt_greater(const Pt &a, const Pt &b) {
  for (int d = 0; d < 3; ++d) {
    if (a.v[d] > b.v[d]) return true;
    if (a.v[d] < b.v[d]) return false;
  }
  return false;
}
double hier_tet3_shape(const std::vector<Pt> &X, unsigned i, const Pt &p) {
  const double zeta[4] = {1 - p.v[0] - p.v[1] - p.v[2], p.v[0], p.v[1], p.v[2]};
  const unsigned totalorder = 3;
  if (i < 4) return zeta[i];
  static const unsigned EN[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
  if (i < 6u * totalorder - 2u) {
    const unsigned edge_num = (i - 4) / (totalorder - 1u);
    const unsigned basisorder = i - 2 - ((totalorder - 1u) * edge_num);
    const unsigned v0 = EN[edge_num][0], v1 = EN[edge_num][1];
    double flip = 1;
    if (basisorder % 2 && pt_greater(X[v0], X[v1])) flip = -1;
    const double crossval = zeta[v0] + zeta[v1];
    const double edgenumerator = zeta[v1] - zeta[v0];
    if (crossval == 0.) {
      unsigned basisfactorial = 1;
      for (unsigned n = 2; n <= basisorder; ++n) basisfactorial *= n;
      return std::pow(edgenumerator, basisorder) / basisfactorial;
    }
    const double edgeval = edgenumerator / crossval;
    const double crossfunc = std::pow(crossval, basisorder);
    return flip * crossfunc * hier_1d(basisorder, edgeval);
  }
  static const unsigned SN[4][3] = {{0, 2, 1}, {0, 1, 3}, {1, 2, 3}, {2, 0, 3}};  // Tet4::side_nodes_map
  const unsigned face_num = i - (6u * totalorder - 2u);
  unsigned fv[3] = {SN[face_num][0], SN[face_num][1], SN[face_num][2]};
  bool lastcheck = true;
  if (pt_greater(X[fv[0]], X[fv[1]])) { std::swap(fv[0], fv[1]); lastcheck = true; }
  if (pt_greater(X[fv[1]], X[fv[2]])) std::swap(fv[1], fv[2]);
  if (lastcheck && pt_greater(X[fv[0]], X[fv[1]])) std::swap(fv[0], fv[1]);
  // basisnum 0: triangular_number_column[0] = triangular_number_row[0] = 0
  const unsigned exp0 = 0 + 1, exp1 = 0 + 1 - 0;
  double returnval = 1;
  for (unsigned n = 0; n != exp0; ++n) returnval *= zeta[fv[0]];
  for (unsigned n = 0; n != exp1; ++n) returnval *= zeta[fv[1]];
  returnval *= zeta[fv[2]];
  return returnval;
}
double hier_tet3_deriv(const std::vector<Pt> &X, unsigned i, unsigned j, const Pt &p) {
  const double eps = 1.e-6;
  Pt pp = p, pm = p;
  pp.v[j] += eps;
  pm.v[j] -= eps;
  return (hier_tet3_shape(X, i, pp) - hier_tet3_shape(X, i, pm)) / 2. / eps;
}

// ------------------------------------------------ HIERARCHIC prisms, p = 2, 3
// FE<3,HIERARCHIC>::shape on PRISM18 / PRISM20 / PRISM21
// (fe_hierarchic_shape_3D.C:2290-2345): prism_indices (:764-1150) picks the
// triangle index i01 and the 1-D index i2, remapping (xi, eta) and zeta for
// the quadrilateral faces by the face's minimum vertex and
// positive_face_orientation, and reflecting zeta on a vertical edge with
// positive_edge_orientation; the value is the 2-D HIERARCHIC triangle shape
// i01 (fe_hierarchic_shape_2D.C:965-1026, edge bases through
// fe_triangle_helper :915-948, negated for odd orders when the triangle's
// edge runs from the greater point) on a Tri3 built from vertices 0-2 or 3-5
// (with the two nodes of an odd square-face basis's edge put in ascending
// order), times the 1-D HIERARCHIC shape i2 of zeta.  Derivatives are central
// differences, eps = 1e-6 (fe_fdm_deriv, fe.C:911-928).  Restated literally,
// including face 2's first orientation case, which takes triangle basis
// s0 + 1 + 3 where its other cases take s0 + 1 + e.
namespace prism {
const unsigned EDGE[9][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 4}, {2, 5}, {3, 4}, {4, 5}, {3, 5}};
const unsigned SIDE[5][4] = {{0, 2, 1, 99}, {0, 1, 4, 3}, {1, 2, 5, 4}, {2, 0, 3, 5}, {3, 4, 5, 99}};
const unsigned SQ_ROW[4] = {0, 1, 1, 0}, SQ_COL[4] = {0, 0, 1, 1};  // square_number_row / _column
const unsigned TRI_ROW[1] = {0}, TRI_COL[1] = {0};                  // triangular_number_row / _column
const unsigned PR_TRI[2] = {0, 0}, PR_PAGE[2] = {0, 1};             // prism_number_triangle / _page

bool edge_positive(const std::vector<Pt> &X, unsigned e) { return pt_greater(X[EDGE[e][0]], X[EDGE[e][1]]); }

bool face_positive(const std::vector<Pt> &X, unsigned s) {
  const unsigned *nodes = SIDE[s];
  const unsigned N = (s == 0 || s == 4) ? 3 : 4;
  unsigned v = 0;
  for (unsigned k = 1; k < N; ++k)
    if (pt_less(X[nodes[k]], X[nodes[v]])) v = k;
  return pt_less(X[nodes[(v + N - 1) % N]], X[nodes[(v + 1) % N]]);
}

void indices(const std::vector<Pt> &X, unsigned totalorder, unsigned i, double &xi, double &eta, double &zeta,
             unsigned &i01, unsigned &i2) {
  const unsigned e = totalorder - 1u;
  const double xs = xi, es = eta, zs = zeta;
  if (i < 6) {
    i01 = i % 3;
    i2 = i / 3;
  } else if (i < 6 + 3 * e) {
    i01 = i - 3;
    i2 = 0;
  } else if (i < 6 + 6 * e) {
    i01 = (i - 6 - 3 * e) / e;
    i2 = (i - 6 - 3 * e) % e + 2;
    if (edge_positive(X, i01 + 3)) zeta = -zeta;
  } else if (i < 6 + 9 * e) {
    i01 = i - 3 - 6 * e;
    i2 = 1;
  } else if (i < 6 + 9 * e + e * e) {  // face 1
    const unsigned b = i - 6 - 9 * e;
    const double xe_scale = 1 - es;
    const double xe_fraction = (xe_scale == 0) ? 0 : xs / xe_scale;
    const unsigned s0 = SQ_ROW[b] + 2, s1 = SQ_COL[b] + 2;
    const Pt mp = min_point(X, 0, 1, 3, 4);
    const bool pos = face_positive(X, 1);
    if (pt_eq(X[0], mp)) {
      if (!pos) { i01 = s0 + 1; i2 = s1; }
      else { i01 = s1 + 1; i2 = s0; zeta = 2 * xe_fraction - 1; xi = (zs + 1) * xe_scale / 2; }
    } else if (pt_eq(X[3], mp)) {
      if (!pos) { i01 = s1 + 1; i2 = s0; zeta = 1 - 2 * xe_fraction; xi = (zs + 1) * xe_scale / 2; }
      else { i01 = s0 + 1; i2 = s1; zeta = -zs; }
    } else if (pt_eq(X[1], mp)) {
      if (!pos) { i01 = s1 + 1; i2 = s0; zeta = 2 * xe_fraction - 1; xi = (1 - zs) * xe_scale / 2; }
      else { i01 = s0 + 1; i2 = s1; xi = (1 - xe_fraction) * xe_scale; }
    } else if (pt_eq(X[4], mp)) {
      if (!pos) { i01 = s0 + 1; i2 = s1; xi = (1 - xe_fraction) * xe_scale; zeta = -zs; }
      else { i01 = s1 + 1; i2 = s0; zeta = 1 - 2 * xe_fraction; xi = (1 - zs) * xe_scale / 2; }
    }
  } else if (i < 6 + 9 * e + 2 * e * e) {  // face 2
    const unsigned b = i - 6 - 9 * e - e * e;
    const double xe_scale = xs + es;
    const double xe_fraction = (xe_scale == 0) ? 0 : xs / xe_scale;
    const unsigned s0 = SQ_ROW[b] + 2, s1 = SQ_COL[b] + 2;
    const Pt mp = min_point(X, 1, 2, 4, 5);
    const bool pos = face_positive(X, 2);
    auto set_xe = [&](double xe) {
      eta = xe * xe_scale;
      xi = xe_scale - eta;
    };
    if (pt_eq(X[1], mp)) {
      if (!pos) { i01 = s0 + 1 + 3; i2 = s1; }
      else { i01 = s1 + 1 + e; i2 = s0; zeta = 2 * xe_fraction - 1; set_xe((zs + 1) / 2); }
    } else if (pt_eq(X[4], mp)) {
      if (!pos) { i01 = s1 + 1 + e; i2 = s0; zeta = 1 - 2 * xe_fraction; set_xe((zs + 1) / 2); }
      else { i01 = s0 + 1 + e; i2 = s1; zeta = -zs; }
    } else if (pt_eq(X[2], mp)) {
      if (!pos) { i01 = s1 + 1 + e; i2 = s0; zeta = 2 * xe_fraction - 1; set_xe((1 - zs) / 2); }
      else { i01 = s0 + 1 + e; i2 = s1; set_xe(1 - xe_fraction); }
    } else if (pt_eq(X[5], mp)) {
      if (!pos) { i01 = s0 + 1 + e; i2 = s1; zeta = -zs; set_xe(1 - xe_fraction); }
      else { i01 = s1 + 1 + e; i2 = s0; zeta = 1 - 2 * xe_fraction; set_xe((1 - zs) / 2); }
    }
  } else if (i < 6 + 9 * e + 3 * e * e) {  // face 3
    const unsigned b = i - 6 - 9 * e - 2 * e * e;
    const double xe_scale = 1 - xs;
    const double xe_fraction = (xe_scale == 0) ? 0 : (xe_scale - es) / xe_scale;
    const unsigned s0 = SQ_ROW[b] + 2, s1 = SQ_COL[b] + 2;
    const Pt mp = min_point(X, 0, 2, 3, 5);
    const bool pos = face_positive(X, 3);
    auto set_xe = [&](double xe) { eta = xe_scale - xe * xe_scale; };
    if (pt_eq(X[2], mp)) {
      if (!pos) { i01 = s0 + 1 + 2 * e; i2 = s1; }
      else { i01 = s1 + 1 + 2 * e; i2 = s0; zeta = 2 * xe_fraction - 1; set_xe((zs + 1) / 2); }
    } else if (pt_eq(X[5], mp)) {
      if (!pos) { i01 = s1 + 1 + 2 * e; i2 = s0; zeta = 1 - 2 * xe_fraction; set_xe((zs + 1) / 2); }
      else { i01 = s0 + 1 + 2 * e; i2 = s1; zeta = -zs; }
    } else if (pt_eq(X[0], mp)) {
      if (!pos) { i01 = s1 + 1 + 2 * e; i2 = s0; zeta = 2 * xe_fraction - 1; set_xe((1 - zs) / 2); }
      else { i01 = s0 + 1 + 2 * e; i2 = s1; set_xe(1 - xe_fraction); }
    } else if (pt_eq(X[3], mp)) {
      if (!pos) { i01 = s0 + 1 + 2 * e; i2 = s1; zeta = -zs; set_xe(1 - xe_fraction); }
      else { i01 = s1 + 1 + 2 * e; i2 = s0; zeta = 1 - 2 * xe_fraction; set_xe((1 - zs) / 2); }
    }
  } else if (i < 6 + 9 * e + 3 * e * e + e * (e - 1) / 2) {  // face 0
    i01 = i - 3 - 6 * e - 3 * e * e;
    i2 = 0;
  } else if (i < 6 + 9 * e + 3 * e * e + e * (e - 1)) {  // face 4
    i01 = i - 3 - 6 * e - 3 * e * e - e * (e - 1) / 2;
    i2 = 1;
  } else {  // interior
    const unsigned b = i - 6 - 9 * e - 3 * e * e - e * (e - 1);
    i01 = PR_TRI[b] + 3 + 3 * e;
    i2 = PR_PAGE[b] + 2;
  }
}

// fe_triangle_helper on the triangle with vertex points T[0..2].
double tri_edge(const Pt *T, double num, double cross, unsigned basisorder, unsigned noden) {
  double flip = 1;
  if (basisorder % 2 && pt_greater(T[noden], T[(noden + 1) % 3])) flip = -1.;
  if (cross == 0.) {
    unsigned basisfactorial = 1;
    for (unsigned n = 2; n <= basisorder; ++n) basisfactorial *= n;
    return std::pow(num, basisorder) / basisfactorial;
  }
  const double edgeval = num / cross;
  const double crossfunc = std::pow(cross, basisorder);
  return flip * crossfunc * hier_1d(basisorder, edgeval);
}

// FE<2,L2_HIERARCHIC>::shape on a TRI3 with vertex points T.
double tri_shape(const Pt *T, unsigned totalorder, unsigned i, double x, double y) {
  const double zeta1 = x, zeta2 = y, zeta0 = 1. - zeta1 - zeta2;
  if (i == 0) return zeta0;
  if (i == 1) return zeta1;
  if (i == 2) return zeta2;
  if (i < totalorder + 2u) return tri_edge(T, zeta1 - zeta0, zeta0 + zeta1, i - 1, 0);
  if (i < 2u * totalorder + 1) return tri_edge(T, zeta2 - zeta1, zeta2 + zeta1, i - totalorder, 1);
  if (i < 3u * totalorder) return tri_edge(T, zeta0 - zeta2, zeta0 + zeta2, i - (2u * totalorder) + 1, 2);
  const unsigned basisnum = i - (3u * totalorder);
  const unsigned exp0 = TRI_COL[basisnum] + 1, exp1 = TRI_ROW[basisnum] + 1 - TRI_COL[basisnum];
  double r = 1;
  for (unsigned n = 0; n != exp0; ++n) r *= zeta0;
  for (unsigned n = 0; n != exp1; ++n) r *= zeta1;
  r *= zeta2;
  return r;
}

double shape(const std::vector<Pt> &X, unsigned totalorder, unsigned i, const Pt &p) {
  double xi = p.v[0], eta = p.v[1], zeta = p.v[2];
  unsigned i01 = 0, i2 = 0;
  indices(X, totalorder, i, xi, eta, zeta, i01, i2);
  Pt T[3];
  if (i2 == 1) {
    T[0] = X[3]; T[1] = X[4]; T[2] = X[5];
  } else {
    T[0] = X[0]; T[1] = X[1]; T[2] = X[2];
    if (i2 > 1 && i01 > 2 && i01 < 3u * totalorder) {
      const bool odd_basis = ((i01 - 1) % (totalorder - 1)) % 2;
      if (odd_basis) {
        const unsigned te = (i01 - 3) / (totalorder - 1);
        if (pt_greater(T[te], T[(te + 1) % 3])) std::swap(T[te], T[(te + 1) % 3]);
      }
    }
  }
  return tri_shape(T, totalorder, i01, xi, eta) * hier_1d(i2, zeta);
}

double deriv(const std::vector<Pt> &X, unsigned totalorder, unsigned i, unsigned j, const Pt &p) {
  const double eps = 1.e-6;
  Pt pp = p, pm = p;
  pp.v[j] += eps;
  pm.v[j] -= eps;
  return (shape(X, totalorder, i, pp) - shape(X, totalorder, i, pm)) / 2. / eps;
}
}  // namespace prism

// FE<3,HIERARCHIC>::shape on a PRISM6, totalorder 1 (prism_indices vertices,
// fe_hierarchic_shape_3D.C:764-810): the TRI vertex function (zeta0 =
// 1 - xi - eta, xi, eta; fe_hierarchic_shape_2D.C:969-983) times the 1-D
// end function in zeta.
double hier_prism_shape(unsigned i, const Pt &p) {
  const unsigned i01 = i % 3, i2 = i / 3;
  const double zeta1 = p.v[0], zeta2 = p.v[1], zeta0 = 1. - zeta1 - zeta2;
  const double t = i01 == 0 ? zeta0 : (i01 == 1 ? zeta1 : zeta2);
  return t * hier_1d(i2, p.v[2]);
}

double hier_shape(int type, unsigned i, const Pt &p) {
  if (type == PRISM6) return hier_prism_shape(i, p);
  return (type == TET4 || type == TET10) ? hier_tet_shape(i, p) : hier_hex_shape(i, p);
}

double hier_deriv(int type, unsigned i, unsigned j, const Pt &p) {
  if (type == HEX8 || type == HEX27) return hier_hex_deriv(i, j, p);
  const double eps = 1.e-6;
  Pt pp = p, pm = p;
  pp.v[j] += eps;
  pm.v[j] -= eps;
  return (hier_shape(type, i, pp) - hier_shape(type, i, pm)) / 2. / eps;
}

bool hierarchic_built(int type, int order) {
  return (type == HEX8 && order == 1) || (type == HEX27 && order == 2) || (type == TET4 && order == 1) ||
         (type == TET10 && order == 2) || (type == PRISM6 && order == 1);
}

void all_shapes_hierarchic(int type, int order, const std::vector<Pt> &pts, std::vector<std::vector<double>> &phi,
                           std::vector<std::vector<double>> d[3]) {
  const bool tet = (type == TET4 || type == TET10);
  const unsigned n = type == PRISM6 ? (order + 1) * (order + 1) * (order + 2) / 2
                     : tet      ? (order + 1) * (order + 2) * (order + 3) / 6
                                : (order + 1) * (order + 1) * (order + 1);
  const unsigned np = (unsigned)pts.size();
  phi.assign(n, std::vector<double>(np));
  for (int c = 0; c < 3; ++c) d[c].assign(n, std::vector<double>(np));
  for (unsigned q = 0; q < np; ++q)
    for (unsigned i = 0; i < n; ++i) {
      phi[i][q] = hier_shape(type, i, pts[q]);
      for (unsigned c = 0; c < 3; ++c) d[c][i][q] = hier_deriv(type, i, c, pts[q]);
    }
}

}  // namespace

namespace {

// ------------------------------------------------------------------ affine test
// relative_fuzzy_equals (include/utils/fuzzy_equals.h:78-84) with affine_tol = TOLERANCE^2.
bool rfe(const Pt &a, const Pt &b) {
  const double tol = 1.e-6 * 1.e-6;
  double d = 0, la = 0, lb = 0;
  for (int i = 0; i < 3; ++i) d += std::abs(a.v[i] - b.v[i]);
  for (int i = 0; i < 3; ++i) la += std::abs(a.v[i]);
  for (int i = 0; i < 3; ++i) lb += std::abs(b.v[i]);
  return d <= tol * (la + lb);
}
Pt sub(const Pt &a, const Pt &b) { return {{a.v[0] - b.v[0], a.v[1] - b.v[1], a.v[2] - b.v[2]}}; }
Pt scl(const Pt &a, double s) { return {{a.v[0] * s, a.v[1] * s, a.v[2] * s}}; }
Pt dvd(const Pt &a, double s) { return {{a.v[0] / s, a.v[1] / s, a.v[2] / s}}; }

// Elem::has_affine_map: cell_hex8.C:121, cell_hex27.C:125, cell_tet4.h:136, cell_tet10.C:143.
bool has_affine_map(int type, const std::vector<Pt> &p) {
  if (type == TET4) return true;
  if (type == PRISM6) {  // cell_prism6.C:199-207
    const Pt v = sub(p[3], p[0]);
    return rfe(v, sub(p[4], p[1])) && rfe(v, sub(p[5], p[2]));
  }
  if (type == TET10 || type == TET14) {
    const int E[6][3] = {{1, 0, 4}, {2, 1, 5}, {2, 0, 6}, {3, 0, 7}, {3, 1, 8}, {3, 2, 9}};
    for (auto &e : E)
      if (!rfe(sub(p[e[0]], p[e[1]]), scl(sub(p[e[2]], p[e[1]]), 2))) return false;
    if (type == TET10) return true;
    // cell_tet14.C:181-193: each face node at the face centroid
    const Pt v10 = sub(p[1], p[0]), v20 = sub(p[2], p[0]), v30 = sub(p[3], p[0]), v21 = sub(p[2], p[1]),
             v31 = sub(p[3], p[1]);
    auto add = [](const Pt &a, const Pt &b) { return Pt{{a.v[0] + b.v[0], a.v[1] + b.v[1], a.v[2] + b.v[2]}}; };
    return rfe(add(v20, v10), scl(sub(p[10], p[0]), 3)) && rfe(add(v30, v10), scl(sub(p[11], p[0]), 3)) &&
           rfe(add(v31, v21), scl(sub(p[12], p[1]), 3)) && rfe(add(v30, v20), scl(sub(p[13], p[0]), 3));
  }
  Pt v = sub(p[1], p[0]);
  if (!rfe(v, sub(p[2], p[3])) || !rfe(v, sub(p[5], p[4])) || !rfe(v, sub(p[6], p[7]))) return false;
  if (type == HEX27) {
    v = dvd(v, 2);
    const int X[9][2] = {{8, 0}, {10, 3}, {16, 4}, {18, 7}, {20, 11}, {21, 12}, {23, 15}, {25, 19}, {26, 24}};
    for (auto &x : X) if (!rfe(v, sub(p[x[0]], p[x[1]]))) return false;
  }
  v = sub(p[4], p[0]);
  if (!rfe(v, sub(p[7], p[3]))) return false;
  if (type == HEX27) {
    v = dvd(v, 2);
    const int Z[6][2] = {{12, 0}, {13, 1}, {14, 2}, {15, 3}, {22, 9}, {24, 11}};
    for (auto &z : Z) if (!rfe(v, sub(p[z[0]], p[z[1]]))) return false;
    v = dvd(sub(p[3], p[0]), 2);
    const int Y[4][2] = {{11, 0}, {9, 1}, {17, 5}, {19, 4}};
    for (auto &y : Y) if (!rfe(v, sub(p[y[0]], p[y[1]]))) return false;
  }
  return true;
}

// ------------------------------------------------------------------ FE object
// FE<3,LAGRANGE>::reinit (src/fe/fe.C:197-368) with its FEMap
// (src/fe/fe_map.C:109-444, 448-1078, 1167-1374) and H1FETransformation::map_dphi
// (src/fe/h1_fe_transformation.C:64-195).  Shape tables are built once per
// element type (the reference caches them while the type does not change).
struct OracleFE {
  int type = 0, order = 0, n = 0, n_geo = 0, nq = 0;
  std::vector<Pt> qp;
  std::vector<double> qw;
  std::vector<std::vector<double>> phi, dref[3];      // FE shapes
  std::vector<std::vector<double>> phi_map, dmap[3];  // mapping shapes (default order)
  // per-element results
  std::vector<double> JxW, jac, G[9];                 // G[3*m+d] = dxi_m/dx_d
  std::vector<std::vector<Pt>> dphi;                  // dphi[i][q]

  int family = 0;  // 0 LAGRANGE, 1 HIERARCHIC (order <= 2)
  bool prism_hi = false;  // HIERARCHIC order 2 on PRISM18 / 3 on PRISM21
  bool init(int type_, int order_, int q_order, int family_ = 0) {
    family = family_;
    type = type_; order = order_;
    if (!qgauss_3d(type, q_order, qp, qw)) return false;
    nq = (int)qp.size();
    prism_hi = family == 1 && ((order == 2 && type == PRISM18) || (order == 3 && type == PRISM21));
    const bool p3 = prism_hi ||
                    (family == 1 && ((order == 3 && (type == HEX27 || type == TET14)) || (order == 2 && type == HEX27)));
    n = prism_hi ? (order + 1) * (order + 1) * (order + 2) / 2
                 : (p3 ? (type == HEX27 ? (order + 1) * (order + 1) * (order + 1) : 20) : n_shapes(type, order));
    // PRISM18 / PRISM21 (affine only): the map and the load interpolation by
    // the six vertices' PRISM6 basis -- the same affine Jacobian as their own
    // 18- / 21-node bases up to rounding
    const int geo_type = prism_hi ? PRISM6 : type;
    const int geo_order = (type == HEX27 || type == TET10) ? 2 : (type == TET14 ? 3 : 1);
    n_geo = n_shapes(geo_type, geo_order);
    if (!n || !n_geo) return false;
    if (p3) {  // element-dependent: filled by orient() per element
      phi.assign(n, std::vector<double>(nq));
      for (int c = 0; c < 3; ++c) dref[c].assign(n, std::vector<double>(nq));
    } else if (family == 1) all_shapes_hierarchic(type, order, qp, phi, dref);
    else all_shapes(type, order, qp, phi, dref);
    all_shapes(geo_type, geo_order, qp, phi_map, dmap);
    JxW.assign(nq, 0); jac.assign(nq, 0);
    for (auto &g : G) g.assign(nq, 0);
    dphi.assign(n, std::vector<Pt>(nq));
    return true;
  }

  // compute_single_point_map, 3-D branch (fe_map.C:980-1078).  Returns false
  // when jac <= jacobian_tolerance (0), i.e. libMesh would throw DegenerateMap.
  bool single_point_map(const std::vector<Pt> &X, int p) {
    double dxi[3] = {0, 0, 0}, deta[3] = {0, 0, 0}, dzeta[3] = {0, 0, 0};
    for (int i = 0; i < n_geo; ++i)
      for (int c = 0; c < 3; ++c) {
        dxi[c] += dmap[0][i][p] * X[i].v[c];
        deta[c] += dmap[1][i][p] * X[i].v[c];
        dzeta[c] += dmap[2][i][p] * X[i].v[c];
      }
    const double dx_dxi = dxi[0], dy_dxi = dxi[1], dz_dxi = dxi[2];
    const double dx_deta = deta[0], dy_deta = deta[1], dz_deta = deta[2];
    const double dx_dzeta = dzeta[0], dy_dzeta = dzeta[1], dz_dzeta = dzeta[2];
    jac[p] = (dx_dxi * (dy_deta * dz_dzeta - dz_deta * dy_dzeta) +
              dy_dxi * (dz_deta * dx_dzeta - dx_deta * dz_dzeta) +
              dz_dxi * (dx_deta * dy_dzeta - dy_deta * dx_dzeta));
    const bool ok = jac[p] > 0.0;
    JxW[p] = jac[p] * qw[p];
    const double inv_jac = 1. / jac[p];
    G[0][p] = (dy_deta * dz_dzeta - dz_deta * dy_dzeta) * inv_jac;
    G[1][p] = (dz_deta * dx_dzeta - dx_deta * dz_dzeta) * inv_jac;
    G[2][p] = (dx_deta * dy_dzeta - dy_deta * dx_dzeta) * inv_jac;
    G[3][p] = (dz_dxi * dy_dzeta - dy_dxi * dz_dzeta) * inv_jac;
    G[4][p] = (dx_dxi * dz_dzeta - dz_dxi * dx_dzeta) * inv_jac;
    G[5][p] = (dy_dxi * dx_dzeta - dx_dxi * dy_dzeta) * inv_jac;
    G[6][p] = (dy_dxi * dz_deta - dz_dxi * dy_deta) * inv_jac;
    G[7][p] = (dz_dxi * dx_deta - dx_dxi * dz_deta) * inv_jac;
    G[8][p] = (dx_dxi * dy_deta - dy_dxi * dx_deta) * inv_jac;
    return ok;
  }

  // HIERARCHIC cubic shapes depend on the element's edge and face orientation:
  // recomputed for every element (fe.C:174-192 re-inits when the cached
  // element does not match).
  void orient(const std::vector<Pt> &X) {
    if (prism_hi) {
      for (int q = 0; q < nq; ++q)
        for (int i = 0; i < n; ++i) {
          phi[i][q] = prism::shape(X, (unsigned)order, i, qp[q]);
          for (int c = 0; c < 3; ++c) dref[c][i][q] = prism::deriv(X, (unsigned)order, i, c, qp[q]);
        }
      return;
    }
    if (!(family == 1 && ((order == 3 && (type == HEX27 || type == TET14)) || (order == 2 && type == HEX27)))) return;
    const bool tet = type == TET14;
    for (int q = 0; q < nq; ++q)
      for (int i = 0; i < n; ++i) {
        phi[i][q] = tet ? hier_tet3_shape(X, i, qp[q]) : hier_hexo_shape(X, order, i, qp[q]);
        for (int c = 0; c < 3; ++c)
          dref[c][i][q] = tet ? hier_tet3_deriv(X, i, c, qp[q]) : hier_hexo_deriv(X, order, i, c, qp[q]);
      }
  }

  bool reinit(const std::vector<Pt> &X) {
    bool ok = true;
    if (has_affine_map(prism_hi ? PRISM6 : type, X)) {  // compute_affine_map, fe_map.C:1167-1245
      ok = single_point_map(X, 0);
      for (int p = 1; p < nq; ++p) {
        for (int k = 0; k < 9; ++k) G[k][p] = G[k][0];
        jac[p] = jac[0];
        JxW[p] = JxW[0] / qw[0] * qw[p];
      }
    } else {
      for (int p = 0; p < nq; ++p) ok = single_point_map(X, p) && ok;
    }
    // map_dphi: dphi/dx = dphi/dxi dxi/dx + dphi/deta deta/dx + dphi/dzeta dzeta/dx
    for (int i = 0; i < n; ++i)
      for (int p = 0; p < nq; ++p)
        for (int d = 0; d < 3; ++d)
          dphi[i][p].v[d] = (dref[0][i][p] * G[0 + d][p] + dref[1][i][p] * G[3 + d][p] +
                             dref[2][i][p] * G[6 + d][p]);
    return ok;
  }
};

double dot(const Pt &a, const Pt &b) { return (a.v[0] * b.v[0] + a.v[1] * b.v[1] + a.v[2] * b.v[2]); }

// ------------------------------------------------------------------ dense algebra
struct Dense {
  int m = 0, n = 0;
  std::vector<double> v;  // row-major, include/numerics/dense_matrix.h:969-977
  void resize(int m_, int n_) { m = m_; n = n_; v.assign((size_t)m * n, 0.0); }
  double &operator()(int i, int j) { return v[(size_t)i * n + j]; }
  double operator()(int i, int j) const { return v[(size_t)i * n + j]; }
};

// DenseMatrix::_left_multiply_transpose (include/numerics/dense_matrix_impl.h:109-168), this <- A^T this.
void left_multiply_transpose(Dense &self, const Dense &A) {
  Dense B = self;
  self.resize(A.n, B.n);
  for (int i = 0; i < A.n; i++)
    for (int k = 0; k < A.m; k++)
      if (A(k, i) != 0.)
        for (int j = 0; j < self.n; j++) self(i, j) += A(k, i) * B(k, j);
}
// DenseMatrix::right_multiply -> DenseMatrixBase::multiply (dense_matrix_base_impl.h:46-68), this <- this M3.
void right_multiply(Dense &self, const Dense &M3) {
  Dense M2 = self;
  self.resize(M2.m, M3.n);
  for (int k = 0; k < M2.n; k++)
    for (int j = 0; j < self.n; j++)
      if (M3(k, j) != 0.)
        for (int i = 0; i < M2.m; i++) self(i, j) += M2(i, k) * M3(k, j);
}

}  // namespace

namespace {

// ------------------------------------------------------------------ element assembly
const int ADVDIFF = 2;

struct Problem {
  int form, type, fe_order, q_order, npe, n_vars, nl;
  int64_t n_nodes, n_elem, n_dofs;
  const double *xyz;
  const int32_t *conn, *elem_dofs;
  const uint8_t *constrained;
  const double *coef, *nodal_f;
  double nu;
  const int32_t *row_ptr, *col;
  // constraint rows (NULL: every constrained dof has an empty row)
  const int64_t *cons_ptr;
  const int32_t *cons_col;
  const double *cons_val;
  // ADVDIFF: {kappa, n_modes, then per mode a[3], k[3], phase}
  const double *params;
  int n_params;
};

// Constraint row of dof d as (dof, coefficient) pairs in ascending dof order
// (DofConstraintRow is a std::map).
void constraint_row(const Problem &P, int32_t d, std::vector<std::pair<int32_t, double>> &row) {
  row.clear();
  if (!P.cons_ptr) return;
  for (int64_t k = P.cons_ptr[d]; k < P.cons_ptr[d + 1]; ++k) row.emplace_back(P.cons_col[k], P.cons_val[k]);
}

// DofMap::build_constraint_matrix (src/base/dof_map_constraints.C:3433-3540).
void build_constraint_matrix(const Problem &P, Dense &C, std::vector<int32_t> &elem_dofs, bool called_recursively) {
  std::set<int32_t> dof_set;
  bool we_have_constraints = false;
  std::vector<std::pair<int32_t, double>> row;
  for (const auto &dof : elem_dofs)
    if (P.constrained[dof]) {
      we_have_constraints = true;
      constraint_row(P, dof, row);
      for (const auto &item : row) dof_set.insert(item.first);
    }
  if (!we_have_constraints) return;
  for (const auto &dof : elem_dofs) dof_set.erase(dof);
  if (!dof_set.empty() || !called_recursively) {
    const int old_size = (int)elem_dofs.size();
    elem_dofs.insert(elem_dofs.end(), dof_set.begin(), dof_set.end());
    C.resize(old_size, (int)elem_dofs.size());
    for (int i = 0; i != old_size; i++)
      if (P.constrained[elem_dofs[i]]) {
        constraint_row(P, elem_dofs[i], row);
        for (const auto &item : row)
          for (int j = 0, n_elem_dofs = (int)elem_dofs.size(); j != n_elem_dofs; j++)
            if (elem_dofs[j] == item.first) C(i, j) = item.second;
      } else {
        C(i, i) = 1.;
      }
    Dense Cnew;
    build_constraint_matrix(P, Cnew, elem_dofs, true);
    if ((C.n == Cnew.m) && (Cnew.n == (int)elem_dofs.size())) right_multiply(C, Cnew);
  }
}

// Transport velocity b = curl psi of psi = sum_m a_m sin(k_m . x + phase_m):
// b = sum_m cos(k_m . x + phase_m) (k_m x a_m).
void velocity(const Problem &P, const Pt &x, double b[3]) {
  b[0] = b[1] = b[2] = 0.;
  const int nm = P.n_params > 1 ? (int)P.params[1] : 0;
  for (int m = 0; m < nm; ++m) {
    const double *md = P.params + 2 + 7 * m;
    const double *a = md, *k = md + 3;
    const double c = std::cos(k[0] * x.v[0] + k[1] * x.v[1] + k[2] * x.v[2] + md[6]);
    b[0] += c * (k[1] * a[2] - k[2] * a[1]);
    b[1] += c * (k[2] * a[0] - k[0] * a[2]);
    b[2] += c * (k[0] * a[1] - k[1] * a[0]);
  }
}

// Lamé form of the elasticity tensor (systems_of_equations_ex6.C:120-150) with Young's modulus E.
double elasticity_tensor(double E, double nu, unsigned i, unsigned j, unsigned k, unsigned l) {
  auto kd = [](unsigned a, unsigned b) { return a == b ? 1. : 0.; };
  const double lambda_1 = (E * nu) / ((1. + nu) * (1. - 2. * nu));
  const double lambda_2 = E / (2. * (1. + nu));
  return lambda_1 * kd(i, j) * kd(k, l) + lambda_2 * (kd(i, k) * kd(j, l) + kd(i, l) * kd(j, k));
}

// One element: reinit, weak form, constrain_element_matrix_and_vector.
// Returns false on a degenerate map.
bool element_matrix(const Problem &P, OracleFE &fe, int64_t e, Dense &Ke, std::vector<double> &Fe,
                    std::vector<int32_t> &dofs) {
  std::vector<Pt> X(P.npe);
  for (int a = 0; a < P.npe; ++a)
    for (int d = 0; d < 3; ++d) X[a].v[d] = P.xyz[3 * (int64_t)P.conn[e * P.npe + a] + d];
  fe.orient(X);
  const bool ok = fe.reinit(X);
  const int n = fe.n, nl = P.nl;
  dofs.assign(P.elem_dofs + e * nl, P.elem_dofs + (e + 1) * nl);
  Ke.resize(nl, nl);
  Fe.assign(nl, 0.0);
  const double coef = P.coef ? P.coef[e] : 1.0;
  std::vector<double> f(n * P.n_vars, 0.0);
  if (P.nodal_f && n == P.npe)
    for (int a = 0; a < n; ++a)
      for (int v = 0; v < P.n_vars; ++v) f[a * P.n_vars + v] = P.nodal_f[(int64_t)P.conn[e * P.npe + a] * P.n_vars + v];
  // More shapes than nodes (HIERARCHIC cubic on HEX27): the nodal load is
  // interpolated by the mapping basis, f(x_q) = sum_g phi_map_g(q) f_g.
  const bool geo_load = n != P.npe || fe.prism_hi;
  std::vector<double> fq(fe.nq, 0.0);
  if (P.nodal_f && geo_load)
    for (int qp = 0; qp < fe.nq; qp++)
      for (int g = 0; g < fe.n_geo; ++g) fq[qp] += fe.phi_map[g][qp] * P.nodal_f[(int64_t)P.conn[e * P.npe + g]];
  if (P.form == ADVDIFF) {
    // Steady Galerkin convection-diffusion (adaptivity_ex2.C:660-690 without
    // the time terms): Ke(i,j) += JxW [(b . dphi_j) phi_i + kappa_e dphi_i . dphi_j],
    // Fe(i) += JxW f phi_i, with kappa_e = kappa * coef_e and b at the mapped point.
    const double kappa = P.params[0] * coef;
    for (int qp = 0; qp < fe.nq; qp++) {
      Pt xq = {{0., 0., 0.}};
      for (int a = 0; a < fe.n_geo; ++a)
        for (int d = 0; d < 3; ++d) xq.v[d] += fe.phi_map[a][qp] * X[a].v[d];
      double bv[3];
      velocity(P, xq, bv);
      const Pt b = {{bv[0], bv[1], bv[2]}};
      for (int i = 0; i != n; i++)
        for (int j = 0; j != n; j++)
          Ke(i, j) += fe.JxW[qp] * (dot(b, fe.dphi[j][qp]) * fe.phi[i][qp] +
                                    kappa * dot(fe.dphi[i][qp], fe.dphi[j][qp]));
    }
    for (int qp = 0; qp < fe.nq; qp++) {
      double fxy = 0.0;
      for (int j = 0; j < n; ++j) fxy += fe.phi[j][qp] * f[j];
      if (geo_load) fxy = fq[qp];
      for (int i = 0; i != n; i++) Fe[i] += fe.JxW[qp] * fxy * fe.phi[i][qp];
    }
  } else if (P.form == POISSON) {
    // introduction_ex4.C:464-467 and 536 with nodal f interpolated by phi.
    for (int qp = 0; qp < fe.nq; qp++)
      for (int i = 0; i != n; i++)
        for (int j = 0; j != n; j++)
          Ke(i, j) += (coef * fe.JxW[qp]) * dot(fe.dphi[i][qp], fe.dphi[j][qp]);
    for (int qp = 0; qp < fe.nq; qp++) {
      double fxy = 0.0;
      for (int j = 0; j < n; ++j) fxy += fe.phi[j][qp] * f[j];
      if (geo_load) fxy = fq[qp];
      for (int i = 0; i != n; i++) Fe[i] += fe.JxW[qp] * fxy * fe.phi[i][qp];
    }
  } else {
    // systems_of_equations_ex6.C:214-236: Ke_var[i][k](dof_i,dof_j) += JxW C_ijkl dphi_j(l) dphi_i(j).
    for (int qp = 0; qp < fe.nq; qp++) {
      for (int dof_i = 0; dof_i < n; dof_i++)
        for (int dof_j = 0; dof_j < n; dof_j++)
          for (unsigned i = 0; i < 3; i++)
            for (unsigned j = 0; j < 3; j++)
              for (unsigned k = 0; k < 3; k++)
                for (unsigned l = 0; l < 3; l++)
                  Ke(i * n + dof_i, k * n + dof_j) += fe.JxW[qp] * elasticity_tensor(coef, P.nu, i, j, k, l) *
                                                      fe.dphi[dof_j][qp].v[l] * fe.dphi[dof_i][qp].v[j];
      double f_vec[3] = {0, 0, 0};
      for (int i = 0; i < 3; ++i)
        for (int b = 0; b < n; ++b) f_vec[i] += fe.phi[b][qp] * f[b * 3 + i];
      for (int dof_i = 0; dof_i < n; dof_i++)
        for (int i = 0; i < 3; i++) Fe[i * n + dof_i] += fe.JxW[qp] * (f_vec[i] * fe.phi[dof_i][qp]);
    }
  }
  // DofMap::constrain_element_matrix_and_vector (dof_map_constraints.C:2439-2515)
  // with asymmetric constraint rows (the default, include/base/dof_map.h:1351-1354).
  Dense C;
  build_constraint_matrix(P, C, dofs, false);
  if ((C.m == Ke.m) && (C.n == (int)dofs.size())) {
    left_multiply_transpose(Ke, C);
    right_multiply(Ke, C);
    std::vector<std::pair<int32_t, double>> row;
    for (int i = 0, n_elem_dofs = (int)dofs.size(); i != n_elem_dofs; i++)
      if (P.constrained[dofs[i]]) {
        for (int j = 0; j < Ke.n; ++j) Ke(i, j) = 0.;
        Ke(i, i) = 1.;
        constraint_row(P, dofs[i], row);
        for (const auto &item : row)
          for (int j = 0; j != n_elem_dofs; j++)
            if (dofs[j] == item.first) Ke(i, j) = -item.second;
      }
    std::vector<double> old_rhs = Fe;
    Fe.assign(C.n, 0.);
    for (int i = 0; i < C.n; i++)  // DenseMatrix::vector_mult_transpose
      for (int j = 0; j < C.m; j++) Fe[i] += C(j, i) * old_rhs[j];
  }
  return ok;
}

// PetscMatrix::add_matrix (MatSetValues ADD_VALUES, petsc_matrix.C:735-755) into a
// preallocated AIJ pattern; a missing entry is an error (MAT_NEW_NONZERO_ALLOCATION_ERR).
bool add_matrix(const Problem &P, const Dense &Ke, const std::vector<int32_t> &dofs, double *K) {
  for (int i = 0; i < Ke.m; ++i) {
    const int32_t r = dofs[i];
    const int32_t *b = P.col + P.row_ptr[r], *en = P.col + P.row_ptr[r + 1];
    for (int j = 0; j < Ke.n; ++j) {
      const int32_t *it = std::lower_bound(b, en, dofs[j]);
      if (it == en || *it != dofs[j]) return false;
      K[it - P.col] += Ke(i, j);
    }
  }
  return true;
}

// SparsityPattern::Build::handle_vi_vj (sparsity_pattern.C:152-275): merge the
// sorted element dofs into each sorted row.
void merge_row(std::vector<int32_t> &row, const std::vector<int32_t> &add) {
  std::vector<int32_t> out;
  out.reserve(row.size() + add.size());
  std::set_union(row.begin(), row.end(), add.begin(), add.end(), std::back_inserter(out));
  row.swap(out);
}

}  // namespace

extern "C" {

int orc_qgauss(int type, int order, double *pts, double *w, int cap) {
  std::vector<Pt> P;
  std::vector<double> W;
  if (!qgauss_3d(type, order, P, W)) return -1;
  const int n = (int)W.size();
  for (int q = 0; q < n && q < cap; ++q) {
    for (int d = 0; d < 3; ++d) pts[3 * q + d] = P[q].v[d];
    w[q] = W[q];
  }
  return n;
}

// phi [n][np], dphi [3][n][np]
int orc_shapes(int type, int order, int np, const double *pts, double *phi, double *dphi) {
  std::vector<Pt> P(np);
  for (int q = 0; q < np; ++q)
    for (int d = 0; d < 3; ++d) P[q].v[d] = pts[3 * q + d];
  std::vector<std::vector<double>> ph, dr[3];
  const int family = (order & 0x100) ? 1 : 0;  // HIERARCHIC flag
  order &= 0xff;
  const int n = n_shapes(type, order);
  if (!n) return -1;
  if (family == 1) {
    if (!hierarchic_built(type, order)) return -1;
    all_shapes_hierarchic(type, order, P, ph, dr);
  } else {
    all_shapes(type, order, P, ph, dr);
  }
  for (int i = 0; i < n; ++i)
    for (int q = 0; q < np; ++q) {
      phi[i * np + q] = ph[i][q];
      for (int c = 0; c < 3; ++c) dphi[(c * n + i) * np + q] = dr[c][i][q];
    }
  return n;
}

// The 64 cubic HIERARCHIC shapes of one HEX27 element (its 27 node
// coordinates X) and their difference-quotient derivatives: phi [64][np],
// dphi [3][64][np].
int orc_shapes_hier3(const double *X27, int np, const double *pts, double *phi, double *dphi) {
  std::vector<Pt> X(27);
  for (int a = 0; a < 27; ++a)
    for (int d = 0; d < 3; ++d) X[a].v[d] = X27[3 * a + d];
  for (int q = 0; q < np; ++q) {
    const Pt p = {{pts[3 * q], pts[3 * q + 1], pts[3 * q + 2]}};
    for (int i = 0; i < 64; ++i) {
      phi[i * np + q] = hier_hex3_shape(X, i, p);
      for (int c = 0; c < 3; ++c) dphi[(c * 64 + i) * np + q] = hier_hex3_deriv(X, i, c, p);
    }
  }
  return 64;
}

// HIERARCHIC shapes of one HEX27 (node coordinates X27 [27][3]) at order 2
// or 3 with the element's edge and face orientation: phi [n][np], dphi
// [3][n][np], n = (order + 1)^3.
int orc_shapes_hier_hex(const double *X27, int order, int np, const double *pts, double *phi, double *dphi) {
  if (order < 2 || order > 3) return -1;
  std::vector<Pt> X(27);
  for (int a = 0; a < 27; ++a)
    for (int d = 0; d < 3; ++d) X[a].v[d] = X27[3 * a + d];
  const int n = (order + 1) * (order + 1) * (order + 1);
  for (int q = 0; q < np; ++q) {
    const Pt p = {{pts[3 * q], pts[3 * q + 1], pts[3 * q + 2]}};
    for (int i = 0; i < n; ++i) {
      phi[i * np + q] = hier_hexo_shape(X, (unsigned)order, i, p);
      for (int c = 0; c < 3; ++c) dphi[(c * n + i) * np + q] = hier_hexo_deriv(X, (unsigned)order, i, c, p);
    }
  }
  return n;
}

// HIERARCHIC shapes of order 2 or 3 on one prism (vertex coordinates X6 [6][3]).
int orc_shapes_hier_prism(const double *X6, int order, int np, const double *pts, double *phi, double *dphi) {
  if (order < 2 || order > 3) return -1;
  std::vector<Pt> X(6);
  for (int a = 0; a < 6; ++a)
    for (int d = 0; d < 3; ++d) X[a].v[d] = X6[3 * a + d];
  const int n = (order + 1) * (order + 1) * (order + 2) / 2;
  for (int q = 0; q < np; ++q) {
    const Pt p = {{pts[3 * q], pts[3 * q + 1], pts[3 * q + 2]}};
    for (int i = 0; i < n; ++i) {
      phi[i * np + q] = prism::shape(X, (unsigned)order, i, p);
      for (int c = 0; c < 3; ++c) dphi[(c * n + i) * np + q] = prism::deriv(X, (unsigned)order, i, c, p);
    }
  }
  return n;
}

// Cubic HIERARCHIC shapes of one TET14 (node coordinates X14 [14][3]).
int orc_shapes_tet3(const double *X14, int np, const double *pts, double *phi, double *dphi) {
  std::vector<Pt> X(14);
  for (int a = 0; a < 14; ++a)
    for (int d = 0; d < 3; ++d) X[a].v[d] = X14[3 * a + d];
  for (int q = 0; q < np; ++q) {
    const Pt p = {{pts[3 * q], pts[3 * q + 1], pts[3 * q + 2]}};
    for (int i = 0; i < 20; ++i) {
      phi[i * np + q] = hier_tet3_shape(X, i, p);
      for (int c = 0; c < 3; ++c) dphi[(c * 20 + i) * np + q] = hier_tet3_deriv(X, i, c, p);
    }
  }
  return 20;
}

int orc_has_affine_map(int type, const double *X) {
  const int n = (type == TET4) ? 4 : (type == TET10) ? 10 : (type == TET14) ? 14 : (type == HEX8) ? 8
              : (type == PRISM6) ? 6 : 27;
  std::vector<Pt> p(n);
  for (int a = 0; a < n; ++a)
    for (int d = 0; d < 3; ++d) p[a].v[d] = X[3 * a + d];
  return has_affine_map(type, p) ? 1 : 0;
}

// DofMap::distribute_local_dofs_var_major (dof_map.C:1417-1537) and dof_indices.
int orc_distribute_dofs(int64_t n_nodes, int64_t n_elem, int npe, const int32_t *conn, int n_vars,
                        int32_t *elem_dofs, int64_t *n_dofs) {
  std::vector<int64_t> base(n_nodes, -1);
  int64_t next_free_dof = 0;
  for (int64_t e = 0; e < n_elem; ++e)
    for (int n = 0; n < npe; ++n) {
      const int32_t node = conn[e * npe + n];
      if (base[node] == -1) {
        base[node] = next_free_dof;
        next_free_dof += n_vars * 1;
      }
    }
  for (int64_t node = 0; node < n_nodes; ++node)
    if (base[node] == -1) {
      base[node] = next_free_dof;
      next_free_dof += n_vars;
    }
  *n_dofs = next_free_dof;
  const int nl = n_vars * npe;
  for (int64_t e = 0; e < n_elem; ++e)
    for (int v = 0; v < n_vars; ++v)
      for (int n = 0; n < npe; ++n)
        elem_dofs[e * nl + v * npe + n] = (int32_t)(base[conn[e * npe + n]] + v * 1 + 0);
  return 0;
}

// FEType{THIRD, HIERARCHIC} on HEX27, one variable: HIERARCHIC_n_dofs_at_node
// (fe_hierarchic.C:236-290) gives vertices 1, edge nodes o-1 = 2, face nodes
// (o-1)^2 = 4 and the centre node 0 dofs; the (o-1)^3 = 8 interior dofs belong
// to the element (n_dofs_per_elem).  distribute_local_dofs_var_major numbers,
// per element in order, the not yet numbered nodes, then the element's own
// dofs.  dof_indices (dof_map.h:2619-2760) lists each node's dofs, non-vertex
// nodes in reverse (extra_hanging_dofs is true for HIERARCHIC), then the
// element dofs.
static int hier3_node_dofs(int n) { return n < 8 ? 1 : (n < 20 ? 2 : (n < 26 ? 4 : 0)); }

int orc_distribute_dofs_hier3(int64_t n_nodes, int64_t n_elem, const int32_t *conn, int32_t *elem_dofs,
                              int64_t *n_dofs) {
  std::vector<int64_t> base(n_nodes, -1), ebase(n_elem);
  int64_t next_free_dof = 0;
  for (int64_t e = 0; e < n_elem; ++e) {
    for (int n = 0; n < 27; ++n) {
      const int32_t node = conn[e * 27 + n];
      if (hier3_node_dofs(n) > 0 && base[node] == -1) {
        base[node] = next_free_dof;
        next_free_dof += hier3_node_dofs(n);
      }
    }
    ebase[e] = next_free_dof;
    next_free_dof += 8;
  }
  *n_dofs = next_free_dof;
  for (int64_t e = 0; e < n_elem; ++e) {
    int32_t *d = elem_dofs + e * 64;
    int k = 0;
    for (int n = 0; n < 27; ++n) {
      const int nc = hier3_node_dofs(n);
      const int64_t b = base[conn[e * 27 + n]];
      if (n < 8) {
        for (int i = 0; i < nc; ++i) d[k++] = (int32_t)(b + i);
      } else {
        for (int i = nc - 1; i >= 0; --i) d[k++] = (int32_t)(b + i);
      }
    }
    for (int i = 0; i < 8; ++i) d[k++] = (int32_t)(ebase[e] + i);
  }
  return 0;
}

// FEType{THIRD, HIERARCHIC} on TET14 (HIERARCHIC_n_dofs_at_node,
// fe_hierarchic.C:440-470): vertex 1, edge node p - 1 = 2, face node
// (p - 1)(p - 2)/2 = 1, no element dofs; first-touch numbering per element
// and dof_indices listing a non-vertex node's dofs last to first.
static int tet3_node_dofs(int n) { return n < 4 ? 1 : (n < 10 ? 2 : 1); }

int orc_distribute_dofs_tet3(int64_t n_nodes, int64_t n_elem, const int32_t *conn, int32_t *elem_dofs,
                             int64_t *n_dofs) {
  std::vector<int64_t> base(n_nodes, -1);
  int64_t next_free_dof = 0;
  for (int64_t e = 0; e < n_elem; ++e)
    for (int n = 0; n < 14; ++n) {
      const int32_t node = conn[e * 14 + n];
      if (base[node] == -1) {
        base[node] = next_free_dof;
        next_free_dof += tet3_node_dofs(n);
      }
    }
  *n_dofs = next_free_dof;
  for (int64_t e = 0; e < n_elem; ++e) {
    int32_t *d = elem_dofs + e * 20;
    int k = 0;
    for (int n = 0; n < 14; ++n) {
      const int nc = tet3_node_dofs(n);
      const int64_t b = base[conn[e * 14 + n]];
      if (n < 4) {
        for (int i = 0; i < nc; ++i) d[k++] = (int32_t)(b + i);
      } else {
        for (int i = nc - 1; i >= 0; --i) d[k++] = (int32_t)(b + i);
      }
    }
  }
  return 0;
}

int orc_dirichlet_tet3(int64_t n_elem, const int32_t *elem_dofs, const int8_t *side_bid, const int32_t *bids,
                       int n_bids, uint8_t *constrained) {
  static const int T14[4][7] = {{0, 2, 1, 6, 5, 4, 10}, {0, 1, 3, 4, 8, 7, 11}, {1, 2, 3, 5, 9, 8, 12},
                                {2, 0, 3, 6, 7, 9, 13}};  // cell_tet14.C:45-51
  int first[14];
  for (int n = 0, k = 0; n < 14; ++n) { first[n] = k; k += tet3_node_dofs(n); }
  for (int64_t e = 0; e < n_elem; ++e)
    for (int s = 0; s < 4; ++s) {
      const int b = side_bid[e * 4 + s];
      if (b < 0 || std::find(bids, bids + n_bids, b) == bids + n_bids) continue;
      for (int a : T14[s])
        for (int i = 0; i < tet3_node_dofs(a); ++i) constrained[elem_dofs[e * 20 + first[a] + i]] = 1;
    }
  return 0;
}

// HIERARCHIC of order p = 2 on PRISM18 or p = 3 on PRISM21
// (HIERARCHIC_n_dofs_at_node, fe_hierarchic.C:289-340; no element dofs,
// fe_hierarchic.C:433-439): vertex 1, edge node p - 1, quad-face node
// (p - 1)^2, triangle-face node (p - 1)(p - 2)/2, interior node 20 of PRISM21
// (p - 1)^2 (p - 2)/2; first-touch numbering per element, dof_indices listing
// a non-vertex node's dofs last to first.
static int prism_node_dofs(int p, int n) {
  if (n < 6) return 1;
  if (n < 15) return p - 1;
  if (n < 18) return (p - 1) * (p - 1);
  if (n < 20) return (p - 1) * (p - 2) / 2;
  return (p - 1) * (p - 1) * (p - 2) / 2;
}

int orc_distribute_dofs_prism(int p, int64_t n_nodes, int64_t n_elem, const int32_t *conn, int32_t *elem_dofs,
                              int64_t *n_dofs) {
  const int npe = p == 2 ? 18 : 21, nl = (p + 1) * (p + 1) * (p + 2) / 2;
  std::vector<int64_t> base(n_nodes, -1);
  int64_t next_free_dof = 0;
  for (int64_t e = 0; e < n_elem; ++e)
    for (int n = 0; n < npe; ++n) {
      const int32_t node = conn[e * npe + n];
      if (prism_node_dofs(p, n) > 0 && base[node] == -1) {
        base[node] = next_free_dof;
        next_free_dof += prism_node_dofs(p, n);
      }
    }
  *n_dofs = next_free_dof;
  for (int64_t e = 0; e < n_elem; ++e) {
    int32_t *d = elem_dofs + e * nl;
    int k = 0;
    for (int n = 0; n < npe; ++n) {
      const int nc = prism_node_dofs(p, n);
      const int64_t b = base[conn[e * npe + n]];
      if (n < 6) {
        for (int i = 0; i < nc; ++i) d[k++] = (int32_t)(b + i);
      } else {
        for (int i = nc - 1; i >= 0; --i) d[k++] = (int32_t)(b + i);
      }
    }
  }
  return 0;
}

int orc_dirichlet_prism(int p, int64_t n_elem, const int32_t *elem_dofs, const int8_t *side_bid, const int32_t *bids,
                        int n_bids, uint8_t *constrained) {
  // cell_prism21.C side_nodes_map (PRISM18: the same without nodes 18, 19)
  static const int P21[5][9] = {{0, 2, 1, 8, 7, 6, 18, -1, -1}, {0, 1, 4, 3, 6, 10, 12, 9, 15},
                                {1, 2, 5, 4, 7, 11, 13, 10, 16}, {2, 0, 3, 5, 8, 9, 14, 11, 17},
                                {3, 4, 5, 12, 13, 14, 19, -1, -1}};
  const int npe = p == 2 ? 18 : 21, nl = (p + 1) * (p + 1) * (p + 2) / 2;
  int first[21];
  for (int n = 0, k = 0; n < npe; ++n) { first[n] = k; k += prism_node_dofs(p, n); }
  for (int64_t e = 0; e < n_elem; ++e)
    for (int s = 0; s < 5; ++s) {
      const int b = side_bid[e * 5 + s];
      if (b < 0 || std::find(bids, bids + n_bids, b) == bids + n_bids) continue;
      for (int a : P21[s])
        if (a >= 0 && a < npe)
          for (int i = 0; i < prism_node_dofs(p, a); ++i) constrained[elem_dofs[e * nl + first[a] + i]] = 1;
    }
  return 0;
}

// Homogeneous Dirichlet for the cubic HIERARCHIC hex: every dof on a node of
// a boundary side (vertex, edge and face dofs) has an empty row.
int orc_dirichlet_hier3(int64_t n_elem, const int32_t *elem_dofs, const int8_t *side_bid, const int32_t *bids,
                        int n_bids, uint8_t *constrained) {
  static const int H27[6][9] = {{0, 3, 2, 1, 11, 10, 9, 8, 20}, {0, 1, 5, 4, 8, 13, 16, 12, 21},
                                {1, 2, 6, 5, 9, 14, 17, 13, 22}, {2, 3, 7, 6, 10, 15, 18, 14, 23},
                                {3, 0, 4, 7, 11, 12, 19, 15, 24}, {4, 5, 6, 7, 16, 17, 18, 19, 25}};
  int first[27];
  for (int n = 0, k = 0; n < 27; ++n) { first[n] = k; k += hier3_node_dofs(n); }
  for (int64_t e = 0; e < n_elem; ++e)
    for (int s = 0; s < 6; ++s) {
      const int b = side_bid[e * 6 + s];
      if (b < 0 || std::find(bids, bids + n_bids, b) == bids + n_bids) continue;
      for (int a : H27[s])
        for (int i = 0; i < hier3_node_dofs(a); ++i) constrained[elem_dofs[e * 64 + first[a] + i]] = 1;
    }
  return 0;
}

// Dofs a homogeneous DirichletBoundary constrains on the given side ids
// (ConstrainDirichlet, dof_map_constraints.C:257-1560: LAGRANGE dofs of the side's nodes).
int orc_dirichlet(int64_t n_elem, int type, int n_vars, const int32_t *elem_dofs, const int8_t *side_bid,
                  const int32_t *bids, int n_bids, const int32_t *vars, int n_bc_vars, uint8_t *constrained) {
  static const int H8[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}, {4, 5, 6, 7}};
  static const int H27[6][9] = {{0, 3, 2, 1, 11, 10, 9, 8, 20}, {0, 1, 5, 4, 8, 13, 16, 12, 21},
                                {1, 2, 6, 5, 9, 14, 17, 13, 22}, {2, 3, 7, 6, 10, 15, 18, 14, 23},
                                {3, 0, 4, 7, 11, 12, 19, 15, 24}, {4, 5, 6, 7, 16, 17, 18, 19, 25}};
  static const int T4[4][3] = {{0, 2, 1}, {0, 1, 3}, {1, 2, 3}, {2, 0, 3}};
  static const int T10[4][6] = {{0, 2, 1, 6, 5, 4}, {0, 1, 3, 4, 8, 7}, {1, 2, 3, 5, 9, 8}, {2, 0, 3, 6, 7, 9}};
  static const int P6[5][4] = {{0, 2, 1, -1}, {0, 1, 4, 3}, {1, 2, 5, 4}, {2, 0, 3, 5}, {3, 4, 5, -1}};
  const int npe = (type == TET4) ? 4 : (type == TET10) ? 10 : (type == HEX8) ? 8 : (type == PRISM6) ? 6 : 27;
  const int ns = (type == TET4 || type == TET10) ? 4 : (type == PRISM6) ? 5 : 6;
  const int nl = n_vars * npe;
  for (int64_t e = 0; e < n_elem; ++e)
    for (int s = 0; s < ns; ++s) {
      const int b = side_bid[e * ns + s];
      if (b < 0 || std::find(bids, bids + n_bids, b) == bids + n_bids) continue;
      std::vector<int> sn;
      if (type == HEX8) sn.assign(H8[s], H8[s] + 4);
      else if (type == HEX27) sn.assign(H27[s], H27[s] + 9);
      else if (type == TET4) sn.assign(T4[s], T4[s] + 3);
      else if (type == PRISM6) sn.assign(P6[s], P6[s] + ((s == 0 || s == 4) ? 3 : 4));
      else sn.assign(T10[s], T10[s] + 6);
      for (int iv = 0; iv < n_bc_vars; ++iv)
        for (int a : sn) constrained[elem_dofs[e * nl + vars[iv] * npe + a]] = 1;
    }
  return 0;
}

// DofMap::compute_sparsity for a single rank: row_ptr [n_dofs+1], col [nnz].
// Call with row_ptr/col NULL to get nnz only.
int orc_sparsity(int64_t n_dofs, int64_t n_elem, int nl, const int32_t *elem_dofs, int64_t *nnz,
                 int32_t *row_ptr, int32_t *col) {
  std::vector<std::vector<int32_t>> rows(n_dofs);
  std::vector<int32_t> ed;
  for (int64_t e = 0; e < n_elem; ++e) {
    ed.assign(elem_dofs + e * nl, elem_dofs + (e + 1) * nl);
    std::sort(ed.begin(), ed.end());
    ed.erase(std::unique(ed.begin(), ed.end()), ed.end());
    for (int32_t r : ed) merge_row(rows[r], ed);
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

// Assembly over elements [e_begin, e_end) into K (CSR values) and F, both
// zeroed here first.  n_threads > 1 splits the range into contiguous chunks,
// each thread builds element matrices and inserts under one mutex, as
// FEMSystem::assembly does (src/systems/fem_system.C:940-944, 362-369).
// Returns 0, 4 (degenerate element, *bad_elem set) or 6 (entry outside the pattern).
// orc_assemble2 adds the constraint rows (cons_ptr [n_dofs+1], cons_col,
// cons_val; NULL = empty rows) and the form parameters (ADVDIFF).
int orc_assemble2(int form, int type, int fe_order, int q_order, int64_t n_nodes, const double *xyz,
                  int64_t n_elem, const int32_t *conn, int n_vars, const int32_t *elem_dofs, int64_t n_dofs,
                  const uint8_t *constrained, const double *coef, const double *nodal_f, double nu,
                  const int32_t *row_ptr, const int32_t *col, double *K, double *F, int n_threads,
                  int64_t e_begin, int64_t e_end, int64_t *bad_elem, double *loop_seconds,
                  const int64_t *cons_ptr, const int32_t *cons_col, const double *cons_val,
                  const double *params, int n_params);

int orc_assemble(int form, int type, int fe_order, int q_order, int64_t n_nodes, const double *xyz,
                 int64_t n_elem, const int32_t *conn, int n_vars, const int32_t *elem_dofs, int64_t n_dofs,
                 const uint8_t *constrained, const double *coef, const double *nodal_f, double nu,
                 const int32_t *row_ptr, const int32_t *col, double *K, double *F, int n_threads,
                 int64_t e_begin, int64_t e_end, int64_t *bad_elem, double *loop_seconds) {
  return orc_assemble2(form, type, fe_order, q_order, n_nodes, xyz, n_elem, conn, n_vars, elem_dofs, n_dofs,
                       constrained, coef, nodal_f, nu, row_ptr, col, K, F, n_threads, e_begin, e_end, bad_elem,
                       loop_seconds, nullptr, nullptr, nullptr, nullptr, 0);
}

int orc_assemble2(int form, int type, int fe_order, int q_order, int64_t n_nodes, const double *xyz,
                  int64_t n_elem, const int32_t *conn, int n_vars, const int32_t *elem_dofs, int64_t n_dofs,
                  const uint8_t *constrained, const double *coef, const double *nodal_f, double nu,
                  const int32_t *row_ptr, const int32_t *col, double *K, double *F, int n_threads,
                  int64_t e_begin, int64_t e_end, int64_t *bad_elem, double *loop_seconds,
                  const int64_t *cons_ptr, const int32_t *cons_col, const double *cons_val,
                  const double *params, int n_params) {
  Problem P{};
  const int family = (fe_order & 0x100) ? 1 : 0;  // HIERARCHIC flag (FEType family)
  fe_order &= 0xff;
  const bool prism_hi = family == 1 && ((fe_order == 2 && type == PRISM18) || (fe_order == 3 && type == PRISM21));
  const bool p3 = prism_hi || (family == 1 && fe_order == 3 && (type == HEX27 || type == TET14));
  if (family == 1 && !hierarchic_built(type, fe_order) && !p3) return 8;
  if (p3 && (n_vars != 1 || form == ELASTICITY)) return 8;
  P.cons_ptr = cons_ptr; P.cons_col = cons_col; P.cons_val = cons_val;
  P.params = params; P.n_params = n_params;
  if (form == ADVDIFF && n_params < 2) return 1;
  P.form = form; P.type = type; P.fe_order = fe_order; P.q_order = q_order;
  P.npe = prism_hi ? (type == PRISM18 ? 18 : 21)
                   : n_shapes(type, (type == HEX27 || type == TET10) ? 2 : (type == TET14 ? 3 : 1));
  P.n_vars = n_vars;
  P.nl = n_vars * (prism_hi ? (fe_order + 1) * (fe_order + 1) * (fe_order + 2) / 2
                            : (p3 ? (type == HEX27 ? 64 : 20) : P.npe));
  P.n_nodes = n_nodes; P.n_elem = n_elem; P.n_dofs = n_dofs;
  P.xyz = xyz; P.conn = conn; P.elem_dofs = elem_dofs; P.constrained = constrained;
  P.coef = coef; P.nodal_f = nodal_f; P.nu = nu; P.row_ptr = row_ptr; P.col = col;
  if (!p3 && n_shapes(type, fe_order) != P.npe) return 8;
  std::fill(K, K + row_ptr[n_dofs], 0.0);
  std::fill(F, F + n_dofs, 0.0);
  if (e_end > n_elem) e_end = n_elem;
  if (n_threads < 1) n_threads = 1;
  std::mutex mtx;
  int status = 0;
  int64_t first_bad = -1;
  auto work = [&](int64_t b, int64_t en) {
    OracleFE fe;
    fe.init(type, fe_order, q_order, family);
    Dense Ke;
    std::vector<double> Fe;
    std::vector<int32_t> dofs;
    for (int64_t e = b; e < en; ++e) {
      const bool ok = element_matrix(P, fe, e, Ke, Fe, dofs);
      std::lock_guard<std::mutex> lk(mtx);
      if (!ok && status == 0) { status = 4; first_bad = e; }
      if (!add_matrix(P, Ke, dofs, K) && status == 0) status = 6;
      for (size_t i = 0; i < dofs.size(); ++i) F[dofs[i]] += Fe[i];  // PetscVector::add_vector
    }
  };
  const auto t0 = std::chrono::steady_clock::now();
  if (n_threads == 1) {
    work(e_begin, e_end);
  } else {
    std::vector<std::thread> th;
    const int64_t n = e_end - e_begin;
    for (int t = 0; t < n_threads; ++t)
      th.emplace_back(work, e_begin + n * t / n_threads, e_begin + n * (t + 1) / n_threads);
    for (auto &t : th) t.join();
  }
  if (loop_seconds)
    *loop_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (bad_elem) *bad_elem = first_bad;
  return status;
}

}  // extern "C"
